"""vis_draw, the particle splat rasteriser (src/visualization.c:258-740),
and vis_save's image writers (src/visualization_io.c).

Golden fixture: the compiled reference's vis_draw of a 2048-body Plummer
sphere at step 7, 96 x 64 pixels, and its PPM file of that render
(tests/golden/make_golden.py).

CPU: the oracle's restatement reproduces the reference's accumulation and
render buffers bit for bit; the library's vis_save writes the reference's
PPM bytes and a PFM of the render.  GPU: sfgpu_vis_draw and the drop-in
vis_draw against the fixture.  The GPU evaluates logf / cosf / sinf / tanh
with CUDA's functions, which may differ from the host libm by an ulp, so a
sample whose coordinate falls within an ulp of a pixel edge can move one
pixel: at least 99.5 % of the int32 entries must be identical, the total
sample count (alpha) must agree to 0.1 %, and the L1 difference of the
accumulation buffer must stay below 0.5 % of its L1 norm."""
import ctypes as C
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "vis_plummer_n2048_96x64_step7.npz")
GOLD_PPM = os.path.join(HERE, "golden", "vis_plummer_n2048_96x64_step7.ppm")


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def close_accum(got, ref):
    got = np.asarray(got, np.int64)
    ref = np.asarray(ref, np.int64)
    same = float((got == ref).mean())
    alpha = abs(int(got[..., 3].sum()) - int(ref[..., 3].sum())) / max(1, int(ref[..., 3].sum()))
    l1 = float(np.abs(got - ref).sum()) / max(1.0, float(np.abs(ref).sum()))
    return same, alpha, l1


def test_oracle_vis_matches_reference(oracle32):
    d = np.load(GOLD)
    acc, ren = oracle32.vis_draw(d["pos"], d["vel"], d["pot"], int(d["step"]), float(d["timestep"]),
                                 int(d["sizex"]), int(d["sizey"]))
    np.testing.assert_array_equal(acc, d["accum"])
    np.testing.assert_array_equal(ren, d["render"])


def _host_vis(sf, render):
    """A vis_t over numpy buffers (vis_save needs no device)."""
    sizey, sizex = render.shape[:2]
    render = np.ascontiguousarray(render, np.float32)
    binary = np.zeros(3 * sizex * sizey * 4, np.uint8)
    vis = sf.VisT()
    vis.sizex, vis.sizey = sizex, sizey
    vis.render_buffer = render.ctypes.data
    vis.binary_buffer = binary.ctypes.data
    return vis, (render, binary)


def test_vis_save_ppm_matches_reference(sf, tmp_path):
    d = np.load(GOLD)
    L = sf.compat_functions()
    vis, keep = _host_vis(sf, d["render"])
    out = str(tmp_path / "frame.ppm")
    assert L.vis_save(C.byref(vis), out.encode(), 1) == 0
    assert open(out, "rb").read() == open(GOLD_PPM, "rb").read()


def test_vis_save_pfm(sf, tmp_path):
    d = np.load(GOLD)
    L = sf.compat_functions()
    vis, keep = _host_vis(sf, d["render"])
    out = str(tmp_path / "frame.pfm")
    assert L.vis_save(C.byref(vis), out.encode(), 0) == 0
    raw = open(out, "rb").read()
    header = b"PF\n96 64\n-1.0\n"
    assert raw.startswith(header)
    body = np.frombuffer(raw[len(header):], np.float32).reshape(64, 96, 3)
    np.testing.assert_array_equal(body, d["render"][..., :3])
    # PNG is not built in: reported on stderr, 0 returned as the reference does
    assert L.vis_save(C.byref(vis), str(tmp_path / "frame.png").encode(), 2) == 0
    assert not os.path.exists(tmp_path / "frame.png")


@pytest.mark.gpu
def test_gpu_vis_draw_vs_reference(sf):
    d = np.load(GOLD)
    n = len(d["pos"])
    sx, sy = int(d["sizex"]), int(d["sizey"])
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=float(d["timestep"]))
    with sf.Sim(n, p) as s:
        slab = np.zeros(n * 13, np.float32)
        v = sf.slab_views(slab, n, 13)
        v["pos"][:] = d["pos"]
        v["vel"][:] = d["vel"]
        v["mas"][:] = d["mas"]
        v["pot"][:] = d["pot"]
        s.upload(slab)
        acc, ren = s.vis_draw(int(d["step"]), sx, sy)
    same, alpha, l1 = close_accum(acc, d["accum"])
    assert same >= 0.995, same
    assert alpha <= 1e-3, alpha
    assert l1 <= 5e-3, l1
    # the render buffer follows the accumulation buffer
    assert float(np.abs(ren - d["render"]).max()) < 0.05


@pytest.mark.gpu
def test_compat_vis_draw(sf):
    d = np.load(GOLD)
    n = len(d["pos"])
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=float(d["timestep"])))
    sim = sf.SimT()
    assert L.sim_init(C.byref(sim), n) == 0
    try:
        slab = np.frombuffer((C.c_float * (n * 13)).from_address(sim.mem), np.float32)
        v = sf.slab_views(slab, n, 13)
        v["pos"][:] = d["pos"]
        v["vel"][:] = d["vel"]
        v["mas"][:] = d["mas"]
        v["pot"][:] = d["pot"]
        sim.step_number = int(d["step"])
        vis = sf.VisT()
        assert L.vis_init(C.byref(vis), int(d["sizex"]), int(d["sizey"])) == 0
        try:
            assert L.vis_draw(C.byref(vis), C.byref(sim)) == 0
            px = int(d["sizex"]) * int(d["sizey"])
            acc = np.frombuffer((C.c_int32 * (4 * px)).from_address(vis.atomic_buffer), np.int32)
            same, alpha, l1 = close_accum(acc.reshape(d["accum"].shape), d["accum"])
            assert same >= 0.995 and alpha <= 1e-3 and l1 <= 5e-3, (same, alpha, l1)
        finally:
            L.vis_free(C.byref(vis))
    finally:
        L.sim_free(C.byref(sim))
