"""Raw snapshots (src/simulation_io.c:16-149): the slab, N*SIM_DOF floats,
no header.  The golden file was written by the compiled reference's
sim_save_raw after two PP steps of 64 bodies (tests/golden/make_golden.py).

CPU tests: the drop-in sim_save_raw / sim_read_raw on a host slab write and
read exactly the reference's bytes.  GPU tests: resident snapshots
(sfgpu_save_raw, asynchronous while stepping) equal the downloaded state,
and sfgpu_read_raw restores it."""
import ctypes as C
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD_BIN = os.path.join(HERE, "golden", "raw_pp_n64_2steps.bin")
GOLD_NPZ = os.path.join(HERE, "golden", "raw_pp_n64_2steps.npz")


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def host_sim(sf, slab, n):
    sim = sf.SimT()
    sim.N = n
    sim.mem = slab.ctypes.data
    return sim


def test_golden_file_is_the_slab():
    d = np.load(GOLD_NPZ)
    raw = np.fromfile(GOLD_BIN, np.float32)
    assert raw.size == int(d["n"]) * int(d["dof"])
    np.testing.assert_array_equal(raw, d["slab"])


def test_compat_save_raw_matches_reference_bytes(sf, tmp_path):
    d = np.load(GOLD_NPZ)
    n = int(d["n"])
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params())
    slab = np.ascontiguousarray(d["slab"], np.float32)
    sim = host_sim(sf, slab, n)
    out = str(tmp_path / "snap.bin")
    assert L.sim_save_raw(C.byref(sim), out.encode()) == 0
    assert open(out, "rb").read() == open(GOLD_BIN, "rb").read()


def test_compat_read_raw_and_errors(sf, tmp_path):
    d = np.load(GOLD_NPZ)
    n = int(d["n"])
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params())
    slab = np.zeros(n * int(d["dof"]), np.float32)
    sim = host_sim(sf, slab, n)
    assert L.sim_read_raw(C.byref(sim), GOLD_BIN.encode()) == 0
    np.testing.assert_array_equal(slab, d["slab"])
    # missing file and NULL name fail; a short file is reported, not failed (as the reference)
    assert L.sim_read_raw(C.byref(sim), str(tmp_path / "missing.bin").encode()) == -1
    assert L.sim_save_raw(C.byref(sim), None) == -1
    short = tmp_path / "short.bin"
    short.write_bytes(open(GOLD_BIN, "rb").read()[:100])
    assert L.sim_read_raw(C.byref(sim), str(short).encode()) == 0


@pytest.mark.gpu
def test_resident_snapshots_while_stepping(sf, tmp_path):
    from starflood_gb300.ics import uniform_ball
    n = 5000
    pos, vel, mas = uniform_ball(n, seed=21)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3)
    files, states = [], []
    with sf.Sim(n, p) as s, sf.Sim(n, p) as twin:
        for x in (s, twin):
            x.set_state(pos, vel, mas)
            x.solve(0)
        for k in range(3):
            s.run(5 * k, 5)
            f = str(tmp_path / ("step_%04d.raw" % (5 * k + 5)))
            s.save_raw(f)   # queued behind the steps, no sync
            files.append(f)
            twin.run(5 * k, 5)
            states.append(twin.download().copy())
        s.snapshot_wait()
        for f, st in zip(files, states):
            np.testing.assert_array_equal(np.fromfile(f, np.float32), st)
        # restore the first snapshot into the twin and step on: same as s from that state
        twin.read_raw(files[0])
        np.testing.assert_array_equal(twin.download(), states[0])
        bad = str(tmp_path / "no_such_dir" / "x.raw")
        s.save_raw(bad)
        with pytest.raises(sf.SfgpuError):
            s.snapshot_wait()
        with pytest.raises(sf.SfgpuError):
            twin.read_raw(str(tmp_path / "missing.raw"))


@pytest.mark.gpu
def test_resident_read_reference_snapshot(sf):
    d = np.load(GOLD_NPZ)
    n = int(d["n"])
    with sf.Sim(n, sf.default_params(solver=sf.SOLVER_PP, eps=0.01)) as s:
        s.read_raw(GOLD_BIN)
        np.testing.assert_array_equal(s.download(), d["slab"])
