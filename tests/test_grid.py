"""The particle-mesh grid: grid_init / grid_solve_fft (src/grid.c:26-536)
and the deposit of solve_gravity_part_mesh (src/gravity.c:116-238).

Parity is unpinned: the reference's grid_solve_fft needs FFTW (absent here)
and its deposit is compiled out by #if 0 (it does not compile as written),
so the checker is the oracle's own restatement: the deposit in FP32 with the
host libm, the solve in FP64 by the DFT's definition.  CPU: that DFT solve
against numpy's FFT, the deposit's invariants, grid_init's argument checks.
GPU: the device deposit against the oracle (CUDA's logf / cosf / sinf may
differ from the host libm by an ulp, so a sample within an ulp of a cell
face can move one cell: at least 99.5 % of cells identical, totals within
0.1 %), the cuFFT solve against the FP64 oracle (relative L2 error <= 2e-5,
FP32 FFT rounding), and at the reference's full size (256^3, [-2, 2]^3) the
size-independent properties: a unit sample at the centre returns side^3
times the stencil, and the solve is linear."""
import ctypes as C

import numpy as np
import pytest

LO, HI = (-2.0, -2.0, -2.0), (2.0, 2.0, 2.0)
SOLVE_TOL = 2e-5


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def rel_l2(got, ref):
    return float(np.linalg.norm((np.asarray(got, np.float64) - ref).ravel()) / np.linalg.norm(ref.ravel()))


def numpy_solve(samp, stencil):
    d = samp.shape[0]
    out = np.real(np.fft.ifftn(np.fft.fftn(samp.astype(np.float64)) * np.fft.fftn(stencil.astype(np.float64))))
    return np.roll(out * d ** 3, shift=(-(d // 2),) * 3, axis=(0, 1, 2))


@pytest.mark.parametrize("side", [1, 2, 8, 15, 16])
def test_oracle_solve_is_the_dft_convolution(oracle32, side):
    rng = np.random.default_rng(side)
    samp = rng.random((side,) * 3).astype(np.float32)
    out = oracle32.grid_solve_fft(side, LO, HI, samp)
    ref = numpy_solve(samp, oracle32.grid_stencil(side, LO, HI))
    assert np.abs(out - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_oracle_stencil_values(oracle32):
    """grid.c:286-306: the corner of cell (x, y, z) is min + wid * idx / side
    in FP32; r = 0 gives 0."""
    d = 8
    st = oracle32.grid_stencil(d, LO, HI, G=1.0)
    assert st[d // 2, d // 2, d // 2] == 0.0
    c = np.float32(4.0) * (np.arange(d, dtype=np.float32) / np.float32(d)) + np.float32(-2.0)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    r2 = (x * x + y * y) + z * z
    with np.errstate(divide="ignore"):
        ref = np.where(r2 > 0, np.float32(-1.0) * (np.float32(1.0) / np.sqrt(r2)), np.float32(0.0))
    np.testing.assert_array_equal(st, ref.astype(np.float32))


def test_oracle_deposit_invariants(oracle32):
    rng = np.random.default_rng(3)
    pos = (rng.random((500, 3)) * 2.0 - 1.0).astype(np.float32)
    acc, pot = oracle32.grid_deposit(32, LO, HI, pos, step=4)
    # every sample of a body 1 unit inside the box lands on the grid
    assert int(acc.sum()) == 500 * 128
    np.testing.assert_array_equal(pot, (acc.astype(np.float64) / 128.0).astype(np.float32))
    acc2, _ = oracle32.grid_deposit(32, LO, HI, pos, step=4)
    np.testing.assert_array_equal(acc, acc2)
    acc3, _ = oracle32.grid_deposit(32, LO, HI, pos, step=5)
    assert not np.array_equal(acc, acc3)
    # the samples of one body scatter with sigma 0.5 cell around it
    one = np.array([[0.3, -0.2, 0.7]], np.float32)
    a1, _ = oracle32.grid_deposit(64, LO, HI, one, step=0, samples=4096)
    idx = np.argwhere(a1 > 0)
    w = a1[a1 > 0].astype(np.float64)
    mean = (idx * w[:, None]).sum(0) / w.sum()
    centre = (one[0][::-1] + 2.0) / 4.0 * 64  # [z, y, x]
    assert np.all(np.abs(mean - centre) < 0.1)


def test_grid_init_rejects_bad_sides(sf):
    """grid.c:29-35: side_length outside [1, 256] fails before any device work."""
    L = sf.compat_functions()
    lo = (C.c_float * 3)(*LO)
    hi = (C.c_float * 3)(*HI)
    for side in (0, 257):
        g = sf.GridT()
        assert L.grid_init(C.byref(g), side, lo, hi) == -1
        assert not g.mem


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("side", [1, 2, 8, 15, 16, 32, 64])
def test_gpu_solve_matches_oracle(sf, oracle32, side):
    rng = np.random.default_rng(100 + side)
    samp = rng.random((side,) * 3).astype(np.float32)
    ref = oracle32.grid_solve_fft(side, LO, HI, samp)
    with sf.Grid(side, LO, HI) as g:
        g.upload(samp)
        g.solve_fft()
        got = g.download()
    if side == 1:
        np.testing.assert_array_equal(got, ref.astype(np.float32))
    else:
        assert rel_l2(got, ref) <= SOLVE_TOL


@pytest.mark.gpu
def test_gpu_solve_other_bounds_and_G(sf, oracle32):
    lo, hi = (-1.0, -3.0, -2.5), (3.0, 1.0, 1.5)
    samp = np.random.default_rng(7).random((24,) * 3).astype(np.float32)
    ref = oracle32.grid_solve_fft(24, lo, hi, samp, G=0.5)
    with sf.Grid(24, lo, hi, G=0.5) as g:
        g.upload(samp)
        g.solve_fft()
        assert rel_l2(g.download(), ref) <= SOLVE_TOL


def close_counts(got, ref):
    same = float((got == ref).mean())
    tot = abs(int(got.sum()) - int(ref.sum())) / max(1, int(ref.sum()))
    return same, tot


@pytest.mark.gpu
@pytest.mark.parametrize("side,n,samples", [(32, 2000, 128), (64, 5000, 128), (16, 300, 100)])
def test_gpu_deposit_matches_oracle(sf, oracle32, side, n, samples):
    from starflood_gb300.ics import plummer
    pos, vel, mas = plummer(n, seed=side)
    pos = pos.astype(np.float32)
    acc_ref, pot_ref = oracle32.grid_deposit(side, LO, HI, pos, step=9, samples=samples)
    p = sf.default_params(solver=sf.SOLVER_PP)
    sim = sf.Sim(n, p)
    try:
        sim.set_state(pos, vel, mas)
        with sf.Grid(side, LO, HI) as g:
            g.deposit(sim, 9, samples)
            samp, acc = g.download(counts=True)
    finally:
        sim.close()
    same, tot = close_counts(acc, acc_ref)
    assert same >= 0.995 and tot <= 1e-3, (same, tot)
    np.testing.assert_array_equal(samp, (acc.astype(np.float64) / samples).astype(np.float32))


@pytest.mark.gpu
def test_gpu_centre_delta_returns_stencil_full_size(sf, oracle32):
    """256^3 over [-2, 2]^3 (GRID_SIZE 8): the convolution of a unit sample
    at cell (128, 128, 128) with the stencil, rolled by 128, is side^3 times
    the stencil itself."""
    d = 256
    samp = np.zeros((d, d, d), np.float32)
    samp[d // 2, d // 2, d // 2] = 1.0
    st = oracle32.grid_stencil(d, LO, HI).astype(np.float64) * float(d) ** 3
    with sf.Grid(d, LO, HI) as g:
        g.upload(samp)
        g.solve_fft()
        got = g.download()
    assert rel_l2(got, st) <= SOLVE_TOL


@pytest.mark.gpu
def test_gpu_solve_linear_full_size(sf):
    d = 256
    rng = np.random.default_rng(11)
    a = rng.random((d, d, d), np.float32)
    b = np.zeros((d, d, d), np.float32)
    b[rng.integers(0, d, 200), rng.integers(0, d, 200), rng.integers(0, d, 200)] = 1.0
    outs = []
    with sf.Grid(d, LO, HI) as g:
        for x in (a, b, (np.float32(2.0) * a + np.float32(3.0) * b).astype(np.float32)):
            g.upload(x)
            g.solve_fft()
            outs.append(g.download().astype(np.float64))
    lin = 2.0 * outs[0] + 3.0 * outs[1]
    assert rel_l2(outs[2], lin) <= SOLVE_TOL


@pytest.mark.gpu
def test_gpu_compat_grid_and_mesh(sf, oracle32):
    """grid_init / grid_solve_fft / solve_gravity_part_mesh over sim_t."""
    from starflood_gb300.ics import plummer
    L = sf.compat_functions()
    n, side = 3000, 32
    lo = (C.c_float * 3)(*LO)
    hi = (C.c_float * 3)(*HI)
    g = sf.GridT()
    assert L.grid_init(C.byref(g), side, lo, hi) == 0
    try:
        assert list(g.dim) == [side] * 3 and g.mem and g.mem_fft0 and not g.mem_fft1
        cells = side ** 3
        samp = np.ctypeslib.as_array(C.cast(L.grid_samp(C.byref(g)), C.POINTER(C.c_float)), (cells,))
        x = np.random.default_rng(5).random(cells).astype(np.float32)
        samp[:] = x
        assert L.grid_solve_fft(C.byref(g)) == 0
        ref = oracle32.grid_solve_fft(side, LO, HI, x.reshape((side,) * 3))
        assert rel_l2(samp.reshape((side,) * 3), ref) <= SOLVE_TOL
        # the mesh deposit of a sim_t's bodies, then the solve
        s = sf.SimT()
        assert L.sim_init(C.byref(s), n) == 0
        try:
            pos, vel, mas = plummer(n, seed=2)
            P = np.ctypeslib.as_array(C.cast(s.mem, C.POINTER(C.c_float)), (3 * n,))
            P[:] = pos.astype(np.float32).ravel()
            s.step_number = 6
            assert L.solve_gravity_part_mesh(C.byref(s), C.byref(g)) == 0
            counts = np.ctypeslib.as_array(C.cast(g.mem + 4 * cells, C.POINTER(C.c_int32)), (cells,))
            acc_ref, pot_ref = oracle32.grid_deposit(side, LO, HI, pos.astype(np.float32), step=6)
            same, tot = close_counts(counts.reshape((side,) * 3), acc_ref)
            assert same >= 0.995 and tot <= 1e-3
            ref = oracle32.grid_solve_fft(side, LO, HI, (counts.astype(np.float64) / 128.0).astype(np.float32)
                                          .reshape((side,) * 3))
            assert rel_l2(samp.reshape((side,) * 3), ref) <= SOLVE_TOL
        finally:
            L.sim_free(C.byref(s))
    finally:
        L.grid_free(C.byref(g))
