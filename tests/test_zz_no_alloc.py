"""sfgpu_gravity_pp_noalloc: the PP force for callers that cannot allocate
device memory (a host whose own memory pool owns the GPU's memory, a loop
that cannot take cudaMalloc's implicit synchronisation).  Its work array is
built into the library instead of cudaMalloc'd.  Checked through the C ABI
against sfgpu_gravity_pp on the same device arrays, for two calls in a row
(the built-in array is shared and reused between calls).  This file is
collected last so that a failure here comes after every other test has run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def _rel(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b.astype(np.float64)))


@pytest.mark.parametrize("form", ["plain", "compensated"])
def test_noalloc_matches_allocating_entry_point(sf, form):
    from starflood_gb300.ics import uniform_ball
    n = 20000
    pos, vel, mas = uniform_ball(n, seed=77)
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01,
                          form=sf.FORM_COMPENSATED if form == "compensated" else sf.FORM_PLAIN)
    L = sf.lib()
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        base = L.sfgpu_device_slab(s.h)
        f = 4
        args = (C.c_void_p(base), C.c_void_p(base + 9 * n * f), C.c_void_p(base + 6 * n * f),
                C.c_void_p(base + 10 * n * f), C.c_void_p(L.sfgpu_stream(s.h)))
        assert L.sfgpu_gravity_pp(C.byref(p), n, *args) == 0, sf.last_error()
        s.sync()
        want = sf.slab_views(s.download(), n, 13)
        want_acc, want_pot = want["acc"].copy(), want["pot"].copy()
        got = []
        for _ in range(2):  # two calls in a row share the built-in array
            assert L.sfgpu_gravity_pp_noalloc(C.byref(p), n, *args) == 0, sf.last_error()
            s.sync()
            v = sf.slab_views(s.download(), n, 13)
            got.append((v["acc"].copy(), v["pot"].copy()))
    for acc, pot in got:
        # same kernels, possibly fewer j-splits: float sums in another order
        assert _rel(acc, want_acc) < 1e-6
        assert _rel(pot, want_pot) < 1e-6
    np.testing.assert_array_equal(got[0][0], got[1][0])
    np.testing.assert_array_equal(got[0][1], got[1][1])


def test_noalloc_rejects_sizes_beyond_its_array(sf):
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01)
    rc = sf.lib().sfgpu_gravity_pp_noalloc(C.byref(p), (1 << 20) + 1, None, None, None, None, None)
    assert rc != 0
    assert "exceeds the maximum" in sf.last_error()
    pc = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, form=sf.FORM_COMPENSATED)
    rc = sf.lib().sfgpu_gravity_pp_noalloc(C.byref(pc), (1 << 19) + 1, None, None, None, None, None)
    assert rc != 0
    assert "exceeds the maximum" in sf.last_error()


def test_noalloc_exact_has_no_size_limit(sf):
    """EXACT math needs no work array: N above the FAST limit is accepted
    and gives the allocating entry point's result bit for bit."""
    n = (1 << 20) + 3
    rng = np.random.default_rng(5)
    pos = rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    mas = np.full(n, 1.0 / n, np.float32)
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, math=sf.MATH_EXACT)
    L = sf.lib()
    with sf.Sim(n, p) as s:
        s.set_state(pos, np.zeros_like(pos), mas)
        base = L.sfgpu_device_slab(s.h)
        f = 4
        args = (C.c_void_p(base), C.c_void_p(base + 9 * n * f), C.c_void_p(base + 6 * n * f),
                C.c_void_p(base + 10 * n * f), C.c_void_p(L.sfgpu_stream(s.h)))
        out = []
        for fn in (L.sfgpu_gravity_pp, L.sfgpu_gravity_pp_noalloc):
            assert fn(C.byref(p), n, *args) == 0, sf.last_error()
            s.sync()
            v = sf.slab_views(s.download(), n, 13)
            out.append((v["acc"].copy(), v["pot"].copy()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
