"""PP gravity and the KDK step on the GPU against the oracle (GPU only).

Tolerances: EXACT arithmetic is bit-identical to the reference; FAST is
within 1e-5 global relative L2 of the FP32 reference (gravity.c with Kahan);
the COMPENSATED form within 1e-6 of the FP64 oracle."""
import numpy as np
import pytest

from conftest import golden
from oracle.pyoracle import make_params, slab_views

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(np.asarray(b, np.float64)))


def _sim_from(sf, d, **kw):
    n = len(d["pos"])
    p = sf.default_params(**kw)
    s = sf.Sim(n, p)
    s.set_state(d["pos"], d["vel"], d["mas"], d["rad"] if "rad" in d else None)
    return s, n


def test_pp_exact_bit_identical_c1(sf):
    d = golden("pp_uniform_n4096_eps0.01_10steps.npz")
    s, n = _sim_from(sf, d, solver=sf.SOLVER_PP, eps=0.01, dt=1e-3, math=sf.MATH_EXACT)
    s.solve(0)
    v = slab_views(s.download(), n, 13)
    np.testing.assert_array_equal(v["acc"], d["solv_acc"])
    np.testing.assert_array_equal(v["pot"], d["solv_pot"])
    for k in range(int(d["steps"])):
        s.step(k)
    np.testing.assert_array_equal(s.download(), d["final_slab"])
    s.close()


def test_pp_exact_graph_run_matches_steps(sf):
    d = golden("pp_uniform_n4096_eps0.01_10steps.npz")
    s, n = _sim_from(sf, d, solver=sf.SOLVER_PP, eps=0.01, dt=1e-3, math=sf.MATH_EXACT)
    s.solve(0)
    s.run(0, int(d["steps"]))  # replayed CUDA graph
    np.testing.assert_array_equal(s.download(), d["final_slab"])
    s.close()


def test_pp_fast_c1(sf, oracle32, oracle64):
    d = golden("pp_uniform_n4096_eps0.01_10steps.npz")
    s, n = _sim_from(sf, d, solver=sf.SOLVER_PP, eps=0.01, dt=1e-3)
    s.solve(0)
    v = slab_views(s.download(), n, 13)
    assert rel_l2(v["acc"], d["solv_acc"]) < 1e-5
    assert rel_l2(v["pot"], d["solv_pot"]) < 1e-6
    a64, p64 = oracle64.pp(d["pos"].astype(np.float64), d["mas"].astype(np.float64), make_params(eps=0.01))
    assert rel_l2(v["acc"], a64) < 1e-5
    for k in range(int(d["steps"])):
        s.step(k)
    out = slab_views(s.download(), n, 13)
    ref = slab_views(d["final_slab"], n, 13)
    assert rel_l2(out["pos"], ref["pos"]) < 1e-6
    assert rel_l2(out["vel"], ref["vel"]) < 1e-5
    s.close()


def test_pp_plummer_eps0005(sf):
    d = golden("pp_plummer_n2048_eps0.005_2steps.npz")
    s, n = _sim_from(sf, d, solver=sf.SOLVER_PP, eps=0.005, dt=1e-3, math=sf.MATH_EXACT)
    s.solve(0)
    v = slab_views(s.download(), n, 13)
    np.testing.assert_array_equal(v["acc"], d["solv_acc"])
    for k in range(int(d["steps"])):
        s.step(k)
    np.testing.assert_array_equal(s.download(), d["final_slab"])
    s.close()


@pytest.mark.parametrize("n", [1, 2, 7, 129, 1000, 5003])
def test_pp_ragged_sizes(sf, oracle32, n):
    from starflood_gb300.ics import uniform_ball
    pos, vel, mas = uniform_ball(n, seed=100 + n)
    for math in (sf.MATH_EXACT, sf.MATH_FAST):
        p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, math=math)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            v = slab_views(s.download(), n, 13)
        a, pt = oracle32.pp(pos, mas, make_params(eps=0.01))
        if math == sf.MATH_EXACT:
            np.testing.assert_array_equal(v["acc"], a)
            np.testing.assert_array_equal(v["pot"], pt)
        else:
            if n > 1:
                assert rel_l2(v["acc"], a) < 1e-5
            assert rel_l2(v["pot"], pt) < 1e-6


def test_pp_single_body_self_term(sf):
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, G=1.0)
    with sf.Sim(1, p) as s:
        s.set_state(np.array([[0.3, -0.2, 0.1]], np.float32), np.zeros((1, 3), np.float32), np.array([2.0], np.float32))
        s.solve(0)
        v = slab_views(s.download(), 1, 13)
    assert np.all(v["acc"] == 0.0)
    assert abs(v["pot"][0] - (-2.0 / 0.01)) < 1e-3  # j == i included (gravity.c:725-732)


def test_pp_compensated_vs_fp64(sf, oracle64):
    from starflood_gb300.ics import plummer
    n = 16384
    pos, vel, mas = plummer(n, seed=9)
    p64 = make_params(eps=0.005)
    a64, pot64 = oracle64.pp(pos.astype(np.float64), mas.astype(np.float64), p64)
    errs = {}
    for form in (sf.FORM_PLAIN, sf.FORM_COMPENSATED):
        p = sf.default_params(solver=sf.SOLVER_PP, eps=0.005, form=form)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            v = slab_views(s.download(), n, 13)
        errs[form] = rel_l2(v["acc"], a64)
    assert errs[sf.FORM_COMPENSATED] <= 1e-6, errs
    assert errs[sf.FORM_COMPENSATED] <= errs[sf.FORM_PLAIN] * 1.01, errs


def test_stateless_pp_on_device_arrays(sf, oracle32):
    import ctypes as C
    from starflood_gb300.ics import uniform_ball
    n = 3000
    pos, vel, mas = uniform_ball(n, seed=5)
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, math=sf.MATH_EXACT)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        base = sf.lib().sfgpu_device_slab(s.h)
        f = 4
        rc = sf.lib().sfgpu_gravity_pp(C.byref(p), n, C.c_void_p(base), C.c_void_p(base + 9 * n * f),
                                       C.c_void_p(base + 6 * n * f), C.c_void_p(base + 10 * n * f),
                                       C.c_void_p(sf.lib().sfgpu_stream(s.h)))
        assert rc == 0, sf.last_error()
        s.sync()
        v = slab_views(s.download(), n, 13)
    a, pt = oracle32.pp(pos, mas, make_params(eps=0.01))
    np.testing.assert_array_equal(v["acc"], a)


def test_energies_match_reference_sums(sf, oracle32):
    d = golden("pp_uniform_n4096_eps0.01_10steps.npz")
    s, n = _sim_from(sf, d, solver=sf.SOLVER_PP, eps=0.01, dt=1e-3, math=sf.MATH_EXACT)
    p = make_params(dt=1e-3, eps=0.01)
    osim, oslab, _ = oracle32.new_sim(n, p)
    ov = slab_views(oslab, n, 13)
    ov["pos"][:] = d["pos"]
    ov["vel"][:] = d["vel"]
    ov["mas"][:] = d["mas"]
    oracle32.sim_solv(p, osim, 0)
    s.solve(0)
    for k in range(3):
        _, T, V = oracle32.sim_step(p, osim, k)
        s.step(k)
        Tg, Vg = s.energies()
        assert abs(Tg - T) <= 1e-14 * abs(T) and abs(Vg - V) <= 1e-14 * abs(V)
    s.close()
