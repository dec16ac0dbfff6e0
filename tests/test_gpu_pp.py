"""PP gravity and the KDK step on the GPU against the oracle (GPU only).

Tolerances: EXACT arithmetic is bit-identical to the reference; FAST is
within 1e-5 global relative L2 of the FP32 reference (gravity.c with Kahan);
the COMPENSATED form within 1e-6 of the FP64 oracle."""
import numpy as np
import pytest

from conftest import err_summary, golden, per_body_rel
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
    # per-particle relative L2 against the reference (FP32, Kahan) and FP64
    e32 = per_body_rel(v["acc"], d["solv_acc"])
    e64 = per_body_rel(v["acc"], a64)
    print("PP FAST C1 per-body acc err vs FP32 ref", err_summary(e32), "vs FP64", err_summary(e64))
    assert e32.max() < 1e-5 and e64.max() < 1e-5
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


@pytest.mark.parametrize("form", ["plain", "compensated"])
def test_pp_plummer1m_subsample_per_body(sf, oracle64, form):
    """The N = 1,048,576 Plummer sphere (eps = 0.005) of the PP benchmark:
    per-particle force error on a seeded 8192-body subsample against the
    FP64 oracle over all j.  Plain (one FP32 sum over each j-split): every
    body within 1e-5 of the sum of its terms' magnitudes, median and p99 of
    |da|/|a| within 5e-6 and 1e-5; compensated: every body within 1e-6 of
    |a|."""
    from starflood_gb300.ics import plummer
    n = 1 << 20
    pos, vel, mas = plummer(n, seed=5)
    sub = np.sort(np.random.default_rng(8192).choice(n, 8192, replace=False)).astype(np.uint32)
    a64, _, mag = oracle64.pp_subset(pos.astype(np.float64), mas.astype(np.float64), sub, make_params(eps=0.005),
                                     with_mag=True)
    f = sf.FORM_PLAIN if form == "plain" else sf.FORM_COMPENSATED
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.005, form=f)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        v = slab_views(s.download(), n, 13)
    e = per_body_rel(v["acc"][sub], a64)
    e_mag = np.linalg.norm(v["acc"][sub].astype(np.float64) - a64, axis=1) / mag
    print("PP N=1M %s per-body acc err vs FP64" % form, err_summary(e), "over sum|terms|", err_summary(e_mag),
          "global", rel_l2(v["acc"][sub], a64))
    if form == "plain":
        # FP32 sums over 1M terms: within 1e-5 of the terms' magnitudes
        assert e_mag.max() < 1e-5 and np.median(e) < 5e-6 and np.quantile(e, 0.99) < 1e-5
    else:
        assert e.max() < 1e-6


@pytest.mark.parametrize("form", ["plain", "compensated"])
def test_energies_corrected_vs_fp64(sf, form):
    """sfgpu_energies_corrected after a step: T = sum v^2 / 2 (the kinetic
    term of the reference's m_i-scaled dynamics) and V = (1/2) sum_{i != j}
    -G m_i m_j / sqrt(r^2 + eps^2) (each pair once, no self term; the
    reference's V, simulation.c:449-451, has neither), against FP64 sums of
    the downloaded state."""
    from starflood_gb300.ics import uniform_ball
    n = 4096
    pos, vel, mas = uniform_ball(n, seed=31)
    f = sf.FORM_PLAIN if form == "plain" else sf.FORM_COMPENSATED
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=1e-3, form=f)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        s.step(0)
        T, V, E = s.energies_corrected()
        v = slab_views(s.download(), n, 13)
    x = v["pos"].astype(np.float64)
    m = v["mas"].astype(np.float64)
    T64 = 0.5 * (v["vel"].astype(np.float64) ** 2).sum()
    d = x[:, None, :] - x[None, :, :]
    inv = 1.0 / np.sqrt((d * d).sum(-1) + 0.01 ** 2)
    np.fill_diagonal(inv, 0.0)
    V64 = -0.5 * (m[:, None] * m[None, :] * inv).sum()
    assert abs(T - T64) <= 1e-7 * abs(T64), (T, T64)
    assert abs(V - V64) <= 1e-6 * abs(V64), (V, V64)
    assert abs(E - (T + V)) <= 1e-15 * abs(T - V)


@pytest.mark.parametrize("solver", ["pp", "tree"])
def test_compensated_trajectory_vs_fp64_oracle(sf, oracle64, solver):
    """20 KDK steps of the precision form (compensated forces, FP64
    positions and velocities) against 20 steps of the FP64 oracle, beside
    the plain FP32 form: per-body relative position and velocity errors."""
    from starflood_gb300.ics import uniform_ball
    n, steps = 4096, 20
    pos, vel, mas = uniform_ball(n, seed=17)
    tree = solver == "tree"
    op = make_params(dt=1e-3, eps=0.01, theta=0.5, use_tree=1 if tree else 0)
    osim, oslab, _ = oracle64.new_sim(n, op)
    ov = slab_views(oslab, n, 13)
    ov["pos"][:] = pos
    ov["vel"][:] = vel
    ov["mas"][:] = mas
    oracle64.sim_solv(op, osim, 0)
    for k in range(steps):
        oracle64.sim_step(op, osim, k)
    errs = {}
    for form in (sf.FORM_PLAIN, sf.FORM_COMPENSATED):
        p = sf.default_params(solver=sf.SOLVER_TREE if tree else sf.SOLVER_PP, eps=0.01, dt=1e-3, theta=0.5,
                              form=form)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            s.run(0, steps)
            v = slab_views(s.download(), n, 13)
        errs[form] = (per_body_rel(v["pos"], ov["pos"]), per_body_rel(v["vel"], ov["vel"]))
        print(solver, "form", form, "pos", err_summary(errs[form][0]), "vel", err_summary(errs[form][1]))
    ep, ev = errs[sf.FORM_COMPENSATED]
    pp_, pv_ = errs[sf.FORM_PLAIN]
    if not tree:
        assert ep.max() < 1e-7 and ev.max() < 1e-6
        assert np.median(ep) <= np.median(pp_) and np.median(ev) <= np.median(pv_)
    else:
        # the FP64 oracle builds its tree in FP64: opening decisions within
        # rounding of theta may differ, so the bound is on the bulk
        assert np.quantile(ep, 0.99) < 1e-6 and np.median(ev) < 1e-6
