"""Size-independent properties at the benchmark sizes, where the oracle is
too slow to run (GPU only).

* G enters the force and the potential as one final FP32 product, so the
  solve with G = 2 is bit-identical to twice the solve with G = 1 (scaling
  by a power of two is exact): PP at N = 1,048,576 and Barnes-Hut at
  N = 65,536, every form.
* The PP forces are pairwise antisymmetric, so the total momentum change
  sum_i m_i a_i vanishes up to FP32 rounding: |sum m a| <= 1e-5 sum |m a|.
* A Barnes-Hut step keeps the bodies' count and order: the slab's masses
  come back unchanged and every output is finite.
"""
import numpy as np
import pytest

from oracle.pyoracle import slab_views

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def _solve(sf, n, pos, vel, mas, **kw):
    p = sf.default_params(**kw)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        return slab_views(s.download(), n, 13)


@pytest.mark.parametrize("form", ["plain", "compensated"])
def test_pp_full_size_g_linear_and_momentum(sf, form):
    from starflood_gb300.ics import plummer
    n = 1 << 20
    pos, vel, mas = plummer(n, seed=5)
    f = sf.FORM_PLAIN if form == "plain" else sf.FORM_COMPENSATED
    v1 = _solve(sf, n, pos, vel, mas, solver=sf.SOLVER_PP, eps=0.005, G=1.0, form=f)
    v2 = _solve(sf, n, pos, vel, mas, solver=sf.SOLVER_PP, eps=0.005, G=2.0, form=f)
    assert np.array_equal(v2["acc"], 2.0 * v1["acc"])
    assert np.array_equal(v2["pot"], 2.0 * v1["pot"])
    ma = v1["acc"].astype(np.float64) * mas.astype(np.float64)[:, None]
    resid = np.abs(ma.sum(axis=0)).max()
    assert resid <= 1e-5 * np.abs(ma).sum(axis=0).max(), resid


@pytest.mark.parametrize("form", ["plain", "compensated"])
def test_bh_full_size_g_linear(sf, form):
    from starflood_gb300.ics import uniform_ball
    n = 65536
    pos, vel, mas = uniform_ball(n, seed=3)
    f = sf.FORM_PLAIN if form == "plain" else sf.FORM_COMPENSATED
    kw = dict(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, form=f)
    v1 = _solve(sf, n, pos, vel, mas, G=1.0, **kw)
    v2 = _solve(sf, n, pos, vel, mas, G=2.0, **kw)
    assert np.array_equal(v2["acc"], 2.0 * v1["acc"])
    assert np.array_equal(v2["pot"], 2.0 * v1["pot"])


def test_bh_full_size_steps_keep_bodies(sf):
    from starflood_gb300.ics import uniform_ball
    n = 65536
    pos, vel, mas = uniform_ball(n, seed=4)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, dt=1e-3)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        s.run(0, 20)
        v = slab_views(s.download(), n, 13)
    assert np.array_equal(v["mas"], mas)
    for k in ("pos", "vel", "acc", "pot", "ken", "pen"):
        assert np.all(np.isfinite(v[k])), k


@pytest.mark.parametrize("form", ["plain", "compensated"])
def test_momentum_diagnostics_vs_fp64_and_conserved_by_pp(sf, form):
    """sfgpu_momentum against numpy FP64 sums of the same state, then
    conserved over 20 PP steps (pairwise antisymmetric forces)."""
    from starflood_gb300.ics import plummer
    n = 16384
    pos, vel, mas = plummer(n, seed=11)
    m = mas.astype(np.float64)[:, None]
    x, v = pos.astype(np.float64), vel.astype(np.float64)
    P_ref = (m * v).sum(axis=0)
    L_ref = (m * np.cross(x, v)).sum(axis=0)
    scale_p = float((np.abs(m * v)).sum())
    scale_l = float((np.abs(m * np.cross(x, v))).sum())
    f = sf.FORM_PLAIN if form == "plain" else sf.FORM_COMPENSATED
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=1e-3, form=f)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        P0, L0 = s.momentum()
        assert np.abs(P0 - P_ref).max() <= 1e-12 * scale_p, (P0, P_ref)
        assert np.abs(L0 - L_ref).max() <= 1e-12 * scale_l, (L0, L_ref)
        s.solve(0)
        s.run(0, 20)
        P1, L1 = s.momentum()
    assert np.abs(P1 - P0).max() <= 1e-6 * scale_p, (P0, P1)
    assert np.abs(L1 - L0).max() <= 1e-5 * scale_l, (L0, L1)
