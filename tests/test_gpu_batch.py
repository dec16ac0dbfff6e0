"""Batched and adjoint forms on the GPU (GPU only).

Batched PP: every system's forces within 1e-5 global relative L2 of the
oracle PP on that system alone; K graph-replayed KDK steps within 1e-5 of the
oracle's K steps.  Adjoint: gradients of loss = sum_b mean_i |x_i|^2 at the
final step w.r.t. initial positions and velocities within 1e-4 of central
finite differences (h = 1e-3) of an FP64 forward integration, and of an FP64
reverse sweep."""
import numpy as np
import pytest

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


def ensemble(sizes, seed=0):
    from starflood_gb300.ics import uniform_ball
    P, V, M = [], [], []
    for k, n in enumerate(sizes):
        p, v, m = uniform_ball(int(n), seed=seed + 17 * k)
        P.append(p)
        V.append(v)
        M.append(m)
    return np.concatenate(P), np.concatenate(V), np.concatenate(M)


SIZES = [1, 2, 7, 130, 1000, 3000, 33, 4096, 257]


def test_batch_forces_per_system(sf, oracle32):
    pos, vel, mas = ensemble(SIZES)
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=1e-3)
    with sf.Batch(SIZES, p) as b:
        b.upload(pos, vel, mas)
        b.solve()
        _, _, acc, pot = b.download()
    off = np.concatenate([[0], np.cumsum(SIZES)])
    for k in range(len(SIZES)):
        s = slice(off[k], off[k + 1])
        a, pt = oracle32.pp(pos[s], mas[s], make_params(eps=0.01))
        if SIZES[k] > 1:
            assert rel_l2(acc[s], a) < 1e-5, k
        assert rel_l2(pot[s], pt) < 1e-6, k


def test_batch_run_graph_vs_oracle_steps(sf, oracle32):
    sizes = [500, 1200, 64, 2048]
    pos, vel, mas = ensemble(sizes, seed=3)
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=1e-3)
    K = 10
    with sf.Batch(sizes, p) as b:
        b.upload(pos, vel, mas)
        b.solve()
        b.run(K)
        b.sync()
        gpos, gvel, _, _ = b.download()
    off = np.concatenate([[0], np.cumsum(sizes)])
    op = make_params(dt=1e-3, eps=0.01)
    for k, n in enumerate(sizes):
        s = slice(off[k], off[k + 1])
        sim, slab, _ = oracle32.new_sim(n, op)
        v = slab_views(slab, n, 13)
        v["pos"][:] = pos[s]
        v["vel"][:] = vel[s]
        v["mas"][:] = mas[s]
        oracle32.sim_solv(op, sim, 0)
        for t in range(K):
            oracle32.sim_step(op, sim, t)
        assert rel_l2(gpos[s], v["pos"]) < 1e-6
        assert rel_l2(gvel[s], v["vel"]) < 1e-5


def test_batch_autotune_keeps_results(sf):
    sizes = [3000, 5000, 1024]
    pos, vel, mas = ensemble(sizes, seed=5)
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01)
    with sf.Batch(sizes, p) as b:
        b.upload(pos, vel, mas)
        b.solve()
        a0 = b.download()[2]
        cfg = b.autotune()
        assert 0 <= cfg < 5
        b.solve()
        a1 = b.download()[2]
    assert rel_l2(a1, a0) < 1e-6


# ---- FP64 reference trajectory and gradient (test infrastructure) ---------
def _acc64(x, m, eps, G=1.0):
    d = x[None, :, :] - x[:, None, :]          # d[i, j] = x_j - x_i
    r2 = (d * d).sum(-1) + eps * eps
    w = m[None, :] * r2 ** -1.5
    return G * m[:, None] * (d * w[..., None]).sum(1)   # reference semantics: m_i-scaled


def _loss64(pos, vel, mas, sizes, K, dt, eps):
    off = np.concatenate([[0], np.cumsum(sizes)])
    L = 0.0
    for k in range(len(sizes)):
        s = slice(off[k], off[k + 1])
        x, v, m = pos[s].copy(), vel[s].copy(), mas[s]
        a = _acc64(x, m, eps)
        for _ in range(K):
            v = v + 0.5 * dt * a
            x = x + dt * v
            a = _acc64(x, m, eps)
            v = v + 0.5 * dt * a
        L += (x * x).sum() / len(x)
    return L


def _vjp64(x, m, eps, abar, G=1.0):
    d = x[None, :, :] - x[:, None, :]
    r2 = (d * d).sum(-1) + eps * eps
    phi = r2 ** -1.5
    psi = r2 ** -2.5
    b = G * m[:, None] * abar
    w = m[:, None, None] * b[None, :, :] - m[None, :, None] * b[:, None, :]   # m_k b_j - m_j b_k
    dw = (d * w).sum(-1)
    return (phi[..., None] * w - 3.0 * psi[..., None] * d * dw[..., None]).sum(1)


def _grad64(pos, vel, mas, sizes, K, dt, eps):
    off = np.concatenate([[0], np.cumsum(sizes)])
    gp, gv = np.zeros_like(pos, dtype=np.float64), np.zeros_like(vel, dtype=np.float64)
    for k in range(len(sizes)):
        s = slice(off[k], off[k + 1])
        x, v, m = pos[s].astype(np.float64), vel[s].astype(np.float64), mas[s].astype(np.float64)
        xs = [x]
        a = _acc64(x, m, eps)
        for _ in range(K):
            v = v + 0.5 * dt * a
            x = x + dt * v
            a = _acc64(x, m, eps)
            v = v + 0.5 * dt * a
            xs.append(x)
        xb = 2.0 * x / len(x)
        vb = np.zeros_like(xb)
        for t in range(K - 1, -1, -1):
            vb = vb + dt * xb
            c = dt if t > 0 else 0.5 * dt
            xb = xb + _vjp64(xs[t], m, eps, c * vb)
        gp[s], gv[s] = xb, vb
    return gp, gv


@pytest.mark.parametrize("checkpoint", [20, 7])
def test_adjoint_vs_finite_differences(sf, checkpoint):
    sizes = [64, 100, 37, 150]
    pos, vel, mas = ensemble(sizes, seed=11)
    K, dt, eps = 40, 1e-3, 0.01
    p = sf.default_params(solver=sf.SOLVER_PP, eps=eps, dt=dt)
    with sf.Batch(sizes, p) as b:
        b.upload(pos, vel, mas)
        loss, gp, gv = b.grad(K, checkpoint)
        fpos, _, _, _ = b.download()
    L64 = _loss64(pos.astype(np.float64), vel.astype(np.float64), mas.astype(np.float64), sizes, K, dt, eps)
    assert abs(loss - L64) < 1e-5 * abs(L64)
    gp64, gv64 = _grad64(pos, vel, mas, sizes, K, dt, eps)
    assert rel_l2(gp, gp64) < 1e-4
    assert rel_l2(gv, gv64) < 1e-4
    # central finite differences, h = 1e-3, FP64 forward
    rng = np.random.default_rng(1)
    h = 1e-3
    p64, v64, m64 = pos.astype(np.float64), vel.astype(np.float64), mas.astype(np.float64)
    gscale = max(np.abs(gp64).max(), np.abs(gv64).max())
    for idx in rng.choice(len(pos) * 3, 6, replace=False):
        i, c = divmod(int(idx), 3)
        for which, g in (("pos", gp), ("vel", gv)):
            a, bb = p64.copy(), v64.copy()
            arr = a if which == "pos" else bb
            arr[i, c] += h
            lp = _loss64(a, bb, m64, sizes, K, dt, eps)
            arr[i, c] -= 2 * h
            lm = _loss64(a, bb, m64, sizes, K, dt, eps)
            fd = (lp - lm) / (2 * h)
            assert abs(g[i, c] - fd) <= 1e-4 * gscale, (which, i, c, g[i, c], fd)
    # the batch is left at the final state
    assert np.all(np.isfinite(fpos))


def test_adjoint_c5_ensemble_vs_finite_differences(sf, oracle64):
    """The batched-adjoint benchmark ensemble itself: 256 uniform spheres
    with N log-uniform in [1024, 32768], 200 KDK steps at dt = 1e-3,
    checkpoints every 20 steps.  On its two smallest systems, the gradient of
    one position and one velocity coordinate each is checked against central
    finite differences (h = 1e-3) of an FP64 forward integration of that
    system (the oracle's FP64 build; the systems are independent, so the
    ensemble loss changes only through that system's mean r^2)."""
    from starflood_gb300.ics import log_uniform_sizes, uniform_ball
    sizes = [int(x) for x in log_uniform_sizes(256, 1024, 32768, seed=7)]
    P, V, M = [], [], []
    for k, n in enumerate(sizes):
        a, b_, c = uniform_ball(n, seed=1000 + k)
        P.append(a)
        V.append(b_)
        M.append(c)
    pos, vel, mas = np.concatenate(P), np.concatenate(V), np.concatenate(M)
    off = np.concatenate([[0], np.cumsum(sizes)])
    K, ckpt, dt, eps, h = 200, 20, 1e-3, 0.01, 1e-3
    p = sf.default_params(solver=sf.SOLVER_PP, eps=eps, dt=dt)
    with sf.Batch(sizes, p) as b:
        b.upload(pos, vel, mas)
        loss, gp, gv = b.grad(K, ckpt)
    assert np.isfinite(loss) and np.all(np.isfinite(gp)) and np.all(np.isfinite(gv))
    op = make_params(dt=dt, eps=eps)

    def loss64(x0, v0, m):
        n = len(m)
        sim, slab, _ = oracle64.new_sim(n, op)
        sv = slab_views(slab, n, 13)
        sv["pos"][:] = x0
        sv["vel"][:] = v0
        sv["mas"][:] = m
        oracle64.sim_solv(op, sim, 0)
        for t in range(K):
            oracle64.sim_step(op, sim, t)
        return float((sv["pos"] ** 2).sum() / n)

    rng = np.random.default_rng(2)
    for k in np.argsort(sizes)[:2]:
        s = slice(off[k], off[k + 1])
        x0, v0, m = pos[s].astype(np.float64), vel[s].astype(np.float64), mas[s].astype(np.float64)
        gscale = max(np.abs(gp[s]).max(), np.abs(gv[s]).max())
        i, c = int(rng.integers(sizes[k])), int(rng.integers(3))
        for which, g in (("pos", gp[s]), ("vel", gv[s])):
            xp, vp = x0.copy(), v0.copy()
            arr = xp if which == "pos" else vp
            arr[i, c] += h
            lp = loss64(xp, vp, m)
            arr[i, c] -= 2 * h
            lm = loss64(xp, vp, m)
            fd = (lp - lm) / (2 * h)
            print("C5 adjoint system %d (N=%d) %s[%d,%d]: %.9g fd %.9g" % (k, sizes[k], which, i, c, g[i, c], fd))
            assert abs(g[i, c] - fd) <= 1e-4 * gscale, (k, which, i, c, g[i, c], fd)
