"""Barnes-Hut tree build and walk on the GPU against the oracle (GPU only).

Bit-exact: root cube, octree keys / membership, node count, per-body
interaction and opening-test counts (the same cells are accepted), and with
EXACT arithmetic the forces, potentials and whole KDK steps.  FAST
arithmetic (FP64 centres of mass, rsqrt): within 1e-5 global relative L2 of
the reference."""
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


def leaf_paths(nodes, n):
    """body -> octant path (list) and leaf depth, from an oracle node array."""
    path = {}

    def rec(v, pre):
        nd = nodes[v]
        if nd["bodies"] > 8:
            for o in range(8):
                rec(int(nd["branch"][o]), pre + [o])
        else:
            for k in range(int(nd["bodies"])):
                path[int(nd["branch"][k])] = pre
    rec(0, [])
    return path


def key_digits(key, depth):
    return [int((int(key) >> (3 * (15 - L))) & 7) for L in range(depth)]


def check_membership(sim, nodes, n):
    keys, idx, nin, _ = sim.tree_keys()
    paths = leaf_paths(nodes, n)
    assert nin == len(paths)
    for k in range(nin):
        p = int(idx[k])
        want = paths[p]
        assert key_digits(keys[k], len(want)) == want, (p, want)
    assert np.all(keys[nin:] >= (1 << 48))


def test_root_bounds_bitexact(sf, oracle32):
    from starflood_gb300.ics import uniform_ball, plummer
    for n, gen in ((4096, uniform_ball), (10000, plummer)):
        pos, vel, mas = gen(n, seed=21)
        p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            for step in (0, 1, 17, 12345):
                s.solve(step)
                _, _, _, b = s.tree_keys()
                np.testing.assert_array_equal(b, oracle32.root_bounds(pos, step))


@pytest.mark.parametrize("math", ["exact", "fast"])
def test_tree_uniform_golden(sf, oracle32, math):
    d = golden("tree_uniform_n4096_theta0.5_3steps.npz")
    n = len(d["pos"])
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5, flags=sf.FLAG_STATS,
                          math=sf.MATH_EXACT if math == "exact" else sf.MATH_FAST)
    with sf.Sim(n, p) as s:
        s.set_state(d["pos"], d["vel"], d["mas"])
        s.solve(0)
        assert s.status() == 0
        assert s.num_nodes() == len(d["tree_bodies"])
        v = slab_views(s.download(), n, 13)
        op = make_params(eps=0.01, theta=0.5, use_tree=1)
        st, nodes = oracle32.tree_build(d["pos"], d["mas"], oracle32.root_bounds(d["pos"], 0), op)
        check_membership(s, nodes, n)
        _, _, stats = oracle32.walk(d["pos"], d["mas"], nodes, op)
        ni, no = s.walk_stats()
        np.testing.assert_array_equal(ni, stats[:, 0])
        np.testing.assert_array_equal(no, stats[:, 1])
        if math == "exact":
            np.testing.assert_array_equal(v["acc"], d["solv_acc"])
            np.testing.assert_array_equal(v["pot"], d["solv_pot"])
        else:
            assert rel_l2(v["acc"], d["solv_acc"]) < 1e-5
            assert rel_l2(v["pot"], d["solv_pot"]) < 1e-5
        for k in range(int(d["steps"])):
            s.step(k)
        final = s.download()
        if math == "exact":
            np.testing.assert_array_equal(final, d["final_slab"])
        else:
            out = slab_views(final, n, 13)
            ref = slab_views(d["final_slab"], n, 13)
            assert rel_l2(out["pos"], ref["pos"]) < 1e-6
            assert rel_l2(out["acc"], ref["acc"]) < 1e-4


def test_tree_lattice_ties(sf, oracle32):
    """Bodies exactly on cell midplanes: strict vs non-strict octant rule."""
    d = golden("tree_lattice_ties.npz")
    n = len(d["pos"])
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, math=sf.MATH_EXACT, flags=sf.FLAG_STATS)
    with sf.Sim(n, p) as s:
        s.set_state(d["pos"], np.zeros((n, 3), np.float32), d["mas"])
        s.tree_build(d["bounds"])
        assert s.status() == 0
        assert s.num_nodes() == len(d["tree_bodies"])
        op = make_params(eps=0.01, theta=0.5, use_tree=1)
        st, nodes = oracle32.tree_build(d["pos"], d["mas"], d["bounds"], op)
        check_membership(s, nodes, n)
        s.gravity_tree()
        v = slab_views(s.download(), n, 13)
        _, _, stats = oracle32.walk(d["pos"], d["mas"], nodes, op)
        ni, no = s.walk_stats()
        np.testing.assert_array_equal(ni, stats[:, 0])
        np.testing.assert_array_equal(v["acc"], d["walk_acc"])
        np.testing.assert_array_equal(v["pot"], d["walk_pot"])


def test_tree_depth_overflow_flag(sf):
    d = golden("tree_depth_overflow.npz")
    n = len(d["pos"])
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01)
    with sf.Sim(n, p) as s:
        s.set_state(d["pos"], np.zeros((n, 3), np.float32), d["mas"])
        s.tree_build(d["bounds"])
        assert s.status() & sf.STATUS_TREE_DEPTH


def test_tree_node_overflow_flag(sf):
    from starflood_gb300.ics import uniform_ball
    n = 4096
    pos, vel, mas = uniform_ball(n, seed=4)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, nodes_max=200)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        assert s.status() & sf.STATUS_TREE_NODES


def test_tree_outside_bodies(sf, oracle32):
    """Bodies outside the root cube are left out of the tree but still
    receive forces (tree.c:141-146)."""
    from starflood_gb300.ics import uniform_ball
    n = 3000
    pos, vel, mas = uniform_ball(n, seed=6)
    pos[:5] *= 10.0
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, math=sf.MATH_EXACT)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(3)
        keys, idx, nin, b = s.tree_keys()
        v = slab_views(s.download(), n, 13)
    op = make_params(eps=0.01, theta=0.5, use_tree=1)
    bounds = oracle32.root_bounds(pos, 3)
    st, nodes = oracle32.tree_build(pos, mas, bounds, op)
    assert nin == nodes[0]["bodies"] < n
    a, pt, _ = oracle32.walk(pos, mas, nodes, op)
    np.testing.assert_array_equal(v["acc"], a)
    np.testing.assert_array_equal(v["pot"], pt)


@pytest.mark.parametrize("math", ["exact", "fast"])
def test_tree_nan_body(sf, oracle32, math):
    """A NaN coordinate is not skipped by the reference's root-cube test
    (every comparison with NaN is false, tree.c:141-146): the body is
    inserted, takes octant 0 at every level (tree.c:244-247, 282-285) and
    makes the centre of mass of every node on its path NaN.  Built in an
    explicit root cube (a NaN would also poison the mean radius), the GPU
    tree has the reference's node count and membership; EXACT forces and
    potentials are bit-identical (NaN where the reference has NaN); FAST
    has NaN exactly where the reference has NaN and the per-body
    interaction counts of every finite body.  The NaN reaches every body
    here: a leaf is never opened, so every walk meets the NaN body's leaf or
    one of its ancestors."""
    from starflood_gb300.ics import uniform_ball
    n = 3000
    pos, vel, mas = uniform_ball(n, seed=9)
    pos[11, 1] = np.nan
    bounds = np.array([-1.5, -1.5, -1.5, 1.5, 1.5, 1.5], np.float32)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, flags=sf.FLAG_STATS,
                          math=sf.MATH_EXACT if math == "exact" else sf.MATH_FAST)
    op = make_params(eps=0.01, theta=0.5, use_tree=1)
    st, nodes = oracle32.tree_build(pos, mas, bounds, op)
    assert st == 0 and nodes[0]["bodies"] == n
    a, pt, stats = oracle32.walk(pos, mas, nodes, op)
    # every body meets the NaN leaf (a leaf is never opened) or one of its
    # ancestors, so the reference's forces are all NaN
    assert np.isnan(a).all(axis=1).all()
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.tree_build(bounds)
        assert s.num_nodes() == len(nodes)
        check_membership(s, nodes, n)
        s.gravity_tree()
        v = slab_views(s.download(), n, 13)
        ni, no = s.walk_stats()
    if math == "exact":
        np.testing.assert_array_equal(v["acc"], a)
        np.testing.assert_array_equal(v["pot"], pt)
        np.testing.assert_array_equal(ni, stats[:, 0])
    else:
        np.testing.assert_array_equal(np.isnan(v["acc"]), np.isnan(a))
        np.testing.assert_array_equal(np.isnan(v["pot"]), np.isnan(pt))
        fin = np.isfinite(pos).all(1)
        np.testing.assert_array_equal(ni[fin], stats[fin, 0])


@pytest.mark.parametrize("split,group", [(0, 0), (0, 8), (0, 16), (0, 32), (1, 0), (8, 0), (64, 0)])
@pytest.mark.parametrize("n,seed", [(65536, 2), (20000, 8)])
def test_tree_fast_large(sf, oracle32, oracle64, n, seed, split, group):
    """FAST walks (group walk of 8, 16, 32 bodies; one thread per body; per
    body and root octant; 32-body groups split over 8 warps).  Per body:
    |a_i - a_ref,i| within 1e-5 of sum_k |F_k| (the magnitudes of its
    terms; |a_i| itself unless they cancel), or within twice the reference's
    own FP32 error (its insertion-order centre-of-mass sums, against the
    FP64 oracle on the same root cube) where that is larger; median and p99
    of |a_i - a_ref,i| / |a_i| below 1e-6 and 1e-5, or below twice the
    median and p99 of the reference's own FP32 error where those are larger
    (a Plummer sphere's dense core, where insertion-order FP32 centre-of-mass
    sums err by ~5e-6).  Potentials the same way, per body."""
    from starflood_gb300.ics import uniform_ball, plummer
    gen = uniform_ball if n == 65536 else plummer
    pos, vel, mas = gen(n, seed=seed)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, flags=sf.FLAG_STATS, walk_split=split,
                          walk_group=group)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(5)
        assert s.status() == 0
        v = slab_views(s.download(), n, 13)
        ni, no = s.walk_stats()
    op = make_params(eps=0.01, theta=0.5, use_tree=1)
    st, nodes = oracle32.tree_build(pos, mas, oracle32.root_bounds(pos, 5), op)
    a, pt, stats, mag = oracle32.walk(pos, mas, nodes, op, with_mag=True)
    np.testing.assert_array_equal(ni, stats[:, 0])
    assert rel_l2(v["acc"], a) < 1e-5
    assert rel_l2(v["pot"], pt) < 1e-5
    # per-particle bounds: on every body, not on the ensemble
    e = per_body_rel(v["acc"], a)
    ep = per_body_rel(v["pot"], pt)
    b = oracle32.root_bounds(pos, 5).astype(np.float64)
    op64 = make_params(eps=0.01, theta=0.5, use_tree=1)
    st64, nodes64 = oracle64.tree_build(pos.astype(np.float64), mas.astype(np.float64), b, op64)
    a64, pt64, _ = oracle64.walk(pos.astype(np.float64), mas.astype(np.float64), nodes64, op64)
    d_gpu = np.linalg.norm(v["acc"].astype(np.float64) - a, axis=1)
    d_ref = np.linalg.norm(a.astype(np.float64) - a64, axis=1)  # the reference's own FP32 error
    e_mag = d_gpu / mag
    print("BH FAST per-body acc err (split %d, group %d, n %d): |da|/|a|" % (split, group, n), err_summary(e),
          "|da|/sum|terms|", err_summary(e_mag), "ref vs FP64 /|a|", err_summary(d_ref / np.linalg.norm(a64, axis=1)),
          "pot:", err_summary(ep))
    # every body within 1e-5 of the sum of its terms' magnitudes (= |a_i|
    # where they do not cancel), or within twice the reference's own FP32
    # error where that is larger
    bad = d_gpu > np.maximum(1e-5 * mag, 2.0 * d_ref)
    assert not bad.any(), (np.nonzero(bad)[0], e[bad], e_mag[bad])
    e_ref = d_ref / np.linalg.norm(a64, axis=1)
    e_gpu64 = np.linalg.norm(v["acc"].astype(np.float64) - a64, axis=1) / np.linalg.norm(a64, axis=1)
    print("  GPU vs FP64 /|a|", err_summary(e_gpu64))
    assert np.median(e) < max(1e-6, 2.0 * np.median(e_ref))
    assert np.quantile(e, 0.99) < max(1e-5, 2.0 * np.quantile(e_ref, 0.99))
    # no further from the FP64 sums than the reference itself, in the bulk
    assert np.median(e_gpu64) < max(1e-6, 1.5 * np.median(e_ref))
    dp_gpu = np.abs(v["pot"].astype(np.float64) - pt)
    dp_ref = np.abs(pt.astype(np.float64) - pt64)
    assert not (dp_gpu > np.maximum(1e-5 * np.abs(pt), 2.0 * dp_ref)).any()


@pytest.mark.parametrize("leaf", [16, 4])
def test_tree_other_leaf_capacity(sf, oracle32, leaf):
    """Leaf capacities other than the reference's 8 (its node_t holds 8
    bodies, so these are checked against the restatement only): the same
    cells, per-body interaction counts identical, forces within 1e-5."""
    from starflood_gb300.ics import uniform_ball
    n = 20000
    pos, vel, mas = uniform_ball(n, seed=31)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, flags=sf.FLAG_STATS, leaf_cap=leaf)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(3)
        assert s.status() == 0
        v = slab_views(s.download(), n, 13)
        ni, no = s.walk_stats()
        nn = s.num_nodes()
    op = make_params(eps=0.01, theta=0.5, use_tree=1, leaf_cap=leaf)
    st, nodes = oracle32.tree_build(pos, mas, oracle32.root_bounds(pos, 3), op)
    assert st == 0 and nn == len(nodes)
    a, pt, stats = oracle32.walk(pos, mas, nodes, op)
    np.testing.assert_array_equal(ni, stats[:, 0])
    assert rel_l2(v["acc"], a) < 1e-5
    assert rel_l2(v["pot"], pt) < 1e-5


def test_tree_run_graph_matches_eager(sf):
    from starflood_gb300.ics import uniform_ball
    n = 8192
    pos, vel, mas = uniform_ball(n, seed=12)
    outs = []
    for flags in (sf.FLAG_NOGRAPH, 0):
        p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, flags=flags)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            s.run(0, 5)
            outs.append(s.download())
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("fixture", ["tree_uniform_n4096_theta0.5_3steps.npz", "tree_lattice_ties.npz"])
def test_tree_export_reference_numbering(sf, oracle32, fixture):
    """node_t array in the reference's numbering, bit-identical (EXACT)."""
    d = golden(fixture)
    n = len(d["pos"])
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, math=sf.MATH_EXACT)
    with sf.Sim(n, p) as s:
        s.set_state(d["pos"], d["vel"] if "vel" in d else np.zeros((n, 3), np.float32), d["mas"])
        if "bounds" in d:
            s.tree_build(d["bounds"])
        else:
            s.solve(0)
        t = s.tree_export()
    for k in ("parent", "bodies", "branch", "bounds", "params"):
        np.testing.assert_array_equal(t[k], d["tree_" + k], err_msg=k)


@pytest.mark.parametrize("group", [8, 16, 32])
def test_walk_totals_match_per_body_counts(sf, group):
    """The device totals of a walk without per-body statistics (what the
    benchmark's flop count uses) equal the sums of the per-body counts."""
    from starflood_gb300.ics import uniform_ball
    n = 20000
    pos, vel, mas = uniform_ball(n, seed=13)
    totals = []
    for flags in (0, sf.FLAG_STATS):
        p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, flags=flags, walk_group=group)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(3)
            s.walk_totals()  # reset by reading
            s.solve(3)
            ti, to = s.walk_totals()
            if flags:
                ni, no = s.walk_stats()
                assert (int(ni.sum()), int(no.sum())) == (ti, to)
            totals.append((ti, to))
    assert totals[0] == totals[1]


def test_tree_clustered_bucket_overflow(sf, oracle32):
    """60 % of 65,536 bodies in a sphere of radius 0.02: the sort's top-digit
    bucket holding the cluster exceeds one CTA's shared memory, so the tree
    keys go through the sort's cooperative fallback; membership, node count
    and per-body interaction counts must still be the reference's."""
    from starflood_gb300.ics import uniform_ball
    n = 65536
    pos, vel, mas = uniform_ball(n, seed=21)
    rng = np.random.default_rng(21)
    m = int(0.6 * n)
    d = rng.normal(size=(m, 3))
    d *= (0.02 * rng.random(m) ** (1.0 / 3.0) / np.linalg.norm(d, axis=1))[:, None]
    pos[:m] = (np.array([0.3, 0.3, 0.3]) + d).astype(np.float32)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, flags=sf.FLAG_STATS)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(2)
        assert s.status() == 0
        v = slab_views(s.download(), n, 13)
        op = make_params(eps=0.01, theta=0.5, use_tree=1)
        st, nodes = oracle32.tree_build(pos, mas, oracle32.root_bounds(pos, 2), op)
        assert s.num_nodes() == len(nodes)
        check_membership(s, nodes, n)
        a, pt, stats = oracle32.walk(pos, mas, nodes, op)
        ni, no = s.walk_stats()
        np.testing.assert_array_equal(ni, stats[:, 0])
        assert rel_l2(v["acc"], a) < 1e-5


@pytest.mark.parametrize("math", ["exact", "fast"])
def test_tree_step_energies(sf, oracle32, math):
    """The step's energy totals (computed in the walk's epilogue with FAST
    arithmetic, by the separate kick kernel with EXACT) against the
    reference's FP64 Kahan sums of ken and pen."""
    d = golden("tree_uniform_n4096_theta0.5_3steps.npz")
    n = len(d["pos"])
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5,
                          math=sf.MATH_EXACT if math == "exact" else sf.MATH_FAST)
    op = make_params(eps=0.01, theta=0.5, dt=1e-3, use_tree=1)
    osim, oslab, _ = oracle32.new_sim(n, op)
    ov = slab_views(oslab, n, 13)
    ov["pos"][:] = d["pos"]
    ov["vel"][:] = d["vel"]
    ov["mas"][:] = d["mas"]
    oracle32.sim_solv(op, osim, 0)
    with sf.Sim(n, p) as s:
        s.set_state(d["pos"], d["vel"], d["mas"])
        s.solve(0)
        for k in range(3):
            _, T, V = oracle32.sim_step(op, osim, k)
            s.step(k)
            Tg, Vg = s.energies()
            tol = 1e-13 if math == "exact" else 1e-5
            assert abs(Tg - T) <= tol * abs(T) and abs(Vg - V) <= tol * abs(V), (k, Tg, T, Vg, V)


def test_tree_fast_trajectory_uniform65536(sf, oracle32):
    """20 FAST KDK steps of the 65,536-body benchmark workload (uniform
    sphere, theta = 0.5, leaf 8, dt = 1e-3) against 20 reference steps of
    the FP32 restatement: positions, velocities and accelerations per body."""
    from starflood_gb300.ics import uniform_ball
    n, steps = 65536, 20
    pos, vel, mas = uniform_ball(n, seed=2024)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5)
    op = make_params(dt=1e-3, eps=0.01, theta=0.5, use_tree=1)
    osim, oslab, _ = oracle32.new_sim(n, op)
    ov = slab_views(oslab, n, 13)
    ov["pos"][:] = pos
    ov["vel"][:] = vel
    ov["mas"][:] = mas
    oracle32.sim_solv(op, osim, 0)
    for k in range(steps):
        oracle32.sim_step(op, osim, k)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        s.run(0, steps)
        v = slab_views(s.download(), n, 13)
        assert s.status() == 0
    ex = per_body_rel(v["pos"], ov["pos"])
    ev = per_body_rel(v["vel"], ov["vel"])
    ea = per_body_rel(v["acc"], ov["acc"])
    print("BH FAST 20-step trajectory per-body rel err: pos", err_summary(ex), "vel", err_summary(ev),
          "acc", err_summary(ea))
    assert ex.max() < 1e-5 and np.quantile(ex, 0.99) < 1e-6
    assert np.quantile(ev, 0.99) < 1e-5
    assert np.median(ea) < 1e-6 and np.quantile(ea, 0.99) < 1e-5


def test_status_ties_overflow(sf):
    """More bodies exactly on cell midplanes than the tie pass holds (1024):
    the build says so through SFGPU_STATUS_TIES instead of failing silently."""
    g = (np.arange(16, dtype=np.float32) - 8.0) / 8.0  # multiples of 1/8 in [-1, 0.875]
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    n = len(pos)
    mas = np.full(n, 1.0 / n, np.float32)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5)
    with sf.Sim(n, p) as s:
        s.set_state(pos, np.zeros_like(pos), mas)
        s.tree_build(np.array([-1, -1, -1, 1, 1, 1], np.float32))
        assert s.status() & sf.STATUS_TIES


@pytest.mark.parametrize("split,group", [(0, 16), (0, 32), (1, 0), (0, 0)])
def test_status_walk_limit(sf, split, group):
    """A walk stopped by its loop bound (walk_limit rounds per warp) returns
    and sets SFGPU_STATUS_WALK; the same simulation then walks normally."""
    from starflood_gb300.ics import uniform_ball
    n = 8192
    pos, vel, mas = uniform_ball(n, seed=14)
    for math in (sf.MATH_FAST, sf.MATH_EXACT):
        p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, walk_limit=3, walk_split=split,
                              walk_group=group, math=math)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            assert s.status() & sf.STATUS_WALK
            assert np.all(np.isfinite(slab_views(s.download(), n, 13)["acc"]))
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, walk_split=split, walk_group=group)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        assert s.status() == 0


def test_status_spin_withheld_lookback(sf):
    """The sort's decoupled look-back waits a bounded number of rounds: with
    one tile told not to publish, the tiles after it give up, set
    SFGPU_STATUS_SPIN and the call returns; the same entry point sorts
    correctly when no tile is withheld, before and after."""
    rng = np.random.default_rng(5)
    n = 300000
    keys = rng.integers(0, 1 << 40, n, dtype=np.uint64)
    want = np.argsort(keys & np.uint64(127), kind="stable")
    out, idx, st = sf.sort_withheld_check(keys)
    assert st == 0
    np.testing.assert_array_equal(idx, want)
    out, idx, st = sf.sort_withheld_check(keys, withheld_tile=3, spin_limit=4096)
    assert st & sf.STATUS_SPIN
    out, idx, st = sf.sort_withheld_check(keys)
    assert st == 0
    np.testing.assert_array_equal(idx, want)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_paired_decisions_match_scalar(sf, seed):
    """The walk's opening test for two cells per paired FP32 instruction and
    the SPH density pass's neighbour test for two candidates decide every
    case as the scalar FP32 expressions, on 4M random cases each placed
    within a few ulps of the decision boundary (where a fused product would
    flip some)."""
    walk_bad, sph_bad = sf.paired_check(1 << 22, seed)
    assert (walk_bad, sph_bad) == (0, 0)
