"""Barnes-Hut tree build and walk on the GPU against the oracle (GPU only).

Bit-exact: root cube, octree keys / membership, node count, per-body
interaction and opening-test counts (the same cells are accepted), and with
EXACT arithmetic the forces, potentials and whole KDK steps.  FAST
arithmetic (FP64 centres of mass, rsqrt): within 1e-5 global relative L2 of
the reference."""
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


def test_tree_outside_and_nan_bodies(sf, oracle32):
    """Bodies outside the root cube (and NaN) are left out of the tree but
    still receive forces (tree.c:186-190)."""
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


@pytest.mark.parametrize("split,group", [(0, 0), (0, 8), (0, 16), (0, 32), (1, 0), (8, 0), (64, 0)])
@pytest.mark.parametrize("n,seed", [(65536, 2), (20000, 8)])
def test_tree_fast_large(sf, oracle32, n, seed, split, group):
    """FAST walks (group walk of 8, 16, 32 bodies; one thread per body; per
    body and root octant; 32-body groups split over 8 warps)."""
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
    a, pt, stats = oracle32.walk(pos, mas, nodes, op)
    np.testing.assert_array_equal(ni, stats[:, 0])
    assert rel_l2(v["acc"], a) < 1e-5
    assert rel_l2(v["pot"], pt) < 1e-5


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
