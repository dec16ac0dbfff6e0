"""The drop-in surface (include/starflood_compat.h) on the GPU: sim_init,
sim_find, sim_solv, sim_step, tree_init/tree_build, solve_* through the C
ABI with the reference's sim_t, checked against the golden fixtures."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def _fill(L, sf, sim, d, dof):
    n = sim.N
    buf = (C.c_float * (n * dof)).from_address(sim.mem)
    slab = np.frombuffer(buf, np.float32)
    v = sf.slab_views(slab, n, dof)
    # through sim_find, as a reference program would
    pos = (C.c_float * (3 * n)).from_address(L.sim_find(C.byref(sim), 0))
    np.frombuffer(pos, np.float32)[:] = d["pos"].ravel()
    v["vel"][:] = d["vel"]
    v["mas"][:] = d["mas"]
    if "rad" in d:
        v["rad"][:] = d["rad"]
    return slab


def test_compat_pp_exact_c1(sf):
    d = golden("pp_uniform_n4096_eps0.01_10steps.npz")
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=1e-3, math=sf.MATH_EXACT))
    sim = sf.SimT()
    assert L.sim_init(C.byref(sim), len(d["pos"])) == 0
    slab = _fill(L, sf, sim, d, 13)
    assert L.sim_solv(C.byref(sim)) == 0
    n = sim.N
    np.testing.assert_array_equal(slab[6 * n:9 * n].reshape(n, 3), d["solv_acc"])
    for k in range(int(d["steps"])):
        sim.step_number = k
        assert L.sim_step(C.byref(sim)) == 0
    np.testing.assert_array_equal(slab, d["final_slab"])
    assert L.sim_free(C.byref(sim)) == 0


def test_compat_tree_exact_steps(sf):
    d = golden("tree_uniform_n4096_theta0.5_3steps.npz")
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5,
                                          math=sf.MATH_EXACT, flags=sf.FLAG_EXPORT_TREE))
    sim = sf.SimT()
    assert L.sim_init(C.byref(sim), len(d["pos"])) == 0
    slab = _fill(L, sf, sim, d, 13)
    assert L.sim_solv(C.byref(sim)) == 0
    nn = len(d["tree_bodies"])
    assert sim.tree.num_nodes == nn
    nodes = np.ctypeslib.as_array(sim.tree.node, shape=(nn,))
    np.testing.assert_array_equal(nodes["bodies"], d["tree_bodies"])
    np.testing.assert_array_equal(nodes["branch"], d["tree_branch"])
    np.testing.assert_array_equal(nodes["params"], d["tree_params"])
    for k in range(int(d["steps"])):
        sim.step_number = k
        assert L.sim_step(C.byref(sim)) == 0
    np.testing.assert_array_equal(slab, d["final_slab"])
    L.sim_free(C.byref(sim))
    L.tree_free(C.byref(sim.tree))


def test_compat_tree_build_direct(sf):
    """tree_build(tree_t*, n, pos, mas) on caller arrays, reference node_t out."""
    d = golden("tree_lattice_ties.npz")
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, theta=0.5, math=sf.MATH_EXACT))
    tree = sf.TreeT()
    assert L.tree_init(C.byref(tree), 4096) == 0
    for a in range(6):
        tree.bounds[a] = float(d["bounds"][a])
    pos = np.ascontiguousarray(d["pos"], np.float32)
    mas = np.ascontiguousarray(d["mas"], np.float32)
    assert L.tree_build(C.byref(tree), len(pos), pos.ctypes.data, mas.ctypes.data) == 0
    nn = len(d["tree_bodies"])
    nodes = np.ctypeslib.as_array(tree.node, shape=(nn,))
    np.testing.assert_array_equal(nodes["parent"], d["tree_parent"])
    np.testing.assert_array_equal(nodes["branch"], d["tree_branch"])
    np.testing.assert_array_equal(nodes["bounds"], d["tree_bounds"])
    np.testing.assert_array_equal(nodes["params"], d["tree_params"])
    L.tree_free(C.byref(tree))


def test_compat_tree_build_depth_overflow(sf):
    d = golden("tree_depth_overflow.npz")
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_TREE, eps=0.01))
    tree = sf.TreeT()
    assert L.tree_init(C.byref(tree), 4096) == 0
    for a in range(6):
        tree.bounds[a] = float(d["bounds"][a])
    pos = np.ascontiguousarray(d["pos"], np.float32)
    mas = np.ascontiguousarray(d["mas"], np.float32)
    assert L.tree_build(C.byref(tree), len(pos), pos.ctypes.data, mas.ctypes.data) == -1  # tree.c:186-189
    L.tree_free(C.byref(tree))


def test_compat_sph_reference(sf, oracle32):
    d = golden("tree_sph_plummer_n1024_h0.05_2steps.npz")
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_TREE, sph=sf.SPH_REFERENCE, eps=0.01, dt=5e-4,
                                          theta=0.5))
    sim = sf.SimT()
    assert L.sim_init(C.byref(sim), len(d["pos"])) == 0
    slab = _fill(L, sf, sim, d, 16)
    assert L.sim_solv(C.byref(sim)) == 0
    n = sim.N
    v = sf.slab_views(slab, n, 16)
    rel = lambda a, b: np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b.astype(np.float64))
    assert rel(v["rho"], d["solv_rho"]) < 1e-5
    assert rel(v["acc"], d["solv_acc"]) < 1e-5
    L.sim_free(C.byref(sim))
    L.tree_free(C.byref(sim.tree))


def test_host_step_graph_matches_eager(sf):
    """sfgpu_host_step on a page-locked slab (one captured graph with the
    copies) and on a pageable slab (queued calls) give identical slabs, for
    steps and solve-only calls, and a changed slab pointer is followed."""
    from starflood_gb300.ics import uniform_ball
    L = sf.lib()
    n = 4096
    pos, vel, mas = uniform_ball(n, seed=31)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5)
    outs = []
    for pinned in (True, False):
        dof = sf.dof(p)
        slabs = [np.zeros(n * dof, np.float32) for _ in range(2)]
        for slab in slabs:
            v = sf.slab_views(slab, n, dof)
            v["pos"][:] = pos
            v["vel"][:] = vel
            v["mas"][:] = mas
            if pinned:
                sf.check(L.sfgpu_host_register(slab.ctypes.data, slab.nbytes), "register")
        st = (C.c_uint32 * 1)()
        with sf.Sim(n, p) as s:
            for k in range(4):
                slab = slabs[k // 2]  # the second pair of calls moves to another slab
                if k == 2:
                    slab[:] = slabs[0]
                sf.check(L.sfgpu_host_step(s.h, slab.ctypes.data, k, 1 if k == 0 else 0, st), "host_step")
                assert st[0] == 0
            outs.append(slabs[1].copy())
        if pinned:
            for slab in slabs:
                L.sfgpu_host_unregister(slab.ctypes.data)
    np.testing.assert_array_equal(outs[0], outs[1])


def test_sync_host_after_resident_steps(sf):
    """Steps queued on the handle behind a sim_t (sfgpu_run, one graph per
    step, no host copies) and then sfgpu_sync_host give the same slab as the
    same steps made by drop-in sim_step calls."""
    d = golden("tree_uniform_n4096_theta0.5_3steps.npz")
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5,
                                          math=sf.MATH_EXACT))
    slabs = []
    for resident in (False, True):
        sim = sf.SimT()
        assert L.sim_init(C.byref(sim), len(d["pos"])) == 0
        slab = _fill(L, sf, sim, d, 13)
        assert L.sim_solv(C.byref(sim)) == 0
        steps = int(d["steps"])
        if resident:
            h = L.sfgpu_compat_handle(C.byref(sim))
            assert h
            sf.check(sf.lib().sfgpu_run(h, 0, steps), "sfgpu_run")
            assert L.sfgpu_sync_host(C.byref(sim)) == 0
        else:
            for k in range(steps):
                sim.step_number = k
                assert L.sim_step(C.byref(sim)) == 0
        slabs.append(slab.copy())
        L.sim_free(C.byref(sim))
        L.tree_free(C.byref(sim.tree))
    np.testing.assert_array_equal(slabs[1], slabs[0])
    np.testing.assert_array_equal(slabs[0], d["final_slab"])
