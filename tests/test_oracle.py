"""The CPU oracle against the reference's golden vectors (CPU only).

The fixtures in tests/golden/ were produced by the unmodified Starflood
reference (tests/golden/make_golden.py).  The FP32 restatement must reproduce
them bit for bit; the FP64 build is pinned against the reference's FP64 PP.
"""
import numpy as np
import pytest

from conftest import golden
from oracle.pyoracle import make_params, slab_views


def _sim(oracle, params, d, dof=13):
    n = len(d["pos"])
    s, slab, nodes = oracle.new_sim(n, params)
    v = slab_views(slab, n, dof)
    v["pos"][:] = d["pos"]
    v["vel"][:] = d["vel"]
    v["mas"][:] = d["mas"]
    if "rad" in d:
        v["rad"][:] = d["rad"]
    return s, slab, nodes, v


def test_pcg4d_known_answer(oracle32):
    # pcg4d of (1,2,3,4): from the reference's rng.h, one round
    assert oracle32.pcg4d([1, 2, 3, 4]) == [908250390, 4044648920, 3775961919, 45698095]
    from starflood_gb300.ics import pcg4d
    a = pcg4d([1], [2], [3], [4])
    assert [int(x[0]) for x in a] == [908250390, 4044648920, 3775961919, 45698095]


def test_pp_uniform_c1_bitexact(oracle32):
    d = golden("pp_uniform_n4096_eps0.01_10steps.npz")
    p = make_params(dt=1e-3, eps=0.01)
    s, slab, _, v = _sim(oracle32, p, d)
    oracle32.sim_solv(p, s, 0)
    np.testing.assert_array_equal(v["acc"], d["solv_acc"])
    np.testing.assert_array_equal(v["pot"], d["solv_pot"])
    for k in range(int(d["steps"])):
        oracle32.sim_step(p, s, k)
    np.testing.assert_array_equal(slab, d["final_slab"])


def test_pp_plummer_eps005_bitexact(oracle32):
    d = golden("pp_plummer_n2048_eps0.005_2steps.npz")
    p = make_params(dt=1e-3, eps=0.005)
    s, slab, _, v = _sim(oracle32, p, d)
    oracle32.sim_solv(p, s, 0)
    np.testing.assert_array_equal(v["acc"], d["solv_acc"])
    for k in range(int(d["steps"])):
        oracle32.sim_step(p, s, k)
    np.testing.assert_array_equal(slab, d["final_slab"])


def test_pp_fp64_bitexact(oracle64):
    d = golden("pp64_uniform_n512_eps0.01.npz")
    p = make_params(eps=0.01)
    acc, pot = oracle64.pp(d["pos"].astype(np.float64), d["mas"].astype(np.float64), p)
    np.testing.assert_array_equal(acc, d["solv_acc"])
    np.testing.assert_array_equal(pot, d["solv_pot"])


def _check_tree(nodes, d):
    np.testing.assert_array_equal(nodes["parent"], d["tree_parent"])
    np.testing.assert_array_equal(nodes["bodies"], d["tree_bodies"])
    np.testing.assert_array_equal(nodes["branch"][:, :8], d["tree_branch"])
    np.testing.assert_array_equal(nodes["bounds"], d["tree_bounds"])
    np.testing.assert_array_equal(nodes["params"], d["tree_params"])


def test_tree_uniform_bitexact(oracle32):
    d = golden("tree_uniform_n4096_theta0.5_3steps.npz")
    p = make_params(dt=1e-3, eps=0.01, theta=0.5, use_tree=1)
    s, slab, nodes, v = _sim(oracle32, p, d)
    oracle32.sim_solv(p, s, 0)
    assert s.tree_status == 0
    assert s.num_nodes == len(d["tree_bodies"])
    _check_tree(nodes[: s.num_nodes], d)
    np.testing.assert_array_equal(v["acc"], d["solv_acc"])
    np.testing.assert_array_equal(v["pot"], d["solv_pot"])
    for k in range(int(d["steps"])):
        oracle32.sim_step(p, s, k)
    np.testing.assert_array_equal(slab, d["final_slab"])


def test_tree_lattice_ties_bitexact(oracle32):
    d = golden("tree_lattice_ties.npz")
    p = make_params(eps=0.01, theta=0.5, use_tree=1)
    st, nodes = oracle32.tree_build(d["pos"], d["mas"], d["bounds"], p)
    assert st == int(d["status"]) == 0
    _check_tree(nodes, d)
    acc, pot, _ = oracle32.walk(d["pos"], d["mas"], nodes, p)
    np.testing.assert_array_equal(acc, d["walk_acc"])
    np.testing.assert_array_equal(pot, d["walk_pot"])


def test_tree_depth_overflow_status(oracle32):
    d = golden("tree_depth_overflow.npz")
    st, _ = oracle32.tree_build(d["pos"], d["mas"], d["bounds"], make_params(use_tree=1))
    assert st == int(d["status"]) == -1


def test_sph_reference_bitexact(oracle32):
    d = golden("tree_sph_plummer_n1024_h0.05_2steps.npz")
    p = make_params(dt=5e-4, eps=0.01, theta=0.5, use_tree=1, use_sph=1)
    s, slab, nodes, v = _sim(oracle32, p, d, dof=16)
    oracle32.sim_solv(p, s, 0)
    np.testing.assert_array_equal(v["rho"], d["solv_rho"])
    np.testing.assert_array_equal(v["prs"], d["solv_prs"])
    np.testing.assert_array_equal(v["acc"], d["solv_acc"])
    for k in range(int(d["steps"])):
        oracle32.sim_step(p, s, k)
    np.testing.assert_array_equal(slab, d["final_slab"])


def test_fp32_vs_fp64_gap_pp(oracle32, oracle64):
    """The FP32 reference arithmetic sits within 1e-5 (global L2) of FP64."""
    d = golden("pp_uniform_n4096_eps0.01_10steps.npz")
    p = make_params(eps=0.01)
    a32, _ = oracle32.pp(d["pos"], d["mas"], p)
    a64, _ = oracle64.pp(d["pos"].astype(np.float64), d["mas"].astype(np.float64), p)
    err = np.linalg.norm(a32 - a64) / np.linalg.norm(a64)
    assert err < 1e-6
