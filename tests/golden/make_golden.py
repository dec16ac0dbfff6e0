"""Write the golden fixtures in tests/golden/ from the compiled reference.

Runs the unmodified Starflood reference (built in place by oracle/build.py into
oracle/_ref/) on seeded inputs and stores inputs plus outputs as .npz files.
The fixtures pin the CPU restatement in oracle/ (tests/test_oracle.py) and,
through it, the GPU path.  Needs the reference sources; run from the repo root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle.pyoracle import Reference  # noqa: E402
from starflood_gb300.ics import plummer, uniform_ball  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def _sim_run(variant, pos, vel, mas, rad=None, steps=0):
    """Initial sim_solv (step 0) then `steps` sim_step calls, as main.c does."""
    ref = Reference(variant)
    n = len(pos)
    v = ref.init(n)
    v["pos"][:] = pos
    v["vel"][:] = vel
    v["mas"][:] = mas
    if rad is not None:
        v["rad"][:] = rad
    out = {}
    assert ref.solv(0) == 0
    out["solv_acc"] = v["acc"].copy()
    out["solv_pot"] = v["pot"].copy()
    if rad is not None:
        out["solv_rho"] = v["rho"].copy()
        out["solv_prs"] = v["prs"].copy()
    if ref.has_tree:
        t = ref.tree()
        for k in ("parent", "bodies", "branch", "bounds", "params"):
            out["tree_" + k] = t[k]
    for s in range(steps):
        assert ref.step(s) == 0
    if steps:
        out["final_slab"] = ref.slab.copy()
    ref.free()
    return out


def pp_c1():
    n = 4096
    pos, vel, mas = uniform_ball(n, seed=1)
    out = _sim_run("pp_e0.01", pos, vel, mas, steps=10)
    np.savez_compressed(os.path.join(OUT, "pp_uniform_n4096_eps0.01_10steps.npz"), pos=pos, vel=vel,
                        mas=mas, eps=0.01, dt=1e-3, steps=10, **out)


def pp_plummer():
    n = 2048
    pos, vel, mas = plummer(n, seed=4)
    out = _sim_run("pp_e0.005", pos, vel, mas, steps=2)
    np.savez_compressed(os.path.join(OUT, "pp_plummer_n2048_eps0.005_2steps.npz"), pos=pos, vel=vel,
                        mas=mas, eps=0.005, dt=1e-3, steps=2, **out)


def pp_fp64():
    n = 512
    pos, vel, mas = uniform_ball(n, seed=5)
    out = _sim_run("pp64_e0.01", pos.astype(np.float64), vel.astype(np.float64),
                   mas.astype(np.float64), steps=0)
    np.savez_compressed(os.path.join(OUT, "pp64_uniform_n512_eps0.01.npz"), pos=pos, vel=vel,
                        mas=mas, eps=0.01, **out)


def tree_uniform():
    n = 4096
    pos, vel, mas = uniform_ball(n, seed=2)
    out = _sim_run("tree_e0.01", pos, vel, mas, steps=3)
    np.savez_compressed(os.path.join(OUT, "tree_uniform_n4096_theta0.5_3steps.npz"), pos=pos, vel=vel,
                        mas=mas, eps=0.01, dt=1e-3, theta=0.5, steps=3, **out)


def tree_ties():
    """Lattice points sitting exactly on cell midpoints, in shuffled order, so
    that the strict/non-strict octant rule of tree.c:244-247 vs tree.c:282-285 and the
    closed-interval self test of gravity.c:473 are exercised."""
    g = np.arange(-4, 4, dtype=np.float32) * np.float32(0.25)
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(11)
    lat = lat[rng.permutation(len(lat))]
    extra = rng.uniform(-0.9, 0.9, size=(256, 3)).astype(np.float32)
    pos = np.concatenate([lat, extra]).astype(np.float32)
    n = len(pos)
    mas = np.full(n, np.float32(1.0) / np.float32(n), np.float32)
    ref = Reference("tree_e0.01")
    v = ref.init(n)
    v["pos"][:] = pos
    v["mas"][:] = mas
    bounds = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    status = ref.lib.refh_tree_build(n, bounds.ctypes.data)
    t = ref.tree()
    assert ref.lib.refh_walk() == 0
    out = {"tree_" + k: t[k] for k in ("parent", "bodies", "branch", "bounds", "params")}
    out["walk_acc"] = v["acc"].copy()
    out["walk_pot"] = v["pot"].copy()
    ref.free()
    np.savez_compressed(os.path.join(OUT, "tree_lattice_ties.npz"), pos=pos, mas=mas, bounds=bounds,
                        status=status, eps=0.01, theta=0.5, **out)


def tree_overflow():
    """Nine coincident bodies: the build must fail on the depth limit."""
    pos = np.concatenate([np.full((9, 3), 0.3, np.float32),
                          np.array([[0.1, -0.2, 0.4], [-0.5, 0.5, 0.0]], np.float32)])
    n = len(pos)
    mas = np.full(n, np.float32(1.0) / np.float32(n), np.float32)
    ref = Reference("tree_e0.01")
    v = ref.init(n)
    v["pos"][:] = pos
    v["mas"][:] = mas
    bounds = np.array([-1, -1, -1, 1, 1, 1], np.float32)
    status = ref.lib.refh_tree_build(n, bounds.ctypes.data)
    ref.free()
    np.savez_compressed(os.path.join(OUT, "tree_depth_overflow.npz"), pos=pos, mas=mas,
                        bounds=bounds, status=status)


def sph_reference():
    n = 1024
    pos, vel, mas = plummer(n, seed=3)
    rad = np.full(n, np.float32(0.05), np.float32)
    out = _sim_run("tree_sph_e0.01", pos, vel, mas, rad=rad, steps=2)
    np.savez_compressed(os.path.join(OUT, "tree_sph_plummer_n1024_h0.05_2steps.npz"), pos=pos, vel=vel,
                        mas=mas, rad=rad, eps=0.01, dt=5e-4, theta=0.5, steps=2, **out)


def raw_snapshot():
    """A raw snapshot (src/simulation_io.c:81-149) written by the reference
    after 2 PP steps of 64 bodies, with the slab it holds."""
    n = 64
    pos, vel, mas = uniform_ball(n, seed=9)
    ref = Reference("pp_e0.01")
    v = ref.init(n)
    v["pos"][:] = pos
    v["vel"][:] = vel
    v["mas"][:] = mas
    assert ref.solv(0) == 0
    for s in range(2):
        assert ref.step(s) == 0
    path = os.path.join(OUT, "raw_pp_n64_2steps.bin")
    assert ref.save_raw(path) == 0
    np.savez_compressed(os.path.join(OUT, "raw_pp_n64_2steps.npz"), slab=ref.slab.copy(), n=n, dof=ref.dof)
    ref.free()


def vis_splat():
    """vis_draw (src/visualization.c) of a 2048-body Plummer sphere after one
    PP solve (potentials set), step 7, 96 x 64 pixels, shipped settings
    (128 samples, exposure -1, ortho -1, autoscaling, tanh)."""
    n = 2048
    pos, vel, mas = plummer(n, seed=13)
    ref = Reference("pp_e0.01")
    v = ref.init(n)
    v["pos"][:] = pos
    v["vel"][:] = vel
    v["mas"][:] = mas
    assert ref.solv(0) == 0
    accum, render = ref.vis_draw(7, 96, 64)
    np.savez_compressed(os.path.join(OUT, "vis_plummer_n2048_96x64_step7.npz"), pos=v["pos"].copy(),
                        vel=v["vel"].copy(), pot=v["pot"].copy(), mas=mas, step=7, timestep=1e-3,
                        sizex=96, sizey=64, accum=accum, render=render)
    assert ref.vis_save_ppm(render, os.path.join(OUT, "vis_plummer_n2048_96x64_step7.ppm")) == 0
    ref.free()


def initcond_c1():
    """initcond_generate (src/initcond.c) of 4096 bodies, G = 1."""
    n = 4096
    ref = Reference("pp_e0.01")
    v = ref.init(n)
    assert ref.initcond() == 0
    np.savez_compressed(os.path.join(OUT, "initcond_n4096.npz"), pos=v["pos"].copy(), vel=v["vel"].copy(),
                        mas=v["mas"].copy(), G=1.0)
    ref.free()


def main():
    if not obuild.reference_available():
        raise SystemExit("the Starflood reference sources are needed to regenerate fixtures")
    obuild.build()
    for f in (pp_c1, pp_plummer, pp_fp64, tree_uniform, tree_ties, tree_overflow, sph_reference,
              raw_snapshot, vis_splat, initcond_c1):
        f()
        print("wrote", f.__name__)


if __name__ == "__main__":
    main()
