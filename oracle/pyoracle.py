"""ctypes bindings for the test oracle (TEST INFRASTRUCTURE ONLY).

``Oracle`` wraps ``liboracle_f32.so`` / ``liboracle_f64.so`` (the C
restatement, see ``oracle/oracle.c``); ``Reference`` wraps the compiled
Starflood reference in ``oracle/_ref`` (present only where the reference
sources were available at build time).  Arrays use the reference layout:
positions, velocities and accelerations are (N, 3) row-major.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

u32p = C.POINTER(C.c_uint32)


class Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("eps", C.c_double), ("G", C.c_double),
                ("theta", C.c_double), ("use_tree", C.c_int32), ("use_sph", C.c_int32),
                ("kahan", C.c_int32), ("leaf_cap", C.c_uint32), ("depth_max", C.c_uint32),
                ("nodes_max", C.c_uint32)]


def make_params(dt=1e-3, eps=0.01, G=1.0, theta=0.5, use_tree=0, use_sph=0, kahan=1,
                leaf_cap=8, depth_max=16, nodes_max=262144) -> Params:
    return Params(dt, eps, G, theta, use_tree, use_sph, kahan, leaf_cap, depth_max, nodes_max)


def node_dtype(real):
    return np.dtype([("parent", np.uint32), ("bodies", np.uint32), ("branch", np.uint32, (16,)),
                     ("bounds", real, (6,)), ("params", real, (4,))], align=True)


class Oracle:
    """The C restatement at one precision ('f32' reference arithmetic, 'f64')."""

    def __init__(self, precision: str = "f32"):
        path = os.path.join(HERE, "liboracle_%s.so" % precision)
        if not os.path.exists(path):
            from oracle import build as _b
            _b.build_oracle()
        self.lib = C.CDLL(path)
        self.real = np.float32 if precision == "f32" else np.float64
        self.creal = C.c_float if precision == "f32" else C.c_double
        self.node_dtype = node_dtype(self.real)
        rp = C.POINTER(self.creal)
        self._rp = rp
        L = self.lib
        L.orc_real_size.restype = C.c_int
        assert L.orc_real_size() == np.dtype(self.real).itemsize
        L.orc_mean_radius.restype = C.c_double
        L.orc_mean_radius.argtypes = [C.c_uint32, rp]
        L.orc_root_bounds.argtypes = [C.c_uint32, rp, C.c_uint32, rp]
        L.orc_tree_build.restype = C.c_int
        L.orc_tree_build.argtypes = [C.POINTER(Params), C.c_uint32, rp, rp, rp, C.c_void_p, u32p]
        L.orc_gravity_tree.argtypes = [C.POINTER(Params), C.c_uint32, rp, rp, C.c_void_p, rp, rp, u32p]
        L.orc_gravity_pp.argtypes = [C.POINTER(Params), C.c_uint32, rp, rp, rp, rp]
        L.orc_sph_reference.argtypes = [C.POINTER(Params), C.c_uint32, rp, rp, rp, rp, rp, rp, u32p]
        L.orc_pcg4d.argtypes = [u32p]
        L.orc_sim_dof.restype = C.c_uint32
        L.orc_sim_dof.argtypes = [C.POINTER(Params)]
        L.orc_threads.restype = C.c_int
        fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
        L.orc_sph_cubic.argtypes = [C.c_uint32, fp, fp, fp, fp, fp, C.c_double, C.c_double, C.c_double,
                                    dp, dp, dp, dp, u32p]
        L.orc_initcond.argtypes = [C.c_uint32, C.c_double, fp, fp, fp, fp]
        L.orc_vis_draw.argtypes = [C.c_uint32, fp, fp, fp, C.c_uint32, C.c_double, C.c_uint32, C.c_uint32,
                                   C.c_uint32, C.c_double, C.c_double, C.c_int, C.c_int,
                                   C.POINTER(C.c_int32), fp]
        L.orc_grid_deposit.argtypes = [C.c_uint32, fp, fp, C.c_uint32, fp, C.c_uint32, C.c_uint32,
                                       C.POINTER(C.c_int32), fp]
        L.orc_grid_stencil.argtypes = [C.c_uint32, fp, fp, C.c_double, fp]
        L.orc_grid_solve_fft.argtypes = [C.c_uint32, fp, fp, C.c_double, fp, dp]

        class Sim(C.Structure):
            _fields_ = [("step_number", C.c_uint32), ("N", C.c_uint32), ("mem", C.c_void_p),
                        ("nodes", C.c_void_p), ("num_nodes", C.c_uint32), ("tree_status", C.c_int32),
                        ("bounds", self.creal * 6)]
        self.Sim = Sim
        L.orc_sim_solv.restype = C.c_int
        L.orc_sim_solv.argtypes = [C.POINTER(Params), C.POINTER(Sim)]
        L.orc_sim_step.restype = C.c_int
        L.orc_sim_step.argtypes = [C.POINTER(Params), C.POINTER(Sim), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]

    def threads(self) -> int:
        return int(self.lib.orc_threads())

    def _arr(self, a, n_cols=None):
        a = np.ascontiguousarray(a, dtype=self.real)
        return a, a.ctypes.data_as(self._rp)

    def pcg4d(self, s):
        a = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in s])
        self.lib.orc_pcg4d(a)
        return [a[i] for i in range(4)]

    def mean_radius(self, pos):
        pos, pp = self._arr(pos)
        return float(self.lib.orc_mean_radius(len(pos), pp))

    def root_bounds(self, pos, step):
        pos, pp = self._arr(pos)
        out = np.zeros(6, self.real)
        self.lib.orc_root_bounds(len(pos), pp, step, out.ctypes.data_as(self._rp))
        return out

    def tree_build(self, pos, mas, bounds, params: Params | None = None):
        p = params or make_params(use_tree=1)
        pos, pp = self._arr(pos)
        mas, mp = self._arr(mas)
        b, bp = self._arr(bounds)
        nodes = np.zeros(p.nodes_max, self.node_dtype)
        nn = C.c_uint32(0)
        st = self.lib.orc_tree_build(C.byref(p), len(pos), pp, mp, bp,
                                     nodes.ctypes.data_as(C.c_void_p), C.byref(nn))
        return st, nodes[: nn.value].copy() if st == 0 else nodes[: nn.value].copy()

    def walk(self, pos, mas, nodes, params: Params | None = None, with_mag=False):
        """(acc, pot, stats), and with with_mag the per-body sum of the
        terms' magnitudes G m_i sum |F|."""
        p = params or make_params(use_tree=1)
        pos, pp = self._arr(pos)
        mas, mp = self._arr(mas)
        n = len(pos)
        full = np.zeros(max(p.nodes_max, len(nodes)), self.node_dtype)
        full[: len(nodes)] = nodes
        acc = np.zeros((n, 3), self.real)
        pot = np.zeros(n, self.real)
        stats = np.zeros((n, 2), np.uint32)
        if with_mag:
            mag = np.zeros(n, self.real)
            self.lib.orc_gravity_tree_mag(C.byref(p), n, pp, mp, full.ctypes.data_as(C.c_void_p),
                                          acc.ctypes.data_as(self._rp), pot.ctypes.data_as(self._rp),
                                          stats.ctypes.data_as(u32p), mag.ctypes.data_as(self._rp))
            return acc, pot, stats, mag
        self.lib.orc_gravity_tree(C.byref(p), n, pp, mp, full.ctypes.data_as(C.c_void_p),
                                  acc.ctypes.data_as(self._rp), pot.ctypes.data_as(self._rp),
                                  stats.ctypes.data_as(u32p))
        return acc, pot, stats

    def pp(self, pos, mas, params: Params | None = None):
        p = params or make_params()
        pos, pp = self._arr(pos)
        mas, mp = self._arr(mas)
        n = len(pos)
        acc = np.zeros((n, 3), self.real)
        pot = np.zeros(n, self.real)
        self.lib.orc_gravity_pp(C.byref(p), n, pp, mp, acc.ctypes.data_as(self._rp),
                                pot.ctypes.data_as(self._rp))
        return acc, pot

    def pp_subset(self, pos, mas, idx, params: Params | None = None, with_mag=False):
        """orc_gravity_pp for the bodies idx only, over all bodies: (acc,
        pot), and with with_mag the per-body G m_i sum_j |F_ij|."""
        p = params or make_params()
        pos, pp = self._arr(pos)
        mas, mp = self._arr(mas)
        idx = np.ascontiguousarray(idx, np.uint32)
        acc = np.zeros((len(idx), 3), self.real)
        pot = np.zeros(len(idx), self.real)
        mag = np.zeros(len(idx), self.real)
        self.lib.orc_gravity_pp_subset(C.byref(p), len(pos), pp, mp, len(idx), idx.ctypes.data_as(u32p),
                                       acc.ctypes.data_as(self._rp), pot.ctypes.data_as(self._rp),
                                       mag.ctypes.data_as(self._rp) if with_mag else None)
        return (acc, pot, mag) if with_mag else (acc, pot)

    def sph_reference(self, pos, mas, rad, acc_in=None, params: Params | None = None):
        p = params or make_params(use_sph=1)
        pos, pp = self._arr(pos)
        mas, mp = self._arr(mas)
        rad, rp = self._arr(rad)
        n = len(pos)
        acc = np.zeros((n, 3), self.real) if acc_in is None else np.array(acc_in, self.real)
        rho = np.zeros(n, self.real)
        prs = np.zeros(n, self.real)
        nbr = np.zeros(n, np.uint32)
        self.lib.orc_sph_reference(C.byref(p), n, pp, mp, rp, rho.ctypes.data_as(self._rp),
                                   prs.ctypes.data_as(self._rp), acc.ctypes.data_as(self._rp),
                                   nbr.ctypes.data_as(u32p))
        return rho, prs, acc, nbr

    def initcond(self, n, G=1.0, sph=False):
        """initcond_generate (src/initcond.c:11-255): (pos (n,3), vel (n,3), mas, rad or None)."""
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        mas = np.zeros(n, np.float32)
        rad = np.zeros(n, np.float32) if sph else None
        fp = C.POINTER(C.c_float)
        self.lib.orc_initcond(n, G, pos.ctypes.data_as(fp), vel.ctypes.data_as(fp), mas.ctypes.data_as(fp),
                              rad.ctypes.data_as(fp) if sph else None)
        return pos, vel, mas, rad

    def vis_draw(self, pos, vel, pot, step, timestep, sizex, sizey, samples=128, exposure=-1.0,
                 ortho_scale=-1.0, autoscale=1, tonemap=1):
        """vis_draw (src/visualization.c:258-740): (accum int32 (sizey, sizex, 4),
        render float32 (sizey, sizex, 4))."""
        f = lambda a: np.ascontiguousarray(a, np.float32)
        pos, vel, pot = f(pos), f(vel), f(pot)
        accum = np.zeros((sizey, sizex, 4), np.int32)
        render = np.zeros((sizey, sizex, 4), np.float32)
        fp = C.POINTER(C.c_float)
        self.lib.orc_vis_draw(len(pos), pos.ctypes.data_as(fp), vel.ctypes.data_as(fp), pot.ctypes.data_as(fp),
                              step, timestep, sizex, sizey, samples, exposure, ortho_scale, autoscale, tonemap,
                              accum.ctypes.data_as(C.POINTER(C.c_int32)), render.ctypes.data_as(fp))
        return accum, render

    def grid_deposit(self, side, bmin, bmax, pos, step, samples=128):
        """The particle-mesh deposit (src/gravity.c:116-230): (accum int32
        (side, side, side), poten float32 of the same shape), index [z, y, x]."""
        fp = C.POINTER(C.c_float)
        pos = np.ascontiguousarray(pos, np.float32)
        lo, hi = np.asarray(bmin, np.float32), np.asarray(bmax, np.float32)
        accum = np.zeros((side, side, side), np.int32)
        poten = np.zeros((side, side, side), np.float32)
        self.lib.orc_grid_deposit(side, lo.ctypes.data_as(fp), hi.ctypes.data_as(fp), len(pos),
                                  pos.ctypes.data_as(fp), step, samples,
                                  accum.ctypes.data_as(C.POINTER(C.c_int32)), poten.ctypes.data_as(fp))
        return accum, poten

    def grid_stencil(self, side, bmin, bmax, G=1.0):
        """grid.c:281-315: the FP32 stencil -G/|x| at the cell corners, [z, y, x]."""
        fp = C.POINTER(C.c_float)
        lo, hi = np.asarray(bmin, np.float32), np.asarray(bmax, np.float32)
        out = np.zeros((side, side, side), np.float32)
        self.lib.orc_grid_stencil(side, lo.ctypes.data_as(fp), hi.ctypes.data_as(fp), G, out.ctypes.data_as(fp))
        return out

    def grid_solve_fft(self, side, bmin, bmax, samp, G=1.0):
        """grid_solve_fft (src/grid.c:197-536) in FP64 by the DFT definition."""
        fp = C.POINTER(C.c_float)
        lo, hi = np.asarray(bmin, np.float32), np.asarray(bmax, np.float32)
        samp = np.ascontiguousarray(samp, np.float32)
        out = np.zeros((side, side, side), np.float64)
        self.lib.orc_grid_solve_fft(side, lo.ctypes.data_as(fp), hi.ctypes.data_as(fp), G,
                                    samp.ctypes.data_as(fp), out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def sph_cubic(self, pos, vel, mas, rad, u, gamma=5.0 / 3.0, alpha=1.0, beta=2.0):
        """Cubic-spline SPH (FP64 physics, FP32 neighbour decisions)."""
        f = lambda a: np.ascontiguousarray(a, np.float32)
        pos, vel, mas, rad, u = f(pos), f(vel), f(mas), f(rad), f(u)
        n = len(pos)
        rho, prs, dudt = np.zeros(n), np.zeros(n), np.zeros(n)
        acc = np.zeros((n, 3))
        nbr = np.zeros(n, np.uint32)
        fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
        self.lib.orc_sph_cubic(n, pos.ctypes.data_as(fp), vel.ctypes.data_as(fp), mas.ctypes.data_as(fp),
                               rad.ctypes.data_as(fp), u.ctypes.data_as(fp), gamma, alpha, beta,
                               rho.ctypes.data_as(dp), prs.ctypes.data_as(dp), acc.ctypes.data_as(dp),
                               dudt.ctypes.data_as(dp), nbr.ctypes.data_as(u32p))
        return rho, prs, acc, dudt, nbr

    # --- slab-level simulation (simulation.c) -------------------------------
    def new_sim(self, n, params: Params):
        dof = int(self.lib.orc_sim_dof(C.byref(params)))
        slab = np.zeros(n * dof, self.real)
        nodes = np.zeros(params.nodes_max if params.use_tree else 1, self.node_dtype)
        s = self.Sim()
        s.N = n
        s.mem = slab.ctypes.data
        s.nodes = nodes.ctypes.data
        # the struct holds raw pointers: keep the arrays alive as long as it
        # lives, even when a caller drops the returned arrays
        s._arrays = (slab, nodes)
        return s, slab, nodes

    def sim_solv(self, params, sim, step):
        sim.step_number = step
        return self.lib.orc_sim_solv(C.byref(params), C.byref(sim))

    def sim_step(self, params, sim, step):
        sim.step_number = step
        T = C.c_double()
        V = C.c_double()
        rc = self.lib.orc_sim_step(C.byref(params), C.byref(sim), C.byref(T), C.byref(V))
        return rc, T.value, V.value


def slab_views(slab, n, dof):
    """Views of the reference slab (simulation.h:17-51)."""
    v = {"pos": slab[0: 3 * n].reshape(n, 3), "vel": slab[3 * n: 6 * n].reshape(n, 3),
         "acc": slab[6 * n: 9 * n].reshape(n, 3), "mas": slab[9 * n: 10 * n],
         "pot": slab[10 * n: 11 * n], "ken": slab[11 * n: 12 * n], "pen": slab[12 * n: 13 * n]}
    if dof >= 16:
        v["rad"] = slab[13 * n: 14 * n]
        v["rho"] = slab[14 * n: 15 * n]
        v["prs"] = slab[15 * n: 16 * n]
    return v


class Reference:
    """The compiled Starflood reference (one configuration per library)."""

    def __init__(self, variant: str):
        path = os.path.join(HERE, "_ref", "libref_%s.so" % variant)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.variant = variant
        self.lib = C.CDLL(path)
        L = self.lib
        L.refh_real_size.restype = C.c_int
        self.real = np.float32 if L.refh_real_size() == 4 else np.float64
        L.refh_dof.restype = C.c_int
        L.refh_has_tree.restype = C.c_int
        self.dof = int(L.refh_dof())
        self.has_tree = bool(L.refh_has_tree())
        L.refh_init.argtypes = [C.c_uint]
        L.refh_init.restype = C.c_int
        L.refh_mem.restype = C.c_void_p
        L.refh_solv.argtypes = [C.c_uint]
        L.refh_step.argtypes = [C.c_uint]
        if self.has_tree:
            L.refh_tree_nodes.restype = C.c_uint
            L.refh_tree_dump.restype = C.c_uint
            L.refh_tree_dump.argtypes = [C.c_uint, u32p, u32p, u32p, C.c_void_p, C.c_void_p]
            L.refh_tree_bounds.argtypes = [C.c_void_p]
            L.refh_tree_build.argtypes = [C.c_uint, C.c_void_p]
        self.n = 0

    def init(self, n):
        assert self.lib.refh_init(n) == 0
        self.n = n
        ptr = self.lib.refh_mem()
        buf = (C.c_char * (n * self.dof * np.dtype(self.real).itemsize)).from_address(ptr)
        self.slab = np.frombuffer(buf, dtype=self.real)
        self.views = slab_views(self.slab, n, self.dof)
        return self.views

    def solv(self, step):
        return self.lib.refh_solv(step)

    def step(self, step):
        return self.lib.refh_step(step)

    def tree(self):
        cnt = int(self.lib.refh_tree_nodes())
        parent = np.zeros(cnt, np.uint32)
        bodies = np.zeros(cnt, np.uint32)
        branch = np.zeros((cnt, 8), np.uint32)
        bounds = np.zeros((cnt, 6), self.real)
        params = np.zeros((cnt, 4), self.real)
        self.lib.refh_tree_dump(cnt, parent.ctypes.data_as(u32p), bodies.ctypes.data_as(u32p),
                                branch.ctypes.data_as(u32p), bounds.ctypes.data, params.ctypes.data)
        tb = np.zeros(6, self.real)
        self.lib.refh_tree_bounds(tb.ctypes.data)
        return dict(parent=parent, bodies=bodies, branch=branch, bounds=bounds, params=params,
                    root_bounds=tb)

    def vis_draw(self, step, sizex, sizey):
        """src/visualization.c vis_draw of the current state (FP32 variants):
        (accum int32 (sizey, sizex, 4), render float32 (sizey, sizex, 4))."""
        accum = np.zeros((sizey, sizex, 4), np.int32)
        render = np.zeros((sizey, sizex, 4), np.float32)
        assert self.lib.refh_vis_draw(step, sizex, sizey, accum.ctypes.data, render.ctypes.data) == 0
        return accum, render

    def vis_save_ppm(self, render, filename):
        """src/visualization_io.c vis_save(IMAGE_FILETYPE_PPM) of a render buffer."""
        render = np.ascontiguousarray(render, np.float32)
        sizey, sizex = render.shape[:2]
        return self.lib.refh_vis_save(render.ctypes.data, sizex, sizey, filename.encode(), 1)

    def initcond(self):
        """src/initcond.c initcond_generate on the current simulation (FP32 variants)."""
        return self.lib.refh_initcond()

    def save_raw(self, filename):
        """src/simulation_io.c:81-149 (FP32 variants)."""
        return self.lib.refh_save_raw(filename.encode())

    def read_raw(self, filename):
        """src/simulation_io.c:16-79 (FP32 variants)."""
        return self.lib.refh_read_raw(filename.encode())

    def free(self):
        self.lib.refh_free()
