"""starflood_gb300 -- Starflood's force-and-step path on one GB300.

Python host mirror of the C ABI in include/sfgpu.h (resident simulations)
and include/starflood_compat.h (the reference's sim_t surface), through
ctypes.  The compute path is libsfgpu.so (hand-written CUDA for sm_103a);
there is no fallback: importing works without a GPU, but every call that
reaches the device fails loudly when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsfgpu.so")

SOLVER_PP, SOLVER_TREE = 0, 1
SPH_OFF, SPH_REFERENCE, SPH_CUBIC = 0, 1, 2
MATH_FAST, MATH_EXACT = 0, 1
FORM_PLAIN, FORM_COMPENSATED = 0, 1
ACC_REFERENCE, ACC_PHYSICAL = 0, 1
FLAG_STATS, FLAG_TIMING, FLAG_NOGRAPH, FLAG_EXPORT_TREE, FLAG_VERBOSE = 0x1, 0x2, 0x4, 0x8, 0x10
STATUS_TREE_NODES, STATUS_TREE_DEPTH, STATUS_TIES, STATUS_SPIN, STATUS_WALK, STATUS_SPH_CELLS = (
    0x01, 0x02, 0x04, 0x08, 0x10, 0x20)


class SfgpuError(RuntimeError):
    pass


class Params(C.Structure):
    """sfgpu_params (include/sfgpu.h)."""
    _fields_ = [("dt", C.c_double), ("eps", C.c_double), ("G", C.c_double), ("theta", C.c_double),
                ("solver", C.c_int32), ("sph", C.c_int32), ("math", C.c_int32), ("form", C.c_int32),
                ("acc_mode", C.c_int32), ("leaf_cap", C.c_uint32), ("depth_max", C.c_uint32),
                ("nodes_max", C.c_uint32), ("sph_gamma", C.c_double), ("sph_alpha", C.c_double),
                ("sph_beta", C.c_double), ("flags", C.c_uint32), ("walk_split", C.c_uint32),
                ("sph_path", C.c_uint32), ("walk_group", C.c_uint32), ("spin_limit", C.c_uint32),
                ("walk_limit", C.c_uint32), ("reserved", C.c_uint32 * 2)]


_lib = None


def lib():
    """The loaded libsfgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SfgpuError("libsfgpu.so is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        vp, u32, i32, f32p, u32p = C.c_void_p, C.c_uint32, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_uint32)
        P = C.POINTER(Params)
        sig = {
            "sfgpu_params_default": (None, [P]),
            "sfgpu_dof": (u32, [P]),
            "sfgpu_last_error": (C.c_char_p, []),
            "sfgpu_create": (i32, [C.POINTER(vp), u32, P]),
            "sfgpu_destroy": (i32, [vp]),
            "sfgpu_upload": (i32, [vp, vp]),
            "sfgpu_download": (i32, [vp, vp]),
            "sfgpu_upload_arrays": (i32, [vp, vp, u32, u32]),
            "sfgpu_download_arrays": (i32, [vp, vp, u32, u32]),
            "sfgpu_solve": (i32, [vp, u32]),
            "sfgpu_step": (i32, [vp, u32]),
            "sfgpu_run": (i32, [vp, u32, u32]),
            "sfgpu_synchronize": (i32, [vp]),
            "sfgpu_energies": (i32, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "sfgpu_energies_corrected": (i32, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                               C.POINTER(C.c_double)]),
            "sfgpu_momentum": (i32, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "sfgpu_status": (i32, [vp, u32p]),
            "sfgpu_stream": (vp, [vp]),
            "sfgpu_device_slab": (vp, [vp]),
            "sfgpu_stage_times": (i32, [vp, C.POINTER(C.c_char_p), C.POINTER(C.c_double), u32p, i32]),
            "sfgpu_walk_stats": (i32, [vp, u32p, u32p]),
            "sfgpu_walk_totals": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
            "sfgpu_tree_build": (i32, [vp, f32p]),
            "sfgpu_gravity_tree": (i32, [vp]),
            "sfgpu_gravity_part": (i32, [vp]),
            "sfgpu_solve_sph": (i32, [vp]),
            "sfgpu_sph_neighbours": (i32, [vp, u32p]),
            "sfgpu_sph_neighbour_hashes": (i32, [vp, C.POINTER(C.c_uint64)]),
            "sfgpu_sort_withheld_check": (i32, [vp, u32, u32, u32, vp, vp, u32p]),
            "sfgpu_sort_keys": (i32, [vp, u32, i32, vp, vp, u32p]),
            "sfgpu_paired_check": (i32, [u32, u32, vp]),
            "sfgpu_sph_set_u": (i32, [vp, f32p]),
            "sfgpu_sph_get_u": (i32, [vp, f32p, f32p]),
            "sfgpu_tree_keys": (i32, [vp, C.POINTER(C.c_uint64), u32p, u32p, f32p]),
            "sfgpu_tree_num_nodes": (i32, [vp, u32p]),
            "sfgpu_tree_export": (i32, [vp, u32p, u32p, u32p, f32p, f32p]),
            "sfgpu_gravity_pp": (i32, [P, u32, vp, vp, vp, vp, vp]),
            "sfgpu_gravity_pp_noalloc": (i32, [P, u32, vp, vp, vp, vp, vp]),
            "sfgpu_batch_create": (i32, [C.POINTER(vp), u32, u32p, P]),
            "sfgpu_batch_destroy": (i32, [vp]),
            "sfgpu_batch_upload": (i32, [vp, vp, vp, vp]),
            "sfgpu_batch_download": (i32, [vp, vp, vp, vp, vp]),
            "sfgpu_batch_solve": (i32, [vp]),
            "sfgpu_batch_run": (i32, [vp, u32]),
            "sfgpu_batch_autotune": (i32, [vp, C.POINTER(C.c_int)]),
            "sfgpu_batch_synchronize": (i32, [vp]),
            "sfgpu_batch_stream": (vp, [vp]),
            "sfgpu_batch_grad": (i32, [vp, u32, u32, vp, vp, C.POINTER(C.c_double)]),
            "sfgpu_batch_force_vjp": (i32, [vp, vp, vp]),
            "sfgpu_kernel_launches": (C.c_ulonglong, []),
            "sfgpu_host_register": (i32, [vp, C.c_size_t]),
            "sfgpu_host_unregister": (i32, [vp]),
            "sfgpu_flush_l2": (i32, [vp]),
            "sfgpu_save_raw": (i32, [vp, C.c_char_p]),
            "sfgpu_initcond": (i32, [vp]),
            "sfgpu_host_step": (i32, [vp, vp, u32, i32, u32p]),
            "sfgpu_vis_params_default": (None, [vp]),
            "sfgpu_vis_draw": (i32, [vp, vp, u32, u32, u32, vp, vp]),
            "sfgpu_vis_buffers_alloc": (i32, [u32, u32, C.POINTER(vp), C.POINTER(vp)]),
            "sfgpu_vis_buffers_free": (None, [vp, vp]),
            "sfgpu_vis_download": (i32, [vp, u32, u32, vp, vp, vp, vp]),
            "sfgpu_snapshot_wait": (i32, [vp]),
            "sfgpu_read_raw": (i32, [vp, C.c_char_p]),
            "sfgpu_grid_create": (i32, [C.POINTER(vp), u32, f32p, f32p, C.c_double, vp]),
            "sfgpu_grid_destroy": (i32, [vp]),
            "sfgpu_grid_samp": (vp, [vp]),
            "sfgpu_grid_accum": (vp, [vp]),
            "sfgpu_grid_stream": (vp, [vp]),
            "sfgpu_grid_side": (u32, [vp]),
            "sfgpu_grid_deposit_arrays": (i32, [vp, u32, vp, u32, u32]),
            "sfgpu_grid_deposit": (i32, [vp, vp, u32, u32]),
            "sfgpu_grid_solve_fft": (i32, [vp]),
            "sfgpu_grid_upload": (i32, [vp, vp]),
            "sfgpu_grid_download": (i32, [vp, vp, vp]),
            "sfgpu_grid_synchronize": (i32, [vp]),
            "sfgpu_compat_configure": (i32, [P]),
            "sfgpu_compat_params": (None, [P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def mix64(idx):
    """splitmix64's output function on body indices (uint64 array), the
    per-member term of the neighbour-set hashes."""
    with np.errstate(over="ignore"):
        x = np.asarray(idx, np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def sort_withheld_check(keys, withheld_tile=0xFFFFFFFF, spin_limit=0):
    """sfgpu_sort_withheld_check: (sorted keys, index, status word)."""
    keys = np.ascontiguousarray(keys, np.uint64)
    n = len(keys)
    out = np.zeros(n, np.uint64)
    idx = np.zeros(n, np.uint32)
    st = C.c_uint32()
    check(lib().sfgpu_sort_withheld_check(_ptr(keys), n, withheld_tile, spin_limit, _ptr(out), _ptr(idx),
                                          C.byref(st)), "sfgpu_sort_withheld_check")
    return out, idx, st.value


def sort_keys(keys, bits):
    """sfgpu_sort_keys: (sorted keys, original index per slot, status word)."""
    keys = np.ascontiguousarray(keys, np.uint64)
    n = len(keys)
    out = np.zeros(n, np.uint64)
    idx = np.zeros(n, np.uint32)
    st = C.c_uint32()
    check(lib().sfgpu_sort_keys(_ptr(keys), n, bits, _ptr(out), _ptr(idx), C.byref(st)), "sfgpu_sort_keys")
    return out, idx, st.value


def paired_check(n, seed=1):
    """sfgpu_paired_check: (walk mismatches, SPH mismatches)."""
    out = np.zeros(2, np.uint64)
    check(lib().sfgpu_paired_check(n, seed, _ptr(out)), "sfgpu_paired_check")
    return int(out[0]), int(out[1])


def last_error() -> str:
    return (lib().sfgpu_last_error() or b"").decode()


def check(rc, what=""):
    if rc != 0:
        raise SfgpuError("%s failed: %s" % (what, last_error()))


def default_params(**kw) -> Params:
    """The reference's config.h defaults, then keyword overrides."""
    p = Params()
    lib().sfgpu_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def dof(p: Params) -> int:
    return int(lib().sfgpu_dof(C.byref(p)))


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class Sim:
    """A resident simulation (sfgpu_sim) of N bodies."""

    def __init__(self, n: int, params: Params):
        self.n = int(n)
        self.params = params
        self.dof = dof(params)
        h = C.c_void_p()
        check(lib().sfgpu_create(C.byref(h), self.n, C.byref(params)), "sfgpu_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().sfgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # host transfers ------------------------------------------------------
    def upload(self, slab: np.ndarray):
        slab = np.ascontiguousarray(slab, np.float32)
        assert slab.size == self.n * self.dof
        check(lib().sfgpu_upload(self.h, _ptr(slab)), "sfgpu_upload")

    def download(self) -> np.ndarray:
        out = np.empty(self.n * self.dof, np.float32)
        check(lib().sfgpu_download(self.h, _ptr(out)), "sfgpu_download")
        return out

    def set_state(self, pos, vel, mas, rad=None):
        slab = np.zeros(self.n * self.dof, np.float32)
        n = self.n
        slab[0:3 * n] = np.asarray(pos, np.float32).ravel()
        slab[3 * n:6 * n] = np.asarray(vel, np.float32).ravel()
        slab[9 * n:10 * n] = np.asarray(mas, np.float32)
        if rad is not None:
            slab[13 * n:14 * n] = np.asarray(rad, np.float32)
        self.upload(slab)
        return slab

    # steps -----------------------------------------------------------------
    def solve(self, step=0):
        check(lib().sfgpu_solve(self.h, step), "sfgpu_solve")

    def step(self, step):
        check(lib().sfgpu_step(self.h, step), "sfgpu_step")

    def run(self, first, nsteps):
        check(lib().sfgpu_run(self.h, first, nsteps), "sfgpu_run")

    def sync(self):
        check(lib().sfgpu_synchronize(self.h), "sfgpu_synchronize")

    def energies(self):
        T, V = C.c_double(), C.c_double()
        check(lib().sfgpu_energies(self.h, C.byref(T), C.byref(V)), "sfgpu_energies")
        return T.value, V.value

    def energies_corrected(self):
        T, V, E = C.c_double(), C.c_double(), C.c_double()
        check(lib().sfgpu_energies_corrected(self.h, C.byref(T), C.byref(V), C.byref(E)), "energies")
        return T.value, V.value, E.value

    def momentum(self):
        """(P, L): total linear and angular momentum of the current state, FP64."""
        P, L = (C.c_double * 3)(), (C.c_double * 3)()
        check(lib().sfgpu_momentum(self.h, P, L), "sfgpu_momentum")
        return np.array(P[:]), np.array(L[:])

    def status(self) -> int:
        s = C.c_uint32()
        check(lib().sfgpu_status(self.h, C.byref(s)), "sfgpu_status")
        return s.value

    def stream(self) -> int:
        return int(lib().sfgpu_stream(self.h) or 0)

    def stage_times(self):
        cap = 64
        names = (C.c_char_p * cap)()
        ms = (C.c_double * cap)()
        la = (C.c_uint32 * cap)()
        m = lib().sfgpu_stage_times(self.h, names, ms, la, cap)
        if m < 0:
            raise SfgpuError(last_error())
        return {names[i].decode(): (ms[i], la[i]) for i in range(m)}

    def initcond(self):
        """initcond_generate (src/initcond.c) into the device slab."""
        check(lib().sfgpu_initcond(self.h), "sfgpu_initcond")

    def save_raw(self, filename):
        """Queue a raw snapshot of the current state (written asynchronously)."""
        check(lib().sfgpu_save_raw(self.h, os.fsencode(filename)), "sfgpu_save_raw")

    def snapshot_wait(self):
        check(lib().sfgpu_snapshot_wait(self.h), "sfgpu_snapshot_wait")

    def read_raw(self, filename):
        check(lib().sfgpu_read_raw(self.h, os.fsencode(filename)), "sfgpu_read_raw")

    def vis_draw(self, step, sizex, sizey, samples=128):
        """vis_draw of the current state: (accum int32 (sizey, sizex, 4),
        render float32 (sizey, sizex, 4))."""
        L = lib()
        vp = (C.c_byte * 64)()
        L.sfgpu_vis_params_default(vp)
        C.c_uint32.from_buffer(vp, 0).value = samples
        da, dr = C.c_void_p(), C.c_void_p()
        check(L.sfgpu_vis_buffers_alloc(sizex, sizey, C.byref(da), C.byref(dr)), "sfgpu_vis_buffers_alloc")
        try:
            check(L.sfgpu_vis_draw(self.h, vp, step, sizex, sizey, da, dr), "sfgpu_vis_draw")
            acc = np.zeros((sizey, sizex, 4), np.int32)
            ren = np.zeros((sizey, sizex, 4), np.float32)
            check(L.sfgpu_vis_download(self.h, sizex, sizey, da, dr, acc.ctypes.data, ren.ctypes.data),
                  "sfgpu_vis_download")
        finally:
            L.sfgpu_vis_buffers_free(da, dr)
        return acc, ren

    def walk_stats(self):
        a = np.zeros(self.n, np.uint32)
        b = np.zeros(self.n, np.uint32)
        check(lib().sfgpu_walk_stats(self.h, a.ctypes.data_as(C.POINTER(C.c_uint32)),
                                     b.ctypes.data_as(C.POINTER(C.c_uint32))), "sfgpu_walk_stats")
        return a, b

    def walk_totals(self):
        a, b = C.c_uint64(), C.c_uint64()
        check(lib().sfgpu_walk_totals(self.h, C.byref(a), C.byref(b)), "sfgpu_walk_totals")
        return a.value, b.value

    def tree_build(self, bounds):
        b = np.ascontiguousarray(bounds, np.float32)
        check(lib().sfgpu_tree_build(self.h, b.ctypes.data_as(C.POINTER(C.c_float))), "sfgpu_tree_build")

    def gravity_tree(self):
        check(lib().sfgpu_gravity_tree(self.h), "sfgpu_gravity_tree")

    def gravity_part(self):
        check(lib().sfgpu_gravity_part(self.h), "sfgpu_gravity_part")

    def solve_sph(self):
        check(lib().sfgpu_solve_sph(self.h), "sfgpu_solve_sph")

    def sph_neighbours(self):
        a = np.zeros(self.n, np.uint32)
        check(lib().sfgpu_sph_neighbours(self.h, a.ctypes.data_as(C.POINTER(C.c_uint32))), "sfgpu_sph_neighbours")
        return a

    def sph_neighbour_hashes(self):
        a = np.zeros(self.n, np.uint64)
        check(lib().sfgpu_sph_neighbour_hashes(self.h, a.ctypes.data_as(C.POINTER(C.c_uint64))),
              "sfgpu_sph_neighbour_hashes")
        return a

    def sph_set_u(self, u):
        u = np.ascontiguousarray(u, np.float32)
        check(lib().sfgpu_sph_set_u(self.h, u.ctypes.data_as(C.POINTER(C.c_float))), "sfgpu_sph_set_u")

    def sph_get_u(self):
        u = np.zeros(self.n, np.float32)
        du = np.zeros(self.n, np.float32)
        f = C.POINTER(C.c_float)
        check(lib().sfgpu_sph_get_u(self.h, u.ctypes.data_as(f), du.ctypes.data_as(f)), "sfgpu_sph_get_u")
        return u, du

    def tree_keys(self):
        keys = np.zeros(self.n, np.uint64)
        idx = np.zeros(self.n, np.uint32)
        nin = C.c_uint32()
        b = np.zeros(6, np.float32)
        check(lib().sfgpu_tree_keys(self.h, keys.ctypes.data_as(C.POINTER(C.c_uint64)),
                                    idx.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(nin),
                                    b.ctypes.data_as(C.POINTER(C.c_float))), "sfgpu_tree_keys")
        return keys, idx, nin.value, b

    def num_nodes(self):
        nn = C.c_uint32()
        check(lib().sfgpu_tree_num_nodes(self.h, C.byref(nn)), "sfgpu_tree_num_nodes")
        return nn.value

    def tree_export(self):
        nn = self.num_nodes()
        u = C.POINTER(C.c_uint32)
        f = C.POINTER(C.c_float)
        parent = np.zeros(nn, np.uint32)
        bodies = np.zeros(nn, np.uint32)
        branch = np.zeros((nn, 8), np.uint32)
        bounds = np.zeros((nn, 6), np.float32)
        params = np.zeros((nn, 4), np.float32)
        check(lib().sfgpu_tree_export(self.h, parent.ctypes.data_as(u), bodies.ctypes.data_as(u),
                                      branch.ctypes.data_as(u), bounds.ctypes.data_as(f),
                                      params.ctypes.data_as(f)), "sfgpu_tree_export")
        return dict(parent=parent, bodies=bodies, branch=branch, bounds=bounds, params=params)


class Grid:
    """A particle-mesh grid (sfgpu_grid): side^3 FP32 samples over
    [bounds_min, bounds_max], resident in HBM; arrays are indexed [z, y, x]."""

    def __init__(self, side: int, bounds_min=(-2.0, -2.0, -2.0), bounds_max=(2.0, 2.0, 2.0), G=1.0, stream=None):
        self.side = int(side)
        lo = np.ascontiguousarray(bounds_min, np.float32)
        hi = np.ascontiguousarray(bounds_max, np.float32)
        f = C.POINTER(C.c_float)
        h = C.c_void_p()
        check(lib().sfgpu_grid_create(C.byref(h), self.side, lo.ctypes.data_as(f), hi.ctypes.data_as(f), G,
                                      stream), "sfgpu_grid_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().sfgpu_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return lib().sfgpu_grid_stream(self.h)

    @property
    def samp_ptr(self):
        return lib().sfgpu_grid_samp(self.h)

    def upload(self, samp):
        a = np.ascontiguousarray(samp, np.float32).reshape(-1)
        assert a.size == self.side ** 3
        check(lib().sfgpu_grid_upload(self.h, _ptr(a)), "sfgpu_grid_upload")

    def download(self, counts=False):
        d = self.side
        samp = np.zeros((d, d, d), np.float32)
        acc = np.zeros((d, d, d), np.int32) if counts else None
        check(lib().sfgpu_grid_download(self.h, _ptr(samp), _ptr(acc) if counts else None), "sfgpu_grid_download")
        return (samp, acc) if counts else samp

    def deposit(self, sim: "Sim", step: int, samples: int = 128):
        check(lib().sfgpu_grid_deposit(self.h, sim.h, step, samples), "sfgpu_grid_deposit")

    def deposit_arrays(self, n: int, d_pos, step: int, samples: int = 128):
        check(lib().sfgpu_grid_deposit_arrays(self.h, n, d_pos, step, samples), "sfgpu_grid_deposit_arrays")

    def solve_fft(self):
        check(lib().sfgpu_grid_solve_fft(self.h), "sfgpu_grid_solve_fft")

    def synchronize(self):
        check(lib().sfgpu_grid_synchronize(self.h), "sfgpu_grid_synchronize")


def slab_views(slab: np.ndarray, n: int, dof_: int):
    """Views of a slab in the reference layout (src/simulation.h:17-51)."""
    v = {"pos": slab[0:3 * n].reshape(n, 3), "vel": slab[3 * n:6 * n].reshape(n, 3),
         "acc": slab[6 * n:9 * n].reshape(n, 3), "mas": slab[9 * n:10 * n], "pot": slab[10 * n:11 * n],
         "ken": slab[11 * n:12 * n], "pen": slab[12 * n:13 * n]}
    if dof_ >= 16:
        v["rad"] = slab[13 * n:14 * n]
        v["rho"] = slab[14 * n:15 * n]
        v["prs"] = slab[15 * n:16 * n]
    return v


# ---- the reference's sim_t surface (include/starflood_compat.h) -------------
class NodeT(C.Structure):
    _fields_ = [("parent", C.c_uint32), ("bodies", C.c_uint32), ("branch", C.c_uint32 * 8),
                ("bounds", C.c_float * 6), ("params", C.c_float * 4)]


class TreeT(C.Structure):
    _fields_ = [("max_nodes", C.c_uint32), ("num_nodes", C.c_uint32), ("bounds", C.c_float * 6),
                ("node", C.POINTER(NodeT))]


class SimT(C.Structure):
    _fields_ = [("step_number", C.c_uint), ("N", C.c_uint), ("mem", C.c_void_p), ("tree", TreeT)]


class VisT(C.Structure):
    """src/visualization.h:19-27"""
    _fields_ = [("sizex", C.c_uint), ("sizey", C.c_uint), ("mem", C.c_void_p), ("atomic_buffer", C.c_void_p),
                ("render_buffer", C.c_void_p), ("binary_buffer", C.c_void_p)]


def compat_configure(p: Params):
    check(lib().sfgpu_compat_configure(C.byref(p)), "sfgpu_compat_configure")


class GridT(C.Structure):
    """src/grid.h:11-24 (ENABLE_FFT layout)."""
    _fields_ = [("dim", C.c_uint * 3), ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3),
                ("mem", C.c_void_p), ("mem_fft0", C.c_void_p), ("mem_fft1", C.c_void_p), ("mem_fft2", C.c_void_p)]


def compat_functions():
    """The drop-in entry points with their C signatures."""
    L = lib()
    S = C.POINTER(SimT)
    T = C.POINTER(TreeT)
    V = C.POINTER(VisT)
    G = C.POINTER(GridT)
    fp = C.POINTER(C.c_float)
    for name, args in (("grid_init", [G, C.c_uint, fp, fp]), ("grid_free", [G]), ("grid_solve_fft", [G]),
                       ("solve_gravity_part_mesh", [S, G])):
        fn = getattr(L, name)
        fn.restype = C.c_int
        fn.argtypes = args
    L.grid_samp.restype = C.c_void_p
    L.grid_samp.argtypes = [G]
    for name, args in (("sim_init", [S, C.c_uint]), ("sim_free", [S]), ("sim_solv", [S]), ("sim_step", [S]),
                       ("solve_gravity_part_part", [S]), ("solve_gravity_part_tree", [S]), ("solve_sph", [S]),
                       ("tree_init", [T, C.c_uint]), ("tree_free", [T]),
                       ("sim_save_raw", [S, C.c_char_p]), ("sim_read_raw", [S, C.c_char_p]),
                       ("vis_init", [V, C.c_uint, C.c_uint]), ("vis_free", [V]), ("initcond_generate", [S]),
                       ("vis_draw", [V, S]), ("vis_save", [V, C.c_char_p, C.c_int]),
                       ("tree_build", [T, C.c_uint, C.c_void_p, C.c_void_p])):
        fn = getattr(L, name)
        fn.restype = C.c_int
        fn.argtypes = args
    L.sim_find.restype = C.c_void_p
    L.sim_find.argtypes = [S, C.c_int]
    L.sfgpu_sync_host.restype = C.c_int
    L.sfgpu_sync_host.argtypes = [S]
    L.sfgpu_compat_handle.restype = C.c_void_p
    L.sfgpu_compat_handle.argtypes = [S]
    return L


class Batch:
    """Many independent systems (sfgpu_batch): batched PP + KDK, and the
    adjoint of a trajectory."""

    def __init__(self, sizes, params: Params):
        self.sizes = [int(x) for x in sizes]
        off = np.zeros(len(self.sizes) + 1, np.uint32)
        off[1:] = np.cumsum(self.sizes)
        self.off = off
        self.total = int(off[-1])
        self.params = params
        h = C.c_void_p()
        check(lib().sfgpu_batch_create(C.byref(h), len(self.sizes), off.ctypes.data_as(C.POINTER(C.c_uint32)),
                                       C.byref(params)), "sfgpu_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().sfgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, pos, vel, mas):
        f = lambda a: np.ascontiguousarray(a, np.float32)
        pos, vel, mas = f(pos), f(vel), f(mas)
        check(lib().sfgpu_batch_upload(self.h, _ptr(pos), _ptr(vel), _ptr(mas)), "sfgpu_batch_upload")

    def download(self):
        pos = np.zeros((self.total, 3), np.float32)
        vel = np.zeros((self.total, 3), np.float32)
        acc = np.zeros((self.total, 3), np.float32)
        pot = np.zeros(self.total, np.float32)
        check(lib().sfgpu_batch_download(self.h, _ptr(pos), _ptr(vel), _ptr(acc), _ptr(pot)), "download")
        return pos, vel, acc, pot

    def solve(self):
        check(lib().sfgpu_batch_solve(self.h), "sfgpu_batch_solve")

    def run(self, nsteps):
        check(lib().sfgpu_batch_run(self.h, nsteps), "sfgpu_batch_run")

    def sync(self):
        check(lib().sfgpu_batch_synchronize(self.h), "sfgpu_batch_synchronize")

    def stream(self) -> int:
        return int(lib().sfgpu_batch_stream(self.h) or 0)

    def autotune(self) -> int:
        c = C.c_int()
        check(lib().sfgpu_batch_autotune(self.h, C.byref(c)), "sfgpu_batch_autotune")
        return c.value

    def grad(self, nsteps, checkpoint=20):
        gp = np.zeros((self.total, 3), np.float32)
        gv = np.zeros((self.total, 3), np.float32)
        loss = C.c_double()
        check(lib().sfgpu_batch_grad(self.h, nsteps, checkpoint, _ptr(gp), _ptr(gv), C.byref(loss)),
              "sfgpu_batch_grad")
        return loss.value, gp, gv
