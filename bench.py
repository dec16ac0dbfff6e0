"""Benchmark: Barnes-Hut KDK steps of the 65,536-body expanding uniform sphere
(theta = 0.5 squared criterion, leaf 8, eps = 0.01, dt = 1e-3) on one GB300,
plus three sub-benchmarks in the same JSON line: PP gravity at N = 1,048,576
(Plummer, eps = 0.005), plain and compensated forms ("pp"); Barnes-Hut +
cubic-spline SPH on a 262,144-body Plummer gas ("sph"); 256 batched systems
of 1024..32768 bodies, forward and adjoint ("batch").

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--no-pp] [--no-sph] [--no-batch] [--no-cpu]

value  particle-steps/s of K steps with the state resident in HBM, each step
       one replay of the captured CUDA graph of sim_step; the L2 is flushed
       (256 MiB memset) between timed steps and the flush is not timed.
e2e    the same K steps through the drop-in sim_step() with host slabs:
       every call uploads the slab from page-locked host memory, steps and
       downloads the slab (host wall clock).
roofline  the dominant kernel (the walk), from a CUDA-event-instrumented twin
       run of the same K steps: algorithmic FP32 flops = 22 per monopole
       interaction (20 force + 2 potential, the conventional count) + 12 per
       opening test (both counted on the device), against the FP32 FMA peak.
cpu_baseline  the CPU restatement of the reference path (oracle/, OpenMP,
       all host threads) on a bounded sample of the same workload.
--impl reference  times that CPU path as the reference arm.
Multi-GPU (torchrun): every rank runs an independent replica of the workload
on its own GPU (the walk and the tree are replicated, "replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_BH = 65536
N_PP = 1 << 20
N_SPH = 1 << 18
METRIC = "particle-steps/s & PP interactions/s, chosen vs plain, 1 GB300, rel err<=1e-6"
WORKLOAD = "Barnes-Hut KDK step, N=65536 uniform unit sphere, v=0.5r, m=1/N, G=1, eps=0.01, theta=0.5, leaf=8, dt=1e-3"
FLOP_INTERACTION = 22  # conventional count: 20 for the force, 2 more with the potential
FLOP_OPEN = 12
BH_EXTRA = {}  # extra sfgpu_params of the Barnes-Hut workload (--walk-split)


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def nvml_index(local):
    """NVML numbers every GPU of the machine: the first CUDA_VISIBLE_DEVICES
    entry when it is an index, else the local rank."""
    first = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].strip()
    return int(first) if first.isdigit() else local


class NvmlClocks:
    """SM clock, maximum clock, power and throttle reasons read through NVML
    (libnvidia-ml, ctypes: read-only queries), sampled by the caller inside
    the timed loop (once per step); nvidia-smi polling as the fallback."""
    # nvmlClocksEventReasons bits
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap"}

    def __init__(self, index: int):
        import ctypes as C
        self.samples = []
        self.h = None
        try:
            self.nv = C.CDLL("libnvidia-ml.so.1")
            if self.nv.nvmlInit_v2() != 0:
                raise OSError("nvmlInit")
            h = C.c_void_p()
            if self.nv.nvmlDeviceGetHandleByIndex_v2(index, C.byref(h)) != 0 and \
                    self.nv.nvmlDeviceGetHandleByIndex_v2(0, C.byref(h)) != 0:
                raise OSError("handle")
            self.h = h
            mx = C.c_uint()
            self.max_mhz = float(mx.value) if self.nv.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 else None
        except OSError:
            self.h = None

    def sample(self):
        if self.h is None:
            return
        import ctypes as C
        clk, pw, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(clk)) != 0:
            return
        self.nv.nvmlDeviceGetPowerUsage(self.h, C.byref(pw))
        fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        fn(self.h, C.byref(rs))
        self.samples.append((float(clk.value), pw.value / 1000.0, int(rs.value)))

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        reasons = sorted({name for _, _, r in self.samples for bit, name in self.REASONS.items() if r & bit})
        return {"sm_mhz": statistics.median(s[0] for s in self.samples), "sm_max_mhz": self.max_mhz,
                "power_w_max": max(s[1] for s in self.samples), "reasons": reasons,
                "samples": len(self.samples), "source": "NVML, one sample per timed step"}


def fp32_peak_tflops():
    """FP32 FMA peak: SMs x 128 lanes x 2 flop x the maximum SM clock recorded
    in MEASURED_PEAKS.json (the file has no FP32 figure of its own)."""
    mhz, src = 2070.0, "nominal 2070 MHz"
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        mhz, src = float(mp.get("sm_max_mhz", mhz)), "sm_max_mhz of MEASURED_PEAKS.json"
    except Exception:
        pass
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    return sms * 128 * 2 * mhz * 1e6 / 1e12, "derived: %d SMs x 128 FP32 lanes x 2 flop x %.0f MHz (%s)" % (
        sms, mhz, src)


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of MEASURED_PEAKS.json, else the
    6.8 TB/s fallback."""
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(mp["hbm_gbs"]), "measured: hbm_gbs of MEASURED_PEAKS.json"
    except Exception:
        return 6800.0, "fallback: 6.8 TB/s (no MEASURED_PEAKS.json)"


def bh_inputs(n=N_BH):
    from starflood_gb300.ics import uniform_ball
    return uniform_ball(n, seed=2024)


# ---------------------------------------------------------------------------
# CPU reference path (the oracle restatement, or the compiled reference here)
# ---------------------------------------------------------------------------
def cpu_bh_rate(max_seconds=12.0, max_steps=200, n=N_BH):
    from oracle import build as ob
    ob.build_oracle()
    from oracle.pyoracle import Oracle, make_params, slab_views
    pos, vel, mas = bh_inputs(n)
    orc = Oracle("f32")
    p = make_params(dt=1e-3, eps=0.01, theta=0.5, use_tree=1)
    sim, slab, nodes = orc.new_sim(n, p)
    v = slab_views(slab, n, 13)
    v["pos"][:] = pos
    v["vel"][:] = vel
    v["mas"][:] = mas
    orc.sim_solv(p, sim, 0)
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps and (time.perf_counter() - t0) < max_seconds:
        orc.sim_step(p, sim, steps)
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": "particle-steps/s", "cores": orc.threads(), "kind": "port",
            "sample": "%d sim_step calls of the N=%d Barnes-Hut workload (%.1f s)" % (steps, n, dt)}


def cpu_pp_rate(max_seconds=10.0):
    from oracle.pyoracle import Oracle, make_params
    from starflood_gb300.ics import plummer
    orc = Oracle("f32")
    n = 32768
    pos, _, mas = plummer(n, seed=5)
    p = make_params(eps=0.005)
    t0 = time.perf_counter()
    evals = 0
    while evals < 1 or (time.perf_counter() - t0) < max_seconds and evals < 20:
        orc.pp(pos, mas, p)
        evals += 1
    dt = time.perf_counter() - t0
    return {"value": float(n) * n * evals / dt, "unit": "interactions/s", "cores": orc.threads(), "kind": "port",
            "sample": "%d solve_gravity_part_part evals at N=%d (per-interaction rate is size independent)" % (
                evals, n)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def gpu_bh(steps, warmup, sf):
    import ctypes as C
    pos, vel, mas = bh_inputs()
    n = N_BH
    L = sf.lib()

    def new_sim(flags):
        p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5, flags=flags, **BH_EXTRA)
        s = sf.Sim(n, p)
        s.set_state(pos, vel, mas)
        s.solve(0)
        return s

    # --- headline: graph replays, L2 flushed between timed steps -------------
    import torch
    s = new_sim(0)
    stream = s.stream()
    ext = torch.cuda.ExternalStream(stream)
    s.run(0, warmup)
    s.sync()
    launches0 = sf.lib().sfgpu_kernel_launches()
    s.run(warmup, 1)  # the graph exists now; count one eager capture's launches below
    s.sync()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    rank, world, local = env_rank()
    clk = NvmlClocks(nvml_index(local))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(steps):
        sf.check(L.sfgpu_flush_l2(C.c_void_p(stream)), "flush")
        with torch.cuda.stream(ext):
            events[k][0].record(ext)
        s.run(warmup + 1 + k, 1)
        with torch.cuda.stream(ext):
            events[k][1].record(ext)
        clk.sample()  # host-side query while the GPU works through the queued steps
    s.sync()
    torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in events]
    total_ms = float(sum(step_ms))
    status = s.status()
    s.close()

    # kernels per step: one eager (uncaptured) step
    p0 = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5, flags=sf.FLAG_NOGRAPH, **BH_EXTRA)
    with sf.Sim(n, p0) as s2:
        s2.set_state(pos, vel, mas)
        s2.solve(0)
        s2.sync()
        c0 = L.sfgpu_kernel_launches()
        s2.step(0)
        s2.sync()
        per_step = int(L.sfgpu_kernel_launches() - c0)
    del launches0

    # --- instrumented twin: per-stage CUDA events, walk counters ------------
    st = new_sim(sf.FLAG_TIMING)
    st.run(0, warmup)
    st.sync()
    st.stage_times()
    st.walk_totals()
    for k in range(steps):
        sf.check(L.sfgpu_flush_l2(C.c_void_p(st.stream())), "flush")
        st.step(warmup + k)
    st.sync()
    stages = st.stage_times()
    n_int, n_open = st.walk_totals()
    st.close()

    # --- e2e through the drop-in sim_step() ---------------------------------
    e2e = gpu_bh_e2e(steps, warmup, sf, pos, vel, mas)
    return dict(total_ms=total_ms, step_ms=step_ms, status=status, stages=stages, n_int=n_int, n_open=n_open,
                per_step=per_step, clocks=clk.summary(), e2e=e2e)


def bh_per_particle_err(sf, oracle_threads_ok=True):
    """Per-particle relative L2 error |a_i - a_ref,i| / |a_ref,i| of one FAST
    solve of the headline's initial state against the FP32 restatement of the
    reference's tree build and walk (bit-identical to the compiled reference),
    all 65,536 bodies: median, p99, max."""
    from oracle import build as ob
    ob.build_oracle()
    from oracle.pyoracle import Oracle, make_params
    pos, vel, mas = bh_inputs()
    n = N_BH
    orc = Oracle("f32")
    op = make_params(eps=0.01, theta=0.5, use_tree=1)
    st, nodes = orc.tree_build(pos, mas, orc.root_bounds(pos, 0), op)
    a_ref, p_ref, _, mag = orc.walk(pos, mas, nodes, op, with_mag=True)
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5, **BH_EXTRA)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        v = sf.slab_views(s.download(), n, 13)
    a = v["acc"].astype(np.float64)
    r = a_ref.astype(np.float64)
    e = np.linalg.norm(a - r, axis=1) / np.linalg.norm(r, axis=1)
    em = np.linalg.norm(a - r, axis=1) / mag.astype(np.float64)
    return {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)), "max": float(e.max()),
            "max_over_term_magnitudes": float(em.max()),
            "global_l2": float(np.linalg.norm(a - r) / np.linalg.norm(r)),
            "against": "FP32 restatement of tree.c + gravity.c (bit-identical to the reference), N=65536, step 0"}


def bh_variant_rates(sf, steps=20, warmup=3):
    """Particle-steps/s of the headline workload with leaf 16 (the leaf size
    of the published Barnes-Hut configuration) and with EXACT arithmetic (the
    reference's FP32 expressions, bit-identical results), each K graph
    replays with the L2 flushed between steps (CUDA events)."""
    import ctypes as C
    import torch
    pos, vel, mas = bh_inputs()
    n = N_BH
    L = sf.lib()
    out = {}
    for name, kw in (("leaf16", dict(leaf_cap=16)), ("exact", dict(math=sf.MATH_EXACT))):
        p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5, **kw)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            s.run(0, warmup)
            s.sync()
            ext = torch.cuda.ExternalStream(s.stream())
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            for k in range(steps):
                sf.check(L.sfgpu_flush_l2(C.c_void_p(s.stream())), "flush")
                with torch.cuda.stream(ext):
                    ev[k][0].record(ext)
                s.run(warmup + k, 1)
                with torch.cuda.stream(ext):
                    ev[k][1].record(ext)
            s.sync()
            ms = sum(a.elapsed_time(b) for a, b in ev) / steps
            out[name] = {"value": n / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms,
                         "device_status": s.status()}
    return out


def walk_vs_n(sf, sizes=(262144, 1048576), steps=5, warmup=2):
    """The walk's roofline fraction at larger N (uniform sphere, theta 0.5,
    leaf 8): stage times from CUDA events of the instrumented step, device
    counts of interactions and opening tests."""
    import ctypes as C
    from starflood_gb300.ics import uniform_ball
    peak, _ = fp32_peak_tflops()
    L = sf.lib()
    out = {}
    for n in sizes:
        pos, vel, mas = uniform_ball(n, seed=2024)
        p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5, flags=sf.FLAG_TIMING)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            s.run(0, warmup)
            s.sync()
            s.stage_times()
            s.walk_totals()
            for k in range(steps):
                sf.check(L.sfgpu_flush_l2(C.c_void_p(s.stream())), "flush")
                s.step(warmup + k)
            s.sync()
            st = s.stage_times()
            ni, no = s.walk_totals()
        wms = st["walk"][0] / max(1, st["walk"][1])
        step_ms = sum(v[0] for v in st.values()) / steps
        flops = (FLOP_INTERACTION * ni + FLOP_OPEN * no) / max(1, st["walk"][1])
        ach = flops / (wms * 1e-3) / 1e12
        out[str(n)] = {"walk_ms": wms, "walk_tflops": ach, "walk_frac": ach / peak,
                       "interactions_per_step": ni / max(1, st["walk"][1]),
                       "eager_step_ms": step_ms, "particle_steps_per_s_eager": n / (step_ms * 1e-3)}
    return out


def gpu_bh_e2e(steps, warmup, sf, pos, vel, mas):
    import ctypes as C
    n = N_BH
    L = sf.compat_functions()
    sf.compat_configure(sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5, **BH_EXTRA))
    sim = sf.SimT()
    sf.check(L.sim_init(C.byref(sim), n), "sim_init")
    dof = 13
    buf = (C.c_float * (n * dof)).from_address(sim.mem)
    slab = np.frombuffer(buf, np.float32)
    v = sf.slab_views(slab, n, dof)
    v["pos"][:] = pos
    v["vel"][:] = vel
    v["mas"][:] = mas
    sf.check(L.sim_solv(C.byref(sim)), "sim_solv")
    for k in range(warmup):
        sim.step_number = k
        sf.check(L.sim_step(C.byref(sim)), "sim_step")
    t0 = time.perf_counter()
    for k in range(steps):
        sim.step_number = warmup + k
        sf.check(L.sim_step(C.byref(sim)), "sim_step")
    dt = time.perf_counter() - t0
    # sfgpu_host_step uploads the arrays a step reads (pos, vel, acc, mas: 10
    # floats per body; 11 with SPH's rad) and downloads the whole slab
    h2d = 4 * n * (10 + (1 if dof > 13 else 0))
    d2h = 4 * n * dof
    L.sim_free(C.byref(sim))
    return {"value": n * steps / dt, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "api": "sim_step() of include/starflood_compat.h, host slab"}


def gpu_pp(sf, reps=2, n=N_PP, exact=True):
    """PP solves at N = 1,048,576 (CUDA events around the force stage): the
    plain form (FP32, FAST), the compensated form, and the plain form with
    EXACT arithmetic (the reference's expression and Kahan sums, one rep)."""
    from starflood_gb300.ics import plummer
    pos, vel, mas = plummer(n, seed=5)
    out = {}
    forms = [("plain", sf.FORM_PLAIN, sf.MATH_FAST, reps), ("compensated", sf.FORM_COMPENSATED, sf.MATH_FAST, reps)]
    if exact:
        forms.append(("plain_exact", sf.FORM_PLAIN, sf.MATH_EXACT, 1))
    for name, form, math, r in forms:
        p = sf.default_params(solver=sf.SOLVER_PP, eps=0.005, dt=1e-3, form=form, math=math, flags=sf.FLAG_TIMING)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            s.sync()
            s.stage_times()
            for _ in range(r):
                s.solve(0)
            s.sync()
            ms = s.stage_times()["pp"][0] / r
        out[name] = {"interactions_per_s": float(n) * n / (ms * 1e-3), "ms_per_eval": ms}
    return out


def pp_energy_drift(sf, steps=20):
    """Relative drift of the corrected total energy (kinetic + pair potential,
    FP64 sums) over `steps` KDK steps at dt = 1e-3 of the N = 1,048,576
    Plummer sphere, plain FP32 state against the compensated form (FP64
    state, compensated forces)."""
    from starflood_gb300.ics import plummer
    pos, vel, mas = plummer(N_PP, seed=5)
    out = {"steps": steps}
    for name, form in (("plain", sf.FORM_PLAIN), ("compensated", sf.FORM_COMPENSATED)):
        p = sf.default_params(solver=sf.SOLVER_PP, eps=0.005, dt=1e-3, form=form)
        with sf.Sim(N_PP, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            s.run(0, 1)
            e0 = s.energies_corrected()[2]
            s.run(1, steps - 1)
            e1 = s.energies_corrected()[2]
        out[name] = {"E_first": e0, "E_last": e1, "relative_drift": abs(e1 - e0) / abs(e0)}
    return out


def pp_accuracy(sf):
    """Force error of plain vs compensated against the FP64 oracle on a seeded
    8192-body subsample of the N=1,048,576 Plummer sphere (i in the sample,
    all j): the global relative L2 and the per-particle distribution."""
    from oracle import build as ob
    ob.build_oracle()
    from oracle.pyoracle import Oracle, make_params
    from starflood_gb300.ics import plummer
    n = N_PP
    pos, vel, mas = plummer(n, seed=5)
    sub = np.sort(np.random.default_rng(8192).choice(n, 8192, replace=False)).astype(np.uint32)
    a64, _ = Oracle("f64").pp_subset(pos.astype(np.float64), mas.astype(np.float64), sub, make_params(eps=0.005))
    errs = {}
    for name, form, math in (("plain", sf.FORM_PLAIN, sf.MATH_FAST), ("compensated", sf.FORM_COMPENSATED, sf.MATH_FAST),
                             ("plain_exact", sf.FORM_PLAIN, sf.MATH_EXACT)):
        p = sf.default_params(solver=sf.SOLVER_PP, eps=0.005, form=form, math=math)
        with sf.Sim(n, p) as s:
            s.set_state(pos, vel, mas)
            s.solve(0)
            v = sf.slab_views(s.download(), n, 13)
        a = v["acc"][sub].astype(np.float64)
        e = np.linalg.norm(a - a64, axis=1) / np.linalg.norm(a64, axis=1)
        errs[name] = float(np.linalg.norm(a - a64) / np.linalg.norm(a64))
        errs[name + "_per_particle"] = {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)),
                                        "max": float(e.max())}
    return errs


# ---------------------------------------------------------------------------
# Barnes-Hut + cubic-spline SPH, N = 262,144 Plummer gas
# ---------------------------------------------------------------------------
def sph_inputs(n=N_SPH):
    from starflood_gb300.ics import plummer
    pos, vel, mas = plummer(n, seed=7)
    return pos, vel, mas, np.full(n, 0.05, np.float32), np.full(n, 0.05, np.float32)


def sph_cell_tile_records(pos, h):
    """sum over occupied cells c of sum over the 27 cells c' around c of |c'|:
    the body records one pass streams when each cell loads its 27-cell
    neighbourhood once (cell side 2 h (1 + 1/4096), the search radius)."""
    side = 2.0 * float(h) * (1.0 + 1.0 / 4096.0)
    c = np.floor(pos.astype(np.float64) / side).astype(np.int64)
    c -= c.min(0)
    span = c.max(0) + 3
    key = ((c[:, 0] + 1) * span[1] + (c[:, 1] + 1)) * span[2] + (c[:, 2] + 1)
    cells, counts = np.unique(key, return_counts=True)
    occ = dict(zip(cells.tolist(), counts.tolist()))
    offs = [(dx * span[1] + dy) * span[2] + dz for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)]
    total = 0
    for k in cells.tolist():
        total += sum(occ.get(k + o, 0) for o in offs)
    return total


def gpu_sph(sf, steps, warmup, sph_path=0, mode="cubic"):
    """Barnes-Hut + SPH steps of the 262,144-body Plummer gas: mode "cubic"
    (cubic spline, ideal gas, Monaghan viscosity) or "reference" (the
    reference's Gaussian SPH of sph.c, FAST arithmetic: cell-grid search)."""
    import ctypes as C
    import torch
    n = N_SPH
    pos, vel, mas, rad, u = sph_inputs()
    L = sf.lib()
    cubic = mode == "cubic"

    def new_sim(flags):
        if cubic:
            p = sf.default_params(solver=sf.SOLVER_TREE, sph=sf.SPH_CUBIC, eps=0.01, dt=5e-4, theta=0.5,
                                  acc_mode=sf.ACC_PHYSICAL, sph_gamma=5.0 / 3.0, sph_alpha=1.0, sph_beta=2.0,
                                  flags=flags, sph_path=sph_path)
        else:
            p = sf.default_params(solver=sf.SOLVER_TREE, sph=sf.SPH_REFERENCE, eps=0.01, dt=5e-4, theta=0.5,
                                  flags=flags, sph_path=sph_path)
        s = sf.Sim(n, p)
        s.set_state(pos, vel, mas, rad)
        if cubic:
            s.sph_set_u(u)
        s.solve(0)
        return s

    s = new_sim(0)
    stream = s.stream()
    ext = torch.cuda.ExternalStream(stream)
    s.run(0, warmup + 1)
    s.sync()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        sf.check(L.sfgpu_flush_l2(C.c_void_p(stream)), "flush")
        with torch.cuda.stream(ext):
            events[k][0].record(ext)
        s.run(warmup + 1 + k, 1)
        with torch.cuda.stream(ext):
            events[k][1].record(ext)
    s.sync()
    torch.cuda.synchronize()
    total_ms = float(sum(a.elapsed_time(b) for a, b in events))
    status = s.status()
    mid = sf.slab_views(s.download(), n, 16)["pos"].copy()
    s.close()

    st = new_sim(sf.FLAG_TIMING)
    st.run(0, warmup)
    st.sync()
    st.stage_times()
    tsteps = max(3, steps // 5)
    for k in range(tsteps):
        sf.check(L.sfgpu_flush_l2(C.c_void_p(st.stream())), "flush")
        st.step(warmup + k)
    st.sync()
    stages = st.stage_times()
    pairs = float(st.sph_neighbours().astype(np.float64).sum())
    st.close()
    d_ms = stages["sph_density"][0] / max(1, stages["sph_density"][1])
    f_ms = stages["sph_force"][0] / max(1, stages["sph_force"][1])
    out = {
        "value": n * steps / (total_ms * 1e-3), "unit": "particle-steps/s", "steps": steps,
        "ms_per_step": total_ms / steps, "device_status": status,
        "l2": "flushed between timed steps (256 MiB memset, untimed)",
        "stage_ms_per_step": {k: round(v[0] / max(1, v[1]), 4) for k, v in stages.items()},
    }
    if not cubic:
        out["workload"] = ("Barnes-Hut (theta=0.5, leaf 8, eps=0.01) + the reference's SPH (sph.c: Gaussian kernel, "
                           "P=(0.1 rho)^2, momentum over r<=1; FAST arithmetic, cell-grid neighbour search by "
                           "warps of 32 sorted bodies), "
                           "h=0.05, N=262144 Plummer a=1 M=1, dt=5e-4")
        out["momentum_set_pairs_per_pass"] = pairs
        out["set_pairs_per_s"] = pairs / (f_ms * 1e-3)
        return out
    records = 0.5 * (sph_cell_tile_records(pos, 0.05) + sph_cell_tile_records(mid, 0.05))
    dens_bytes = records * 16 + n * 32    # x, y, z, m per tile record; 16 B in + 16 B out per body
    force_bytes = records * 48 + n * 32   # + vx, vy, vz, u and rho, P/rho^2, c, h per tile record
    peak = hbm_peak()
    dens_gbs = dens_bytes / (d_ms * 1e-3) / 1e9
    force_gbs = force_bytes / (f_ms * 1e-3) / 1e9
    dom = ("sph_force", force_gbs, force_bytes, f_ms) if f_ms >= d_ms else ("sph_density", dens_gbs, dens_bytes, d_ms)
    out.update({
        "workload": "Barnes-Hut (theta=0.5, leaf 8, eps=0.01) + cubic-spline SPH (h=0.05, gamma=5/3, u0=0.05, "
                    "alpha=1, beta=2), N=262144 Plummer a=1 M=1 with isotropic velocities, dt=5e-4",
        "neighbour_pairs_per_pass": pairs,
        "pairs_per_s": {"density": pairs / (d_ms * 1e-3), "force": pairs / (f_ms * 1e-3)},
        "roofline": {"kernel": "k_cubic_warp<%s> (one warp per 32 sorted bodies)" % (
                         "true" if dom[0] == "sph_force" else "false"),
                     "bound": "hbm", "achieved": dom[1], "peak": peak[0], "unit": "GB/s", "frac": dom[1] / peak[0],
                     "traffic": profiled_traffic("sph_cubic_warp_plummer262144.md"),
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum per launch of the force pass, "
                                       "profiles/sph_cubic_warp_plummer262144.md (ncu)",
                     "peak_source": peak[1],
                     "algorithmic_bytes_per_launch": dom[2], "avg_launch_ms": dom[3],
                     "density_pass_gbs": dens_gbs, "force_pass_gbs": force_gbs,
                     "cell_tile_records_per_pass": records,
                     "bytes_model": "the 27-cell tile stream of side-2h cells (sum over cells of the records of their "
                                    "27 neighbours) + 32 B per body"},
    })
    return out


def cpu_sph_rate(max_seconds=20.0):
    """The reference's own BH + SPH step (SPH mode A: Gaussian all-pairs,
    sph.c) on a sample of the same Plummer gas, extrapolated to N = 262,144 by
    N^2 (the all-pairs SPH passes dominate)."""
    from oracle import build as ob
    ob.build_oracle()
    from oracle.pyoracle import Oracle, make_params, slab_views
    from starflood_gb300.ics import plummer
    n = 16384
    pos, vel, mas = plummer(n, seed=7)
    orc = Oracle("f32")
    p = make_params(dt=5e-4, eps=0.01, theta=0.5, use_tree=1, use_sph=1)
    sim, slab, _ = orc.new_sim(n, p)
    v = slab_views(slab, n, 16)
    v["pos"][:] = pos
    v["vel"][:] = vel
    v["mas"][:] = mas
    v["rad"][:] = 0.05
    orc.sim_solv(p, sim, 0)
    t0 = time.perf_counter()
    steps = 0
    while steps < 1 or (time.perf_counter() - t0) < max_seconds and steps < 5:
        orc.sim_step(p, sim, steps)
        steps += 1
    dt = (time.perf_counter() - t0) / steps
    dt_full = dt * (N_SPH / n) ** 2
    return {"value": N_SPH / dt_full, "unit": "particle-steps/s", "cores": orc.threads(), "kind": "port",
            "sample": "%d sim_step calls (Barnes-Hut + reference SPH, Gaussian all-pairs) at N=%d, %.2f s each, "
                      "scaled by N^2 to N=%d" % (steps, n, dt, N_SPH)}


# ---------------------------------------------------------------------------
# batched + adjoint: 256 independent uniform spheres, N log-uniform in [1024, 32768]
# ---------------------------------------------------------------------------
def batch_inputs():
    from starflood_gb300.ics import log_uniform_sizes, uniform_ball
    sizes = log_uniform_sizes(256, 1024, 32768, seed=7)
    P, V, M = [], [], []
    for k, n in enumerate(sizes):
        p, v, m = uniform_ball(int(n), seed=1000 + k)
        P.append(p)
        V.append(v)
        M.append(m)
    return [int(x) for x in sizes], np.concatenate(P), np.concatenate(V), np.concatenate(M)


def fp64_pp(pos, mas, eps, idx):
    x = pos.astype(np.float64)
    m = mas.astype(np.float64)
    out = np.zeros((len(idx), 3))
    for a in range(0, len(idx), 512):
        ii = idx[a:a + 512]
        d = x[None, :, :] - x[ii][:, None, :]
        r2 = (d * d).sum(-1) + eps * eps
        out[a:a + 512] = (d * (m[None, :] / (r2 * np.sqrt(r2)))[..., None]).sum(1) * m[ii][:, None]
    return out


def gpu_batch(sf, steps=200, ckpt=20):
    import torch
    sizes, pos, vel, mas = batch_inputs()
    off = np.concatenate([[0], np.cumsum(sizes)])
    inter_per_eval = float(sum(n * n for n in sizes))
    p = sf.default_params(solver=sf.SOLVER_PP, eps=0.01, dt=1e-3)
    out = {"workload": "256 uniform spheres, N log-uniform in [1024, 32768] (total %d), PP eps=0.01, "
                       "%d KDK steps at dt=1e-3, loss = sum over systems of mean r^2 at the last step, "
                       "checkpoint every %d steps" % (int(off[-1]), steps, ckpt),
           "interactions_per_eval": inter_per_eval}
    check_sys = [int(np.argmin(sizes)), int(np.argsort(sizes)[len(sizes) // 2])]
    with sf.Batch(sizes, p) as b:
        b.upload(pos, vel, mas)
        b.solve()
        cfg = b.autotune()
        b.solve()
        _, _, acc, _ = b.download()
        errs = []
        for k in check_sys:
            sl = slice(off[k], off[k + 1])
            idx = np.arange(0, sizes[k], max(1, sizes[k] // 512))
            ref = fp64_pp(pos[sl], mas[sl], 0.01, idx)
            errs.append(float(np.linalg.norm(acc[sl][idx] - ref) / np.linalg.norm(ref)))
        ext = torch.cuda.ExternalStream(b.stream())
        b.run(3)
        b.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            e0.record(ext)
        b.run(steps)
        with torch.cuda.stream(ext):
            e1.record(ext)
        b.sync()
        fwd_ms = e0.elapsed_time(e1)
        t0 = time.perf_counter()
        b.run(steps)
        b.sync()
        fwd_wall = time.perf_counter() - t0
        b.upload(pos, vel, mas)
        t0 = time.perf_counter()
        loss, gp, gv = b.grad(steps, ckpt)
        adj_s = time.perf_counter() - t0
    out["batched"] = {"value": inter_per_eval * steps / (fwd_ms * 1e-3), "unit": "interactions/s",
                      "particle_steps_per_s": float(off[-1]) * steps / (fwd_ms * 1e-3), "ms": fwd_ms,
                      "wall_clock_value": inter_per_eval * steps / fwd_wall,
                      "tile_config": cfg, "force_error_vs_fp64": max(errs),
                      "launch": "one CUDA graph of all %d steps, persistent PP kernel per step" % steps}
    out["adjoint"] = {"seconds": adj_s, "loss": loss, "grad_finite": bool(np.isfinite(gp).all() and np.isfinite(gv).all()),
                      "note": "forward with checkpoints + reverse sweep with recomputation (host wall clock, "
                              "includes the gradient download)"}
    # plain form: one simulation per system, its own graph of the same steps
    sims, plain_errs = [], []
    try:
        for k, n in enumerate(sizes):
            sl = slice(off[k], off[k + 1])
            s = sf.Sim(n, p)
            s.set_state(pos[sl], vel[sl], mas[sl])
            s.solve(0)
            if k in check_sys:
                a = sf.slab_views(s.download(), n, 13)["acc"]
                idx = np.arange(0, n, max(1, n // 512))
                ref = fp64_pp(pos[sl], mas[sl], 0.01, idx)
                plain_errs.append(float(np.linalg.norm(a[idx] - ref) / np.linalg.norm(ref)))
            s.run(0, 1)
            sims.append(s)
        for s in sims:
            s.sync()
        t0 = time.perf_counter()
        for s in sims:
            s.run(1, steps)
        for s in sims:
            s.sync()
        plain_s = time.perf_counter() - t0
    finally:
        for s in sims:
            s.close()
    out["plain"] = {"value": inter_per_eval * steps / plain_s, "unit": "interactions/s", "seconds": plain_s,
                    "force_error_vs_fp64": max(plain_errs),
                    "launch": "one simulation per system, each a CUDA graph per step, host wall clock"}
    out["batched_over_plain"] = out["batched"]["value"] / out["plain"]["value"]
    return out


# ---------------------------------------------------------------------------
# vis_draw: splat rasteriser, N = 65,536 bodies x 128 samples into 1920 x 1080
# ---------------------------------------------------------------------------
def gpu_vis(sf, reps=5, sizex=1920, sizey=1080):
    import ctypes as C
    import torch
    pos, vel, mas = bh_inputs()
    n = N_BH
    L = sf.lib()
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5)
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.solve(0)
        s.sync()
        vp = (C.c_byte * 64)()
        L.sfgpu_vis_params_default(vp)
        da, dr = C.c_void_p(), C.c_void_p()
        sf.check(L.sfgpu_vis_buffers_alloc(sizex, sizey, C.byref(da), C.byref(dr)), "vis buffers")
        try:
            ext = torch.cuda.ExternalStream(s.stream())
            sf.check(L.sfgpu_vis_draw(s.h, vp, 0, sizex, sizey, da, dr), "vis")
            s.sync()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
            for k in range(reps):
                sf.check(L.sfgpu_flush_l2(C.c_void_p(s.stream())), "flush")
                with torch.cuda.stream(ext):
                    ev[k][0].record(ext)
                sf.check(L.sfgpu_vis_draw(s.h, vp, k + 1, sizex, sizey, da, dr), "vis")
                with torch.cuda.stream(ext):
                    ev[k][1].record(ext)
            s.sync()
            ms = sum(a.elapsed_time(b) for a, b in ev) / reps
            acc = np.zeros((sizey, sizex, 4), np.int32)
            sf.check(L.sfgpu_vis_download(s.h, sizex, sizey, da, dr, acc.ctypes.data, None), "download")
        finally:
            L.sfgpu_vis_buffers_free(da, dr)
        state = sf.slab_views(s.download(), n, 13)
    samples = n * 128
    out = {"workload": "vis_draw of the N=65536 Barnes-Hut state, 128 samples per body, 1920x1080, shipped "
                       "camera and tonemapping (L2 flushed before each draw)",
           "value": samples / (ms * 1e-3), "unit": "splat samples/s", "ms_per_frame": ms,
           "samples_in_frame": int(acc[..., 3].sum()),
           "atomic_bytes_per_frame": int(acc[..., 3].sum()) * 16}
    try:
        from oracle.pyoracle import Oracle
        orc = Oracle("f32")
        t0 = time.perf_counter()
        orc.vis_draw(state["pos"], state["vel"], state["pot"], 1, 1e-3, sizex, sizey)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": samples / dt, "unit": "splat samples/s", "cores": orc.threads(),
                               "kind": "port", "sample": "one orc_vis_draw frame of the same state (%.2f s)" % dt}
    except Exception as e:
        out["cpu_baseline"] = {"error": str(e)}
    return out


def gpu_pm(sf, reps=5, side=256):
    """Particle-mesh grid: the deposit (128 jittered samples per body) of the
    N=65536 Barnes-Hut state and grid_solve_fft on the reference's 256^3 grid
    over [-2, 2]^3 (GRID_SIZE 8).  The solve's compulsory HBM traffic: the
    R2C transform reads side^3 x 4 B and writes the half spectrum (side^2 x
    (side/2+1) x 8 B), the product reads it and the stencil's spectrum and
    writes it back, the C2R transform reads it and writes side^3 x 4 B."""
    import torch
    pos, vel, mas = bh_inputs()
    n = N_BH
    p = sf.default_params(solver=sf.SOLVER_TREE, eps=0.01, dt=1e-3, theta=0.5)
    cells = side ** 3
    half = side * side * (side // 2 + 1)
    solve_bytes = 4 * cells + 8 * half + 3 * 8 * half + 8 * half + 4 * cells
    with sf.Sim(n, p) as s:
        s.set_state(pos, vel, mas)
        s.sync()
        ext = torch.cuda.ExternalStream(s.stream())
        with sf.Grid(side, (-2.0, -2.0, -2.0), (2.0, 2.0, 2.0), G=1.0, stream=s.stream()) as g:
            g.deposit(s, 0)
            g.solve_fft()
            g.synchronize()
            ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(reps)]
            for k in range(reps):
                sf.check(sf.lib().sfgpu_flush_l2(s.stream()), "flush")
                with torch.cuda.stream(ext):
                    ev[k][0].record(ext)
                g.deposit(s, k + 1)
                with torch.cuda.stream(ext):
                    ev[k][1].record(ext)
                g.solve_fft()
                with torch.cuda.stream(ext):
                    ev[k][2].record(ext)
            g.synchronize()
            dep = sum(e[0].elapsed_time(e[1]) for e in ev) / reps
            sol = sum(e[1].elapsed_time(e[2]) for e in ev) / reps
            samp, acc = g.download(counts=True)
    gbs = solve_bytes / (sol * 1e-3) / 1e9
    peak, src = hbm_peak()
    out = {"workload": "deposit of the N=65536 Barnes-Hut state (128 samples per body) + grid_solve_fft on a "
                       "256^3 grid over [-2,2]^3 (R2C/C2R cuFFT, stencil spectrum cached; L2 flushed each rep)",
           "value": cells / (sol * 1e-3), "unit": "grid cells solved/s", "solve_ms": sol, "deposit_ms": dep,
           "deposit_samples_per_s": n * 128 / (dep * 1e-3), "samples_on_grid": int(acc.sum()),
           "roofline": {"kernel": "grid_solve_fft (cuFFT R2C + k_grid_mul + cuFFT C2R)", "bound": "hbm",
                        "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                        "algorithmic_bytes": solve_bytes, "peak_source": src},
           "potential_centre": float(samp[side // 2, side // 2, side // 2])}
    try:
        from oracle.pyoracle import Oracle
        orc = Oracle("f32")
        sub = 8192
        t0 = time.perf_counter()
        orc.grid_deposit(side, (-2.0, -2.0, -2.0), (2.0, 2.0, 2.0), pos[:sub], 1)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sub * 128 / dt, "unit": "deposit samples/s", "cores": orc.threads(),
                               "kind": "port", "sample": "orc_grid_deposit of %d bodies (%.2f s); the reference's "
                               "FFT solve needs FFTW, absent here, so it has no CPU timing" % (sub, dt)}
    except Exception as e:
        out["cpu_baseline"] = {"error": str(e)}
    return out


def profiled_traffic(name):
    """DRAM bytes per launch recorded in a profiles/ summary (the line
    'dram bytes per launch: N'), or None."""
    import re
    try:
        m = re.search(r"dram bytes per launch:\s*([0-9]+)", open(os.path.join(ROOT, "profiles", name)).read())
        return int(m.group(1)) if m else None
    except OSError:
        return None


def kdk_roofline(stages, n):
    """The two leapfrog kernels against the HBM copy bandwidth: kick+drift
    reads pos, vel, acc and writes pos, vel (60 B per body), kick+energies
    reads vel, acc, mas, pot and writes vel, ken, pen (52 B per body)."""
    peak, src = hbm_peak()
    out = {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": src,
           "note": "without SPH the second kick and the energies run in the walk's epilogue (no kick_energy stage)"}
    for key, b in (("kick_drift", 60), ("kick_energy", 52)):
        if key in stages and stages[key][1]:
            ms = stages[key][0] / stages[key][1]
            gbs = b * n / (ms * 1e-3) / 1e9
            out[key] = {"bytes_per_body": b, "ms": ms, "achieved": gbs, "frac": gbs / peak}
    return out


def max_over_ranks(t_ms, world):
    """The slowest rank's timed region (the job ends when it does); the
    process group is gloo, so this runs on host tensors."""
    if world <= 1:
        return t_ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([t_ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, n, steps, t_ms):
    """Whole-job particle-steps/s: every rank runs its own replica of n bodies
    for `steps` steps (weak scaling), all within the slowest rank's time."""
    return world * n * steps / (t_ms * 1e-3)


def bh_config(world):
    """The `config` object of both arms (same keys, so the two lines name the
    same workload)."""
    return {"workload": WORKLOAD, "N": N_BH, "leaf": 8, "theta": 0.5, "eps": 0.01, "dt": 1e-3,
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "flushed between timed steps (256 MiB memset, untimed)",
            "step": "one sim_step (kick, drift, bounds, tree build, walk, kick, energies)"}


def reference_line(args):
    """--impl reference: the reference path on the host cores (the FP32
    restatement, bit-identical to the compiled reference; OpenMP, all host
    threads).  `warmup` untimed steps, then `steps` timed steps."""
    from oracle import build as ob
    ob.build_oracle()
    from oracle.pyoracle import Oracle, make_params, slab_views
    pos, vel, mas = bh_inputs()
    n = N_BH
    orc = Oracle("f32")
    p = make_params(dt=1e-3, eps=0.01, theta=0.5, use_tree=1)
    sim, slab, _ = orc.new_sim(n, p)
    v = slab_views(slab, n, 13)
    v["pos"][:] = pos
    v["vel"][:] = vel
    v["mas"][:] = mas
    orc.sim_solv(p, sim, 0)
    for k in range(args.warmup):
        orc.sim_step(p, sim, k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        orc.sim_step(p, sim, args.warmup + k)
    dt = time.perf_counter() - t0
    value = n * args.steps / dt
    cb = {"value": value, "unit": "particle-steps/s", "cores": orc.threads(), "kind": "port",
          "sample": "%d timed sim_step calls of the N=%d Barnes-Hut workload after %d untimed (%.2f s)" % (
              args.steps, n, args.warmup, dt)}
    config = bh_config(1)
    config["parallelism"] = "host OpenMP, %d threads" % orc.threads()
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded uniform unit sphere, pcg4d)", "config": config, "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def compact_summary(line):
    """The sub-benchmarks' key figures, short enough to sit in the last
    ~1.4 kB of the line (what a log tail keeps)."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return float("%.4g" % d) if isinstance(d, float) else d
    out = {"headline_roofline_frac": g(line, "roofline", "frac"),
           "per_particle_err": {k: g(line, "per_particle_err", k)
                                for k in ("median", "p99", "max", "max_over_term_magnitudes")}}
    pp = line.get("pp")
    if isinstance(pp, dict):
        out["pp"] = {"plain_ips": g(pp, "plain", "interactions_per_s"),
                     "comp_ips": g(pp, "compensated", "interactions_per_s"),
                     "comp_over_plain": g(pp, "compensated_over_plain"),
                     "exact_ips": g(pp, "plain_exact", "interactions_per_s"),
                     "comp_over_plain_at_1e-6": g(pp, "compensated_over_plain_at_1e-6"),
                     "plain_frac": g(pp, "plain", "roofline_frac"), "comp_frac": g(pp, "compensated", "roofline_frac"),
                     "err_fp64": {k: g(pp, "force_error_vs_fp64", k) for k in ("plain", "compensated", "plain_exact")},
                     "err_fp64_per_particle_max": {k: g(pp, "force_error_vs_fp64", k + "_per_particle", "max")
                                                   for k in ("plain", "compensated", "plain_exact")},
                     "drift": {k: g(pp, "energy_drift_20_steps", k, "relative_drift") for k in ("plain", "compensated")}}
    for key in ("sph", "sph_reference"):
        sp = line.get(key)
        if isinstance(sp, dict):
            out[key] = {"value": g(sp, "value"), "ms": g(sp, "ms_per_step"), "frac": g(sp, "roofline", "frac"),
                        "vs_cpu_mode_a": g(sp, "vs_cpu_mode_a")}
    bt = line.get("batch")
    if isinstance(bt, dict):
        out["batch"] = {"ips": g(bt, "batched", "value"), "over_plain": g(bt, "batched_over_plain"),
                        "err_fp64": g(bt, "batched", "force_error_vs_fp64"), "adjoint_s": g(bt, "adjoint", "seconds")}
    out["bh_variants"] = {k: g(line, "bh_variants", k, "value") for k in ("leaf16", "exact")}
    out["walk_frac_vs_n"] = {k: g(v, "walk_frac") for k, v in (line.get("walk_vs_n") or {}).items()}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-pp", action="store_true", help="skip the N=1M PP sub-benchmark")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-sph", action="store_true", help="skip the N=262144 Barnes-Hut + SPH sub-benchmarks")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched + adjoint sub-benchmark")
    ap.add_argument("--no-vis", action="store_true", help="skip the vis_draw splat sub-benchmark")
    ap.add_argument("--no-pm", action="store_true", help="skip the particle-mesh grid sub-benchmark")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the leaf-16 / EXACT lines, the walk at larger N and the per-particle error")
    ap.add_argument("--walk-split", type=int, default=0, help="Barnes-Hut walk variant (sfgpu_params.walk_split)")
    ap.add_argument("--walk-group", type=int, default=0, help="bodies per warp of the group walk (sfgpu_params.walk_group)")
    ap.add_argument("--only", choices=["pp", "sph", "sph_reference", "pm", "batch"], default=None,
                    help="run one sub-benchmark alone and print its object (profiling runs)")
    ap.add_argument("--pp-n", type=int, default=N_PP, help="bodies of the PP sub-benchmark with --only pp")
    ap.add_argument("--sph-path", type=int, default=0, help="SPH pass variant with --only sph (sfgpu_params.sph_path)")
    args = ap.parse_args()
    if args.walk_split:
        BH_EXTRA["walk_split"] = args.walk_split
    if args.walk_group:
        BH_EXTRA["walk_group"] = args.walk_group
    rank, world, local = env_rank()

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(reference_line(args)))
        return

    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    import __graft_entry__
    if rank == 0 or not os.path.exists(os.path.join(ROOT, "starflood_gb300", "libsfgpu.so")):
        __graft_entry__.build()
    if world > 1:
        dist.barrier()
    import starflood_gb300 as sf

    if args.only == "pp":
        print(json.dumps({"only": "pp", "n": args.pp_n, "pp": gpu_pp(sf, n=args.pp_n)}))
        return
    if args.only == "pm":
        print(json.dumps({"only": "pm", "pm": gpu_pm(sf)}))
        return
    if args.only == "batch":
        print(json.dumps({"only": "batch", "batch": gpu_batch(sf)}))
        return
    if args.only in ("sph", "sph_reference"):
        mode = "cubic" if args.only == "sph" else "reference"
        print(json.dumps({"only": args.only, args.only: gpu_sph(sf, max(3, args.steps), args.warmup, args.sph_path,
                                                              mode=mode)}))
        return

    r = gpu_bh(args.steps, args.warmup, sf)
    t_ms = r["total_ms"]
    t_ms = max_over_ranks(t_ms, world)
    value = job_value(world, N_BH, args.steps, t_ms)

    peak, peak_src = fp32_peak_tflops()
    walk_ms, walk_launches = r["stages"].get("walk", (0.0, 0))
    walk_avg_ms = walk_ms / max(1, walk_launches)
    flops_per_launch = (FLOP_INTERACTION * r["n_int"] + FLOP_OPEN * r["n_open"]) / max(1, walk_launches)
    achieved = flops_per_launch / (walk_avg_ms * 1e-3) / 1e12 if walk_avg_ms > 0 else 0.0
    stage_ms = {k: round(v[0] / max(1, v[1]), 4) for k, v in r["stages"].items()}

    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform unit sphere, pcg4d)",
            "config": bh_config(world),
            "clocks": r["clocks"], "e2e": r["e2e"], "gpu_launches": r["per_step"] * args.steps,
            "roofline": {"kernel": "k_walk_sib (Barnes-Hut group walk over sibling groups; its epilogue also "
                                   "applies the second kick and the energy sums, included in its duration)",
                         "bound": "fp32", "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                         "traffic": profiled_traffic("walk_sib_uniform65536.md"),
                         "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum per launch, "
                                           "profiles/walk_sib_uniform65536.md (ncu)",
                         "peak_source": peak_src,
                         "flops_per_launch": flops_per_launch, "avg_launch_ms": walk_avg_ms,
                         "interactions_per_step": r["n_int"] / max(1, walk_launches),
                         "opening_tests_per_step": r["n_open"] / max(1, walk_launches)},
            "stage_ms_per_step": stage_ms, "device_status": r["status"],
            "kdk": kdk_roofline(r["stages"], N_BH)}
    if rank == 0:
        try:
            line["cpu_baseline"] = {"skipped": "--no-cpu"} if args.no_cpu else cpu_bh_rate(max_seconds=10.0)
        except Exception as e:  # the baseline must not hide the GPU line
            line["cpu_baseline"] = {"error": str(e)}
        if not args.no_extra:
            for key, fn in (("per_particle_err", lambda: bh_per_particle_err(sf)),
                            ("bh_variants", lambda: bh_variant_rates(sf)), ("walk_vs_n", lambda: walk_vs_n(sf))):
                try:
                    line[key] = fn()
                except Exception as e:
                    line[key] = {"error": str(e)}
        if not args.no_pp:
            pp = gpu_pp(sf)
            try:
                pp["force_error_vs_fp64"] = pp_accuracy(sf)
            except Exception as e:
                pp["force_error_vs_fp64"] = {"error": str(e)}
            try:
                pp["energy_drift_20_steps"] = pp_energy_drift(sf)
            except Exception as e:
                pp["energy_drift_20_steps"] = {"error": str(e)}
            for k in ("plain", "compensated", "plain_exact"):
                if k in pp:
                    pp[k]["roofline_frac"] = pp[k]["interactions_per_s"] * FLOP_INTERACTION / (peak * 1e12)
            pp["compensated_over_plain"] = pp["compensated"]["interactions_per_s"] / pp["plain"]["interactions_per_s"]
            if "plain_exact" in pp:
                # at force error <= 1e-6 of FP64 the plain form needs EXACT arithmetic (FAST: about 3e-6)
                pp["compensated_over_plain_at_1e-6"] = (pp["compensated"]["interactions_per_s"] /
                                                        pp["plain_exact"]["interactions_per_s"])
            try:
                pp["cpu_baseline"] = {"skipped": "--no-cpu"} if args.no_cpu else cpu_pp_rate()
            except Exception as e:
                pp["cpu_baseline"] = {"error": str(e)}
            pp["workload"] = "PP gravity N=1048576 Plummer a=1 M=1 eps=0.005, %d flop/interaction" % FLOP_INTERACTION
            line["pp"] = pp
        if not args.no_sph:
            nsteps = max(10, min(args.steps, 50))
            try:
                cpu_a = None if args.no_cpu else cpu_sph_rate()
            except Exception as e:
                cpu_a = {"error": str(e)}
            for key, mode in (("sph", "cubic"), ("sph_reference", "reference")):
                sp = gpu_sph(sf, nsteps if mode == "cubic" else max(3, nsteps // 5), args.warmup, mode=mode)
                sp["cpu_baseline"] = cpu_a if cpu_a is not None else {"skipped": "--no-cpu"}
                if isinstance(cpu_a, dict) and "value" in cpu_a:
                    sp["vs_cpu_mode_a"] = sp["value"] / cpu_a["value"]
                    sp["vs_cpu_mode_a_kind"] = ("like for like: the reference's SPH on both sides" if mode != "cubic"
                                                else "cross-algorithm: cubic-spline SPH on the GPU against the "
                                                     "reference's Gaussian all-pairs SPH on the CPU")
                line[key] = sp
        if not args.no_batch:
            bt = gpu_batch(sf)
            if not args.no_cpu and isinstance(line.get("pp", {}).get("cpu_baseline"), dict) \
                    and "value" in line["pp"]["cpu_baseline"]:
                cpu = line["pp"]["cpu_baseline"]
                bt["cpu_baseline"] = dict(cpu, sample=cpu["sample"] + "; the batched workload at this rate")
            line["batch"] = bt
        if not args.no_vis:
            try:
                line["vis"] = gpu_vis(sf)
            except Exception as e:
                line["vis"] = {"error": str(e)}
        if not args.no_pm:
            try:
                line["pm"] = gpu_pm(sf)
            except Exception as e:
                line["pm"] = {"error": str(e)}
        line["summary"] = compact_summary(line)
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
