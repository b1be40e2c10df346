#!/usr/bin/env python
"""Benchmark: atom-timesteps/s of the 1M-atom LJ NVE step (mixed precision vs FP64).

Workload (the benchmark's configuration 1): N = 1,048,576 LJ atoms
(eps = 1, sigma = 1, cut 2.5 sigma') on a 128x128x64 simple-cubic lattice at
number density 0.8 sigma'^-3 with a +-0.05 sigma' jitter, Gaussian velocities
at T = 1, neighbour-list skin 0.3 sigma', CollectionVerlet with dt = 0.002.
A "step" is one time step of the whole system (drift, pair forces, kick,
rebuild test, and the list rebuild whenever the test fires).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun every rank runs an independent
replica of the system (the single-system step has no data-parallel split).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "atom-timesteps/s (1M LJ, mixed vs FP64) at stated error"
UNIT = "atom-timesteps/s"
DT = 0.002
SHAPE = (128, 128, 64)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """Largest `value` over all ranks (the slowest replica sets the job time)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(atoms_per_rank: int, steps: int, ms_max: float, world: int) -> float:
    """Whole-job atom-timesteps/s: every rank advances its own replica (weak scaling)."""
    return world * atoms_per_rank * steps / (ms_max / 1000.0)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def traffic_from_profiles(kernel: str):
    """DRAM bytes per launch of `kernel` on this workload from its committed ncu summary."""
    p = ROOT / "profiles" / f"{kernel}_lj1m.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class Clocks:
    """Sample nvidia-smi clocks / throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_system(w, precision, device):
    from parm_gb300 import System
    s = System(w.sizes, ndim=w.ndim, precision=precision)
    s.set_boxes(w.L)
    s.set_atoms(x=w.x, v=w.v, a=np.zeros_like(w.x), f=np.zeros_like(w.x), m=w.m)
    s.set_interaction(w.kind, w.params, w.skin)
    # Collection::initialize
    s.nlist_update(False)
    s.set_forces(True)
    s.nlist_update(False)
    return s


def host_cpu() -> str:
    """Core model and count of this host (for the CPU baseline's description)."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return f"{model or 'unknown CPU'}, {os.cpu_count()} logical cores"


def cpu_baseline_sample(w, max_steps=3):
    """Time the oracle (a single-threaded restatement of the reference step) on the same system.

    The reference's O(N^2) list build is infeasible at 1M atoms; the list is
    installed through the oracle's cell-list construction (same pair set, not
    timed) and only time steps without a rebuild are timed.  The O(N^2)
    rebuild cost is measured at 16384 atoms and extrapolated by N^2.
    """
    from oracle.oracle import Oracle
    o = Oracle(w.n, 3)
    o.set_box(w.L[0])
    o.set_state(x=w.x, v=w.v, a=np.zeros_like(w.x), f=np.zeros_like(w.x), m=w.m)
    o.set_interaction(w.kind, w.params, w.skin)
    o.build_fast()
    o.set_forces(True)
    which0 = o.which()
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        o.verlet(DT, 1)
        steps += 1
        if time.perf_counter() - t0 > 25:
            break
    dt = time.perf_counter() - t0
    rebuilt = o.which() != which0
    del o
    tb, t_rebuild = rebuild_cost(w.n)
    return {"value": w.n * steps / dt, "steps": steps, "seconds": dt, "rebuilt": rebuilt,
            "rebuild_s_16k": tb, "rebuild_s_extrapolated": t_rebuild}


def rebuild_cost(n_target: int):
    """The reference's O(N^2) NeighborList::update_list(true) timed at 16384 atoms (oracle port, one
    thread) and extrapolated by N^2 to `n_target` atoms: (seconds at 16384, extrapolated seconds)."""
    from oracle.oracle import Oracle
    from parm_gb300 import workloads as W
    ws = W.lj_lattice(shape=(32, 32, 16), skin_prime=0.3)
    o = Oracle(ws.n, 3)
    o.set_box(ws.L[0])
    o.set_state(x=ws.x, v=ws.v, m=ws.m)
    o.set_interaction(ws.kind, ws.params, ws.skin)
    t1 = time.perf_counter()
    o.nl_update(True)
    tb = time.perf_counter() - t1
    return tb, tb * (n_target / ws.n) ** 2


def _replica_steps(job):
    """One host thread: `warm` untimed, then `steps` timed oracle steps of an independent replica
    (spawned process)."""
    seed, steps, warm = job
    import numpy as np_
    from oracle.oracle import Oracle
    from parm_gb300 import workloads as W
    w = W.lj_lattice(shape=SHAPE, skin_prime=0.3, seed=seed)
    o = Oracle(w.n, 3)
    o.set_box(w.L[0])
    o.set_state(x=w.x, v=w.v, a=np_.zeros_like(w.x), f=np_.zeros_like(w.x), m=w.m)
    o.set_interaction(w.kind, w.params, w.skin)
    o.build_fast()
    o.set_forces(True)
    if warm:
        o.verlet(DT, warm)
    t0 = time.perf_counter()
    o.verlet(DT, steps)
    return w.n * steps, time.perf_counter() - t0, t0


def run_reference(args, rank):
    """The reference's CPU step (the oracle port, bit-exact with it) on every host thread.

    Each host thread runs an independent replica of the 1M-atom system (the
    reference step is single-threaded); value = all replicas' atom-steps over
    the wall time from the first start to the last finish.
    """
    import multiprocessing as mp
    from oracle.build import build as build_oracle
    build_oracle()
    ncpu = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    nrep = max(1, min(ncpu, 64))
    steps = max(1, min(args.steps, 3))
    warm = max(0, min(args.warmup, 3))
    ctx = mp.get_context("spawn")
    with ctx.Pool(nrep) as pool:
        res = pool.map(_replica_steps, [(12345 + r, steps, warm) for r in range(nrep)])
    total = sum(r[0] for r in res)
    wall = max(r[2] + r[1] for r in res) - min(r[2] for r in res)
    value = total / wall
    n = res[0][0] // steps
    tb, t_rebuild = rebuild_cost(n)
    sample = (f"oracle port of the reference step (bit-exact with the reference's compiled sources), "
              f"{nrep} independent {n}-atom replicas, one per host thread of {host_cpu()}, {warm} untimed + {steps} "
              f"timed CollectionVerlet steps each without a list rebuild ({wall:.1f} s wall); the reference's "
              f"O(N^2) list rebuild "
              f"(~{t_rebuild:.3g} s per rebuild at this size, extrapolated by N^2 from {tb:.2f} s measured "
              f"at 16384 atoms) is excluded")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
           "warmup": warm, "ms_per_step": 1000 * wall / steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": f"lj_nve_{n}_atoms", "n_atoms": n, "dt": DT,
                      "skin_sigma": 0.3 * 2.0 ** (-1.0 / 6.0), "lattice": list(SHAPE),
                      "replicas": nrep},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": nrep, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if rank == 0:
        print(json.dumps(out), flush=True)


def _timed_verlet(g, steps, stream, dist=None, clocks=None):
    """Time `steps` Verlet steps of handle `g` between CUDA events on its stream (graphs already captured)."""
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    ev0.record(stream)
    g.verlet(DT, steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    ck = clocks.stop() if clocks else None
    return ev0.elapsed_time(ev1), ck


def _capture_graphs(g, steps, graph_steps):
    """Run the graph shapes a call of `steps` steps uses (full chunks and the remainder), so that capture
    and instantiation happen before a timed region."""
    if graph_steps:
        g.verlet(DT, min(steps, graph_steps))
        if steps % graph_steps and steps > graph_steps:
            g.verlet(DT, steps % graph_steps)
    else:
        g.verlet(DT, 1)
    g.sync()


def energy_drift(w, precision, steps, sample_every=100, graph_steps=50):
    """NVE drift of one path from the workload's initial state: total energy sampled every `sample_every`
    steps over `steps` steps, least-squares slope scaled to 10^5 steps relative to |E(0)|."""
    g = make_system(w, precision, 0)
    g.set_graph_steps(graph_steps)
    if precision == "mixed":
        g.autotune()
    E = [g.energy()[0] + g.kinetic_energy()[0]]
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        k = min(sample_every, steps - done)
        g.verlet(DT, k)
        done += k
        E.append(g.energy()[0] + g.kinetic_energy()[0])
    wall = time.perf_counter() - t0
    g.close()
    E = np.array(E)
    t = np.concatenate([[0], np.cumsum([min(sample_every, steps - q) for q in range(0, steps, sample_every)])])
    A = np.stack([t, np.ones_like(t)], 1).astype(np.float64)
    coef, res, *_ = np.linalg.lstsq(A, E, rcond=None)
    resid = E - A @ coef
    dof = max(1, len(E) - 2)
    se = math.sqrt((resid ** 2).sum() / dof / ((t - t.mean()) ** 2).sum())
    scale = 1e5 / abs(E[0])
    # the energy error is correlated over many steps, so the least-squares error understates the slope's
    # spread; the spread of the slopes of five consecutive blocks gives a second estimate
    nb = 5
    blk = [q for q in np.array_split(np.arange(len(E)), nb) if len(q) >= 3]
    bslopes = [np.polyfit(t[q], E[q], 1)[0] for q in blk]
    se_blk = float(np.std(bslopes, ddof=1) / math.sqrt(len(bslopes)) * scale) if len(bslopes) > 1 else None
    return {"per_1e5_steps": float(coef[0] * scale), "std_err": float(se * scale), "std_err_blocks": se_blk,
            "block_slopes_per_1e5_steps": [float(b * scale) for b in bslopes], "steps": int(steps),
            "samples": int(len(E)), "rms_fluctuation_rel": float(resid.std() / abs(E[0])),
            "net_change_rel": float((E[-1] - E[0]) / abs(E[0])), "wall_s": wall}


def run_ours(args, rank, world, local_rank):
    import torch
    from parm_gb300 import capi, workloads as W
    lib = capi.load()
    capi.check(lib.parm_use_device(local_rank))
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    w = W.lj_lattice(shape=SHAPE, skin_prime=0.3, seed=12345 + rank)
    n = w.n
    log(f"[rank {rank}] building mixed system, n={n}")
    g = make_system(w, "mixed", local_rank)
    g.set_graph_steps(args.graph_steps)
    variant = g.autotune() if args.tpa == 0 else (g.set_threads_per_atom(args.tpa) or args.tpa)
    log(f"[rank {rank}] kernel variant: {variant}")
    g.verlet(DT, args.warmup)
    if args.rsq:
        # the device mean-square-displacement tracker, updated inside every step
        g.rsq_start([1, 10, 100], usecom=True)
    _capture_graphs(g, args.steps, args.graph_steps)
    stream = torch.cuda.ExternalStream(g.stream())
    clocks = Clocks(local_rank)

    # --- the timed region: K steps, graphs captured beforehand, no per-kernel events ---
    ms, ck = _timed_verlet(g, args.steps, stream, dist, clocks)
    launches = g.last_launches()
    if dist:
        ms = max_over_ranks(ms, dist, "cuda")
        dist.barrier()
    value = job_throughput(n, args.steps, ms, world)
    npairs = int(g.numpairs()[0])

    # --- per-kernel durations (CUDA events around the force kernels of every step), a separate run ---
    g.timing(True)
    _capture_graphs(g, args.steps, args.graph_steps)
    g.timing(True)   # resets the counters
    ms_t, _ = _timed_verlet(g, args.steps, stream)
    tr = g.timing_read()
    g.timing(False)

    # --- roofline of the dominant kernel (the mixed pair-force kernel) ---
    # algorithmic bytes per atom-timestep of the mixed step (fused, list
    # reused): x and v in FP64 read and written (96 B), the FP32 force/
    # acceleration read and written (24 B) and 4 B per half-list pair; one
    # launch of the force kernel advances every atom by one step
    force_ms = tr["force_ms"] / max(1, tr["force_launches"])
    n_half = npairs / n
    staged = variant == 2000 or variant == 200
    kernel = "k_force_stg" if staged else "k_force32"
    bytes_per_atom = 96.0 + 24.0 + 4.0 * n_half
    algo_bytes = n * bytes_per_atom
    achieved = algo_bytes / (force_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = traffic_from_profiles(kernel)

    result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (mixed)", "data": "synthetic",
              "config": {"workload": f"lj_nve_{n}_atoms_mixed", "n_atoms": n, "lattice": list(SHAPE),
                         "box": [float(v) for v in w.L[0]], "dt": DT, "skin_sigma": w.skin,
                         "cutoff_sigma": float(w.params[0, 2]), "precision": "mixed",
                         "parallelism": f"replicas{world}" if world > 1 else "single",
                         "l2": "inputs larger than L2 (state + neighbour lists ~1 GB)",
                         "steps_per_graph": args.graph_steps, "kernel_variant": variant},
              "clocks": ck,
              "gpu_launches": launches,
              "rebuilds": tr["rebuilds"]}
    result["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": traffic,
                          "kernel": f"{kernel} (mixed-precision pair forces)",
                          "algorithmic_bytes_per_atom": bytes_per_atom, "half_list_pairs_per_atom": n_half,
                          "step_achieved_gbs": bytes_per_atom * value / 1e9,
                          "algorithmic_bytes_per_launch": algo_bytes, "force_ms_per_launch": force_ms,
                          "timing_run_ms_per_step": ms_t / args.steps,
                          "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                          else "fallback 6800 GB/s"}
    if args.rsq:
        result["config"]["msd_tracker"] = "device RsqTracker, windows of 1, 10, 100 steps, centre of mass"

    if args.only_timed:
        g.close()
        if rank == 0:
            print(json.dumps(result), flush=True)
        return

    # --- FP64 path on the same system, and mixed-vs-FP64 error at one state ---
    st = g.get_atoms(capi.X | capi.V | capi.A)
    # the equilibrated state after the timed runs: start of the drift fits
    from dataclasses import replace
    w_eq = replace(w, x=st["x"].copy(), v=st["v"].copy())
    w64 = W.lj_lattice(shape=SHAPE, skin_prime=0.3, seed=12345 + rank)
    w64.x, w64.v = st["x"], st["v"]
    g64 = make_system(w64, "fp64", local_rank)
    g64.set_graph_steps(args.graph_steps)
    k64 = max(1, args.fp64_steps)
    g64.verlet(DT, 2)
    _capture_graphs(g64, k64, args.graph_steps)
    s64 = torch.cuda.ExternalStream(g64.stream())
    ms64, _ = _timed_verlet(g64, k64, s64)
    v64 = n * k64 / (ms64 / 1000.0)
    # forces at one common state
    st64 = g64.get_atoms(capi.X)
    g.set_atoms(x=st64["x"])
    g.nlist_update(True)
    g64.nlist_update(True)
    g.set_forces(False)
    g64.set_forces(False)
    F32 = g.get_atoms(capi.F)["f"]
    F64 = g64.get_atoms(capi.F)["f"]
    ferr = float(np.sqrt(((F32 - F64) ** 2).sum(1)).max() / np.sqrt((F64 ** 2).sum(1).mean()))
    E32, E64 = g.energy()[0], g64.energy()[0]
    result["fp64_value"] = world * v64
    result["fp64_steps_timed"] = k64
    result["mixed_vs_fp64"] = value / (world * v64)
    result["accuracy"] = {"max_force_err_over_rms_force": ferr, "rel_energy_err": abs(E32 - E64) / abs(E64)}
    g64.close()

    # --- end to end through the C ABI with host buffers ---
    stride = 4 * 3 + 1
    nbytes = n * stride * 8
    import ctypes as C
    hp = C.c_void_p()
    capi.check(lib.parm_host_alloc(C.byref(hp), nbytes))
    buf = np.ctypeslib.as_array((C.c_double * (n * stride)).from_address(hp.value)).reshape(n, stride)
    cur = g.get_atoms()
    buf[:, 0:3], buf[:, 3:6], buf[:, 6:9], buf[:, 9:12], buf[:, 12] = cur["x"], cur["v"], cur["a"], cur["f"], cur["m"]
    fields = capi.X | capi.V | capi.A | capi.F | capi.M   # whole Atom records, as an AtomVec holds them
    dptr = buf.ctypes.data_as(C.POINTER(C.c_double))
    n_e2e = max(3, min(args.e2e_steps, args.steps))
    for _ in range(2):
        capi.check(lib.parm_set_atoms(g.h, dptr, stride, fields))
        capi.check(lib.parm_verlet(g.h, DT, 1))
        capi.check(lib.parm_get_atoms(g.h, dptr, stride, fields))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        capi.check(lib.parm_set_atoms(g.h, dptr, stride, fields))
        capi.check(lib.parm_verlet(g.h, DT, 1))
        capi.check(lib.parm_get_atoms(g.h, dptr, stride, fields))
    t_e2e = time.perf_counter() - t0
    if dist:
        t_e2e = max_over_ranks(t_e2e, dist, "cuda")
    result["e2e"] = {"value": world * n * n_e2e / t_e2e, "unit": UNIT, "h2d_bytes_per_step": n * stride * 8,
                     "d2h_bytes_per_step": n * stride * 8, "steps": n_e2e,
                     "api": "parm_set_atoms + parm_verlet(dt, 1) + parm_get_atoms on whole Atom records "
                            "{x,v,a,f,m} in pinned host memory"}
    lib.parm_host_free(hp)
    g.close()

    # --- NVE energy drift of both paths from the same initial state (fitted slope) ---
    if args.drift_steps > 0 and rank == 0:
        log(f"[rank 0] NVE drift over {args.drift_steps} steps, mixed and FP64")
        dm = energy_drift(w_eq, "mixed", args.drift_steps, graph_steps=args.graph_steps)
        d64 = energy_drift(w_eq, "fp64", args.drift_steps, graph_steps=args.graph_steps)
        result["drift"] = {"mixed": dm, "fp64": d64,
                           "ratio_mixed_over_fp64": dm["per_1e5_steps"] / d64["per_1e5_steps"]
                           if d64["per_1e5_steps"] != 0 else None,
                           "definition": "least-squares slope of E_total(t) sampled every 100 steps, "
                                         "times 1e5 steps, over |E_total(0)|, both paths from the same state: "
                                         "the mixed run's state after its warm-up and timed steps"}

    if rank == 0 and world == 1 and not args.no_cpu:
        log("[rank 0] timing the CPU oracle sample")
        s = cpu_baseline_sample(w)
        result["cpu_baseline"] = {
            "value": s["value"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": (f"oracle port, {s['steps']} CollectionVerlet steps of the same {n}-atom system on one "
                       f"host thread of {host_cpu()} ({s['seconds']:.1f} s), list installed by the cell-list construction "
                       f"(untimed); reference O(N^2) rebuild: {s['rebuild_s_16k']:.2f} s at 16384 atoms, "
                       f"~{s['rebuild_s_extrapolated']:.0f} s extrapolated to {n} (excluded)")}
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result), flush=True)


# ---------------------------------------------------------------------------
# further workloads (not the headline line): batched packings, Langevin
# replicas and the 2D disk minimisation; each prints its own JSON line
# ---------------------------------------------------------------------------
def _sync_time(g):
    g.sync()
    return time.perf_counter()


# CollectionNLCGV (fixed box) parameters of the packing minimisations: the
# constructor's defaults (src/collection.cpp:877-898) with dt = 0.1
CG_PARAMS = np.array([0.1, 0.0, 1.0, 1000, 10, 1e-4, 0.0, 0.0, 0.0, 0.0, 0.0])


def _cg_handle(ws, precision, tune=False, cell_scale=1.0):
    """A handle with CollectionNLCGV set up on every system (Collection initialise, then reset())."""
    g = make_system(ws, precision, 0)
    g.set_graph_steps(25)
    if cell_scale != 1.0:
        g.set_cell_scale(cell_scale)
        g.nlist_update(False)
    variant = g.autotune() if (tune and precision == "mixed") else None
    g.nlcg_init(CG_PARAMS, boxed=False)
    g.nlcg_reset()
    return g, variant


def _cg_prepare(g):
    g.nlcg_init(CG_PARAMS, boxed=False)
    g.nlcg_reset()


def _tuned(w, make, step, skins, prepare=None):
    """The workload with the autotuned skin, the cell scale, and the tuner's summary."""
    from dataclasses import replace
    from parm_gb300 import autotune
    res = autotune.tune(w, make, step, skins, cell_scales=(1.0, 1.5), prepare=prepare)
    log(f"autotune: skin {res['skin']}, cell scale {res['cell_scale']}, variant {res['variant']}")
    return replace(w, skin=res["skin"]), res["cell_scale"], autotune.summarise(res)


def _minimise_cg(g, tol, max_steps, chunk, stall=0):
    """Conjugate-gradient time steps until every system's max |F| < tol (finished systems frozen).

    stall > 0: a system also finishes when its max |F| fell by less than a
    factor 2 over its last `stall` checks (the floor of FP32 forces, for the
    mixed-precision phase)."""
    nsys = g.nsys
    act = np.ones(nsys, bool)
    steps = np.zeros(nsys, dtype=np.int64)
    hist = []
    done = 0
    while done < max_steps and act.any():
        g.set_active(act)
        g.nlcg_timestep(chunk)
        steps[act] += chunk
        done += chunk
        fmax = np.sqrt(g.max_force_sq())
        hist.append(fmax)
        fin = fmax < tol
        if stall and len(hist) > stall:
            fin |= fmax > 0.5 * hist[-1 - stall]
        act &= ~fin
    g.set_active(np.ones(nsys, bool))
    return steps, np.sqrt(g.max_force_sq())


def _cg_protocol(ws, tol32, tol64, cap32, cap64, chunk, tune=False, cell_scale=1.0, stall=4):
    """Mixed-precision conjugate-gradient bulk phase (until max|F| < tol32 or its FP32 floor), then an FP64
    phase from its positions to max|F| < tol64."""
    g, variant = _cg_handle(ws, "mixed", tune, cell_scale)
    ta = _sync_time(g)
    s32, f32 = _minimise_cg(g, tol32, cap32, chunk, stall)
    x = g.get_atoms(1)["x"]
    tb = _sync_time(g)
    g.close()
    from parm_gb300 import workloads as W
    w64 = W.Workload(ws.name, ws.ndim, ws.sizes, ws.L, x, np.zeros_like(x), ws.m, ws.kind, ws.params, ws.skin)
    g64, _ = _cg_handle(w64, "fp64", cell_scale=cell_scale)
    tc = _sync_time(g64)
    s64, f64 = _minimise_cg(g64, tol64, cap64, chunk)
    td = _sync_time(g64)
    E = g64.energy()
    g64.close()
    return {"variant": variant, "t32": tb - ta, "t64": td - tc, "f32": f32, "f64": f64, "E": E, "s32": s32,
            "s64": s64}


def run_packings(args):
    """Batched 3D packings minimised by the conjugate-gradient minimiser (CollectionNLCGV, fixed box).

    Every system: a mixed-precision phase until max |F| < 1e-7 (about the
    error of FP32 forces on these contacts), then an FP64 phase until
    max |F| < 1e-12; finished systems are frozen while the others continue.  A packing counts only when its system reached
    max |F| < 1e-12 within the step caps.  Reported: converged packings/s of
    the batch, the converged fraction, the same protocol run one system per
    handle and launch (speed-up), and the final-energy error of converged
    systems against an FP64-only minimisation of a sample of systems.
    """
    from parm_gb300 import shard, workloads as W
    nsys = args.nsys or 4096
    w = W.packings(nsys=nsys, nmin=64, nmax=4096, phi_lo=0.62, phi_hi=0.66, exponent=2.5, seed=3, skin=args.skin)
    # FP32 forces on these contacts carry ~1e-7 of error, so the mixed phase ends at 1e-7
    tol32, tol64, chunk = 1e-7, 1e-12, 250
    cap32, cap64 = args.min_steps, args.fp64_cap
    log(f"packings: {nsys} systems, {w.n} atoms")
    # skin, cell width and kernel variant tuned on the batch's first systems
    w, cscale, tuned = _tuned(w, lambda ws: make_system(ws, "mixed", 0), lambda g, k: g.nlcg_timestep(k),
                              (0.05, 0.1, 0.2, 0.3), prepare=_cg_prepare)
    r = _cg_protocol(w, tol32, tol64, cap32, cap64, chunk, tune=True, cell_scale=cscale, stall=0)
    wall = r["t32"] + r["t64"]
    conv = r["f64"] < tol64
    value = float(conv.sum()) / wall
    # FP64-only minimisation of a sample (same tolerance and total cap)
    ns = min(nsys, args.sample_sys)
    gr, _ = _cg_handle(shard.select(w, list(range(ns))), "fp64")
    _, fr = _minimise_cg(gr, tol64, cap32 + cap64, chunk)
    Er = gr.energy()
    gr.close()
    both = conv[:ns] & (fr < tol64)
    sizes_s = np.asarray(w.sizes[:ns], dtype=np.float64)
    e_mix, e_64 = r["E"][:ns] / sizes_s, Er / sizes_s
    # below jamming both minima have zero energy (to rounding); above it the
    # two runs (different force rounding from the first step) can end in
    # different minima of the same landscape
    unjammed = both & (e_mix < 1e-16) & (e_64 < 1e-16)
    jammed = both & ~unjammed
    rel = np.abs(e_mix - e_64) / np.maximum(np.abs(e_64), 1e-300)
    same = jammed & (rel < 1e-6)
    # one system per handle and launch sequence, same protocol
    nsingle = min(nsys, args.single_sys)
    t_single, c_single = 0.0, 0
    for q in range(nsingle):
        rs = _cg_protocol(shard.select(w, [q]), tol32, tol64, cap32, cap64, chunk, cell_scale=cscale, stall=0)
        t_single += rs["t32"] + rs["t64"]
        c_single += int((rs["f64"] < tol64).sum())
    single_rate = c_single / t_single
    sizes = np.asarray(w.sizes)
    out = {"metric": "converged packings/s (batched 3D soft-sphere conjugate-gradient minimisation to max|F| < 1e-12)",
           "value": value, "unit": "packings/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32/f64 (mixed) then f64", "data": "synthetic",
           "config": {"workload": f"packings_{nsys}_systems", "systems": nsys, "atoms": w.n,
                      "n_range": [64, 4096], "phi_range": [0.62, 0.66], "exponent": 2.5, "skin": w.skin,
                      "minimiser": "CollectionNLCGV (fixed box), dt 0.1, secmax 10, seceps 1e-4, kmax 1000",
                      "tol_mixed": tol32, "tol_fp64": tol64, "step_cap_mixed": cap32, "step_cap_fp64": cap64,
                      "mixed_phase_end": "max|F| < tol_mixed",
                      "steps_per_check": chunk, "kernel_variant": r["variant"], "autotune": tuned},
           "wall_s": wall, "mixed_s": r["t32"], "fp64_s": r["t64"],
           "converged": int(conv.sum()), "converged_fraction": float(conv.mean()),
           "steps_median": {"mixed": float(np.median(r["s32"])), "fp64": float(np.median(r["s64"]))},
           "steps_p90": {"mixed": float(np.percentile(r["s32"], 90)), "fp64": float(np.percentile(r["s64"], 90))},
           "converged_within_fp64_steps": {str(k): int((conv & (r["s64"] <= k)).sum())
                                           for k in (500, 1000, 2000, 5000, 10000, 20000) if k <= cap64},
           "mixed_atom_steps_per_s": float((r["s32"] * sizes).sum() / r["t32"]),
           "fp64_atom_steps_per_s": float((r["s64"] * sizes).sum() / max(r["t64"], 1e-9)),
           "max_force": {"after_mixed_median": float(np.median(r["f32"])), "after_fp64_max": float(r["f64"].max())},
           "final_energy_vs_fp64_only": {
               "systems_converged_in_both": int(both.sum()), "unjammed_both_zero": int(unjammed.sum()),
               "jammed": int(jammed.sum()), "jammed_same_minimum": int(same.sum()),
               "jammed_rel_diff_median": float(np.median(rel[jammed])) if jammed.any() else None,
               "jammed_rel_diff_max": float(rel[jammed].max()) if jammed.any() else None,
               "note": "FP64-only minimisation of the same initial systems; energy per atom compared"},
           "one_system_per_launch": {"systems": nsingle, "converged": c_single, "packings_per_s": single_rate,
                                     "batched_speedup": value / single_rate if single_rate > 0 else None}}
    print(json.dumps(out), flush=True)


def _msd(x, x0, sizes):
    d = ((x - x0) ** 2).sum(1)
    off = np.cumsum([0] + list(sizes))
    return np.array([d[off[s]:off[s + 1]].mean() for s in range(len(sizes))])


def run_replicas(args):
    """Batched WCA Langevin replicas: mixed vs FP64 on MSD and potential energy."""
    from parm_gb300 import workloads as W
    nrep = args.nsys or 512
    w = W.wca_replicas(nrep=nrep, nmin=256, nmax=32768, rho_lo=0.5, rho_hi=0.9, seed=4)
    dt, damping, T, seed = 0.001, 1.0, 1.0, 20261204
    steps, chunk = args.steps, 1000
    steps64 = min(steps, args.fp64_steps)
    res = {}

    def make(ws):
        g = make_system(ws, "mixed", 0)
        g.set_graph_steps(args.graph_steps)
        return g
    w, cscale, tuned = _tuned(w, make, lambda g, k: g.sol(dt, damping, T, seed, k), (0.1, 0.2, 0.3, 0.45))
    res["autotune"] = tuned
    for prec, nst in (("mixed", steps), ("fp64", steps64)):
        g = make_system(w, prec, 0)
        g.set_graph_steps(args.graph_steps)
        if cscale != 1.0:
            g.set_cell_scale(cscale)
            g.nlist_update(False)
        if prec == "mixed":
            res["kernel"] = g.autotune()
        x0 = g.get_atoms(1)["x"]
        msd, pe, tt = [], [], 0.0
        done = 0
        while done < nst:
            k = min(chunk, nst - done)
            ta = _sync_time(g)
            g.sol(dt, damping, T, seed, k)
            tt += _sync_time(g) - ta
            done += k
            msd.append(_msd(g.get_atoms(1)["x"], x0, w.sizes))
            pe.append(g.energy() / np.array(w.sizes))
        res[prec] = {"atom_steps_per_s": w.n * nst / tt, "steps": nst, "seconds": tt, "launches": g.last_launches(),
                     "msd": np.array(msd), "pe": np.array(pe)}
        g.close()
    k = len(res["fp64"]["msd"])
    m32, m64 = res["mixed"]["msd"][:k], res["fp64"]["msd"][:k]
    p32, p64 = res["mixed"]["pe"][:k], res["fp64"]["pe"][:k]
    msd_rel = np.abs(m32.mean(1) - m64.mean(1)) / m64.mean(1)
    spread = m64.std(1) / np.sqrt(nrep) / m64.mean(1)
    out = {"metric": "atom-timesteps/s (batched WCA Langevin replicas), mixed vs FP64 on MSD and PE",
           "value": res["mixed"]["atom_steps_per_s"], "unit": "atom-timesteps/s", "n_gpus": 1,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (mixed)",
           "data": "synthetic",
           "config": {"workload": f"wca_replicas_{nrep}", "replicas": nrep, "atoms": w.n, "n_range": [256, 32768],
                      "rho_range": [0.5, 0.9], "T": T, "damping": damping, "dt": dt, "steps": steps,
                      "fp64_steps": steps64, "kernel": res["kernel"], "skin": w.skin, "autotune": res["autotune"],
                      "steps_per_graph": args.graph_steps},
           "ms_per_step": 1e3 * res["mixed"]["seconds"] / res["mixed"]["steps"],
           "fp64_value": res["fp64"]["atom_steps_per_s"],
           "mixed_vs_fp64": res["mixed"]["atom_steps_per_s"] / res["fp64"]["atom_steps_per_s"],
           "msd_batch_mean_rel_diff": [float(q) for q in msd_rel],
           "msd_rel_standard_error": [float(q) for q in spread],
           "pe_per_atom_rel_diff": float(np.abs(p32.mean() - p64.mean()) / abs(p64.mean())),
           "pe_per_atom_max_replica_rel_diff": float((np.abs(p32[-1] - p64[-1]) / np.abs(p64[-1])).max())}
    print(json.dumps(out), flush=True)


def run_disks(args):
    """2D bidisperse harmonic disks at phi = 0.84: conjugate-gradient minimisation (CollectionNLCGV),
    a mixed-precision phase then FP64 until max|F| < 1e-12, against an FP64-only minimisation."""
    from parm_gb300 import workloads as W
    w = W.soft_disks(n=65536, phi=0.84, exponent=2.0, seed=2, skin=args.skin)
    tol32, tol64, chunk = 1e-10, 1e-12, 1000
    cap = args.min_steps
    r = _cg_protocol(w, tol32, tol64, cap, cap, chunk, tune=True)
    gr, _ = _cg_handle(w, "fp64")
    t3 = _sync_time(gr)
    sr, fr = _minimise_cg(gr, tol64, 2 * cap, chunk)
    t4 = _sync_time(gr)
    Er = float(gr.energy()[0])
    gr.close()
    E = float(r["E"][0])
    out = {"metric": "seconds to minimise 65536 2D disks at phi 0.84 to max|F| < 1e-12 (mixed bulk + FP64 finish)",
           "value": r["t32"] + r["t64"], "unit": "s", "n_gpus": 1, "higher_is_better": False, "scaling": "strong",
           "vs_baseline": None, "dtype": "f32/f64 (mixed) then f64", "data": "synthetic",
           "config": {"workload": "disks2d_65536", "phi": 0.84, "exponent": 2.0, "skin": w.skin,
                      "minimiser": "CollectionNLCGV (fixed box), dt 0.1, secmax 10, seceps 1e-4, kmax 1000",
                      "tol_mixed": tol32, "tol_fp64": tol64, "step_cap_each_phase": cap, "kernel_variant": r["variant"],
                      "mixed_phase_end": "max|F| < tol_mixed, or less than a factor 2 over 4 checks"},
           "steps_mixed": int(r["s32"][0]), "steps_fp64": int(r["s64"][0]), "max_force": float(r["f64"][0]),
           "converged": bool(r["f64"][0] < tol64), "energy": E,
           "fp64_alone": {"seconds": t4 - t3, "steps": int(sr[0]), "max_force": float(fr[0]), "energy": Er,
                          "converged": bool(fr[0] < tol64)},
           "energy_rel_diff": abs(E - Er) / max(abs(Er), 1e-300),
           "energy_per_atom": {"mixed_then_fp64": E / w.n, "fp64_alone": Er / w.n},
           "note": "energies per atom below 1e-16 mean an unjammed minimum (no overlaps left): both zero"}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--graph-steps", type=int, default=50,
                    help="time steps per CUDA graph launch (0: direct kernel launches, for profilers)")
    ap.add_argument("--tpa", type=int, default=0,
                    help="pair-kernel variant (0: autotune; 200 cell blocks, 1/2/4 tiled, 100+t gather)")
    ap.add_argument("--rsq", action="store_true",
                    help="run the device mean-square-displacement tracker inside the timed steps")
    ap.add_argument("--only-timed", action="store_true",
                    help="run only the timed mixed-precision region (used for profiler captures)")
    ap.add_argument("--workload", default="lj1m", choices=["lj1m", "packings", "replicas", "disks"],
                    help="lj1m: the headline line; the others print their own line")
    ap.add_argument("--nsys", type=int, default=0, help="systems in the batched workloads")
    ap.add_argument("--min-steps", type=int, default=20000, help="step cap of each minimisation phase")
    ap.add_argument("--fp64-cap", type=int, default=5000, help="packings: step cap of the FP64 phase")
    ap.add_argument("--skin", type=float, default=0.1, help="neighbour-list skin of the packing workloads")
    ap.add_argument("--fp64-steps", type=int, default=0,
                    help="lj1m: timed FP64 steps (default 200); replicas: FP64 steps of the comparison (2000)")
    ap.add_argument("--drift-steps", type=int, default=10000,
                    help="steps of the NVE drift fit of each path (0: skip)")
    ap.add_argument("--sample-sys", type=int, default=64, help="packings minimised by FP64 alone")
    ap.add_argument("--single-sys", type=int, default=16, help="packings run one system per launch")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.fp64_steps == 0:
        args.fp64_steps = 200 if args.workload == "lj1m" else 2000
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args, rank)
        return
    if args.workload != "lj1m":
        import torch
        torch.cuda.set_device(local_rank)
        {"packings": run_packings, "replicas": run_replicas, "disks": run_disks}[args.workload](args)
        return
    run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
