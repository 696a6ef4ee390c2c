#!/usr/bin/env python
"""Benchmark of the GB300 OVERTURNS-2D hot path.

Workload (the configuration the headline metric is quoted on): viscous
RANS-SA, NACA 0012 C-mesh 513x129 (first wall spacing 1e-6 chords), M=0.15,
alpha=10 deg, Re=6e6 per chord, MUSCL kappa=1/3 + Roe, LU-SGS, local CFL 50
-- run as a batch of B independent requests (alpha varied, seeded) resident
in HBM.  A "step" is one iteration of the reference's step.f loop
(time_step, bc, rhsup + visrhs, norms, rbc, ilu2d, vmu_sa, update, monitor)
over the whole batch.  The meshes are generated algebraically from a seed
(no dataset exists); flow fields start from freestream.

  value   FP32-mixed batched cell-updates/s, device-resident (kernel path)
  e2e     the same through the host-buffer C-ABI path: every step copies the
          state of every request host->device and back (pinned buffers)
  fp64    the plain FP64 path on the same batch (reported beside it)

--impl reference times the reference's algorithm on the host cores: the
CPU FP64 oracle (a line-by-line C++ restatement of the Fortran; the
Fortran itself cannot be compiled here -- no Fortran compiler), one request
per thread.
"""
import argparse
import ctypes as C
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

METRIC = "cell-updates/s & converged solves/s (FP32-mixed batched vs FP64 plain) + p50/p99"
UNIT = "cell-updates/s"
JMAX, KMAX = 513, 129
WORKLOAD = "RANS-SA NACA0012 C-mesh 513x129, M0.15 a10 Re6e6, MUSCL+Roe, LU-SGS CFL50"

# algorithmic bytes per interior cell per launch of each kernel family of
# the FP32-mixed path (the compulsory array traffic of each kernel family)
ALG_BYTES_F32 = {0: 44, 1: 0, 2: 80, 3: 0, 4: 188, 5: 200, 6: 96}
# the same arrays in the plain FP64 path: 8 bytes per element (iblank 4);
# the update has no f32 shadow to write
ALG_BYTES_F64 = {0: 88, 1: 0, 2: 156, 3: 0, 4: 376, 5: 400, 6: 108}
PHASES = ["time_step", "bc", "residual", "rbc", "lusgs", "sa", "update"]
# DRAM bytes per interior cell per launch measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum of the batch-8 capture, 0.52 M cells, summarised in
# profiles/top_kernels_rans_sa_513x129_b8_fp32mixed.md), scaled to the batch
TRAFFIC_PER_CELL = {"residual": (40.496384e6 + 1.447168e6) / (8 * 65536),
                    # k_lu_prep + both sweeps (k_lu_edges, ~1 % of the phase, not captured)
                    "lusgs": (31.611136e6 + 7.541504e6 + 62.385408e6 + 2.267648e6 + 62.397696e6 + 1.084416e6)
                    / (8 * 65536),
                    # k_update as the phase timer runs it, without the folded time step
                    "update": (27.421952e6 + 0.079360e6) / (8 * 65536)}
NPH = len(PHASES)


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def rank_max(x, dist, device):
    """The slowest rank's value of x (a time): every rank gets the maximum."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """Whole-job throughput of replicas with the same per-rank work (weak
    scaling): all ranks' units over the slowest rank's time."""
    return world * units_per_rank / seconds


def rank_seed(rank):
    """Each rank serves its own requests: seeds 1000 apart."""
    return 1000 * rank


def batch_alfas(n, seed=0):
    """Angles of attack of the batch: 10 deg, then seeded U[0, 10]."""
    rng = np.random.default_rng(seed)
    return [10.0 if i == 0 else float(rng.uniform(0.0, 10.0)) for i in range(n)]


def batch_cases(n, seed=0, jmax=JMAX, kmax=KMAX):
    """The batch for the GPU arm, built by the library's own set-up calls."""
    from turns2d_urans_git_gb300 import api
    return [api.config_c2(jmax=jmax, kmax=kmax, alfa=a) for a in batch_alfas(n, seed)]


def oracle_batch(n, seed=0, jmax=JMAX, kmax=KMAX):
    """The same batch for the CPU legs, built without the product library:
    the oracle's read_inputs over namelist inputs and the numpy restatement
    of the mesh generator (bitwise the same meshes).  Returns (params, xv, yv)."""
    from tests import oracle_binding as ob
    oc = ob.oracle_cases()
    out = []
    for a in batch_alfas(n, seed):
        inp, xv, yv = oc.c2_inputs(jmax, kmax, alfa=a)
        out.append((ob.read_inputs(inp), xv, yv))
    return out


def bench_config(batch, world):
    """The workload description, the same dict for both arms."""
    return {"workload": WORKLOAD, "batch_per_gpu": batch, "interior_cells": (JMAX - 1) * (KMAX - 1),
            "parallelism": "replicas x%d" % world,
            "l2": "inputs larger than L2: %d requests x %d cells, ~25 MB of state each (L2 129 MB)"
                  % (batch, (JMAX - 1) * (KMAX - 1)),
            "launch_choices": "GPU arm: autotuned per mesh-size class (the line's `tuning`)"}


def autotune(device, classes_fp32, workload_class, batch):
    """Launch choices of the GPU arm from the autotuner (cached per GPU,
    precision, size class and batch; searched on a miss): every FP32 class
    at 16 requests (the served stream), and the workload's class at the
    workload's batch in both precisions (the timed batches)."""
    import torch
    from turns2d_urans_git_gb300 import tune
    from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED, OT2D_FP64
    gpu = torch.cuda.get_device_name(device)
    t0 = time.perf_counter()
    c32, _ = tune.tune(tune.gpu_measure_for_class(OT2D_FP32_MIXED, batch=16, device=device), classes_fp32, gpu,
                       OT2D_FP32_MIXED)
    w32, _ = tune.tune(tune.gpu_measure_for_class(OT2D_FP32_MIXED, batch=batch, device=device), (workload_class,),
                       gpu, OT2D_FP32_MIXED)
    w64, _ = tune.tune(tune.gpu_measure_for_class(OT2D_FP64, batch=batch, iters=2, device=device), (workload_class,),
                       gpu, OT2D_FP64)
    return c32, w32, w64, time.perf_counter() - t0


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (read-only queries
    of libnvidia-ml) every 2 ms on a thread during the timed region, so that
    a timed region of tens of milliseconds still has samples."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, dev):
        import ctypes as C
        import threading
        self.C, self.threading = C, threading
        self.nv = C.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        uuid = None
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(dev).uuid)
        except Exception:
            pass
        cnt = C.c_uint(0)
        self.nv.nvmlDeviceGetCount_v2(C.byref(cnt))
        found = False
        for i in range(cnt.value):
            h = C.c_void_p()
            if self.nv.nvmlDeviceGetHandleByIndex_v2(i, C.byref(h)) != 0:
                continue
            buf = C.create_string_buffer(96)
            if uuid and self.nv.nvmlDeviceGetUUID(h, buf, 96) == 0 and buf.value.decode().endswith(uuid):
                self.h, found = h, True
                break
        if not found and self.nv.nvmlDeviceGetHandleByIndex_v2(dev, C.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        try:
            self.get_reasons = self.nv.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            self.get_reasons = self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        self.get_clock = self.nv.nvmlDeviceGetClockInfo
        mx = C.c_uint(0)
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx))
        self.max_mhz = float(mx.value)
        self.samples, self.reasons, self.run = [], set(), False

    def _loop(self):
        C = self.C
        clk, rs = C.c_uint(0), C.c_ulonglong(0)
        while self.run:
            if self.get_clock(self.h, 1, C.byref(clk)) == 0:
                self.samples.append(float(clk.value))
            if self.get_reasons(self.h, C.byref(rs)) == 0:
                for bit, nm in self.REASONS.items():
                    if rs.value & bit:
                        self.reasons.add(nm)
            time.sleep(0.002)

    def start(self):
        self.run = True
        self.t = self.threading.Thread(target=self._loop, daemon=True)
        self.t.start()

    def stop(self):
        self.run = False
        self.t.join()
        self.nv.nvmlShutdown()
        sm = self.samples
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(self.reasons), "samples": len(sm), "source": "nvml, 2 ms"}


def clock_sampler(dev):
    try:
        return NvmlClocks(dev)
    except (OSError, AttributeError):
        return ClockSampler(dev)


class ClockSampler:
    """nvidia-smi sampling of SM clock, power and throttle reasons during the
    timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev, self.proc, self.path = dev, None, None

    def start(self):
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), "ot2d_clocks_%d.csv" % os.getpid())
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def cpu_reference(cases, target_s=12.0, max_threads=None):
    """The reference algorithm on the host cores: the -O3 build of the CPU
    FP64 oracle (a line-by-line restatement of the Fortran, which cannot be
    compiled here: no Fortran compiler), every request of the batch run for
    the same bounded number of iterations on a pool of one thread per core.
    Returns (cell-updates/s, threads, sample description)."""
    from tests import oracle_binding as ob
    ob.lib_fast()
    ncores = os.cpu_count() or 1
    nthr = max(1, min(max_threads or ncores, ncores, len(cases)))
    prm, xv, yv = cases[0]
    t0 = time.perf_counter()
    ob.solve(prm, xv.ravel(), yv.ravel(), 2, fast=True)
    per_it = (time.perf_counter() - t0) / 2
    # wall ~ (requests / threads) x iterations x per-iteration time
    iters = max(2, int(target_s * nthr / (len(cases) * max(per_it, 1e-6))))
    done = [0] * len(cases)
    nxt = [0]
    lock = threading.Lock()

    def work():
        while True:
            with lock:
                i = nxt[0]
                nxt[0] += 1
            if i >= len(cases):
                return
            p, x, y = cases[i]
            n, _, _, _ = ob.solve(p, x.ravel(), y.ravel(), iters, fast=True)
            done[i] = abs(n) * (p.jmax - 1) * (p.kmax - 1)

    th = [threading.Thread(target=work) for _ in range(nthr)]
    t0 = time.perf_counter()
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.perf_counter() - t0
    value = sum(done) / wall
    sample = ("all %d requests of the batch x %d iterations each (513x129 RANS-SA, FP64 oracle -O3) on %d threads, "
              "%.1f s wall" % (len(cases), iters, nthr, wall))
    return value, nthr, sample


def serve_stream(precision, reqs, arrivals, max_iters, check_every, device, cap_s, budget_mb=0, choices=None):
    """Continuous-batching service of a request stream: each request is
    submitted at the first status check after its arrival time (admitted at
    once when it fits the memory budget, queued otherwise) and retired when
    converged -- FP64: its L2 norm `orders` decades below its peak; FP32-mixed:
    the mixed rule (api.MIXED_RULE) -- failed or capped.  Stops submitting and
    gives up after cap_s seconds.  Returns per-request (index, arrival,
    result), the makespan (s) and the most requests ever queued."""
    from turns2d_urans_git_gb300 import api
    from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED, OT2D_OPT_BUDGET_MB
    sv = api.Solver(precision, device=device, check_every=check_every)
    if choices:
        from turns2d_urans_git_gb300 import tune
        tune.apply(sv, choices)
    if precision == OT2D_FP32_MIXED:
        sv.set_mixed_rule()
    if budget_mb:
        sv.set_option(OT2D_OPT_BUDGET_MB, budget_mb)
    t0 = time.perf_counter()
    pending = sorted(zip(arrivals, range(len(reqs))))
    submitted = {}
    max_queued = 0
    while True:
        now = time.perf_counter() - t0
        while pending and pending[0][0] <= now and now <= cap_s:
            ta, i = pending.pop(0)
            (_, prm, xv, yv), orders = reqs[i]
            submitted[sv.add(prm, xv, yv, orders=orders, max_iters=max_iters)] = (i, ta)
        max_queued = max(max_queued, sv.queued())
        if sv.live() == 0:
            if not pending or now > cap_s:
                break
            time.sleep(max(0.0, min(pending[0][0] - now, 0.05)))
            continue
        if now > cap_s:
            break
        sv.iterate(check_every)
    sv.sync()
    t_end = time.perf_counter() - t0
    out = [(i, ta, sv.result(iid)) for iid, (i, ta) in submitted.items()]
    sv.close()
    return out, t_end, max_queued


def time_accurate_section(device, batch=64, nsteps=12, itnmax=4):
    """Time-accurate throughput: `batch` pitching RANS-SA requests (257x65,
    M 0.3, alpha(t) = 2 deg * (1 - cos(0.5 t)), dt 0.1, itnmax Newton
    iterations per physical step, second order), FP32-mixed, timed with CUDA
    events over nsteps physical steps after 2 warm-up steps."""
    import torch
    from turns2d_urans_git_gb300 import api
    from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED
    _, prm, xv, yv = api.config_pitching(jmax=257, kmax=65, viscous=True, iturb=1, ntac=2, itnmax=itnmax, dt=0.1,
                                         rf=0.5, angmax=2.0, fsmach=0.3, rey=3e6)
    sv = api.Solver(OT2D_FP32_MIXED, device=device, check_every=10 ** 6)
    for _ in range(batch):
        sv.add(prm, xv, yv, orders=0.0, max_iters=nsteps + 2)
    sv.iterate(2 * itnmax)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(sv.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sv.iterate(nsteps * itnmax - 1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    its = nsteps * itnmax - 1
    cells = (prm.jmax - 1) * (prm.kmax - 1)
    sv.close()
    return {"workload": "%d pitching RANS-SA requests, NACA0012 257x65, M0.3 Re3e6, dt 0.1, %d Newton iterations "
                        "per physical step (ntac 2), fp32-mixed" % (batch, itnmax),
            "ms_per_newton_iteration": ms / its, "physical_steps_per_s_per_request": 1e3 * its / itnmax / ms,
            "cell_updates_per_s": batch * cells * its / (ms / 1e3)}


def serve_requests(n, seed=7):
    """The config-5 stream: 80 % steady RANS-SA requests drawn as the batched
    configuration (NACA m, p, t; all five mesh sizes; M, alpha, Re), 20 %
    time-spectral pitching NACA 0012 257x65 requests (N_ts in {3, 5, 7},
    alpha0 in U[0, 10], k in U[0.05, 0.15], M 0.3); each with its own
    tolerance, an L2 drop of 8, 9 or 10 decades."""
    from turns2d_urans_git_gb300 import api
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        case = api.config_c5_ts(rng) if rng.random() < 0.2 else api.config_c4_sample(rng)
        out.append((case, float(rng.integers(8, 11))))
    return out


def serving_section(args, device, choices=None):
    """FP32-mixed vs FP64 on the same seeded Poisson request stream:
    converged solves/s, p50/p99 time from submission to a converged
    solution, and the force differences of the requests both converged."""
    from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED, OT2D_FP64
    reqs = serve_requests(args.serve_requests)
    rng = np.random.default_rng(8)
    gaps = rng.exponential(1.0 / args.serve_rate, len(reqs))
    arrivals = np.cumsum(gaps) - gaps[0]
    res, forces = {}, {}
    for name, prec in (("fp32_mixed", OT2D_FP32_MIXED), ("fp64", OT2D_FP64)):
        out, t_end, maxq = serve_stream(prec, reqs, arrivals, args.serve_max_iters, 25, device, args.serve_seconds,
                                        args.serve_budget_mb, (choices or {}).get(prec))
        conv = [(i, r) for (i, ta, r) in out if r.converged and r.status == 0]
        lat = [r.t_done - r.t_submit for (i, r) in conv]
        ts = sum(1 for (i, r) in conv if reqs[i][0][1].nspec > 1)
        res[name] = {"requests": len(reqs), "submitted": len(out), "converged": len(conv),
                     "converged_time_spectral": ts,
                     "failed": sum(1 for (i, ta, r) in out if r.status != 0),
                     "capped_or_unfinished": sum(1 for (i, ta, r) in out if r.status == 0 and not r.converged),
                     "max_queued": maxq,
                     "solves_per_s": len(conv) / t_end if t_end > 0 else None,
                     "p50_s": float(np.percentile(lat, 50)) if lat else None,
                     "p99_s": float(np.percentile(lat, 99)) if lat else None,
                     "makespan_s": t_end}
        forces[name] = {i: (r.cl, r.cd, r.cm) for (i, r) in conv}
    a, b = forces["fp32_mixed"], forces["fp64"]
    both = sorted(set(a) & set(b))
    d = np.array([[abs(a[i][k] - b[i][k]) for k in range(3)] for i in both]) if both else np.zeros((0, 3))
    sm, sd = res["fp32_mixed"]["solves_per_s"], res["fp64"]["solves_per_s"]
    return {"workload": "%d seeded requests, Poisson arrivals %.2f/s: 80%% steady RANS-SA (NACA m,p,t; meshes "
                        "129x33..769x193; M 0.3-0.85; a -2..8 deg; Re 1e6-1e7), 20%% time-spectral pitching NACA0012 "
                        "257x65 (N_ts 3/5/7, M 0.3); per-request tolerance 8-10 decades; %d-iteration cap per "
                        "request, %.0f s cap per precision"
                        % (len(reqs), args.serve_rate, args.serve_max_iters, args.serve_seconds),
            "convergence": {"fp64": "L2 norm (step.f:86-93) `orders` decades below its peak",
                            "fp32_mixed": "f32 floor rule: norm 2 decades below its peak and CL, CD within 2e-6, "
                                          "4e-7 over 8 samples 200 iterations apart"},
            "fp32_mixed": res["fp32_mixed"], "fp64": res["fp64"],
            "speedup_solves_per_s": (sm / sd) if sm and sd else None,
            "compared": len(both),
            "max_abs_dcl_vs_fp64": float(d[:, 0].max()) if both else None,
            "max_abs_dcd_vs_fp64": float(d[:, 1].max()) if both else None,
            "max_abs_dcm_vs_fp64": float(d[:, 2].max()) if both else None}


def run_reference(args):
    """The reference arm: the oracle (the reference's algorithm restated in
    C++; the Fortran itself cannot be built here) on the host cores over the
    same 64-request batch as the GPU arm, built without the product library.
    Rank 0 alone runs it; other ranks exit without work."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    t0 = time.perf_counter()
    cases = oracle_batch(args.batch)
    per_step = max(1.0, min(args.ref_seconds, 150.0 / max(args.steps, 1)))
    # warm-up: page in the library and the meshes (one short request)
    from tests import oracle_binding as ob
    for _ in range(min(args.warmup, 1)):
        prm, xv, yv = cases[0]
        ob.solve(prm, xv.ravel(), yv.ravel(), 1, fast=True)
    vals = []
    for _ in range(args.steps):
        v, thr, sample = cpu_reference(cases, target_s=per_step)
        vals.append(v)
    value = float(np.median(vals))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded algebraic NACA0012 C-meshes, freestream start)",
            "config": bench_config(len(cases), world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": thr, "kind": "port",
                             "sample": sample + "; median of %d such samples" % args.steps},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)
    return 0


def e2e_rate(sv, ids, cases, steps, world, dist):
    """Cell-updates/s through the host-buffer C-ABI path
    (ot2d_solver_iterate_host): every step uploads every request's
    q(jd,kd,nspec,nq) from pinned host memory, runs the iteration and reads q
    back.  Returns (rate, bytes each way per step)."""
    import torch
    from turns2d_urans_git_gb300 import api
    B = len(ids)
    qh = [np.zeros(prm.jd * prm.kd * prm.nspec * prm.nq) for (_, prm, _, _) in cases]
    for iid, (_, prm, _, _), q in zip(ids, cases, qh):
        q[:] = sv.get_q(iid, prm)
    pinned = [torch.from_numpy(q).pin_memory() for q in qh]
    ptrs = (C.POINTER(C.c_double) * B)(*[C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)) for t in pinned])
    idarr = (C.c_int32 * B)(*ids)
    L = api.lib()
    L.ot2d_solver_iterate_host.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                           C.POINTER(C.POINTER(C.c_double)), C.c_int32]
    L.ot2d_solver_iterate_host(sv._h, B, idarr, ptrs, 1)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = L.ot2d_solver_iterate_host(sv._h, B, idarr, ptrs, steps)
    torch.cuda.synchronize()
    secs = rank_max(time.perf_counter() - t0, dist, "cuda")
    cells = sum((prm.jmax - 1) * (prm.kmax - 1) for (_, prm, _, _) in cases)
    link = host_link(pinned)
    return (whole_job_rate(cells * steps, world, secs) if rc == 0 else None), sum(q.nbytes for q in qh), link


def host_link(pinned, reps=5):
    """The host link's copy rates for the bytes the host-buffer path moves per
    step (the bound of that path): one pinned buffer of that size copied up,
    down, and both ways at once on two streams, timed with CUDA events (best
    of reps, so that no host-side issue time enters), GB/s."""
    import torch
    nbytes = sum(t.numel() * t.element_size() for t in pinned)
    h_up = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h_dn = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d_up = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d_dn = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    out = {}
    for kind in ("h2d", "d2h", "both"):
        best = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(torch.cuda.current_stream())
            s1.wait_event(e0)
            s2.wait_event(e0)
            if kind in ("h2d", "both"):
                with torch.cuda.stream(s1):
                    d_up.copy_(h_up, non_blocking=True)
            if kind in ("d2h", "both"):
                with torch.cuda.stream(s2):
                    h_dn.copy_(d_dn, non_blocking=True)
            e1.record(s1)
            e2.record(s2)
            torch.cuda.synchronize()
            best = min(best, max(e0.elapsed_time(e1), e0.elapsed_time(e2)) / 1e3)
        out[kind + "_gbs"] = (2 if kind == "both" else 1) * nbytes / best / 1e9
    del h_up, h_dn, d_up, d_dn
    return out


def phase_roofline(sv, alg_bytes, cells, peaks, traffic=None):
    """Per-phase CUDA-event timers of the batch (ot2d_solver_profile) and the
    HBM roofline of the dominant phase: algorithmic bytes of its arrays over
    its measured time, against the measured copy bandwidth."""
    from turns2d_urans_git_gb300 import api
    prof = (C.c_double * NPH)()
    api.lib().ot2d_solver_profile.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int32]
    rc = api.lib().ot2d_solver_profile(sv._h, 5, prof, NPH)
    if rc != 0:
        return {}, None
    phase_ms = {PHASES[i]: prof[i] for i in range(NPH)}
    dom = max(range(NPH), key=lambda i: prof[i])
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg_bytes[dom] * cells / (prof[dom] * 1e-3) / 1e9 if prof[dom] > 0 else None
    roof = {"bound": "hbm", "kernel": PHASES[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "alg_bytes_per_cell": alg_bytes[dom],
            "traffic": (traffic[PHASES[dom]] * cells if traffic and PHASES[dom] in traffic else None),
            "traffic_note": "bytes per launch, ncu batch-8 capture scaled by cells",
            "peak_source": "measured" if peaks else "fallback"}
    return phase_ms, roof


def run_ours(args):
    import torch
    from turns2d_urans_git_gb300 import api
    from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED, OT2D_FP64

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cases = batch_cases(args.batch, seed=rank_seed(rank))
    cells = (JMAX - 1) * (KMAX - 1)
    B = len(cases)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass

    from turns2d_urans_git_gb300 import tune
    c32, w32, c64, tune_s = autotune(local, tune.SIZE_CLASSES, (JMAX, KMAX), B)
    # the timed batches use the choices searched at their own batch; the
    # served stream those searched at 16 requests
    choices = {OT2D_FP32_MIXED: {**c32, **w32}, OT2D_FP64: c64}
    serve_choices = {OT2D_FP32_MIXED: c32, OT2D_FP64: c64}

    def make(precision):
        sv = api.Solver(precision, device=local, check_every=10 ** 8)
        tune.apply(sv, choices[precision])
        ids = [sv.add(prm, xv, yv, orders=0.0, max_iters=10 ** 8) for (_, prm, xv, yv) in cases]
        return sv, ids

    def timed(sv, steps):
        stream = torch.cuda.ExternalStream(sv.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        sv.iterate(steps)
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        return rank_max(e0.elapsed_time(e1), dist, "cuda")

    # ---- FP32-mixed batched, device resident (value)
    sv, ids = make(OT2D_FP32_MIXED)
    sv.iterate(args.warmup)
    torch.cuda.synchronize()
    kernels_per_step = sv.graph_kernels()
    clk = clock_sampler(local)
    clk.start()
    ms = timed(sv, args.steps)
    clocks = clk.stop()
    value = whole_job_rate(B * cells * args.steps, world, ms / 1e3)
    phase_ms, roof = phase_roofline(sv, ALG_BYTES_F32, B * cells, peaks, TRAFFIC_PER_CELL)
    e2e, qbytes, link = e2e_rate(sv, ids, cases, max(3, args.steps // 2), world, dist)
    sv.close()
    # ---- plain FP64 on the same batch, with its own e2e and roofline
    fp64 = None
    if not args.skip_fp64:
        sv64, ids64 = make(OT2D_FP64)
        sv64.iterate(1)
        torch.cuda.synchronize()
        k64 = max(2, args.fp64_steps)
        ms64 = timed(sv64, k64)
        ph64, roof64 = phase_roofline(sv64, ALG_BYTES_F64, B * cells, peaks)
        e64, qb64, _ = e2e_rate(sv64, ids64, cases, 2, world, dist)
        fp64 = {"value": whole_job_rate(B * cells * k64, world, ms64 / 1e3), "unit": UNIT, "steps": k64,
                "ms_per_step": ms64 / k64, "phase_ms": ph64, "roofline": roof64,
                "e2e": {"value": e64, "unit": UNIT, "h2d_bytes_per_step": qb64, "d2h_bytes_per_step": qb64}}
        sv64.close()
    # ---- served request stream (rank 0 only): converged solves/s, p50/p99
    serve = None
    if rank == 0 and not args.skip_serve:
        serve = serving_section(args, local, serve_choices)
    unsteady = time_accurate_section(local) if rank == 0 and not args.skip_serve else None
    # ---- CPU baseline (rank 0, N=1 only): the oracle on the host cores
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        v, thr, sample = cpu_reference(oracle_batch(args.batch), target_s=args.ref_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": thr, "kind": "port", "sample": sample}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (f64 state update, norms, forces)",
                "data": "synthetic (seeded algebraic NACA0012 C-meshes, freestream start)",
                "config": bench_config(B, world),
                "precision": "fp32-mixed",
                "tuning": {"fp32_mixed": tune.describe(w32), "fp64": tune.describe(c64),
                           "fp32_mixed_served_b16": tune.describe(c32), "batch": B,
                           "search_s": tune_s, "cache": tune.default_cache_path()},
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": qbytes, "d2h_bytes_per_step": qbytes,
                        # the host link's rates for the same buffers, and the
                        # rate the path would have if its copies alone bound it
                        "host_link": link,
                        "copy_bound_value": B * cells / (2 * qbytes / (link["both_gbs"] * 1e9))},
                "fp64_plain": fp64,
                "gpu_launches": kernels_per_step * args.steps,
                "kernels_per_step": kernels_per_step,
                "phase_ms": phase_ms,
                "roofline": roof,
                "clocks": clocks}
        if cpu:
            line["cpu_baseline"] = cpu
        if serve:
            line["serving"] = serve
        if unsteady:
            line["time_accurate"] = unsteady
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_replica_check(args):
    """The replica launch and aggregation without a GPU (gloo): each rank
    times one oracle iteration of the first request of its own seeded batch;
    rank 0 prints the whole-job line (all ranks' cell-updates over the
    slowest rank's time) and every rank's angles of attack."""
    import torch.distributed as dist
    rank, world, _ = env_rank()
    dist.init_process_group("gloo")
    from tests import oracle_binding as ob
    cases = oracle_batch(args.batch, seed=rank_seed(rank), jmax=65, kmax=25)
    prm, xv, yv = cases[0]
    dist.barrier()
    t0 = time.perf_counter()
    ob.solve(prm, xv.ravel(), yv.ravel(), 1, fast=True)
    secs = rank_max(time.perf_counter() - t0, dist, "cpu")
    units = (prm.jmax - 1) * (prm.kmax - 1)
    alfas = [None] * world
    dist.all_gather_object(alfas, [float(p.alfa) for (p, _, _) in cases])
    if rank == 0:
        print(json.dumps({"n_gpus": world, "seconds": secs, "value": whole_job_rate(units, world, secs),
                          "units_per_rank": units, "alfas": alfas}), flush=True)
    dist.destroy_process_group()
    return 0


def spawn_replicas(n, argv):
    """`bench.py --gpus N` outside torchrun: relaunch this script as N
    replica processes, one per GPU, with the launcher the multi-GPU runs use
    (torch.distributed.run, rendezvous on 127.0.0.1)."""
    import socket
    sk = socket.socket()
    sk.bind(("127.0.0.1", 0))
    port = sk.getsockname()[1]
    sk.close()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + argv
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=16.0)
    ap.add_argument("--serve-max-iters", type=int, default=30000)
    ap.add_argument("--serve-seconds", type=float, default=75.0)
    ap.add_argument("--serve-budget-mb", type=int, default=0)
    ap.add_argument("--skip-serve", action="store_true")
    # the replica launch and aggregation on CPU ranks (gloo); no GPU work
    ap.add_argument("--cpu-replica-check", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_replicas(args.gpus, sys.argv[1:])
    if args.cpu_replica_check:
        return run_replica_check(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
