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
PHASES = ["time_step", "bc", "residual", "rbc", "lusgs", "sa", "update"]
# DRAM bytes per interior cell per launch measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum of the batch-8 capture, 0.52 M cells, summarised in
# profiles/top_kernels_rans_sa_513x129_b8_fp32mixed.md), scaled to the batch
TRAFFIC_PER_CELL = {"residual": (40.552192e6 + 0.333312e6) / (8 * 65536),
                    # k_lu_prep + both sweeps (k_lu_edges, ~1 % of the phase, not captured)
                    "lusgs": (31.611648e6 + 9.395712e6 + 62.382336e6 + 2.520320e6 + 62.393856e6 + 1.144576e6)
                    / (8 * 65536)}
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


def batch_cases(n, seed=0, jmax=JMAX, kmax=KMAX):
    from turns2d_urans_git_gb300 import api
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        alfa = 10.0 if i == 0 else float(rng.uniform(0.0, 10.0))
        out.append(api.config_c2(jmax=jmax, kmax=kmax, alfa=alfa))
    return out


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
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference(cases, max_threads=None, target_s=12.0):
    """The reference algorithm (CPU FP64 oracle) on the host cores: one
    request per thread, each a bounded number of iterations.  Returns
    (cell-updates/s, threads, sample description)."""
    from tests import oracle_binding as ob
    ob.lib()
    ncores = os.cpu_count() or 1
    nthr = min(max_threads or ncores, ncores, len(cases))
    # size the sample from one short probe
    _, prm, xv, yv = cases[0]
    t0 = time.perf_counter()
    ob.solve(prm, xv.ravel(), yv.ravel(), 2)
    per_it = (time.perf_counter() - t0) / 2
    iters = max(2, int(target_s / max(per_it, 1e-6)))
    cells = (prm.jmax - 1) * (prm.kmax - 1)
    results = [None] * nthr

    def work(i):
        _, p, x, y = cases[i % len(cases)]
        t = time.perf_counter()
        n, _, _, _ = ob.solve(p, x.ravel(), y.ravel(), iters)
        results[i] = (abs(n), time.perf_counter() - t)

    th = [threading.Thread(target=work, args=(i,)) for i in range(nthr)]
    t0 = time.perf_counter()
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.perf_counter() - t0
    done = sum(r[0] for r in results)
    value = done * cells / wall
    sample = "%d requests x %d iterations of the 513x129 SA case on %d threads (%.1f s wall)" % (nthr, iters, nthr, wall)
    return value, nthr, sample


def serve_stream(precision, reqs, arrivals, orders, max_iters, check_every, device, cap_s, force_tol):
    """Continuous-batching service of a request stream: requests are
    admitted at the first status check after their arrival time and retired
    when converged (L2 norm `orders` decades below its running peak), failed
    or capped.  Returns per-request (arrival, done, result) and the makespan
    (s); stops admitting and gives up after cap_s seconds."""
    from turns2d_urans_git_gb300 import api
    sv = api.Solver(precision, device=device, check_every=check_every)
    if force_tol:
        sv.set_force_tol(*force_tol)
    t0 = time.perf_counter()
    pending = sorted(zip(arrivals, range(len(reqs))))
    admitted = {}
    while True:
        now = time.perf_counter() - t0
        while pending and pending[0][0] <= now:
            ta, i = pending.pop(0)
            _, prm, xv, yv = reqs[i]
            admitted[sv.add(prm, xv, yv, orders=orders, max_iters=max_iters)] = (i, ta, now)
        if sv.live() == 0:
            if not pending or now > cap_s:
                break
            time.sleep(max(0.0, min(pending[0][0] - now, 0.05)))
            continue
        if now > cap_s:
            break
        sv.iterate(check_every)
        sv.sync()
    sv.sync()
    t_end = time.perf_counter() - t0
    out = []
    for iid, (i, ta, tadm) in admitted.items():
        r = sv.result(iid)
        out.append((i, ta, r))
    # the solver clock starts at creation, the same origin as t0 up to the
    # constructor's duration (t_done in its own seconds)
    sv.close()
    return out, t_end


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


def serving_section(args, device):
    """FP32-mixed vs FP64 on the same seeded request stream: converged
    solves/s and p50/p99 time to a converged solution."""
    from turns2d_urans_git_gb300 import api
    from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED, OT2D_FP64
    rng = np.random.default_rng(7)
    sizes = ((129, 33), (257, 65))
    reqs = [api.config_c4_sample(rng, sizes=sizes) for _ in range(args.serve_requests)]
    gaps = rng.exponential(1.0 / args.serve_rate, len(reqs))
    arrivals = np.cumsum(gaps) - gaps[0]
    res = {}
    for name, prec in (("fp32_mixed", OT2D_FP32_MIXED), ("fp64", OT2D_FP64)):
        out, t_end = serve_stream(prec, reqs, arrivals, args.serve_orders, args.serve_max_iters, 25, device,
                                  args.serve_seconds, (args.serve_dcl, args.serve_dcd))
        lat = [r.t_done - ta for (i, ta, r) in out if r.converged]
        conv = len(lat)
        res[name] = {"requests": len(reqs), "admitted": len(out), "converged": conv,
                     "solves_per_s": conv / t_end if t_end > 0 else None,
                     "p50_s": float(np.percentile(lat, 50)) if lat else None,
                     "p99_s": float(np.percentile(lat, 99)) if lat else None,
                     "makespan_s": t_end,
                     "forces": {i: (r.cl, r.cd, r.cm) for (i, ta, r) in out if r.converged}}
    a, b = res["fp32_mixed"].pop("forces"), res["fp64"].pop("forces")
    both = sorted(set(a) & set(b))
    dcls = sorted(abs(a[i][0] - b[i][0]) for i in both)
    dcl = dcls[-1] if dcls else None
    dcd = max((abs(a[i][1] - b[i][1]) for i in both), default=None)
    sm, sd = res["fp32_mixed"]["solves_per_s"], res["fp64"]["solves_per_s"]
    return {"workload": "%d seeded RANS-SA requests (NACA 4-digit m,p,t; M 0.3-0.85; a -2..8 deg; Re 1e6-1e7; "
                        "meshes %s), Poisson arrivals %.1f/s; converged = L2 norm %.0f decades below its peak, or "
                        "CL/CD within a band of %.0e/%.0e over 8 checks of 25 iterations with the norm a decade "
                        "below its peak"
                        % (len(reqs), "/".join("%dx%d" % s_ for s_ in sizes), args.serve_rate, args.serve_orders,
                           args.serve_dcl, args.serve_dcd),
            "fp32_mixed": res["fp32_mixed"], "fp64": res["fp64"],
            "speedup_solves_per_s": (sm / sd) if sm and sd else None,
            "max_abs_dcl_vs_fp64": dcl, "max_abs_dcd_vs_fp64": dcd, "compared": len(both),
            "p50_abs_dcl_vs_fp64": float(np.percentile(dcls, 50)) if dcls else None,
            "n_abs_dcl_over_1e-3": sum(1 for v in dcls if v > 1e-3)}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    cases = batch_cases(max(args.batch, os.cpu_count() or 1))
    t0 = time.perf_counter()
    vals = []
    for _ in range(args.warmup):
        pass  # the oracle has no warm state
    per_step = max(1.0, min(args.ref_seconds, 150.0 / max(args.steps, 1)))
    for _ in range(args.steps):
        v, thr, sample = cpu_reference(cases, target_s=per_step)
        vals.append(v)
    value = float(np.median(vals))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded algebraic C-meshes)",
            "config": {"workload": WORKLOAD, "batch": len(cases), "per_step": "bounded sample, see cpu_baseline"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": thr, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)
    return 0


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

    def make(precision):
        sv = api.Solver(precision, device=local, check_every=10 ** 8)
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
    resident = sv.device_bytes()
    sv.iterate(args.warmup)
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    ms = timed(sv, args.steps)
    clocks = clk.stop()
    value = whole_job_rate(B * cells * args.steps, world, ms / 1e3)
    # phase timers of the same batch -> dominant kernel + roofline
    prof = (C.c_double * NPH)()
    api.lib().ot2d_solver_profile.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int32]
    rc = api.lib().ot2d_solver_profile(sv._h, 5, prof, NPH)
    phase_ms = {PHASES[i]: prof[i] for i in range(NPH)} if rc == 0 else {}
    dom = max(range(NPH), key=lambda i: prof[i]) if rc == 0 else 4
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    alg = ALG_BYTES_F32[dom] * B * cells
    achieved = alg / (prof[dom] * 1e-3) / 1e9 if rc == 0 and prof[dom] > 0 else None
    # ---- e2e through the host-buffer ABI path
    qh = [np.zeros(prm.jd * prm.kd * prm.nspec * prm.nq) for (_, prm, _, _) in cases]
    for iid, (_, prm, _, _), q in zip(ids, cases, qh):
        q[:] = sv.get_q(iid, prm)
    pinned = []
    for q in qh:
        t = torch.from_numpy(q).pin_memory()
        pinned.append(t)
    ptrs = (C.POINTER(C.c_double) * B)(*[C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)) for t in pinned])
    idarr = (C.c_int32 * B)(*ids)
    L = api.lib()
    L.ot2d_solver_iterate_host.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                           C.POINTER(C.POINTER(C.c_double)), C.c_int32]
    e2e_steps = max(3, args.steps // 2)
    L.ot2d_solver_iterate_host(sv._h, B, idarr, ptrs, 1)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc2 = L.ot2d_solver_iterate_host(sv._h, B, idarr, ptrs, e2e_steps)
    torch.cuda.synchronize()
    e2e_s = rank_max(time.perf_counter() - t0, dist, "cuda")
    qbytes = sum(q.nbytes for q in qh)
    e2e = whole_job_rate(B * cells * e2e_steps, world, e2e_s) if rc2 == 0 else None
    sv.close()
    # ---- plain FP64 on the same batch (reported beside the headline)
    fp64 = None
    if not args.skip_fp64:
        sv64, _ = make(OT2D_FP64)
        sv64.iterate(1)
        torch.cuda.synchronize()
        k64 = max(2, args.fp64_steps)
        ms64 = timed(sv64, k64)
        fp64 = whole_job_rate(B * cells * k64, world, ms64 / 1e3)
        sv64.close()
    # ---- served request stream (rank 0 only): converged solves/s, p50/p99
    serve = None
    if rank == 0 and not args.skip_serve:
        serve = serving_section(args, local)
    unsteady = time_accurate_section(local) if rank == 0 else None
    # ---- CPU baseline (rank 0, N=1 only): the oracle on the host cores
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        v, thr, sample = cpu_reference(batch_cases(os.cpu_count() or 1), target_s=args.ref_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": thr, "kind": "port", "sample": sample}
    if rank == 0:
        # kernels per iteration: iter_begin, time_step, 5 BC entries + the
        # halo-ring pass, resid + norm_final, rbc, 4 LU-SGS, update, and 6 of SA
        launches_per_step = 16 + 6
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (f64 state update, norms, forces)",
                "data": "synthetic (seeded algebraic NACA0012 C-meshes, freestream start)",
                "config": {"workload": WORKLOAD, "batch_per_gpu": B, "interior_cells": cells,
                           "parallelism": "replicas x%d" % world, "precision": "fp32-mixed",
                           "l2": "inputs larger than L2: %.0f MB resident per GPU (L2 129 MB)" % (resident / 1e6)},
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": qbytes, "d2h_bytes_per_step": qbytes},
                "fp64_plain": {"value": fp64, "unit": UNIT},
                "gpu_launches": launches_per_step * args.steps,
                "phase_ms": phase_ms,
                "roofline": {"bound": "hbm", "kernel": PHASES[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": (achieved / peak) if achieved else None,
                             "traffic": (TRAFFIC_PER_CELL[PHASES[dom]] * B * cells
                                         if PHASES[dom] in TRAFFIC_PER_CELL else None),
                             "traffic_note": "bytes per launch, ncu batch-8 capture scaled by cells",
                             "peak_source": "measured" if peaks else "fallback"},
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--serve-rate", type=float, default=8.0)
    ap.add_argument("--serve-orders", type=float, default=10.0)
    ap.add_argument("--serve-dcl", type=float, default=1e-5)
    ap.add_argument("--serve-dcd", type=float, default=1e-6)
    ap.add_argument("--serve-max-iters", type=int, default=20000)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--skip-serve", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
