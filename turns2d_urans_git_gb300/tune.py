"""Autotuner of the batched solver's launch choices.

For each mesh-size class it times a batch of that class under every
candidate choice and keeps the fastest:

  rt_shape   the fused residual's tile, 16x16, 32x8, 8x32 (256 threads) or
             32x16 (512 threads) interior cells per CTA (staged halo per
             cell against threads per face line)
  lu_group   LU-SGS record chunks streamed per bulk copy (4 or 8)
  lu_lag     LU-SGS hyperplane schedule: steps each 32-row band trails the
             band it depends on beyond the minimum (0 or 4)
  pipeline   a batch of 16 or more time instances as one graph (0), as two
             halves on two streams with each half's residual beside the
             other half's sweeps (1), or as four independent parts on four
             streams (2)

The fastest choice depends on the batch as well as on the mesh: the
pipelined halves pay off when the sweeps of a small batch leave most SMs
idle, and not at 64 instances of 513x129.  A search is therefore made at a
stated batch size (the measuring function's `batch`), and that size is part
of the cache key; a caller tunes at the batch it serves.

Every candidate computes the same state bit for bit (the choices change
launch geometry and schedule only; the L2 norm's partial sums follow the
residual tile, so the norms agree to rounding), so the search is free to
pick on time alone.  Choices are cached in a JSON file keyed by GPU name, precision and
size class, and handed to a solver as its tuning table
(ot2d_solver_set_tuning), which applies the entry of each batch's largest
mesh when it builds the batch.
"""
import ctypes as C
import json
import os
import statistics
import time

from .abi import (OT2D_FP64, OT2D_FP32_MIXED, OT2D_OPT_LU_GROUP, OT2D_OPT_LU_LAG, OT2D_OPT_PIPELINE,
                  OT2D_OPT_RT_SHAPE, Tuning)

# the mesh sizes of the batched configuration (vertices); a class covers
# meshes up to its array size (jd = jmax + 1, kd = kmax + 1)
SIZE_CLASSES = ((129, 33), (257, 65), (385, 97), (513, 129), (769, 193))
SHAPES = {0: "16x16", 1: "32x8", 2: "8x32", 3: "32x16"}
CANDIDATES = tuple((shape, group, lag, pipe) for shape in (0, 1, 2, 3) for group in (4, 8) for lag in (0, 4)
                   for pipe in (0, 1, 2))


def default_cache_path():
    root = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(root, "turns2d_gb300", "tuning.json")


def class_key(gpu, precision, jmax, kmax, batch=None):
    key = "%s|%s|%dx%d" % (gpu, "fp64" if precision == OT2D_FP64 else "fp32-mixed", jmax, kmax)
    return key + ("|b%d" % batch if batch else "")


def search(candidates, measure, repeats=3):
    """The candidate with the smallest median of `repeats` measurements
    (ms); returns (best, {candidate: median ms}).  Ties keep the earlier
    candidate."""
    times = {}
    for c in candidates:
        times[c] = statistics.median(measure(c) for _ in range(repeats))
    best = min(candidates, key=lambda c: (times[c], candidates.index(c)))
    return best, times


def load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(path, cache):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tuning_table(choices):
    """ot2d_tuning entries from {(jmax, kmax): (shape, group, lag, pipeline)},
    smallest class first (the solver takes the first entry that bounds a
    batch's largest mesh)."""
    rows = sorted(choices.items(), key=lambda kv: (kv[0][1], kv[0][0]))
    table = (Tuning * len(rows))()
    for t, ((jmax, kmax), (shape, group, lag, pipe)) in zip(table, rows):
        t.kd_max, t.jd_max = kmax + 1, jmax + 1
        t.rt_shape, t.lu_group, t.lu_lag, t.pipeline = shape, group, lag, pipe
    return table


def tune(measure_for_class, classes, gpu, precision, cache_path=None, retune=False, batch=None):
    """Choices for every class: from the cache, or searched with
    measure_for_class(jmax, kmax) -> measure(candidate) and then cached.
    `batch` (default: measure_for_class.batch, if it has one) is the batch
    size the search runs at, part of the cache key.
    Returns ({(jmax, kmax): choice}, {class: timings or None if cached})."""
    if batch is None:
        batch = getattr(measure_for_class, "batch", None)
    cache_path = cache_path or default_cache_path()
    cache = load_cache(cache_path)
    choices, timings = {}, {}
    changed = False
    for (jmax, kmax) in classes:
        key = class_key(gpu, precision, jmax, kmax, batch)
        hit = cache.get(key)
        if hit and not retune and tuple(hit["choice"]) in CANDIDATES:
            choices[(jmax, kmax)] = tuple(hit["choice"])
            timings[(jmax, kmax)] = None
            continue
        measure = measure_for_class(jmax, kmax)
        try:
            best, times = search(CANDIDATES, measure)
        finally:
            sv = getattr(measure, "solver", None)
            if sv is not None:
                sv.close()
        choices[(jmax, kmax)] = best
        timings[(jmax, kmax)] = times
        cache[key] = {"choice": list(best), "ms": {",".join(str(x) for x in c): t for c, t in times.items()},
                      "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
        changed = True
    if changed:
        save_cache(cache_path, cache)
    return choices, timings


def gpu_measure_for_class(precision, batch=16, iters=10, device=0, case_for_class=None):
    """measure_for_class on the GPU: a batch of `batch` requests of the class,
    each candidate timed with CUDA events over `iters` iterations of the
    captured iteration after 3 warm-up iterations."""
    import torch
    from . import api

    def for_class(jmax, kmax):
        if case_for_class is None:
            # NACA 0012 RANS-SA requests of the class at moderate incidence
            # (requests that stay finite over the timed iterations)
            cases = [api.config_c2(jmax, kmax, fsmach=0.3, alfa=0.25 * i, rey=5e6, ds_wall=api.wall_spacing(kmax))
                     for i in range(batch)]
        else:
            cases = [case_for_class(jmax, kmax, i) for i in range(batch)]
        sv = api.Solver(precision, device=device, check_every=10 ** 8)
        for (_, prm, xv, yv) in cases:
            sv.add(prm, xv, yv, orders=0.0, max_iters=10 ** 8)

        def measure(c):
            shape, group, lag, pipe = c
            sv.set_option(OT2D_OPT_RT_SHAPE, shape)
            sv.set_option(OT2D_OPT_LU_GROUP, group)
            sv.set_option(OT2D_OPT_LU_LAG, lag)
            sv.set_option(OT2D_OPT_PIPELINE, pipe)
            sv.iterate(3)
            st = torch.cuda.ExternalStream(sv.stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            sv.iterate(iters)
            e1.record(st)
            e1.synchronize()
            return e0.elapsed_time(e1) / iters

        measure.solver = sv
        return measure

    for_class.batch = batch
    return for_class


def apply(solver, choices):
    """Hand the choices to a solver (api.Solver) as its tuning table."""
    from . import api
    table = tuning_table(choices)
    f = api.lib().ot2d_solver_set_tuning
    f.argtypes = [C.c_void_p, C.POINTER(Tuning), C.c_int32]
    rc = f(solver._h, table, len(table))
    if rc != 0:
        raise RuntimeError("ot2d_solver_set_tuning failed (%d)" % rc)
    return table


def describe(choices):
    return {"%dx%d" % k: {"rt_tile": SHAPES[v[0]], "lu_group": v[1], "lu_lag": v[2], "pipeline": v[3]}
            for k, v in sorted(choices.items())}
