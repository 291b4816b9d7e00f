"""Autotuner for the batched launch.

Picks the sweep CTA size (modes per CTA tile), the number of persistent
CTAs per SM and the lines per CTA of the output-transform passes for a batch
shape by timing candidates on the device with the library's stage timers
(CUDA events around each stage: first the sweep shape on the sweep's time,
then the transform lines on the transforms' time), and caches the
winner in a JSON file keyed by GPU name and a coarse shape signature (total
solved modes, deepest level count, number of cases).
Cache file: $BLDFM_GB300_CACHE or ~/.cache/bldfm_gb300/autotune.json.
"""

import json
import os

import numpy as np
import torch

from . import _lib
from .batch import BatchSolver

# sweep launch shapes (threads per CTA, CTAs per SM; 0 = as many as fit).
# (256, 3) and (128, 7) leave registers free on every SM for a transform CTA
# of another stream, which the pipelined timing below can reward.
CANDIDATES = [(256, 0), (256, 6), (128, 0), (128, 12), (128, 18), (256, 3), (128, 7)]
# transform passes: 16 = register-resident lines, the column pass zoomed
# for the cases whose band and kept window allow it, 8 = register-resident
# lines unzoomed (both one launch per group of cases sharing their line
# configs; a batch with an unsupported line length falls back to the
# shared-memory passes), 4 / 2 / 1 = shared-memory passes with that many
# lines per CTA
XFORM_LINES = [16, 8, 4, 2, 1]
SIGNATURE_VERSION = 4  # bumped when the candidates or the kernels behind them change: older winners are ignored


def _cache_path():
    p = os.environ.get("BLDFM_GB300_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "bldfm_gb300", "autotune.json")


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
    except OSError:
        pass


def signature(cases):
    """Coarse shape key: modes to 2^k buckets, levels to 16s, cases to 2^k."""
    from .solver import make_desc, plan

    total, maxnz = 0, 0
    for kw in cases:
        d = make_desc(np.shape(kw["srf_flx"]), len(kw["z"]), kw["domain"], kw.get("modes", (512, 512)),
                      kw.get("meas_pt", (0.0, 0.0)), 0.0, bool(kw.get("footprint", False)), False, kw.get("halo"),
                      kw.get("precision", "single"), "fp32")
        info = plan(d, 1)
        total += int(info.nsolved)
        maxnz = max(maxnz, len(kw["z"]))
    b = lambda v: 1 << max(0, int(v - 1).bit_length())  # noqa: E731
    return "v%d|%s|modes%d|nz%d|cases%d" % (SIGNATURE_VERSION, torch.cuda.get_device_name(), b(total),
                                            16 * ((maxnz + 15) // 16), b(len(cases)))


def _time(cases, reps, stage, **opts):
    """Device time of one stage of the batched solve (the library's stage
    timers: 1 = sweep, 2 = output transforms), averaged over reps solves."""
    import ctypes

    lib = _lib.load()
    s = BatchSolver(use_graph=False, **opts)
    s.solve(cases)  # warm
    s.stream.synchronize()
    _lib.check(lib.bldfm_set_stage_timing(1), "stage timing")
    try:
        for _ in range(reps):
            s.solve(cases)
        s.stream.synchronize()
        arr = (ctypes.c_float * 8)()
        nst = lib.bldfm_stage_times(arr, 8)
    finally:
        lib.bldfm_set_stage_timing(0)
    if s.status() != 0 or nst <= stage:
        return None
    return float(arr[stage])


def _time_pipeline(cases, streams, nbatch, **opts):
    """Device time of nbatch solves of the batch taken in turn by `streams`
    solvers (own stream, workspace and graphs each), as solve_stream runs
    them: one batch's transforms overlap the next batch's sweep."""
    solvers = [BatchSolver(use_graph=True, **opts) for _ in range(streams)]
    preps = [s.prepare_cached(cases) for s in solvers]
    for s, p in zip(solvers, preps):
        s.solve_prepared(p)  # warm: captures each solver's graph
    torch.cuda.synchronize()
    main = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(main)
    for s in solvers:
        s.stream.wait_event(e0)
    for i in range(nbatch):
        solvers[i % streams].solve_prepared(preps[i % streams])
    for s in solvers:
        done = torch.cuda.Event()
        done.record(s.stream)
        main.wait_event(done)
    e1.record(main)
    e1.synchronize()
    if any(s.status() != 0 for s in solvers):
        return None
    return e0.elapsed_time(e1)


def tune(cases, reps=5, use_cache=True, streams=4):
    """Return (threads, ctas_per_sm, xform_lines) for this batch shape (timed or cached).

    The sweep shape is timed alone first and the transform lines per CTA for
    it.  With streams > 1 (the solve_stream default of four solvers), every
    sweep shape is then timed again in the pipelined run, where a shape that
    leaves room for the other streams' transforms can win although its sweep
    alone is slower; streams=1 tunes for synchronous solve_batch calls."""
    key = signature(cases) + ("|streams%d" % streams if streams > 1 else "")
    cache = _load() if use_cache else {}
    if key in cache and "xform_lines" in cache[key]:
        v = cache[key]
        return int(v["threads"]), int(v["ctas_per_sm"]), int(v["xform_lines"])
    best, best_ms = CANDIDATES[0], None
    for threads, per_sm in CANDIDATES:
        ms = _time(cases, reps, 1, threads=threads, ctas_per_sm=per_sm)
        if ms is not None and (best_ms is None or ms < best_ms):
            best, best_ms = (threads, per_sm), ms
    best_xl, best_xms = 0, None
    for xl in XFORM_LINES:
        ms = _time(cases, reps, 2, threads=best[0], ctas_per_sm=best[1], xform_lines=xl)
        if ms is not None and (best_xms is None or ms < best_xms):
            best_xl, best_xms = xl, ms
    if streams > 1:
        best_pms = None
        for threads, per_sm in CANDIDATES:
            runs = [_time_pipeline(cases, streams, 8 * streams, threads=threads, ctas_per_sm=per_sm,
                                   xform_lines=best_xl) for _ in range(2)]
            runs = [r for r in runs if r is not None]
            if runs and (best_pms is None or min(runs) < best_pms):
                best, best_pms = (threads, per_sm), min(runs)
    if use_cache:
        cache[key] = {"threads": best[0], "ctas_per_sm": best[1], "xform_lines": best_xl, "ms": best_xms}
        _save(cache)
    return best[0], best[1], best_xl
