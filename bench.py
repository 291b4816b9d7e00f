#!/usr/bin/env python
"""Benchmark: footprints/s of the steady-state transport solve on one GB300.

Workload (the reference's headline configuration, synthetic met timeseries):
footprint mode, 512 x 512 physical grid on a 1000 m x 1000 m domain with the
default halo (1536 x 1536 extended grid), 512 x 512 Fourier modes,
vertical_profiles(n=128, z_m=20 m) -> 207 levels, unstable MOST profiles
(L = -50 m, u* ~ 0.3 m/s, 4 m/s wind around 225 deg), tower at (500, 500) m.
One step = one batch of B footprints for B met cases (seeded).

Reported:
  value          batched FP32 invariant-imbedding path (bldfm_solve_batch,
                 replayed as a CUDA graph, device-resident outputs),
                 footprints/s over K timed steps cycling 4 met batches
  single_fp32    one bldfm_solve per footprint (no batching)
  fp64           the FP64 path (reference rounding), one solve per footprint
  e2e            the public batched API solve_batch (numpy in, numpy out,
                 host<->device copies inside); also the single-case drop-in
  roofline       the batched sweep kernel against the measured FP32 FMA peak
  surrogate      the learned surrogate (trained weights in
                 bldfm_gb300/weights): footprints/s and relL2 against FP64
  timeseries     512 mixed-grid met cases (8 towers, 256^2..1024^2,
                 n = 64..256) in one batched call per step
  production     the 1024^2-extended, n = 256 footprint: FP64 / FP64
                 accurate / FP32 on the GPU, the CPU port, analytic check
  serving        surrogate serving with fallback on a 1024^2 footprint
                 timeseries (10% outside the training box)
  cpu_baseline   the CPU oracle port (reference arithmetic, OpenMP on all
                 host cores) on a bounded sample

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""

import argparse
import gc
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

NX = NY = 512
DOMAIN = (1000.0, 1000.0)
N_LEVELS = 128
ZM = 20.0
MODES = (512, 512)
MEAS = (500.0, 500.0)
# DRAM traffic per launch of the batched FP32 sweep (16 footprints of the
# workload), dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture:
# 0.81 MB read + 9.01 MB written (a compute kernel; most of the spectra
# stay in L2 for the transforms)
RICC_BATCH_DRAM_BYTES = 9.82e6

# algorithmic flops per (mode, sweep step), FMA counted as 2; the FP32 sweep's
# count per mode comes from bldfm_sweep32_flops (it depends on the output level)
F64_FLOPS_PER_MODE_STEP = 88  # reference shooting step, both IVPs (src/bldfm/solver.py:357-368)
WORKLOAD_NAME = "footprint 512x512 (ext 1536x1536), modes 512x512, n=128 (207 levels), unstable MOST"


def met_cases(batch, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(batch):
        out.append(
            dict(
                ustar=float(rng.uniform(0.25, 0.35)),
                mol=-50.0,
                wind_speed=4.0,
                wind_dir=float(225.0 + rng.uniform(-30.0, 30.0)),
            )
        )
    return out


def profiles_for(case, device_profiles):
    from bldfm_gb300.utils import compute_wind_fields

    wind = compute_wind_fields(case["wind_speed"], case["wind_dir"])
    if device_profiles:
        from bldfm_gb300 import vertical_profiles
    else:
        from oracle.bldfm_oracle import vertical_profiles
    return vertical_profiles(N_LEVELS, ZM, wind, ustar=case["ustar"], mol=case["mol"])


def solver_kwargs(z, profs, precision="double"):
    return dict(
        srf_flx=np.zeros((NY, NX)), z=z, profiles=profs, domain=DOMAIN, levels=N_LEVELS, modes=MODES,
        meas_pt=MEAS, footprint=True, precision=precision,
    )


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler delivers (bounded wait)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": smax,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def cpu_port_time(kw, reps=2):
    """Oracle C port (reference arithmetic) on all host cores: seconds/footprint."""
    from oracle import bldfm_oracle as O
    from oracle import build_oracle

    build_oracle()
    O.steady_state_transport_solver(**kw)  # warm (thread pool, pages)
    best = 1e30
    for _ in range(reps):
        t = time.perf_counter()
        O.steady_state_transport_solver(**kw)
        best = min(best, time.perf_counter() - t)
    return best


def run_reference(args):
    """--impl reference: the reference's CPU implementation of the path (the
    oracle port: the reference's arithmetic, OpenMP over modes on all cores,
    numpy FFT) on the same workload; one footprint per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cases = met_cases(max(args.steps + args.warmup, 1), seed=1)
    kws = []
    for c in cases:
        z, p = profiles_for(c, device_profiles=False)
        kws.append(solver_kwargs(z, p))
    from oracle import bldfm_oracle as O
    from oracle import build_oracle

    build_oracle()
    for i in range(args.warmup):
        O.steady_state_transport_solver(**kws[i % len(kws)])
    t = time.perf_counter()
    for i in range(args.steps):
        O.steady_state_transport_solver(**kws[(args.warmup + i) % len(kws)])
    dt = time.perf_counter() - t
    fps = args.steps / dt
    cores = os.cpu_count()
    line = {
        "impl": "reference",
        "metric": "footprints/s",
        "value": fps,
        "unit": "footprints/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "footprints_per_step": 1, "path": "CPU oracle port"},
        "cpu_baseline": {
            "value": fps, "unit": "footprints/s", "cores": cores, "kind": "port",
            "sample": "1 footprint per step: C port of the reference sweep (OpenMP, %d threads) + numpy FFT" % cores,
        },
        "e2e": {"value": fps, "unit": "footprints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def measured_peaks():
    """HBM GB/s and dense BF16 TFLOP/s measured on the GB300s
    (MEASURED_PEAKS.json), else the fallback figures."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def transform_section(stages_b, B, dev, xlines):
    """Achieved GB/s of the batched output transform (algorithmic bytes: the
    two FP32 spectra read, conc and flx written) against the HBM peak, and a
    cuFFT timing of the same transform size (torch.fft, comparison only).
    xlines: the transform setting the step ran with (16 or 0: register-
    resident passes with the zoomed column pass where the geometry allows it,
    8: register-resident passes, else shared-memory passes with that many
    lines per CTA)."""
    import torch

    peaks = measured_peaks()
    bytes_fp = MODES[0] * MODES[1] * 8 * 2 + 2 * NY * NX * 8
    ms = stages_b[2] if stages_b and len(stages_b) > 2 else None
    achieved = B * bytes_fp / (ms * 1e-3) / 1e9 if ms else None
    # cuFFT: the full 1536 x 1536 complex64 2D inverse transform of B spectra
    n = 3 * NX
    x = torch.randn(B, n, n, dtype=torch.complex64, device=dev)
    torch.fft.ifft2(x)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        torch.fft.ifft2(x)
    e1.record()
    torch.cuda.synchronize()
    cufft_ms = e0.elapsed_time(e1) / 5
    del x
    return {
        "kernels": ("rz_cols_batch_kernel (zoomed register-resident column lines) + rx2_rows_batch_kernel"
                    if xlines in (0, 16) else
                    "rx_cols_batch_kernel + rx2_rows_batch_kernel (register-resident lines)" if xlines == 8
                    else "out_cols_batch_kernel + out_rows_batch_kernel (shared-memory lines, %d per CTA)" % xlines),
        "ms_per_footprint": ms / B if ms else None,
        "bytes_per_footprint": bytes_fp,
        "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": achieved / peaks["hbm_gbs"] if achieved else None, "peak_source": peaks["source"],
        "cufft_full_2d_ifft_1536x1536_c64_ms_per_footprint": cufft_ms / B,
    }


def timeseries_section(args, dev):
    """The 512-case mixed-grid met timeseries (8 towers, 256^2 / 512^2 /
    1024^2, n = 64..256) as one batched FP32 call per step: footprints/s with
    device-resident outputs, and relL2 against the exact discrete solution on
    one case per tower."""
    import torch

    from bldfm_gb300 import steady_state_transport_solver, vertical_profiles
    from bldfm_gb300.batch import BatchSolver
    from tests.timeseries_cases import met_cases

    cases = met_cases(512, seed=0)
    kws = []
    for c in cases:
        z, prof = vertical_profiles(c["n"], c["zm"], c["wind"], ustar=c["ustar"], mol=c["mol"])
        kws.append(dict(srf_flx=np.zeros((c["grid"], c["grid"])), z=z, profiles=prof, domain=c["domain"],
                        levels=c["n"], modes=(c["grid"], c["grid"]), meas_pt=c["meas_pt"], footprint=True,
                        precision="double"))
    solver = BatchSolver(use_graph=True)
    prep = solver.prepare_cached(kws)
    for _ in range(2):
        solver.solve_prepared(prep)
    solver.stream.synchronize()
    steps = 3
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(solver.stream)
    for _ in range(steps):
        solver.solve_prepared(prep)
    e1.record(solver.stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if solver.status() != 0:
        raise RuntimeError("timeseries device status %d" % solver.status())
    outs = prep[1]
    errs, seen = [], set()
    for c, kw, (conc, flx) in zip(cases, kws, outs):
        if c["tower"] in seen:
            continue
        seen.add(c["tower"])
        _, cr, fr = steady_state_transport_solver(**kw, mode="fp64r")
        ca, fa = conc[0].cpu().numpy(), flx[0].cpu().numpy()
        errs.append(max(np.linalg.norm(ca - cr) / np.linalg.norm(cr), np.linalg.norm(fa - fr) / np.linalg.norm(fr)))
    return {
        "workload": "512 met cases, 8 towers on 256^2/512^2/1024^2 grids (default halo, all modes), n=64..256, "
                    "u*~U[0.1,0.8], 1/L~U[-0.1,0.05], dir~U[0,360), z0 log-U[0.01,1], z_m~U[2,50] (seed 0)",
        "value": 512 / (ms * 1e-3), "unit": "footprints/s", "ms_per_batch": ms,
        "path": "one bldfm_solve_batch call (persistent FP32 sweep + batched transforms, CUDA graph)",
        "relL2_vs_exact_max_8_towers": max(errs),
    }


def production_section(args, lib, dev, sptr, cpu):
    """The production footprint: 512^2 physical, 500 m halo (1024^2 extended),
    all 1024^2 modes, n = 256, unstable MOST (L = -50 m, u* = 0.3, z_m = 20 m,
    4 m/s at 225 deg), FP64 (reference rounding), FP64 accurate and FP32 on
    the GPU, the CPU port timed on the host cores, plus the constant-profile
    analytic check."""
    import ctypes

    import torch

    from bldfm_gb300 import _lib
    from bldfm_gb300 import steady_state_transport_solver, vertical_profiles
    from bldfm_gb300.solver import make_desc, plan
    from bldfm_gb300.utils import compute_wind_fields

    wind = compute_wind_fields(4.0, 225.0)
    z, prof = vertical_profiles(256, 20.0, wind, ustar=0.3, mol=-50.0)
    zz = np.ascontiguousarray(z, dtype=np.float64)
    pr = np.ascontiguousarray(np.stack([np.broadcast_to(np.asarray(p, dtype=np.float64), zz.shape) for p in prof]))
    lv = np.array([256], dtype=np.int64)
    res = {}
    outs = {}
    for mode, reps in (("fp64", 2), ("fp64r", 2), ("fp32", 5)):
        d = make_desc((512, 512), zz.size, (1000.0, 1000.0), (1024, 1024), (500.0, 500.0), 0.0, True, False, 500.0,
                      "double", mode)
        info = plan(d, 1)
        ws = torch.empty(int(info.workspace_bytes), dtype=torch.uint8, device=dev)
        co = torch.empty((info.out_ny, info.out_nx), dtype=torch.float64, device=dev)
        fo = torch.empty_like(co)

        def run():
            _lib.check(lib.bldfm_solve(d, None, _lib.ptr(zz), _lib.ptr(pr), _lib.ptr(lv), 1,
                                       ctypes.c_void_p(co.data_ptr()), ctypes.c_void_p(fo.data_ptr()),
                                       ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()), sptr), mode)

        run()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.current_stream(dev))
        for _ in range(reps):
            run()
        e1.record(torch.cuda.current_stream(dev))
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[mode] = {"ms_per_footprint": ms, "footprints_per_s": 1e3 / ms}
        outs[mode] = (co.cpu().numpy(), fo.cpu().numpy())
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    cr, fr = outs["fp64r"]
    for mode in ("fp64", "fp32"):
        res[mode]["relL2_vs_exact"] = max(rel(outs[mode][0], cr), rel(outs[mode][1], fr))
    if cpu:
        kw = dict(srf_flx=np.zeros((512, 512)), z=zz, profiles=tuple(pr), domain=(1000.0, 1000.0), levels=256,
                  modes=(1024, 1024), meas_pt=(500.0, 500.0), footprint=True, precision="double", halo=500.0)
        sec = cpu_port_time(kw, reps=1)
        res["cpu_port"] = {"footprints_per_s": 1.0 / sec, "cores": os.cpu_count(), "kind": "port"}
    # constant K / constant u: the analytic branch against the numerical solve
    nz = zz.size
    const = tuple(np.full(nz, v) for v in (2.83, 2.83, 1.5, 1.5, 1.5))
    kwc = dict(srf_flx=np.zeros((256, 256)), z=zz, profiles=const, domain=(1000.0, 1000.0), levels=128,
               modes=(256, 256), meas_pt=(500.0, 500.0), footprint=True, precision="double")
    _, ca, fa = steady_state_transport_solver(**kwc, analytic=True, mode="fp64")
    _, cn, fn = steady_state_transport_solver(**kwc, mode="fp64r")
    res["analytic_check_relL2"] = max(rel(cn, ca), rel(fn, fa))
    res["workload"] = ("footprint 512^2, halo 500 m (1024^2 extended), modes 1024^2, n=256 (%d levels), "
                       "unstable MOST, u*=0.3, z_m=20 m" % nz)
    return res


def serving_cases(nsteps, seed=7):
    """The production footprint as a met timeseries for surrogate serving:
    512^2 grid on 1000 m with a 500 m halo (1024^2 extended, all 1024^2
    modes), n = 256 (413 levels), z_m = 20 m, 4 m/s, the met case of the
    production configuration varied around it (u* ~ U[0.22, 0.38] m/s,
    1/L ~ U[-0.045, 0.01] 1/m, wind direction ~ U[0, 360) deg), 10% of the
    steps drawn outside the network's training box (1/L ~ U[-0.1, -0.06]:
    strongly unstable)."""
    from bldfm_gb300.surrogate import BOX, met_scalars

    rng = np.random.default_rng(seed)
    out = []
    while len(out) < nsteps:
        outside = len(out) % 10 == 9
        ustar = float(rng.uniform(0.22, 0.38))
        inv_l = float(rng.uniform(-0.1, -0.06) if outside else rng.uniform(-0.045, 0.01))
        mol = 1.0 / inv_l if abs(inv_l) > 1e-6 else 1e6
        wd = np.deg2rad(float(rng.uniform(0.0, 360.0)))
        wind = (-4.0 * np.sin(wd), -4.0 * np.cos(wd))
        _, s1, s2, _ = met_scalars(20.0, wind, ustar=ustar, mol=mol)
        inside = BOX["s1"][0] <= s1 <= BOX["s1"][1] and BOX["s2"][0] <= s2 <= BOX["s2"][1]
        if inside == outside:
            continue
        out.append(dict(n=256, zm=20.0, wind=wind, srf_shape=(512, 512), domain=(1000.0, 1000.0),
                        modes=(1024, 1024), meas_pt=(500.0, 500.0), halo=500.0, ustar=ustar, mol=mol))
    return out


def serving_section(args, dev, nsteps=10000):
    """Surrogate serving with fallback on the production footprint as a
    10k-step met timeseries: wall time of Surrogate.serve (batched fused
    launches of the n = 256 network, accurate-FP64 fallback for the out-of-box steps,
    the per-case accuracy guard with FP32 re-solves, accurate-FP64 spot
    checks of every 64th served step), the path counts, and the relL2
    distribution of 16 served steps (sampled before the run) against the exact
    solution."""
    import torch

    from bldfm_gb300 import steady_state_transport_solver
    from bldfm_gb300 import surrogate as S

    if not os.path.exists(S.WEIGHTS_N256):
        return {"unavailable": "no trained n=256 weights (python -m bldfm_gb300.surrogate train --n 256 --kmax 48)"}
    net, box, meta = S.load(S.WEIGHTS_N256)
    items = serving_cases(nsteps)
    sur = S.Surrogate(net, box=box, spot_every=64, tol=1e-3)
    sur.serve(items[:16])  # warm (plans, twiddles, fallback path)
    sur = S.Surrogate(net, box=box, spot_every=64, tol=1e-3)
    # 12 in-box steps and 4 out-of-box ones (every 10th step, index 9 mod 10)
    sampled = sorted(set(list(range(5, nsteps, max(1, nsteps // 12)))[:12] +
                         list(range(9, nsteps, max(10, (nsteps // 40) * 10)))[:4]))
    torch.cuda.synchronize()
    t = time.perf_counter()
    out, paths = sur.serve(items, keep=sampled)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    # error distribution of the sampled steps' returned results against the
    # exact discrete solution, by the path that produced them
    errs = {}
    for k in sampled:
        pr = sur.prepare(**items[k])
        _, cr, fr = steady_state_transport_solver(**pr["kw"], mode="fp64r")
        c, f = out[k]
        c = c.cpu().numpy() if hasattr(c, "cpu") else np.asarray(c)
        f = f.cpu().numpy() if hasattr(f, "cpu") else np.asarray(f)
        errs.setdefault(paths[k], []).append(max(np.linalg.norm(c - cr) / np.linalg.norm(cr),
                                                 np.linalg.norm(f - fr) / np.linalg.norm(fr)))

    def dist(v):
        if not v:
            return None
        v = np.asarray(v)
        return {"n": int(v.size), "median": float(np.median(v)), "p90": float(np.quantile(v, 0.9)),
                "max": float(v.max()), "frac_le_1e-3": float((v <= 1e-3).mean())}

    st = sur.stats
    return {
        "workload": "%d-step footprint timeseries (10%% outside the training box): 512^2 grid, 1000 m domain, "
                    "500 m halo (1024^2 extended), modes 1024^2, n=256 (413 levels), z_m=20 m, u*~U[0.22,0.38], "
                    "1/L~U[-0.045,0.01] (outside: U[-0.1,-0.06]), 4 m/s, dir~U[0,360)" % nsteps,
        "network": {"weights": os.path.basename(S.WEIGHTS_N256), "box": box,
                    "train_steps": meta.get("steps"), "val_loss": meta.get("val_loss")},
        "value": len(items) / dt, "unit": "footprints/s (wall, incl. fallbacks, guard re-solves and spot checks)",
        "wall_s": dt,
        "paths": {p: paths.count(p) for p in set(paths)},
        "spot_checks": st["spot"], "spot_fail": st["spot_fail"],
        "spot_relL2": {"n": len(st["errors"]), "median": float(np.median(st["errors"])) if st["errors"] else None,
                       "max": float(np.max(st["errors"])) if st["errors"] else None},
        "guard": {"re_solved_fp32": st["guard_fail"], "checked": len(st["guard"]),
                  "estimate": dist(st["guard"]),
                  "guard_tol": sur.guard_tol,
                  "rule": "stratified sample (k = 0, |kx|,|ky| <= 2, every 61st solved mode) re-solved exactly on "
                          "the device; estimate > guard_tol (network's guard factor x 1e-3) -> FP32 solve"},
        "returned_relL2_vs_exact": {"sampled_steps": len(sampled),
                                    "by_path": {p: dist(v) for p, v in sorted(errs.items())},
                                    "all": dist([x for v in errs.values() for x in v])},
    }


def surrogate_section(kwb, inputs, s64, B, args, dev, dist, world, sr):
    """Footprints/s of the surrogate on batch 0's met cases (device-resident
    outputs, descriptors prepared once), its relL2 against the FP64 path, and
    the training throughput of the tensor-core MLP kernels."""
    import torch

    from bldfm_gb300 import surrogate as S
    from bldfm_gb300.mlp import MLP

    if not os.path.exists(S.WEIGHTS):
        return {"unavailable": "no trained weights at bldfm_gb300/weights (python -m bldfm_gb300.surrogate train)"}
    net, box, meta = S.load(S.WEIGHTS)
    sur = S.Surrogate(net, spot_every=0)
    preps, in_box = [], []
    for (z, p), c in zip(inputs, met_cases(B, seed=1000 + 97 * int(os.environ.get("RANK", "0")))):
        wd = np.deg2rad(c["wind_dir"])
        wind = (-c["wind_speed"] * np.sin(wd), -c["wind_speed"] * np.cos(wd))
        kw = dict(n=N_LEVELS, zm=ZM, wind=wind, srf_shape=(NY, NX), domain=DOMAIN, modes=MODES, meas_pt=MEAS,
                  ustar=c["ustar"], mol=c["mol"])
        pr = sur.prepare(**kw)
        pr["args"] = kw
        preps.append(pr)
        s1, s2, _ = pr["s"]
        in_box.append(sur.in_box(N_LEVELS, ZM, s1, s2, S.mode_kmax((NY, NX), DOMAIN, MODES)))
    # one step = the B footprints in one fused launch + the batched output
    # transform; two surrogate workspaces on two streams take the steps in turn
    # (one step's transforms overlap the next step's fused kernel)
    bat = sur.prepare_batch([pr["args"] for pr in preps])
    outs = bat["outs"]
    stream = torch.cuda.current_stream(dev)
    sur2 = S.Surrogate(net, spot_every=0)
    bat2 = sur2.prepare_batch([pr["args"] for pr in preps])
    pair = [(sur, bat, torch.cuda.Stream(dev)), (sur2, bat2, torch.cuda.Stream(dev))]
    for i in range(max(args.warmup, 2)):
        sv, bt, st = pair[i % 2]
        sv.solve_batch_prepared(bt, stream=st)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    from bldfm_gb300 import _lib
    import ctypes

    lib = _lib.load()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _, _, st in pair:
        st.wait_event(e0)
    for i in range(args.steps):
        sv, bt, st = pair[i % 2]
        sv.solve_batch_prepared(bt, stream=st)
    for _, _, st in pair:
        done = torch.cuda.Event()
        done.record(st)
        stream.wait_event(done)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    for sv, _, st in pair:
        if sv.status(stream=st) != 0:
            raise RuntimeError("surrogate device status %d" % sv.status(stream=st))
    # per-stage times (CUDA events inside the library) over the same steps
    lib.bldfm_set_stage_timing(1)
    for _ in range(args.steps):
        sur.solve_batch_prepared(bat)
    torch.cuda.synchronize()
    arr = (ctypes.c_float * 8)()
    nst = lib.bldfm_stage_times(arr, 8)
    lib.bldfm_set_stage_timing(0)
    stages = [float(arr[i]) for i in range(max(nst, 0))]
    serve_ms = stages[1] / B if len(stages) > 1 else None  # per footprint
    band_ms = stages[2] / B if len(stages) > 2 else None  # exact low band, per footprint
    guard_ms = stages[3] / B if len(stages) > 3 else None  # accuracy guard, per footprint
    nsolved = 131583
    npad = (nsolved + 127) // 128 * 128
    tflop = npad * (2 * 32 * 256 + 3 * 2 * 256 * 256) / 1e12  # tensor-core work per footprint
    peaks = measured_peaks()
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    errs = []
    if sur.status() != 0:
        raise RuntimeError("surrogate device status %d" % sur.status())
    for (c, f), b in zip(outs, s64):
        cb, fb = b[3].cpu().numpy(), b[4].cpu().numpy()
        ca, fa = c.cpu().numpy(), f.cpu().numpy()
        errs.append(max(np.linalg.norm(ca - cb) / np.linalg.norm(cb), np.linalg.norm(fa - fb) / np.linalg.norm(fb)))
    # against the exact discrete solution (accurate FP64 mode) on the first cases
    errx = []
    for (c, f), r in zip(outs, sr):
        cr, fr = r[3].cpu().numpy(), r[4].cpu().numpy()
        ca, fa = c.cpu().numpy(), f.cpu().numpy()
        errx.append(max(np.linalg.norm(ca - cr) / np.linalg.norm(cr), np.linalg.norm(fa - fr) / np.linalg.norm(fr)))
    # training throughput of the project's forward/backward kernels (batch 65536)
    pool = S.TransferPool(ncases=1024, seed=5)
    tnet = MLP(batch=65536, seed=9)
    S.train(tnet, pool, 3, batch=65536, log_every=1000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nsteps = 20
    S.train(tnet, pool, nsteps, batch=65536, log_every=1000)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    return {
        "value": world * B * args.steps / (ms * 1e-3),
        "unit": "footprints/s",
        "ms_per_footprint": ms / (args.steps * B),
        "relL2_vs_fp64_max": max(errs),
        "relL2_vs_fp64_median": float(np.median(errs)),
        "relL2_vs_exact_max": max(errx),
        "in_box": int(sum(in_box)),
        "kernel": "sur_serve_kernel (features -> 4 tcgen05 BF16 layers, split-BF16 input layer -> 256x4 -> spectra) "
                  "over the step's footprints, the exact low band (|k| z_m < %g by the FP32 sweep, "
                  "sur_lowband_kernel) and the accuracy guard, then the batched output FFT; two workspaces on two "
                  "streams take the steps in turn" % sur.exact_kz,
        "stage_ms_per_step": stages,
        "stages": ["upload", "serve kernel", "exact low band", "accuracy guard", "output transform"],
        "low_band_ms_per_footprint": band_ms,
        "guard_ms_per_footprint": guard_ms,
        "serve_kernel": {
            "ms_per_footprint": serve_ms,
            "bound": "tensor",
            "tensor_tflop_per_footprint": tflop,
            "achieved": (tflop / (serve_ms * 1e-3)) if serve_ms else None,
            "peak": peaks["bf16_tflops"],
            "unit": "TFLOP/s",
            "frac": (tflop / (serve_ms * 1e-3) / peaks["bf16_tflops"]) if serve_ms else None,
            "peak_source": peaks["source"],
        },
        "weights": {"box": box, **{k: meta[k] for k in meta if k in ("steps", "batch", "val_loss", "train_s")}},
        "training": {"ms_per_step": train_s / nsteps * 1e3, "samples_per_s": 65536 * nsteps / train_s,
                     "batch": 65536},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-extra", action="store_true", help="skip the timeseries and production sub-benchmarks")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import ctypes

    import torch

    from bldfm_gb300 import _lib
    from bldfm_gb300 import steady_state_transport_solver
    from bldfm_gb300.solver import make_desc, plan

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)

    B = args.batch
    NB = 4  # distinct met batches cycled through the timed steps
    batches = []
    for j in range(NB):
        cs = met_cases(B, seed=1000 + 97 * rank + j)
        batches.append([profiles_for(c, device_profiles=True) for c in cs])
    inputs = batches[0]
    kwb = [[solver_kwargs(z, p) for z, p in bt] for bt in batches]

    from bldfm_gb300 import autotune
    from bldfm_gb300.batch import BatchSolver, solve_batch

    threads, per_sm, xlines = autotune.tune(kwb[0])

    def make_solves(mode):
        solves = []
        for z, p in inputs:
            d = make_desc((NY, NX), len(z), DOMAIN, MODES, MEAS, 0.0, True, False, None, "double", mode)
            info = plan(d, 1)
            ws = torch.empty(int(info.workspace_bytes), dtype=torch.uint8, device=dev)
            conc = torch.empty((info.out_ny, info.out_nx), dtype=torch.float64, device=dev)
            flx = torch.empty_like(conc)
            zz = np.ascontiguousarray(z, dtype=np.float64)
            prof = np.ascontiguousarray(np.stack(p))
            lv = np.array([N_LEVELS], dtype=np.int64)
            solves.append((d, info, ws, conc, flx, zz, prof, lv))
        return solves

    def run_batch(solves):
        for d, info, ws, conc, flx, zz, prof, lv in solves:
            st = lib.bldfm_solve(
                d, None, _lib.ptr(zz), _lib.ptr(prof), _lib.ptr(lv), 1, ctypes.c_void_p(conc.data_ptr()),
                ctypes.c_void_p(flx.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()), sptr,
            )
            _lib.check(st, "bench")

    def timed(solves, steps, warmup, stage_timing=False):
        for _ in range(warmup):
            run_batch(solves)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        if stage_timing:
            lib.bldfm_set_stage_timing(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            run_batch(solves)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        stages = None
        if stage_timing:
            arr = (ctypes.c_float * 8)()
            n = lib.bldfm_stage_times(arr, 8)
            stages = [float(arr[i]) for i in range(max(n, 0))]
            lib.bldfm_set_stage_timing(0)
        if dist is not None:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, stages

    def timed_batches(solvers, steps, warmup, stage_timing=False):
        # descriptors built once per met batch (input preparation); each timed
        # step is one bldfm_solve_batch call: level tables, k = 0 values and
        # maps are computed from the profiles inside the call.  With several
        # solvers (own stream, workspace and graphs each) consecutive steps
        # go to them in turn, so one step's transforms overlap the next
        # step's sweep; the timed region spans all the streams.
        if not isinstance(solvers, (list, tuple)):
            solvers = [solvers]
        ns = len(solvers)
        preps = [[s.prepare_cached(kwb[j]) for j in range(NB)] for s in solvers]
        for i in range(max(warmup, ns)):
            solvers[i % ns].solve_prepared(preps[i % ns][i % NB])
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        if stage_timing:
            lib.bldfm_set_stage_timing(1)
        main = torch.cuda.current_stream(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(main)
        for s in solvers:
            s.stream.wait_event(e0)
        for i in range(steps):
            solvers[i % ns].solve_prepared(preps[i % ns][i % NB])
        for s in solvers:
            done = torch.cuda.Event()
            done.record(s.stream)
            main.wait_event(done)
        e1.record(main)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        stages = None
        if stage_timing:
            arr = (ctypes.c_float * 8)()
            n = lib.bldfm_stage_times(arr, 8)
            stages = [float(arr[i]) for i in range(max(n, 0))]
            lib.bldfm_set_stage_timing(0)
        if dist is not None:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, stages

    # --- headline: batched FP32 path replayed as a CUDA graph ---
    gsolvers = [BatchSolver(threads=threads, ctas_per_sm=per_sm, use_graph=True, xform_lines=xlines)
                for _ in range(4)]
    with ClockSampler(local) as clk:
        msb, _ = timed_batches(gsolvers, args.steps, args.warmup)
    fps_batch = world * B * args.steps / (msb * 1e-3)
    for gs in gsolvers:
        if gs.status() != 0:
            raise RuntimeError("device status %d" % gs.status())
    # same batches without the graph, with per-stage CUDA-event timers (roofline)
    tsolver = BatchSolver(threads=threads, ctas_per_sm=per_sm, use_graph=False, xform_lines=xlines)
    msnb, stages_b = timed_batches(tsolver, args.steps, args.warmup, stage_timing=True)
    fps_nograph = world * B * args.steps / (msnb * 1e-3)

    # --- single-footprint FP32 solves (bldfm_solve), for comparison ---
    s32 = make_solves("fp32")
    steps32 = min(args.steps, 60)
    ms32, stages32 = timed(s32, steps32, args.warmup, stage_timing=True)
    fps32 = world * B * steps32 / (ms32 * 1e-3)

    # --- e2e through the public batched API (numpy in, numpy out), measured
    # right after the device-resident runs, before the FP64 path, the CPU
    # oracle checks and the long sections, so that it sees the process state
    # a user's process has (the CPU checks and the 10k-step serving run leave
    # busy host threads and a large heap behind); the median of three passes ---
    from bldfm_gb300.batch import solve_stream, stream_depth

    esolver = BatchSolver(threads=threads, ctas_per_sm=per_sm, use_graph=True, xform_lines=xlines)
    e2e_steps = max(2, min(args.steps, 300))
    solve_batch(kwb[0], solver=esolver)
    gc.collect()
    t = time.perf_counter()
    for i in range(e2e_steps):
        solve_batch(kwb[i % NB], solver=esolver)
    e2e_sync = world * B * e2e_steps / (time.perf_counter() - t)
    # the pipelined timeseries API over the same steps: its default number of
    # solvers (batches in flight) take the steps in turn
    depth = stream_depth(kwb[0])
    ssolvers = tuple(BatchSolver(threads=threads, ctas_per_sm=per_sm, use_graph=True, xform_lines=xlines)
                     for _ in range(depth))
    # warm: graphs of every solver and the pinned host blocks a consumer that
    # holds one result while the next is produced keeps alive
    warm = list(solve_stream([kwb[i % NB] for i in range(2 * depth)], solvers=ssolvers))
    del warm
    e2e_passes = []
    for _ in range(3):
        gc.collect()
        t = time.perf_counter()
        nres = 0
        for res in solve_stream((kwb[i % NB] for i in range(e2e_steps)), solvers=ssolvers):
            nres += len(res)
        e2e_passes.append(world * nres / (time.perf_counter() - t))
    e2e_fps = statistics.median(e2e_passes)
    nz = len(inputs[0][0])
    # per case: FP32 table, float-pair table (the check's), FP64 columns, slot
    # map, k = 0 values, case record and maps (the upload blob)
    h2d = B * ((nz - 1) * (12 * 4 + 12 * 8 + 12 * 8) + nz * 4 + 32 + 640)
    d2h = B * 2 * NY * NX * 8
    # the single-footprint drop-in, for comparison
    kws = kwb[0]
    steady_state_transport_solver(**kws[0], mode="fp32")
    t = time.perf_counter()
    for kw in kws:
        steady_state_transport_solver(**kw, mode="fp32")
    e2e_single = world * B / (time.perf_counter() - t)

    # --- FP64 path (reference rounding) ---
    s64 = make_solves("fp64")
    ms64, stages64 = timed(s64, args.fp64_steps, 1, stage_timing=True)
    fps64 = world * B * args.fp64_steps / (ms64 * 1e-3)

    # accuracy of the batched FP32 path against the FP64 path on batch 0
    outs = gsolvers[0].solve(kwb[0])
    gsolvers[0].stream.synchronize()
    errs = []
    for (ca, fa), b in zip(outs, s64):
        ca, fa = ca[0].cpu().numpy(), fa[0].cpu().numpy()
        cb, fb = b[3].cpu().numpy(), b[4].cpu().numpy()
        errs.append(max(np.linalg.norm(ca - cb) / np.linalg.norm(cb), np.linalg.norm(fa - fb) / np.linalg.norm(fb)))
    rel32 = max(errs)
    # against the exact discrete solution (accurate FP64 mode) on 4 cases: the
    # accuracy bar of the fast path, and the reference rounding's own error
    sr = make_solves("fp64r")[:4]
    run_batch(sr)
    torch.cuda.synchronize()
    e32x, e64x = [], []
    for (ca, fa), b, r in zip(outs, s64, sr):
        ca, fa = ca[0].cpu().numpy(), fa[0].cpu().numpy()
        cb, fb = b[3].cpu().numpy(), b[4].cpu().numpy()
        cr, fr = r[3].cpu().numpy(), r[4].cpu().numpy()
        e32x.append(max(np.linalg.norm(ca - cr) / np.linalg.norm(cr), np.linalg.norm(fa - fr) / np.linalg.norm(fr)))
        e64x.append(max(np.linalg.norm(cb - cr) / np.linalg.norm(cr), np.linalg.norm(fb - fr) / np.linalg.norm(fr)))

    # the checker, outside every timed region: each case of the step against
    # the oracle's double-double shooting (the reference's own algorithm in
    # extended precision); the reference-rounding FP64 results beside it
    from oracle import bldfm_oracle as O
    from oracle import build_oracle

    build_oracle()
    e32e, e64e = [], []
    for (ca, fa), b, kw in zip(outs, s64, kwb[0]):
        _, ce, fe = O.steady_state_transport_solver(**kw, sweep="shooting_dd")
        ca, fa = ca[0].cpu().numpy(), fa[0].cpu().numpy()
        cb, fb = b[3].cpu().numpy(), b[4].cpu().numpy()
        e32e.append(max(np.linalg.norm(ca - ce) / np.linalg.norm(ce), np.linalg.norm(fa - fe) / np.linalg.norm(fe)))
        e64e.append(max(np.linalg.norm(cb - ce) / np.linalg.norm(ce), np.linalg.norm(fb - fe) / np.linalg.norm(fe)))

    # --- learned surrogate: fused features -> tcgen05 MLP -> spectra, trained weights ---
    sur_line = surrogate_section(kwb, inputs, s64, B, args, dev, dist, world, sr)
    if sur_line is not None:
        # the comparison that decides whether the network earns its place:
        # the batched FP32 solver (no network) on the same workload
        sur_line["vs_batched_fp32"] = {
            "surrogate_footprints_per_s": sur_line["value"], "fp32_footprints_per_s": fps_batch,
            "speed_ratio": sur_line["value"] / fps_batch,
            "surrogate_relL2_vs_exact_max": sur_line.get("relL2_vs_exact_max"),
            "fp32_relL2_vs_oracle_ext_max": max(e32e),
            "note": "the network costs ~200 kflop per mode (4 layers of 256) against ~10 kflop per mode for the "
                    "FP32 sweep; on this GPU the solver without the network is the faster and more accurate path",
        }

    # --- the mixed-grid timeseries and the production footprint (rank 0, N = 1) ---
    ts_line = prod_line = serve_line = None
    if rank == 0 and world == 1 and not args.no_extra:
        ts_line = timeseries_section(args, dev)
        prod_line = production_section(args, lib, dev, sptr, not args.no_cpu_baseline)
        serve_line = serving_section(args, dev)

    # --- roofline of the batched FP32 sweep kernel ---
    peak1 = ctypes.c_double(0)
    _lib.check(lib.bldfm_fma_peak(0, ctypes.byref(peak1), sptr), "fma_peak")
    peak2 = ctypes.c_double(0)
    _lib.check(lib.bldfm_fma_peak(2, ctypes.byref(peak2), sptr), "fma_peak")
    peak = ctypes.c_double(max(peak1.value, peak2.value))  # the sweep issues f32x2 FMAs
    peak64 = ctypes.c_double(0)
    _lib.check(lib.bldfm_fma_peak(1, ctypes.byref(peak64), sptr), "fma_peak")
    nsolved = int(s32[0][1].nsolved)
    steps_z = nz - 1
    flops_launch = 0.0
    for d, info, ws, conc, flx, zz, prof, lv in s32:  # the step's cases: same grid, own profiles
        fpm = ctypes.c_double(0)
        _lib.check(lib.bldfm_sweep32_flops(len(zz), _lib.ptr(prof), _lib.ptr(lv), len(lv), ctypes.byref(fpm)),
                   "sweep32_flops")
        flops_launch += fpm.value * int(info.nsolved)
    sweep_ms = stages_b[1] if stages_b and len(stages_b) > 1 else None
    achieved = flops_launch / (sweep_ms * 1e-3) / 1e12 if sweep_ms else None
    flops64 = F64_FLOPS_PER_MODE_STEP * nsolved * steps_z
    sweep64_ms = stages64[1] if stages64 and len(stages64) > 1 else None
    achieved64 = flops64 / (sweep64_ms * 1e-3) / 1e12 if sweep64_ms else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sec = cpu_port_time(kws[0])
        cpu = {
            "value": 1.0 / sec, "unit": "footprints/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "1 footprint of the workload: C port of the reference sweep (OpenMP, all cores) + numpy FFT",
        }

    if rank == 0:
        line = {
            "metric": "footprints/s",
            "value": fps_batch,
            "unit": "footprints/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": msb / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": {
                "workload": WORKLOAD_NAME,
                "footprints_per_step": B,
                "path": "batched fp32 invariant-imbedding sweep + fp32 transforms, CUDA graph, device-resident; "
                        "four solver streams take the steps in turn, so a step's transforms overlap the next "
                        "step's sweep",
                "met_batches": NB,
                "sweep_launch": {"threads": threads, "ctas_per_sm": per_sm, "xform_lines": xlines, "autotuned": True,
                                 "tuned_for": "four solver streams (pipelined)"},
                "l2": "inputs larger than L2: a step's 16 footprints use ~170 MB of spectra and outputs",
                "parallelism": "replicas" if world > 1 else "single",
            },
            "relL2_fp32_vs_oracle_ext": max(e32e),
            "relL2_fp32_vs_oracle_ext_per_case": e32e,
            "relL2_fp64_reference_rounding_vs_oracle_ext_per_case": e64e,
            "oracle_ext": "the reference's shooting sweep and combination (src/bldfm/solver.py:220-235, 307-374) "
                          "in double-double arithmetic on the host (oracle/sweep_port.c), every case of step 0",
            "relL2_fp32_vs_fp64": rel32,
            "relL2_fp32_vs_exact": max(e32x),
            "relL2_fp64_reference_rounding_vs_exact": max(e64x),
            "batched_no_graph": {"value": fps_nograph, "unit": "footprints/s", "stage_ms": stages_b},
            "single_fp32": {"value": fps32, "unit": "footprints/s", "stage_ms": stages32},
            "fp64": {"value": fps64, "unit": "footprints/s", "ms_per_footprint": ms64 / (args.fp64_steps * B),
                     "stage_ms": stages64, "sweep_tflops": achieved64,
                     "fp64_peak_tflops": peak64.value / 1e12,
                     "frac": (achieved64 / (peak64.value / 1e12)) if achieved64 else None},
            "e2e": {"value": e2e_fps, "unit": "footprints/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "api": "bldfm_gb300.batch.solve_stream over the timed steps (numpy in, numpy out, "
                           "pinned copies inside, each step's arrays fresh; its default %d solvers in turn, "
                           "so %d steps in flight); median of three passes of %d steps" % (depth, depth, e2e_steps),
                    "passes": e2e_passes,
                    "solve_batch_synchronous": e2e_sync,
                    "single_case_dropin": e2e_single},
            "roofline": {
                "bound": "fp32-pipe",
                "kernel": "riccati32_batch_kernel",
                "achieved": achieved,
                "peak": peak.value / 1e12,
                "unit": "TFLOP/s",
                "frac": (achieved / (peak.value / 1e12)) if achieved else None,
                "peak_source": "measured FP32 FMA throughput, max of scalar and packed f32x2 "
                               "(bldfm_fma_peak); not in MEASURED_PEAKS.json",
                "peak_scalar_fp32": peak1.value / 1e12,
                "peak_packed_fp32x2": peak2.value / 1e12,
                # DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu
                # capture of this kernel on this workload, 16 footprints per launch
                "traffic": RICC_BATCH_DRAM_BYTES,
                "traffic_source": "ncu capture, profiles/riccati32_batch_kernel_metric_batch16.md",
                "flops_per_launch": flops_launch,
            },
            "transform": transform_section(stages_b, B, dev, xlines),
            "surrogate": sur_line,
            "timeseries": ts_line,
            "production": prod_line,
            "serving": serve_line,
            "cpu_baseline": cpu,
            # per timed step: the sweep, the column and row transform passes
            # and the accuracy check
            "gpu_launches": 4 * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
