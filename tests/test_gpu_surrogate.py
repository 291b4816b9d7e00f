"""The learned surrogate on the GPU: its training data against the FP64 CPU
oracle, its serving path against the solver, and what training gains."""

import math
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_transfer_samples_match_oracle():
    """FP32 device sweep of the nondimensional transfer vs the FP64 oracle."""
    from bldfm_gb300.surrogate import TransferPool
    from oracle.transfer_oracle import transfer

    s1 = np.array([-1.5, -0.4, 0.0, 0.8])
    s2 = np.array([2.5, 6.0, 4.6, 7.5])
    pool = TransferPool(s1=s1, s2=s2)
    rng = np.random.default_rng(0)
    m = 512
    cid = rng.integers(0, 4, m).astype(np.int32)
    k = np.exp(rng.uniform(np.log(1e-3), np.log(40.0), m))
    th = rng.uniform(0, np.pi / 2, m)
    kpar, kperp = (k * np.cos(th)).astype(np.float32), (k * np.sin(th)).astype(np.float32)
    dev = pool.device
    T = pool.eval(*(torch.from_numpy(a).to(dev) for a in (cid, kpar, kperp))).cpu().numpy()
    for c in range(4):
        sel = cid == c
        _, _, ref = transfer(s1[c], s2[c], 128, kpar[sel].astype(np.float64), kperp[sel].astype(np.float64))
        err = np.abs(T[sel] - ref)
        assert err.max() < 2e-4, (c, err.max(axis=0))


def test_sample_weights_and_features():
    from bldfm_gb300.surrogate import TransferPool

    pool = TransferPool(ncases=64, seed=3)
    norm = pool.energies(per_case=256)
    assert torch.isfinite(norm).all() and (norm > 0).all()
    X, T, W = pool.buffers(4096)
    pool.samples(7, 4096, X, T, W, norm=norm)
    for a in (X, T, W):
        assert torch.isfinite(a).all()
    assert (W > 0).all()
    # the same seed gives the same samples
    X2, T2, W2 = pool.buffers(4096)
    pool.samples(7, 4096, X2, T2, W2, norm=norm)
    assert torch.equal(X, X2) and torch.equal(T, T2)


@pytest.mark.parametrize("wdir,mol", [(225.0, -50.0), (270.0, 1e9), (40.0, 80.0)])
def test_exact_transfer_serving_matches_solver(wdir, mol):
    """The serving path with the exact nondimensional transfer in place of the
    network reproduces the solver's footprint (checks features, rotation,
    conjugation, phase shift, k = 0 values and the output transform)."""
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import Surrogate

    th = np.deg2rad(wdir)
    wind = (-4.0 * np.sin(th), -4.0 * np.cos(th))
    sur = Surrogate(variant=1, spot_every=0)
    args = dict(n=32, zm=20.0, wind=wind, srf_shape=(128, 128), domain=(1000.0, 1000.0), modes=(128, 128),
                meas_pt=(500.0, 500.0), ustar=0.3, mol=mol)
    (grid, conc, flx), path = sur.footprint(**args)
    assert path == "surrogate"
    p = sur.prepare(**args)
    _, c64, f64 = steady_state_transport_solver(**p["kw"], mode="fp64r")
    assert conc.shape == c64.shape
    assert _rel(flx, f64) < 2e-5
    assert _rel(conc, c64) < 2e-5
    assert abs(flx.sum() - f64.sum()) / abs(f64.sum()) < 1e-5


def test_single_footprint_states_its_error():
    """Surrogate.footprint with the fused kernel runs as a batch of one: the
    same footprint as serve(), with the guard's estimate as its error
    statement (here within a factor of 3 of the true error)."""
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import Surrogate, load

    net, box, meta = load()
    kw = dict(n=128, zm=20.0, wind=(2.83, 2.83), srf_shape=(256, 256), domain=(500.0, 500.0), modes=(256, 256),
              meas_pt=(250.0, 250.0), ustar=0.3, mol=-50.0)
    sur = Surrogate(net, spot_every=0, tol=1e-3)
    (grid, conc, flx), path, stated = sur.footprint(**kw, return_error=True)
    assert path == "surrogate" and stated is not None
    out, paths = Surrogate(net, spot_every=0, tol=1e-3).serve([kw])
    assert paths == ["surrogate"]
    assert _rel(conc, out[0][0].cpu().numpy()) < 1e-12 and _rel(flx, out[0][1].cpu().numpy()) < 1e-12
    p = sur.prepare(**kw)
    _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
    true = max(_rel(conc, cr), _rel(flx, fr))
    print("stated %.2e true %.2e" % (stated, true))
    assert true / 3 <= stated <= 3 * true


def test_fused_serving_matches_layerwise():
    """The fused features -> MLP -> spectra kernel computes what the
    layer-by-layer tensor-core MLP and the spectra kernel compute."""
    from bldfm_gb300.mlp import MLP
    from bldfm_gb300.surrogate import Surrogate

    net = MLP(batch=16384, seed=11)
    p = net.params()
    p *= 0.5  # keep the untrained outputs moderate
    net.set_params(p)
    args = dict(n=128, zm=20.0, wind=(2.83, 2.83), srf_shape=(256, 256), domain=(1000.0, 1000.0),
                modes=(256, 256), meas_pt=(500.0, 500.0), ustar=0.3, mol=-50.0)
    outs = []
    for variant in (0, 2):
        sur = Surrogate(net, variant=variant, spot_every=0)
        c, f = sur.solve_prepared(sur.prepare(**args))
        outs.append((c.cpu().numpy(), f.cpu().numpy()))
    assert np.all(np.isfinite(outs[0][0])) and np.all(np.isfinite(outs[0][1]))
    # the fused kernel's input layer runs as split BF16 MMAs (relative 2^-16),
    # which can flip the BF16 rounding of a few activations
    assert _rel(outs[0][0], outs[1][0]) < 1e-4
    assert _rel(outs[0][1], outs[1][1]) < 1e-4


def test_batched_serving_matches_single():
    """One fused launch over several footprints (mixed grids, directions and
    met cases) gives the single-footprint results."""
    from bldfm_gb300.surrogate import Surrogate, load

    net, box, meta = load()
    sur = Surrogate(net, spot_every=0)
    items = [
        dict(n=128, zm=20.0, wind=(2.83, 2.83), srf_shape=(256, 256), domain=(1000.0, 1000.0), modes=(256, 256),
             meas_pt=(500.0, 500.0), ustar=0.3, mol=-50.0),
        dict(n=128, zm=12.0, wind=(-3.0, 1.0), srf_shape=(128, 192), domain=(600.0, 900.0), modes=(128, 192),
             meas_pt=(300.0, 200.0), ustar=0.35, mol=-40.0),
        dict(n=128, zm=30.0, wind=(0.5, -4.0), srf_shape=(256, 256), domain=(1500.0, 1500.0), modes=(128, 128),
             meas_pt=(700.0, 800.0), ustar=0.4, mol=-200.0),
    ]
    b = sur.prepare_batch(items)
    outs = [(c.cpu().numpy(), f.cpu().numpy()) for c, f in sur.solve_batch_prepared(b)]
    assert sur.status() == 0
    for kw, (cb, fb) in zip(items, outs):
        cs, fs = sur.solve_prepared(sur.prepare(**kw))
        cs, fs = cs.cpu().numpy(), fs.cpu().numpy()
        assert _rel(cb, cs) < 1e-6 and _rel(fb, fs) < 1e-6


def test_exact_low_band():
    """The footprint's lowest wavenumbers through the exact FP32 sweep in
    place of the network: with the band over every mode (exact_kz huge,
    mirror pairs and the unpaired Nyquist modes) the served footprint is the
    FP32 solver's, in the single and the batched path, on square and
    non-square grids; with the default band
    (|k| z_m < 4) the trained network's error against the exact solution drops
    at least threefold against the network alone."""
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import Surrogate, load

    net, box, meta = load()
    items = [dict(n=128, zm=20.0, wind=(2.83, 2.83), srf_shape=(256, 256), domain=(500.0, 500.0), modes=(256, 256),
                  meas_pt=(250.0, 250.0), ustar=0.3, mol=-50.0),
             dict(n=128, zm=15.0, wind=(-3.0, 2.0), srf_shape=(256, 256), domain=(500.0, 500.0), modes=(256, 256),
                  meas_pt=(200.0, 300.0), ustar=0.33, mol=-80.0),
             dict(n=128, zm=12.0, wind=(-3.0, 1.0), srf_shape=(128, 192), domain=(600.0, 900.0), modes=(128, 192),
                  meas_pt=(300.0, 200.0), ustar=0.35, mol=-40.0)]
    full = Surrogate(net, spot_every=0, exact_kz=1e9)
    bouts = [(c.cpu().numpy(), f.cpu().numpy()) for c, f in full.solve_batch_prepared(full.prepare_batch(items))]
    assert full.status() == 0
    for kw, (cb, fb) in zip(items, bouts):
        p = full.prepare(**kw)
        c, f = full.solve_prepared(p)
        c, f = c.cpu().numpy(), f.cpu().numpy()
        _, c32, f32 = steady_state_transport_solver(**p["kw"], mode="fp32")
        assert _rel(c, c32) < 1e-5 and _rel(f, f32) < 1e-5, (_rel(c, c32), _rel(f, f32))
        assert _rel(cb, c) < 1e-6 and _rel(fb, f) < 1e-6
    errs = {}
    for kz in (0.0, None):
        sur = Surrogate(net, spot_every=0, exact_kz=kz)
        e = []
        for kw in items:
            p = sur.prepare(**kw)
            c, f = sur.solve_prepared(p)
            _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
            e.append(max(_rel(c.cpu().numpy(), cr), _rel(f.cpu().numpy(), fr)))
        errs[kz] = np.array(e)
    print("network alone", errs[0.0], "with the exact band", errs[None])
    assert np.all(errs[None] <= errs[0.0] / 3), errs


def test_trained_network_gains_over_solver():
    """What the trained network buys: inside its training box it reproduces
    the FP64 footprint to relL2 <= 1e-3 at a fraction of the FP64 solver's
    cost, where the untrained network of the same shape is useless."""
    import time

    from bldfm_gb300.mlp import MLP
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import Surrogate, load

    net, box, meta = load()
    kw = dict(n=128, zm=20.0, wind=(2.83, 2.83), srf_shape=(512, 512), domain=(1000.0, 1000.0), modes=(512, 512),
              meas_pt=(500.0, 500.0), ustar=0.3, mol=-50.0)
    sur = Surrogate(net, spot_every=0)
    p = sur.prepare(**kw)
    c, f = sur.solve_prepared(p)
    c, f = c.cpu().numpy(), f.cpu().numpy()
    _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
    err = max(_rel(c, cr), _rel(f, fr))
    assert err <= 1e-3, err
    raw = Surrogate(MLP(batch=65536, seed=0), spot_every=0)
    cu, fu = raw.solve_prepared(raw.prepare(**kw))
    err_untrained = max(_rel(cu.cpu().numpy(), cr), _rel(fu.cpu().numpy(), fr))
    assert err_untrained > 100 * err
    # speed: surrogate vs the FP64 solver on the device, same footprint
    from bldfm_gb300 import _lib
    from bldfm_gb300.solver import make_desc, plan
    import ctypes

    lib = _lib.load()
    d = make_desc((512, 512), p["z"].size, (1000.0, 1000.0), (512, 512), (500.0, 500.0), 0.0, True, False, None,
                  "double", "fp64")
    info = plan(d, 1)
    ws = torch.empty(int(info.workspace_bytes), dtype=torch.uint8, device="cuda")
    co = torch.empty((512, 512), dtype=torch.float64, device="cuda")
    fo = torch.empty_like(co)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def fp64_solve():
        _lib.check(lib.bldfm_solve(d, None, _lib.ptr(p["z"]), _lib.ptr(p["prof"]), _lib.ptr(p["lv"]), 1,
                                   ctypes.c_void_p(co.data_ptr()), ctypes.c_void_p(fo.data_ptr()),
                                   ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()), st), "fp64")

    def timeit(fn, reps):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps

    t64 = timeit(fp64_solve, 5)
    b = sur.prepare_batch([kw] * 16)
    tsur = timeit(lambda: sur.solve_batch_prepared(b), 5) / 16
    assert t64 / tsur > 10, (t64, tsur)
    # against the method without the network: the batched FP32 solver on the
    # same 16 footprints.  On this GPU the FP32 solver is the faster and the
    # more accurate of the two (its sweep costs ~10 kflop per mode against
    # ~200 kflop per mode for the network), which the numbers below state.
    from bldfm_gb300.batch import BatchSolver

    s32 = BatchSolver(use_graph=True)
    prep = s32.prepare_cached([dict(p["kw"], precision="double")] * 16)
    t32 = timeit(lambda: s32.solve_prepared(prep), 5) / 16
    c32, f32 = (t[0].cpu().numpy() for t in prep[1][0])
    err32 = max(_rel(c32, cr), _rel(f32, fr))
    print("per footprint: surrogate %.1f us (relL2 %.1e), batched FP32 %.1f us (relL2 %.1e), FP64 %.0f us"
          % (tsur * 1e6, err, t32 * 1e6, err32, t64 * 1e6))
    assert err32 <= 1e-5


def test_serve_timeseries_with_fallback():
    """A short footprint timeseries: in-box steps through the network (with
    spot checks), out-of-box steps through the FP64 fallback."""
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import Surrogate, load

    net, box, meta = load()
    rng = np.random.default_rng(2)
    items = []
    for k in range(18):
        th = rng.uniform(0, 2 * np.pi)
        mol = -150.0 if k % 9 else -12.0  # z_m / L = -1.7: outside the box
        items.append(dict(n=128, zm=20.0, wind=(-4 * np.sin(th), -4 * np.cos(th)), srf_shape=(256, 256),
                          domain=(500.0, 500.0), modes=(256, 256), meas_pt=(250.0, 250.0),
                          ustar=float(rng.uniform(0.25, 0.35)), mol=mol))
    sur = Surrogate(net, spot_every=8, tol=1e-3)
    out, paths = sur.serve(items, batch=8)
    assert paths.count("fp64-box") == 2 and sur.stats["out_of_box"] == 2
    # every 8th footprint the network serves (the guard passed it) is spot-checked
    passed = paths.count("surrogate") + paths.count("fp64-spot")
    assert sur.stats["spot"] == passed // 8
    assert len(sur.stats["guard"]) == 16
    assert all(p in ("surrogate", "fp32-guard", "fp64-spot") for k, p in enumerate(paths) if k % 9)
    for k in (1, 9):
        p = sur.prepare(**items[k])
        _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
        c, f = out[k]
        c = c.cpu().numpy() if hasattr(c, "cpu") else c
        f = f.cpu().numpy() if hasattr(f, "cpu") else f
        tol = 2e-3 if k == 1 else 1e-12  # the fallback is the accurate FP64 solve itself
        assert _rel(c, cr) <= tol and _rel(f, fr) <= tol, (k, _rel(c, cr), _rel(f, fr))
    # fallback="fp64": the out-of-box step returns the reference-rounding solve
    ref = Surrogate(net, spot_every=0, tol=1e-3, fallback="fp64")
    out2, paths2 = ref.serve(items[9:10])
    assert paths2 == ["fp64-box"]
    _, cr, fr = steady_state_transport_solver(**sur.prepare(**items[9])["kw"], mode="fp64")
    c, f = (np.asarray(a.cpu().numpy() if hasattr(a, "cpu") else a) for a in out2[0])
    assert _rel(c, cr) <= 1e-12 and _rel(f, fr) <= 1e-12


def test_guard_estimates_and_guarded_serving():
    """The accuracy guard (a stratified sample of modes re-solved exactly on
    the device) estimates each served case's relative L2 error: on 20 in-box
    footprints of the benchmark's met distribution the estimate stays within
    a factor of 3 of the true error against the exact discrete solution, and
    with the guard on no served footprint exceeds the 1e-3 bar."""
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import Surrogate, load

    net, box, meta = load()
    rng = np.random.default_rng(11)
    items = []
    while len(items) < 20:
        th = rng.uniform(0, 2 * np.pi)
        kw = dict(n=128, zm=20.0, wind=(-4 * np.sin(th), -4 * np.cos(th)), srf_shape=(512, 512),
                  domain=(1000.0, 1000.0), modes=(512, 512), meas_pt=(500.0, 500.0),
                  ustar=float(rng.uniform(0.22, 0.38)), mol=float(1.0 / rng.uniform(-0.045, 0.01)))
        if Surrogate(net).classify(kw):
            items.append(kw)
    sur = Surrogate(net, spot_every=0, guard_tol=1.0)  # estimates only: nothing re-solved
    b = sur.prepare_batch(items)
    outs = [(c.cpu().numpy(), f.cpu().numpy()) for c, f in sur.solve_batch_prepared(b)]
    est = sur.guard_estimates(b)
    errs = []
    for kw, (c, f) in zip(items, outs):
        p = sur.prepare(**kw)
        _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
        errs.append(max(_rel(c, cr), _rel(f, fr)))
    errs = np.array(errs)
    print("guard estimate / true error:", " ".join("%.1e/%.1e" % (a, e) for a, e in zip(est, errs)))
    assert np.all(est >= errs / 3) and np.all(est <= errs * 3), (est, errs)
    # the estimate errs on the safe side for this network (measured with the
    # exact low band: 0.9 to 2.0 times the true error of 0.8e-4 to 1.2e-4;
    # its guard factor is 1)
    assert np.all(est >= 0.85 * errs), (est, errs)
    # guarded serving: cases above the guard's tolerance are re-solved exactly
    sur = Surrogate(net, spot_every=0, tol=1e-3)
    out, paths = sur.serve(items, batch=16)
    for kw, (c, f), path in zip(items, out, paths):
        c = c.cpu().numpy() if hasattr(c, "cpu") else c
        f = f.cpu().numpy() if hasattr(f, "cpu") else f
        p = sur.prepare(**kw)
        _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
        assert max(_rel(c, cr), _rel(f, fr)) <= 1e-3, (path, max(_rel(c, cr), _rel(f, fr)))
    print("guarded serving paths:", {q: paths.count(q) for q in set(paths)})


def test_production_network_serves_the_production_footprint():
    """The n = 256 network (|k| z_m <= 48) on the production footprint's
    neighbourhood: 512^2 grid on 1000 m, 500 m halo (1024^2 extended, all
    modes), 413 levels, z_m = 20 m.  Every guarded served footprint is within
    1e-3 of the exact discrete solution; out-of-box steps go to the accurate
    FP64 solver; outputs outside ``keep`` are dropped."""
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import WEIGHTS_N256, Surrogate, load

    if not os.path.exists(WEIGHTS_N256):
        pytest.skip("no n = 256 weights")
    net, box, meta = load(WEIGHTS_N256)
    assert box["n"] == 256 and box["kmax"] >= 45.5
    rng = np.random.default_rng(5)
    sur = Surrogate(net, box=box, spot_every=0, tol=1e-3)
    items = []
    while len(items) < 10:
        th = rng.uniform(0, 2 * np.pi)
        outside = len(items) == 9  # the last one outside the box (strongly unstable)
        inv_l = float(rng.uniform(-0.1, -0.06) if outside else rng.uniform(-0.045, 0.01))
        kw = dict(n=256, zm=20.0, wind=(-4 * np.sin(th), -4 * np.cos(th)), srf_shape=(512, 512),
                  domain=(1000.0, 1000.0), modes=(1024, 1024), meas_pt=(500.0, 500.0), halo=500.0,
                  ustar=float(rng.uniform(0.22, 0.38)), mol=1.0 / inv_l)
        if sur.classify(kw) != outside:
            items.append(kw)
    keep = [0, 3, 7, 9]
    out, paths, errs = sur.serve(items, batch=8, keep=keep, return_errors=True)
    # every step states its error: the guard's estimate (served), the FP32
    # path's statement (guard re-solve), None for the FP64 fallback
    assert errs[9] is None
    assert all(e is not None and 0 < e < 1e-3 for e in errs[:9]), errs
    assert paths[9] == "fp64-box" and all(p in ("surrogate", "fp32-guard") for p in paths[:9]), paths
    assert all((out[k] is None) == (k not in keep) for k in range(10))
    for k in keep:
        p = sur.prepare(**items[k])
        _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
        c, f = out[k]
        c = c.cpu().numpy() if hasattr(c, "cpu") else c
        f = f.cpu().numpy() if hasattr(f, "cpu") else f
        err = max(_rel(c, cr), _rel(f, fr))
        print("step %d path %s relL2 %.2e" % (k, paths[k], err))
        # the out-of-box step is the accurate FP64 solve itself
        assert err <= (1e-3 if k != 9 else 1e-12), (k, paths[k], err)
    print("guard estimates:", " ".join("%.1e" % e for e in sur.stats["guard"]))


def test_production_guard_calibration():
    """The accuracy guard on the n = 256 network's production footprints
    (1024^2 extended, 413 levels): estimate against the true error of 20
    in-box cases, and guarded serving at the network's guard tolerance keeps
    every served footprint within 1e-3 of the exact discrete solution."""
    from bldfm_gb300.solver import steady_state_transport_solver
    from bldfm_gb300.surrogate import WEIGHTS_N256, Surrogate, load

    if not os.path.exists(WEIGHTS_N256):
        pytest.skip("no n = 256 weights")
    net, box, meta = load(WEIGHTS_N256)
    rng = np.random.default_rng(17)
    probe = Surrogate(net, box=box)
    items = []
    while len(items) < 20:
        th = rng.uniform(0, 2 * np.pi)
        kw = dict(n=256, zm=20.0, wind=(-4 * np.sin(th), -4 * np.cos(th)), srf_shape=(512, 512),
                  domain=(1000.0, 1000.0), modes=(1024, 1024), meas_pt=(500.0, 500.0), halo=500.0,
                  ustar=float(rng.uniform(0.22, 0.38)), mol=float(1.0 / rng.uniform(-0.045, 0.01)))
        if probe.classify(kw):
            items.append(kw)
    sur = Surrogate(net, box=box, spot_every=0, guard_tol=1.0)  # estimates only
    b = sur.prepare_batch(items)
    outs = [(c.cpu().numpy(), f.cpu().numpy()) for c, f in sur.solve_batch_prepared(b)]
    est = sur.guard_estimates(b)
    errs = []
    for kw, (c, f) in zip(items, outs):
        p = sur.prepare(**kw)
        _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
        errs.append(max(_rel(c, cr), _rel(f, fr)))
    errs = np.array(errs)
    print("n256 guard estimate / true error:", " ".join("%.1e/%.1e" % (a, e) for a, e in zip(est, errs)))
    print("ratio min %.2f median %.2f" % ((est / errs).min(), np.median(est / errs)))
    sur = Surrogate(net, box=box, spot_every=0, tol=1e-3)
    out, paths = sur.serve(items, batch=10)
    worst = 0.0
    for kw, (c, f), path in zip(items, out, paths):
        c = c.cpu().numpy() if hasattr(c, "cpu") else c
        f = f.cpu().numpy() if hasattr(f, "cpu") else f
        p = sur.prepare(**kw)
        _, cr, fr = steady_state_transport_solver(**p["kw"], mode="fp64r")
        worst = max(worst, max(_rel(c, cr), _rel(f, fr)))
    print("guarded serving paths:", {q: paths.count(q) for q in set(paths)}, "worst %.2e" % worst)
    assert worst <= 1e-3, worst
