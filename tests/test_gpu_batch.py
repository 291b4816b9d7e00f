"""Batched FP32 solves (bldfm_solve_batch) against single solves and the oracle.

A batch mixes footprint and dispersion cases, different grids, level counts,
multi-level outputs and non-isotropic (MOSTM) profiles; every case must match
the single-case FP32 path (same arithmetic) and the reference arithmetic of
the oracle within the FP32 bar (relative L2 1e-3).
"""

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-3
SAME_KERNELS_TOL = 1e-6


def _cases(seed):
    from oracle import bldfm_oracle as O

    rng = np.random.default_rng(seed)
    out = []
    # footprint, 96 x 128, one level
    z, p = O.vertical_profiles(20, 10.0, (float(rng.uniform(1, 4)), -2.0), ustar=float(rng.uniform(0.2, 0.5)),
                               mol=-60.0)
    out.append(dict(srf_flx=np.zeros((96, 128)), z=z, profiles=p, domain=(200.0, 150.0), levels=20,
                    modes=(128, 96), meas_pt=(80.0, 70.0), footprint=True, precision="double"))
    # dispersion with shift, 64 x 64, several levels incl. a duplicate
    z, p = O.vertical_profiles(12, 6.0, (3.0, 1.0), z0=0.05, mol=1e9)
    out.append(dict(srf_flx=O.ideal_source((64, 64), (300.0, 300.0), shape="circle"), z=z, profiles=p,
                    domain=(300.0, 300.0), levels=[0, 6, 6, 12], modes=(64, 64), meas_pt=(100.0, 120.0),
                    footprint=False, precision="double", srf_bg_conc=0.5))
    # MOSTM (Kx != Ky): generic coefficient path, footprint, 80 x 48
    z, p = O.vertical_profiles(16, 8.0, (2.0, 2.5), ustar=0.3, mol=-30.0, closure="MOSTM")
    out.append(dict(srf_flx=np.zeros((48, 80)), z=z, profiles=p, domain=(160.0, 96.0), levels=16, modes=(80, 48),
                    meas_pt=(50.0, 40.0), footprint=True, precision="single"))
    # stable, deeper grid, footprint 128 x 128
    z, p = O.vertical_profiles(40, 15.0, (-3.0, -3.0), ustar=0.4, mol=120.0)
    out.append(dict(srf_flx=np.zeros((128, 128)), z=z, profiles=p, domain=(400.0, 400.0), levels=40,
                    modes=(128, 128), meas_pt=(200.0, 200.0), footprint=True, precision="double"))
    return out


def _single(kw):
    """The single-solve FP32 entry point (bldfm_solve_host: riccati32_kernel
    and the single-solve transforms), not the drop-in, which runs FP32 calls
    through the batched path."""
    from bldfm_gb300 import _lib
    from bldfm_gb300.solver import _normalise_levels, make_desc, output_grid

    lib = _lib.load()
    z = np.ascontiguousarray(kw["z"], dtype=np.float64)
    nz = len(z)
    prof = np.ascontiguousarray(np.stack([np.broadcast_to(np.asarray(a, dtype=np.float64), (nz,))
                                          for a in kw["profiles"]]))
    levels, lv = _normalise_levels(kw["levels"], nz)
    shape = np.shape(kw["srf_flx"])
    d = make_desc(shape, nz, kw["domain"], kw["modes"], kw["meas_pt"], kw.get("srf_bg_conc", 0.0),
                  kw["footprint"], False, kw.get("halo"), kw["precision"], "fp32")
    info = _lib.PlanInfo()
    _lib.check(lib.bldfm_plan(d, int(lv.size), info))
    conc = np.empty((lv.size, info.out_ny, info.out_nx))
    flx = np.empty_like(conc)
    src = None if kw["footprint"] else np.ascontiguousarray(kw["srf_flx"], dtype=np.float64)
    _lib.check(lib.bldfm_solve_host(d, _lib.ptr(src), _lib.ptr(z), _lib.ptr(prof), _lib.ptr(lv), int(lv.size),
                                    _lib.ptr(conc), _lib.ptr(flx)))
    xm, ym = kw["meas_pt"]
    if kw["precision"] == "single" and not kw["footprint"] and not (xm**2 + ym**2 > 0.0):
        conc, flx = conc.astype(np.float32), flx.astype(np.float32)
    return output_grid(z, levels, shape, kw["domain"]), np.squeeze(conc), np.squeeze(flx)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_single_and_oracle(use_graph):
    from bldfm_gb300.batch import BatchSolver, solve_batch
    from oracle import bldfm_oracle as O

    solver = BatchSolver(use_graph=use_graph)
    for seed in (1, 2):  # two batches of the same topology: the second replays the graph
        cases = _cases(seed)
        res = solve_batch(cases, solver=solver)
        for kw, (grid, conc, flx) in zip(cases, res):
            _, sc, sf = _single(kw)
            _, oc, of = O.steady_state_transport_solver(**kw)
            assert conc.shape == sc.shape and conc.dtype == sc.dtype
            assert G.rel_l2(conc, sc) <= SAME_KERNELS_TOL and G.rel_l2(flx, sf) <= SAME_KERNELS_TOL
            assert G.rel_l2(conc, oc) <= FP32_TOL and G.rel_l2(flx, of) <= FP32_TOL
        assert solver.status() == 0


def test_batch_of_golden_footprints():
    """Every footprint fixture solved in one batch, against the stored reference."""
    from bldfm_gb300.batch import solve_batch

    names = [n for n in G.solver_names() if bool(G.load(n)["footprint"])]
    cases = [G.kwargs_of(G.load(n)) for n in names]
    res = solve_batch(cases)
    for n, kw, (_, conc, flx) in zip(names, cases, res):
        d = G.load(n)
        rc, rf = G.reference_fields(d)
        assert G.rel_l2(G.sample(d, conc), rc) <= FP32_TOL, n
        assert G.rel_l2(G.sample(d, flx), rf) <= FP32_TOL, n


def test_autotuner_returns_a_candidate(tmp_path, monkeypatch):
    from bldfm_gb300 import autotune

    monkeypatch.setenv("BLDFM_GB300_CACHE", str(tmp_path / "tune.json"))
    cases = _cases(3)
    t, per_sm, xl = autotune.tune(cases, reps=1)
    assert (t, per_sm) in autotune.CANDIDATES and xl in autotune.XFORM_LINES
    assert (tmp_path / "tune.json").exists()
    assert autotune.tune(cases) == (t, per_sm, xl)  # cached


@pytest.mark.parametrize("xl", [1, 2, 4])
def test_transform_lines_per_cta_agree(xl):
    """Every lines-per-CTA choice of the transform passes gives the same result."""
    from bldfm_gb300.batch import BatchSolver

    cases = _cases(4)
    r = BatchSolver(use_graph=False)
    outs = r.solve(cases)
    r.stream.synchronize()
    ref = [(c.cpu().numpy(), f.cpu().numpy()) for c, f in outs]
    s = BatchSolver(use_graph=False, xform_lines=xl)
    out = s.solve(cases)
    s.stream.synchronize()
    assert s.status() == 0
    for (c, f), (rc, rf) in zip(out, ref):
        np.testing.assert_array_equal(c.cpu().numpy(), rc)
        np.testing.assert_array_equal(f.cpu().numpy(), rf)


def test_solve_stream_matches_solve_batch():
    """The pipelined timeseries API yields, batch by batch, what solve_batch returns."""
    from bldfm_gb300.batch import solve_batch, solve_stream

    batches = [_cases(5), _cases(6), _cases(7)]
    ref = [solve_batch(b) for b in batches]
    got = list(solve_stream(batches))
    assert len(got) == 3
    for rb, gb in zip(ref, got):
        for (rg, rc, rf), (gg, gc, gf) in zip(rb, gb):
            np.testing.assert_array_equal(rc, gc)
            np.testing.assert_array_equal(rf, gf)
            assert rc.dtype == gc.dtype
