"""The register-resident output-transform passes (xform_lines 8, used when
every case of a batch shares a supported line length), the same with the
zoomed column pass (xform_lines 0, the default, for 3 M lines with the band
and kept window of the default halo) against the shared-memory passes (xform_lines 2) and the
CPU oracle, for every supported line length, both transform signs
(footprint: fft2; dispersion: ifft2), several output levels, a phase shift,
different x and y lengths, a band narrower than the window and a window that
does not start at M.

Tolerances (relative L2): register or zoomed vs shared-memory passes 1e-5
(all FP32, different operation order); batched FP32 vs the oracle's
double-double shooting 1e-3 (the fast path's bar)."""

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu

# (ny, nx), domain, modes (nlx, nly), halo -> column length nfy, row length nfx
SHAPES = [
    ((256, 256), (500.0, 500.0), (512, 512), 250.0),     # 512 x 512, no truncation
    ((256, 256), (1000.0, 1000.0), (256, 256), None),    # 768 x 768
    ((512, 512), (1000.0, 1000.0), (1024, 1024), 500.0),  # 1024 x 1024 (the production footprint)
    ((512, 512), (1000.0, 1000.0), (512, 512), None),    # 1536 x 1536 (the benchmark)
    ((512, 512), (1000.0, 1000.0), (512, 512), 1500.0),  # 2048 x 2048
    ((1024, 1024), (2000.0, 2000.0), (1024, 1024), None),  # 3072 x 3072
    ((256, 512), (1000.0, 1000.0), (512, 256), None),    # rows 1536, columns 768
    ((512, 512), (1000.0, 1000.0), (256, 256), None),    # 1536, band of 257 in a zoom of 512
    ((510, 510), (1000.0, 1000.0), (510, 510), 513.5 * 1000.0 / 510),  # 1536, kept window [513, 1023)
]


def _kw(shape, domain, modes, halo, footprint, seed):
    from oracle import bldfm_oracle as O

    rng = np.random.default_rng(seed)
    wind = O.compute_wind_fields(4.0, float(rng.uniform(0, 360)))
    z, p = O.vertical_profiles(24, 10.0, wind, ustar=float(rng.uniform(0.25, 0.4)), mol=-40.0)
    src = np.zeros(shape)
    if not footprint:
        src = rng.random(shape)
    levels = 24 if footprint else [3, 12, 24]
    meas = (0.37 * domain[0], 0.61 * domain[1])
    return dict(srf_flx=src, z=z, profiles=p, domain=domain, levels=levels, modes=modes, meas_pt=meas,
                footprint=footprint, precision="double", halo=halo)


@pytest.mark.parametrize("footprint", [True, False])
@pytest.mark.parametrize("shape,domain,modes,halo", SHAPES)
def test_register_passes_match_shared_memory_passes_and_oracle(shape, domain, modes, halo, footprint):
    from bldfm_gb300.batch import BatchSolver, solve_batch
    from oracle import bldfm_oracle as O

    kws = [_kw(shape, domain, modes, halo, footprint, seed) for seed in (1, 2)]
    zm = solve_batch(kws, solver=BatchSolver(use_graph=False, xform_lines=0))
    rx = solve_batch(kws, solver=BatchSolver(use_graph=False, xform_lines=8))
    sm = solve_batch(kws, solver=BatchSolver(use_graph=False, xform_lines=2))
    for variant in (rx, zm):
        for a, b in zip(variant, sm):
            assert a[1].shape == b[1].shape
            assert G.rel_l2(a[1], b[1]) <= 1e-5 and G.rel_l2(a[2], b[2]) <= 1e-5, (G.rel_l2(a[1], b[1]),
                                                                                G.rel_l2(a[2], b[2]))
    _, oc, of = O.steady_state_transport_solver(**kws[0], sweep="shooting_dd")
    for name, variant in (("rx", rx), ("zoom", zm)):
        err = max(G.rel_l2(variant[0][1], oc), G.rel_l2(variant[0][2], of))
        print(shape, modes, halo, footprint, "%s vs double-double %.2e" % (name, err))
        assert err <= 1e-3, err


def test_mixed_line_lengths_one_launch_per_group():
    """A batch whose cases have different column and row line lengths runs the
    register-resident passes as one launch per group of cases sharing their
    configs (here a zoomed 768 group, a zoomed 1536 group, an unzoomed 1024
    group and a 1536 x 768 group, interleaved in the batch) and matches the
    shared-memory passes, which take the whole batch in one launch."""
    from bldfm_gb300.batch import BatchSolver, solve_batch

    shapes = [SHAPES[1], SHAPES[3], SHAPES[2], SHAPES[6], SHAPES[1], SHAPES[3]]
    kws = [_kw(*s, footprint=bool(i % 2), seed=10 + i) for i, s in enumerate(shapes)]
    grouped = solve_batch(kws, solver=BatchSolver(use_graph=False, xform_lines=0))
    shared = solve_batch(kws, solver=BatchSolver(use_graph=False, xform_lines=2))
    for a, b in zip(grouped, shared):
        assert a[1].shape == b[1].shape
        assert G.rel_l2(a[1], b[1]) <= 1e-5 and G.rel_l2(a[2], b[2]) <= 1e-5, (G.rel_l2(a[1], b[1]),
                                                                            G.rel_l2(a[2], b[2]))
