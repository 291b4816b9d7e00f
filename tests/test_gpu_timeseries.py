"""The mixed-grid met timeseries in one batched call: 512 footprints over 8
towers (256^2 / 512^2 / 1024^2 grids, 64-256 levels) in one persistent sweep
launch, checked against the exact discrete solution (accurate FP64 mode) on
one case per tower, and for footprint mass on every case."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_timeseries_batch_matches_exact():
    from bldfm_gb300 import steady_state_transport_solver, vertical_profiles
    from bldfm_gb300.batch import BatchSolver, solve_batch
    from tests.timeseries_cases import met_cases

    cases = met_cases(512, seed=0)
    kws = []
    for c in cases:
        z, prof = vertical_profiles(c["n"], c["zm"], c["wind"], ustar=c["ustar"], mol=c["mol"])
        kws.append(dict(srf_flx=np.zeros((c["grid"], c["grid"])), z=z, profiles=prof, domain=c["domain"],
                        levels=c["n"], modes=(c["grid"], c["grid"]), meas_pt=c["meas_pt"], footprint=True,
                        precision="double"))
    res = solve_batch(kws, solver=BatchSolver(use_graph=False))
    assert len(res) == 512
    seen = set()
    for c, kw, (grid, conc, flx) in zip(cases, kws, res):
        assert np.all(np.isfinite(conc)) and np.all(np.isfinite(flx))
        if c["tower"] in seen:
            continue
        seen.add(c["tower"])
        _, cr, fr = steady_state_transport_solver(**kw, mode="fp64r")
        assert _rel(conc, cr) < 1e-4 and _rel(flx, fr) < 1e-4, (c, _rel(conc, cr), _rel(flx, fr))
    assert len(seen) == 8
