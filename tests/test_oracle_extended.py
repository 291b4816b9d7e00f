"""Pin "exact" with the reference's own algorithm in extended precision.

The reference's shooting method (src/bldfm/solver.py:220-235, 307-374) cancels
between two growing IVP states, so its FP64 result carries a rounding error of
order eps * e^{2G} in the high-|k| modes.  The oracle's double-double shooting
(``sweep="shooting_dd"``, oracle/sweep_port.c: oracle_sweep_dd) runs the same
recurrence and combination with about 32 significant digits.  These tests show
on the CPU, independently of every GPU kernel, that

* the extended-precision shooting and the FP64 invariant-imbedding restatement
  (``sweep="riccati"``, the yardstick of the accurate and fast GPU modes)
  converge to the same discrete solution, and
* the reference's FP64 rounding sits a measurable distance away from it on the
  benchmark workload (up to the 1e-3 bar for the lowest friction velocity).
"""

import numpy as np
import pytest

import golden_cases as G
from oracle import bldfm_oracle as O


def _metric_kwargs(ustar, wind_dir=225.0):
    """The benchmark workload: 512^2 footprint on a 1000 m domain (1536^2
    extended), 512^2 modes, n = 128 (207 levels), L = -50 m, 4 m/s wind,
    tower at (500, 500) m."""
    wind = O.compute_wind_fields(4.0, wind_dir)
    z, p = O.vertical_profiles(128, 20.0, wind, ustar=ustar, mol=-50.0)
    return dict(srf_flx=np.zeros((512, 512)), z=z, profiles=p, domain=(1000.0, 1000.0), levels=128,
                modes=(512, 512), meas_pt=(500.0, 500.0), footprint=True, precision="double")


def _three_ways(kw):
    _, cd, fd = O.steady_state_transport_solver(**kw, sweep="shooting_dd")
    _, cr, fr = O.steady_state_transport_solver(**kw, sweep="riccati")
    _, cs, fs = O.steady_state_transport_solver(**kw)
    ext_vs_ricc = max(G.rel_l2(cr, cd), G.rel_l2(fr, fd))
    ref_vs_ext = max(G.rel_l2(cs, cd), G.rel_l2(fs, fd))
    return ext_vs_ricc, ref_vs_ext, (cd, fd), (cs, fs)


def test_extended_shooting_pins_exact_on_metric_fixture():
    """metric_footprint_512 (the reference run itself, tests/golden): the
    oracle's FP64 shooting reproduces it bit for bit (test_oracle_golden), the
    double-double shooting agrees with the Riccati restatement to 1e-8, and
    the reference's FP64 result is 1e-6 ... 1e-3 away from both."""
    d = G.load("metric_footprint_512")
    kw = G.kwargs_of(d)
    kw["precision"] = "double"
    ext_vs_ricc, ref_vs_ext, _, (cs, fs) = _three_ways(kw)
    assert ext_vs_ricc <= 1e-8, ext_vs_ricc
    assert 1e-6 <= ref_vs_ext <= 1e-3, ref_vs_ext


def test_extended_shooting_pins_exact_lowest_ustar():
    """u* = 0.25 m/s, the lowest friction velocity of the benchmark's met
    cases: the reference's FP64 rounding exceeds 1e-4 here, while the two
    accurate evaluations still agree to 1e-8."""
    ext_vs_ricc, ref_vs_ext, _, _ = _three_ways(_metric_kwargs(0.25))
    assert ext_vs_ricc <= 1e-8, ext_vs_ricc
    assert 1e-4 <= ref_vs_ext <= 1e-2, ref_vs_ext


@pytest.mark.parametrize("name", [n for n in G.solver_names() if n not in ("analytic_constant", "metric_footprint_512")])
def test_extended_shooting_agrees_with_riccati_on_fixtures(name):
    """Two independent accurate evaluations of each fixture's discrete
    problem (shooting in double-double, invariant imbedding in FP64) agree
    closely on every golden case, ragged, multi-level and source cases
    included."""
    d = G.load(name)
    kw = G.kwargs_of(d)
    kw["precision"] = "double"
    _, cd, fd = O.steady_state_transport_solver(**kw, sweep="shooting_dd")
    _, cr, fr = O.steady_state_transport_solver(**kw, sweep="riccati")
    assert G.rel_l2(cr, cd) <= 1e-10 and G.rel_l2(fr, fd) <= 1e-10, name


def test_hermitian_split_covers_every_mode():
    for nlx, nly in ((8, 6), (512, 512), (6, 10), (4, 4)):
        rep, src = O.hermitian_split(nlx, nly)
        n = nlx * nly - 1
        assert src.shape == (n,)
        mir = np.nonzero(src >= 0)[0]
        assert len(rep) + len(mir) == n
        assert np.all(np.isin(src[mir], rep))
