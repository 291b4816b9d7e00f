"""GPU parity: the CUDA solve against the reference's outputs (golden fixtures
generated by the reference) and against the CPU oracle at full size.

Tolerances (relative L2 over the output fields):
  FP64 sweep (mode="fp64"):         1e-10  (the FP64 path's bar)
  float32 outputs (reference FFT in complex64): 2e-6
  FP32 Riccati sweep (mode="fp32"): 1e-3   (the fast path's bar)

The reference's FP64 output depends on the host's libm (csqrt for the top
eigenvalues, pow for the per-level scalars): its shooting combination
amplifies a one-ulp difference by up to exp(2 G).  The fixtures were made on
x86-64; on another ISA the reference itself lands up to relL2 ~3e-6 away from
them on the 512^2 workload.  So each FP64 case checks (a) 1e-10 against the
oracle evaluated on this host (the oracle is bit-identical to the reference on
x86-64, tests/test_oracle_golden.py) and (b) that the GPU result is no further
from the stored reference output than the oracle on this host is, plus 1e-10.
"""

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
F32_OUT_TOL = 2e-6
FP32_TOL = 1e-3


def _gpu_solve(kw, mode="fp64"):
    from bldfm_gb300 import steady_state_transport_solver

    return steady_state_transport_solver(**kw, mode=mode)


@pytest.mark.parametrize("name", G.solver_names())
def test_fp64_matches_reference(name):
    from oracle import bldfm_oracle as O

    d = G.load(name)
    kw = G.kwargs_of(d)
    grid, conc, flx = _gpu_solve(kw)
    _, oc, of = O.steady_state_transport_solver(**kw)
    assert conc.shape == oc.shape and flx.shape == of.shape
    assert str(conc.dtype) == str(d["conc_dtype"]) and str(flx.dtype) == str(d["conc_dtype"])
    tol = F32_OUT_TOL if str(d["conc_dtype"]) == "float32" else FP64_TOL
    ec, ef = G.rel_l2(conc, oc), G.rel_l2(flx, of)
    rc, rf = G.reference_fields(d)
    gc, gf = G.rel_l2(G.sample(d, conc), rc), G.rel_l2(G.sample(d, flx), rf)
    hc, hf = G.rel_l2(G.sample(d, oc), rc), G.rel_l2(G.sample(d, of), rf)
    print("%s fp64 relL2 vs oracle-here conc %.2e flx %.2e | vs x86 reference conc %.2e flx %.2e "
          "(oracle-here vs x86 reference %.2e %.2e)" % (name, ec, ef, gc, gf, hc, hf))
    assert ec <= tol and ef <= tol, (name, ec, ef)
    assert gc <= hc + tol and gf <= hf + tol, (name, gc, gf, hc, hf)
    # grid as the reference builds it
    X, Y, Z = grid
    assert X.shape == np.squeeze(np.empty((len(np.atleast_1d(kw["levels"])),) + kw["srf_flx"].shape)).shape


@pytest.mark.parametrize("name", [n for n in G.solver_names() if n not in ("analytic_constant",)])
def test_fp32_within_tolerance(name):
    d = G.load(name)
    kw = G.kwargs_of(d)
    _, conc, flx = _gpu_solve(kw, mode="fp32")
    rc, rf = G.reference_fields(d)
    conc, flx = G.sample(d, conc), G.sample(d, flx)
    ec, ef = G.rel_l2(conc, rc), G.rel_l2(flx, rf)
    print("%s fp32 relL2 conc %.2e flx %.2e" % (name, ec, ef))
    assert ec <= FP32_TOL and ef <= FP32_TOL, (name, ec, ef)


def test_fp64_full_metric_size_against_oracle():
    """Headline workload at full size: footprint 512^2, n = 128 (207 levels),
    modes 512^2 on the 1536^2 extended grid, against the oracle (whose C port is
    bit-identical to the reference at this size)."""
    from oracle import bldfm_oracle as O

    d = G.load("metric_footprint_512")
    kw = G.kwargs_of(d)
    _, conc, flx = _gpu_solve(kw)
    _, oc, of = O.steady_state_transport_solver(**kw)
    ec, ef = G.rel_l2(conc, oc), G.rel_l2(flx, of)
    print("metric full fp64 vs oracle relL2 conc %.2e flx %.2e" % (ec, ef))
    assert ec <= FP64_TOL and ef <= FP64_TOL
    # the stored x86 reference output: as close as the oracle on this host
    hc = G.rel_l2(G.sample(d, oc), d["conc"])
    assert G.rel_l2(G.sample(d, conc), d["conc"]) <= hc + FP64_TOL


@pytest.mark.parametrize("name", G.profile_names())
def test_device_profiles_match_reference(name):
    from bldfm_gb300 import vertical_profiles

    d = G.load("profiles_" + name)
    kw = eval(str(d["kwargs"]))  # fixture-written dict literal of keyword arguments
    z, profs = vertical_profiles(int(d["n"]), float(d["meas_height"]), tuple(d["wind"]), **kw)
    assert z.shape == d["z"].shape
    np.testing.assert_allclose(z, d["z"], rtol=1e-13)
    np.testing.assert_allclose(np.stack(profs), d["profiles"], rtol=1e-12, atol=1e-300)


def test_footprint_unit_mass_and_positivity():
    from bldfm_gb300 import steady_state_transport_solver
    from oracle import bldfm_oracle as O

    z, p = O.vertical_profiles(16, 10.0, (0.0, -5.0), ustar=0.4)
    _, conc, flx = steady_state_transport_solver(
        np.zeros((64, 48)), z, p, (480.0, 640.0), 16, modes=(48, 64), footprint=True, halo=0.0, precision="double"
    )
    assert abs(flx.sum() - 1.0) < 1e-12
    zc, pc = O.vertical_profiles(16, 10.0, (0.0, -5.0), ustar=0.4, closure="CONSTANT")
    _, _, flx = steady_state_transport_solver(
        np.zeros((256, 64)), zc, pc, (50.0, 200.0), 16, modes=(64, 128), meas_pt=(25.0, 10.0), footprint=True
    )
    assert np.all(flx >= -1e-15 * np.abs(flx).max())


def test_repeated_calls_are_deterministic():
    d = G.load("multilevel_footprint")
    kw = G.kwargs_of(d)
    a = _gpu_solve(kw)[2]
    b = _gpu_solve(kw)[2]
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", ["source_area", "plume_3d", "multilevel_footprint", "ragged_odd",
                                  "quick_double_shift", "plume_levels_double", "cfg1_gaussian_256"])
def test_fp64r_matches_exact_discrete_solution(name):
    """Accurate FP64 mode against the FP64 invariant-imbedding restatement of
    the oracle: same mathematics, so agreement to FP64 rounding."""
    from oracle import bldfm_oracle as O

    d = G.load(name)
    kw = G.kwargs_of(d)
    _, conc, flx = _gpu_solve(kw, mode="fp64r")
    _, oc, of = O.steady_state_transport_solver(**kw, sweep="riccati")
    tol = F32_OUT_TOL if str(d["conc_dtype"]) == "float32" else 1e-11
    assert G.rel_l2(conc, oc) <= tol and G.rel_l2(flx, of) <= tol


def test_fp32_against_exact_on_headline_workload():
    """FP32 path against the accurate FP64 path on the full 512^2 footprint:
    the bar the batched FP32 and the surrogate are held to (relative L2 1e-3);
    the reference's own FP64 rounding floor on this case is ~5e-5."""
    d = G.load("metric_footprint_512")
    kw = G.kwargs_of(d)
    _, c32, f32 = _gpu_solve(kw, mode="fp32")
    _, cr, fr = _gpu_solve(kw, mode="fp64r")
    _, c64, f64 = _gpu_solve(kw, mode="fp64")
    e32 = max(G.rel_l2(c32, cr), G.rel_l2(f32, fr))
    floor = max(G.rel_l2(c64, cr), G.rel_l2(f64, fr))
    print("headline: fp32 vs exact %.2e, reference rounding vs exact %.2e" % (e32, floor))
    assert e32 <= 1e-4
    assert floor <= 1e-3


@pytest.mark.parametrize("name", ["metric_footprint_512", "plume_3d", "source_area"])
def test_dropin_states_its_error(name):
    """``return_error=True``: an FP32 result comes with its estimated relative
    L2 error against the exact discrete solution (the device accuracy check);
    the estimate stays within a factor 10 of the true error (measured against
    the accurate FP64 path) and below the 1e-3 bar; the FP64 modes state None.
    Without ``return_error`` the result is the plain (grid, conc, flx)."""
    from bldfm_gb300 import steady_state_transport_solver

    d = G.load(name)
    kw = G.kwargs_of(d)
    grid, c32, f32, est = steady_state_transport_solver(**kw, mode="fp32", return_error=True)
    _, cr, fr = _gpu_solve(kw, mode="fp64r")
    true = max(G.rel_l2(c32, cr), G.rel_l2(f32, fr))
    print("%s: stated %.2e, true %.2e" % (name, est, true))
    assert est <= 1e-3 and 0.1 * true <= est <= 10.0 * true, (est, true)
    *_, none = steady_state_transport_solver(**kw, mode="fp64", return_error=True)
    assert none is None
    assert len(steady_state_transport_solver(**kw, mode="fp32")) == 3
