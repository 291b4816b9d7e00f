"""Pin the CPU oracle to the reference: it must reproduce every golden fixture
(generated by running the reference itself, tests/golden/make_golden.py)
bit-for-bit, and the reference's own regression fixture values."""

import numpy as np
import pytest

import golden_cases as G
from oracle import bldfm_oracle as O


@pytest.mark.parametrize("name", G.solver_names())
def test_oracle_matches_reference_fixture(name):
    d = G.load(name)
    kw = G.kwargs_of(d)
    grid, conc, flx = O.steady_state_transport_solver(**kw)
    rc, rf = G.reference_fields(d)
    conc, flx = G.sample(d, conc), G.sample(d, flx)
    assert conc.shape == rc.shape and flx.shape == rf.shape
    assert str(conc.dtype) == str(d["conc_dtype"])
    # identical arithmetic: bitwise equal (allow 1e-14 for libm differences across hosts)
    assert G.rel_l2(conc, rc) <= 1e-14, name
    assert G.rel_l2(flx, rf) <= 1e-14, name


@pytest.mark.parametrize("name", G.solver_names())
def test_oracle_numpy_sweep_matches_port(name):
    """The pure-numpy sweep and the C port are the same arithmetic."""
    d = G.load(name)
    if d["conc"].size > 200000:
        pytest.skip("large case: covered by the port test")
    kw = G.kwargs_of(d)
    _, c1, f1 = O.steady_state_transport_solver(**kw, use_port=True)
    _, c2, f2 = O.steady_state_transport_solver(**kw, use_port=False)
    np.testing.assert_array_equal(c1, c2)
    np.testing.assert_array_equal(f1, f2)


@pytest.mark.parametrize("name", G.profile_names())
def test_oracle_profiles_match_reference(name):
    d = G.load("profiles_" + name)
    kw = eval(str(d["kwargs"]))  # fixture-written dict literal of keyword arguments
    z, profs = O.vertical_profiles(int(d["n"]), float(d["meas_height"]), tuple(d["wind"]), **kw)
    np.testing.assert_allclose(z, d["z"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(np.stack(profs), d["profiles"], rtol=1e-14, atol=1e-300)


def test_footprint_unit_mass_extended_grid():
    """With halo = 0 the footprint integrates to exactly 1 over the extended grid
    (tfftq[:, 0, 0] = 1 / (nxe * nye), solver.py:134,191)."""
    z, p = O.vertical_profiles(16, 10.0, (0.0, -5.0), ustar=0.4)
    _, conc, flx = O.steady_state_transport_solver(
        np.zeros((64, 48)), z, p, (480.0, 640.0), 16, modes=(48, 64), footprint=True, halo=0.0, precision="double"
    )
    assert abs(flx.sum() - 1.0) < 1e-12


def test_snapshot_schedule_semantics():
    slot, n = O.snapshot_schedule(np.array([5, 2, 2, 40]), 10)
    assert n == 2 and slot[2] == 0 and slot[5] == 1 and (slot >= 0).sum() == 2


@pytest.mark.parametrize("name", ["source_area", "plume_3d", "multilevel_footprint", "ragged_odd"])
def test_riccati_oracle_agrees_with_shooting_where_well_conditioned(name):
    """The invariant-imbedding restatement solves the same discrete problem:
    on fixtures whose shooting cancellation is mild both agree closely."""
    d = G.load(name)
    kw = G.kwargs_of(d)
    _, c1, f1 = O.steady_state_transport_solver(**kw)
    _, c2, f2 = O.steady_state_transport_solver(**kw, sweep="riccati")
    assert G.rel_l2(c2, c1) <= 1e-6 and G.rel_l2(f2, f1) <= 1e-6
