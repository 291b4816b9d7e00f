"""Footprint properties the reference's integration tests check
(tests/test_integration.py:87-162 convergence, :402-520 upwind peak;
tests/test_memory.py:25-120 growth), on the GPU paths."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["fp64", "fp32"])
def test_convergence_trend_against_analytic(mode):
    """CONSTANT closure: the error against the analytic solution falls at each
    refinement of modes and levels (setup of test_integration.py:87-162)."""
    from bldfm_gb300 import steady_state_transport_solver, vertical_profiles
    from bldfm_gb300.utils import ideal_source

    nxy, domain, src, halo, zm, wind, ustar = (128, 64), (100.0, 50.0), (5.0, 5.0), 500.0, 5.0, (4.0, 1.0), 0.2
    srf = ideal_source(nxy, domain, src, shape="point")
    res = [((64, 64), 8), ((128, 128), 16), ((256, 256), 32)]
    z, p = vertical_profiles(res[-1][1], zm, wind, ustar, closure="CONSTANT")
    _, _, ana = steady_state_transport_solver(srf, z, p, domain, res[-1][1], modes=res[-1][0], halo=halo,
                                              analytic=True)
    errs = []
    for modes, nz in res:
        z, p = vertical_profiles(nz, zm, wind, ustar, closure="CONSTANT")
        _, _, flx = steady_state_transport_solver(srf, z, p, domain, nz, modes=modes, halo=halo, mode=mode)
        errs.append(np.mean((flx - ana) ** 2) / np.mean(ana**2))
    assert errs[0] > errs[1] > errs[2], errs


@pytest.mark.parametrize("mode", ["fp64", "fp32"])
@pytest.mark.parametrize("wind,nxy,domain,modes,meas", [
    ((0.0, -5.0), (64, 256), (50.0, 200.0), (64, 128), (25.0, 10.0)),   # southward: peak at y > meas_y
    ((-5.0, 0.0), (256, 64), (200.0, 50.0), (128, 64), (10.0, 25.0)),   # westward: peak at x > meas_x
])
def test_footprint_peak_upwind(mode, wind, nxy, domain, modes, meas):
    from bldfm_gb300 import steady_state_transport_solver, vertical_profiles

    z, p = vertical_profiles(16, 10.0, wind, z0=0.1, mol=1e9)
    (X, Y, _), _, flx = steady_state_transport_solver(np.zeros(nxy[::-1]), z, p, domain, 16, modes=modes,
                                                      meas_pt=meas, footprint=True, mode=mode)
    i = np.unravel_index(np.argmax(flx), flx.shape)
    if wind[1] < 0:
        assert Y[i] > meas[1]
    else:
        assert X[i] > meas[0]


def _rss_bytes():
    with open("/proc/self/statm") as f:
        return int(f.read().split()[1]) * 4096


def test_repeated_solves_do_not_grow_memory():
    """Ten solves of one shape: device and host memory stay flat after the
    first (the reference allows 20% growth of host RSS over 10 solves)."""
    import torch

    from bldfm_gb300 import steady_state_transport_solver, vertical_profiles

    z, p = vertical_profiles(64, 10.0, (3.0, -2.0), ustar=0.3, mol=-80.0)
    kw = dict(srf_flx=np.zeros((256, 256)), z=z, profiles=p, domain=(500.0, 500.0), levels=64, modes=(256, 256),
              meas_pt=(250.0, 250.0), footprint=True)
    for mode in ("fp64", "fp32"):
        steady_state_transport_solver(**kw, mode=mode)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rss0 = _rss_bytes()
    for _ in range(10):
        for mode in ("fp64", "fp32"):
            steady_state_transport_solver(**kw, mode=mode)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free0 - free1 < 64 << 20  # device: no per-call growth beyond allocator noise
    assert _rss_bytes() < 1.2 * rss0


def test_bounded_wait_reports_timeout_and_context_survives():
    """Failure detection without a fault: a wait that nothing completes gives
    up after its poll limit and reports BLDFM_ERR_TIMEOUT; the next solve on
    the same context works."""
    import ctypes

    from bldfm_gb300 import _lib, steady_state_transport_solver, vertical_profiles

    z, p = vertical_profiles(16, 10.0, (0.0, -5.0), ustar=0.4)
    kw = dict(srf_flx=np.zeros((64, 48)), z=z, profiles=p, domain=(480.0, 640.0), levels=16, modes=(48, 64),
              meas_pt=(240.0, 320.0), footprint=True)
    before = steady_state_transport_solver(**kw)[2]
    lib = _lib.load()
    st, ns = ctypes.c_int32(0), ctypes.c_int64(0)
    assert lib.bldfm_selftest_wait_timeout(1 << 10, ctypes.byref(st), ctypes.byref(ns)) == 0
    assert st.value == _lib.ERR_TIMEOUT
    assert 0 < ns.value < 10**10
    print(f"bounded wait: 1024 polls in {ns.value / 1e3:.1f} us")
    after = steady_state_transport_solver(**kw)[2]
    assert np.array_equal(before, after)
