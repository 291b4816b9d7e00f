"""The drop-in swapped into the reference itself (the integration notes'
monkeypatch of ``bldfm.interface.steady_state_transport_solver``, reference
src/bldfm/interface.py:15, 115-128), run through the reference's own
``run_bldfm_single``.

This runs on the CPU: the reference tree is imported with its third-party
dependencies stubbed (tests/golden/refshim.py), and only the device call at
the bottom of the drop-in, ``bldfm_solve_host``, is replaced by a stand-in
that rebuilds the solve from the C-ABI descriptor and arrays it receives and
evaluates it with the oracle.  So the test checks what the swap depends on:
the reference calls the drop-in with its own keyword arguments, the drop-in
turns them into the descriptor, profiles and level list of the C ABI
faithfully, and the result dictionaries of the swapped and the unmodified
reference are the same.  The device arithmetic itself is checked against the
same oracle by the GPU tests.  Skips when the reference tree is absent.
"""

import ctypes
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import refshim  # noqa: E402

import interface_configs as IC  # noqa: E402

pytestmark = pytest.mark.skipif(not refshim.reference_available(), reason="reference tree not present")


class _OracleLib:
    """The C library with bldfm_solve_host answered by the oracle."""

    def __init__(self, lib):
        self._lib = lib
        self.calls = 0

    def __getattr__(self, name):
        return getattr(self._lib, name)

    def bldfm_solve_host(self, d, srf, z, prof, levels, nlvls, conc, flx):
        from bldfm_gb300 import _lib
        from oracle import bldfm_oracle as O

        self.calls += 1
        info = _lib.PlanInfo()
        assert self._lib.bldfm_plan(d, nlvls, info) == 0
        nz = d.nz
        arr = lambda p, n: np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), shape=(n,))
        zz = arr(z, nz).copy()
        pr = arr(prof, 5 * nz).reshape(5, nz).copy()
        lv = np.ctypeslib.as_array(ctypes.cast(levels, ctypes.POINTER(ctypes.c_int64)), shape=(nlvls,)).copy()
        src = np.zeros((d.ny, d.nx)) if d.footprint else arr(srf, d.ny * d.nx).reshape(d.ny, d.nx).copy()
        _, c, f = O.steady_state_transport_solver(
            src, zz, tuple(pr), (d.xmax, d.ymax), lv, modes=(d.nlx, d.nly), meas_pt=(d.meas_x, d.meas_y),
            srf_bg_conc=d.srf_bg_conc, footprint=bool(d.footprint), analytic=bool(d.analytic),
            halo=d.halo if d.has_halo else None, precision="single" if d.precision == _lib.PREC_SINGLE else "double")
        shape = (nlvls, info.out_ny, info.out_nx)
        arr(conc, int(np.prod(shape)))[:] = np.asarray(c, dtype=np.float64).ravel()
        arr(flx, int(np.prod(shape)))[:] = np.asarray(f, dtype=np.float64).ravel()
        return 0


@pytest.mark.parametrize("footprint,levels", [(True, None), (False, [4, 16]), (False, None)])
def test_dropin_inside_reference_runner(monkeypatch, footprint, levels):
    bldfm = refshim.import_reference()
    import bldfm.interface as ref_interface

    from bldfm_gb300 import _lib
    from bldfm_gb300 import solver as ours

    cfg = IC.config(n_steps=2, towers=2, footprint=footprint, output_levels=levels)
    if not footprint:
        cfg.solver.precision = "single"
    tower = cfg.towers[1]
    want = ref_interface.run_bldfm_single(cfg, tower, met_index=1)

    fake = _OracleLib(_lib.load())
    monkeypatch.setattr(_lib, "load", lambda: fake)
    monkeypatch.setattr(ref_interface, "steady_state_transport_solver", ours.steady_state_transport_solver)
    monkeypatch.setattr(bldfm.solver, "steady_state_transport_solver", ours.steady_state_transport_solver)
    got = ref_interface.run_bldfm_single(cfg, tower, met_index=1)

    assert fake.calls == 1
    assert set(got) == set(want)
    for key in ("tower_name", "tower_xy", "timestamp", "params"):
        assert got[key] == want[key]
    for a, b in zip(got["grid"], want["grid"]):
        np.testing.assert_array_equal(a, b)
    for key in ("conc", "flx"):
        assert got[key].shape == want[key].shape and got[key].dtype == want[key].dtype
        np.testing.assert_allclose(got[key], want[key], rtol=1e-12, atol=1e-14 * np.abs(want[key]).max())
