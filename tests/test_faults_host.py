"""Failure detection on the host: invalid inputs are turned into a status code
or the reference's exception before any GPU work is enqueued, so these run
without a GPU.

The reference validates modes (src/bldfm/solver.py:89-91), precision
(:187-188) and the ustar / z0 choice (src/bldfm/pbl_model.py:76-77); this
library also rejects profiles the sweep cannot integrate (non-finite values,
z not strictly increasing, Kz <= 0, Kx or Ky < 0: the sweep divides by Kz and
by the top eigenvalue, solver.py:164-174, 357-364) with BLDFM_ERR_PROFILE,
where the reference would return NaN fields.  Each case goes through every
C-ABI entry point that takes profiles: the host entry (the drop-in's path),
the batched planner and the allocation-free entry.
"""

import ctypes

import numpy as np
import pytest

from bldfm_gb300 import _lib
from bldfm_gb300.solver import make_desc, steady_state_transport_solver
from oracle import bldfm_oracle as O


def _good():
    z, p = O.vertical_profiles(16, 10.0, (3.0, -4.0), ustar=0.35, mol=-40.0)
    return np.ascontiguousarray(z), np.ascontiguousarray(np.stack(p))


def _kw(z, prof):
    return dict(srf_flx=np.zeros((48, 64)), z=z, profiles=tuple(prof), domain=(128.0, 96.0), levels=len(z) - 1,
                modes=(64, 48), meas_pt=(40.0, 50.0), footprint=True, precision="double")


def _bad_profiles():
    z, prof = _good()
    out = []
    for name, k, i, v in [("nan u", 0, 3, np.nan), ("inf v", 1, 5, np.inf), ("nan Kx", 2, 0, np.nan),
                          ("Kz zero", 4, 7, 0.0), ("Kz negative", 4, 15, -1.0), ("Kx negative", 2, 4, -0.1),
                          ("Ky negative", 3, 9, -2.0), ("Kz inf", 4, 2, np.inf)]:
        p = prof.copy()
        p[k, i] = v
        out.append((name, z, p))
    zz = z.copy()
    zz[6] = zz[5]  # dz = 0
    out.append(("repeated z", zz, prof))
    zz = z.copy()
    zz[6], zz[7] = zz[7], zz[6]  # negative dz
    out.append(("negative dz", zz, prof))
    zz = z.copy()
    zz[0] = np.nan
    out.append(("nan z", zz, prof))
    return out


@pytest.mark.parametrize("name,z,prof", _bad_profiles(), ids=[b[0] for b in _bad_profiles()])
def test_invalid_profiles_rejected_by_every_entry(name, z, prof):
    lib = _lib.load()
    with pytest.raises(ValueError, match="profiles finite"):
        steady_state_transport_solver(**_kw(z, prof))
    lv = np.array([len(z) - 1], dtype=np.int64)
    d = make_desc((48, 64), len(z), (128.0, 96.0), (64, 48), (40.0, 50.0), 0.0, True, False, None, "double", "fp32")
    out = np.zeros(1)
    st = lib.bldfm_solve_host(d, None, _lib.ptr(z), _lib.ptr(prof), _lib.ptr(lv), 1, _lib.ptr(out), _lib.ptr(out))
    assert st == _lib.ERR_PROFILE
    st = lib.bldfm_solve_noalloc(d, None, _lib.ptr(z), _lib.ptr(prof), _lib.ptr(lv), 1, _lib.ptr(out),
                                 _lib.ptr(out), None, None)
    assert st == _lib.ERR_PROFILE
    case = _lib.Case()
    case.desc = d
    case.z_host, case.prof_host, case.levels_host = z.ctypes.data, prof.ctypes.data, lv.ctypes.data
    case.nlvls = 1
    case.conc_dev = case.flx_dev = out.ctypes.data  # planning never dereferences the outputs
    opts = _lib.BatchOpts(0, 0, 0, 0, 0)
    nb = ctypes.c_int64(0)
    st = lib.bldfm_batch_plan(ctypes.byref(case), 1, ctypes.byref(opts), ctypes.byref(nb))
    assert st == _lib.ERR_PROFILE


def _desc_variants():
    base = dict(shape=(48, 64), nz=16, domain=(128.0, 96.0), modes=(64, 48), meas=(40.0, 50.0), halo=None,
                precision="double", mode="fp64")
    out = []

    def v(name, want, **kw):
        b = dict(base)
        b.update(kw)
        out.append((name, want, b))

    v("odd modes", _lib.ERR_ODD_MODES, modes=(63, 48))
    v("precision", _lib.ERR_PRECISION, precision="quad")
    v("zero nx", _lib.ERR_ARG, shape=(48, 0))
    v("negative domain", _lib.ERR_ARG, domain=(-1.0, 96.0))
    v("nan domain", _lib.ERR_ARG, domain=(np.nan, 96.0))
    v("negative halo", _lib.ERR_ARG, halo=-5.0)
    v("nan halo", _lib.ERR_ARG, halo=np.nan)
    v("huge halo", _lib.ERR_UNSUPPORTED, halo=1e12)
    v("too many levels", _lib.ERR_UNSUPPORTED, nz=1 << 20)
    return out


@pytest.mark.parametrize("name,want,b", _desc_variants(), ids=[v[0] for v in _desc_variants()])
def test_corrupt_descriptor_status(name, want, b):
    lib = _lib.load()
    d = make_desc(b["shape"], b["nz"], b["domain"], b["modes"], b["meas"], 0.0, True, False, b["halo"],
                  b["precision"], b["mode"])
    info = _lib.PlanInfo()
    assert lib.bldfm_plan(d, 1, info) == want


def test_corrupt_mode_field_and_levels():
    lib = _lib.load()
    z, prof = _good()
    d = make_desc((48, 64), len(z), (128.0, 96.0), (64, 48), (40.0, 50.0), 0.0, True, False, None, "double", "fp64")
    d.mode = 7  # not a BLDFM_MODE_*
    info = _lib.PlanInfo()
    assert lib.bldfm_plan(d, 1, info) == _lib.ERR_ARG
    d.mode = _lib.MODE_FP32
    out = np.zeros(1)
    for bad in (len(z), -len(z) - 1, 1 << 40):
        lv = np.array([bad], dtype=np.int64)
        st = lib.bldfm_solve_host(d, None, _lib.ptr(z), _lib.ptr(prof), _lib.ptr(lv), 1, _lib.ptr(out),
                                  _lib.ptr(out))
        assert st == _lib.ERR_ARG, bad
    assert lib.bldfm_plan(d, 0, info) == _lib.ERR_ARG  # no output level
    assert lib.bldfm_solve_host(None, None, None, None, None, 1, None, None) == _lib.ERR_ARG


def test_reference_exceptions():
    z, prof = _good()
    kw = _kw(z, prof)
    with pytest.raises(ValueError, match="modes must consist of even numbers."):
        steady_state_transport_solver(**dict(kw, modes=(63, 48)))
    with pytest.raises(ValueError, match="precision must be single"):
        steady_state_transport_solver(**dict(kw, precision="half"))
    from bldfm_gb300 import vertical_profiles

    with pytest.raises(ValueError, match="Either z0 or ustar"):
        vertical_profiles(16, 10.0, (3.0, -4.0), ustar=0.3, z0=0.1)


def test_status_strings_name_every_code():
    lib = _lib.load()
    codes = [getattr(_lib, n) for n in dir(_lib) if n.startswith("ERR_")]
    names = {lib.bldfm_status_str(c).decode() for c in codes}
    assert "unknown status" not in names and len(names) == len(codes)
    # a C++ exception inside the library (host allocation) arrives as a status
    with pytest.raises(MemoryError, match="host-side failure"):
        _lib.check(_lib.ERR_HOST)


def test_batch_plan_reports_the_first_failing_case():
    """A batch of eight cases is planned on the library's host threads; the
    status is the first failing case's (lowest index), whichever thread
    planned it, and a valid batch plans to the same workspace every time."""
    lib = _lib.load()
    z, prof = _good()
    lv = np.array([len(z) - 1], dtype=np.int64)
    out = np.zeros(1)
    bad = prof.copy()
    bad[4, 3] = -1.0  # Kz < 0: BLDFM_ERR_PROFILE

    def batch(faults):
        arr = (_lib.Case * 8)()
        keep = []
        for k in range(8):
            modes = (63, 48) if faults.get(k) == "odd" else (64, 48)
            p = bad if faults.get(k) == "profile" else prof
            d = make_desc((48, 64), len(z), (128.0, 96.0), modes, (40.0, 50.0), 0.0, True, False, None, "double",
                          "fp32")
            c = arr[k]
            c.desc = d
            c.z_host, c.prof_host, c.levels_host = z.ctypes.data, p.ctypes.data, lv.ctypes.data
            c.nlvls = 1
            c.conc_dev = c.flx_dev = out.ctypes.data  # planning never dereferences the outputs
            keep.append(d)
        nb = ctypes.c_int64(0)
        st = lib.bldfm_batch_plan(arr, 8, ctypes.byref(_lib.BatchOpts(0, 0, 0, 0, 0)), ctypes.byref(nb))
        return st, nb.value

    assert batch({3: "profile", 6: "odd"})[0] == _lib.ERR_PROFILE
    assert batch({2: "odd", 5: "profile"})[0] == _lib.ERR_ODD_MODES
    sizes = {batch({}) for _ in range(20)}
    assert len(sizes) == 1 and next(iter(sizes))[0] == 0 and next(iter(sizes))[1] > 0


def test_batch_plan_from_many_threads():
    """Host threads calling the library at once (each call holds the
    library's lock and reuses its pool of host threads) plan their batches
    exactly as one thread does."""
    import threading

    lib = _lib.load()
    z, prof = _good()
    lv = np.array([len(z) - 1], dtype=np.int64)
    out = np.zeros(1)
    arrs = []
    for n in (4, 6, 8, 12):
        arr = (_lib.Case * n)()
        for k in range(n):
            c = arr[k]
            c.desc = make_desc((48, 64), len(z), (128.0, 96.0), (64, 48), (40.0, 50.0), 0.0, True, False, None,
                               "double", "fp32")
            c.z_host, c.prof_host, c.levels_host = z.ctypes.data, prof.ctypes.data, lv.ctypes.data
            c.nlvls = 1
            c.conc_dev = c.flx_dev = out.ctypes.data
        arrs.append((arr, n))

    def plan(arr, n):
        nb = ctypes.c_int64(0)
        st = lib.bldfm_batch_plan(arr, n, ctypes.byref(_lib.BatchOpts(0, 0, 0, 0, 0)), ctypes.byref(nb))
        return st, nb.value

    want = [plan(a, n) for a, n in arrs]
    got, errs = [], []

    def worker(i):
        try:
            for _ in range(50):
                a, n = arrs[i % len(arrs)]
                got.append((i % len(arrs), plan(a, n)))
        except Exception as e:  # surfaced below
            errs.append(e)

    th = [threading.Thread(target=worker, args=(i,)) for i in range(8)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs
    assert len(got) == 400 and all(r == want[i] for i, r in got)
