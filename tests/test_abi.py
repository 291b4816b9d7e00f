"""C-ABI library: loads without a GPU, exports every declared symbol, and its
host-side planning matches the reference's grid arithmetic (solver.py:94-131)."""

import os
import re

import numpy as np
import pytest

from bldfm_gb300 import _lib
from bldfm_gb300.solver import make_desc, plan
from oracle import bldfm_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(bldfm_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_declared_symbols():
    lib = _lib.load()
    declared = _declared()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) <= set(_lib.exported_symbols()) | set(declared)


def test_version_string():
    assert b"sm_103a" in _lib.load().bldfm_version()


CASES = [
    ((512, 512), (1000.0, 1000.0), (512, 512), None),
    ((256, 256), (1000.0, 700.0), (512, 512), None),
    ((128, 64), (500.0, 250.0), (512, 512), 1.0),
    ((37, 53), (53.0, 37.0), (200, 200), 7.3),
    ((64, 128), (100.0, 700.0), (64, 128), None),
    ((100, 90), (123.4, 98.7), (64, 32), 11.0),
]


@pytest.mark.parametrize("shape,domain,modes,halo", CASES)
def test_plan_matches_reference_grid(shape, domain, modes, halo):
    d = make_desc(shape, 20, domain, modes, (0, 0), 0.0, True, False, halo, "double", "fp64")
    info = plan(d, 1)
    ref = O.solve_plan(shape, np.zeros(20), domain, 1, modes, halo)
    for k in ("nxe", "nye", "nlx", "nly", "px", "py"):
        assert getattr(info, k) == ref[k], k
    assert info.nfx == ref["nlx"] + 2 * ref["dlx"] and info.nfy == ref["nly"] + 2 * ref["dly"]
    nlx, nly = ref["nlx"], ref["nly"]
    # solved modes: Hermitian half plus unpaired modes
    kx = np.fft.fftfreq(nlx, 1.0 / nlx).astype(int)
    ky = np.fft.fftfreq(nly, 1.0 / nly).astype(int)
    KX, KY = np.meshgrid(kx, ky)
    mirror = np.isin(-KX, kx) & np.isin(-KY, ky)
    nonzero = ~((KX == 0) & (KY == 0))
    rep = (~mirror) | (KX > 0) | ((KX == 0) & (KY > 0))
    assert info.nsolved == int((rep & nonzero).sum())


def test_plan_errors_follow_reference():
    with pytest.raises(ValueError, match="modes must consist of even numbers"):
        plan(make_desc((64, 64), 10, (10.0, 10.0), (63, 64), (0, 0), 0.0, True, False, None, "single", "fp64"), 1)
    with pytest.raises(ValueError, match="precision must be single"):
        plan(make_desc((64, 64), 10, (10.0, 10.0), (64, 64), (0, 0), 0.0, True, False, None, "quad", "fp64"), 1)
    with pytest.raises(ValueError, match="broadcast"):
        plan(make_desc((64, 64), 10, (10.0, 10.0), (64, 64), (0, 0), 0.0, False, True, None, "single", "fp64"), 3)
    # non-footprint with an odd padding difference: the reference's truncated
    # spectrum does not fit the mode mask (IndexError)
    with pytest.raises(IndexError):
        plan(make_desc((63, 64), 10, (64.0, 63.0), (64, 64), (0, 0), 0.0, False, False, 3.0, "single", "fp64"), 1)


def test_odd_modes_reference_message_through_solver():
    from bldfm_gb300 import steady_state_transport_solver as S

    z = np.linspace(0.1, 10, 12)
    prof = tuple(np.ones(12) for _ in range(5))
    with pytest.raises(ValueError, match="modes must consist of even numbers"):
        S(np.zeros((32, 32)), z, prof, (10.0, 10.0), 5, modes=(31, 32))
    with pytest.raises(ValueError, match="precision must be single"):
        S(np.zeros((32, 32)), z, prof, (10.0, 10.0), 5, modes=(32, 32), precision="quad")
    with pytest.raises(IndexError):
        S(np.zeros((32, 32)), z, prof, (10.0, 10.0), 50, modes=(32, 32))


@pytest.mark.parametrize("xform_lines", [0, 1, 2, 4])
def test_batch_plan_sizes_without_device_cache(xform_lines):
    """bldfm_batch_plan sizes a mixed batch on the host for every transform
    setting (1 = the persistent one-line passes), without a device."""
    import ctypes

    lib = _lib.load()
    keep, arr = [], (_lib.Case * 2)()
    for k, (shape, modes, n) in enumerate([((96, 128), (128, 96), 20), ((64, 64), (64, 64), 12)]):
        z, p = O.vertical_profiles(n, 10.0, (2.0, -1.0), ustar=0.3, mol=-50.0)
        zz = np.ascontiguousarray(z, dtype=np.float64)
        prof = np.ascontiguousarray(np.stack(p))
        lv = np.array([n], dtype=np.int64)
        keep += [zz, prof, lv]
        c = arr[k]
        c.desc = make_desc(shape, len(zz), (200.0, 150.0), modes, (80.0, 70.0), 0.0, True, False, None, "double",
                           "fp32")
        c.z_host, c.prof_host, c.levels_host, c.nlvls = zz.ctypes.data, prof.ctypes.data, lv.ctypes.data, 1
        c.conc_dev = c.flx_dev = 256  # output addresses are only checked for presence when planning
    opts = _lib.BatchOpts(0, 0, 0, xform_lines, 0)
    need = ctypes.c_int64(0)
    assert lib.bldfm_batch_plan(arr, 2, ctypes.byref(opts), ctypes.byref(need)) == 0
    assert need.value > 0


def test_host_level_table_rounds_like_the_reference():
    """The FP64 path's per-level scalars (dz**2, dz**3, Kzinv**2 through libm's
    pow, src/bldfm/solver.py:361-364) equal the reference's numpy values bit
    for bit over many grids.  A compiler that turned pow(x, 2.0) into x * x
    would differ by one ulp for rare x, which the shooting method amplifies
    by up to e^{2G} (about 1e25 on the 1024^2, n = 256 footprint)."""
    import ctypes

    lib = ctypes.CDLL(_lib.LIB_PATH)
    lib.hx_level_table.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hx_level_table.restype = None
    bad = 0
    for n in range(16, 520, 11):
        for ustar in (0.2, 0.3, 0.5):
            z, p = O.vertical_profiles(n, 20.0, O.compute_wind_fields(4.0, 225.0), ustar=ustar, mol=-50.0)
            nz = len(z)
            prof = np.ascontiguousarray(np.stack(p))
            zz = np.ascontiguousarray(z)
            lv = np.zeros((nz - 1, 12))
            lib.hx_level_table(nz, zz.ctypes.data, prof.ctypes.data, lv.ctypes.data)
            bad += int(np.sum(lv[:, :11] != O.level_table(z, p)[:, :11]))
    assert bad == 0
