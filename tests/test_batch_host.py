"""Host side of the batched solver (no GPU): the conversion of a case's
inputs into the arrays the library reads, and the results built from the
copied-back output buffer."""

from types import SimpleNamespace

import numpy as np
import pytest
import torch

from bldfm_gb300.batch import _finish_batch, _grid, _host_inputs


def _case(nz=9, levels=4, profiles=None, **kw):
    z = np.linspace(0.0, 40.0, nz)
    if profiles is None:
        profiles = tuple(np.arange(nz, dtype=np.float64) + 10 * j for j in range(5))
    d = dict(srf_flx=np.zeros((6, 8)), z=z, profiles=profiles, domain=(80.0, 60.0), levels=levels, modes=(8, 6))
    d.update(kw)
    return d


def test_host_inputs_pack_z_and_profiles():
    kw = _case()
    zp, nz, levels, lv, lvp = _host_inputs(kw)
    assert nz == 9 and zp.dtype == np.float64 and zp.flags.c_contiguous
    np.testing.assert_array_equal(zp[:nz], kw["z"])
    np.testing.assert_array_equal(zp[nz:].reshape(5, nz), np.stack(kw["profiles"]))
    assert lv.dtype == np.int64 and list(lv) == [4] and lvp == lv.ctypes.data
    np.testing.assert_array_equal(np.asarray(kw["z"])[levels], kw["z"][[4]])


def test_host_inputs_broadcast_scalar_profiles_and_other_dtypes():
    nz = 7
    kw = _case(nz=nz, profiles=(1.5, np.float32(-2.0), 3, np.full(nz, 4.0, np.float32), 0.25), levels=-1)
    kw["z"] = list(range(nz))  # a list of ints
    zp, n, levels, lv, _ = _host_inputs(kw)
    assert n == nz
    np.testing.assert_array_equal(zp[:nz], np.arange(nz, dtype=np.float64))
    np.testing.assert_array_equal(zp[nz:].reshape(5, nz), np.array([[1.5], [-2.0], [3.0], [4.0], [0.25]]) * np.ones(nz))
    assert list(lv) == [-1]


def test_host_inputs_level_arrays_and_errors():
    zp, nz, levels, lv, lvp = _host_inputs(_case(levels=[0, 3, 8]))
    assert list(lv) == [0, 3, 8] and lvp == lv.ctypes.data
    with pytest.raises(IndexError):
        _host_inputs(_case(levels=[2, 9]))
    with pytest.raises(ValueError):
        _host_inputs(_case(profiles=(np.zeros(9), np.zeros(9), np.zeros(9), np.zeros(9), np.zeros(5))))


def test_shared_integer_level_arrays_are_read_only():
    _, _, levels, lv, _ = _host_inputs(_case(levels=3))
    _, _, levels2, lv2, _ = _host_inputs(_case(levels=np.int32(3)))
    assert lv is lv2 and not lv.flags.writeable and not levels.flags.writeable


def _pending(cases, shapes, host, sums=None):
    keep = []
    for kw in cases:
        zp, nz, levels, lv, _ = _host_inputs(kw)
        keep.append((zp, nz, lv, levels))
    solver = SimpleNamespace(stream=SimpleNamespace(synchronize=lambda: None))
    # workspace head as the library leaves it: status word, then from byte 64
    # the accuracy check's four float sums per case
    head = torch.zeros(64 + 16 * len(cases), dtype=torch.uint8)
    if sums is not None:
        head[64:].view(torch.float32)[:] = torch.tensor(np.asarray(sums, np.float32).ravel())
    return (solver, cases, shapes, keep, torch.from_numpy(host), head)


def test_finish_states_each_case_error_from_the_check_sums():
    from bldfm_gb300.batch import BatchResults, error_estimate

    cases = [_case(footprint=True), _case(footprint=True), _case(footprint=True)]
    shapes = [(1, 6, 8)] * 3
    host = np.zeros(2 * 3 * 48)
    # (sum |dXp|^2, sum |Xp|^2, sum |dXq|^2, sum |Xq|^2) per case
    sums = [[1e-12, 1.0, 4e-12, 1.0], [9e-14, 1e-2, 0.0, 4.0], [0.0, 0.0, 0.0, 0.0]]
    res = _finish_batch(_pending(cases, shapes, host, sums))
    assert isinstance(res, BatchResults) and len(res) == 3
    u2 = 2.0**-48  # the transform's rounding term, squared, per unit of field
    want = [((4e-12 + 2 * u2) / 1.0) ** 0.5, ((9e-14 + 4.01 * u2) / 1e-2) ** 0.5, 0.0]
    np.testing.assert_allclose(res.error_estimates, want, rtol=1e-6)
    assert error_estimate(sums[0]) == pytest.approx(want[0])
    # a flux field 100 times smaller than the concentration: the transform's
    # rounding dominates its statement
    assert error_estimate([0.0, 1.0, 0.0, 1e-4]) == pytest.approx(2.0**-24 * (1.0001 / 1e-4) ** 0.5)


@pytest.mark.parametrize("mixed", [False, True])
def test_finish_builds_results_like_slicing_and_squeeze(mixed):
    rng = np.random.default_rng(1)
    cases = [_case(footprint=True), _case(levels=[1, 2], footprint=True), _case(footprint=True)]
    shapes = [(1, 6, 8), (2, 6, 8), (1, 6, 8)]
    if not mixed:
        cases, shapes = [cases[0], cases[2]], [shapes[0], shapes[2]]
    sizes = [int(np.prod(s)) for s in shapes]
    host = rng.standard_normal(2 * sum(sizes) + 5)  # the pinned buffer may be longer
    res = _finish_batch(_pending(cases, shapes, host))
    off = 0
    for kw, shape, sz, (grid, conc, flx) in zip(cases, shapes, sizes, res):
        np.testing.assert_array_equal(conc, np.squeeze(host[off : off + sz].reshape(shape)))
        np.testing.assert_array_equal(flx, np.squeeze(host[off + sz : off + 2 * sz].reshape(shape)))
        assert conc.dtype == np.float64
        ref = _grid(kw["z"], np.atleast_1d(kw["levels"]), (6, 8), kw["domain"])
        for a, b in zip(grid, ref):
            np.testing.assert_array_equal(a, b)
        off += 2 * sz


def test_finish_single_precision_without_shift_gives_float32():
    cases = [_case(precision="single", meas_pt=(0.0, 0.0)), _case(precision="single", meas_pt=(10.0, 0.0))]
    shapes = [(1, 6, 8)] * 2
    host = np.arange(4 * 48, dtype=np.float64)
    (_, c0, f0), (_, c1, f1) = _finish_batch(_pending(cases, shapes, host))
    assert c0.dtype == np.float32 and f0.dtype == np.float32
    assert c1.dtype == np.float64 and c0.shape == (6, 8)
    np.testing.assert_array_equal(f0, host[48:96].reshape(6, 8).astype(np.float32))


def test_prepare_fills_the_case_array():
    """prepare() with a host stand-in for the device output buffer: every
    case's pointers address its packed inputs and its slots of the output
    buffer (conc then flx, back to back)."""
    import ctypes

    from bldfm_gb300 import _lib
    from bldfm_gb300.batch import BatchSolver

    s = object.__new__(BatchSolver)
    s.device, s._srf, s._keep = torch.device("cpu"), {}, None
    s._out_buf = torch.empty(10_000, dtype=torch.float64)
    cases = [_case(footprint=True), _case(levels=[1, 2, 3], footprint=True, domain=(90.0, 60.0))]
    arr, shapes, keep = s.prepare(cases, views=False)
    base = s._out_buf.data_ptr()
    off = 0
    for k, (c, shape, (zp, nz, lv, levels)) in enumerate(zip(arr, shapes, keep)):
        assert shape[0] == len(lv)
        assert c.z_host == zp.ctypes.data and c.prof_host == c.z_host + 8 * nz
        assert c.levels_host == lv.ctypes.data and c.nlvls == len(lv)
        assert c.desc.footprint == 1 and c.desc.mode == _lib.MODE_FP32
        got = np.ctypeslib.as_array((ctypes.c_double * (6 * nz)).from_address(c.z_host))
        np.testing.assert_array_equal(got, np.concatenate((cases[k]["z"], *cases[k]["profiles"])))
        sz = int(np.prod(shape))
        assert c.conc_dev == base + 8 * off and c.flx_dev == base + 8 * (off + sz)
        off += 2 * sz
    assert s.out_elems == off
    assert arr[0].desc.xmax == 80.0 and arr[1].desc.xmax == 90.0
