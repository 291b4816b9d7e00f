"""Failure detection on the device without a GPU fault: a NaN in the surface
flux (device memory, which the host does not scan) spreads through the
forward transform into every output value; the final output pass flags it in
the device status word (BLDFM_ERR_NONFINITE), and each entry point reports it
while the context stays usable for the next solve."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _kw(src):
    from oracle import bldfm_oracle as O

    z, p = O.vertical_profiles(16, 10.0, (3.0, -4.0), ustar=0.35, mol=-40.0)
    return dict(srf_flx=src, z=z, profiles=p, domain=(128.0, 96.0), levels=[4, 16], modes=(64, 48),
                meas_pt=(40.0, 50.0), footprint=False, precision="double")


def _nan_source():
    src = np.random.default_rng(0).random((48, 64))
    src[10, 20] = np.nan
    return src


@pytest.mark.parametrize("mode", ["fp64", "fp32", "fp64r"])
def test_nonfinite_output_raises_then_context_recovers(mode):
    from bldfm_gb300 import steady_state_transport_solver

    with pytest.raises(FloatingPointError, match="non-finite"):
        steady_state_transport_solver(**_kw(_nan_source()), mode=mode)
    good = _kw(np.random.default_rng(1).random((48, 64)))
    a = steady_state_transport_solver(**good, mode=mode)[2]
    b = steady_state_transport_solver(**good, mode=mode)[2]
    assert np.all(np.isfinite(a)) and np.array_equal(a, b)


def test_nonfinite_status_word_of_workspace_and_batch():
    import torch

    from bldfm_gb300 import _lib
    from bldfm_gb300.batch import BatchSolver, solve_batch
    from bldfm_gb300.solver import make_desc, plan

    lib = _lib.load()
    kw = _kw(_nan_source())
    z = np.ascontiguousarray(kw["z"])
    prof = np.ascontiguousarray(np.stack(kw["profiles"]))
    lv = np.array([4, 16], dtype=np.int64)
    d = make_desc((48, 64), len(z), kw["domain"], kw["modes"], kw["meas_pt"], 0.0, False, False, None, "double",
                  "fp32")
    info = plan(d, 2)
    dev = torch.device("cuda", 0)
    ws = torch.empty(int(info.workspace_bytes), dtype=torch.uint8, device=dev)
    srf = torch.from_numpy(kw["srf_flx"]).to(dev)
    c = torch.empty((2, info.out_ny, info.out_nx), dtype=torch.float64, device=dev)
    f = torch.empty_like(c)
    st = lib.bldfm_solve(d, ctypes.c_void_p(srf.data_ptr()), _lib.ptr(z), _lib.ptr(prof), _lib.ptr(lv), 2,
                         ctypes.c_void_p(c.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                         ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()), None)
    assert st == _lib.OK  # enqueued; the device status comes with the results
    torch.cuda.synchronize()
    assert int(ws[:4].view(torch.int32)[0]) == _lib.ERR_NONFINITE
    # the batched path: the bad case among good ones fails the batch
    good = _kw(np.random.default_rng(2).random((48, 64)))
    with pytest.raises(FloatingPointError, match="non-finite"):
        solve_batch([good, kw, good], solver=BatchSolver(use_graph=False))
    res = solve_batch([good, good], solver=BatchSolver(use_graph=False))
    assert np.all(np.isfinite(res[0][2]))
