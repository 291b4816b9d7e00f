"""Vertical profiles on the GPU (reference: src/bldfm/pbl_model.py:8-204).

``vertical_profiles`` has the reference's signature and returns host numpy
arrays ``z, (u, v, Kx, Ky, Kz)``; the per-level evaluation (log-stretched grid,
Businger-Dyer psi/phi, closures MOST, CONSTANT, MOSTM, OAAHOC) runs in the
CUDA library.  Results agree with the reference to about 1e-15 relative
(different libm); the FP64 solver is exact for whatever profiles it is given.
"""

import ctypes

import numpy as np
import torch

from . import _lib


def _params(n, meas_height, wind, ustar=None, z0=None, mol=1e9, prsc=1.0, closure="MOST", domain_height=None,
            stretch=None, z0_min=0.001, z0_max=2.0, tke=None):
    """Checked C arguments of one evaluation (the reference's argument rules)."""
    if closure not in _lib.CLOSURES:
        raise ValueError(
            f"Invalid closure type: {closure}. " "Supported closures are 'MOST', 'CONSTANT', and 'OAAHOC'."
        )
    if closure != "OAAHOC":
        if (z0 is None) == (ustar is None):
            if z0 is not None:
                raise ValueError("Either z0 or ustar must be provided.")
    um, vm = wind
    return (
        int(n),
        float(meas_height),
        float(um),
        float(vm),
        float(ustar) if ustar is not None else -1.0,
        float(z0) if (z0 is not None and closure != "OAAHOC") else -1.0,
        float(mol),
        float(prsc),
        _lib.CLOSURES[closure],
        float(domain_height) if domain_height is not None else -1.0,
        float(stretch) if stretch is not None else -1.0,
        float(np.ravel(tke)[0]) if tke is not None else -1.0,
    )


def vertical_profiles_batch(cases):
    """``vertical_profiles`` for a list of keyword-argument dicts in one device
    launch and one copy back; returns the list of ``(z, profiles)``."""
    lib = _lib.load()
    n = len(cases)
    if n == 0:
        return []
    arr = (_lib.ProfileParams * n)()
    for k, kw in enumerate(cases):
        a = _params(**kw)
        p = arr[k]
        (p.n, p.meas_height, p.um, p.vm, p.ustar, p.z0, p.mol, p.prsc, p.closure, p.domain_height, p.stretch,
         p.tke) = a
    nz = np.zeros(n, dtype=np.int32)
    zoff = np.zeros(n, dtype=np.int64)
    need = ctypes.c_size_t(0)
    _lib.check(lib.bldfm_vertical_profiles_batch(n, ctypes.addressof(arr), nz.ctypes.data, zoff.ctypes.data,
                                                 ctypes.byref(need), None, None, None, 0, None),
               "vertical_profiles")
    total = int(zoff[-1] + nz[-1])
    dev = torch.device("cuda", torch.cuda.current_device())
    buf = torch.empty(6 * total, dtype=torch.float64, device=dev)  # z, then the profile rows
    ws = torch.empty(max(int(need.value), 16), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(lib.bldfm_vertical_profiles_batch(n, ctypes.addressof(arr), nz.ctypes.data, zoff.ctypes.data,
                                                 ctypes.byref(need), ctypes.c_void_p(buf.data_ptr()),
                                                 ctypes.c_void_p(buf.data_ptr() + 8 * total),
                                                 ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                                 ctypes.c_void_p(stream)),
               "vertical_profiles")
    host = buf.cpu().numpy()
    zs, ps = host[:total], host[total:]
    out = []
    for k in range(n):
        o, m = int(zoff[k]), int(nz[k])
        z = zs[o:o + m].copy()
        rows = ps[5 * o:5 * (o + m)].reshape(5, m)
        out.append((z, tuple(rows[i].copy() for i in range(5))))
    return out


def vertical_profiles(
    n,
    meas_height,
    wind,
    ustar=None,
    z0=None,
    mol=1e9,
    prsc=1.0,
    closure="MOST",
    domain_height=None,
    stretch=None,
    z0_min=0.001,
    z0_max=2.0,
    tke=None,
):
    if closure not in _lib.CLOSURES:
        raise ValueError(
            f"Invalid closure type: {closure}. " "Supported closures are 'MOST', 'CONSTANT', and 'OAAHOC'."
        )
    if closure != "OAAHOC":
        if (z0 is None) == (ustar is None):
            # the reference derives z0 when it is None, else ustar, else raises
            if z0 is not None:
                raise ValueError("Either z0 or ustar must be provided.")
    lib = _lib.load()
    um, vm = wind
    args = (
        int(n),
        float(meas_height),
        float(um),
        float(vm),
        float(ustar) if ustar is not None else -1.0,
        float(z0) if (z0 is not None and closure != "OAAHOC") else -1.0,
        float(mol),
        float(prsc),
        _lib.CLOSURES[closure],
        float(domain_height) if domain_height is not None else -1.0,
        float(stretch) if stretch is not None else -1.0,
        float(np.ravel(tke)[0]) if tke is not None else -1.0,
    )
    nz = ctypes.c_int32(0)
    _lib.check(lib.bldfm_vertical_profiles(*args, ctypes.byref(nz), None, None, None), "vertical_profiles")
    dev = torch.device("cuda", torch.cuda.current_device())
    zd = torch.empty(nz.value, dtype=torch.float64, device=dev)
    pd = torch.empty((5, nz.value), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(
        lib.bldfm_vertical_profiles(
            *args, ctypes.byref(nz), ctypes.c_void_p(zd.data_ptr()), ctypes.c_void_p(pd.data_ptr()),
            ctypes.c_void_p(stream)
        ),
        "vertical_profiles",
    )
    z = zd.cpu().numpy()
    p = pd.cpu().numpy()
    u, v, Kx, Ky, Kz = (p[i].copy() for i in range(5))
    return z, (u, v, Kx, Ky, Kz)
