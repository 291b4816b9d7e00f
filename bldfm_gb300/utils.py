"""Helpers of the reference's src/bldfm/utils.py.

``compute_wind_fields`` (utils.py:7-27) and ``ideal_source`` (utils.py:30-77)
produce solver inputs on the host, as in the reference.  ``point_measurement``
(utils.py:80-92) is the footprint-weighted sum: on host arrays it is the
reference's numpy sum; ``point_measurement_batch`` takes device tensors of
many (footprint, flux) pairs, e.g. a met timeseries, and reduces them on the
GPU in one launch (``bldfm_point_measurement``, FP64, deterministic).
"""

import ctypes

import numpy as np


def compute_wind_fields(u_rot, wind_dir):
    wind_dir = np.deg2rad(wind_dir)
    return -u_rot * np.sin(wind_dir), -u_rot * np.cos(wind_dir)


def ideal_source(nxy, domain, src_loc=None, shape="diamond"):
    nx, ny = nxy
    xmx, ymx = domain
    dx = xmx / nx
    if src_loc is None:
        src_loc = (xmx / 2, ymx / 2)
    xs, ys = src_loc
    X, Y = np.meshgrid(np.linspace(0.0, xmx, nx), np.linspace(0.0, ymx, ny))
    q0 = np.zeros([ny, nx])
    if shape == "diamond":
        q0 = np.where(np.abs(X - xs) + np.abs(Y - ys) < xmx / 12, 1.0, 0.0)
    if shape == "circle":
        q0 = np.where(np.sqrt((X - xs) ** 2 + (Y - ys) ** 2) < xmx / 12, 1.0, 0.0)
    if shape == "point":
        sig = 4.0 * dx
        q0 = np.exp(-((X - xs) ** 2 + (Y - ys) ** 2) / 2.0 / sig**2) / sig / np.sqrt(2.0 * np.pi)
    return q0


def point_measurement(f, g):
    """np.sum(f * g) (utils.py:80-92); device tensors go to the GPU reduction."""
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(f, torch.Tensor) and f.is_cuda:
        return float(point_measurement_batch(f.reshape(1, -1), g.reshape(1, -1))[0])
    return np.sum(f * g)


def point_measurement_batch(F, G):
    """sum over all but the first axis of F * G for CUDA float64 tensors of
    equal shape (B, ...); returns a (B,) device tensor."""
    import torch

    from . import _lib

    if F.shape != G.shape or F.dim() < 1:
        raise ValueError("F and G must have the same shape (B, ...)")
    F = F.to(torch.float64).reshape(F.shape[0], -1).contiguous()
    G = G.to(torch.float64).reshape(G.shape[0], -1).contiguous()
    B, n = F.shape
    lib = _lib.load()
    need = int(lib.bldfm_point_measurement_workspace(n, B))
    ws = torch.empty(max(need // 8, 1), dtype=torch.float64, device=F.device)
    out = torch.empty(B, dtype=torch.float64, device=F.device)
    st = lib.bldfm_point_measurement(
        ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(G.data_ptr()), n, n, B, ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel() * 8),
        ctypes.c_void_p(torch.cuda.current_stream(F.device).cuda_stream),
    )
    _lib.check(st, "point_measurement")
    return out
