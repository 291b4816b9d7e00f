"""Drop-in replacement of the reference's ``steady_state_transport_solver``.

Reference: src/bldfm/solver.py:16-304.  Same signature, argument meaning,
return convention ``(grid, conc, flx)``, output dtypes and error behaviour; the
work runs on the GPU through the C ABI (include/bldfm_gb300.h).

Swap it in by import (``from bldfm_gb300.solver import
steady_state_transport_solver``) or by assigning it to
``bldfm.solver.steady_state_transport_solver`` and
``bldfm.interface.steady_state_transport_solver``.
"""

import threading

import numpy as np

from . import _lib

_MODES = {"fp64": _lib.MODE_FP64, "fp32": _lib.MODE_FP32, "fp64r": _lib.MODE_FP64R}


def _normalise_levels(levels, nz):
    """Reference semantics: a scalar becomes a 1-element array (solver.py:102-105);
    ``z[levels]`` must index (solver.py:295), so non-integer or out-of-range
    levels raise IndexError as numpy does."""
    if np.ndim(levels) == 0:
        levels = np.array([levels])
    arr = np.asarray(levels)
    if arr.size == 0:
        raise ValueError("levels must not be empty")
    if arr.dtype.kind not in "iu":
        raise IndexError("arrays used as indices must be of integer (or boolean) type")
    lv = arr.astype(np.int64).ravel()
    bad = (lv < -nz) | (lv >= nz)
    if np.any(bad):
        raise IndexError("index %d is out of bounds for axis 0 with size %d" % (int(lv[bad][0]), nz))
    return levels, np.ascontiguousarray(lv)


_GRID_CACHE = {}


def output_grid(z, levels, shape, domain):
    """The reference's output grid (solver.py:292-297), squeezed like the
    reference's, as read-only arrays shared between calls with the same
    levels, shape and domain (building three fresh (ny, nx) arrays costs
    more host time than an FP32 solve)."""
    # one level (an integer): its height is the key, without indexing z
    zk = float(z[levels]) if isinstance(levels, (int, np.integer)) else np.asarray(z)[levels].tobytes()
    key = (zk, tuple(shape), tuple(domain))
    g = _GRID_CACHE.get(key)
    if g is None:
        zl = np.asarray(z)[levels]
        ny, nx = shape
        x = np.linspace(0, domain[0], nx, endpoint=False)
        y = np.linspace(0, domain[1], ny, endpoint=False)
        Z, Y, X = np.meshgrid(zl, y, x, indexing="ij")
        g = tuple(np.squeeze(a) for a in (X, Y, Z))
        for a in g:
            a.flags.writeable = False
        if len(_GRID_CACHE) > 64:
            _GRID_CACHE.clear()
        _GRID_CACHE[key] = g
    return g


_FP32_SOLVERS = {}  # (device index, check) -> one-case batch solver of the FP32 drop-in calls
_FP32_LOCK = threading.Lock()


def _solve_fp32_one(kw, check):
    """One FP32 solve through the batched path: cached plan and descriptors,
    the case's host data in one pinned upload, graph replay while the shapes
    repeat, outputs back in one copy into pinned memory.  Returns the result
    and, with ``check``, its estimated relative L2 error against the exact
    FP64 solution (the device accuracy check), else None."""
    import torch

    from .batch import BatchSolver, _enqueue_batch, _finish_batch

    dev = torch.cuda.current_device()
    with _FP32_LOCK:
        s = _FP32_SOLVERS.get((dev, check))
        if s is None:
            s = _FP32_SOLVERS[(dev, check)] = BatchSolver(device=dev, use_graph=True, check=check)
        res = _finish_batch(_enqueue_batch(s, [kw]))
        return res[0], (float(res.error_estimates[0]) if check else None)


def make_desc(shape, nz, domain, modes, meas_pt, srf_bg_conc, footprint, analytic, halo, precision, mode):
    ny, nx = shape
    nlx, nly = modes
    d = _lib.Desc()
    d.nx, d.ny, d.nz = int(nx), int(ny), int(nz)
    d.nlx, d.nly = int(nlx), int(nly)
    d.footprint = 1 if footprint else 0
    d.analytic = 1 if analytic else 0
    if precision == "single":
        d.precision = _lib.PREC_SINGLE
    elif precision == "double":
        d.precision = _lib.PREC_DOUBLE
    else:
        d.precision = 99  # rejected by the library with the reference's message
    d.mode = _MODES[mode]
    d.has_halo = 0 if halo is None else 1
    d.halo = 0.0 if halo is None else float(halo)
    d.xmax, d.ymax = float(domain[0]), float(domain[1])
    d.meas_x, d.meas_y = float(meas_pt[0]), float(meas_pt[1])
    d.srf_bg_conc = float(np.real(srf_bg_conc))
    return d


def plan(desc, nlvls):
    """Derived sizes of a solve (bldfm_plan)."""
    lib = _lib.load()
    info = _lib.PlanInfo()
    _lib.check(lib.bldfm_plan(desc, int(nlvls), info), "plan")
    return info


def steady_state_transport_solver(
    srf_flx,
    z,
    profiles,
    domain,
    levels,
    modes=(512, 512),
    meas_pt=(0.0, 0.0),
    srf_bg_conc=0.0,
    footprint=False,
    analytic=False,
    halo=None,
    precision="single",
    cache=None,
    *,
    mode="fp64",
    return_error=False,
):
    """Steady-state advection-diffusion solve on the GPU (solver.py:16-304).

    Parameters are the reference's.  The keyword-only ``mode`` selects the
    sweep: ``"fp64"`` (default) integrates the reference's shooting method with
    the reference's rounding; ``"fp32"`` integrates the same discrete problem
    with the FP32 invariant-imbedding sweep (relative L2 about 1e-6 against
    the exact discrete solution), through the batched path as a batch of one;
    ``"fp64r"`` is the invariant imbedding in FP64.  The grid arrays are
    shared, read-only arrays (the same values and shapes as the reference's).
    ``cache`` is a Green's-function cache with the reference's ``get``/``put``
    interface (src/bldfm/cache.py:19-83), consulted in footprint mode only;
    results of ``mode`` "fp32"/"fp64r" are stored under their own key and only
    in caches that support it (bldfm_gb300.cache.GreensFunctionCache).
    Raises ``ValueError`` for invalid profiles (non-finite values, z not
    strictly increasing, Kz <= 0) and ``FloatingPointError`` when the output
    holds non-finite values (the reference returns such fields silently).
    ``return_error=True`` (keyword-only) appends the result's error statement:
    in mode "fp32" the relative L2 error against the exact FP64 solution of
    the same discrete problem, estimated on the device from 32 modes re-solved
    in FP64 (float); in the FP64 modes None (the result is the FP64 solution
    itself).
    """
    if mode not in _MODES:
        raise ValueError("mode must be 'fp64', 'fp32' or 'fp64r'")
    from .cache import cache_args

    use_cache, ckw = cache_args(cache if footprint else None, mode)
    if use_cache:
        cached = cache.get(z, profiles, domain, modes, meas_pt, halo, precision, **ckw)
        if cached is not None:
            return (*cached, None) if return_error else cached
    lib = _lib.load()
    shape = np.shape(srf_flx)
    if len(shape) != 2:
        raise ValueError("srf_flx must be a 2D array")
    if mode == "fp32" and not analytic:
        if (modes[0] % 2) or (modes[1] % 2):
            raise ValueError("modes must consist of even numbers.")
        if precision not in ("single", "double"):
            raise ValueError("precision must be single (default) or double.")
        # the device accuracy check runs when the caller asks for the error
        result, err = _solve_fp32_one(dict(srf_flx=srf_flx, z=z, profiles=profiles, domain=domain, levels=levels,
                                           modes=modes, meas_pt=meas_pt, srf_bg_conc=srf_bg_conc,
                                           footprint=footprint, halo=halo, precision=precision), bool(return_error))
        if use_cache:
            cache.put(z, profiles, domain, modes, meas_pt, halo, precision, *result, **ckw)
        return (*result, err) if return_error else result
    zz = np.ascontiguousarray(z, dtype=np.float64)
    nz = zz.shape[0]
    prof = np.ascontiguousarray(np.stack([np.broadcast_to(np.asarray(p, dtype=np.float64), (nz,)) for p in profiles]))
    levels, lv = _normalise_levels(levels, nz)
    d = make_desc(shape, nz, domain, modes, meas_pt, srf_bg_conc, footprint, analytic, halo, precision, mode)
    info = _lib.PlanInfo()
    _lib.check(lib.bldfm_plan(d, int(lv.size), info), "steady_state_transport_solver")
    conc = np.empty((lv.size, info.out_ny, info.out_nx), dtype=np.float64)
    flx = np.empty_like(conc)
    src = None if footprint else np.ascontiguousarray(srf_flx, dtype=np.float64)
    st = lib.bldfm_solve_host(
        d, _lib.ptr(src), _lib.ptr(zz), _lib.ptr(prof), _lib.ptr(lv), int(lv.size), _lib.ptr(conc), _lib.ptr(flx)
    )
    _lib.check(st, "steady_state_transport_solver")

    xm, ym = meas_pt
    # output dtype rule: complex64 spectra stay complex64 unless the complex128
    # phase shift multiplied them (solver.py:177-188, 253-262)
    if precision == "single" and not footprint and not (xm**2 + ym**2 > 0.0):
        conc = conc.astype(np.float32)
        flx = flx.astype(np.float32)
    grid = output_grid(zz, levels, shape, domain)
    result = (grid, np.squeeze(conc), np.squeeze(flx))
    if use_cache:
        cache.put(z, profiles, domain, modes, meas_pt, halo, precision, *result, **ckw)
    return (*result, None) if return_error else result
