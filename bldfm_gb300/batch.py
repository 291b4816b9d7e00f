"""Batched FP32 solves on the GPU: many towers x timesteps in one launch.

The reference solves one case per Python call and parallelises over cases
with a process pool (src/bldfm/interface.py:141-326).  Here a batch of cases,
each with its own grid, modes, levels and profiles, goes to the C ABI entry
point ``bldfm_solve_batch``: one persistent sweep launch over every
(case, mode tile), one launch per transform pass, replayed as a CUDA graph
when the batch topology repeats (e.g. a met timeseries on fixed towers).

``solve_batch(cases)`` takes a list of keyword-argument dicts of
``steady_state_transport_solver`` and returns the list of ``(grid, conc, flx)``
tuples; ``solve_stream(batches)`` does the same for a sequence of batches
with the host work of one batch overlapping the GPU work of the previous.
``BatchSolver`` keeps workspace and device outputs between batches.

Every result states its error: the returned lists are ``BatchResults`` whose
``error_estimates`` hold, per case, the relative L2 error of the FP32 result
against the exact solution of the same discrete problem: the device
re-solves a stratified sample of 32 modes per case (the k = 0 mode, the 12
modes with |kx|, |ky| <= 2 and 19 equal slices of the mode list) in
float-float arithmetic at every output level, and the output transform's
rounding is added (``error_estimate``).
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .solver import _normalise_levels, make_desc, output_grid, plan


def _count(shape):
    """Number of elements of a (nlvls, ny, nx) output shape."""
    n = 1
    for v in shape:
        n *= int(v)
    return n


_INT_LEVELS = {}  # one integer output level -> (int64 array, its address, index array), read-only


def _int_level(level):
    """The shared read-only index arrays of one integer output level."""
    key = int(level)
    hit = _INT_LEVELS.get(key)
    if hit is None:
        lv = np.array([key], dtype=np.int64)
        idx = np.array([level])
        lv.flags.writeable = False
        idx.flags.writeable = False
        if len(_INT_LEVELS) > 4096:
            _INT_LEVELS.clear()
        hit = (lv, lv.ctypes.data, idx)
        _INT_LEVELS[key] = hit
    return hit


def _host_inputs(kw):
    """A case's host inputs as the library reads them: ``zp`` = z followed by
    the five profiles (u, v, Kx, Ky, Kz), nz float64 values each, in one
    array; the output levels as given (an index array for the grid) and as
    int64 with its address.  Returns (zp, nz, levels, lv, lv_address)."""
    z, p = kw["z"], kw["profiles"]
    nz = len(z)
    zp = None
    try:  # five length-nz profiles: one conversion for the six arrays
        if len(p) == 5:
            zp = np.concatenate((z, *p), dtype=np.float64)
    except (ValueError, TypeError):
        zp = None
    if zp is None or zp.shape != (6 * nz,):  # scalars broadcast over the levels
        zz = np.ascontiguousarray(z, dtype=np.float64).ravel()
        prof = np.stack([np.broadcast_to(np.asarray(a, dtype=np.float64), (nz,)) for a in p])
        zp = np.concatenate((zz, prof.ravel()))
    levels = kw["levels"]
    if isinstance(levels, (int, np.integer)) and -nz <= int(levels) < nz:
        lv, lvp, levels = _int_level(levels)
    else:
        levels, lv = _normalise_levels(levels, nz)
        lvp = lv.ctypes.data
    return zp, nz, levels, lv, lvp


# rounding of the FP32 output transform, per unit of the field it transforms:
# one FP32 ulp (the transform carries conc + i flux as one complex field, so
# each part's rounding scales with the norm of both)
XFORM_ROUNDING = 2.0**-24


def error_estimate(sums):
    """Relative L2 error estimate of one case from the accuracy check's sums
    (sum |dXp|^2, sum |Xp|^2, sum |dXq|^2, sum |Xq|^2, weighted over the
    sampled modes and the output levels): for the concentration and the flux
    spectra, the measured sweep error sqrt(sum |dX|^2 / sum |X|^2) combined
    with the output transform's rounding, XFORM_ROUNDING times the combined
    norm over the field's own, sqrt((|Xp|^2 + |Xq|^2) / |X|^2); the larger
    of the two fields'."""
    dp, p, dq, q = (float(v) for v in sums)
    tot = p + q
    ep = (dp / p + XFORM_ROUNDING**2 * tot / p) ** 0.5 if p > 0 else 0.0
    eq = (dq / q + XFORM_ROUNDING**2 * tot / q) ** 0.5 if q > 0 else 0.0
    return max(ep, eq)


def error_estimates(sums):
    """``error_estimate`` of every row of an (n, 4) array of check sums."""
    a = np.asarray(sums, dtype=np.float64).reshape(-1, 4)
    dp, p, dq, q = a[:, 0], a[:, 1], a[:, 2], a[:, 3]
    tot = p + q
    u2 = XFORM_ROUNDING**2
    with np.errstate(divide="ignore", invalid="ignore"):
        ep = np.where(p > 0, np.sqrt((dp + u2 * tot) / np.where(p > 0, p, 1.0)), 0.0)
        eq = np.where(q > 0, np.sqrt((dq + u2 * tot) / np.where(q > 0, q, 1.0)), 0.0)
    return np.maximum(ep, eq)


class BatchResults(list):
    """A list of ``(grid, conc, flx)`` results with ``error_estimates``: per
    case, the estimated relative L2 error against the exact FP64 solution
    (None when the solver ran without the accuracy check), computed from the
    device check's sums when first read."""

    _sums = None
    _est = None

    @property
    def error_estimates(self):
        if self._est is None and self._sums is not None:
            self._est = error_estimates(self._sums)
        return self._est

    @error_estimates.setter
    def error_estimates(self, v):
        self._est = v


class BatchSolver:
    """Solve batches of FP32 cases with persistent device buffers.

    ``solve(cases)`` enqueues a batch on ``self.stream`` and returns device
    tensors ``(conc, flx)`` per case, shape (nlvls, out_ny, out_nx).  Buffers
    are reused while the batch shape repeats.
    """

    def __init__(self, device=None, threads=0, ctas_per_sm=0, use_graph=True, xform_lines=0, check=True):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.stream = torch.cuda.Stream(device=self.device)
        self.check = bool(check)  # the device accuracy check (error statement of every result)
        self.opts = _lib.BatchOpts(threads=int(threads), ctas_per_sm=int(ctas_per_sm), use_graph=int(use_graph),
                                   xform_lines=int(xform_lines), skip_check=int(not check))
        self._ws = None
        self._out_buf = None  # one device buffer holding every case's conc and flx
        self._srf = {}
        self._keep = None

    def _srf_dev(self, k, srf):
        a = np.ascontiguousarray(srf, dtype=np.float64)
        t = self._srf.get(k)
        if t is None or tuple(t.shape) != a.shape:
            t = torch.empty(a.shape, dtype=torch.float64, device=self.device)
            self._srf[k] = t
        with torch.cuda.stream(self.stream):
            t.copy_(torch.from_numpy(a).pin_memory(), non_blocking=True)
        return t

    def prepare(self, cases, views=True):
        """Build the C descriptors of a batch; returns (array, outputs, keepalive).

        views=False skips the torch views of the outputs (outputs is then the
        list of (nlvls, out_ny, out_nx) shapes; the results sit back to back,
        conc then flx per case, at the start of the solver's output buffer)."""
        n = len(cases)
        arr = (_lib.Case * n)()
        outs, keep = [], []
        metas = []
        for kw in cases:
            zp, nz, levels, lv, lvp = _host_inputs(kw)
            get = kw.get
            bg = get("srf_bg_conc", 0.0)
            if type(bg) is not float:
                bg = float(np.real(bg))
            key = (np.shape(kw["srf_flx"]), nz, tuple(kw["domain"]), tuple(get("modes", (512, 512))),
                   tuple(get("meas_pt", (0.0, 0.0))), bg, bool(get("footprint", False)), get("halo"),
                   get("precision", "single"), lv.size)
            hit = _DESC_CACHE.get(key)
            if hit is None:
                d = make_desc(
                    np.shape(kw["srf_flx"]), nz, kw["domain"], get("modes", (512, 512)), get("meas_pt", (0.0, 0.0)),
                    get("srf_bg_conc", 0.0), bool(get("footprint", False)), False, get("halo"),
                    get("precision", "single"), "fp32",
                )
                info = plan(d, lv.size)
                shape = (lv.size, info.out_ny, info.out_nx)
                hit = (d, shape, _count(shape), bool(d.footprint))
                if len(_DESC_CACHE) > 256:
                    _DESC_CACHE.clear()
                _DESC_CACHE[key] = hit
            metas.append((hit, zp, nz, levels, lv, lvp))
        total = 2 * sum(m[0][2] for m in metas)
        if self._out_buf is None or self._out_buf.numel() < total:
            if self._out_buf is not None:  # an earlier batch on the stream may still use it
                self.stream.synchronize()
            self._out_buf = torch.empty(total, dtype=torch.float64, device=self.device)
        self.out_elems = total
        base = self._out_buf.data_ptr()
        off = 0
        for k, ((d, shape, sz, footprint), zp, nz, levels, lv, lvp) in enumerate(metas):
            c = arr[k]
            c.desc = d
            if not footprint:
                c.srf_flx_dev = self._srf_dev(k, cases[k]["srf_flx"]).data_ptr()
            zptr = zp.ctypes.data
            c.z_host = zptr
            c.prof_host = zptr + 8 * nz
            c.levels_host = lvp
            c.nlvls = lv.size
            c.conc_dev = base + 8 * off
            c.flx_dev = base + 8 * (off + sz)
            if views:
                ob = self._out_buf
                outs.append((ob[off : off + sz].view(shape), ob[off + sz : off + 2 * sz].view(shape)))
            else:
                outs.append(shape)
            off += 2 * sz
            keep.append((zp, nz, lv, levels))
        return arr, outs, keep

    def solve(self, cases):
        """Enqueue a batch given as keyword-argument dicts; returns device outputs."""
        return self.solve_prepared(self.prepare(cases))

    def solve_prepared(self, prepared):
        """Enqueue a batch whose C descriptors were built by :meth:`prepare`
        (reusable across calls: the library reads the host arrays at every
        call, so refreshing their contents in place needs no new descriptors)."""
        lib = _lib.load()
        arr, outs, keep = prepared[:3]
        n = len(arr)

        def run():
            return lib.bldfm_solve_batch(
                arr, n, self.opts, ctypes.c_void_p(self._ws.data_ptr()), ctypes.c_size_t(self._ws.numel()),
                ctypes.c_void_p(self.stream.cuda_stream),
            )

        # with a workspace in place, solve first: the library checks the size
        # before it touches the stream, so a batch that needs more returns
        # ERR_WORKSPACE with nothing enqueued and is planned and retried
        st = _lib.ERR_WORKSPACE
        if self._ws is not None and (len(prepared) <= 3 or self._ws.numel() >= prepared[3]):
            st = run()
        if st == _lib.ERR_WORKSPACE:
            if len(prepared) > 3:
                need = prepared[3]
            else:
                nb = ctypes.c_int64(0)
                _lib.check(lib.bldfm_batch_plan(arr, n, self.opts, ctypes.byref(nb)), "solve_batch")
                need = int(nb.value)
            if self._ws is None or self._ws.numel() < need:
                if self._ws is not None:  # an earlier batch on the stream may still use it
                    self.stream.synchronize()
                self._ws = torch.empty(int(need), dtype=torch.uint8, device=self.device)
            st = run()
        _lib.check(st, "solve_batch")
        self._keep = keep
        return outs

    def prepare_cached(self, cases):
        """:meth:`prepare` plus the workspace size, for repeated solves."""
        lib = _lib.load()
        arr, outs, keep = self.prepare(cases)
        need = ctypes.c_int64(0)
        _lib.check(lib.bldfm_batch_plan(arr, len(cases), self.opts, ctypes.byref(need)), "solve_batch")
        return (arr, outs, keep, int(need.value))

    def status(self):
        """Device status word of the last batch (0, or a BLDFM_ERR_* code),
        read through this solver's stream only (no device-wide sync)."""
        if self._ws is None:
            return 0
        st = torch.empty(1, dtype=torch.int32, pin_memory=True)
        with torch.cuda.stream(self.stream):
            st.copy_(self._ws[:4].view(torch.int32), non_blocking=True)
        self.stream.synchronize()
        return int(st[0])

    def error_estimates(self, n):
        """Estimated relative L2 error of each of the last batch's n cases
        against the exact FP64 solution (the device accuracy check's sums at
        byte 64 of the workspace), read through this solver's stream."""
        if self._ws is None:
            return np.zeros(0)
        h = torch.empty(16 * n, dtype=torch.uint8, pin_memory=True)
        with torch.cuda.stream(self.stream):
            h.copy_(self._ws[64 : 64 + 16 * n], non_blocking=True)
        self.stream.synchronize()
        return error_estimates(h.view(torch.float32).numpy())


_DESC_CACHE = {}  # descriptor and output shape per case geometry
_grid = output_grid


def _enqueue_batch(solver, cases):
    """Enqueue a batch and the copy of its outputs and of the workspace head
    (status word, the check's sums) into one fresh pinned host buffer on the
    solver's stream; returns the pending state."""
    shapes = solver.solve_prepared(solver.prepare(cases, views=False))
    nout = 8 * solver.out_elems
    nhead = 64 + 16 * len(cases)
    block = torch.empty(nout + nhead, dtype=torch.uint8, pin_memory=True)
    host = block[:nout].view(torch.float64)
    head = block[nout:]
    lib = _lib.load()
    s = ctypes.c_void_p(solver.stream.cuda_stream)
    base = block.data_ptr()
    _lib.check(lib.bldfm_memcpy_async(ctypes.c_void_p(base), ctypes.c_void_p(solver._out_buf.data_ptr()), nout, s),
               "solve_batch")
    _lib.check(lib.bldfm_memcpy_async(ctypes.c_void_p(base + nout), ctypes.c_void_p(solver._ws.data_ptr()), nhead,
                                      s), "solve_batch")
    return (solver, cases, shapes, solver._keep, host, head)


def _finish_batch(pending):
    """Wait for an enqueued batch and build its (grid, conc, flx) results."""
    solver, cases, shapes, keep, host, head = pending
    solver.stream.synchronize()
    hd = head.numpy()
    st = int(hd[:4].view(np.int32)[0])
    if st != 0:
        _lib.check(st, "solve_batch")
    hn = host.numpy()
    results = BatchResults()
    n = len(cases)
    if getattr(solver, "check", True):
        results._sums = hd[64 : 64 + 16 * n].view(np.float32).reshape(n, 4).copy()
    if n and all(sh == shapes[0] for sh in shapes):  # one geometry: views of one reshaped array
        sq = tuple(v for v in shapes[0] if v != 1)
        hv = hn[: 2 * n * _count(shapes[0])].reshape((n, 2) + sq)
        pairs = [(hv[k, 0, ...], hv[k, 1, ...]) for k in range(n)]
    else:
        pairs, off = [], 0
        for shape in shapes:
            sz = _count(shape)
            pairs.append((np.squeeze(hn[off : off + sz].reshape(shape)),
                          np.squeeze(hn[off + sz : off + 2 * sz].reshape(shape))))
            off += 2 * sz
    for kw, (zp, nz, _, levels), (conc, flx) in zip(cases, keep, pairs):
        footprint = bool(kw.get("footprint", False))
        if kw.get("precision", "single") == "single" and not footprint:
            xm, ym = kw.get("meas_pt", (0.0, 0.0))
            if not (xm**2 + ym**2 > 0.0):
                conc, flx = conc.astype(np.float32), flx.astype(np.float32)
        grid = _grid(zp[:nz], levels, np.shape(kw["srf_flx"]), kw["domain"])
        results.append((grid, conc, flx))
    return results


STREAM_BYTES = 1 << 30  # output bytes in flight solve_stream's default depth allows
STREAM_DEPTH = 8  # most batches in flight by default


def stream_depth(cases):
    """Default number of solvers (batches in flight) of ``solve_stream`` for
    batches like ``cases``: eight, fewer when eight batches' FP64 outputs
    (conc and flux, device and pinned host copies) would exceed ~1 GiB, at
    least two.  Measured on the 16-footprint 512^2 batch, end to end: 29.9k
    footprints/s with four batches in flight, 30.9k with six and 31.2k with
    eight (the device-resident rate is 31.4k): the copy back and the host
    work of the oldest batches need more than three batches of kernels
    queued behind them to stay hidden."""
    per = 0
    for kw in cases:
        ny, nx = np.shape(kw["srf_flx"])[-2:]
        lv = kw.get("levels", 0)
        nl = 1 if np.ndim(lv) == 0 else max(1, int(np.size(lv)))
        per += 16 * int(ny) * int(nx) * nl
    return int(max(2, min(STREAM_DEPTH, STREAM_BYTES // max(per, 1))))


def solve_stream(batches, *, solvers=None, **opts):
    """Solve an iterable of batches (each a list of keyword-argument dicts of
    ``steady_state_transport_solver``) in FP32, yielding each batch's list of
    ``(grid, conc, flx)`` in order.  The solvers (each with its own stream,
    workspace and outputs; by default ``stream_depth`` of the first batch,
    created as they are first needed) take the batches in turn: batch i is
    prepared and enqueued before batch i - len(solvers) + 1 is waited for, so
    the host work, the kernels and the copies back of up to len(solvers)
    batches overlap (with two, the copy back and the host work of a batch sit
    in the latency the next batch has to hide).  ``opts`` go to the default
    BatchSolvers."""
    from collections import deque

    solvers = list(solvers) if solvers else None
    pending = deque()
    for i, cases in enumerate(batches):
        if solvers is None:
            solvers = [None] * stream_depth(cases)
        ns = len(solvers)
        if solvers[i % ns] is None:
            solvers[i % ns] = BatchSolver(**opts)
        pending.append(_enqueue_batch(solvers[i % ns], cases))
        if len(pending) == ns:
            yield _finish_batch(pending.popleft())
    while pending:
        yield _finish_batch(pending.popleft())


def solve_batch(cases, *, solver=None):
    """Solve a list of cases (keyword-argument dicts of
    ``steady_state_transport_solver``) in FP32 on the GPU; returns a list of
    ``(grid, conc, flx)`` with the single-case function's shapes and dtypes.
    All outputs come back in one device-to-host copy into a fresh pinned
    buffer that the returned arrays view; the grid arrays are shared
    read-only arrays."""
    solver = solver or BatchSolver()
    return _finish_batch(_enqueue_batch(solver, cases))
