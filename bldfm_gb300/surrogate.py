"""Learned surrogate of the per-mode sweep, with the FP64 solver as fallback.

Footprint mode with MOST profiles (reference: ``steady_state_transport_solver``,
src/bldfm/solver.py:16-304, fed by ``vertical_profiles``,
src/bldfm/pbl_model.py:8-204).  Per Fourier mode the solver's transfer from the
surface to z_m depends only on the rotated, z_m-scaled wavenumbers and on
s1 = z_m / L, s2 = ln(z_m / z0) (plus the level count n, default stretch and
top).  A 8 -> 4 x 256 GELU -> 4 MLP (``mlp.MLP``, tcgen05 BF16 GEMMs with FP32
accumulation) learns that transfer from data the FP32 invariant-imbedding
sweep generates on the device (``TransferPool``), trained with Adam
(``train``); ``Surrogate`` serves footprints through it inside the training
box and through the FP64 solver outside it.  The footprint's lowest
wavenumbers, |k| z_m < ``exact_kz`` (default 4), where its L2 norm and almost
all of the network's error sit, take the exact FP32 sweep instead of the
network (about 1% of the modes of the production footprint, 11% of the
benchmark's 512^2 one).  Every served case of a batch is
checked by the library's accuracy guard: a stratified sample of modes (the
k = 0 mode, the lowest wavenumbers, every 61st solved mode) is re-solved
exactly (FP32 sweep) on the device and compared with the served spectrum,
which estimates the case's relative L2 error; cases whose estimate exceeds
``guard_tol`` (the network's guard factor times ``tol``) are re-solved by the
FP32 solver.  Every ``spot_every``-th case
is also re-solved in full by the FP64 solver, returning the solver's result
when the surrogate's relative L2 error exceeds ``tol``.

The reference solve of a spot check and the fallback are the accurate FP64
mode (``mode="fp64r"``: the same discrete problem solved without the
shooting method's cancellation), because the reference-rounding FP64 result
itself carries an error of order eps e^{2G} in high-|k| modes that exceeds
1e-3 for tall towers on fine grids (on the production footprint, 1024^2
modes and 413 levels, it is ~2e9 away from the exact solution).
``fallback="fp64"`` returns the reference-rounding result instead, which
reproduces the reference's own output bit for bit.
"""

import ctypes
import json
import math
import os

import numpy as np
import torch

from . import _lib
from .mlp import MLP
from .pbl_model import vertical_profiles
from .solver import make_desc, steady_state_transport_solver

KAPPA = 0.4
# serving box: s1 = z_m / L, s2 = ln(z_m / z0), |k| z_m, levels below z_m;
# the network is trained on TRAIN_BOX, which has a margin around it
BOX = {"s1": (-1.0, 0.25), "s2": (4.5, 7.5), "kmin": 1e-3, "kmax": 40.0, "n": 128}
TRAIN_BOX = {"s1": (-1.25, 0.35), "s2": (4.25, 7.75), "kmin": 1e-3, "kmax": 40.0, "n": 128}
WEIGHT_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")
WEIGHTS = os.path.join(WEIGHT_DIR, "surrogate_n128.npz")
# the network of the production footprint's level count (n = 256, 413 levels;
# |k| z_m up to 48 covers all modes of a 1024^2 extended grid at dx = 1.95 m
# and z_m = 20 m)
WEIGHTS_N256 = os.path.join(WEIGHT_DIR, "surrogate_n256.npz")
# |k| z_m below which the served modes are solved exactly (a network's box may
# set its own "exact_kz").  On the production footprint this band holds 1.2% of
# the modes and 97% (flux) to 99.7% (concentration) of the network's squared
# L2 error: the exact band divides the error by ~6 for ~1% of an FP32 solve.
EXACT_KZ = 4.0


def boxes(n=128, kmax=40.0):
    """(serving box, training box) of a network for n levels below z_m and
    |k| z_m <= kmax: the training box keeps the margin in s1 and s2."""
    return dict(BOX, n=int(n), kmax=float(kmax)), dict(TRAIN_BOX, n=int(n), kmax=float(kmax))


def psi(x):
    """Businger-Dyer integrated stability function (pbl_model.py:207-230)."""
    if x > 0:
        return 5.0 * x
    xi = (1.0 - 16.0 * x) ** 0.25
    return -2.0 * math.log(0.5 * (1 + xi)) - math.log(0.5 * (1 + xi * xi)) + 2.0 * math.atan(xi) - 0.5 * math.pi


def met_scalars(zm, wind, ustar=None, z0=None, mol=1e9):
    """(U, s1, s2, s3): wind speed at z_m, z_m / L, ln(z_m / z0), u* / U, with
    z0 or u* following from the other as in vertical_profiles (pbl_model.py:68-78)."""
    U = math.hypot(float(wind[0]), float(wind[1]))
    s1 = zm / mol
    if z0 is None:
        s2 = KAPPA * U / ustar - psi(zm / mol)
    else:
        s2 = math.log(zm / z0)
    s3 = KAPPA / (s2 + psi(s1))
    return U, s1, s2, s3


def mode_kmax(srf_shape, domain, modes, halo=None):
    """Largest |k| (1/m) of the solved modes (the solver's grid, solver.py:110-140)."""
    ny, nx = srf_shape
    dx, dy = domain[0] / nx, domain[1] / ny
    h = max(domain) if halo is None else halo
    nxe, nye = nx + 2 * int(h / dx), ny + 2 * int(h / dy)
    nlx, nly = modes
    if nlx > nxe or nly > nye:
        nlx, nly = nxe, nye
    return math.hypot(2 * math.pi / dx / nxe * (nlx // 2), 2 * math.pi / dy / nye * (nly // 2))


class TransferPool:
    """Nondimensional MOST met cases on the device (bldfm_transfer_pool_*)."""

    def __init__(self, ncases=16384, seed=0, box=TRAIN_BOX, s1=None, s2=None):
        self.lib = _lib.load()
        self.box = dict(box)
        rng = np.random.default_rng(seed)
        self.s1 = np.ascontiguousarray(rng.uniform(*box["s1"], ncases) if s1 is None else s1, dtype=np.float64)
        self.s2 = np.ascontiguousarray(rng.uniform(*box["s2"], ncases) if s2 is None else s2, dtype=np.float64)
        self.ncases = self.s1.size
        h = ctypes.c_void_p()
        _lib.check(
            self.lib.bldfm_transfer_pool_create(
                _lib.ptr(self.s1), _lib.ptr(self.s2), self.ncases, int(box["n"]), ctypes.byref(h)
            ),
            "transfer_pool_create",
        )
        self.h = h
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.norm = None

    def close(self):
        if self.h:
            self.lib.bldfm_transfer_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def buffers(self, m):
        f = dict(dtype=torch.float32, device=self.device)
        return torch.empty((m, 8), **f), torch.empty((m, 4), **f), torch.empty((m, 4), **f)

    def samples(self, seed, m, X, T, W, norm=None, floor=1e-3, cid=None, stream=None):
        s = (stream or torch.cuda.current_stream()).cuda_stream
        _lib.check(
            self.lib.bldfm_transfer_samples(
                self.h, int(seed) & (2**64 - 1), int(m), float(self.box["kmin"]), float(self.box["kmax"]),
                ctypes.c_void_p(norm.data_ptr()) if norm is not None else None, float(floor),
                ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(W.data_ptr()),
                ctypes.c_void_p(cid.data_ptr()) if cid is not None else None, ctypes.c_void_p(s),
            ),
            "transfer_samples",
        )

    def eval(self, cid, kpar, kperp):
        """Targets (m, 4) for device tensors of case ids and wavenumbers."""
        m = cid.numel()
        T = torch.empty((m, 4), dtype=torch.float32, device=self.device)
        s = torch.cuda.current_stream().cuda_stream
        _lib.check(
            self.lib.bldfm_transfer_eval(
                self.h, ctypes.c_void_p(cid.data_ptr()), ctypes.c_void_p(kpar.data_ptr()),
                ctypes.c_void_p(kperp.data_ptr()), ctypes.c_void_p(T.data_ptr()), m, ctypes.c_void_p(s),
            ),
            "transfer_eval",
        )
        return T

    def energies(self, per_case=2048, seed=12345):
        """Per-case reciprocals (1/Eq, 1/Ep) of the flux and concentration
        spectral energies, from per_case * ncases raw samples."""
        m = per_case * self.ncases
        chunk = 1 << 22
        eq = torch.zeros(self.ncases, dtype=torch.float64, device=self.device)
        ep = torch.zeros_like(eq)
        cnt = torch.zeros_like(eq)
        X, T, W = self.buffers(min(m, chunk))
        cid = torch.empty(min(m, chunk), dtype=torch.int32, device=self.device)
        for k, off in enumerate(range(0, m, chunk)):
            n = min(chunk, m - off)
            self.samples(seed + 7919 * k, n, X, T, W, cid=cid)
            c = cid[:n].long()
            eq.index_add_(0, c, W[:n, 0].double())
            ep.index_add_(0, c, W[:n, 2].double())
            cnt.index_add_(0, c, torch.ones(n, dtype=torch.float64, device=self.device))
        eq = eq / cnt.clamp(min=1)
        ep = ep / cnt.clamp(min=1)
        self.norm = torch.stack([1.0 / eq, 1.0 / ep], 1).float().contiguous()
        return self.norm


def train(net, pool, steps, batch=65536, lr=1e-3, lr_final=1e-5, decay_from=0.3, seed=1, floor=1e-3,
          log_every=100, callback=None, conc_weight=1.0):
    """Adam on fresh device-generated samples every step; the learning rate
    stays at ``lr`` for the first ``decay_from`` of the steps, then decays on a
    cosine to ``lr_final``.  ``conc_weight`` scales the concentration part of
    the loss against the flux part.  Returns [(step, loss)] every
    ``log_every`` steps."""
    norm = pool.norm if pool.norm is not None else pool.energies()
    norm = norm * torch.tensor([1.0, float(conc_weight)], device=norm.device)
    X, T, W = pool.buffers(batch)
    hist = []
    for it in range(steps):
        f = it / max(steps - 1, 1)
        if f < decay_from:
            lr_t = lr
        else:
            g = (f - decay_from) / max(1.0 - decay_from, 1e-9)
            lr_t = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * g))
        pool.samples(seed * 1000003 + it, batch, X, T, W, norm=norm, floor=floor)
        net.train_step(X, T, W, lr_t)
        if (it + 1) % log_every == 0 or it + 1 == steps:
            _, loss = net.grads()
            hist.append((it + 1, loss))
            if callback:
                callback(it + 1, loss)
    return hist


def validation_loss(net, pool, m=65536, seed=999, floor=1e-3):
    """Weighted loss of the network on fresh samples (no update)."""
    norm = pool.norm if pool.norm is not None else pool.energies()
    X, T, W = pool.buffers(m)
    pool.samples(seed, m, X, T, W, norm=norm, floor=floor)
    net.train_step(X, T, W, 0.0)
    return net.grads()[1]


def save(net, path, meta=None, box=None):
    """Save the parameters with the serving box they hold for (default BOX)."""
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez(path, params=net.params(), box=json.dumps(BOX if box is None else box), meta=json.dumps(meta or {}))


def load(path=WEIGHTS, batch=65536):
    """MLP with saved parameters, and the box and metadata it was trained with."""
    d = np.load(path)
    net = MLP(batch=batch, seed=0)
    net.set_params(d["params"])
    return net, json.loads(str(d["box"])), json.loads(str(d["meta"]))


def _rell2(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


class Surrogate:
    """Footprints at z_m through the MLP, with the FP64 solver as fallback.

    ``footprint(...)`` takes the met case as ``vertical_profiles`` does and the
    footprint grid as ``steady_state_transport_solver`` does, and returns
    ``(grid, conc, flx)`` like the solver.  ``stats`` counts the cases served
    by the network, out-of-box fallbacks, spot checks and their failures.
    """

    def __init__(self, net=None, box=None, spot_every=64, tol=1e-3, variant=0, spot_mode="fp64r", fallback="fp64r",
                 guard_tol=None, guard_mode="fp32", exact_kz=None):
        self.lib = _lib.load()
        self.net = net
        self.box = dict(BOX if box is None else box)
        self.spot_every = int(spot_every)
        self.tol = float(tol)
        self.variant = int(variant)  # 0 fused kernel, 1 exact transfer (check), 2 layer by layer
        self.spot_mode = spot_mode
        self.fallback = fallback
        # the guard's estimate is the sampled spectral error over the extended
        # grid; its ratio to the true error of the cropped fields depends on
        # the network and the grid, so the network's box carries a safety
        # factor (guard_factor, default 1): cases whose estimate exceeds
        # guard_tol = guard_factor * tol are re-solved.  Measured with the
        # exact low band (errors 0.8e-4 to 1.3e-4): n = 128 network on 512^2
        # footprints 0.9 to 2.0 (factor 1); n = 256 network on the production
        # footprint 1.05 to 2.1, median 1.3 (factor 0.5, set when the network
        # served every mode: 0.77 to 2.4, one case near 0.6)
        factor = float(self.box.get("guard_factor", 1.0))
        self.guard_tol = self.tol * factor if guard_tol is None else float(guard_tol)
        self.guard_mode = guard_mode
        # |k| z_m of the exact low band (0: every mode from the network)
        self.exact_kz = float(self.box.get("exact_kz", EXACT_KZ) if exact_kz is None else exact_kz)
        self.device = torch.device("cuda", torch.cuda.current_device())
        self._ws = None
        self._out = None
        self.count = 0
        self.served = 0
        self.stats = {"surrogate": 0, "out_of_box": 0, "spot": 0, "spot_fail": 0, "errors": [], "guard": [],
                      "guard_fail": 0, "spot_guard": []}

    def in_box(self, n, zm, s1, s2, kmax):
        b = self.box
        return (
            n == b["n"]
            and b["s1"][0] <= s1 <= b["s1"][1]
            and b["s2"][0] <= s2 <= b["s2"][1]
            and zm * kmax <= b["kmax"]
        )

    def prepare(self, n, zm, wind, srf_shape, domain, modes=(512, 512), meas_pt=(0.0, 0.0), halo=None,
                ustar=None, z0=None, mol=1e9):
        """Host inputs of one surrogate solve (reusable across calls)."""
        z, prof = vertical_profiles(n, zm, wind, ustar=ustar, z0=z0, mol=mol)
        z = np.ascontiguousarray(z, dtype=np.float64)
        prof = np.ascontiguousarray(np.stack([np.broadcast_to(np.asarray(p, dtype=np.float64), z.shape) for p in prof]))
        U, s1, s2, s3 = met_scalars(zm, wind, ustar, z0, mol)
        d = make_desc(srf_shape, z.size, domain, modes, meas_pt, 0.0, True, False, halo, "single", "fp32")
        info = _lib.PlanInfo()
        _lib.check(self.lib.bldfm_plan(d, 1, info), "surrogate")
        met = _lib.SurrogateCase(zm=float(z[n]), wind=U, s1=s1, s2=s2, s3=s3, variant=self.variant,
                                 exact_kz=self.exact_kz)
        lv = np.array([n], dtype=np.int64)
        need = ctypes.c_int64(0)
        _lib.check(self.lib.bldfm_surrogate_plan(d, 1, ctypes.byref(need)), "surrogate")
        return {"desc": d, "met": met, "z": z, "prof": prof, "lv": lv, "shape": (info.out_ny, info.out_nx),
                "need": int(need.value), "s": (s1, s2, s3), "zm": zm,
                "kw": dict(srf_flx=np.zeros(srf_shape), z=z, profiles=tuple(prof), domain=domain, levels=n,
                           modes=modes, meas_pt=meas_pt, footprint=True, halo=halo)}

    def solve_prepared(self, p, conc=None, flx=None, stream=None):
        """Enqueue one surrogate solve; returns device (conc, flx) of shape (out_ny, out_nx)."""
        if self._ws is None or self._ws.numel() < p["need"]:
            self._ws = torch.empty(p["need"], dtype=torch.uint8, device=self.device)
        if conc is None:
            sz = p["shape"][0] * p["shape"][1]
            if self._out is None or self._out.numel() < 2 * sz:
                self._out = torch.empty(2 * sz, dtype=torch.float64, device=self.device)
            conc = self._out[:sz].view(p["shape"])
            flx = self._out[sz : 2 * sz].view(p["shape"])
        s = (stream or torch.cuda.current_stream()).cuda_stream
        st = self.lib.bldfm_surrogate_solve(
            self.net.h if self.net is not None else None, p["desc"], p["met"], _lib.ptr(p["z"]), _lib.ptr(p["prof"]),
            _lib.ptr(p["lv"]), 1, ctypes.c_void_p(conc.data_ptr()), ctypes.c_void_p(flx.data_ptr()),
            ctypes.c_void_p(self._ws.data_ptr()), ctypes.c_size_t(self._ws.numel()), ctypes.c_void_p(s),
        )
        _lib.check(st, "surrogate_solve")
        return conc, flx

    def prepare_batch(self, items):
        """Descriptors of a batch of footprints (keyword dicts of ``prepare``),
        reusable across calls; outputs are views of one device buffer."""
        preps = [self.prepare(**kw) for kw in items]
        n = len(preps)
        arr = (_lib.Case * n)()
        mets = (_lib.SurrogateCase * n)()
        sizes = [p["shape"][0] * p["shape"][1] for p in preps]
        out = torch.empty(2 * sum(sizes), dtype=torch.float64, device=self.device)
        outs, off = [], 0
        for k, p in enumerate(preps):
            sz = sizes[k]
            conc = out[off : off + sz].view(p["shape"])
            flx = out[off + sz : off + 2 * sz].view(p["shape"])
            off += 2 * sz
            c = arr[k]
            c.desc = p["desc"]
            c.srf_flx_dev = None
            c.z_host = p["z"].ctypes.data
            c.prof_host = p["prof"].ctypes.data
            c.levels_host = p["lv"].ctypes.data
            c.nlvls = 1
            c.conc_dev = conc.data_ptr()
            c.flx_dev = flx.data_ptr()
            mets[k] = p["met"]
            mets[k].variant = 0
            outs.append((conc, flx))
        need = ctypes.c_int64(0)
        _lib.check(self.lib.bldfm_surrogate_batch_plan(arr, mets, n, ctypes.byref(need)), "surrogate_batch")
        return {"arr": arr, "mets": mets, "outs": outs, "out": out, "keep": preps, "need": int(need.value), "n": n}

    def solve_batch_prepared(self, b, stream=None):
        """Enqueue a prepared batch (one fused launch + the batched output
        transform); returns the list of device (conc, flx)."""
        if self._ws is None or self._ws.numel() < b["need"]:
            self._ws = torch.empty(b["need"], dtype=torch.uint8, device=self.device)
        s = (stream or torch.cuda.current_stream()).cuda_stream
        st = self.lib.bldfm_surrogate_solve_batch(
            self.net.h, b["arr"], b["mets"], b["n"], ctypes.c_void_p(self._ws.data_ptr()),
            ctypes.c_size_t(self._ws.numel()), ctypes.c_void_p(s),
        )
        _lib.check(st, "surrogate_solve_batch")
        return b["outs"]

    def guard_estimates(self, b, stream=None):
        """Per-case relative L2 error estimates of the last solve of prepared
        batch b from the library's accuracy guard (sampled spectra against
        the exact FP32 sweep): max over p and q of sqrt(sum |dX|^2 / sum |X|^2)."""
        n = b["n"]
        gb = (16 * n + 255) & ~255
        off = b["need"] - gb
        s = stream or torch.cuda.current_stream(self.device)
        host = torch.empty(4 * n, dtype=torch.float32, pin_memory=True)
        with torch.cuda.stream(s):
            host.copy_(self._ws[off : off + 16 * n].view(torch.float32), non_blocking=True)
        s.synchronize()
        a = host.numpy().reshape(n, 4).astype(np.float64)
        tiny = 1e-300
        return np.sqrt(np.maximum(a[:, 0] / np.maximum(a[:, 1], tiny), a[:, 2] / np.maximum(a[:, 3], tiny)))

    def status(self, stream=None):
        """Device status word of the last launch (0, or a BLDFM_ERR_* code),
        read through the launch stream (default: the current stream)."""
        if self._ws is None:
            return 0
        s = stream or torch.cuda.current_stream(self.device)
        st = torch.empty(1, dtype=torch.int32, pin_memory=True)
        with torch.cuda.stream(s):
            st.copy_(self._ws[:4].view(torch.int32), non_blocking=True)
        s.synchronize()
        return int(st[0])

    def classify(self, kw):
        """True when the case (keyword dict of ``prepare``) lies in the training box."""
        _, s1, s2, _ = met_scalars(kw["zm"], kw["wind"], kw.get("ustar"), kw.get("z0"), kw.get("mol", 1e9))
        km = mode_kmax(kw["srf_shape"], kw["domain"], kw.get("modes", (512, 512)), kw.get("halo"))
        return self.in_box(kw["n"], kw["zm"], s1, s2, km)

    def serve(self, items, batch=16, keep=None, return_errors=False):
        """Footprints of a met timeseries (keyword dicts of ``prepare``):
        in-box cases through the network in batched fused launches, every
        ``spot_every``-th footprint the network serves (the guard passed it)
        also through the ``spot_mode`` solve (the FP64 result is kept when
        the surrogate misses ``tol``), out-of-box
        cases through the fallback solver; a served case whose guard estimate
        exceeds ``guard_tol`` is re-solved by ``guard_mode``.  Returns
        (outputs, paths): outputs[k] = (conc, flx) (device tensors for served
        cases, host arrays for solver results), paths[k] in "surrogate",
        "fp32-guard", "fp64-spot", "fp64-box".  ``keep``: indices whose
        outputs are returned (default all); the others are computed, checked
        and dropped (outputs[k] = None), so a long timeseries does not hold
        every footprint in memory.  ``return_errors``: also return each
        step's error statement, the estimated relative L2 error against the
        exact solution: the guard's estimate for a served footprint, the FP32
        path's own statement for a guard re-solve, None for an FP64 result
        (the FP64 solution itself, as the drop-in states it), and the measured
        error for a served footprint that a spot check compared."""
        out, paths = [None] * len(items), [None] * len(items)
        errs = [None] * len(items)
        kept = None if keep is None else set(keep)
        inbox = []
        for k, kw in enumerate(items):
            if self.classify(kw):
                inbox.append(k)
            else:
                self.stats["out_of_box"] += 1
                p = self.prepare(**kw)
                _, c, f = steady_state_transport_solver(**p["kw"], mode=self.fallback)
                out[k], paths[k] = ((c, f) if kept is None or k in kept else None), "fp64-box"
        for i in range(0, len(inbox), batch):
            ks = inbox[i : i + batch]
            b = self.prepare_batch([items[k] for k in ks])
            res = self.solve_batch_prepared(b)
            est = self.guard_estimates(b)
            for k, pr, (c, f), e in zip(ks, b["keep"], res, est):
                self.count += 1
                self.stats["surrogate"] += 1
                self.stats["guard"].append(float(e))
                out[k], paths[k] = (c, f), "surrogate"
                errs[k] = float(e)
                if not e <= self.guard_tol:
                    self.stats["guard_fail"] += 1
                    res = steady_state_transport_solver(**pr["kw"], mode=self.guard_mode, return_error=True)
                    out[k], paths[k], errs[k] = (res[1], res[2]), "fp32-guard", res[3]
                    continue
                # spot checks count the footprints the network serves (those
                # the guard passed): the re-solved ones are exact already
                self.served += 1
                if self.spot_every > 0 and self.served % self.spot_every == 0:
                    ref = steady_state_transport_solver(**pr["kw"], mode=self.spot_mode)
                    ca, fa = c.cpu().numpy(), f.cpu().numpy()
                    err = max(_rell2(ca, ref[1]), _rell2(fa, ref[2]))
                    self.stats["spot"] += 1
                    self.stats["errors"].append(err)
                    self.stats["spot_guard"].append(float(e))
                    if err > self.tol:
                        self.stats["spot_fail"] += 1
                        if self.fallback != self.spot_mode:
                            ref = steady_state_transport_solver(**pr["kw"], mode=self.fallback)
                        out[k], paths[k], errs[k] = (ref[1], ref[2]), "fp64-spot", None
                    else:
                        errs[k] = err  # measured: the spot check's exact solve
            if kept is not None:
                for k in ks:
                    if k not in kept:
                        out[k] = None
        return (out, paths, errs) if return_errors else (out, paths)

    def footprint(self, n, zm, wind, srf_shape, domain, modes=(512, 512), meas_pt=(0.0, 0.0), halo=None,
                  ustar=None, z0=None, mol=1e9, return_error=False):
        """One footprint at z_m: (grid, conc, flx) as the solver returns them,
        and the path that produced it ("surrogate", "fp32-guard", "fp64-box",
        "fp64-spot").  With the fused kernel (variant 0) the footprint goes
        through the batched path as a batch of one, so it gets the exact low
        band and the accuracy guard, and a footprint whose estimate exceeds
        ``guard_tol`` is re-solved by ``guard_mode``.  ``return_error``: also
        return its error statement (as ``serve`` states it: the guard's
        estimate, the FP32 path's statement after a guard re-solve, the
        measured error after a spot check, None for an FP64 result)."""
        p = self.prepare(n, zm, wind, srf_shape, domain, modes, meas_pt, halo, ustar, z0, mol)
        s1, s2, _ = p["s"]
        self.count += 1

        def ret(res, path, err):
            return (res, path, err) if return_error else (res, path)

        if not (self.variant == 1 or self.in_box(n, zm, s1, s2, mode_kmax(srf_shape, domain, modes, halo))):
            self.stats["out_of_box"] += 1
            return ret(steady_state_transport_solver(**p["kw"], mode=self.fallback), "fp64-box", None)
        stated = None
        if self.variant == 0 and self.net is not None:
            kw = dict(n=n, zm=zm, wind=wind, srf_shape=srf_shape, domain=domain, modes=modes, meas_pt=meas_pt,
                      halo=halo, ustar=ustar, z0=z0, mol=mol)
            b = self.prepare_batch([kw])
            (conc_d, flx_d), = self.solve_batch_prepared(b)
            stated = float(self.guard_estimates(b)[0])
            self.stats["guard"].append(stated)
            if not stated <= self.guard_tol:
                self.stats["guard_fail"] += 1
                res = steady_state_transport_solver(**p["kw"], mode=self.guard_mode, return_error=True)
                return ret(tuple(res[:3]), "fp32-guard", res[3])
        else:
            conc_d, flx_d = self.solve_prepared(p)
        conc, flx = conc_d.cpu().numpy(), flx_d.cpu().numpy()
        grid = _grid(p["z"], n, srf_shape, domain)
        self.stats["surrogate"] += 1
        if self.spot_every > 0 and self.count % self.spot_every == 0:
            ref = steady_state_transport_solver(**p["kw"], mode=self.spot_mode)
            err = max(_rell2(conc, ref[1]), _rell2(flx, ref[2]))
            self.stats["spot"] += 1
            self.stats["errors"].append(err)
            if err > self.tol:
                self.stats["spot_fail"] += 1
                if self.fallback != self.spot_mode:
                    ref = steady_state_transport_solver(**p["kw"], mode=self.fallback)
                return ret(ref, "fp64-spot", None)
            stated = err
        return ret((grid, conc, flx), "surrogate", stated)


def _grid(z, level, shape, domain):
    ny, nx = shape
    x = np.linspace(0, domain[0], nx, endpoint=False)
    y = np.linspace(0, domain[1], ny, endpoint=False)
    Z, Y, X = np.meshgrid(np.asarray(z)[[level]], y, x, indexing="ij")
    return tuple(np.squeeze(a) for a in (X, Y, Z))


def _main(argv=None):
    """python -m bldfm_gb300.surrogate train [--steps N] [--n LEVELS]
    [--kmax K] [--out PATH]: train the network on the GPU from
    solver-generated transfer functions for n levels below z_m and
    |k| z_m <= K, and save it with its serving box (the shipped weights were
    made this way: n = 128, K = 40, 300k steps; n = 256, K = 48)."""
    import argparse
    import time

    ap = argparse.ArgumentParser(prog="python -m bldfm_gb300.surrogate")
    ap.add_argument("command", choices=["train"])
    ap.add_argument("--steps", type=int, default=100000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--cases", type=int, default=16384)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=None)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--kmax", type=float, default=40.0)
    ap.add_argument("--conc-weight", type=float, default=1.0)
    a = ap.parse_args(argv)
    serve_box, train_box = boxes(a.n, a.kmax)
    out = a.out or os.path.join(WEIGHT_DIR, "surrogate_n%d.npz" % a.n)
    pool = TransferPool(ncases=a.cases, seed=0, box=train_box)
    net = MLP(batch=a.batch, seed=a.seed)
    t0 = time.time()
    hist = train(net, pool, a.steps, batch=a.batch, lr=a.lr, seed=a.seed, log_every=max(a.steps // 50, 1),
                 conc_weight=a.conc_weight,
                 callback=lambda i, l: print("step %d loss %.3e (%.0f s)" % (i, l, time.time() - t0), flush=True))
    torch.cuda.synchronize()
    dt = time.time() - t0
    val = validation_loss(net, pool)
    save(net, out, {"steps": a.steps, "batch": a.batch, "lr": a.lr, "cases": a.cases, "seed": a.seed,
                    "conc_weight": a.conc_weight,
                    "train_s": dt, "val_loss": float(val), "train_box": train_box, "history": hist[-10:]},
         box=serve_box)
    print("saved %s: validation loss %.3e, %.1f s" % (out, val, dt))


if __name__ == "__main__":
    _main()
