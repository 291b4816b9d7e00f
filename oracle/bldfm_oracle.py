"""CPU oracle for the BLDFM steady-state transport solve -- test infrastructure.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its cpu_baseline
leg and its ``--impl reference`` arm) may import this module, and only as the
test oracle or the timed CPU baseline.  The GPU product path never imports it.

This is a restatement of the reference algorithm in numpy, written so that
every floating-point operation of the reference's numpy evaluation happens in
the same order (see ``sweep_port.c`` for the rounding model).  Functions and the
reference lines they follow:

* :func:`steady_state_transport_solver` -- src/bldfm/solver.py:16-304
* :func:`ivp_sweep_numpy` -- src/bldfm/solver.py:307-374 (``ivp_solver``)
* :func:`shooting_dd_sweep` -- src/bldfm/solver.py:220-235 and 307-374 in
  double-double arithmetic (the extended-precision yardstick)
* :func:`vertical_profiles` -- src/bldfm/pbl_model.py:8-204
* :func:`psi`, :func:`phi` -- src/bldfm/pbl_model.py:207-250
* :func:`compute_wind_fields` -- src/bldfm/utils.py:7-27
* :func:`ideal_source` -- src/bldfm/utils.py:30-77
* :func:`point_measurement` -- src/bldfm/utils.py:80-92

Parity pin: tests/test_oracle_golden.py checks this oracle against the five
regression fixtures the reference ships (tests/references/*.npz) and against
fixtures generated by running the reference itself (tests/golden/).
"""

import ctypes
import os

import numpy as np
from numpy.fft import fftfreq, fftshift, ifftshift

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libbldfm_oracle.so")
_lib = None

# level-table columns, identical to the enum in sweep_port.c
LV_STRIDE = 12


def load_port():
    """Load the C port of the sweep (built by oracle/Makefile), or None."""
    global _lib
    if _lib is None and os.path.exists(_LIB_PATH):
        lib = ctypes.CDLL(_LIB_PATH)
        lib.oracle_sweep.restype = ctypes.c_int
        lib.oracle_sweep.argtypes = [
            ctypes.c_int64,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_double,
            ctypes.c_int,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_int,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_int,
        ]
        lib.oracle_csqrt.restype = None
        lib.oracle_csqrt.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_sweep_dd.restype = ctypes.c_int
        lib.oracle_sweep_dd.argtypes = [
            ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
        ]
        _lib = lib
    return _lib


# ---------------------------------------------------------------------------
# helpers shared with the sweep
# ---------------------------------------------------------------------------


def snapshot_schedule(levels, nz):
    """Map sweep steps to output slots the way the reference fills them.

    The reference snapshots inside ``for i in range(nz-1): if i in levels``
    and once more after the loop for ``nz-1`` (solver.py:350-372), bumping the
    slot counter once per matching step.  So slot s holds the s-th smallest
    distinct level in [0, nz-1]; duplicate or out-of-range levels leave the
    trailing slots empty (zero).
    """
    lv = np.atleast_1d(np.asarray(levels))
    slot = np.full(nz, -1, dtype=np.int32)
    s = 0
    for i in range(nz):
        if i in lv:
            slot[i] = s
            s += 1
    return slot, s


def level_table(z, profiles):
    """Per-step scalars of the reference's ivp_solver, rounded exactly as numpy does.

    Row i (step i -> i+1) holds Kx, Ky, u, v, 0.5*Kzinv, dz**2,
    1/6*Kzinv**2, dz**3, -Kzinv*dz, 1/6*Kzinv, dz (solver.py:357-364).
    """
    u, v, Kx, Ky, Kz = profiles
    nz = len(z)
    dz = np.diff(z)
    lv = np.zeros((max(nz - 1, 0), LV_STRIDE))
    for i in range(nz - 1):
        Kzinv = 1.0 / Kz[i]
        dzi = dz[i]
        lv[i, 0] = Kx[i]
        lv[i, 1] = Ky[i]
        lv[i, 2] = u[i]
        lv[i, 3] = v[i]
        lv[i, 4] = 0.5 * Kzinv
        lv[i, 5] = dzi**2
        lv[i, 6] = 1.0 / 6.0 * Kzinv**2
        lv[i, 7] = dzi**3
        lv[i, 8] = -Kzinv * dzi
        lv[i, 9] = 1.0 / 6.0 * Kzinv
        lv[i, 10] = dzi
    return lv


def ivp_sweep_numpy(p0, q0, profiles, z, levels, Lx, Ly):
    """Linear-shooting IVP sweep in numpy (solver.py:307-374).

    Returns (p_top, q_top, p_snap, q_snap) with snapshots (nlvls, nmodes).
    """
    u, v, Kx, Ky, Kz = profiles
    nz = len(z)
    dz = np.diff(z)
    slot, _ = snapshot_schedule(levels, nz)
    nlvls = len(np.atleast_1d(levels))
    p = np.array(p0, dtype=np.complex128)
    q = np.array(q0, dtype=np.complex128)
    ps = np.zeros((nlvls, p.shape[0]), dtype=np.complex128)
    qs = np.zeros_like(ps)
    for i in range(nz - 1):
        if slot[i] >= 0:
            ps[slot[i]] = p
            qs[slot[i]] = q
        T = -(Kx[i] * Lx**2 + Ky[i] * Ly**2) - 1j * u[i] * Lx - 1j * v[i] * Ly
        Kzinv = 1.0 / Kz[i]
        h = dz[i]
        a = 1.0 - 0.5 * Kzinv * T * h**2
        b = -Kzinv * h - 1.0 / 6.0 * Kzinv**2 * T * h**3
        c = T * h - 1.0 / 6.0 * Kzinv * T**2 * h**3
        p, q = a * p + b * q, c * p + a * q
    if nz >= 1 and slot[nz - 1] >= 0:
        ps[slot[nz - 1]] = p
        qs[slot[nz - 1]] = q
    return p, q, ps, qs


def riccati_sweep(Lx, Ly, q0, eigval, Kz_top, profiles, z, levels):
    """The same discrete boundary-value problem as the shooting sweep, solved by
    invariant imbedding in FP64 (no cancellation): R_i = p_i/q_i from the top
    radiation condition R_L = 1/(Kz_top eigval) downwards,
    R_i = (a R_{i+1} - b)/(a - c R_{i+1}), q_{i+1} = (c R_i + a) q_i.
    Returns (p, q) of shape (nlvls, nmodes)."""
    u, v, Kx, Ky, Kz = profiles
    nz = len(z)
    dz = np.diff(z)
    slot, nsnap = snapshot_schedule(levels, nz)
    nlvls = len(np.atleast_1d(levels))
    n = Lx.shape[0]
    R = 1.0 / (Kz_top * eigval)
    logQ = np.zeros(n, dtype=np.complex128)  # log of prod_{k >= i} f_k
    Rs = {}
    Ls = {}
    if slot[nz - 1] >= 0:
        Rs[nz - 1], Ls[nz - 1] = R.copy(), logQ.copy()
    for i in range(nz - 2, -1, -1):
        T = -(Kx[i] * Lx**2 + Ky[i] * Ly**2) - 1j * (u[i] * Lx + v[i] * Ly)
        k = 1.0 / Kz[i]
        h = dz[i]
        a = 1 - 0.5 * k * h * h * T
        b = -k * h - k * k * h**3 / 6.0 * T
        c = T * h - k * h**3 / 6.0 * T * T
        R = (a * R - b) / (a - c * R)
        logQ = logQ + np.log(c * R + a)
        if slot[i] >= 0:
            Rs[i], Ls[i] = R.copy(), logQ.copy()
    p = np.zeros((nlvls, n), dtype=np.complex128)
    q = np.zeros_like(p)
    for i, s in enumerate(slot):
        if s >= 0:
            # q_j = q0 prod_{k<j} f_k = q0 exp(logQ_0 - logQ_j)
            q[s] = q0 * np.exp(logQ - Ls[i])
            p[s] = Rs[i] * q[s]
    return p, q


def hermitian_split(nlx, nly):
    """Representatives of the masked modes under k -> -k.

    Masked modes are the (nly, nlx) fftfreq grid in row-major order without
    (0, 0), the order of the reference's ``Lx[msk]`` (solver.py:147-162).
    Returns (rep, src): ``rep`` indexes the modes to solve (no mirror in the
    grid, kx > 0, or kx = 0 and ky > 0); for every other mode ``src`` is the
    masked index of its mirror, whose transfer is the complex conjugate.
    """
    fx = np.rint(fftfreq(nlx, d=1.0 / nlx)).astype(np.int64)
    fy = np.rint(fftfreq(nly, d=1.0 / nly)).astype(np.int64)
    FX, FY = np.meshgrid(fx, fy)
    FX, FY = FX.ravel()[1:], FY.ravel()[1:]
    has = (-FX >= fx.min()) & (-FX <= fx.max()) & (-FY >= fy.min()) & (-FY <= fy.max())
    rep = ~has | (FX > 0) | ((FX == 0) & (FY > 0))
    mflat = (np.mod(-FY, nly) * nlx + np.mod(-FX, nlx)) - 1
    src = np.where(rep, -1, mflat)
    return np.nonzero(rep)[0], src


def shooting_dd_sweep(Lx, Ly, q0, eigval, profiles, z, levels, nlx, nly, nthreads=0):
    """The reference's shooting sweep and combination (solver.py:220-235,
    307-374) in double-double arithmetic (sweep_port.c: oracle_sweep_dd).

    Solves one mode of each Hermitian pair (the transfer of the mirror is the
    conjugate) and scales the per-unit-flux transfer by the source spectrum.
    Returns (p, q) of shape (nlvls, nmodes).
    """
    lib = load_port()
    if lib is None:
        raise RuntimeError("oracle C port not built (oracle/build_oracle.py)")
    nz = len(z)
    nlvls = len(np.atleast_1d(levels))
    slot, nsnap = snapshot_schedule(levels, nz)
    rep, src = hermitian_split(nlx, nly)
    lxr = np.ascontiguousarray(np.asarray(Lx, dtype=np.float64)[rep])
    lyr = np.ascontiguousarray(np.asarray(Ly, dtype=np.float64)[rep])
    eig = np.ascontiguousarray(np.asarray(eigval, dtype=np.complex128)[rep])
    zz = np.ascontiguousarray(z, dtype=np.float64)
    prof = np.ascontiguousarray(np.stack([np.asarray(a, dtype=np.float64) for a in profiles]))
    n = lxr.shape[0]
    ps = np.zeros((max(nsnap, 1), n), dtype=np.complex128)
    qs = np.zeros_like(ps)
    rc = lib.oracle_sweep_dd(n, lxr.ctypes.data, lyr.ctypes.data, eig.ctypes.data, nz, zz.ctypes.data,
                             prof.ctypes.data, slot.ctypes.data, nsnap, ps.ctypes.data, qs.ctypes.data,
                             int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle_sweep_dd failed")
    nm = np.asarray(Lx).shape[0]
    P = np.zeros((nlvls, nm), dtype=np.complex128)
    Q = np.zeros_like(P)
    P[:nsnap, rep] = ps[:nsnap]
    Q[:nsnap, rep] = qs[:nsnap]
    mir = np.nonzero(src >= 0)[0]
    P[:, mir] = np.conj(P[:, src[mir]])
    Q[:, mir] = np.conj(Q[:, src[mir]])
    q0 = np.asarray(q0, dtype=np.complex128)
    return P * q0, Q * q0


def shooting_sweep(Lx, Ly, q0, eigval, Kz_top, profiles, z, levels, nthreads=0, use_port=True):
    """Both IVPs plus the alpha combination; returns (p, q) of shape (nlvls, nmodes)."""
    nz = len(z)
    nlvls = len(np.atleast_1d(levels))
    lib = load_port() if use_port else None
    if lib is not None:
        slot, nsnap = snapshot_schedule(levels, nz)
        lv = np.ascontiguousarray(level_table(z, profiles))
        Lx = np.ascontiguousarray(Lx, dtype=np.float64)
        Ly = np.ascontiguousarray(Ly, dtype=np.float64)
        q0c = np.ascontiguousarray(q0, dtype=np.complex128)
        eig = np.ascontiguousarray(eigval, dtype=np.complex128)
        n = Lx.shape[0]
        p = np.zeros((nlvls, n), dtype=np.complex128)
        q = np.zeros((nlvls, n), dtype=np.complex128)
        ps = np.zeros((max(nsnap, 1), n), dtype=np.complex128)
        qs = np.zeros_like(ps)
        rc = lib.oracle_sweep(
            n,
            Lx.ctypes.data,
            Ly.ctypes.data,
            q0c.ctypes.data,
            eig.ctypes.data,
            float(Kz_top),
            nz,
            lv.ctypes.data,
            slot.ctypes.data,
            nsnap,
            ps.ctypes.data,
            qs.ctypes.data,
            int(nthreads),
        )
        if rc != 0:
            raise RuntimeError("oracle_sweep failed")
        p[:nsnap] = ps[:nsnap]
        q[:nsnap] = qs[:nsnap]
        return p, q
    one = np.ones(Lx.shape[0], dtype=np.complex128)
    zero = np.zeros(Lx.shape[0], dtype=np.complex128)
    p1, q1, pm1, qm1 = ivp_sweep_numpy(one, zero, profiles, z, levels, Lx, Ly)
    p2, q2, pm2, qm2 = ivp_sweep_numpy(zero, q0, profiles, z, levels, Lx, Ly)
    alpha = -(q2 - Kz_top * eigval * p2) / (q1 - Kz_top * eigval * p1)
    return alpha * pm1 + pm2, alpha * qm1 + qm2


# ---------------------------------------------------------------------------
# the solve
# ---------------------------------------------------------------------------


def solve_plan(srf_shape, z, domain, levels, modes, halo):
    """Grid bookkeeping of solver.py:94-131 (no arrays)."""
    ny, nx = srf_shape
    nlx, nly = modes
    xmx, ymx = domain
    if (nlx % 2 > 0) or (nly % 2 > 0):
        raise ValueError("modes must consist of even numbers.")
    dx, dy = xmx / nx, ymx / ny
    if halo is None:
        halo = max(xmx, ymx)
    px = int(halo / dx)
    py = int(halo / dy)
    nxe = nx + 2 * px
    nye = ny + 2 * py
    if (nlx > nxe) or (nly > nye):
        nlx, nly = nxe, nye
    dlx, dly = (nxe - nlx) // 2, (nye - nly) // 2
    return dict(
        nx=nx, ny=ny, nz=len(z), dx=dx, dy=dy, halo=halo, px=px, py=py,
        nxe=nxe, nye=nye, nlx=nlx, nly=nly, dlx=dlx, dly=dly,
    )


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
    nthreads=0,
    use_port=True,
    sweep="shooting",
):
    """Oracle restatement of the reference solve (solver.py:16-304).

    Same signature and return convention as the reference.  ``cache`` is
    accepted and ignored (the oracle never memoises).  ``sweep="riccati"``
    replaces the shooting sweep by :func:`riccati_sweep` (the exact solution of
    the same discrete problem, the yardstick of the accurate modes);
    ``sweep="shooting_dd"`` runs the reference's own shooting method in
    double-double arithmetic (:func:`shooting_dd_sweep`), an independent
    extended-precision evaluation of the same discrete problem.
    """
    q0 = np.asarray(srf_flx)
    p000 = srf_bg_conc
    u, v, Kx, Ky, Kz = profiles
    xmx, ymx = domain
    xm, ym = meas_pt
    if np.ndim(levels) == 0:
        levels = np.array([levels])
    nlvls = len(levels)

    pl = solve_plan(q0.shape, z, domain, levels, modes, halo)
    nz = pl["nz"]
    nx, ny, dx, dy = pl["nx"], pl["ny"], pl["dx"], pl["dy"]
    halo, px, py = pl["halo"], pl["px"], pl["py"]
    nxe, nye, nlx, nly = pl["nxe"], pl["nye"], pl["nlx"], pl["nly"]
    dlx, dly = pl["dlx"], pl["dly"]
    dz = np.diff(z)

    # source spectrum (solver.py:132-145)
    if footprint:
        tfftq0 = np.ones((nly, nlx), dtype=np.complex128) / nxe / nye
    else:
        q0p = np.pad(q0, ((py, py), (px, px)), mode="constant", constant_values=0.0)
        f = np.fft.fft2(q0p, norm="forward")
        f = fftshift(f)
        tfftq0 = ifftshift(f[dly : nye - dly, dlx : nxe - dlx])
        if tfftq0.shape != (nly, nlx):
            raise ValueError(
                "truncated source spectrum %s does not match modes %s"
                % (tfftq0.shape, (nly, nlx))
            )

    # wavenumbers (solver.py:147-162)
    ilx = fftfreq(nlx, d=1.0 / nlx)
    ily = fftfreq(nly, d=1.0 / nly)
    lx = 2.0 * np.pi / dx / nxe * ilx
    ly = 2.0 * np.pi / dy / nye * ily
    Lx, Ly = np.meshgrid(lx, ly)
    msk = np.ones((nly, nlx), dtype=bool)
    msk[0, 0] = False

    # top eigenvalue (solver.py:164-174)
    Kzinv = 1.0 / Kz[nz - 1]
    KxKzinv = Kx[nz - 1] * Kzinv
    KyKzinv = Ky[nz - 1] * Kzinv
    eigval = np.sqrt(
        KxKzinv * Lx[msk] ** 2
        + KyKzinv * Ly[msk] ** 2
        + 1j * u[nz - 1] * Kzinv * Lx[msk]
        + 1j * v[nz - 1] * Kzinv * Ly[msk]
    )

    if precision == "single":
        cdt = np.complex64
    elif precision == "double":
        cdt = np.complex128
    else:
        raise ValueError("precision must be single (default) or double.")
    tfftp = np.zeros((nlvls, nly, nlx), dtype=cdt)
    tfftq = np.zeros((nlvls, nly, nlx), dtype=cdt)
    tfftp[0, 0, 0] = p000
    tfftq[:, 0, 0] = tfftq0[0, 0]

    if analytic:
        # constant-profile closed form (solver.py:193-202)
        h = z[levels] - z[0]
        tfftp[0, msk] = tfftq0[msk] * Kzinv / eigval
        tfftp[:, 0, 0] = p000 - tfftq0[0, 0] * Kzinv * h
        tfftq[:, msk] = tfftq0[msk] * np.exp(-eigval * h)
        tfftp[:, msk] = tfftq[:, msk] * Kzinv / eigval
    else:
        if sweep == "riccati":
            pm, qm = riccati_sweep(Lx[msk], Ly[msk], tfftq0[msk], eigval, Kz[nz - 1], profiles, z, levels)
        elif sweep == "shooting_dd":
            pm, qm = shooting_dd_sweep(Lx[msk], Ly[msk], tfftq0[msk], eigval, profiles, z, levels, nlx, nly,
                                       nthreads=nthreads)
        elif sweep == "shooting":
            pm, qm = shooting_sweep(
                Lx[msk], Ly[msk], tfftq0[msk], eigval, Kz[nz - 1], profiles, z, levels,
                nthreads=nthreads, use_port=use_port,
            )
        else:
            raise ValueError("sweep must be 'shooting', 'shooting_dd' or 'riccati'")
        tfftp[:, msk] = pm
        tfftq[:, msk] = qm
        # k = 0 mode by the trapezoid rule (solver.py:237-251)
        slot, _ = snapshot_schedule(levels, nz)
        p00 = p000
        for i in range(nz - 1):
            if slot[i] >= 0:
                tfftp[slot[i], 0, 0] = p00
            p00 = p00 - tfftq0[0, 0] * dz[i] * (0.5 / Kz[i] + 0.5 / Kz[i + 1])
        if slot[nz - 1] >= 0:
            tfftp[slot[nz - 1], 0, 0] = p00

    # measurement-point phase shift (solver.py:253-262)
    if footprint:
        shift = np.exp(1j * (Lx * (xm + halo) + Ly * (ym + halo)))
        tfftp = tfftp * shift
        tfftq = tfftq * shift
    elif xm**2 + ym**2 > 0.0:
        shift = np.exp(1j * (Lx * (xm - xmx / 2) + Ly * (ym - ymx / 2)))
        tfftp = tfftp * shift
        tfftq = tfftq * shift

    # un-truncate and transform back (solver.py:264-287)
    pad = ((0, 0), (dly, dly), (dlx, dlx))
    fftp = ifftshift(np.pad(fftshift(tfftp, axes=(1, 2)), pad), axes=(1, 2))
    fftq = ifftshift(np.pad(fftshift(tfftq, axes=(1, 2)), pad), axes=(1, 2))
    if footprint:
        p = np.fft.fft2(fftp, norm="backward").real
        q = np.fft.fft2(fftq, norm="backward").real
    else:
        p = np.fft.ifft2(fftp, norm="forward").real
        q = np.fft.ifft2(fftq, norm="forward").real

    conc = p[:, py : nye - py, px : nxe - px]
    flx = q[:, py : nye - py, px : nxe - px]
    x = np.linspace(0, xmx, nx, endpoint=False)
    y = np.linspace(0, ymx, ny, endpoint=False)
    Z, Y, X = np.meshgrid(z[levels], y, x, indexing="ij")
    grid = (np.squeeze(X), np.squeeze(Y), np.squeeze(Z))
    return grid, np.squeeze(conc), np.squeeze(flx)


# ---------------------------------------------------------------------------
# profiles and helpers
# ---------------------------------------------------------------------------

KAPPA = 0.4


def psi(x):
    """Businger-Dyer momentum stability correction (pbl_model.py:207-230)."""
    x = np.asarray(x, dtype=np.float64)
    xi = np.where(x > 0.0, np.nan, np.power(1.0 - 16.0 * x, 0.25, dtype=complex).real)
    return np.where(
        x > 0.0,
        5.0 * x,
        -2.0 * np.log(0.5 * (1.0 + xi))
        - np.log(0.5 * (1.0 + xi**2))
        + 2.0 * np.arctan(xi)
        - 0.5 * np.pi,
    )


def phi(x):
    """Businger-Dyer diffusivity stability function (pbl_model.py:233-250)."""
    x = np.asarray(x, dtype=np.float64)
    return np.where(x > 0.0, 1.0 + 5.0 * x, np.power(1.0 - 16.0 * x, -0.5, dtype=complex).real)


def vertical_profiles(
    n, meas_height, wind, ustar=None, z0=None, mol=1e9, prsc=1.0, closure="MOST",
    domain_height=None, stretch=None, z0_min=0.001, z0_max=2.0, tke=None,
):
    """Stretched z grid and u, v, Kx, Ky, Kz profiles (pbl_model.py:8-204)."""
    zm, (um, vm) = meas_height, wind
    kap = KAPPA
    absum = np.sqrt(um**2 + vm**2)
    if closure in ("CONSTANT", "MOST", "MOSTM"):
        if z0 is None:
            z0 = zm * np.exp(-kap * absum / ustar + psi(zm / mol))
        elif ustar is None:
            ustar = absum * kap / (np.log(zm / z0) + psi(zm / mol))
        else:
            raise ValueError("Either z0 or ustar must be provided.")
    elif closure == "OAAHOC":
        cl, cm, ch = 0.845, 0.0856, 0.204
        if tke is None:
            tke = 1.0
        tke = np.array(tke)[..., np.newaxis]
        absum = np.sqrt(um**2 + vm**2)
        z0 = zm * np.exp(-cm * cl * absum * np.sqrt(tke) / ustar**2)
    else:
        raise ValueError(
            f"Invalid closure type: {closure}. "
            "Supported closures are 'MOST', 'CONSTANT', and 'OAAHOC'."
        )
    h = 2.0 * meas_height if stretch is None else stretch
    zmx = 2.0 * meas_height if domain_height is None else domain_height
    bb = zm / (np.exp(-z0 / h) - np.exp(-zm / h))
    aa = bb * np.exp(-z0 / h)
    zetamx = aa - bb * np.exp(-zmx / h)
    dzeta = zm / n
    zeta = np.arange(0.0, np.squeeze(zetamx).item() + dzeta, dzeta)
    z = -h * np.log(-(zeta - aa) / bb)
    if closure == "CONSTANT":
        Km = kap * ustar * zm / prsc
        u = um * np.ones(len(z))
        v = vm * np.ones(len(z))
        K = Km * np.ones(len(z))
        Kx = Ky = Kz = K
    elif closure == "MOST":
        absu = ustar / kap * (np.log(z / z0) + psi(z / mol))
        u = um / absum * absu
        v = vm / absum * absu
        K = kap * ustar * z / phi(z / mol) / prsc
        Kx = Ky = Kz = K
    elif closure == "MOSTM":
        absu = ustar / kap * (np.log(z / z0) + psi(z / mol))
        u = um / absum * absu
        v = vm / absum * absu
        K = kap * ustar * z / phi(z / mol) / prsc
        Kx = K * v**2 / (u**2 + v**2)
        Ky = K * u**2 / (u**2 + v**2)
        Kz = K
    else:  # OAAHOC
        absu = ustar**2 / cm / cl / np.sqrt(tke) * np.log(z / z0)
        u = um / absum * absu
        v = vm / absum * absu
        K = ch * cl * z * np.sqrt(tke)
        Kx = Ky = Kz = K
    return z, (u, v, Kx, Ky, Kz)


def compute_wind_fields(u_rot, wind_dir):
    """(speed, meteorological direction) -> (u, v) (utils.py:7-27)."""
    wind_dir = np.deg2rad(wind_dir)
    return -u_rot * np.sin(wind_dir), -u_rot * np.cos(wind_dir)


def ideal_source(nxy, domain, src_loc=None, shape="diamond"):
    """Synthetic source fields (utils.py:30-77)."""
    nx, ny = nxy
    xmx, ymx = domain
    dx = xmx / nx
    if src_loc is None:
        src_loc = (xmx / 2, ymx / 2)
    xs, ys = src_loc
    X, Y = np.meshgrid(np.linspace(0.0, xmx, nx), np.linspace(0.0, ymx, ny))
    q0 = np.zeros([ny, nx])
    if shape == "diamond":
        R0 = xmx / 12
        q0 = np.where(np.abs(X - xs) + np.abs(Y - ys) < R0, 1.0, 0.0)
    if shape == "circle":
        R0 = xmx / 12
        q0 = np.where(np.sqrt((X - xs) ** 2 + (Y - ys) ** 2) < R0, 1.0, 0.0)
    if shape == "point":
        sig = 4.0 * dx
        q0 = np.exp(-((X - xs) ** 2 + (Y - ys) ** 2) / 2.0 / sig**2) / sig / np.sqrt(2.0 * np.pi)
    return q0


def point_measurement(f, g):
    """Footprint-weighted sum (utils.py:80-92)."""
    return np.sum(f * g)
