"""CPU oracle of the surrogate's training data: nondimensional transfer functions.

TEST INFRASTRUCTURE ONLY: imported by tests/ and nothing on the product path.

For MOST profiles (pbl_model.py:8-204: u = u*/kappa (ln z/z0 + psi(z/L)),
K = kappa u* z / phi(z/L), Kx = Ky = Kz, fixed wind direction) and the
stretched grid with the default stretch and top (2 z_m), the reference's
discrete per-mode problem (solver.py:307-374, top radiation condition
solver.py:194-212) depends on the met case only through s1 = z_m / L and
s2 = ln(z_m / z0) once heights are scaled by z_m, velocities by the wind
speed U at z_m and diffusivities by U z_m.  For a mode with wind-parallel and
wind-normal wavenumbers (k_par, k_perp) scaled by z_m, the flux transfer
Tq = q(z_m) / q(0) and R~ = U p(z_m) / q(z_m) follow from the invariant
imbedding recursion of ``bldfm_oracle.riccati_sweep`` in FP64.  Targets, as
learned by the network: log|Tq| / (1 + k), arg Tq / (1 + k) (arg unwrapped as
the sum of the per-step factor arguments), log|R~ / R~top|, arg(R~ / R~top),
k = |k~|, R~top = 1 / (K~top lam) the top radiation ratio.
"""

import numpy as np

from .bldfm_oracle import vertical_profiles

KAPPA = 0.4


def nondim_profiles(s1, s2, n):
    """z~ and (U~, K~) on the n-level stretched grid of the case (s1, s2)."""
    mol = 1e9 if abs(s1) < 1e-9 else 1.0 / s1
    z, (u, v, Kx, Ky, Kz) = vertical_profiles(n, 1.0, (1.0, 0.0), z0=float(np.exp(-s2)), mol=mol)
    return np.asarray(z, dtype=np.float64), np.asarray(u, dtype=np.float64), np.asarray(Kz, dtype=np.float64)


def ustar_ratio(s1, s2):
    """u* / U of the case (the log-law at z_m)."""
    from .bldfm_oracle import psi

    return KAPPA / (s2 + float(psi(s1)))


def transfer(s1, s2, n, kpar, kperp):
    """Complex Tq, R~ and the four targets for wavenumbers kpar, kperp (arrays)."""
    z, U, K = nondim_profiles(s1, s2, n)
    kpar = np.asarray(kpar, dtype=np.float64)
    kperp = np.asarray(kperp, dtype=np.float64)
    k2 = kpar**2 + kperp**2
    nz = len(z)
    jm = n
    lam = np.sqrt(k2 + 1j * U[-1] * kpar / K[-1])
    R = 1.0 / (K[-1] * lam)
    Rj = R.copy()
    la = np.zeros_like(k2)
    ph = np.zeros_like(k2)
    dz = np.diff(z)
    for i in range(nz - 2, -1, -1):
        T = -K[i] * k2 - 1j * U[i] * kpar
        kap = 1.0 / K[i]
        h = dz[i]
        a = 1 - 0.5 * kap * h * h * T
        b = -kap * h - kap * kap * h**3 / 6.0 * T
        c = T * h - kap * h**3 / 6.0 * T * T
        R = (a * R - b) / (a - c * R)
        if i == jm:
            Rj = R.copy()
        if i < jm:
            f = c * R + a
            la += np.log(np.abs(f))
            ph += np.angle(f)
    Tq = np.exp(la + 1j * ph)
    kk = 1.0 + np.sqrt(k2)
    rr = Rj * K[-1] * lam  # R~ / R~top
    targets = np.stack([la / kk, ph / kk, np.log(np.abs(rr)), np.angle(rr)], axis=-1)
    return Tq, Rj, targets
