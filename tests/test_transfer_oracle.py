"""The surrogate's nondimensional transfer functions (oracle/transfer_oracle.py)
against the dimensional FP64 invariant-imbedding oracle: a MOST footprint
case's per-mode (p, q) at z_m must equal q0 Tq and (R~ / U) q0 Tq after the
rotation and scaling of the wavenumbers by the wind direction and z_m."""

import numpy as np
import pytest

from oracle import bldfm_oracle as O
from oracle.transfer_oracle import nondim_profiles, transfer, ustar_ratio


@pytest.mark.parametrize(
    "zm,ustar,mol,wdir",
    [(20.0, 0.3, -50.0, 225.0), (10.0, 0.4, 1e9, 270.0), (5.0, 0.2, 30.0, 37.0)],
)
def test_nondimensional_mapping(zm, ustar, mol, wdir):
    n = 32
    th = np.deg2rad(wdir)
    speed = 4.0
    wind = (-speed * np.sin(th), -speed * np.cos(th))
    z, prof = O.vertical_profiles(n, zm, wind, ustar=ustar, mol=mol)
    z = np.asarray(z)
    u, v, Kx, Ky, Kz = (np.broadcast_to(np.asarray(p, dtype=np.float64), z.shape) for p in prof)
    U = np.hypot(u[n], v[n])
    ex, ey = u[n] / U, v[n] / U
    rng = np.random.default_rng(1)
    Lx = rng.uniform(-0.3, 0.3, 64)
    Ly = rng.uniform(-0.3, 0.3, 64)
    eig = np.sqrt((Kx[-1] * Lx**2 + Ky[-1] * Ly**2) / Kz[-1] + 1j * (u[-1] * Lx + v[-1] * Ly) / Kz[-1])
    q0 = np.ones(64, dtype=np.complex128)
    p, q = O.riccati_sweep(Lx, Ly, q0, eig, Kz[-1], (u, v, Kx, Ky, Kz), z, [n])
    # nondimensional case: s1 = zm / L, s2 = ln(zm / z0)
    z0 = zm * np.exp(-0.4 * U / ustar + O.psi(zm / mol))
    s1, s2 = zm / mol, np.log(zm / z0)
    kpar = zm * (ex * Lx + ey * Ly)
    kperp = zm * (-ey * Lx + ex * Ly)
    Tq, Rt, _ = transfer(s1, s2, n, np.abs(kpar), np.abs(kperp))
    neg = kpar < 0
    Tq = np.where(neg, np.conj(Tq), Tq)
    Rt = np.where(neg, np.conj(Rt), Rt)
    np.testing.assert_allclose(q[0], Tq, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(p[0], Rt / U * Tq, rtol=1e-9, atol=1e-14)
    assert abs(ustar_ratio(s1, s2) - ustar / U) < 1e-12


def test_grid_is_nondimensional():
    z, U, K = nondim_profiles(-0.4, np.log(400.0), 128)
    assert len(z) == 207
    assert abs(z[128] - 1.0) < 1e-12 and abs(U[128] - 1.0) < 1e-12
