"""The mixed-grid met timeseries workload: 512 seeded met cases over 8 towers
on 256^2 / 512^2 / 1024^2 grids with 64 <= n <= 256 levels to z_m.

Met draws: u* ~ U[0.1, 0.8] m/s, 1/L ~ U[-0.1, 0.05] 1/m, wind direction
~ U[0, 360) deg, z0 log-uniform in [0.01, 1] m, z_m ~ U[2, 50] m (per tower).
``vertical_profiles`` takes u* or z0, not both (pbl_model.py:68-78), so the
wind speed at z_m is the one that makes both hold:
U = u*/kappa (ln(z_m/z0) + psi(z_m/L)); draws with U < 0.5 m/s are redrawn.
"""

import math

import numpy as np

TOWERS = [  # (grid, n, domain m)
    (256, 64, 1000.0),
    (512, 128, 1000.0),
    (1024, 256, 2000.0),
    (256, 96, 600.0),
    (512, 160, 1500.0),
    (256, 200, 800.0),
    (1024, 128, 3000.0),
    (512, 256, 1200.0),
]


def _psi(x):
    if x > 0:
        return 5.0 * x
    xi = (1.0 - 16.0 * x) ** 0.25
    return -2.0 * math.log(0.5 * (1 + xi)) - math.log(0.5 * (1 + xi * xi)) + 2.0 * math.atan(xi) - 0.5 * math.pi


def met_cases(ncases=512, seed=0):
    """List of dicts: tower index, grid, n, domain, zm, ustar, mol, wind (u, v)."""
    rng = np.random.default_rng(seed)
    zms = rng.uniform(2.0, 50.0, len(TOWERS))
    out = []
    while len(out) < ncases:
        t = len(out) % len(TOWERS)
        grid, n, dom = TOWERS[t]
        zm = float(zms[t])
        ustar = float(rng.uniform(0.1, 0.8))
        inv_l = float(rng.uniform(-0.1, 0.05))
        mol = 1.0 / inv_l if abs(inv_l) > 1e-6 else 1e6
        z0 = float(math.exp(rng.uniform(math.log(0.01), math.log(1.0))))
        wdir = float(rng.uniform(0.0, 360.0))
        if z0 >= zm:
            continue
        U = ustar / 0.4 * (math.log(zm / z0) + _psi(zm / mol))
        if not U >= 0.5:
            continue
        th = math.radians(wdir)
        out.append(dict(tower=t, grid=grid, n=n, domain=(dom, dom), zm=zm, ustar=ustar, mol=mol, z0=z0,
                        wind=(-U * math.sin(th), -U * math.cos(th)), meas_pt=(dom / 2, dom / 2)))
    return out
