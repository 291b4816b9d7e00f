"""Host-side logic of the surrogate (no GPU): met scalars, training box, mode
wavenumber range, and the shipped weights' metadata."""

import math
import os

import numpy as np
import pytest

from oracle.bldfm_oracle import psi as ref_psi
from oracle.bldfm_oracle import vertical_profiles


def test_met_scalars_follow_vertical_profiles():
    from bldfm_gb300.surrogate import met_scalars, psi

    for x in (-3.0, -0.4, -1e-3, 0.0, 0.2, 1.5):
        assert abs(psi(x) - float(ref_psi(x))) < 1e-12
    # u* given: z0 follows as in pbl_model.py:68-78; s2 = ln(zm / z0)
    zm, wind, ustar, mol = 20.0, (2.83, 2.83), 0.3, -50.0
    U, s1, s2, s3 = met_scalars(zm, wind, ustar=ustar, mol=mol)
    z0 = zm * math.exp(-0.4 * math.hypot(*wind) / ustar + float(ref_psi(zm / mol)))
    assert abs(s2 - math.log(zm / z0)) < 1e-12 and abs(s1 + 0.4) < 1e-15
    assert abs(s3 - ustar / U) < 1e-12
    # z0 given: u* follows
    U2, _, s2b, s3b = met_scalars(zm, wind, z0=0.05, mol=mol)
    z, prof = vertical_profiles(32, zm, wind, z0=0.05, mol=mol)
    assert abs(s2b - math.log(zm / 0.05)) < 1e-12
    assert abs(np.hypot(prof[0][32], prof[1][32]) - U2) < 1e-9 * U2


def test_mode_kmax_and_box():
    from bldfm_gb300.surrogate import BOX, TRAIN_BOX, mode_kmax

    k = mode_kmax((512, 512), (1000.0, 1000.0), (512, 512))
    # 1536-point extended grid, modes up to 256: 2 pi 256 / 3000 per axis
    assert abs(k - math.hypot(*(2 * math.pi * 256 / 3000.0,) * 2)) < 1e-12
    for key in ("s1", "s2"):
        assert TRAIN_BOX[key][0] <= BOX[key][0] and TRAIN_BOX[key][1] >= BOX[key][1]


def test_shipped_weights_metadata():
    import json

    from bldfm_gb300.surrogate import WEIGHTS

    if not os.path.exists(WEIGHTS):
        pytest.skip("no shipped weights")
    d = np.load(WEIGHTS)
    assert d["params"].dtype == np.float32 and d["params"].size == 200708
    assert np.all(np.isfinite(d["params"]))
    meta = json.loads(str(d["meta"]))
    assert meta["batch"] == 65536 and meta["steps"] >= 100000
