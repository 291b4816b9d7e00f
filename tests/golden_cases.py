"""Load the golden fixtures of tests/golden/ and run a solver on their inputs."""

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def solver_names():
    return sorted(
        os.path.basename(p)[:-4]
        for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
        if not os.path.basename(p).startswith("profiles_")
    )


def profile_names():
    return sorted(os.path.basename(p)[9:-4] for p in glob.glob(os.path.join(GOLDEN, "profiles_*.npz")))


def load(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return d


def kwargs_of(d):
    """Solver arguments stored in a fixture."""
    shape = tuple(int(s) for s in d["srf_shape"])
    srf = d["srf_flx"] if "srf_flx" in d else np.zeros(shape)
    levels = int(d["levels"][0]) if bool(d["levels_scalar"]) else d["levels"]
    halo = float(d["halo"])
    profs = tuple(d["profiles"][i] for i in range(5))
    return dict(
        srf_flx=srf,
        z=d["z"],
        profiles=profs,
        domain=tuple(float(x) for x in d["domain"]),
        levels=levels,
        modes=tuple(int(m) for m in d["modes"]),
        meas_pt=tuple(float(x) for x in d["meas_pt"]),
        srf_bg_conc=float(d["srf_bg_conc"]),
        footprint=bool(d["footprint"]),
        analytic=bool(d["analytic"]),
        halo=None if np.isnan(halo) else halo,
        precision=str(d["precision"]),
    )


def reference_fields(d):
    return d["conc"], d["flx"]


def sample(d, field):
    """Apply the fixture's subsampling to a full solver output."""
    s = int(d["subsample"]) if "subsample" in d else 1
    return field[..., ::s, ::s]


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
