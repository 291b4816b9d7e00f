"""Golden cache keys from the reference's GreensFunctionCache
(src/bldfm/cache.py:34-45), for tests/test_cache.py.

Run in a container that has the reference sources (see refshim.py):
    python tests/golden/make_cache_key.py
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refshim  # noqa: E402


def cases():
    rng = np.random.default_rng(7)
    z = np.linspace(0.01, 40.0, 17)
    prof = [rng.uniform(0.1, 5.0, 17) for _ in range(5)]
    yield dict(z=z, profiles=prof, domain=(1000.0, 700.0), modes=(128, 96), meas_pt=(500.0, 300.0), halo=None,
               precision="single")
    yield dict(z=z[:9], profiles=[p[:9] for p in prof], domain=[200, 200], modes=[64, 64], meas_pt=(0.0, 0.0),
               halo=250.0, precision="double")


def main():
    bldfm = refshim.import_reference()
    import importlib

    cache_mod = importlib.import_module("bldfm.cache")
    c = cache_mod.GreensFunctionCache(cache_dir="/tmp/bldfm_refshim_cache")
    out = []
    for kw in cases():
        key = c._compute_key(**kw)
        out.append({"z": np.asarray(kw["z"]).tolist(), "profiles": [np.asarray(p).tolist() for p in kw["profiles"]],
                    "domain": list(kw["domain"]), "domain_type": type(kw["domain"][0]).__name__,
                    "modes": list(kw["modes"]), "meas_pt": list(kw["meas_pt"]), "halo": kw["halo"],
                    "precision": kw["precision"], "key": key})
    with open(os.path.join(HERE, "cache_keys.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(out), "keys")


if __name__ == "__main__":
    main()
