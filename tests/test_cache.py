"""Green's-function cache: the key matches the reference's
(GreensFunctionCache._compute_key, src/bldfm/cache.py:34-45) on golden inputs,
and the HBM cache behaves like the reference's disk cache."""

import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_cache_key_matches_reference():
    from bldfm_gb300.cache import cache_key

    with open(os.path.join(HERE, "golden", "cache_keys.json")) as f:
        cases = json.load(f)
    for c in cases:
        key = cache_key(
            np.asarray(c["z"]), [np.asarray(p) for p in c["profiles"]], c["domain"], c["modes"], c["meas_pt"],
            c["halo"], c["precision"],
        )
        assert key == c["key"]


@pytest.mark.gpu
def test_device_cache_roundtrip_lru_and_disk(tmp_path):
    import torch

    from bldfm_gb300.cache import GreensFunctionCache

    z = np.linspace(0.1, 10, 5)
    prof = [np.ones(5)] * 5
    grid = tuple(np.zeros((4, 6)) for _ in range(3))
    c = GreensFunctionCache(cache_dir=tmp_path, max_bytes=2 * 2 * 4 * 6 * 8)
    args = lambda m: (z, prof, (100.0, 100.0), (4, 6), (50.0, float(m)), None, "single")
    assert c.get(*args(0)) is None
    for m in range(3):
        c.put(*args(m), grid, np.full((4, 6), float(m)), np.full((4, 6), -float(m)))
    assert len(c) == 2  # LRU kept the last two in HBM
    dev = c.get_device(*args(2))
    assert dev is not None and dev[0].is_cuda and float(dev[0][0, 0]) == 2.0
    # the evicted entry comes back from disk, in the reference's file format
    g, conc, flx = c.get(*args(0))
    assert np.all(conc == 0.0) and np.all(flx == 0.0)
    files = list(tmp_path.glob("*.npz"))
    assert len(files) == 3 and set(np.load(files[0]).files) == {"X", "Y", "Z", "conc", "flx"}
    c.clear()
    assert len(c) == 0 and not list(tmp_path.glob("*.npz"))


@pytest.mark.gpu
def test_point_measurement_batch_matches_numpy():
    import torch

    from bldfm_gb300.utils import point_measurement, point_measurement_batch

    rng = np.random.default_rng(3)
    for shape in [(1, 7), (3, 511, 513), (16, 512, 512), (2, 1)]:
        F = rng.standard_normal(shape)
        G = rng.uniform(0, 1, shape)
        out = point_measurement_batch(torch.from_numpy(F).cuda(), torch.from_numpy(G).cuda()).cpu().numpy()
        ref = np.array([np.sum(F[b] * G[b]) for b in range(shape[0])])
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12 * np.abs(F * G).sum())
    f = rng.uniform(0, 1, (64, 48))
    g = rng.uniform(0, 1, (64, 48))
    assert abs(point_measurement(torch.from_numpy(f).cuda(), torch.from_numpy(g).cuda()) - np.sum(f * g)) < 1e-12
    assert point_measurement(f, g) == np.sum(f * g)


def test_cache_key_variant_keeps_reference_key():
    """The sweep mode keys non-reference results apart; the reference's
    arithmetic (variant None or "fp64") keeps the reference's key."""
    from bldfm_gb300.cache import cache_args, cache_key

    with open(os.path.join(HERE, "golden", "cache_keys.json")) as f:
        c = json.load(f)[0]
    args = (np.asarray(c["z"]), [np.asarray(p) for p in c["profiles"]], c["domain"], c["modes"], c["meas_pt"],
            c["halo"], c["precision"])
    assert cache_key(*args) == cache_key(*args, variant="fp64") == c["key"]
    assert cache_key(*args, variant="fp32") != c["key"]
    assert cache_key(*args, variant="fp32") != cache_key(*args, variant="fp64r")

    class ReferenceLikeCache:  # the reference's class: get/put without variant
        pass

    assert cache_args(ReferenceLikeCache(), "fp64") == (True, {})
    assert cache_args(ReferenceLikeCache(), "fp32") == (False, {})
    assert cache_args(None, "fp64") == (False, {})
