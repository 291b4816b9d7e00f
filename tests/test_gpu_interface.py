"""The batched runners (interface.py:141-326 equivalents) against one-by-one
solves through the drop-in: same result dictionaries, FP32 batches within
the FP32 bar of the FP64 solves and equal to the single FP32 solves."""

import numpy as np
import pytest

import golden_cases as G
import interface_configs as IC

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("footprint", [True, False])
def test_multitower_matches_single_solves(footprint):
    from bldfm_gb300 import interface

    cfg = IC.config(n_steps=3, towers=2, footprint=footprint, output_levels=None if footprint else [4, 16])
    out = interface.run_bldfm_multitower(cfg, batch=4, mode="fp32")
    for tower in cfg.towers:
        for i, r in enumerate(out[tower.name]):
            r64 = interface.run_bldfm_single(cfg, tower, met_index=i, mode="fp64")
            r32 = interface.run_bldfm_single(cfg, tower, met_index=i, mode="fp32")
            assert r["conc"].shape == r64["conc"].shape and r["timestamp"] == i
            for a, b in zip(r["grid"], r64["grid"]):
                np.testing.assert_array_equal(a, b)
            assert G.rel_l2(r["conc"], r64["conc"]) <= 1e-4 and G.rel_l2(r["flx"], r64["flx"]) <= 1e-4
            assert G.rel_l2(r["conc"], r32["conc"]) <= 1e-6 and G.rel_l2(r["flx"], r32["flx"]) <= 1e-6


def test_timeseries_with_cache_enabled():
    from bldfm_gb300 import interface

    cfg = IC.config(n_steps=2, towers=1, use_cache=True)
    cfg.met.ustar = [0.3, 0.3]  # identical steps: identical results through the cached path
    cfg.met.mol = [-50.0, -50.0]
    cfg.met.wind_speed = [4.0, 4.0]
    cfg.met.wind_dir = [225.0, 225.0]
    res = interface.run_bldfm_timeseries(cfg, cfg.towers[0])
    np.testing.assert_array_equal(res[0]["flx"], res[1]["flx"])


def test_fp32_results_never_answer_reference_key():
    """Batched FP32 results go into the cache under the mode's own key: a
    lookup with the reference's key (what the reference's own cache class
    computes, src/bldfm/cache.py:34-45) misses, the FP32 lookup hits."""
    from bldfm_gb300 import interface
    from bldfm_gb300.cache import GreensFunctionCache

    cfg = IC.config(n_steps=1, towers=1, use_cache=True)
    calls = []
    orig = interface._make_cache

    def spy(config):
        c = orig(config)
        calls.append(c)
        return c

    interface._make_cache = spy
    try:
        res = interface.run_bldfm_timeseries(cfg, cfg.towers[0], mode="fp32")
    finally:
        interface._make_cache = orig
    cache = calls[0]
    assert isinstance(cache, GreensFunctionCache) and len(cache) == 1
    kw = interface._case(cfg, cfg.towers[0], 0, None)[0]
    args = (kw["z"], kw["profiles"], kw["domain"], kw["modes"], kw["meas_pt"], kw["halo"], kw["precision"])
    assert cache.get(*args) is None
    hit = cache.get(*args, variant="fp32")
    assert hit is not None and np.array_equal(hit[2], res[0]["flx"])


def test_vertical_profiles_batch_equals_single_calls():
    from bldfm_gb300.pbl_model import vertical_profiles, vertical_profiles_batch

    cases = [dict(n=16, meas_height=10.0, wind=(2.0, -1.0), ustar=0.3, mol=-50.0),
             dict(n=40, meas_height=25.0, wind=(-3.0, 0.5), z0=0.1, mol=120.0, closure="MOSTM"),
             dict(n=24, meas_height=6.0, wind=(1.0, 1.0), ustar=0.2, mol=1e9, closure="CONSTANT"),
             dict(n=32, meas_height=15.0, wind=(4.0, 0.0), ustar=0.35, closure="OAAHOC", tke=0.8)]
    for (zb, pb), kw in zip(vertical_profiles_batch(cases), cases):
        z, p = vertical_profiles(**kw)
        np.testing.assert_array_equal(zb, z)
        for a, b in zip(pb, p):
            np.testing.assert_array_equal(a, b)
