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
    out = interface.run_bldfm_multitower(cfg, batch=4)
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
