"""The reference's runners (src/bldfm/interface.py:31-326) on the host side:
the case each (tower, timestep) pair becomes, result dictionaries and their
order, with the profiles from the oracle and the solves stubbed."""

import numpy as np
import pytest

import interface_configs as IC


@pytest.fixture
def stubbed(monkeypatch):
    from bldfm_gb300 import batch, interface
    from oracle import bldfm_oracle as O

    seen = []
    monkeypatch.setattr(interface, "vertical_profiles", O.vertical_profiles)
    monkeypatch.setattr(interface, "vertical_profiles_batch", lambda cases: [O.vertical_profiles(**c) for c in cases])

    def fake_solver(**kw):
        seen.append(("single", kw))
        return ("grid",), np.full(3, kw["meas_pt"][0]), np.full(3, kw["meas_pt"][1])

    def fake_stream(batches):
        for cases in batches:
            seen.append(("batch", len(cases)))
            yield [(("grid",), np.full(3, c["meas_pt"][0]), np.full(3, c["meas_pt"][1])) for c in cases]

    monkeypatch.setattr(interface, "steady_state_transport_solver", fake_solver)
    monkeypatch.setattr(batch, "solve_stream", fake_stream)
    return seen


def test_single_builds_the_reference_case(stubbed):
    from bldfm_gb300 import interface
    from oracle import bldfm_oracle as O

    cfg = IC.config(n_steps=2)
    res = interface.run_bldfm_single(cfg, cfg.towers[1], met_index=1)
    assert set(res) == {"grid", "conc", "flx", "tower_name", "tower_xy", "timestamp", "params"}
    assert res["tower_name"] == "T1" and res["tower_xy"] == (210.0, 150.0) and res["timestamp"] == 1
    kw = stubbed[0][1]
    u, v = O.compute_wind_fields(3.5, 220.0)
    z, p = O.vertical_profiles(16, 12.0, (u, v), ustar=0.3, mol=-70.0, closure="MOST")
    np.testing.assert_array_equal(kw["z"], z)
    for a, b in zip(kw["profiles"], p):
        np.testing.assert_array_equal(a, b)
    assert kw["levels"] == 16 and kw["meas_pt"] == (210.0, 150.0) and kw["footprint"] and kw["mode"] == "fp64"
    np.testing.assert_array_equal(kw["srf_flx"], O.ideal_source((96, 64), (480.0, 320.0), shape="diamond"))


@pytest.mark.parametrize("output_levels,full_output,want", [([2, 5], False, [2, 5]), (None, True, list(range(17)))])
def test_levels_follow_the_domain_config(stubbed, output_levels, full_output, want):
    from bldfm_gb300 import interface

    cfg = IC.config(n_steps=1, output_levels=output_levels, full_output=full_output)
    interface.run_bldfm_single(cfg, cfg.towers[0])
    assert stubbed[0][1]["levels"] == want


def test_z0_takes_precedence(stubbed):
    from bldfm_gb300 import interface
    from oracle import bldfm_oracle as O

    cfg = IC.config(n_steps=1, z0=0.05)
    interface.run_bldfm_single(cfg, cfg.towers[0])
    u, v = O.compute_wind_fields(3.0, 200.0)
    z, _ = O.vertical_profiles(16, 8.0, (u, v), z0=0.05, mol=-60.0, closure="MOST")
    np.testing.assert_array_equal(stubbed[0][1]["z"], z)


def test_multitower_batches_every_pair_in_order(stubbed):
    from bldfm_gb300 import interface

    cfg = IC.config(n_steps=3, towers=2)
    out = interface.run_bldfm_multitower(cfg, batch=4, mode="fp32")
    assert [e for e in stubbed if e[0] == "batch"] == [("batch", 4), ("batch", 2)]
    assert list(out) == ["T0", "T1"]
    for k, name in enumerate(["T0", "T1"]):
        assert [r["timestamp"] for r in out[name]] == [0, 1, 2]
        for r in out[name]:
            assert r["tower_name"] == name and r["conc"][0] == 150.0 + 60.0 * k


def test_fp64_mode_and_parallel_strategies(stubbed):
    from bldfm_gb300 import interface

    cfg = IC.config(n_steps=2, towers=1)
    res = interface.run_bldfm_timeseries(cfg, cfg.towers[0])  # the default: the reference's arithmetic
    assert len(res) == 2 and all(e[0] == "single" for e in stubbed)
    with pytest.warns(UserWarning):
        out = interface.run_bldfm_parallel(cfg, parallel_over="both", surface_flux=np.zeros((64, 96)))
    assert list(out) == ["T0"] and len(out["T0"]) == 2
    with pytest.raises(ValueError, match="Unknown parallel_over"):
        interface.run_bldfm_parallel(cfg, parallel_over="cells")


def test_stream_depth_bounds_the_outputs_in_flight():
    """solve_stream keeps eight batches in flight for the benchmark's
    16-footprint 512^2 steps and fewer when eight batches' FP64 outputs would
    pass ~1 GiB, never fewer than two."""
    from bldfm_gb300.batch import STREAM_BYTES, stream_depth

    small = [dict(srf_flx=np.zeros((512, 512)), levels=128)] * 16
    assert stream_depth(small) == 8
    big = [dict(srf_flx=np.zeros((1024, 1024)), levels=np.arange(3))] * 64
    assert stream_depth(big) == 2
    mid = [dict(srf_flx=np.zeros((1024, 1024)), levels=5)] * 16  # 256 MiB of outputs per batch
    assert stream_depth(mid) == 4 and 4 * 16 * 16 * 1024 * 1024 <= STREAM_BYTES
