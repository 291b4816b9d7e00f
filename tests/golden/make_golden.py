"""Generate golden fixtures by running the reference BLDFM solver in this container.

Run from the repository root:  python tests/golden/make_golden.py
Needs the reference sources (imported through refshim.py; numba/pyfftw/abltk
are stubbed there).  Writes one .npz per case into tests/golden/: the exact
solver inputs, the reference outputs, and for large cases a subsample.

Cases follow the reference's own test fixtures (tests/conftest.py:41-262,
tests/test_integration.py:28-290) and the workload configurations of the
benchmark (seeded synthetic inputs with the stated shapes).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refshim  # noqa: E402

bldfm = refshim.import_reference()
from bldfm.pbl_model import vertical_profiles  # noqa: E402
from bldfm.solver import steady_state_transport_solver  # noqa: E402
from bldfm.utils import compute_wind_fields, ideal_source  # noqa: E402

# tower x of the reference's timeseries fixtures: lat/lon (50.95, 11.5867)
# relative to (50.95, 11.586), equirectangular with R = 6371000 m
TOWER_X = 6371000.0 * np.radians(11.5867 - 11.586) * np.cos(np.radians(50.95))


def solver_case(name, srf_flx, z, profs, domain, levels, subsample=None, **kw):
    grid, conc, flx = steady_state_transport_solver(srf_flx, z, profs, domain, levels, **kw)
    out = dict(
        z=np.asarray(z, np.float64),
        profiles=np.stack([np.asarray(p, np.float64) for p in profs]),
        domain=np.asarray(domain, np.float64),
        levels=np.atleast_1d(np.asarray(levels)),
        levels_scalar=np.asarray(np.ndim(levels) == 0),
        modes=np.asarray(kw.get("modes", (512, 512))),
        meas_pt=np.asarray(kw.get("meas_pt", (0.0, 0.0)), np.float64),
        srf_bg_conc=np.asarray(kw.get("srf_bg_conc", 0.0)),
        footprint=np.asarray(kw.get("footprint", False)),
        analytic=np.asarray(kw.get("analytic", False)),
        halo=np.asarray(np.nan if kw.get("halo") is None else kw["halo"]),
        precision=np.asarray(kw.get("precision", "single")),
        srf_shape=np.asarray(np.shape(srf_flx)),
        conc_dtype=np.asarray(str(conc.dtype)),
        conc_norm=np.asarray(np.linalg.norm(conc)),
        flx_norm=np.asarray(np.linalg.norm(flx)),
        conc_sum=np.asarray(np.sum(conc, dtype=np.float64)),
        flx_sum=np.asarray(np.sum(flx, dtype=np.float64)),
    )
    if not kw.get("footprint", False):
        out["srf_flx"] = np.asarray(srf_flx, np.float64)
    if subsample:
        out["subsample"] = np.asarray(subsample)
        out["conc"] = conc[..., ::subsample, ::subsample]
        out["flx"] = flx[..., ::subsample, ::subsample]
    else:
        out["conc"] = conc
        out["flx"] = flx
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("%-28s conc %s %s" % (name, conc.shape, conc.dtype))


def profile_case(name, *args, **kw):
    z, profs = vertical_profiles(*args, **kw)
    args_rec = dict(kw)
    np.savez_compressed(
        os.path.join(HERE, "profiles_" + name + ".npz"),
        z=z,
        profiles=np.stack(profs),
        n=args[0],
        meas_height=args[1],
        wind=np.asarray(args[2], np.float64),
        kwargs=np.asarray(repr(args_rec)),
    )
    print("%-28s nz %d" % ("profiles_" + name, len(z)))


def main():
    # reference conftest source_area_result_session (conftest.py:196-230)
    z, p = vertical_profiles(16, 10.0, (0.0, -6.0), 0.5)
    solver_case("source_area", np.zeros((128, 64)), z, p, (100.0, 700.0), 16,
                modes=(64, 128), meas_pt=(50.0, 0.0), footprint=True)
    # plume_3d_result_session (conftest.py:233-262)
    z, p = vertical_profiles(16, 10.0, (6.0, 0.0), 0.4)
    solver_case("plume_3d", ideal_source((64, 32), (800.0, 100.0)), z, p, (800.0, 100.0),
                np.arange(0, 17, 2), modes=(64, 32), meas_pt=(400.0, 50.0), footprint=False)
    # single_footprint / timeseries steps through run_bldfm_single (interface.py:31-138)
    for name, (us, mol, ws, wd) in {
        "single_footprint": (0.5, -100.0, 6.0, 0.0),
        "timeseries_step2": (0.6, -50.0, 7.0, 345.0),
    }.items():
        z, p = vertical_profiles(16, 10.0, compute_wind_fields(ws, wd), ustar=us, mol=mol)
        solver_case(name, ideal_source((64, 128), (100.0, 700.0)), z, p, (100.0, 700.0), 16,
                    modes=(64, 128), meas_pt=(TOWER_X, 0.0), footprint=True)
    # _quick_solve variants (test_integration.py:166-196)
    z, p = vertical_profiles(16, 10.0, (5.0, 0.0), 0.4, closure="MOST")
    src = ideal_source((128, 64), (500.0, 250.0), (250.0, 125.0), shape="point")
    solver_case("quick_double_shift", src, z, p, (500.0, 250.0), 15, modes=(128, 64),
                footprint=False, precision="double", meas_pt=(25.0, 12.5))
    solver_case("quick_single_noshift", src, z, p, (500.0, 250.0), 15, modes=(128, 64),
                footprint=False, precision="single")
    solver_case("quick_footprint_double", src, z, p, (500.0, 250.0), 15, modes=(128, 64),
                footprint=True, precision="double")
    solver_case("halo_clamp", src, z, p, (500.0, 250.0), 15, modes=(512, 512), halo=1.0)
    # analytic known answer, CONSTANT closure (test_integration.py:28-84, reduced size)
    zc, pc = vertical_profiles(32, 5.0, (4.0, 1.0), 0.2, closure="CONSTANT")
    srcp = ideal_source((128, 64), (100.0, 50.0), (5.0, 5.0), shape="point")
    solver_case("analytic_constant", srcp, zc, pc, (100.0, 50.0), 32, modes=(256, 256), halo=500.0,
                analytic=True)
    solver_case("numeric_constant", srcp, zc, pc, (100.0, 50.0), 32, modes=(256, 256), halo=500.0)
    # footprint, several unsorted / duplicate levels, background concentration
    z, p = vertical_profiles(24, 8.0, compute_wind_fields(3.0, 120.0), ustar=0.35, mol=40.0)
    solver_case("multilevel_footprint", np.zeros((48, 40)), z, p, (60.0, 90.0), np.array([24, 3, 3, 0, len(z) - 1]),
                modes=(32, 48), meas_pt=(20.0, 30.0), footprint=True, precision="double", srf_bg_conc=0.7)
    # ragged grid: odd nx, ny (footprint; extended sizes odd -> clamped odd modes)
    z, p = vertical_profiles(12, 6.0, compute_wind_fields(4.0, 200.0), ustar=0.3, mol=-30.0)
    solver_case("ragged_odd", np.zeros((37, 53)), z, p, (53.0, 37.0), 12, modes=(200, 200),
                meas_pt=(10.0, 5.0), footprint=True, precision="double", halo=7.3)
    # non-footprint multi-level dispersion with background concentration
    z, p = vertical_profiles(10, 5.0, compute_wind_fields(2.0, 45.0), z0=0.05, mol=1e9)
    solver_case("plume_levels_double", ideal_source((48, 64), (300.0, 200.0), shape="circle"), z, p,
                (300.0, 200.0), [0, 5, 10], modes=(48, 64), footprint=False, precision="double", srf_bg_conc=1.5)
    # config 1: neutral MOST, Gaussian patch, 256^2, n = 64, domain height 3 z_m
    z, p = vertical_profiles(64, 10.0, compute_wind_fields(5.0, 270.0), z0=0.1, mol=1e9, domain_height=30.0)
    X, Y = np.meshgrid(np.linspace(0, 1000.0, 256), np.linspace(0, 700.0, 256))
    g = np.exp(-((X - 500.0) ** 2 + (Y - 300.0) ** 2) / (2 * 50.0**2))
    solver_case("cfg1_gaussian_256", g, z, p, (1000.0, 700.0), 64, modes=(512, 512), precision="double",
                subsample=2)
    # headline workload: footprint 512^2, n = 128, unstable
    z, p = vertical_profiles(128, 20.0, compute_wind_fields(4.0, 225.0), ustar=0.3, mol=-50.0)
    solver_case("metric_footprint_512", np.zeros((512, 512)), z, p, (1000.0, 1000.0), 128, modes=(512, 512),
                meas_pt=(500.0, 500.0), footprint=True, precision="double", subsample=4)

    # vertical profiles of every closure (pbl_model.py:8-204)
    profile_case("most_unstable", 32, 10.0, (3.0, -4.0), ustar=0.4, mol=-50.0)
    profile_case("most_stable", 32, 10.0, (3.0, -4.0), ustar=0.4, mol=80.0)
    profile_case("most_z0", 64, 20.0, compute_wind_fields(4.0, 225.0), z0=0.05, mol=-50.0)
    profile_case("most_neutral_dh", 64, 10.0, compute_wind_fields(5.0, 270.0), z0=0.1, mol=1e9, domain_height=30.0)
    profile_case("constant", 16, 5.0, (4.0, 1.0), ustar=0.2, closure="CONSTANT")
    profile_case("mostm", 20, 10.0, (2.0, 3.0), ustar=0.3, mol=-20.0, closure="MOSTM")
    profile_case("oaahoc", 20, 10.0, (2.0, 3.0), ustar=0.3, closure="OAAHOC", tke=0.8)
    profile_case("stretch", 16, 10.0, (1.0, 1.0), ustar=0.3, mol=200.0, stretch=15.0, domain_height=25.0)


if __name__ == "__main__":
    main()
