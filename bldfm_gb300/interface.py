"""The reference's high-level runners (src/bldfm/interface.py:31-326) on the GPU.

Same names, arguments and result dictionaries as ``run_bldfm_single``,
``run_bldfm_timeseries``, ``run_bldfm_multitower`` and ``run_bldfm_parallel``.
The configuration objects are read by attribute only (``config.domain``,
``config.solver``, ``config.met.get_step(i)`` / ``n_timesteps``,
``config.towers``, ``config.parallel``, ``tower.name / x / y / z_m``), so the
reference's own ``BLDFMConfig`` and ``TowerConfig`` instances work unchanged.

``run_bldfm_single`` is the reference's three-step workflow with this
package's ``vertical_profiles`` and ``steady_state_transport_solver`` (the
drop-in, FP64 with the reference's rounding by default).  Every runner
defaults to ``mode="fp64"``: the reference's arithmetic, one solve per case,
results equal to the reference's.  With ``mode="fp32"`` the multi-case
runners replace the reference's per-case loop and process pool
(interface.py:141-326) with the batched FP32 solver: every (tower, timestep)
case of the call goes through ``solve_stream`` in batches of ``batch``
cases, the FP32 invariant-imbedding sweep (relative L2 about 1e-6 against
the exact discrete solution, and up to the reference's own rounding floor,
~1e-3, away from the reference's FP64 output).  The profiles of all cases
are evaluated in one device launch.  Cases the batched solver does not take
(the analytic branch) go one by one.  With caching enabled, results of a
mode other than "fp64" are stored under their own key (bldfm_gb300.cache).
"""

import logging
import warnings

from .pbl_model import vertical_profiles, vertical_profiles_batch
from .solver import steady_state_transport_solver
from .utils import compute_wind_fields, ideal_source

logger = logging.getLogger("bldfm_gb300.interface")


def _make_cache(config):
    """A GreensFunctionCache when caching is enabled (interface.py:22-28)."""
    if config.parallel.use_cache and config.solver.footprint:
        from .cache import GreensFunctionCache

        return GreensFunctionCache()
    return None


def _profile_args(config, tower, met_index):
    """vertical_profiles arguments of one (tower, timestep) case and its met
    step (interface.py:71-99: z0 takes precedence over ustar)."""
    dom = config.domain
    met_step = config.met.get_step(met_index)
    u_wind, v_wind = compute_wind_fields(met_step["wind_speed"], met_step["wind_dir"])
    args = dict(n=dom.nz, meas_height=tower.z_m, wind=(u_wind, v_wind), mol=met_step["mol"],
                closure=config.solver.closure)
    z0_val = met_step.get("z0")
    if z0_val is not None:
        args["z0"] = z0_val
    else:
        args["ustar"] = met_step["ustar"]
    return args, met_step


def _source(config, surface_flux):
    """The surface flux of the run: the given field, or the configured ideal
    source (interface.py:101-110)."""
    if surface_flux is not None:
        return surface_flux
    dom, sol = config.domain, config.solver
    return ideal_source((dom.nx, dom.ny), (dom.xmax, dom.ymax), src_loc=sol.src_loc, shape=sol.surface_flux_shape)


def _solver_kwargs(config, tower, z, profiles, surface_flux):
    """Keyword arguments of steady_state_transport_solver (interface.py:112-134)."""
    dom, sol = config.domain, config.solver
    if dom.output_levels:
        levels = dom.output_levels
    elif dom.full_output:
        levels = list(range(dom.nz + 1))
    else:
        levels = dom.nz
    return dict(srf_flx=surface_flux, z=z, profiles=profiles, domain=(dom.xmax, dom.ymax), levels=levels,
                modes=dom.modes, meas_pt=(tower.x, tower.y), footprint=sol.footprint, analytic=sol.analytic,
                halo=dom.halo, precision=sol.precision)


def _case(config, tower, met_index, surface_flux):
    """Solver keyword arguments of one (tower, timestep) case and its met step."""
    args, met_step = _profile_args(config, tower, met_index)
    z, profiles = vertical_profiles(**args)
    return _solver_kwargs(config, tower, z, profiles, _source(config, surface_flux)), met_step


def _result(grid, conc, flx, tower, met_step):
    return {
        "grid": grid,
        "conc": conc,
        "flx": flx,
        "tower_name": tower.name,
        "tower_xy": (tower.x, tower.y),
        "timestamp": met_step["timestamp"],
        "params": met_step,
    }


def run_bldfm_single(config, tower, met_index=0, surface_flux=None, cache=None, *, mode="fp64"):
    """One solve for one tower at one timestep (interface.py:31-138); the
    result dictionary has the reference's keys.  ``mode`` selects the sweep
    of the drop-in solver ("fp64": the reference's rounding, "fp32")."""
    kw, met_step = _case(config, tower, met_index, surface_flux)
    grid, conc, flx = steady_state_transport_solver(**kw, cache=cache, mode=mode)
    return _result(grid, conc, flx, tower, met_step)


def _run_cases(config, pairs, surface_flux, mode, batch):
    """Results of (tower, met_index) pairs in order: one by one through the
    drop-in (mode "fp64", the reference's arithmetic, and "fp64r"), or batched
    FP32 through ``solve_stream`` (mode "fp32").  Cached results are keyed by
    mode: FP32 results never answer a lookup with the reference's key."""
    from .cache import cache_args

    cache = _make_cache(config)
    use_cache, ckw = cache_args(cache, mode)
    if not use_cache:
        cache = None
    # every case's profiles in one device launch, one shared surface flux
    prof_args = [_profile_args(config, tower, i) for tower, i in pairs]
    profs = vertical_profiles_batch([a for a, _ in prof_args])
    src = _source(config, surface_flux)
    cases = [(tower, i, _solver_kwargs(config, tower, z, p, src), met_step)
             for (tower, i), (z, p), (_, met_step) in zip(pairs, profs, prof_args)]
    out = [None] * len(cases)
    todo = []
    for k, (tower, i, kw, met_step) in enumerate(cases):
        hit = None
        if cache is not None:
            hit = cache.get(kw["z"], kw["profiles"], kw["domain"], kw["modes"], kw["meas_pt"], kw["halo"],
                            kw["precision"], **ckw)
        if hit is not None:
            grid, conc, flx = hit
            out[k] = _result(grid, conc, flx, tower, met_step)
        elif mode == "fp32" and not kw["analytic"]:
            todo.append(k)
        else:
            grid, conc, flx = steady_state_transport_solver(**kw, cache=cache, mode=mode)
            out[k] = _result(grid, conc, flx, tower, met_step)
    if todo:
        from .batch import solve_stream

        groups = [todo[a:a + batch] for a in range(0, len(todo), batch)]
        stream = solve_stream([[cases[k][2] for k in g] for g in groups])
        for g, res in zip(groups, stream):
            for k, (grid, conc, flx) in zip(g, res):
                tower, i, kw, met_step = cases[k]
                if cache is not None:
                    cache.put(kw["z"], kw["profiles"], kw["domain"], kw["modes"], kw["meas_pt"], kw["halo"],
                              kw["precision"], grid, conc, flx, **ckw)
                out[k] = _result(grid, conc, flx, tower, met_step)
    return out


def run_bldfm_timeseries(config, tower, surface_flux=None, *, mode="fp64", batch=64):
    """Every timestep of the met config for one tower (interface.py:141-174):
    one result dictionary per timestep.  The default ``mode="fp64"`` is the
    reference's arithmetic; ``mode="fp32"`` batches every timestep through the
    FP32 path (about 100x faster, relative L2 ~1e-6 from the exact discrete
    solution)."""
    n = config.met.n_timesteps
    logger.info("Running timeseries for tower '%s': %d timesteps", tower.name, n)
    return _run_cases(config, [(tower, i) for i in range(n)], surface_flux, mode, batch)


def run_bldfm_multitower(config, surface_flux=None, *, mode="fp64", batch=64):
    """Every tower and timestep (interface.py:177-208): tower name -> list of
    result dictionaries.  All towers' timesteps share the batches."""
    n = config.met.n_timesteps
    logger.info("Running multitower: %d towers x %d timesteps", len(config.towers), n)
    pairs = [(tower, i) for tower in config.towers for i in range(n)]
    flat = _run_cases(config, pairs, surface_flux, mode, batch)
    return {tower.name: flat[t * n:(t + 1) * n] for t, tower in enumerate(config.towers)}


def run_bldfm_parallel(config, max_workers=None, parallel_over="towers", surface_flux=None, *, mode="fp64",
                       batch=64):
    """The reference's process-pool runner (interface.py:244-326) as batched
    GPU launches: same result mapping as ``run_bldfm_multitower``.  The
    strategy only decides how the reference spreads work over processes, so
    every strategy gives the same batches here; as in the reference, an
    explicit ``surface_flux`` is ignored (each case uses the ideal source)."""
    if surface_flux is not None:
        warnings.warn("surface_flux is not passed to worker processes in parallel mode; each case uses the "
                      "configured ideal source. The provided array will be ignored.")
    if parallel_over not in ("towers", "time", "both"):
        raise ValueError(f"Unknown parallel_over={parallel_over!r}. Choose 'towers', 'time', or 'both'.")
    return run_bldfm_multitower(config, surface_flux=None, mode=mode, batch=batch)
