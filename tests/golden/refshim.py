"""Import the reference BLDFM solver in a container that lacks its third-party deps.

Test infrastructure only: used by ``make_golden.py`` (fixture generation) and by
CPU cross-checks that skip themselves when the reference tree is absent.

The reference imports ``numba`` (JIT of ``ivp_solver``, src/bldfm/utils.py:95-106),
``pyfftw`` (src/bldfm/fft_manager.py:1-3), the private ``abltk`` package
(logging/config, src/bldfm/config.py:11-12) and ``yaml``.  None of these is
installed, so stub modules are placed in ``sys.modules`` before import:

* ``numba.jit`` is the identity decorator, so ``ivp_solver`` runs as plain
  numpy (same arithmetic as the JIT without fastmath: no FMA contraction);
* ``pyfftw.interfaces.numpy_fft.fft2/ifft2`` forward to ``numpy.fft``;
* ``abltk.logging.get_logger`` is ``logging.getLogger``;
* ``abltk.plotting.geo.latlon_to_xy`` is an equirectangular projection
  (R = 6371000 m, x scaled by cos(ref_lat)).
"""

import logging
import math
import os
import sys
import types

# The reference's src/ directory: BLDFM_REFERENCE_SRC, else the location of the
# read-only reference checkout in the build container.  The GPU machines have
# no reference tree; everything that imports it skips itself there
# (reference_available()).
REFERENCE_SRC = os.environ.get("BLDFM_REFERENCE_SRC", "/root/reference/src")


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE_SRC, "bldfm", "solver.py"))


def _install_stubs():
    if "numba" not in sys.modules or not hasattr(sys.modules["numba"], "_bldfm_stub"):
        numba = types.ModuleType("numba")
        numba._bldfm_stub = True

        def jit(*args, **kwargs):
            if len(args) == 1 and callable(args[0]) and not kwargs:
                return args[0]
            return lambda f: f

        numba.jit = jit
        numba.njit = jit
        numba.set_num_threads = lambda n: None
        numba.prange = range
        sys.modules["numba"] = numba

    import numpy as np

    pyfftw = types.ModuleType("pyfftw")
    interfaces = types.ModuleType("pyfftw.interfaces")
    numpy_fft = types.ModuleType("pyfftw.interfaces.numpy_fft")
    numpy_fft.fft2 = lambda a, norm="backward", **kw: np.fft.fft2(a, norm=norm)
    numpy_fft.ifft2 = lambda a, norm="backward", **kw: np.fft.ifft2(a, norm=norm)
    cache = types.ModuleType("pyfftw.interfaces.cache")
    cache.enable = lambda: None
    cache.disable = lambda: None
    cache.set_keepalive_time = lambda t: None
    interfaces.numpy_fft = numpy_fft
    interfaces.cache = cache
    pyfftw.interfaces = interfaces
    pyfftw.config = types.SimpleNamespace(NUM_THREADS=1)
    pyfftw.import_wisdom = lambda w: [True]
    pyfftw.export_wisdom = lambda: ()
    sys.modules.update(
        {
            "pyfftw": pyfftw,
            "pyfftw.interfaces": interfaces,
            "pyfftw.interfaces.numpy_fft": numpy_fft,
            "pyfftw.interfaces.cache": cache,
        }
    )

    abltk = types.ModuleType("abltk")
    alog = types.ModuleType("abltk.logging")
    alog.get_logger = lambda name=None: logging.getLogger("refshim." + str(name))
    alog.setup_logging = lambda **kw: None
    acfg = types.ModuleType("abltk.config")
    acfg.init = lambda root: None
    for key in ("DATA_DIR", "CACHE_DIR", "CONFIG_DIR", "OUTPUT_DIR", "LOG_DIR"):
        setattr(acfg, key, "/tmp/bldfm_refshim")
    aplot = types.ModuleType("abltk.plotting")
    ageo = types.ModuleType("abltk.plotting.geo")

    def latlon_to_xy(lat, lon, ref_lat, ref_lon):
        r_earth = 6371000.0
        x = r_earth * math.radians(lon - ref_lon) * math.cos(math.radians(ref_lat))
        y = r_earth * math.radians(lat - ref_lat)
        return x, y

    ageo.latlon_to_xy = latlon_to_xy
    aplot.geo = ageo
    abltk.logging = alog
    abltk.config = acfg
    abltk.plotting = aplot
    sys.modules.update(
        {
            "abltk": abltk,
            "abltk.logging": alog,
            "abltk.config": acfg,
            "abltk.plotting": aplot,
            "abltk.plotting.geo": ageo,
        }
    )
    if "yaml" not in sys.modules:
        try:
            import yaml  # noqa: F401
        except ImportError:
            ymod = types.ModuleType("yaml")
            ymod.safe_load = lambda s: {}
            ymod.safe_dump = lambda d, **kw: ""
            sys.modules["yaml"] = ymod


def import_reference():
    """Return the reference ``bldfm`` package (solver, pbl_model, utils loaded)."""
    if not reference_available():
        raise ImportError("reference BLDFM sources not found at " + REFERENCE_SRC)
    sys.dont_write_bytecode = True
    _install_stubs()
    if REFERENCE_SRC not in sys.path:
        sys.path.insert(0, REFERENCE_SRC)
    import bldfm  # noqa: F401
    import bldfm.solver
    import bldfm.pbl_model
    import bldfm.utils

    return bldfm
