"""GB300-native BLDFM steady-state transport solve (drop-in for the reference's
``steady_state_transport_solver``; see include/bldfm_gb300.h for the C ABI)."""

from .solver import steady_state_transport_solver
from .utils import compute_wind_fields, ideal_source, point_measurement


def vertical_profiles(*args, **kwargs):
    from .pbl_model import vertical_profiles as _vp

    return _vp(*args, **kwargs)


__all__ = [
    "steady_state_transport_solver",
    "vertical_profiles",
    "compute_wind_fields",
    "ideal_source",
    "point_measurement",
]
