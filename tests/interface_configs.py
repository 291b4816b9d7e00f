"""Small configuration objects with the attributes the reference's config
classes carry (src/bldfm/config_parser.py: TowerConfig, DomainConfig,
MetConfig, SolverConfig, ParallelConfig, BLDFMConfig), for the runner tests."""

from types import SimpleNamespace


class Met:
    def __init__(self, ustar=None, mol=1e9, wind_speed=5.0, wind_dir=270.0, z0=None, timestamps=None):
        self.ustar, self.mol, self.wind_speed, self.wind_dir = ustar, mol, wind_speed, wind_dir
        self.z0, self.timestamps = z0, timestamps

    @property
    def n_timesteps(self):
        if isinstance(self.ustar, list):
            return len(self.ustar)
        if isinstance(self.wind_speed, list):
            return len(self.wind_speed)
        return 1

    def get_step(self, i):
        pick = lambda v: None if v is None else (v[i] if isinstance(v, list) else v)  # noqa: E731
        out = {"ustar": pick(self.ustar), "mol": pick(self.mol), "wind_speed": pick(self.wind_speed),
               "wind_dir": pick(self.wind_dir)}
        if self.z0 is not None:
            out["z0"] = self.z0
        out["timestamp"] = self.timestamps[i] if self.timestamps is not None else i
        return out


def config(n_steps=3, towers=2, nxy=(96, 64), modes=(96, 64), nz=16, footprint=True, output_levels=None,
           full_output=False, z0=None, use_cache=False):
    met = Met(ustar=[0.25 + 0.05 * i for i in range(n_steps)] if z0 is None else None,
              mol=[-60.0 - 10.0 * i for i in range(n_steps)], wind_speed=[3.0 + 0.5 * i for i in range(n_steps)],
              wind_dir=[200.0 + 20.0 * i for i in range(n_steps)], z0=z0)
    dom = SimpleNamespace(nx=nxy[0], ny=nxy[1], xmax=480.0, ymax=320.0, nz=nz, modes=modes, halo=None,
                          output_levels=output_levels, full_output=full_output)
    sol = SimpleNamespace(closure="MOST", precision="double", footprint=footprint, surface_flux_shape="diamond",
                          src_loc=None, analytic=False)
    tw = [SimpleNamespace(name="T%d" % k, x=150.0 + 60.0 * k, y=120.0 + 30.0 * k, z_m=8.0 + 4.0 * k)
          for k in range(towers)]
    par = SimpleNamespace(max_workers=2, use_cache=use_cache, num_threads=1)
    return SimpleNamespace(domain=dom, solver=sol, met=met, towers=tw, parallel=par)
