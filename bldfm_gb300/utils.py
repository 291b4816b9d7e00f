"""Small helpers of the reference's src/bldfm/utils.py (host arithmetic).

``compute_wind_fields`` (utils.py:7-27) and ``ideal_source`` (utils.py:30-77)
produce solver inputs; ``point_measurement`` (utils.py:80-92) is the
footprint-weighted sum.  They are O(nx*ny) host numpy, as in the reference.
"""

import numpy as np


def compute_wind_fields(u_rot, wind_dir):
    wind_dir = np.deg2rad(wind_dir)
    return -u_rot * np.sin(wind_dir), -u_rot * np.cos(wind_dir)


def ideal_source(nxy, domain, src_loc=None, shape="diamond"):
    nx, ny = nxy
    xmx, ymx = domain
    dx = xmx / nx
    if src_loc is None:
        src_loc = (xmx / 2, ymx / 2)
    xs, ys = src_loc
    X, Y = np.meshgrid(np.linspace(0.0, xmx, nx), np.linspace(0.0, ymx, ny))
    q0 = np.zeros([ny, nx])
    if shape == "diamond":
        q0 = np.where(np.abs(X - xs) + np.abs(Y - ys) < xmx / 12, 1.0, 0.0)
    if shape == "circle":
        q0 = np.where(np.sqrt((X - xs) ** 2 + (Y - ys) ** 2) < xmx / 12, 1.0, 0.0)
    if shape == "point":
        sig = 4.0 * dx
        q0 = np.exp(-((X - xs) ** 2 + (Y - ys) ** 2) / 2.0 / sig**2) / sig / np.sqrt(2.0 * np.pi)
    return q0


def point_measurement(f, g):
    return np.sum(f * g)
