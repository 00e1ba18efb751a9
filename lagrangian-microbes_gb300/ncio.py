"""NetCDF3 files of the two-phase workflow (particle_data.nc, microbe_data.nc).

The reference writes them with xarray (particle_advecter.py:262-307,
interaction_simulator.py:119-122): variables [particle number, time] float32 longitude/latitude
(+ int8 species), coordinates "particle number" = 1..N and time. Here they are written with
scipy.io.netcdf_file (NetCDF3, 64-bit offsets); time is stored as float64 seconds since the run
start with a CF "units" attribute.
"""

from __future__ import annotations

from datetime import datetime

import numpy as np
from scipy.io import netcdf_file

PARTICLE_DIM = "particle number"
TIME_DIM = "time"


def write_particle_file(path: str, variables: dict, start: datetime, times_s: np.ndarray) -> None:
    """variables: name -> [N, Nt] array (float32 or int8)."""
    first = next(iter(variables.values()))
    n, nt = first.shape
    with netcdf_file(path, "w", version=2) as f:
        f.createDimension(PARTICLE_DIM, n)
        f.createDimension(TIME_DIM, nt)
        pn = f.createVariable(PARTICLE_DIM, "i4", (PARTICLE_DIM,))
        pn[:] = np.arange(1, n + 1, dtype=np.int32)
        tv = f.createVariable(TIME_DIM, "f8", (TIME_DIM,))
        tv[:] = np.asarray(times_s, dtype=np.float64)
        tv.units = "seconds since " + start.strftime("%Y-%m-%d %H:%M:%S")
        for name, arr in variables.items():
            code = {np.dtype(np.float32): "f4", np.dtype(np.int8): "b", np.dtype(np.float64): "f8"}[arr.dtype]
            var = f.createVariable(name, code, (PARTICLE_DIM, TIME_DIM))
            var[:] = arr


def read_particle_file(path: str) -> dict:
    """name -> numpy array in native byte order (NetCDF stores big-endian) for every variable."""
    out = {}
    with netcdf_file(path, "r", mmap=False) as f:
        for name, var in f.variables.items():
            a = np.array(var[:])
            out[name] = a.astype(a.dtype.newbyteorder("="), copy=False)
    return out
