"""Gridded velocity fields for the advection path.

``VelocityField`` is the in-memory stand-in for the OSCAR dataset that the reference downloads
over OPeNDAP (velocity_fields.py:12-32) and wraps in a Parcels RectilinearZGrid / Field /
FieldSet (particle_advecter.py:160-184): float32 u, v in m/s on an ascending, uniformly spaced
lon/lat grid, with frames on a uniform time axis.

``synthetic_psi_field`` builds the seeded synthetic field used by the tests and the benchmark:
a streamfunction made of random Fourier modes on a local tangent plane, u = -dpsi/dy,
v = dpsi/dx (analytic derivatives), scaled to a given rms speed at t = 0, with every mode's phase
advancing by 2*pi per ``period_days``.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from datetime import datetime, timedelta

import numpy as np

EARTH_RADIUS_KM = 6371.228  # the sphere radius of the reference's haversine tools


@dataclass
class VelocityField:
    lon: np.ndarray  # [nx] float64, degrees east, ascending, uniform
    lat: np.ndarray  # [ny] float64, degrees north, ascending, uniform
    times: np.ndarray  # [nt] float64, seconds since `epoch`, ascending, uniform
    u: np.ndarray  # [nt, ny, nx] float32, m/s
    v: np.ndarray  # [nt, ny, nx] float32, m/s
    epoch: datetime = field(default_factory=lambda: datetime(2017, 1, 1))

    def __post_init__(self):
        self.lon = np.ascontiguousarray(self.lon, dtype=np.float64)
        self.lat = np.ascontiguousarray(self.lat, dtype=np.float64)
        self.times = np.ascontiguousarray(self.times, dtype=np.float64)
        self.u = np.ascontiguousarray(self.u, dtype=np.float32)
        self.v = np.ascontiguousarray(self.v, dtype=np.float32)
        nt, ny, nx = self.u.shape
        if self.v.shape != self.u.shape or (nx, ny, nt) != (self.lon.size, self.lat.size, self.times.size):
            raise ValueError("u, v must be [nt, ny, nx] matching times, lat, lon")
        if self.lat.size > 1 and self.lat[1] < self.lat[0]:  # OSCAR stores latitude descending
            self.lat = self.lat[::-1].copy()
            self.u = np.ascontiguousarray(self.u[:, ::-1, :])
            self.v = np.ascontiguousarray(self.v[:, ::-1, :])

    @property
    def shape(self):
        return self.u.shape

    def seconds(self, when) -> float:
        """Field-clock seconds of a datetime (or pass-through for numbers)."""
        if isinstance(when, datetime):
            return (when - self.epoch).total_seconds()
        return float(when)

    @property
    def nbytes(self) -> int:
        return self.u.nbytes + self.v.nbytes


@dataclass
class PsiModes:
    """The random modes of a synthetic streamfunction (enough to re-evaluate it anywhere)."""

    kx: np.ndarray  # rad/m
    ky: np.ndarray
    phase: np.ndarray
    amp: np.ndarray  # psi amplitude (m^2/s), already scaled
    lon0: float
    lat0: float
    omega: float  # rad/s
    radius_m: float

    def velocity(self, lon, lat, t):
        """Analytic (u, v) in m/s at float64 lon/lat (degrees) and time t (s)."""
        lon = np.asarray(lon, dtype=np.float64)
        lat = np.asarray(lat, dtype=np.float64)
        x = self.radius_m * np.cos(np.deg2rad(self.lat0)) * np.deg2rad(lon - self.lon0)
        y = self.radius_m * np.deg2rad(lat - self.lat0)
        th = self.kx * x[..., None] + self.ky * y[..., None] + self.phase + self.omega * t
        s = np.sin(th)
        return (self.amp * self.ky * s).sum(-1), (-self.amp * self.kx * s).sum(-1)


@dataclass
class PsiBasis:
    """A seeded synthetic field before it is sampled in time: every frame is a mix of four basis
    fields, u(t) = us cos(w t) + uc sin(w t), v(t) = vs cos(w t) + vc sin(w t). ``frames(first, n)``
    samples frames first .. first + n - 1 (times frame_seconds * k), bit-identical to the same frames
    of one long sampling, so a long run can stream its field in windows."""

    lon: np.ndarray
    lat: np.ndarray
    us: np.ndarray
    uc: np.ndarray
    vs: np.ndarray
    vc: np.ndarray
    omega: float
    frame_seconds: float
    epoch: datetime
    modes: PsiModes

    def frames(self, first: int, n_frames: int) -> VelocityField:
        ny, nx = self.us.shape
        times = self.frame_seconds * np.arange(first, first + n_frames, dtype=np.float64)
        u = np.empty((n_frames, ny, nx), dtype=np.float32)
        v = np.empty((n_frames, ny, nx), dtype=np.float32)
        chunk = max(1, int(4e6 // (nx * ny)))
        for f0 in range(0, n_frames, chunk):
            f1 = min(n_frames, f0 + chunk)
            c = np.cos(self.omega * times[f0:f1])[:, None, None]
            s = np.sin(self.omega * times[f0:f1])[:, None, None]
            u[f0:f1] = self.us * c + self.uc * s
            v[f0:f1] = self.vs * c + self.vc * s
        return VelocityField(lon=self.lon, lat=self.lat, times=times, u=u, v=v, epoch=self.epoch)


def psi_basis(lon_min: float, lon_max: float, lat_min: float, lat_max: float, resolution: float,
              frame_seconds: float = 3600.0, n_modes: int = 32, wavelength_km=(50.0, 500.0), rms_speed: float = 0.2,
              period_days: float = 10.0, seed: int = 0, epoch: datetime | None = None) -> PsiBasis:
    """The basis fields of synthetic_psi_field (same arguments, same seed -> same field)."""
    rng = np.random.default_rng(seed)
    nx = int(round((lon_max - lon_min) / resolution)) + 1
    ny = int(round((lat_max - lat_min) / resolution)) + 1
    lon = lon_min + resolution * np.arange(nx, dtype=np.float64)
    lat = lat_min + resolution * np.arange(ny, dtype=np.float64)
    lon0 = 0.5 * (lon_min + lon_max)
    lat0 = 0.5 * (lat_min + lat_max)
    radius_m = EARTH_RADIUS_KM * 1e3
    x = radius_m * np.cos(np.deg2rad(lat0)) * np.deg2rad(lon - lon0)  # [nx]
    y = radius_m * np.deg2rad(lat - lat0)  # [ny]

    lo, hi = np.log(wavelength_km[0] * 1e3), np.log(wavelength_km[1] * 1e3)
    wl = np.exp(rng.uniform(lo, hi, n_modes))
    k = 2 * np.pi / wl
    theta = rng.uniform(0, 2 * np.pi, n_modes)
    phase = rng.uniform(0, 2 * np.pi, n_modes)
    kx, ky = k * np.cos(theta), k * np.sin(theta)
    amp = 1.0 / k

    # psi = sum amp cos(a + w t), a = kx x + ky y + phase; u = -dpsi/dy, v = dpsi/dx.
    # sin(a + w t) = sin(a) cos(w t) + cos(a) sin(w t): every frame is a mix of four basis fields.
    us = np.zeros((ny, nx)); uc = np.zeros((ny, nx)); vs = np.zeros((ny, nx)); vc = np.zeros((ny, nx))
    for m in range(n_modes):
        ex = np.exp(1j * (kx[m] * x + phase[m]))  # [nx]
        ey = np.exp(1j * (ky[m] * y))  # [ny]
        e = ey[:, None] * ex[None, :]
        sa, ca = e.imag, e.real
        us += amp[m] * ky[m] * sa
        uc += amp[m] * ky[m] * ca
        vs -= amp[m] * kx[m] * sa
        vc -= amp[m] * kx[m] * ca
    scale = rms_speed / np.sqrt(np.mean(us * us + vs * vs))
    us *= scale; uc *= scale; vs *= scale; vc *= scale
    omega = 2 * np.pi / (period_days * 86400.0)
    modes = PsiModes(kx=kx, ky=ky, phase=phase, amp=amp * scale, lon0=lon0, lat0=lat0, omega=omega, radius_m=radius_m)
    return PsiBasis(lon=lon, lat=lat, us=us, uc=uc, vs=vs, vc=vc, omega=omega, frame_seconds=frame_seconds,
                    epoch=epoch or datetime(2017, 1, 1), modes=modes)


def synthetic_psi_field(lon_min: float, lon_max: float, lat_min: float, lat_max: float, resolution: float,
                        n_frames: int, frame_seconds: float = 3600.0, n_modes: int = 32,
                        wavelength_km=(50.0, 500.0), rms_speed: float = 0.2, period_days: float = 10.0,
                        seed: int = 0, epoch: datetime | None = None, with_modes: bool = False):
    """Seeded streamfunction field sampled on a regular lon/lat grid.

    Wavelengths are log-uniform in ``wavelength_km``, directions and phases uniform; every mode has
    the same velocity amplitude (psi amplitude proportional to its wavelength). Coordinates are a
    local tangent plane at the domain centre: x = R cos(lat0) dlon, y = R dlat.
    """
    basis = psi_basis(lon_min, lon_max, lat_min, lat_max, resolution, frame_seconds, n_modes, wavelength_km,
                      rms_speed, period_days, seed, epoch)
    fld = basis.frames(0, n_frames)
    return (fld, basis.modes) if with_modes else fld


def uniform_field(lon_min, lon_max, lat_min, lat_max, resolution, n_frames, u0=0.2, v0=0.0,
                  frame_seconds=3600.0, epoch=None) -> VelocityField:
    """Constant (u0, v0) m/s everywhere: the known-answer case of the advection tests."""
    nx = int(round((lon_max - lon_min) / resolution)) + 1
    ny = int(round((lat_max - lat_min) / resolution)) + 1
    lon = lon_min + resolution * np.arange(nx)
    lat = lat_min + resolution * np.arange(ny)
    u = np.full((n_frames, ny, nx), u0, np.float32)
    v = np.full((n_frames, ny, nx), v0, np.float32)
    return VelocityField(lon, lat, frame_seconds * np.arange(n_frames), u, v, epoch or datetime(2017, 1, 1))


def field_time_window(fld: VelocityField, start: datetime, n_steps: int, dt: timedelta):
    """(t0 seconds, dt seconds) of a run on the field clock, checked against the time axis."""
    t0 = fld.seconds(start)
    dts = dt.total_seconds()
    t1 = t0 + n_steps * dts
    if min(t0, t1) < fld.times[0] - 1e-6 or max(t0, t1) > fld.times[-1] + 1e-6:
        raise ValueError(f"run [{t0}, {t1}] s lies outside the field's [{fld.times[0]}, {fld.times[-1]}] s")
    return t0, dts
