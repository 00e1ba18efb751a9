"""Advection phase with the reference's call surface (particle_advecter.py).

``uniform_particle_locations`` and ``distribute_particles_across_tiles`` keep the reference's
lattice and tiling semantics (particle_advecter.py:26-66). ``ParticleAdvecter`` keeps its
constructor, ``time_step`` and ``create_netcdf_file`` (particle_advecter.py:69-307), but the RK4
loop runs on the GPU (k_advect.cu) instead of inside Parcels, for all tiles at once: tiles only
shape the per-tile chunk files, as the reference's joblib workers do.

Differences by design: ``velocity_field`` is a VelocityField (the OSCAR download needs network
access); chunk files are plain pickles of the same dict {"time", "lat", "lon"} under the
reference's names; the particle state stays on the GPU between ``time_step`` calls (the
reference reloads the last stored, pre-kick positions from disk because its workers do not
return state; ``restore_from_disk`` does that explicitly).
"""

from __future__ import annotations

import glob
import logging
import os
import pickle
from concurrent.futures import ThreadPoolExecutor
from datetime import timedelta

import numpy as np
from numpy import linspace, repeat, tile

from .engine import Simulation
from .fields import VelocityField
from .ncio import write_particle_file
from .utils import most_symmetric_integer_factorization

logger = logging.getLogger(__name__)


def uniform_particle_locations(N_particles, lat_min, lat_max, lon_min, lon_max):
    """Regular lattice of N_particles positions (particle_advecter.py:26-35).

    The lattice is N_lat x N_lon with (N_lat, N_lon) = most_symmetric_integer_factorization(N);
    particle k = i_lon * N_lat + i_lat, latitude varying fastest; float64 degrees.
    """
    n_lat, n_lon = most_symmetric_integer_factorization(N_particles)
    logger.info("Generating (%d, %d) particles along each (lat, lon).", n_lat, n_lon)
    particle_lons = repeat(linspace(lon_min, lon_max, n_lon), n_lat)
    particle_lats = tile(linspace(lat_min, lat_max, n_lat), n_lon)
    return particle_lons, particle_lats


def distribute_particles_across_tiles(particle_lons, particle_lats, tiles):
    """Split into `tiles` contiguous equal views (particle_advecter.py:38-66)."""
    assert particle_lons.size == particle_lats.size
    n = particle_lons.size
    assert (n / tiles).is_integer()
    per = n // tiles
    lons = [particle_lons[i * per:(i + 1) * per] for i in range(tiles)]
    lats = [particle_lats[i * per:(i + 1) * per] for i in range(tiles)]
    return lons, lats


def _chunk_name(i0: int, i1: int, tile_id: int) -> str:
    return "particle_locations_" + str(i0).zfill(5) + "_" + str(i1).zfill(5) + "_tile" + str(tile_id).zfill(2) + ".pickle"


class ParticleAdvecter:
    def __init__(self, particle_lons, particle_lats, N_procs=-1, velocity_field="OSCAR", output_dir=".",
                 output_chunk_iters=100, Kh=0, device=0, seed=None):
        if isinstance(velocity_field, str):
            assert velocity_field == "OSCAR", "OSCAR is the only supported velocity field right now."
            raise NotImplementedError("the OSCAR field is fetched over OPeNDAP; pass a VelocityField "
                                      "(e.g. fields.synthetic_psi_field) instead")
        if not isinstance(velocity_field, VelocityField):
            raise TypeError("velocity_field must be a VelocityField")
        assert 1 <= N_procs or N_procs == -1, "Number of processors N_procs must be a positive integer " \
                                              "or -1 (use all processors)."
        max_procs = os.cpu_count() or 1
        N_procs = N_procs if 1 <= N_procs <= max_procs else max_procs
        particle_lons = np.asarray(particle_lons)
        particle_lats = np.asarray(particle_lats)
        assert particle_lons.size == particle_lats.size
        N_particles = particle_lons.size
        assert (N_particles / N_procs).is_integer()

        output_dir = os.path.abspath(output_dir)
        os.makedirs(output_dir, exist_ok=True)
        assert output_chunk_iters >= 1

        self._all_lons = np.ascontiguousarray(particle_lons, dtype=np.float64)
        self._all_lats = np.ascontiguousarray(particle_lats, dtype=np.float64)
        self.particle_lons, self.particle_lats = distribute_particles_across_tiles(self._all_lons, self._all_lats,
                                                                                  N_procs)
        self.iteration = 0
        self.velocity_field = velocity_field
        self.N_particles = N_particles
        self.N_procs = N_procs
        self.particles_per_tile = N_particles // N_procs
        self.output_dir = output_dir
        self.output_chunk_iters = output_chunk_iters
        self.Kh = Kh / 1e10  # m^2/s -> deg^2/s with 1 deg = 100 km, the reference's conversion
        if seed is None:
            seed = int(np.random.randint(0, np.iinfo(np.int64).max, dtype=np.int64))
        self.seed = int(seed)
        self.device = device
        self._sim = None
        self._records = None

    def _engine(self) -> Simulation:
        if self._sim is None:
            self._sim = Simulation(self.velocity_field, self._all_lons, self._all_lats, None, radius=0.0,
                                   seed=self.seed, kh=self.Kh, device=self.device)
        return self._sim

    def _write_chunk(self, out, times, iteration, iters_to_do):
        """The per-tile pickles of one chunk (particle_advecter.py:246-249's file names and dicts)."""
        per = self.particles_per_tile
        for tile_id in range(self.N_procs):
            chunk = {"time": times, "lat": np.ascontiguousarray(out["lat"][:, tile_id * per:(tile_id + 1) * per]),
                     "lon": np.ascontiguousarray(out["lon"][:, tile_id * per:(tile_id + 1) * per])}
            path = os.path.join(self.output_dir, _chunk_name(iteration, iteration + iters_to_do, tile_id))
            with open(path, "wb") as f:
                pickle.dump(chunk, f, protocol=pickle.HIGHEST_PROTOCOL)

    def time_step(self, start_time, end_time, dt):
        """Advect for (end_time - start_time) // dt steps, writing a chunk of positions every
        output_chunk_iters steps. Chunk k is pickled by a writer thread while the GPU computes chunk
        k + 1 (at most one chunk waits to be written); within a chunk, each step's positions are
        copied to the host while the next steps compute."""
        sim = self._engine()
        logger.info("Starting time stepping: %s -> %s (dt=%s) on the GPU.", start_time, end_time, dt)
        t = start_time
        iteration = self.iteration
        # two page-locked record buffers, reused from chunk to chunk: the GPU fills one while the
        # writer pickles the other, and each step's copy overlaps the next steps
        if self._records is None:
            self._records = [sim.record_buffers(self.output_chunk_iters) for _ in range(2)]
        chunk = 0
        with ThreadPoolExecutor(max_workers=1) as writer:
            pending = None
            while t < end_time:
                iters_to_do = min(self.output_chunk_iters, (end_time - t) // dt)
                out = sim.step(t, dt, iters_to_do, interact=False, record=True, step0=iteration,
                               out=self._records[chunk % 2])
                chunk += 1
                times = [t + (n + 1) * dt for n in range(iters_to_do)]
                if pending is not None:
                    pending.result()  # raises what the writer raised
                pending = writer.submit(self._write_chunk, out, times, iteration, iters_to_do)
                t = t + iters_to_do * dt
                iteration += iters_to_do
            if pending is not None:
                pending.result()
        self.iteration += (end_time - start_time) // dt

    def newest_stored_positions(self):
        """The last stored row of every tile from the newest chunk on disk, and the iteration that
        chunk ends at (the reference's re-entry restore, particle_advecter.py:124-138).

        The reference takes the newest N_procs files by name; when a tile's file of the newest
        chunk is missing, that mixes positions of different times. Here the newest chunk must hold
        one readable file per tile with [iterations, particles per tile] positions; anything else
        raises (FileNotFoundError for missing files, ValueError for unreadable or misshapen ones).
        """
        files = glob.glob(os.path.join(self.output_dir, "particle_locations_*.pickle"))
        if not files:
            raise FileNotFoundError(f"no particle_locations_*.pickle in {self.output_dir}")
        chunks = {}
        for path in files:
            parts = os.path.basename(path)[: -len(".pickle")].split("_")
            try:
                i0, i1, tile_id = int(parts[2]), int(parts[3]), int(parts[4][4:])
            except (IndexError, ValueError):
                raise ValueError(f"not a chunk file name: {os.path.basename(path)}") from None
            chunks.setdefault((i0, i1), {})[tile_id] = path
        i0, i1 = max(chunks, key=lambda span: (span[1], span[0]))
        tiles = chunks[(i0, i1)]
        missing = [t for t in range(self.N_procs) if t not in tiles]
        if missing:
            raise FileNotFoundError(f"chunk {i0:05d}-{i1:05d} in {self.output_dir} has no file for tile(s) {missing}")
        per = self.particles_per_tile
        lons = self._all_lons.copy()
        lats = self._all_lats.copy()
        for tile_id in range(self.N_procs):
            path = tiles[tile_id]
            try:
                with open(path, "rb") as f:
                    chunk = pickle.load(f)
                lon, lat = np.asarray(chunk["lon"]), np.asarray(chunk["lat"])
            except Exception as e:  # truncated or corrupt pickle, or a dict without positions
                raise ValueError(f"unreadable chunk file {path}: {type(e).__name__}: {e}") from e
            if lon.ndim != 2 or lon.shape[1] != per or lat.shape != lon.shape or lon.shape[0] < 1:
                raise ValueError(f"{path}: expected [iterations, {per}] positions, found lon {lon.shape}, "
                                 f"lat {lat.shape}")
            lons[tile_id * per:(tile_id + 1) * per] = lon[-1, :]
            lats[tile_id * per:(tile_id + 1) * per] = lat[-1, :]
        return lons, lats, i1

    def restore_from_disk(self) -> int:
        """Continue from the newest stored chunk (e.g. after the process that wrote it was killed):
        upload its last positions and continue the iteration count where it ends. Returns that
        iteration."""
        lons, lats, it = self.newest_stored_positions()
        self._engine().upload_particles(lons, lats, None)
        self.iteration = it
        return it

    def create_netcdf_file(self, start_time, end_time, dt):
        iters = (end_time - start_time) // dt
        plons = np.zeros((self.N_particles, iters), dtype=np.float32)
        plats = np.zeros((self.N_particles, iters), dtype=np.float32)
        files = sorted(glob.glob(os.path.join(self.output_dir, "particle_locations_*.pickle")))
        for path in files:
            parts = os.path.basename(path).split("_")
            t1, t2, tile_id = int(parts[2]), int(parts[3]), int(parts[4][4:6])
            with open(path, "rb") as f:
                chunk = pickle.load(f)
            i1, i2 = tile_id * self.particles_per_tile, (tile_id + 1) * self.particles_per_tile
            plons[i1:i2, t1:t2] = np.transpose(chunk["lon"])
            plats[i1:i2, t1:t2] = np.transpose(chunk["lat"])
        times_s = np.array([(n * dt) / timedelta(seconds=1) for n in range(iters)], dtype=np.float64)
        nc_path = os.path.join(self.output_dir, "particle_data.nc")
        write_particle_file(nc_path, {"longitude": plons, "latitude": plats}, start_time, times_s)
        for path in files:
            os.remove(path)
