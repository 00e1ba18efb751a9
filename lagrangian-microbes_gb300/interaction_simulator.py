"""Interaction phase with the reference's call surface (interaction_simulator.py).

``InteractionSimulator(pair_interaction, interaction_radius, interaction_norm=2, ...)`` replays
the positions of particle_data.nc step by step like the reference (interaction_simulator.py:54-122),
but each step is one GPU call (lm_interact): cell binning + fixed-radius pair search with
cKDTree.query_pairs semantics + the rock-paper-scissors rounds, with the species array updated in
place. Only the rock_paper_scissors pair rule is supported (a GPU kernel, not a Python callable);
any other pair function raises NotImplementedError.
"""

from __future__ import annotations

import logging
import os
from datetime import timedelta

import numpy as np

from . import _lib
from .engine import norm_code
from .interactions import rock_paper_scissors_interaction
from .ncio import read_particle_file, write_particle_file

logger = logging.getLogger(__name__)


class InteractionSimulator:
    def __init__(self, pair_interaction, interaction_radius, interaction_norm=2, self_interaction=None,
                 advection_dir=".", output_dir=".", device=0):
        output_dir = os.path.abspath(output_dir)
        os.makedirs(output_dir, exist_ok=True)
        pair_interaction_function, pair_interaction_parameters, microbe_properties = pair_interaction
        if pair_interaction_function is not rock_paper_scissors_interaction:
            raise NotImplementedError("only the rock_paper_scissors pair rule runs on the GPU")
        self._norm = norm_code(interaction_norm)
        self.microbe_properties = microbe_properties
        self.pair_interaction = pair_interaction_function
        self.pair_interaction_parameters = pair_interaction_parameters
        self.interaction_radius = interaction_radius
        self.interaction_norm = interaction_norm
        self.self_interaction = self_interaction
        self.advection_dir = advection_dir
        self.output_dir = output_dir
        self.iteration = 0
        self.device = device
        self._ctx = None

    def _context(self) -> _lib.Context:
        if self._ctx is None:
            self._ctx = _lib.Context(self.device)
        p = self.pair_interaction_parameters
        seed = int(p.get("seed", 0)) & 0xFFFFFFFFFFFFFFFF
        self._ctx.call("lm_set_interaction", float(self.interaction_radius), self._norm, float(p["pRS"]),
                       float(p["pPR"]), float(p["pSP"]), seed)
        return self._ctx

    def time_step(self, start_time, end_time, dt):
        data = read_particle_file(os.path.join(self.advection_dir, "particle_data.nc"))
        plon, plat = data["longitude"], data["latitude"]
        N_particles, Nt = plon.shape
        mlons = np.zeros((N_particles, Nt), dtype=np.float32)
        mlats = np.zeros((N_particles, Nt), dtype=np.float32)
        species_rec = np.zeros((N_particles, Nt), dtype=np.int8)

        ctx = self._context()
        species = self.microbe_properties["species"]
        if species.dtype != np.int8 or species.size != N_particles:
            raise ValueError("species must be int8 with one entry per particle of particle_data.nc")
        sp = np.ascontiguousarray(species)
        ctx.call("lm_species_upload", N_particles, _lib.ptr(sp))

        logger.info("Simulating interactions for %d microbes over %d time steps (%s -> %s).", N_particles, Nt,
                    start_time, end_time)
        t = start_time
        while t < end_time:
            i = self.iteration
            lon = np.ascontiguousarray(plon[:, i], dtype=np.float32)
            lat = np.ascontiguousarray(plat[:, i], dtype=np.float32)
            ctx.call("lm_interact", N_particles, _lib.ptr(lon), _lib.ptr(lat), i, 0)
            ctx.call("lm_particles_download", None, None, _lib.ptr(sp), None)
            species[...] = sp  # in place, as the reference's pair function mutates it
            mlons[:, i] = lon
            mlats[:, i] = lat
            species_rec[:, i] = sp
            t = t + dt
            self.iteration += 1

        times_s = np.array([(n * dt) / timedelta(seconds=1) for n in range(Nt)], dtype=np.float64)
        write_particle_file(os.path.join(self.output_dir, "microbe_data.nc"),
                            {"longitude": mlons, "latitude": mlats, "species": species_rec}, start_time, times_s)
