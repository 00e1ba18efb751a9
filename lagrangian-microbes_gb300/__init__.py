"""GB300-native hot path of lagrangian-microbes: advect (RK4) -> bin -> pair -> interact.

Reference-facing modules (same names and call surface as ali-ramadhan/lagrangian-microbes):
  particle_advecter      uniform_particle_locations, distribute_particles_across_tiles, ParticleAdvecter
  interactions           ROCK/PAPER/SCISSORS, rock_paper_scissors, rock_paper_scissors_interaction
  interaction_simulator  InteractionSimulator
Device-resident engine:
  engine                 Simulation (fused steps, CUDA graphs), PairQuery (cKDTree.query_pairs)
  fields                 VelocityField, synthetic_psi_field
  pairwise_distance_histogram   species / all-pairs great-circle distance histograms
All compute runs in liblmgb300.so (CUDA, sm_103a) through the C-ABI of include/lm_api.h.
"""

from . import _lib, build, fields, utils
from ._lib import LMError, OutOfBoundsError, TimeRangeError
from .fields import VelocityField, synthetic_psi_field, uniform_field
from .interactions import PAPER, ROCK, SCISSORS, rock_paper_scissors, rock_paper_scissors_interaction
from .utils import factor, most_symmetric_integer_factorization

__all__ = [
    "LMError", "OutOfBoundsError", "TimeRangeError", "VelocityField", "synthetic_psi_field", "uniform_field",
    "ROCK", "PAPER", "SCISSORS", "rock_paper_scissors", "rock_paper_scissors_interaction", "factor",
    "most_symmetric_integer_factorization", "Simulation", "PairQuery", "ParticleAdvecter", "InteractionSimulator",
    "uniform_particle_locations", "distribute_particles_across_tiles", "build", "fields", "utils",
]


def __getattr__(name):
    # engine-backed names import lazily so that `import lagrangian_microbes_gb300` never needs a GPU
    if name in ("Simulation", "PairQuery"):
        from . import engine
        return getattr(engine, name)
    if name in ("ParticleAdvecter", "uniform_particle_locations", "distribute_particles_across_tiles"):
        from . import particle_advecter
        return getattr(particle_advecter, name)
    if name == "InteractionSimulator":
        from . import interaction_simulator
        return interaction_simulator.InteractionSimulator
    raise AttributeError(name)
