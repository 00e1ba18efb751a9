"""Rock-paper-scissors interaction with the reference's call surface (interactions.py).

``rock_paper_scissors(N, pRS, pPR, pSP)`` returns the same triple as the reference
(interactions.py:43-54): the pair function, the parameter dict and the properties dict holding the
int8 species array (ROCK=1, PAPER=2, SCISSORS=3, drawn i.i.d. uniform from numpy's global RNG).
InteractionSimulator recognises the returned pair function and applies the rule to every pair of
a step on the GPU (k_rounds.cu). The function object itself is only an identifier: the per-pair
Python call of the reference (interaction_simulator.py:104-105) has no counterpart here, so
calling it raises.
"""

from __future__ import annotations

import numpy as np
from numpy import int8

ROCK, PAPER, SCISSORS = int8(1), int8(2), int8(3)

ROCK_COLOR = "red"
PAPER_COLOR = "limegreen"
SCISSORS_COLOR = "blue"


def rock_paper_scissors_interaction(parameters, microbe_properties, p1, p2):
    """Identifier of the rock-paper-scissors pair rule (interactions.py:13-40).

    The rule: if species differ, r ~ U[0,1); the cyclic winner (rock beats scissors, paper beats
    rock, scissors beats paper) wins with probability pRS / pPR / pSP of its matchup, otherwise the
    other microbe wins; the loser takes the winner's species. InteractionSimulator runs it for all
    pairs of a step at once on the GPU.
    """
    raise NotImplementedError(
        "rock_paper_scissors_interaction is applied to whole pair sets on the GPU by InteractionSimulator; "
        "single-pair host calls are not supported")


rock_paper_scissors_interaction.lm_rule = "rock_paper_scissors"


def rock_paper_scissors(N_microbes, pRS, pPR, pSP, seed=None):
    """(pair function, parameters, properties) for N_microbes rock-paper-scissors microbes.

    ``seed`` keys the Philox stream of the per-pair uniforms; by default it is drawn from numpy's
    global RNG, so ``np.random.seed`` makes a whole run reproducible.
    """
    microbe_properties = {"species": np.random.choice([ROCK, PAPER, SCISSORS], N_microbes).astype(np.int8)}
    if seed is None:
        seed = int(np.random.randint(0, np.iinfo(np.int64).max, dtype=np.int64))
    interaction_parameters = {"pRS": pRS, "pPR": pPR, "pSP": pSP, "seed": int(seed)}
    return rock_paper_scissors_interaction, interaction_parameters, microbe_properties
