"""Value types of the propagator API (types.hpp:23-29 of the reference)."""
from __future__ import annotations

import enum
from dataclasses import dataclass


class ProbType(enum.IntEnum):
    """Channel index a*3+b means P(a -> b) (types.hpp:23-27)."""
    e_e = 0
    e_m = 1
    e_t = 2
    m_e = 3
    m_m = 4
    m_t = 5
    t_e = 6
    t_m = 7
    t_t = 8


class NeutrinoType(enum.IntEnum):
    """types.hpp:29."""
    Neutrino = 0
    Antineutrino = 1


Neutrino = NeutrinoType.Neutrino
Antineutrino = NeutrinoType.Antineutrino


@dataclass(frozen=True)
class Mixing:
    """One oscillation-parameter set: the arguments of setMNSMatrix (angles in radians)
    and setNeutrinoMasses (eV^2, dm23sq = m3^2 - m2^2, negative for inverted ordering)."""
    theta12: float
    theta13: float
    theta23: float
    dcp: float
    dm12sq: float
    dm23sq: float
