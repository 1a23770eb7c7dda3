"""GB300-native Barger propagation (CUDAProb3++ hot path) behind the reference's
Propagator API.  Importing the package loads nothing; the CUDA library is loaded (and must
exist) when a propagator is constructed."""
from .types import Antineutrino, Mixing, Neutrino, NeutrinoType, ProbType  # noqa: F401
from .propagators import (  # noqa: F401
    AtmosCudaPropagatorSingle,
    BeamCudaPropagatorSingle,
    CudaPropagatorSingle,
    Propagator,
)
