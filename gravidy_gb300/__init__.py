"""gravidy_gb300 -- GraviDy's Hermite4 block-timestep force path on GB300.

The hot path (predictor, acc+jerk force sum, corrector, block timesteps, next
block time, energy) runs as hand-written sm_103a CUDA kernels behind the C ABI
of include/gravidy_gb300.h.  This package holds the Python mirror of the
reference's Hermite4GPU interface, the input/log formats and the in-tree
build.
"""
from .hermite4 import Hermite4GPU, NbodySystem, e2_from_softening  # noqa: F401
from .io import EnergyLog, read_input_file  # noqa: F401

__all__ = ["Hermite4GPU", "NbodySystem", "EnergyLog", "read_input_file", "e2_from_softening"]
