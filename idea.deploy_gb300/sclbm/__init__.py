"""GB300-native Shan-Chen multiphase lattice-Boltzmann time step.

Host side of libsclbm.so (hand-written sm_103a CUDA behind a C ABI, see
include/sclbm.h), exposing the reference's class interface:

    from sclbm import ShanChenMultiPhase, XIStencils, FStencils, CUDA_T
"""
from .LBM import XIStencils, FStencils  # noqa: F401
from .MultiPhase import ShanChenMultiPhase, CUDA_T, ComputeCenterOfMass  # noqa: F401

__all__ = ['ShanChenMultiPhase', 'XIStencils', 'FStencils', 'CUDA_T', 'ComputeCenterOfMass']
