"""GB300-native (sm_103a) Lagrangian particle step, a drop-in for the particle
stage of ggeraci/first_repo (particle.h call surface, tensor0/tensor1 field layout).

The compute path is libpstep.so (hand-written CUDA behind the C-ABI in
include/pstep.h); this package only builds and binds it.
"""
from .config import PI, RK4_PRE, RK4_POST, box_params, WORKLOADS  # noqa: F401
