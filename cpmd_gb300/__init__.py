"""GB300-native drop-in for CPMD's Γ-point wavefunction hot path.

rhoofr / vpsi (pair-packed pruned 3D FFT band loop), ortho (Cholesky
Gram-Schmidt, Loewdin), invfftn / fwfftn, rnlsm1 / fnonloc -- hand-written
CUDA for sm_103a behind the C ABI in include/cpmd_gb300.h.
"""
from .api import Batch, Context, GbcpError, kernel_launches  # noqa: F401
from .cell import Basis, make_basis  # noqa: F401
from .restart import RestartData, read_restart, write_restart  # noqa: F401
