"""GB300-native DMRG/TDVP inner loop of FiniteMPTools.

The compute lives in ``libfmpt.so`` (hand-written sm_103a CUDA kernels behind
the C ABI of include/fmpt.h); this package is the host-side mirror of the
reference's Julia interface (environments, sweep!, ac2_prime, updateleft,
DMRG1/DMRG2/TDVP1, expectation).  There is no CPU fallback: every device
call raises ``FMPTError`` when the library or a GPU is missing.
"""

from ._native import FMPTError, lib  # noqa: F401
from .algorithms import (DMRG1, DMRG1S, DMRG2, TDVP1, TDVP1S, TDVP2, Defaults,  # noqa: F401
                         compute_, expectation,  # noqa: F401
                         expectation_local, ground_state_, leftsweep_, rightsweep_, sweep_)
from .auxiliary import (MPSTruncation, default_truncation, leftorth, rightorth,  # noqa: F401
                        stable_tsvd)
from .derivatives import HeffOp, ac2_prime, ac_prime, c_prime, exponentiate  # noqa: F401
from .derivatives import simple_lanczos_solver  # noqa: F401
from .device import DeviceTensor, Handle, default_handle  # noqa: F401
from .expansion import OptimalExpansion, default_expansion  # noqa: F401
from .tebd import (HomogeneousTEBDCache, InhomogeneousTEBDCache, QuantumCircuit,  # noqa: F401
                   QuantumGate, TEBDStepper, apply_, bond_evolution, fuse_gates, make_step_,
                   move_, trotter_propagator)
from .exactdiag import (ExactFiniteMPS, exact_diagonalization, exact_timeevolution,  # noqa: F401
                        init_h_center, max_bond_dimensions)
from .excited import (ProjectedExpectationCache, c2_proj, c_proj, init_cstorage_right,  # noqa: F401
                      overlap_updateleft, overlap_updateright, project_)
from .envs import (ExpectationCache, environments, init_hstorage_, updateleft_,  # noqa: F401
                   updateright_)
from .mps import (FiniteMPS, bond_dimension, canonicalize_, increase_bond_,  # noqa: F401
                  prodmps, randommps)
from .transfer import updateleft, updateright  # noqa: F401
from .u1 import (U1ExpectationCache, U1FiniteMPS, U1HeffOp, U1Space,  # noqa: F401
                 mpo_channel_charges, u1_environments, u1_expectation, u1_randommps, u1_split,
                 u1_twosite, u1_updateleft, u1_updateright)
from .utilities import (FiniteMPO, MPOHamiltonian, SchurMPOTensor,  # noqa: F401
                        heisenberg_xxz_mpo, j1j2_heisenberg_mpo, spin_half_matrices, tfi_mpo)
