"""qudrip_gb300: a GB300-native (sm_103a) engine for QuDrip's exact-diagonalization path.

The public names mirror QuDrip's C++ API (getQbits, getNset, Constrain,
getBoseGate, `ham >> chain`, getState, psi.eval, Arnoldi.getLanczosSolver ...).
Operator algebra is host-side bookkeeping; every numerical step runs in the
CUDA library libqudrip_gb300.so through the C ABI of include/qudrip_gb300.h.
"""
from .operators import (II, id, pauli_x, pauli_y, pauli_z, getQbits, getNset, getNup, getNdo,  # noqa: F401
                        getNd, getNh, getBoseGate, getFermiGate, getHopFermiGate, getHopBoseGate,
                        getEmptyOperator, Operator, OperatorSum, QbitsIndex, SectorSpec)
from .engine import (Context, default_context, Sector, Constrain, LooseConstrain, Hamiltonian,  # noqa: F401
                     State, getState, apply, start_vector, shuffle_state, LanczosSolver, ArnoldiSolver, Arnoldi,
                     batch_lanczos, traj_run, lanczos_evolve, seeded_start, Server, Hermitian,
                     HermitianLanczosSolver, obs_eval, McManager, MC_REAL, MC_COMPLEX)
from .lattice import params_type, Lattice, LatticeFunction, Model, get_reci  # noqa: F401
from .params import param_finder  # noqa: F401
from . import _capi  # noqa: F401
