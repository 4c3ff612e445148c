"""qobgpu -- GB300-native operator application for QuantumOpticsBase.jl's API.

The Python mirror of the reference's types (bases, Ket/Bra, Operator,
LazyTensor, LazySum, LazyProduct, TimeDependentSum) over the C-ABI library
libqobgpu.so, whose hand-written sm_103a kernels do the work.  ``mul_`` is the
reference's 5-argument ``mul!(result, a, b, alpha, beta)``.
"""
from .bases import (Basis, CompositeBasis, FockBasis, GenericBasis, MomentumBasis, NLevelBasis,
                    PositionBasis, SpinBasis, comp_size, samplepoints, spacing)
from .bases import tensor as tensor_basis
from .operators import *  # noqa: F401,F403
from .operators import __all__ as _ops_all
from .states import (Bra, Ket, basisstate, coherentstate, dagger_state, dm, fockstate, spindown, spinup,
                     tensor_states)
from .rng import Rng


def __getattr__(name):
    # device layer is imported lazily so host-only use does not need CUDA
    if name in ("mul_", "apply_alloc", "apply_alloc_bra", "expect", "variance", "norm", "dot", "to_device"):
        from . import mul as _m

        return getattr(_m, name)
    raise AttributeError(name)


__all__ = list(_ops_all) + [
    "Basis", "CompositeBasis", "FockBasis", "GenericBasis", "NLevelBasis", "SpinBasis",
    "tensor_basis", "Ket", "Bra", "basisstate", "dagger_state", "tensor_states", "Rng", "mul_",
    "coherentstate", "fockstate", "spinup", "spindown", "dm",
]
