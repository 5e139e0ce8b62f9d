"""GB300-native tensor-network contraction with Jet's API.

The Python surface follows the reference's `jet` package: `Tensor`,
`TensorNetwork`, `PathInfo`, `TaskBasedContractor` (dtype-dispatching
factories over the TensorC64/C128, ... classes) and the free functions
`contract_tensors`, `add_tensors`, `conj`, `reshape`, `slice_index`,
`transpose`. Tensors live in GPU memory; every contraction, transpose and
slice runs as a CUDA kernel of libjetgpu.so (sm_103a). Importing the package
fails when the native libraries are not built: there is no CPU fallback.

The circuit front-end follows the reference's `jet.Circuit`, `jet.GateFactory`
and state classes; `Circuit.tensor_network()` builds GPU tensors.

Extras: `set_precision` (0 plain FP32, 1 TF32x3 tensor cores, 2 auto, 3 BF16x3, 4 FP16x3) and the
raw C-ABI binding `jet_gb300.capi`.
"""
from ._jet_bindings import (  # noqa: F401
    JetException,
    PathInfo,
    PathStepInfo,
    SlicedContractorC64,
    SlicedContractorC128,
    add_tensors,
    conj,
    contract_tensors,
    get_precision,
    reshape,
    set_precision,
    slice_index,
    transpose,
    version,
)
from .factory import *  # noqa: F401,F403
from .io import TensorFileException, TensorNetworkFile, TensorNetworkSerializer  # noqa: F401
from .gate import *  # noqa: F401,F403
from .state import Qubit, QubitRegister, Qudit, QuditRegister, State  # noqa: F401
from .circuit import Circuit, Operation, Wire  # noqa: F401

PREC_FP32 = 0
PREC_TF32X3 = 1
PREC_AUTO = 2
PREC_BF16X3 = 3
PREC_FP16X3 = 4
PREC_TUNED = 5

__version__ = version()
