"""qandle_gb300: a GB300 (sm_103a) state-vector engine behind qandle's front end.

The public names mirror qandle's (qandle/__init__.py:3-14): gate layers
(RX, RY, RZ, U, CNOT, CZ, SWAP, Invert, Controlled, Reset), AngleEmbedding,
AmplitudeEmbedding, measurements, StronglyEntanglingLayer and QConv build
into torch modules, and ``Circuit`` runs them
on hand-written CUDA kernels through the C ABI of libqandle_gb300.so.
There is no CPU execution path: tensors must live on a CUDA device.
"""
# ruff: noqa: F401 F403
from . import config, errors, qasm, remap, splitter, utils
from .tune import autotune
from .operators import *
from .embeddings import *
from .measurements import *
from .ansaetze import *
from .qcircuit import *
from .convolution import QConv
from .errors import UnbuiltGateError
from .qasm import QasmRepresentation, convert_to_qasm
from .splitter import split, SubcircuitContainer
from .utils import reduce_dot, parse_rot, do_not_implement, get_matrix_transforms

__version__ = "1.0.0"


def library_path() -> str:
    """Path of the CUDA library this package loads."""
    from . import _lib

    return _lib.lib_path()
