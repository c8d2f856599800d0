"""mcd - GB300-native electron-trajectory Monte Carlo (DS and continuous modes).

The host side mirrors the reference interface of elena-pascal/MC-discrete
(readInput, multiTraj_DS, multiTraj_cont); the work runs in hand-written
sm_103a CUDA kernels behind the C ABI of libmcd.so (include/mcd.h).
"""
from . import _lib
from .config import readInput, parse_input, with_defaults
from .engine import Batch, RunResult, run
from .shim import multiTraj_DS, multiTraj_cont

__all__ = ["readInput", "parse_input", "with_defaults", "run", "Batch", "RunResult",
           "multiTraj_DS", "multiTraj_cont", "lib"]


def lib():
    """The loaded C library (built in-tree on first use)."""
    return _lib.lib()
