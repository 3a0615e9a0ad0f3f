"""libcpab_gb300: CPAB integration for NVIDIA GB300 (sm_103a).

Drop-in for the pytorch GPU path of libcpab: ``Cpab.transform_grid``,
``Cpab.interpolate`` and ``Cpab.transform_data`` (forward and gradient) run as
hand-written CUDA kernels behind the C ABI of include/cpab_gb300.h.
"""
from .cpab import Cpab
from .sequential import CpabSequential
from .alignment import CpabAligner
from . import functions

__all__ = ['Cpab', 'CpabSequential', 'CpabAligner', 'functions']
