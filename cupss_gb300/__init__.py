"""GB300-native cuPSS pseudospectral step.

The product is the shared library ``cupss_gb300/libcupss.so`` (CUDA kernels for
sm_103a, the engine, the drop-in C++ API of ``include/cupss.h`` and the C-ABI of
``include/cupss_gb300.h``).  This package loads it with ctypes and mirrors the
reference API in Python (``Evolver``) plus the IR-level ``Solver``.
"""
from .api import Ensemble, Evolver, Server, Solver  # noqa: F401
from .capi import CupssError, load  # noqa: F401
from .workloads import splitmix64_uniform  # noqa: F401
