"""qca_gb300: GB300-native (sm_103a) time evolution for the quantum game of life.

Drop-in GPU implementations of the reference's ``Algorithm`` interface
(``algorithms/algorithm.py:10-63``): ``GpuExact`` for ``--algorithm exact`` and
``GpuTDVP`` for ``1tdvp`` / ``2tdvp``.  The compute runs in hand-written CUDA
kernels behind the C ABI declared in ``include/qca_gb300.h``
(``libqca_gb300.so``); this package only holds host-side glue: the
reference's driver loop (``driver``), a continuous-batching serving loop
(``serving``) and the benchmark workloads (``workloads``).
"""
from .tensor_networks import MPO, MPS, Rules  # noqa: F401
from .algorithms import Algorithm, GpuExact, GpuTDVP, algorithm_class  # noqa: F401

__all__ = ["MPO", "MPS", "Rules", "Algorithm", "GpuExact", "GpuTDVP", "algorithm_class"]
