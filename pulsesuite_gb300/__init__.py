"""GB300-native quantum-wire SBE right-hand side and PSTD field step.

A drop-in for the hot path of PulseSuite (pulsesuite.PSTD3D.SBEs): the
reference-shaped Python surface lives in :mod:`pulsesuite_gb300.SBEs`; the
batched GPU path in :mod:`pulsesuite_gb300.wires`; all arithmetic runs in the
in-tree CUDA library libsbe_gb300.so (C ABI in include/sbe_gb300.h).
"""

__version__ = "0.1.0"
