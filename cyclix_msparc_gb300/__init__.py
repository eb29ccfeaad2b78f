"""GB300-native Chebyshev-filtered subspace iteration for Cyclix (cyclic/helical real-space DFT).

The compute path is ``libcyclix_gpu.so`` (hand-written sm_103a CUDA behind a
C-ABI, ``include/cyclix_gpu.h``); :mod:`cyclix_msparc_gb300.msparc` mirrors the
reference's MATLAB call signatures on top of it through ctypes.
"""
__all__ = ["cychel", "workloads"]
