"""GB300-native Chebyshev-filtered subspace iteration for Tucker-tensor DFT.

Drop-in for the eigensolver path of ttdftdev/ttdft_public (ChebyShevFilter,
AX, MultTM, EigenSolver) with sm_103a CUDA kernels behind a C ABI
(include/ttg.h, lib/libttg.so)."""

__all__ = ["system", "api"]
