"""GB300-native sparse SpMV library: the LeSpMV per-format SpMV path
(COO, CSR, BSR, CSR5, DIA, ELL, S-ELL, SELL-c-sigma, SELL-c-R) as sm_103a
CUDA kernels behind the C ABI declared in include/sspmv.h."""
__version__ = "0.1.0"
