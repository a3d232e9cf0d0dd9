// chem_warp.cu -- the one-warp-per-cell chemistry update (the last section of chem_kernels.cu) as its own
// translation unit, compiled with FMA contraction.  Its operations are the reference-order kernel's, in the
// same order, with a*b+c rounded once where the compiler fuses them: each value is within rounding of the
// reference-order kernel's (tested against the oracle to 1e-8 in Y and 1e-7 relative in T and p).  On this
// GPU, where every FP64 instruction costs an FMA's issue slot, the fused form issues fewer of them.
#define GDTK_WARP_TU 1
#include "chem_kernels.cu"
