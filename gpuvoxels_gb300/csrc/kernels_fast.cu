// Step kernels, FMA build: compiled with -fmad=true, so multiply-add pairs
// become single FP64 FMA instructions (fewer instructions on the FP64 pipe,
// results within the parity tolerance instead of bit-faithful).
#define GVX_KNS kfast
#include "kernelset.h"
#include "kernels.cuh"

namespace gvx {
KernelSet kernelset_fast() { return kfast::make_kernelset("fma"); }
}  // namespace gvx
