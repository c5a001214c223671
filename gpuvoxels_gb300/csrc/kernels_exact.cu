// Step kernels, exact build: compiled with -fmad=false, so every FP64/FP32
// multiply and add is rounded separately, as in the reference CPU path.
#define GVX_KNS kexact
#include "kernelset.h"
#include "kernels.cuh"

namespace gvx {
KernelSet kernelset_exact() { return kexact::make_kernelset("exact"); }
}  // namespace gvx
