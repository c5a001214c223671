// The step kernels are compiled twice (kernels_exact.cu with -fmad=false,
// kernels_fast.cu with -fmad=true); the host engine launches through this table.
#pragma once
#include <cuda_runtime.h>

#include "layout.cuh"

namespace gvx {

struct KernelSet {
    const char* name;
    void (*links)(int grid, int block, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const dev::Item* items, int n, int* tickets);
    void (*contacts)(int grid, int block, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const dev::Item* items, int n, int* tickets);
    void (*voxels)(int grid, int block, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const dev::Item* items, int n, int* tickets,
                   double* partials);
    void (*dt)(int grid, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, int sim);
    void (*init_temp)(int grid, cudaStream_t s, const dev::Sim* sims, int sim, float initial);
    void (*hash_build)(int grid, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, int sim);
    void (*com)(cudaStream_t s, const dev::Sim* sims, int sim, double* out4);
};

KernelSet kernelset_exact();   // every multiply and add rounded separately (the reference's CPU rounding)
KernelSet kernelset_fast();    // multiply-adds contracted into FP64 FMAs

}  // namespace gvx
