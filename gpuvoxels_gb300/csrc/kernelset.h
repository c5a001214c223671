// The step kernels are compiled twice (kernels_exact.cu with -fmad=false,
// kernels_fast.cu with -fmad=true); the host engine launches through this table.
#pragma once
#include <cuda_runtime.h>

#include "layout.cuh"

namespace gvx {

struct KernelSet {
    const char* name;
    // groups the elements of the running simulations by key for two lists at once (links and
    // voxels), in windows of work items
    void (*bins)(int grid, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, dev::BinList links, dev::BinList voxels);
    // perm holds at most `cap` entries; entries name slots below n_slots; warps claim `claim`
    // entries at a time (a multiple of 32)
    void (*links)(int grid, int block, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const int2* perm, const int* total, int cap,
                  int n_slots, int* tickets, int claim);
    void (*contacts)(int grid, int block, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const dev::Item* items, int n, int* tickets);
    void (*voxels)(int grid, int block, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const int2* perm, const int* total, int cap,
                   int n_slots, int* tickets, int claim);
    // the end of the step for n simulations (slot list): centre-of-mass sample, time, stop;
    // simulations whose watch lists go stale append their contact items to stale_items
    // (count in tickets[7])
    void (*sim_end)(cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const int* slots, int n, int* tickets, int* stale_items);
    // VX3 signals relayed between neighbours (after voxels, over the voxel items)
    void (*signals)(int grid, int block, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const dev::Item* items, int n, int* tickets);
    // VX3 attachment: new links for this step's candidate pairs of n simulations (device slot list)
    void (*attach)(cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const int* slots, int n);
    // set-up of n newly uploaded simulations (device slot list), grid = blocks per simulation
    void (*dt)(int grid, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const int* slots, int n);
    void (*init_temp)(int grid, cudaStream_t s, const dev::Sim* sims, const int* slots, const float* initial, int n);
    void (*hash_build)(int grid, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const int* slots, int n);
    void (*com)(cudaStream_t s, const dev::Sim* sims, int sim, double* out4);
    // Packs position, orientation and the reference-order flag byte of the voxels of
    // n simulations (slot[k], output offset off[k]) into pos3 / q4 / flags (one launch).
    void (*gather)(cudaStream_t s, const dev::Sim* sims, const int* slot, const int64_t* off, int n, double* pos3, double* q4,
                   uint8_t* flags);
    // resident blocks per SM of k_links (0) or k_voxels (1) at a block size
    int (*resident_blocks)(int which, int block);
    int max_block;   // largest block k_links / k_voxels are compiled for
    // watch-list regeneration (one pass) of the simulations that need it: over the
    // contact items listed in stale_items (tickets[7] of them, at most n_items) and the batch's
    // slot list
    void (*watch)(int grid, cudaStream_t s, const dev::Sim* sims, dev::Ctl* ctl, const dev::Item* items, int n_items,
                  const int* stale_items, const int* tickets, const int* slots, int n_sims);
};

KernelSet kernelset_exact();   // every multiply and add rounded separately (the reference's CPU rounding)
KernelSet kernelset_fast();    // multiply-adds contracted into FP64 FMAs

}  // namespace gvx
