// GB300 step engine: HBM arena, per-simulation upload, batched stepping with
// work queues captured in CUDA graphs, and the continuous-batching serving loop.
#include "engine.h"
#include "kernelset.h"
#include "layout.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_set>

namespace gvx {

namespace {

#define CK(x)                                                                                 \
    do {                                                                                      \
        cudaError_t _e = (x);                                                                 \
        if (_e != cudaSuccess) {                                                              \
            if (err) *err = std::string(#x) + ": " + cudaGetErrorString(_e);                  \
            return -5;                                                                        \
        }                                                                                     \
    } while (0)

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Control-block updates for a list of slots (one launch instead of per-slot copies).
__global__ void k_ctl_run(dev::Ctl* ctl, const int* __restrict__ slots, const int64_t* __restrict__ targets, int n, int no_stop) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dev::Ctl& c = ctl[slots[k]];
    c.status = SIM_RUNNING;
    c.target = targets[k];
    c.no_stop = no_stop;
}
__global__ void k_ctl_end_steps(dev::Ctl* ctl, const int* __restrict__ slots, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dev::Ctl& c = ctl[slots[k]];
    c.no_stop = 0;
    if (c.status == SIM_DONE) c.status = SIM_IDLE;
}

// One formula evaluated on the device for n variable sets (x, y, z, hit, t, angle,
// closeness, numClosePairs, num_voxel): the evaluator the step kernels use.
__global__ void k_eval_formula(const MathTree* m, const double* __restrict__ vars9, int n, double* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double* v = vars9 + 9 * (size_t)k;
    MathVars mv;
    mv.x = v[0]; mv.y = v[1]; mv.z = v[2]; mv.hit = v[3]; mv.t = v[4]; mv.angle = v[5]; mv.closeness = v[6];
    mv.num_close_pairs = (int)v[7]; mv.num_voxel = (int)v[8];
    out[k] = mathtree_eval(*m, mv);
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Pinned host buffers outlive the contexts that used them: a destroyed context hands its
// staging buffers to this cache and the next context takes them from it, so a process that
// creates contexts again and again pins host memory once (up to kPinnedCacheMax bytes kept).
struct PinnedCache {
    std::mutex mu;
    std::multimap<size_t, char*> free_;   // capacity -> buffer
    size_t bytes = 0;
    static constexpr size_t kPinnedCacheMax = 2ull << 30;
    // the smallest cached buffer of at least `need` bytes, or null
    char* take(size_t need, size_t* cap) {
        std::lock_guard<std::mutex> lock(mu);
        auto it = free_.lower_bound(need);
        if (it == free_.end()) return nullptr;
        char* p = it->second;
        *cap = it->first;
        bytes -= it->first;
        free_.erase(it);
        return p;
    }
    void give(char* p, size_t cap) {
        if (!p) return;
        {
            std::lock_guard<std::mutex> lock(mu);
            if (bytes + cap <= kPinnedCacheMax) { free_.emplace(cap, p); bytes += cap; return; }
        }
        cudaFreeHost(p);
    }
};
PinnedCache& pinned_cache() {
    static PinnedCache* c = new PinnedCache();   // never destroyed: buffers stay pinned until exit
    return *c;
}

// One region of a generation's upload: its image at stage + src (img bytes), copied to
// arena + dst, and the rest of the region (up to total bytes) cleared.  All offsets and
// sizes are multiples of 256 bytes.
struct RegionCopy {
    uint64_t src, dst, img, total;
};
// blockIdx.y picks the region, the blocks along x stride over it in 16-byte words.
__global__ void k_scatter_regions(const char* __restrict__ stage, const RegionCopy* __restrict__ list, char* arena) {
    const RegionCopy c = list[blockIdx.y];
    const uint4* src = (const uint4*)(stage + c.src);
    uint4* dst = (uint4*)(arena + c.dst);
    const size_t ni = c.img / 16, nt = c.total / 16;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = i < ni ? src[i] : make_uint4(0u, 0u, 0u, 0u);
}

// The work-list fields of a new batch's control blocks in one launch: per batch entry the
// number and the first index of the simulation's voxel items and the first index and number
// of its contact items, and the completion counters cleared (one small copy per simulation
// took about a millisecond for 512 of them).
__global__ void k_set_batch_items(dev::Ctl* ctl, const int* __restrict__ slots, const int4* __restrict__ items, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dev::Ctl& c = ctl[slots[i]];
    c.n_vox_items = items[i].x;
    c.item_begin = items[i].y;
    c.c_item_begin = items[i].z;
    c.c_item_count = items[i].w;
    c.done_items = 0;
    c.sig_done_items = 0;
}

// Every contact item listed for the first step of a new batch's watch-list passes (the
// items each simulation's previous step would have listed are not known).
__global__ void k_list_all_items(int* stale_items, int n, int* tickets) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) stale_items[i] = i;
    if (i == 0) tickets[7] = n;
}

// Host tables of the C library's powf(x, -nu) for every float x in [0.5, 2), one per Poisson
// ratio: the reference's CPU path takes the Poisson strain's power from that function
// (CVX_Voxel::strain, Voxelyze3/src/old/VX_Voxel.cpp:327), whose results are not always the
// correctly rounded power, so the engine uses the library's own values.  Computed once per
// process on host threads and kept in pinned memory for the copies to each context's device.
const float* host_pow_table(float nu) {
    static std::mutex mu;
    static std::map<uint32_t, float*> tabs;
    uint32_t key;
    memcpy(&key, &nu, 4);
    std::lock_guard<std::mutex> lock(mu);
    auto it = tabs.find(key);
    if (it != tabs.end()) return it->second;
    float* t = nullptr;
    if (cudaHostAlloc((void**)&t, sizeof(float) * dev::kPowTabSize, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        t = (float*)malloc(sizeof(float) * dev::kPowTabSize);
        if (!t) return nullptr;
    }
    // the library function itself, called through a pointer so that no vector variant replaces it
    float (*volatile lib_powf)(float, float) = powf;
    const float y = -nu;
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        float (*f)(float, float) = lib_powf;
        for (uint32_t c = next++; c < dev::kPowTabSize / 65536; c = next++)
            for (uint32_t i = c * 65536; i < (c + 1) * 65536; i++) {
                const uint32_t u = dev::kPowTabFirst + i;
                float x;
                memcpy(&x, &u, 4);
                t[i] = f(x, y);
            }
    };
    const int nt = std::max(1, std::min(32, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int k = 1; k < nt; k++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    tabs[key] = t;
    return t;
}

// The device copy of a powf table on `device` (current), shared by every context of the
// process on that device: made on first use, read-only afterwards, held until the process
// exits (64 MiB per Poisson ratio and device, outside the contexts' HBM budgets).
const float* device_pow_table(int device, float nu, int64_t* h2d_bytes, std::string* err) {
    static std::mutex mu;
    static std::map<std::pair<int, uint32_t>, float*> tabs;
    uint32_t key;
    memcpy(&key, &nu, 4);
    std::lock_guard<std::mutex> lock(mu);
    auto it = tabs.find({device, key});
    if (it != tabs.end()) return it->second;
    const float* h = host_pow_table(nu);
    if (!h) { if (err) *err = "host memory for the powf table"; return nullptr; }
    float* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float) * dev::kPowTabSize);
    if (e == cudaSuccess) e = cudaMemcpy(d, h, sizeof(float) * dev::kPowTabSize, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);   // complete before any context's stream reads it
    if (e != cudaSuccess) {
        if (d) cudaFree(d);
        if (err) *err = std::string("powf table: ") + cudaGetErrorString(e);
        return nullptr;
    }
    *h2d_bytes += (int64_t)sizeof(float) * dev::kPowTabSize;
    tabs[{device, key}] = d;
    return d;
}

// First-fit allocator over one device allocation (the HBM budget).
struct Arena {
    char* base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free_;   // offset -> length
    size_t used = 0;
    void init(char* b, size_t s) { base = b; size = s; free_.clear(); free_[0] = s; used = 0; }
    bool alloc(size_t n, size_t* off) {
        n = align256(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                size_t rest = it->second - n, o = it->first + n;
                free_.erase(it);
                if (rest) free_[o] = rest;
                used += n;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t n) {
        n = align256(n);
        used -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
};

struct Layout {
    size_t total = 0;
    size_t add(size_t bytes) { size_t o = total; total += align256(bytes); return o; }
};

struct SimRec {
    int64_t id = 0;
    SimWorld w;
    int slot = -1;                 // index into device tables while resident
    bool resident = false;
    size_t off = 0, bytes = 0;
    dev::Sim dsim{};
    int32_t status = SIM_IDLE;
    float dt = 0, optdt = 0;
    int cycle_step = 0;
    double init_com[3] = {0, 0, 0};
    std::vector<double> final_init_pos;   // initial positions reset by the secondary experiment (else empty)
    int num_measured = 0;
    int64_t horizon = 0;
    double submit_s = 0, start_s = 0, finish_s = 0;
    bool retired = false;
    SimResult result{};
    int n_vox_items = 0;
    std::vector<double> final_pos;  // x block, y block, z block at finish (SavePositionOfAllVoxels only)
    dev::Ctl pending_ctl{};         // control block between upload_begin and upload_finish
    dev::Sim pending_sim{};         // device descriptor between upload_begin and upload_finish
};

class EngineImpl final : public Engine {
public:
    int device_ = 0;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, evk_[6] = {};
    Arena arena_;
    char* arena_base_ = nullptr;
    std::map<int64_t, std::unique_ptr<SimRec>> sims_;
    int64_t next_id_ = 1;
    // device tables
    int cap_slots_ = 0;
    dev::Sim* d_sims_ = nullptr;
    dev::Ctl* d_ctl_ = nullptr;
    std::vector<SimRec*> slot_owner_;
    // queue tickets of the step kernels (0 links, 1 contacts, 2 voxels, 3 signals) and the
    // contact spill pool's record count of the step
    static constexpr int kTickets = 8, kSpillTicket = 4;
    int* d_tickets_ = nullptr;
    int32_t* d_spill_p_ = nullptr;
    float* d_spill_f_ = nullptr;
    int spill_cap_ = 0;
    static constexpr int kAttachCandPerVoxel = 16;   // attachment candidate pairs kept per voxel and step
    int contact_inline_ = dev::kContactInline;        // contacts in each voxel's own slots (simulations uploaded later)
    // the powf tables of the Poisson ratios in use (key: the ratio's bits; the process's
    // device copies, shared with the other contexts on this device)
    std::map<uint32_t, const float*> dev_pow_;
    dev::Item* d_items_ = nullptr;
    int* d_stale_items_ = nullptr;   // contact items whose simulations regenerate their watch lists next
    int cap_items_ = 0;
    double* d_com4_ = nullptr;
    // tuning
    int block_links_ = 256, block_voxels_ = 256, items_links_ = 1024, items_voxels_ = 1024, graph_steps_ = 64;
    int claim_links_ = 32, claim_voxels_ = 32;   // elements a warp claims from the step queues at a time
    // link binning: regrouped every bin_every_ steps (the first step after a batch change
    // always); every second step measured 1.9% faster than every step on the 512-creature
    // batch once it has settled (keys change slowly: 0.1% of links a step) and 1% faster on
    // a fresh one, every fourth no faster than every second
    int bin_every_ = 2, bin_phase_ = 0;
    bool bins_dirty_ = true;
    // Small batches (serving at low load) are bound by launch latency, not by the FP64 pipe:
    // their links and voxels are regrouped only when the batch changes and at the start of
    // every graph replay, not every step.
    static constexpr size_t kRegroupEveryStepLinks = 200000;
    size_t batch_links_ = 0, batch_voxels_ = 0;
    int sm_count_ = 152;
    int profiling_ = 0;
    KernelSet ks_ = kernelset_exact();
    int64_t exact_steps_ = -1;     // >= 0 while step() advances a known number of steps
    Timing timing_;
    double t0_ = now_s();
    // serving
    std::deque<int64_t> queue_;
    std::vector<int64_t> active_;
    // cached batch (items + graph) for a set of slots
    std::vector<int> batch_slots_;
    int n_link_items_ = 0, n_contact_items_ = 0, n_vox_items_ = 0;
    bool any_collide_ = false;
    bool any_watch_ = false;   // some simulation of the batch takes its contacts from watch lists
    bool any_signals_ = false;
    // batch-wide grouping of links by key (k_bin_hist / k_bin_scan / k_bin_scatter)
    int* d_link_hist_ = nullptr;
    int* d_link_base_ = nullptr;
    int* d_link_total_ = nullptr;
    int2* d_link_perm_ = nullptr;
    size_t cap_bins_ = 0, cap_perm_ = 0;
    // the same for the voxels, and the batch's slot list for k_sim_end
    int* d_vox_hist_ = nullptr;
    int* d_vox_base_ = nullptr;
    int* d_vox_total_ = nullptr;
    int2* d_vox_perm_ = nullptr;
    size_t cap_vbins_ = 0, cap_vperm_ = 0;
    int* d_batch_slots_ = nullptr;
    int4* d_batch_items_ = nullptr;          // per batch entry: voxel items, first voxel item, first contact item, contact items
    int n_batch_ = 0, cap_batch_ = 0;
    std::vector<int> batch_slots_host_;
    std::vector<int4> batch_items_host_;
    int n_attach_ = 0, cap_attach_ = 0;     // simulations with VX3 attachment in the batch
    int64_t graph_launches_ = 0;            // kernels one replay of the captured graph launches
    int* d_attach_slots_ = nullptr;
    std::vector<int> attach_slots_host_;
    cudaGraphExec_t graph_ = nullptr;
    int graph_len_ = 0;
    bool batch_dirty_ = true;
    // pinned host staging: two upload buffers used in turn (the copy of one simulation's
    // region overlaps filling the next), and one buffer for batched state read-back
    struct Pinned {
        char* p = nullptr;
        size_t cap = 0;
        cudaEvent_t done = nullptr;   // the last copy out of this buffer
    };
    Pinned up_[2];
    int up_next_ = 0;
    Pinned gen_;   // the images of one generation of uploads (upload_many)
    Pinned rb_;
    char* d_gather_ = nullptr;
    size_t cap_gather_ = 0;
    static constexpr size_t kGatherInitial = 16u << 20;
    char* d_stage_ = nullptr;   // a generation's region images on the device (upload_many), when
    size_t cap_stage_ = 0;      // the arena has no room for them
    static constexpr size_t kNoStage = ~(size_t)0;
    size_t stage_off_ = kNoStage, stage_len_ = 0;   // the arena's temporary staging region in use
    void release_stage() {
        if (stage_off_ == kNoStage) return;
        arena_.release(stage_off_, stage_len_);
        stage_off_ = kNoStage;
        stage_len_ = 0;
    }
    static constexpr size_t kPinnedUploadMax = 256u << 20;   // larger regions are copied from pageable memory

    ~EngineImpl() override {
        if (graph_) cudaGraphExecDestroy(graph_);
        cudaSetDevice(device_);
        if (stream_) cudaStreamSynchronize(stream_);
        for (Pinned* b : {&up_[0], &up_[1], &rb_, &gen_}) {
            pinned_cache().give(b->p, b->cap);
            if (b->done) cudaEventDestroy(b->done);
        }
        cudaFree(d_gather_);
        cudaFree(d_stage_);
        cudaFree(d_sims_); cudaFree(d_ctl_); cudaFree(d_tickets_); cudaFree(d_items_); cudaFree(d_stale_items_); cudaFree(d_com4_);
        cudaFree(d_spill_p_); cudaFree(d_spill_f_);
        cudaFree(d_attach_slots_);
        cudaFree(d_link_hist_); cudaFree(d_link_base_); cudaFree(d_link_total_); cudaFree(d_link_perm_);
        cudaFree(d_vox_hist_); cudaFree(d_vox_base_); cudaFree(d_vox_total_); cudaFree(d_vox_perm_); cudaFree(d_batch_slots_); cudaFree(d_batch_items_);
        cudaFree(arena_base_);
        if (ev0_) cudaEventDestroy(ev0_);
        if (ev1_) cudaEventDestroy(ev1_);
        for (auto& e : evk_) if (e) cudaEventDestroy(e);
        if (stream_) cudaStreamDestroy(stream_);
    }

    int init(int device, size_t budget, std::string* err) {
        device_ = device;
        CK(cudaSetDevice(device));
        CK(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device));
        // GVX_LINK_BIN_EVERY: steps between regroupings of the links (tuning knob, default 1)
        if (const char* e = getenv("GVX_LINK_BIN_EVERY")) bin_every_ = std::max(1, atoi(e));
        CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        CK(cudaEventCreate(&ev0_));
        CK(cudaEventCreate(&ev1_));
        for (auto& e : evk_) CK(cudaEventCreate(&e));
        if (budget == 0) {
            size_t fr = 0, tot = 0;
            CK(cudaMemGetInfo(&fr, &tot));
            budget = fr / 2;
        }
        CK(cudaMalloc(&arena_base_, budget));
        arena_.init(arena_base_, budget);
        CK(cudaMalloc(&d_tickets_, kTickets * sizeof(int)));
        CK(cudaMemset(d_tickets_, 0, kTickets * sizeof(int)));
        // contact spill pool: 1/64 of the budget in 16-byte records (partner + force), 1M to 64M records
        spill_cap_ = (int)std::min<size_t>(64u << 20, std::max<size_t>(1u << 20, budget / 64 / 16));
        CK(cudaMalloc(&d_spill_p_, sizeof(int32_t) * (size_t)spill_cap_));
        CK(cudaMalloc(&d_spill_f_, 3 * sizeof(float) * (size_t)spill_cap_));
        CK(cudaMalloc(&d_com4_, 4 * sizeof(double)));
        // device scratch for the per-call tables (slot lists, descriptors, read-back packing):
        // sized for a few thousand simulations up front, so that calls rarely allocate
        CK(cudaMalloc(&d_gather_, kGatherInitial));
        cap_gather_ = kGatherInitial;
        for (Pinned* b : {&up_[0], &up_[1], &rb_, &gen_}) CK(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
        if (int e = reserve_tables(err)) return e;
        return grow_slots(64, err);
    }

    // The step's work tables sized up front for batches of up to 4M links, 2M voxels and
    // 32k work items (about 60 MB), so that running a batch allocates nothing: an allocation
    // right after a context's first pinned host buffer measured several ms on this machine.
    int reserve_tables(std::string* err) {
        cap_bins_ = cap_vbins_ = (size_t)32768 * dev::kOrderKeysBins;
        cap_perm_ = 4u << 20;
        cap_vperm_ = 2u << 20;
        cap_items_ = 65536;
        cap_batch_ = 16384;
        cap_attach_ = 1024;
        CK(cudaMalloc(&d_link_hist_, sizeof(int) * cap_bins_));
        CK(cudaMalloc(&d_link_base_, sizeof(int) * cap_bins_));
        CK(cudaMalloc(&d_link_total_, sizeof(int)));
        CK(cudaMemset(d_link_total_, 0, sizeof(int)));
        CK(cudaMalloc(&d_link_perm_, sizeof(int2) * cap_perm_));
        CK(cudaMalloc(&d_vox_hist_, sizeof(int) * cap_vbins_));
        CK(cudaMalloc(&d_vox_base_, sizeof(int) * cap_vbins_));
        CK(cudaMalloc(&d_vox_total_, sizeof(int)));
        CK(cudaMemset(d_vox_total_, 0, sizeof(int)));
        CK(cudaMalloc(&d_vox_perm_, sizeof(int2) * cap_vperm_));
        CK(cudaMalloc(&d_items_, sizeof(dev::Item) * cap_items_));
        CK(cudaMalloc(&d_stale_items_, sizeof(int) * cap_items_));
        CK(cudaMalloc(&d_batch_slots_, sizeof(int) * cap_batch_));
        CK(cudaMalloc(&d_batch_items_, sizeof(int4) * cap_batch_));
        CK(cudaMalloc(&d_attach_slots_, sizeof(int) * cap_attach_));
        return 0;
    }

    // A pinned buffer of at least `bytes`, once its previous copy has finished.
    // Every host<->device copy of the engine goes through these, which count the bytes
    // (vx3_transfer_bytes).
    int64_t h2d_bytes_ = 0, d2h_bytes_ = 0;
    void count_copy(size_t n, cudaMemcpyKind k) {
        if (k == cudaMemcpyHostToDevice) h2d_bytes_ += (int64_t)n;
        else if (k == cudaMemcpyDeviceToHost) d2h_bytes_ += (int64_t)n;
    }
    cudaError_t copy_async(void* dst, const void* src, size_t n, cudaMemcpyKind k, cudaStream_t st) {
        count_copy(n, k);
        return cudaMemcpyAsync(dst, src, n, k, st);
    }
    cudaError_t copy2d_async(void* dst, size_t dp, const void* src, size_t sp, size_t w, size_t h, cudaMemcpyKind k, cudaStream_t st) {
        count_copy(w * h, k);
        return cudaMemcpy2DAsync(dst, dp, src, sp, w, h, k, st);
    }
    cudaError_t copy_sync(void* dst, const void* src, size_t n, cudaMemcpyKind k) {
        count_copy(n, k);
        return cudaMemcpy(dst, src, n, k);
    }
    void transfer_bytes(int64_t* h2d, int64_t* d2h) const override { *h2d = h2d_bytes_; *d2h = d2h_bytes_; }

    int pinned(Pinned* b, size_t bytes, std::string* err) {
        CK(cudaEventSynchronize(b->done));
        if (b->cap >= bytes) return 0;
        pinned_cache().give(b->p, b->cap);
        b->p = nullptr;
        b->cap = 0;
        size_t cap = 0;
        if (char* p = pinned_cache().take(bytes, &cap)) { b->p = p; b->cap = cap; return 0; }
        cap = std::max<size_t>(bytes, 16u << 20);
        CK(cudaHostAlloc((void**)&b->p, cap, cudaHostAllocPortable));
        b->cap = cap;
        return 0;
    }

    int grow_slots(int n, std::string* err) {
        if (n <= cap_slots_) return 0;
        int nc = std::max(n, 2 * cap_slots_);
        dev::Sim* ns = nullptr;
        dev::Ctl* nctl = nullptr;
        CK(cudaMalloc(&ns, sizeof(dev::Sim) * nc));
        CK(cudaMalloc(&nctl, sizeof(dev::Ctl) * nc));
        CK(cudaMemset(nctl, 0, sizeof(dev::Ctl) * nc));
        if (cap_slots_) {
            CK(cudaStreamSynchronize(stream_));
            CK(copy_sync(ns, d_sims_, sizeof(dev::Sim) * cap_slots_, cudaMemcpyDeviceToDevice));
            CK(copy_sync(nctl, d_ctl_, sizeof(dev::Ctl) * cap_slots_, cudaMemcpyDeviceToDevice));
            cudaFree(d_sims_);
            cudaFree(d_ctl_);
        }
        d_sims_ = ns;
        d_ctl_ = nctl;
        slot_owner_.resize(nc, nullptr);
        cap_slots_ = nc;
        batch_dirty_ = true;
        return 0;
    }

    int64_t sim_bytes_world(const SimWorld& w) const {
        Layout L;
        compute_layout(w, &L, nullptr);
        return (int64_t)L.total;
    }
    int64_t sim_bytes(const SimDesc& d) const override {
        SimWorld w;
        std::string e;
        if (!build_world(d, &w, &e)) return -1;
        return sim_bytes_world(w);
    }
    int64_t sim_bytes_id(int64_t id) override {
        SimRec* r = find(id);
        return r ? sim_bytes_world(r->w) : -6;
    }
    int set_precision(int fma) override {
        ks_ = fma ? kernelset_fast() : kernelset_exact();
        if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
        batch_dirty_ = true;
        return 0;
    }
    int precision() const override { return ks_.name[0] == 'f' ? 1 : 0; }

    // VX3 extras that change the topology during the run (link detachment, material
    // removal): the contact search then lists every voxel and skips interior ones.
    static bool removes_materials(const SimDesc& d) {
        if (!d.secondary_experiment) return false;
        for (auto& m : d.mats) if (m.remove_after > 0) return true;
        return false;
    }
    static bool dynamic_surface(const SimDesc& d) { return d.enable_detach || removes_materials(d) || attaches(d); }
    static int contact_list_size(const SimWorld& w) { return dynamic_surface(w.desc) ? w.nv : w.surface_count; }
    // Contacts from watch lists regenerated as the reference does (collisions on, a surface that
    // does not change during the run); kWatchPerVoxel partners per surface voxel on average fit
    // (the reference's lists hold about 7 on a 40^3 creature at fill 0.5), more fall back to the
    // per-step hash search until the next regeneration
    static bool watches(const SimDesc& d) { return d.collisions && !dynamic_surface(d); }
    static constexpr int kWatchPerVoxel = 32;
    // VX3 attachment needs the contact pass to find touching pairs; links made at run time
    // take slots nl .. 3*nv-1 (every voxel has six link directions)
    static bool attaches(const SimDesc& d) { return d.enable_attach && d.collisions; }
    static int link_capacity(const SimWorld& w) { return attaches(w.desc) ? std::max(w.nl, 3 * w.nv) : w.nl; }
    static int target_count(const SimWorld& w) {
        std::vector<char> target(w.desc.mats.size(), 0);
        bool any = false;
        for (size_t m = 0; m < w.desc.mats.size(); m++) any |= (target[m] = w.desc.mats[m].is_target ? 1 : 0) != 0;
        if (!any) return 0;
        int n = 0;
        for (int i = 0; i < w.nv; i++) n += target[(size_t)w.desc.voxels[4 * i + 3]];
        return n;
    }

    struct Offs {
        size_t vm, lm, ext, pos[3], mom[3], q[4], am[3], temp, ps, vfl, vmat, vext, phase, sf, sm, ss;
        size_t lneg, lpos, lax, lmt, lst, lsf, lfl, surf, ijk, reach, ccount, cforce, cspill, hhead, hnext, cpos, cilia, ffield;
        size_t watch, woff, wlist;
        size_t shift, sig, vlink, targets, init_pos, lnew, cand, cpart, acond;
        size_t zero_from;   // everything from here on starts as zeros
        int hash_size;
    };
    static void compute_layout(const SimWorld& w, Layout* L, Offs* o) {
        Offs t{};
        const size_t nv = w.nv, nl = link_capacity(w);
        const bool col = w.desc.collisions;
        const SimDesc& d = w.desc;
        // arrays with initial data first, then the ones that start as zeros (cleared on the
        // device, so that the host builds and copies only the first part)
        t.vm = L->add(sizeof(dev::VMat) * w.vmats.size());
        t.lm = L->add(sizeof(dev::LMat) * std::max<size_t>(1, w.lmats.size()));
        t.ext = L->add(sizeof(dev::Ext) * std::max<size_t>(1, w.desc.externals.size()));
        t.vfl = L->add(4 * nv);
        t.vmat = L->add(nv);
        t.vext = L->add(4 * nv);
        t.phase = L->add(8 * nv);
        t.lneg = L->add(4 * std::max<size_t>(1, nl));
        t.lpos = L->add(4 * std::max<size_t>(1, nl));
        t.lax = L->add(std::max<size_t>(1, nl));
        t.lmt = L->add(std::max<size_t>(1, nl));
        t.lfl = L->add(std::max<size_t>(1, nl));
        t.ijk = L->add(2 * 3 * nv);
        if (col) {
            size_t ns = std::max(1, contact_list_size(w));
            int hs = 1;
            while (hs < 2 * (int)ns) hs <<= 1;
            t.hash_size = hs;
            t.surf = L->add(4 * ns);
            t.reach = L->add(4 * dev::kReachWords * nv);
            t.hhead = L->add(4 * 2 * (size_t)hs);
        }
        if (w.desc.enable_cilia) t.cilia = L->add(8 * 3 * nv);
        if (w.desc.has_force_field) t.ffield = L->add(sizeof(MathTree) * 3);
        if (d.enable_signals && d.enable_cilia && !d.shift_cilia.empty()) t.shift = L->add(8 * 3 * nv);
        if (d.enable_signals || removes_materials(d) || attaches(d)) t.vlink = L->add(4 * 6 * nv);
        if (attaches(d)) t.acond = L->add(sizeof(MathTree) * 5);
        if (int nt = target_count(w)) t.targets = L->add(4 * (size_t)nt);
        if (d.secondary_experiment) t.init_pos = L->add(8 * 3 * nv);
        t.zero_from = L->total;
        // the initial positions (lattice index x voxel size) and orientations (identity) are
        // written on the device at upload (k_init_temp), so they are not copied
        for (int k = 0; k < 3; k++) t.pos[k] = L->add(8 * nv);
        t.q[0] = L->add(8 * nv);
        for (int k = 0; k < 3; k++) t.mom[k] = L->add(8 * nv);
        for (int k = 1; k < 4; k++) t.q[k] = L->add(8 * nv);
        for (int k = 0; k < 3; k++) t.am[k] = L->add(8 * nv);
        t.temp = L->add(4 * nv);
        t.ps = L->add(4 * 3 * nv);
        t.sf = L->add(8 * 18 * nv);
        t.sm = L->add(8 * 18 * nv);
        t.ss = L->add(4 * 6 * nv);
        t.lst = L->add(8 * 9 * std::max<size_t>(1, nl));
        t.lsf = L->add(4 * 3 * std::max<size_t>(1, nl));
        if (col) {
            t.ccount = L->add(4 * nv);
            t.cforce = L->add(4 * 3 * dev::kContactInline * nv);
            t.cspill = L->add(4 * nv);
            t.hnext = L->add(4 * nv);
            t.cpos = L->add(16 * nv);
            if (watches(d)) {
                const size_t ns = std::max(1, contact_list_size(w));
                t.watch = L->add(16 * nv);
                t.woff = L->add(4 * 2 * ns);   // per surface voxel: its run's start and length
                t.wlist = L->add(4 * (size_t)kWatchPerVoxel * ns);
            }
        }
        if (d.enable_signals) t.sig = L->add(8 * dev::SG_FIELDS * nv);
        if (attaches(d)) {
            t.lnew = L->add(4 * nl);
            t.cand = L->add(8 * (size_t)kAttachCandPerVoxel * nv + 8);
            t.cpart = L->add(4 * (size_t)dev::kContactInline * nv);
        }
        if (o) *o = t;
    }

    int add_sim(const SimDesc& d, int64_t* id, std::string* err) override {
        auto r = std::make_unique<SimRec>();
        if (!prepare(d, r.get(), err)) return -1;
        r->id = next_id_++;
        *id = r->id;
        r->submit_s = now_s() - t0_;
        sims_[r->id] = std::move(r);
        return 0;
    }

    int add_sims(const SimDesc* const* descs, int n, int64_t* ids, std::string* errs) override {
        return add_sims_with(n, [&](int i, SimRec* r, std::string* e) { return prepare(*descs[i], r, e); }, ids, errs);
    }

    int add_sims_read(int n, const std::function<bool(int, SimDesc*, std::string*)>& read, int64_t* ids,
                      std::string* errs) override {
        return add_sims_with(n, [&](int i, SimRec* r, std::string* e) {
            SimDesc d;
            return read(i, &d, e) && prepare(d, r, e);
        }, ids, errs);
    }

    // make(i, rec, err) prepares simulation i's record on one of the host threads
    template <typename Make>
    int add_sims_with(int n, const Make& make, int64_t* ids, std::string* errs) {
        TraceClock tc;
        std::vector<std::unique_ptr<SimRec>> recs((size_t)std::max(n, 0));
        std::vector<char> ok((size_t)std::max(n, 0), 0);
        std::atomic<int> next{0};
        auto work = [&]() {
            for (int i = next++; i < n; i = next++) {
                recs[i] = std::make_unique<SimRec>();
                ok[i] = make(i, recs[i].get(), &errs[i]) ? 1 : 0;
            }
        };
        const int nt = std::max(1, std::min(n, (int)std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; t++) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
        tc.mark("add_sims: topology (threads)");
        int rejected = 0;
        const double now = now_s() - t0_;
        for (int i = 0; i < n; i++) {
            if (!ok[i]) { ids[i] = -1; rejected++; continue; }
            recs[i]->id = next_id_++;
            recs[i]->submit_s = now;
            ids[i] = recs[i]->id;
            sims_[ids[i]] = std::move(recs[i]);
        }
        return rejected;
    }

    // Host part of loading one simulation (thread-safe): topology, materials, initial centre of mass.
    static bool prepare(const SimDesc& d, SimRec* r, std::string* err) {
        if (!build_world(d, &r->w, err)) return false;
        // initial centre of mass from the lattice positions
        double sx = 0, sy = 0, sz = 0, tm = 0;
        for (int i = 0; i < r->w.nv; i++) {
            const VoxelMaterial& m = r->w.vmats[d.voxels[4 * i + 3]];
            if (!m.is_measured) continue;
            r->num_measured++;
            double wgt = m.mass;
            sx += d.voxels[4 * i] * m.nom * wgt; sy += d.voxels[4 * i + 1] * m.nom * wgt; sz += d.voxels[4 * i + 2] * m.nom * wgt;
            tm += wgt;
        }
        if (tm != 0) { r->init_com[0] = sx / tm; r->init_com[1] = sy / tm; r->init_com[2] = sz / tm; }
        return true;
    }

    SimRec* find(int64_t id) {
        auto it = sims_.find(id);
        return it == sims_.end() ? nullptr : it->second.get();
    }

    int set_external(int64_t id, const External& x, std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        if (r->resident) { *err = "externals must be set before the first step"; return -7; }
        if (x.voxel < 0 || x.voxel >= r->w.nv) { *err = "voxel index out of range"; return -6; }
        auto& ex = r->w.desc.externals;
        bool found = false;
        for (auto& e : ex) if (e.voxel == x.voxel) { e = x; found = true; }
        if (!found) ex.push_back(x);
        std::string e2;
        SimDesc dd = r->w.desc;
        if (!build_world(dd, &r->w, &e2)) { *err = e2; return -1; }
        return 0;
    }

    int free_slot() {
        for (int i = 0; i < cap_slots_; i++) if (!slot_owner_[i]) return i;
        return -1;
    }

    // Copies a simulation's topology and initial state to the device.
    int upload(SimRec* r, std::string* err) {
        if (r->resident) return 0;
        std::vector<SimRec*> one;
        if (int e = upload_begin(r, err)) return e;
        one.push_back(r);
        return upload_finish(one, err);
    }

    // Region of one simulation being uploaded: its layout and where it sits in the arena.
    struct UpPlan {
        Layout L;
        Offs o;
        size_t off = 0;
    };

    // The device powf tables of a simulation's Poisson ratios (made on first use).
    int ensure_pow_tables(const SimWorld& w, std::string* err) {
        for (const VoxelMaterial& m : w.vmats) {
            if (m.nu == 0.0f) continue;
            uint32_t key;
            memcpy(&key, &m.nu, 4);
            if (dev_pow_.count(key)) continue;
            const float* d = device_pow_table(device_, m.nu, &h2d_bytes_, err);
            if (!d) return -5;
            dev_pow_[key] = d;
        }
        return 0;
    }
    const float* pow_table_of(float nu) const {
        if (nu == 0.0f) return nullptr;
        uint32_t key;
        memcpy(&key, &nu, 4);
        auto it = dev_pow_.find(key);
        return it == dev_pow_.end() ? nullptr : it->second;
    }

    // Serial part of an upload: layout, arena region and slot.
    int upload_reserve(SimRec* r, UpPlan* p, std::string* err) {
        SimWorld& w = r->w;
        if (int e = ensure_pow_tables(w, err)) return e;
        Layout& L = p->L;
        Offs& o = p->o;
        compute_layout(w, &L, &o);
        size_t& off = p->off;
        if (!arena_.alloc(L.total, &off)) {
            if (err) *err = "HBM budget exhausted";
            return -2;
        }
        int slot = free_slot();
        if (slot < 0) {
            int e = grow_slots(cap_slots_ * 2, err);
            if (e) { arena_.release(off, L.total); return e; }
            slot = free_slot();
        }
        slot_owner_[slot] = r;   // taken now, so that the next begun upload picks another slot
        r->slot = slot;
        r->off = off;
        r->bytes = L.total;
        return 0;
    }

    // Host image of a reserved region's initialised part at hp (o.zero_from bytes), and the
    // simulation's device descriptor and first control block.  Writes only hp and r, so the
    // images of many simulations are filled at once on host threads.
    void upload_fill(SimRec* r, const UpPlan& p, char* hp) const {
        SimWorld& w = r->w;
        const Layout& L = p.L;
        const Offs& o = p.o;
        char* base = arena_base_ + p.off;
        (void)L;
        memset(hp, 0, o.zero_from);
        const size_t nv = w.nv, nl = w.nl;
        auto P = [&](size_t o2) { return hp + o2; };
        // materials
        dev::VMat* vm = (dev::VMat*)P(o.vm);
        for (size_t i = 0; i < w.vmats.size(); i++) {
            const VoxelMaterial& m = w.vmats[i];
            dev::VMat& x = vm[i];
            x.E = m.E; x.nu = m.nu; x.cte = m.cte; x.mus = m.mus; x.muk = m.muk; x.eHat = m.eHat;
            x.mass = m.mass; x.massInv = m.massInv; x.Iinv = m.Iinv;
            x.dampNum = 2 * m.sqrtMass * m.zi;
            x.gDampT = m.zg * m.c2m; x.gDampR = m.zg * m.c2i; x.cDampT = m.zc * m.c2m;
            x.gravForce = -m.mass * 9.80665f * m.grav;
            x.penStiff = (float)(2 * m.E * m.nom);
            x.sizef = (float)m.nom;
            x.nom = m.nom;
            x.measured = m.is_measured;
            x.massInvD = x.massInv; x.IinvD = x.Iinv; x.gDampTD = x.gDampT; x.gDampRD = x.gDampR; x.cDampTD = x.cDampT;
            x.gravForceD = x.gravForce;
            x.halfNom = m.nom / 2;
            x.halfMassInv = 0.5 * (double)x.massInv;
            const PaletteMaterial& pm = w.desc.mats[i];
            x.cilia = pm.cilia;
            x.ciliaOn = pm.cilia_on_after;
            x.thermalOn = pm.thermal_on_after;
            x.vx3 = (pm.is_target ? dev::VM_TARGET : 0) | (pm.is_pacemaker ? dev::VM_PACEMAKER : 0) | (pm.fixed ? dev::VM_FIXED : 0);
            x.pmPeriod = pm.pacemaker_period;
            x.sigDecay = pm.signal_decay;
            x.sigDelay = pm.signal_delay;
            x.sigInactive = pm.inactive_period;
            x.removeAfter = pm.remove_after;
            x.attachLmat = w.attach_lmat.empty() ? -1 : w.attach_lmat[i];
            x.powtab = pow_table_of(m.nu);
            if (pm.sticky) x.vx3 |= dev::VM_STICKY;
        }
        dev::LMat* lm = (dev::LMat*)P(o.lm);
        for (size_t i = 0; i < w.lmats.size(); i++) {
            const LinkMaterial& m = w.lmats[i];
            dev::LMat& x = lm[i];
            x.E = m.E; x.nu = m.nu; x.eHat = m.eHat; x.a1 = m.a1; x.a2 = m.a2; x.b1 = m.b1; x.b2 = m.b2; x.b3 = m.b3;
            x.sqA1 = m.sqA1; x.sqA2xIp = m.sqA2xIp; x.sqB1 = m.sqB1; x.sqB2xFMp = m.sqB2xFMp; x.sqB3xIp = m.sqB3xIp;
            x.epsFail = m.epsFail; x.linear = m.linear; x.n = m.n;
            for (int k = 0; k < 18; k++) { x.strain[k] = k < kMaxModelPoints + 2 ? m.strain[k] : 0; x.stress[k] = k < kMaxModelPoints + 2 ? m.stress[k] : 0; }
            x.a2D = x.a2; x.b1D = x.b1; x.b2D = x.b2; x.b3D = x.b3;
            x.sqA1D = x.sqA1; x.sqA2xIpD = x.sqA2xIp; x.sqB1D = x.sqB1; x.sqB2xFMpD = x.sqB2xFMp; x.sqB3xIpD = x.sqB3xIp;
        }
        dev::Ext* ex = (dev::Ext*)P(o.ext);
        for (size_t i = 0; i < w.desc.externals.size(); i++) {
            const External& e = w.desc.externals[i];
            dev::Ext& x = ex[i];
            x.dof = e.dof_fixed;
            for (int k = 0; k < 3; k++) { x.f[k] = e.force[k]; x.m[k] = e.moment[k]; x.tr[k] = e.translate[k]; }
            double rx = e.rotate[0], ry = e.rotate[1], rz = e.rotate[2];
            if (rx != 0 || ry != 0 || rz != 0) {
                /* CVX_External::rotationChanged -> Quat3D::FromRotationVector (Quat3D.h:128-143) */
                double tx = 0.5 * rx, ty = 0.5 * ry, tz = 0.5 * rz;
                double m2 = tx * tx + ty * ty + tz * tz, qw, s;
                if (m2 * m2 < 5.328e-15) { qw = 1.0 - 0.5 * m2; s = 1.0 - m2 / 6.0; }
                else { double mm = sqrt(m2); qw = cos(mm); s = sin(mm) / mm; }
                x.rq[0] = qw; x.rq[1] = tx * s; x.rq[2] = ty * s; x.rq[3] = tz * s;
            } else { x.rq[0] = 1; x.rq[1] = x.rq[2] = x.rq[3] = 0; }
        }
        uint32_t* vfl = (uint32_t*)P(o.vfl);
        uint8_t* vmat = (uint8_t*)P(o.vmat);
        int32_t* vext = (int32_t*)P(o.vext);
        double* ph = (double*)P(o.phase);
        int16_t* ijk = (int16_t*)P(o.ijk);
        for (size_t i = 0; i < nv; i++) {
            int mi = w.desc.voxels[4 * i + 3];
            double nom = w.vmats[mi].nom;
            uint32_t f = dev::VF_STATIC;
            for (int d = 0; d < 6; d++) if (w.vox_links[i * 6 + d] >= 0) f |= 1u << d;
            if (w.vox_interior[i]) f |= dev::VF_INTERIOR;
            if (w.vox_ext[i] >= 0) f |= dev::VF_EXT;
            if (w.vmats[mi].is_measured) f |= dev::VF_MEASURED;
            if (attaches(w.desc)) f |= dev::VF_ATTACH;   // enableAttach starts true (VX3_Voxel.h:302)
            vfl[i] = f;
            vmat[i] = (uint8_t)mi;
            vext[i] = w.vox_ext[i];
            ph[i] = w.desc.phase.empty() ? 0.0 : w.desc.phase[i];
            for (int k = 0; k < 3; k++) ijk[k * nv + i] = (int16_t)w.desc.voxels[4 * i + k];
        }
        memcpy(P(o.lneg), w.link_neg.data(), 4 * nl);
        memcpy(P(o.lpos), w.link_pos.data(), 4 * nl);
        memcpy(P(o.lax), w.link_axis.data(), nl);
        memcpy(P(o.lmt), w.link_mat.data(), nl);
        memset(P(o.lfl), dev::LF_SMALL, std::max<size_t>(1, nl));
        const size_t nl_cap = link_capacity(w);
        if (nl_cap > nl) memset(P(o.lfl) + nl, dev::LF_GONE, nl_cap - nl);   // slots for links made at run time
        int flags = 0;
        if (w.desc.floor) flags |= dev::SF_FLOOR;
        if (w.desc.collisions) flags |= dev::SF_COLLIDE;
        if (watches(w.desc)) flags |= dev::SF_WATCH;
        if (w.desc.vary_temp && w.desc.temp_period > 0) flags |= dev::SF_VARY;
        if (w.desc.enable_expansion) flags |= dev::SF_EXPAND;
        if (w.desc.enable_cilia) {
            flags |= dev::SF_CILIA;
            double* c = (double*)P(o.cilia);   // 3 blocks of nv; zeros where the VXA gives none
            for (size_t i = 0; i < nv && 3 * i + 2 < w.desc.base_cilia.size(); i++)
                for (int k = 0; k < 3; k++) c[k * nv + i] = w.desc.base_cilia[3 * i + k];
        }
        if (w.desc.has_force_field) {
            flags |= dev::SF_FFIELD;
            memcpy(P(o.ffield), w.desc.force_field, sizeof(MathTree) * 3);
        }
        const SimDesc& dd = w.desc;
        if (dd.enable_signals) {
            flags |= dev::SF_SIGNALS;
            if (dd.enable_cilia && !dd.shift_cilia.empty()) {
                double* c = (double*)P(o.shift);   // 3 blocks of nv
                for (size_t i = 0; i < nv && 3 * i + 2 < dd.shift_cilia.size(); i++)
                    for (int k = 0; k < 3; k++) c[k * nv + i] = dd.shift_cilia[3 * i + k];
            }
        }
        if (dd.enable_signals || removes_materials(dd) || attaches(dd)) memcpy(P(o.vlink), w.vox_links.data(), 4 * 6 * nv);
        if (attaches(dd)) {
            flags |= dev::SF_ATTACH;
            memcpy(P(o.acond), dd.attach_cond, sizeof(MathTree) * 5);
        }
        const int n_targets = target_count(w);
        if (n_targets) {
            flags |= dev::SF_TARGETS;
            int32_t* tg = (int32_t*)P(o.targets);
            int k = 0;
            for (size_t i = 0; i < nv; i++) if (dd.mats[dd.voxels[4 * i + 3]].is_target) tg[k++] = (int32_t)i;
        }
        if (dd.enable_detach) flags |= dev::SF_DETACH;
        if (dd.secondary_experiment) {
            flags |= dev::SF_REMOVE;
            double* ip = (double*)P(o.init_pos);
            for (size_t i = 0; i < nv; i++) {
                const double nom = w.vmats[w.desc.voxels[4 * i + 3]].nom;
                ip[i] = w.desc.voxels[4 * i] * nom; ip[nv + i] = w.desc.voxels[4 * i + 1] * nom; ip[2 * nv + i] = w.desc.voxels[4 * i + 2] * nom;
            }
        }
        for (auto& pm : dd.mats) if (pm.fixed) flags |= dev::SF_FIXEDMAT;
        double max_bsa = 0;
        if (w.desc.collisions) {
            int32_t* surf = (int32_t*)P(o.surf);
            int k = 0;
            const bool all = dynamic_surface(w.desc);
            for (size_t i = 0; i < nv; i++) if (all || !w.vox_interior[i]) surf[k++] = (int32_t)i;
            std::vector<uint32_t> masks = reach_masks(w, 5, dev::kReachWords);
            memcpy(P(o.reach), masks.data(), 4 * masks.size());
            memset(P(o.hhead), 0xFF, 4 * 2 * (size_t)o.hash_size);
            // largest contact distance: 0.625*(bsa1+bsa2) with the largest actuation expansion
            double amp = (flags & dev::SF_VARY) ? fabs(w.desc.temp_amplitude) : fabs(w.desc.initial_temp);
            for (auto& m : w.vmats) max_bsa = std::max(max_bsa, m.nom * (1 + amp * fabs(m.cte)));
        }
        dev::Sim& S = r->dsim;
        S = dev::Sim{};
        S.nv = (int)nv; S.nl = (int)nl_cap; S.nsurf = contact_list_size(w); S.flags = flags;
        S.temp_amp = w.desc.temp_amplitude; S.temp_period = w.desc.temp_period;
        S.cell_size = std::max(1e-9, 2 * 0.625 * max_bsa * 1.01);
        S.hash_size = o.hash_size > 0 ? o.hash_size : 1;
        S.env_radius = 0.625f;
        auto D = [&](size_t o2) { return base + o2; };
        S.vm = (const dev::VMat*)D(o.vm); S.lm = (const dev::LMat*)D(o.lm); S.ext = (const dev::Ext*)D(o.ext);
        S.px = (double*)D(o.pos[0]); S.py = (double*)D(o.pos[1]); S.pz = (double*)D(o.pos[2]);
        S.mx = (double*)D(o.mom[0]); S.my = (double*)D(o.mom[1]); S.mz = (double*)D(o.mom[2]);
        S.qw = (double*)D(o.q[0]); S.qx = (double*)D(o.q[1]); S.qy = (double*)D(o.q[2]); S.qz = (double*)D(o.q[3]);
        S.ax = (double*)D(o.am[0]); S.ay = (double*)D(o.am[1]); S.az = (double*)D(o.am[2]);
        S.temp = (float*)D(o.temp); S.ps = (float*)D(o.ps); S.vfl = (uint32_t*)D(o.vfl);
        S.vmat = (const uint8_t*)D(o.vmat); S.vext = (const int32_t*)D(o.vext); S.phase = (const double*)D(o.phase);
        S.sf = (double*)D(o.sf); S.sm = (double*)D(o.sm); S.ss = (float*)D(o.ss);
        S.lneg = (int32_t*)D(o.lneg); S.lpos = (int32_t*)D(o.lpos);
        S.lax = (uint8_t*)D(o.lax); S.lmt = (uint8_t*)D(o.lmt);
        S.lst = (double*)D(o.lst); S.lsf = (float*)D(o.lsf); S.lfl = (uint8_t*)D(o.lfl);
        S.ijk = (const int16_t*)D(o.ijk);
        if (w.desc.collisions) {
            S.surf = (const int32_t*)D(o.surf); S.reach = (const uint32_t*)D(o.reach);
            S.ccount = (int32_t*)D(o.ccount); S.cforce = (float*)D(o.cforce); S.cspill = (int32_t*)D(o.cspill);
            S.spill_p = d_spill_p_; S.spill_f = d_spill_f_; S.spill_used = d_tickets_ + kSpillTicket; S.spill_cap = spill_cap_;
            S.contact_inline = contact_inline_;
            if (watches(dd)) {
                // the reference's radii (CVoxelyze::updateCollisions, Voxelyze.cpp:673-675), in float
                const float watchVx = 2 * dd.bounding_radius + dd.watch_distance;
                const float watchMm = (float)(dd.vox_size * watchVx);
                const float recalc = (float)(dd.vox_size * dd.watch_distance / 2);
                S.watch = (float4*)D(o.watch);
                S.woff = (int32_t*)D(o.woff);
                S.wlist = (int32_t*)D(o.wlist);
                S.wcap = kWatchPerVoxel * std::max(1, contact_list_size(w));
                S.watch_r2 = watchMm * watchMm;
                S.recalc2 = recalc * recalc;
                S.wcells = (int)std::floor(1.03 * watchMm / S.cell_size) + 1;
            }
            S.hash_head = (int32_t*)D(o.hhead); S.hash_next = (int32_t*)D(o.hnext);
            S.cpos = (float4*)D(o.cpos);
            S.inv_cell = (float)(1.0 / S.cell_size);
        }
        if (w.desc.enable_cilia) S.cilia = (const double*)D(o.cilia);
        if (w.desc.has_force_field) S.ffield = (const MathTree*)D(o.ffield);
        if (dd.enable_signals) {
            S.sig = (double*)D(o.sig);
            if (dd.enable_cilia && !dd.shift_cilia.empty()) S.shift_cilia = (const double*)D(o.shift);
        }
        if (dd.enable_signals || removes_materials(dd) || attaches(dd)) S.vlink = (int32_t*)D(o.vlink);
        if (attaches(dd)) {
            S.nl_cap = (int)nl_cap;
            S.cand_cap = kAttachCandPerVoxel * (int)nv + 1;
            S.safety_guard = dd.safety_guard;
            S.attach_mask = dd.attach_cond_mask;
            S.lnew = (int32_t*)D(o.lnew);
            S.cand = (int32_t*)D(o.cand);
            S.cpart = (int32_t*)D(o.cpart);
            S.attach_cond = (const MathTree*)D(o.acond);
        }
        if (n_targets) { S.targets = (const int32_t*)D(o.targets); S.n_targets = n_targets; }
        S.close_r = dd.max_dist_pairs * dd.vox_size;   // MaxDistInVoxelLengthsToCountAsPair * voxSize
        S.n_mats = (int)w.vmats.size();
        S.reinit_after = dd.reinit_initial_after;
        if (dd.secondary_experiment) S.init_pos = (double*)D(o.init_pos);
        // the descriptor and control block go to the device with the others in upload_finish
        r->pending_sim = S;
        dev::Ctl c{};
        c.status = SIM_IDLE;
        c.stop = w.desc.stop_formula;
        c.hash_parity = 0;
        // currentCenterOfMass starts as the initial one (VX3_SimulationManager.cu:54-55)
        for (int k = 0; k < 3; k++) c.com[k] = c.init_com[k] = r->init_com[k];
        c.n_links = w.nl;
        c.col_stale = 1;   // the first step regenerates the watch lists (the reference's nearbyStale)
        c.watch_ok = 1;    // until the regeneration finds the lists too small
        c.watch_used = 0;
        r->pending_ctl = c;
    }

    // Copies a filled image to its region and clears the rest of the region on the device.
    int upload_copy(SimRec* r, const UpPlan& p, const char* hp, std::string* err) {
        char* base = arena_base_ + p.off;
        const size_t img = p.o.zero_from;
        CK(copy_async(base, hp, img, cudaMemcpyHostToDevice, stream_));
        CK(cudaMemsetAsync(base + img, 0, p.L.total - img, stream_));
        (void)r;
        return 0;
    }

    // First half of an upload of one simulation, without waiting for the device: region
    // image in a pinned staging buffer (pageable for huge regions) whose copy runs while the
    // next simulation's image is filled.  Many simulations are begun and then finished
    // together (one synchronisation for the whole generation); upload_many fills the images
    // of a whole generation at once on host threads.
    int upload_begin(SimRec* r, std::string* err) {
        UpPlan p;
        if (int e = upload_reserve(r, &p, err)) return e;
        const size_t img = p.o.zero_from;
        std::vector<char> hv;
        char* hp = nullptr;
        Pinned* stage = nullptr;
        if (img <= kPinnedUploadMax) {
            stage = &up_[up_next_];
            up_next_ ^= 1;
            if (int e = pinned(stage, img, err)) {
                arena_.release(p.off, p.L.total);
                slot_owner_[r->slot] = nullptr;
                return e;
            }
            hp = stage->p;
        } else {
            hv.resize(img);
            hp = hv.data();
        }
        upload_fill(r, p, hp);
        if (int e = upload_copy(r, p, hp, err)) return e;
        if (stage) CK(cudaEventRecord(stage->done, stream_));
        return 0;
    }

    // Begins the uploads of many simulations: regions reserved in order, every image filled
    // on host threads into one pinned generation buffer, then the copies in order.  Returns
    // the number begun (those before a failure) through *begun.
    int upload_many(const std::vector<SimRec*>& rs, std::vector<SimRec*>* begun, std::string* err) {
        TraceClock tc;
        std::vector<UpPlan> plans(rs.size());
        std::vector<size_t> at(rs.size());
        size_t total = 0;
        size_t k = 0;
        int rc = 0;
        for (; k < rs.size(); k++) {
            if ((rc = upload_reserve(rs[k], &plans[k], err))) break;
            at[k] = total;
            total += (plans[k].o.zero_from + 255) & ~(size_t)255;
        }
        const size_t n = k;
        if (n == 0) return rc;
        // on a failure below, the regions reserved but not begun are given back
        auto unreserve_from = [&](size_t i0) {
            for (size_t i = i0; i < n; i++) {
                arena_.release(plans[i].off, plans[i].L.total);
                slot_owner_[rs[i]->slot] = nullptr;
            }
        };
        if (total > kPinnedUploadMax) {
            // too large for one staging buffer: the regions are already reserved, so fill and
            // copy them one at a time through the double-buffered staging
            for (size_t i = 0; i < n; i++) {
                const size_t img = plans[i].o.zero_from;
                std::vector<char> hv;
                char* hp;
                Pinned* stage = nullptr;
                if (img <= kPinnedUploadMax) {
                    stage = &up_[up_next_];
                    up_next_ ^= 1;
                    if (int e = pinned(stage, img, err)) { unreserve_from(i); return e; }
                    hp = stage->p;
                } else {
                    hv.resize(img);
                    hp = hv.data();
                }
                upload_fill(rs[i], plans[i], hp);
                if (int e = upload_copy(rs[i], plans[i], hp, err)) { unreserve_from(i); return e; }
                if (stage) CK(cudaEventRecord(stage->done, stream_));
                begun->push_back(rs[i]);
            }
            return rc;
        }
        tc.mark("upload_many: reserve");
        // the images, then the list of region copies, in one pinned buffer and one copy to a
        // device staging buffer; one kernel then places every image and clears the rest of
        // every region (per-region copies and clears were a thousand small operations)
        const size_t o_list = align256(total), stage_bytes = o_list + sizeof(RegionCopy) * n;
        if (int e = pinned(&gen_, stage_bytes, err)) { unreserve_from(0); return e; }
        // the staging area: a temporary region of the arena (given back once upload_finish has
        // waited for the copies), else a buffer of the context's own
        char* stage = nullptr;
        size_t stage_off = 0;
        if (stage_off_ == kNoStage && arena_.alloc(stage_bytes, &stage_off)) {
            stage = arena_base_ + stage_off;
            stage_off_ = stage_off;
            stage_len_ = stage_bytes;
        } else {
            if (stage_bytes > cap_stage_) {
                CK(cudaStreamSynchronize(stream_));
                cudaFree(d_stage_);
                d_stage_ = nullptr;
                cap_stage_ = 0;
                if (cudaMalloc(&d_stage_, stage_bytes) != cudaSuccess) { unreserve_from(0); if (err) *err = "device staging buffer"; return -5; }
                cap_stage_ = stage_bytes;
            }
            stage = d_stage_;
        }
        tc.mark("upload_many: pinned buffer");
        std::atomic<size_t> next{0};
        auto work = [&]() {
            for (size_t i = next++; i < n; i = next++) upload_fill(rs[i], plans[i], gen_.p + at[i]);
        };
        const int nt = (int)std::max<size_t>(1, std::min<size_t>(n / 8, std::max(1u, std::thread::hardware_concurrency())));
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; t++) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
        tc.mark("upload_many: fill (threads)");
        RegionCopy* list = (RegionCopy*)(gen_.p + o_list);
        size_t largest = 0;
        for (size_t i = 0; i < n; i++) {
            list[i] = RegionCopy{at[i], plans[i].off, plans[i].o.zero_from, plans[i].L.total};
            largest = std::max(largest, plans[i].L.total);
        }
        if (cudaError_t e = copy_async(stage, gen_.p, stage_bytes, cudaMemcpyHostToDevice, stream_)) {
            unreserve_from(0);
            cudaStreamSynchronize(stream_);
            release_stage();
            if (err) *err = cudaGetErrorString(e);
            return -5;
        }
        const unsigned bx = (unsigned)std::max<size_t>(1, std::min<size_t>(64, largest >> 20));
        for (size_t k0 = 0; k0 < n; k0 += 65535) {
            const unsigned ny = (unsigned)std::min<size_t>(65535, n - k0);
            k_scatter_regions<<<dim3(bx, ny), 256, 0, stream_>>>(stage, (const RegionCopy*)(stage + o_list) + k0, arena_base_);
        }
        if (cudaError_t e = cudaGetLastError()) {
            unreserve_from(0);
            cudaStreamSynchronize(stream_);
            release_stage();
            if (err) *err = cudaGetErrorString(e);
            return -5;
        }
        for (size_t i = 0; i < n; i++) begun->push_back(rs[i]);
        CK(cudaEventRecord(gen_.done, stream_));
        tc.mark("upload_many: copies issued");
        return rc;
    }

    // Copies per-simulation records img[k] to dev[slot of rs[k]]: one copy per run of
    // consecutive slots (a fresh batch takes consecutive slots, so usually one in all).
    template <typename T>
    int copy_runs(T* dev, const T* img, const std::vector<SimRec*>& rs, std::string* err) {
        size_t k = 0;
        while (k < rs.size()) {
            size_t e = k + 1;
            while (e < rs.size() && rs[e]->slot == rs[e - 1]->slot + 1) e++;
            CK(copy_async(dev + rs[k]->slot, img + k, sizeof(T) * (e - k), cudaMemcpyHostToDevice, stream_));
            k = e;
        }
        return 0;
    }

    // Second half: reads every begun simulation's largest link frequency in one strided
    // copy, derives the time steps on the host (the reference's float arithmetic) and
    // writes the control blocks, with one synchronisation in all.
    int upload_finish(const std::vector<SimRec*>& rs, std::string* err) {
        if (rs.empty()) {
            if (stage_off_ != kNoStage) { cudaStreamSynchronize(stream_); release_stage(); }
            return 0;
        }
        const size_t n = rs.size();
        // pinned image: descriptors, first control blocks, slot list, initial temperatures,
        // every slot's frequency word, the final control blocks
        auto al = [](size_t x) { return (x + 63) & ~(size_t)63; };
        const size_t o_sim = 0, o_ctl0 = al(o_sim + sizeof(dev::Sim) * n), o_slot = al(o_ctl0 + sizeof(dev::Ctl) * n);
        const size_t o_init = al(o_slot + 4 * n), o_bits = al(o_init + 4 * n), o_ctl = al(o_bits + 4 * (size_t)cap_slots_);
        const size_t total = al(o_ctl + sizeof(dev::Ctl) * n);
        TraceClock tf;
        if (int e = pinned(&rb_, total, err)) return e;
        tf.mark("upload_finish: pinned buffer");
        if (total > cap_gather_) {
            CK(cudaStreamSynchronize(stream_));
            tf.mark("upload_finish: sync (gather)");
            cudaFree(d_gather_);
            d_gather_ = nullptr;
            cap_gather_ = 0;
            CK(cudaMalloc(&d_gather_, total));
            cap_gather_ = total;
            tf.mark("upload_finish: gather buffer");
        }
        char* h = rb_.p;
        dev::Sim* sim_img = (dev::Sim*)(h + o_sim);
        dev::Ctl* ctl0_img = (dev::Ctl*)(h + o_ctl0);
        int* slot_img = (int*)(h + o_slot);
        float* init_img = (float*)(h + o_init);
        int max_nv = 1, max_nl = 1, max_ns = 1;
        for (size_t k = 0; k < n; k++) {
            SimRec* r = rs[k];
            sim_img[k] = r->pending_sim;
            ctl0_img[k] = r->pending_ctl;
            slot_img[k] = r->slot;
            init_img[k] = r->w.desc.initial_temp;
            max_nv = std::max(max_nv, r->w.nv);
            max_nl = std::max(max_nl, r->w.nl);
            max_ns = std::max(max_ns, r->w.surface_count);
        }
        if (int e = copy_runs(d_sims_, sim_img, rs, err)) return e;
        if (int e = copy_runs(d_ctl_, ctl0_img, rs, err)) return e;
        CK(copy_async(d_gather_ + o_slot, h + o_slot, o_bits - o_slot, cudaMemcpyHostToDevice, stream_));
        const int* d_slots = (const int*)(d_gather_ + o_slot);
        const float* d_init = (const float*)(d_gather_ + o_init);
        // first actuation temperature (t = 0), then the stable step from it, then the collision hash
        auto blocks = [&](int elems) { return std::max(1, std::min(4 * sm_count_, (elems + 255) / 256) / (int)std::min<size_t>(n, 64)); };
        tf.mark("upload_finish: descriptors");
        ks_.init_temp(blocks(max_nv), stream_, d_sims_, d_slots, d_init, (int)n);
        CK(cudaGetLastError());
        ks_.dt(blocks(max_nl), stream_, d_sims_, d_ctl_, d_slots, (int)n);
        CK(cudaGetLastError());
        ks_.hash_build(blocks(max_ns), stream_, d_sims_, d_ctl_, d_slots, (int)n);
        CK(cudaGetLastError());
        uint32_t* bits_all = (uint32_t*)(h + o_bits);
        dev::Ctl* ctl_img = (dev::Ctl*)(h + o_ctl);
        CK(copy2d_async(bits_all, sizeof(uint32_t), &d_ctl_[0].maxf2_bits, sizeof(dev::Ctl), sizeof(uint32_t), cap_slots_,
                             cudaMemcpyDeviceToHost, stream_));
        tf.mark("upload_finish: set-up launches");
        TraceClock tc;
        CK(cudaStreamSynchronize(stream_));
        tc.mark("upload_finish: wait for copies");
        release_stage();   // the scatter of the region images has run
        for (size_t k = 0; k < rs.size(); k++) {
            SimRec* r = rs[k];
            const SimWorld& w = r->w;
            const uint32_t bits = bits_all[r->slot];
            float maxf2;
            memcpy(&maxf2, &bits, 4);
            if (!(maxf2 > 0.0f)) {   // no links: per-voxel frequencies (Voxelyze.cpp:302-307)
                maxf2 = 0.0f;
                for (int i = 0; i < w.nv; i++) {
                    const VoxelMaterial& m = w.vmats[w.desc.voxels[4 * i + 3]];
                    float f2 = (float)(m.E * m.nom / m.mass);
                    if (f2 > maxf2) maxf2 = f2;
                }
            }
            float opt = maxf2 <= 0.0f ? 0.0f : 1.0f / (6.283185f * sqrtf(maxf2));
            if (opt < 1e-10f) opt = 1e-10f;
            r->optdt = opt;
            r->dt = (float)(w.desc.dt_frac * (double)opt);
            r->cycle_step = r->dt > 0 ? (int)(w.desc.temp_period / r->dt) : 0;
            dev::Ctl& c = ctl_img[k];
            c = r->pending_ctl;
            c.dt = r->dt;
            c.optdt = opt;
            c.cycle_step = r->cycle_step;
            c.maxf2_bits = bits;
            // the first step ends at t = dt (currentTime starts at 0)
            c.t_cycles = (w.desc.vary_temp && w.desc.temp_period > 0) ? (0.0 + (double)c.dt) / w.desc.temp_period : 0.0;
        }
        if (int e = copy_runs(d_ctl_, ctl_img, rs, err)) return e;
        CK(cudaEventRecord(rb_.done, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (SimRec* r : rs) {
            r->resident = true;
            r->status = SIM_IDLE;
        }
        batch_dirty_ = true;
        return 0;
    }

    void release(SimRec* r) {
        if (!r->resident) return;
        cudaStreamSynchronize(stream_);
        arena_.release(r->off, r->bytes);
        slot_owner_[r->slot] = nullptr;
        r->resident = false;
        r->slot = -1;
        batch_dirty_ = true;
    }

    // Builds work items for a set of slots: links, contacts and voxels.
    int build_items(const std::vector<int>& slots, std::string* err) {
        std::vector<dev::Item> items;
        std::vector<int> attach_slots;
        n_link_items_ = n_contact_items_ = n_vox_items_ = 0;
        any_collide_ = any_signals_ = any_watch_ = false;
        for (int s : slots) {
            SimRec* r = slot_owner_[s];
            const int nl = link_capacity(r->w);
            for (int b = 0; b < nl; b += items_links_) items.push_back({s, b, std::min(nl, b + items_links_), 0});
        }
        n_link_items_ = (int)items.size();
        bins_dirty_ = true;
        size_t links_total = 0;
        for (int s : slots) links_total += (size_t)link_capacity(slot_owner_[s]->w);
        batch_links_ = links_total;
        const size_t bins = (size_t)std::max(1, n_link_items_) * dev::kOrderKeysBins;
        if (bins > cap_bins_ || !d_link_total_) {
            cudaFree(d_link_hist_); cudaFree(d_link_base_);
            d_link_hist_ = d_link_base_ = nullptr;
            cap_bins_ = std::max(bins, 2 * cap_bins_);
            CK(cudaMalloc(&d_link_hist_, sizeof(int) * cap_bins_));
            CK(cudaMalloc(&d_link_base_, sizeof(int) * cap_bins_));
            if (!d_link_total_) {
                CK(cudaMalloc(&d_link_total_, sizeof(int)));
                CK(cudaMemsetAsync(d_link_total_, 0, sizeof(int), stream_));
            }
        }
        if (std::max<size_t>(1, links_total) > cap_perm_) {
            cudaFree(d_link_perm_);
            d_link_perm_ = nullptr;
            cap_perm_ = std::max(std::max<size_t>(1, links_total), 2 * cap_perm_);
            CK(cudaMalloc(&d_link_perm_, sizeof(int2) * cap_perm_));
        }
        std::vector<std::pair<int, int>> contact_items(slots.size(), std::make_pair(0, 0));   // per batch entry: first, count
        for (size_t k = 0; k < slots.size(); k++) {
            const int s = slots[k];
            SimRec* r = slot_owner_[s];
            if (r->w.desc.enable_signals) any_signals_ = true;
            if (attaches(r->w.desc)) attach_slots.push_back(s);
            const int ns = contact_list_size(r->w);
            if (!r->w.desc.collisions || ns == 0) continue;
            any_collide_ = true;
            if (watches(r->w.desc)) any_watch_ = true;
            const int chunk = 128;   // at most 128 surface voxels an item (the watch passes' work units rely on it)
            const int first = (int)items.size() - n_link_items_;
            for (int b = 0; b < ns; b += chunk) items.push_back({s, b, std::min(ns, b + chunk), 0});
            contact_items[k] = std::make_pair(first, (int)items.size() - n_link_items_ - first);
        }
        n_contact_items_ = (int)items.size() - n_link_items_;
        std::vector<std::pair<int, int>> ctl_items;   // slot -> (begin, count)
        for (int s : slots) {
            SimRec* r = slot_owner_[s];
            int begin = (int)items.size() - n_link_items_ - n_contact_items_;
            int cnt = 0;
            for (int b = 0; b < r->w.nv; b += items_voxels_) { items.push_back({s, b, std::min(r->w.nv, b + items_voxels_), cnt}); cnt++; }
            r->n_vox_items = cnt;
            ctl_items.emplace_back(begin, cnt);
        }
        n_vox_items_ = (int)items.size() - n_link_items_ - n_contact_items_;
        {
            size_t vox_total = 0;
            for (int s : slots) vox_total += (size_t)slot_owner_[s]->w.nv;
            batch_voxels_ = vox_total;
            const size_t vb = (size_t)std::max(1, n_vox_items_) * dev::kOrderKeysBins;
            if (vb > cap_vbins_ || !d_vox_total_) {
                cudaFree(d_vox_hist_); cudaFree(d_vox_base_);
                d_vox_hist_ = d_vox_base_ = nullptr;
                cap_vbins_ = std::max(vb, 2 * cap_vbins_);
                CK(cudaMalloc(&d_vox_hist_, sizeof(int) * cap_vbins_));
                CK(cudaMalloc(&d_vox_base_, sizeof(int) * cap_vbins_));
                if (!d_vox_total_) {
                    CK(cudaMalloc(&d_vox_total_, sizeof(int)));
                    CK(cudaMemsetAsync(d_vox_total_, 0, sizeof(int), stream_));
                }
            }
            if (std::max<size_t>(1, vox_total) > cap_vperm_) {
                cudaFree(d_vox_perm_);
                d_vox_perm_ = nullptr;
                cap_vperm_ = std::max(std::max<size_t>(1, vox_total), 2 * cap_vperm_);
                CK(cudaMalloc(&d_vox_perm_, sizeof(int2) * cap_vperm_));
            }
            n_batch_ = (int)slots.size();
            if (n_batch_ > cap_batch_) {
                cudaFree(d_batch_slots_);
                cudaFree(d_batch_items_);
                d_batch_items_ = nullptr;
                cap_batch_ = std::max(n_batch_, 2 * cap_batch_);
                CK(cudaMalloc(&d_batch_slots_, sizeof(int) * cap_batch_));
                CK(cudaMalloc(&d_batch_items_, sizeof(int4) * cap_batch_));
            }
            batch_slots_host_ = slots;   // kept alive for the asynchronous copies
            batch_items_host_.resize(slots.size());
            for (size_t i = 0; i < slots.size(); i++)
                batch_items_host_[i] = make_int4(ctl_items[i].second, ctl_items[i].first, contact_items[i].first, contact_items[i].second);
            if (n_batch_) {
                CK(copy_async(d_batch_slots_, batch_slots_host_.data(), sizeof(int) * n_batch_, cudaMemcpyHostToDevice, stream_));
                CK(copy_async(d_batch_items_, batch_items_host_.data(), sizeof(int4) * n_batch_, cudaMemcpyHostToDevice, stream_));
                k_set_batch_items<<<(n_batch_ + 255) / 256, 256, 0, stream_>>>(d_ctl_, d_batch_slots_, d_batch_items_, n_batch_);
                CK(cudaGetLastError());
            }
        }
        if ((int)items.size() > cap_items_) {
            cudaFree(d_items_);
            cudaFree(d_stale_items_);
            d_stale_items_ = nullptr;
            cap_items_ = std::max((int)items.size(), 2 * cap_items_);
            CK(cudaMalloc(&d_items_, sizeof(dev::Item) * cap_items_));
            CK(cudaMalloc(&d_stale_items_, sizeof(int) * cap_items_));
        }
        if (!items.empty()) CK(copy_async(d_items_, items.data(), sizeof(dev::Item) * items.size(), cudaMemcpyHostToDevice, stream_));
        n_attach_ = (int)attach_slots.size();
        if (n_attach_ > cap_attach_) {
            cudaFree(d_attach_slots_);
            cap_attach_ = std::max(n_attach_, 2 * cap_attach_);
            CK(cudaMalloc(&d_attach_slots_, sizeof(int) * cap_attach_));
        }
        if (n_attach_) {
            attach_slots_host_ = attach_slots;   // kept alive for the asynchronous copy
            CK(copy_async(d_attach_slots_, attach_slots_host_.data(), sizeof(int) * n_attach_, cudaMemcpyHostToDevice, stream_));
        }
        CK(cudaMemsetAsync(d_tickets_, 0, kTickets * sizeof(int), stream_));
        if (any_watch_ && n_contact_items_ > 0) {
            k_list_all_items<<<(n_contact_items_ + 255) / 256, 256, 0, stream_>>>(d_stale_items_, n_contact_items_, d_tickets_);
            CK(cudaGetLastError());
        }
        return 0;
    }

    int grid_for(int n_items, int block) const {
        int per_sm = block >= 256 ? 4 : 8;
        return std::max(1, std::min(n_items, sm_count_ * per_sm));
    }

    // One step of the batch; returns the number of kernels it launched.
    int launch_step(cudaStream_t st, bool prof) {
        int launched = 3 + (any_collide_ ? 1 : 0) + (any_watch_ ? 3 : 0) + (any_signals_ ? 1 : 0) + (n_attach_ ? 1 : 0);
        const dev::Item* li = d_items_;
        const dev::Item* ci = d_items_ + n_link_items_;
        const dev::Item* vi = d_items_ + n_link_items_ + n_contact_items_;
        const bool regroup = bins_dirty_ || (batch_links_ >= kRegroupEveryStepLinks && bin_phase_ % bin_every_ == 0);
        if (regroup) {
            // links and voxels grouped together (the voxel keys come from the last voxel
            // update, so nothing of this step changes them); windows of about 16k elements keep
            // a window's state in L2 while its key groups run
            dev::BinList lb{li, n_link_items_, 0, std::max(1, 16384 / std::max(1, items_links_)), 0, d_link_hist_, d_link_base_,
                            d_link_total_, d_link_perm_};
            dev::BinList vb{vi, n_vox_items_, 1, std::max(1, 16384 / std::max(1, items_voxels_)), 0, d_vox_hist_, d_vox_base_,
                            d_vox_total_, d_vox_perm_};
            ks_.bins(std::max(1, std::min(n_link_items_ + n_vox_items_, 4 * sm_count_)), st, d_sims_, d_ctl_, lb, vb);
            bins_dirty_ = false;
            bin_phase_ = 0;
            launched += 3;
        }
        bin_phase_++;
        if (prof) cudaEventRecord(evk_[0], st);
        // persistent grids, but no more blocks than the batch has block-sized pieces: every warp
        // of a block claims at least one chunk, and idle claims cost atomics in small batches
        const int bl = std::min(block_links_, ks_.max_block), bv = std::min(block_voxels_, ks_.max_block);
        auto grid_chunks = [&](size_t elems, int block, int which) {
            const size_t full = (size_t)sm_count_ * ks_.resident_blocks(which, block);
            return (int)std::max<size_t>(1, std::min(full, (elems + block - 1) / block));
        };
        ks_.links(grid_chunks(batch_links_, bl, 0), bl, st, d_sims_, d_ctl_, d_link_perm_, d_link_total_,
                  (int)cap_perm_, cap_slots_, d_tickets_, claim_links_);
        if (prof) cudaEventRecord(evk_[1], st);
        // the watch-list passes: a persistent grid of 256-thread blocks over the listed items' work units
        if (any_watch_) ks_.watch(4 * sm_count_, st, d_sims_, d_ctl_, ci, n_contact_items_, d_stale_items_, d_tickets_, d_batch_slots_,
                                  n_batch_);
        if (any_collide_) ks_.contacts(grid_for(n_contact_items_, 128), 128, st, d_sims_, d_ctl_, ci, n_contact_items_, d_tickets_);
        if (n_attach_) ks_.attach(st, d_sims_, d_ctl_, d_attach_slots_, n_attach_);
        if (prof) cudaEventRecord(evk_[2], st);
        if (prof) cudaEventRecord(evk_[3], st);
        ks_.voxels(grid_chunks(batch_voxels_, bv, 1), bv, st, d_sims_, d_ctl_, d_vox_perm_, d_vox_total_,
                   (int)cap_vperm_, cap_slots_, d_tickets_, claim_voxels_);
        if (prof) cudaEventRecord(evk_[4], st);
        ks_.sim_end(st, d_sims_, d_ctl_, d_batch_slots_, n_batch_, d_tickets_, d_stale_items_);
        if (any_signals_) ks_.signals(grid_for(n_vox_items_, 256), 256, st, d_sims_, d_ctl_, vi, n_vox_items_, d_tickets_);
        return launched;
    }

    // Marks the slots running towards their target step counts (no_stop: vx3_step's fixed
    // count, the stop formula is not applied), one copy of the lists and one kernel.
    int set_running(const std::vector<int>& slots, const std::vector<int64_t>& targets, std::string* err, int no_stop = 0) {
        if (slots.empty()) return 0;
        bins_dirty_ = true;   // simulations (re)started: the next step regroups with them
        const size_t n = slots.size(), o_tg = ((4 * n + 15) & ~(size_t)15), total = o_tg + 8 * n;
        if (int e = pinned(&rb_, total, err)) return e;
        if (total > cap_gather_) {
            CK(cudaStreamSynchronize(stream_));
            cudaFree(d_gather_);
            d_gather_ = nullptr;
            cap_gather_ = 0;
            CK(cudaMalloc(&d_gather_, total));
            cap_gather_ = total;
        }
        memcpy(rb_.p, slots.data(), 4 * n);
        memcpy(rb_.p + o_tg, targets.data(), 8 * n);
        CK(copy_async(d_gather_, rb_.p, total, cudaMemcpyHostToDevice, stream_));
        CK(cudaEventRecord(rb_.done, stream_));
        k_ctl_run<<<(unsigned)((n + 255) / 256), 256, 0, stream_>>>(d_ctl_, (const int*)d_gather_, (const int64_t*)(d_gather_ + o_tg),
                                                                   (int)n, no_stop);
        CK(cudaGetLastError());
        // a simulation that stopped at the end of its last step (target reached) was not listed
        // for its watch-list regeneration by k_sim_end: list every contact item again (a batch
        // about to change is listed afresh by build_items)
        if (any_watch_ && n_contact_items_ > 0 && n_contact_items_ <= cap_items_) {
            k_list_all_items<<<(n_contact_items_ + 255) / 256, 256, 0, stream_>>>(d_stale_items_, n_contact_items_, d_tickets_);
            CK(cudaGetLastError());
        }
        return 0;
    }

    // After a vx3_step call: the stop formula applies again and DONE (target reached) is IDLE.
    int end_fixed_steps(const std::vector<int>& slots, std::string* err) {
        if (slots.empty()) return 0;
        const size_t n = slots.size();
        if (int e = pinned(&rb_, 4 * n, err)) return e;
        if (4 * n > cap_gather_) {
            CK(cudaStreamSynchronize(stream_));
            cudaFree(d_gather_);
            d_gather_ = nullptr;
            cap_gather_ = 0;
            CK(cudaMalloc(&d_gather_, 4 * n));
            cap_gather_ = 4 * n;
        }
        memcpy(rb_.p, slots.data(), 4 * n);
        CK(copy_async(d_gather_, rb_.p, 4 * n, cudaMemcpyHostToDevice, stream_));
        CK(cudaEventRecord(rb_.done, stream_));
        k_ctl_end_steps<<<(unsigned)((n + 255) / 256), 256, 0, stream_>>>(d_ctl_, (const int*)d_gather_, (int)n);
        CK(cudaGetLastError());
        return 0;
    }

    int read_ctl(int slot, dev::Ctl* c, std::string* err) {
        CK(copy_async(c, d_ctl_ + slot, offsetof(dev::Ctl, stop), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        return 0;
    }

    // The scalar part of the control blocks of the slots lo..hi (one strided copy, one
    // synchronisation); out[s - lo] holds slot s.
    int read_ctls(int lo, int hi, std::vector<dev::Ctl>* out, std::string* err) {
        out->resize((size_t)(hi - lo + 1));
        CK(copy2d_async(out->data(), sizeof(dev::Ctl), d_ctl_ + lo, sizeof(dev::Ctl), offsetof(dev::Ctl, stop),
                             (size_t)(hi - lo + 1), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        return 0;
    }

    // Runs until every listed simulation has left the RUNNING state.
    int drive(const std::vector<SimRec*>& rs, int mode, std::string* err) {
        int64_t vsteps_before = 0;
        std::vector<int64_t> steps0(rs.size());
        int slo = INT32_MAX, shi = -1;
        for (auto* r : rs) { slo = std::min(slo, r->slot); shi = std::max(shi, r->slot); }
        std::vector<dev::Ctl> cs;
        if (!rs.empty()) {
            if (int e = read_ctls(slo, shi, &cs, err)) return e;
            for (size_t i = 0; i < rs.size(); i++) steps0[i] = cs[(size_t)(rs[i]->slot - slo)].steps;
        }
        timing_.launches = 0;
        double w0 = now_s();
        CK(cudaEventRecord(ev0_, stream_));
        if (mode == MODE_PLAIN) {
            for (size_t i = 0; i < rs.size(); i++) {
                std::vector<int> one{rs[i]->slot};
                if (int e = build_items(one, err)) return e;
                if (exact_steps_ >= 0) {
                    for (int64_t k = 0; k < exact_steps_; k++) { timing_.launches += launch_step(stream_, false); }
                    continue;
                }
                for (;;) {
                    for (int k = 0; k < 16; k++) { timing_.launches += launch_step(stream_, false); }
                    dev::Ctl c;
                    if (int e = read_ctl(rs[i]->slot, &c, err)) return e;
                    if (c.status != SIM_RUNNING) break;
                }
            }
            batch_dirty_ = true;
        } else {
            std::vector<int> slots;
            for (auto* r : rs) slots.push_back(r->slot);
            TraceClock tc;
            if (batch_dirty_ || slots != batch_slots_) {
                if (int e = build_items(slots, err)) return e;
                batch_slots_ = slots;
                if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
                batch_dirty_ = false;
                tc.mark("drive: build_items");
            }
            // a graph is captured only when a whole one will run: fewer steps than a graph holds
            // go out as single launches (a capture the GPU waits for would cost more)
            const bool use_graph = exact_steps_ < 0 ? !profiling_ : (!profiling_ && exact_steps_ >= graph_steps_);
            if (!graph_ && use_graph) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
                bins_dirty_ = true;   // every replay starts by regrouping the links
                graph_launches_ = 0;
                for (int k = 0; k < graph_steps_; k++) graph_launches_ += launch_step(stream_, false);
                CK(cudaStreamEndCapture(stream_, &g));
                bins_dirty_ = true;   // captured kernels have not run: the next eager step regroups
                tc.mark("drive: graph capture");
                CK(cudaGraphInstantiate(&graph_, g, 0));
                cudaGraphDestroy(g);
                graph_len_ = graph_steps_;
                tc.mark("drive: graph instantiate");
            }
            if (exact_steps_ >= 0) {
                // a known step count: whole graphs, then single steps for the remainder, no polling
                int64_t left = exact_steps_;
                while (left > 0) {
                    if (graph_ && !profiling_ && left >= graph_len_) {
                        CK(cudaGraphLaunch(graph_, stream_));
                        timing_.launches += graph_launches_;
                        left -= graph_len_;
                    } else {
                        timing_.launches += launch_step(stream_, profiling_ != 0);
                        left -= 1;
                    }
                }
            } else {
                int lo = INT32_MAX, hi = -1;
                for (auto* r : rs) { lo = std::min(lo, r->slot); hi = std::max(hi, r->slot); }
                std::vector<int32_t> st((size_t)(hi - lo + 1));
                for (;;) {
                    if (profiling_) {
                        timing_.launches += launch_step(stream_, true);
                    } else {
                        CK(cudaGraphLaunch(graph_, stream_));
                        timing_.launches += graph_launches_;
                    }
                    // one strided copy of every status word, then a single synchronisation
                    CK(copy2d_async(st.data(), sizeof(int32_t), &d_ctl_[lo].status, sizeof(dev::Ctl), sizeof(int32_t),
                                         (size_t)(hi - lo + 1), cudaMemcpyDeviceToHost, stream_));
                    CK(cudaStreamSynchronize(stream_));
                    bool running = false;
                    for (auto* r : rs) if (st[(size_t)(r->slot - lo)] == SIM_RUNNING) { running = true; break; }
                    if (!running) break;
                }
            }
        }
        CK(cudaEventRecord(ev1_, stream_));
        CK(cudaEventSynchronize(ev1_));
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0_, ev1_);
        timing_.device_ms = ms;
        timing_.wall_ms = (now_s() - w0) * 1e3;
        if (profiling_) {
            float a = 0, b = 0, c = 0;
            cudaEventElapsedTime(&a, evk_[0], evk_[1]);   // k_links
            cudaEventElapsedTime(&b, evk_[1], evk_[2]);   // k_contacts (and k_attach)
            cudaEventElapsedTime(&c, evk_[3], evk_[4]);   // k_voxels
            timing_.link_kernel_ms = a; timing_.contact_kernel_ms = b; timing_.voxel_kernel_ms = c;
        }
        if (!rs.empty()) {
            if (int e = read_ctls(slo, shi, &cs, err)) return e;
            for (size_t i = 0; i < rs.size(); i++) {
                const dev::Ctl& c = cs[(size_t)(rs[i]->slot - slo)];
                rs[i]->status = c.status;
                vsteps_before += (c.steps - steps0[i]) * rs[i]->w.nv;
            }
        }
        timing_.voxel_steps = vsteps_before;
        return 0;
    }

    int prepare(const int64_t* ids, int n, std::vector<SimRec*>* rs, std::string* err) {
        std::vector<SimRec*> fresh, begun;
        std::unordered_set<SimRec*> seen;
        for (int i = 0; i < n; i++) {
            SimRec* r = find(ids[i]);
            if (!r) { *err = "unknown simulation id"; return -6; }
            if (!r->resident && seen.insert(r).second) fresh.push_back(r);
            rs->push_back(r);
        }
        TraceClock tc;
        int e_many = upload_many(fresh, &begun, err);
        tc.mark("prepare: upload_many");
        if (int e = e_many) {
            std::string e2;
            upload_finish(begun, &e2);
            return e;
        }
        const int ef = upload_finish(begun, err);
        tc.mark("prepare: upload_finish");
        return ef;
    }

    // GVX_TRACE=1: host time of the phases of each call on stderr
    static bool trace_on() {
        static const bool on = [] { const char* v = std::getenv("GVX_TRACE"); return v && *v && *v != '0'; }();
        return on;
    }
    struct TraceClock {
        double t = now_s();
        void mark(const char* what) {
            if (!trace_on()) return;
            const double u = now_s();
            std::fprintf(stderr, "[gvx] %-28s %8.3f ms\n", what, 1e3 * (u - t));
            t = u;
        }
    };

    int step(const int64_t* ids, int n, int mode, int64_t steps, std::string* err) override {
        std::vector<SimRec*> rs;
        TraceClock tc;
        if (int e = prepare(ids, n, &rs, err)) return e;
        tc.mark("step: prepare (uploads)");
        std::vector<int> slots;
        std::vector<int64_t> targets;
        std::vector<SimRec*> act;
        if (rs.empty()) return 0;
        int lo = INT32_MAX, hi = -1;
        for (auto* r : rs) { lo = std::min(lo, r->slot); hi = std::max(hi, r->slot); }
        std::vector<dev::Ctl> cs;
        if (int e = read_ctls(lo, hi, &cs, err)) return e;
        for (auto* r : rs) {
            const dev::Ctl& c = cs[(size_t)(r->slot - lo)];
            if (c.status == SIM_DIVERGED || c.status == SIM_ERROR) continue;
            slots.push_back(r->slot);
            targets.push_back(c.steps + steps);
            act.push_back(r);
        }
        if (slots.empty()) return 0;
        // the stop formula is not applied by step() (no_stop), and reaching the target leaves the
        // simulation IDLE for the next call
        if (int e = set_running(slots, targets, err, 1)) return e;
        tc.mark("step: read/set control");
        exact_steps_ = steps;
        int e = drive(act, mode, err);
        tc.mark("step: drive");
        exact_steps_ = -1;
        if (int e2 = end_fixed_steps(slots, err)) return e2;
        if (int e2 = read_ctls(lo, hi, &cs, err)) return e2;
        for (auto* r : act) r->status = cs[(size_t)(r->slot - lo)].status;
        tc.mark("step: end");
        return e;
    }

    int run(const int64_t* ids, int n, int mode, int64_t max_steps, std::string* err) override {
        std::vector<SimRec*> rs;
        if (int e = prepare(ids, n, &rs, err)) return e;
        std::vector<int> slots;
        std::vector<int64_t> targets;
        std::vector<SimRec*> act;
        if (rs.empty()) return 0;
        int lo = INT32_MAX, hi = -1;
        for (auto* r : rs) { lo = std::min(lo, r->slot); hi = std::max(hi, r->slot); }
        std::vector<dev::Ctl> cs;
        if (int e = read_ctls(lo, hi, &cs, err)) return e;
        for (auto* r : rs) {
            const dev::Ctl& c = cs[(size_t)(r->slot - lo)];
            if (c.status != SIM_IDLE) continue;
            // StopConditionMet is checked before each step (VX3_SimulationManager.cu:62-64)
            if (r->w.desc.stop_formula.n > 0) {
                MathVars mv{c.com[0], c.com[1], c.com[2], 0, c.t, c.recent_angle, 0, 0, r->w.nv};
                if (mathtree_eval(r->w.desc.stop_formula, mv) > 0) { finish(r, SIM_DONE, err); continue; }
            }
            int64_t cap = max_steps > 0 ? max_steps : 1000000;   // VX3 maximum step count
            slots.push_back(r->slot);
            targets.push_back(c.steps + cap);
            act.push_back(r);
        }
        if (act.empty()) return 0;
        if (int e = set_running(slots, targets, err)) return e;
        int e = drive(act, mode, err);
        if (e) return e;
        for (auto* r : act) finish(r, r->status, err);
        return 0;
    }

    int com(SimRec* r, double* out, std::string* err) {
        ks_.com(stream_, d_sims_, r->slot, d_com4_);
        CK(cudaGetLastError());
        double c4[4];
        CK(copy_async(c4, d_com4_, sizeof(c4), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        if (c4[3] == 0) out[0] = out[1] = out[2] = 0;
        else for (int k = 0; k < 3; k++) out[k] = c4[k] / c4[3];
        return 0;
    }

    // Final centre of mass and fitness (VX3_SimulationManager.cu:116-117, VX3_VoxelyzeKernel.cu:530-534)
    int finish(SimRec* r, int status, std::string* err) {
        dev::Ctl c;
        if (int e = read_ctl(r->slot, &c, err)) return e;
        SimResult& R = r->result;
        R = SimResult{};
        R.id = r->id;
        R.status = status == SIM_RUNNING ? SIM_DONE : status;
        R.num_voxel = r->w.nv;
        R.num_measured_voxel = r->num_measured;
        R.steps = c.steps;
        R.current_time = c.t;
        R.vox_size = r->w.desc.vox_size;
        // initial centre of mass: the host's, or the one the secondary experiment reset it to
        for (int k = 0; k < 3; k++) R.initial_com[k] = c.reinit_done ? c.init_com[k] : r->init_com[k];
        if (int e = com(r, R.current_com, err)) return e;
        R.num_close_pairs = c.num_close_pairs;
        MathVars mv{R.current_com[0] - R.initial_com[0], R.current_com[1] - R.initial_com[1], R.current_com[2] - R.initial_com[2],
                    (double)c.hit_count, c.t, c.recent_angle, c.closeness, c.num_close_pairs, r->w.nv};
        R.fitness = mathtree_eval(r->w.desc.fitness, mv);
        // total distance travelled by measured voxels from their initial positions
        // (VX3_SimulationManager.cu:442-452)
        const size_t nv = r->w.nv;
        std::vector<double> p(3 * nv), ip;
        CK(copy_async(p.data(), r->dsim.px, 8 * nv, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(p.data() + nv, r->dsim.py, 8 * nv, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(p.data() + 2 * nv, r->dsim.pz, 8 * nv, cudaMemcpyDeviceToHost, stream_));
        if (c.reinit_done) {
            ip.resize(3 * nv);
            CK(copy_async(ip.data(), r->dsim.init_pos, 8 * 3 * nv, cudaMemcpyDeviceToHost, stream_));
        }
        CK(cudaStreamSynchronize(stream_));
        double tot = 0;
        for (size_t i = 0; i < nv; i++) {
            if (!r->w.vmats[r->w.desc.voxels[4 * i + 3]].is_measured) continue;
            double nom = r->w.vmats[r->w.desc.voxels[4 * i + 3]].nom;
            const double ix = ip.empty() ? r->w.desc.voxels[4 * i] * nom : ip[i];
            const double iy = ip.empty() ? r->w.desc.voxels[4 * i + 1] * nom : ip[nv + i];
            const double iz = ip.empty() ? r->w.desc.voxels[4 * i + 2] * nom : ip[2 * nv + i];
            double dx = p[i] - ix, dy = p[nv + i] - iy, dz = p[2 * nv + i] - iz;
            tot += sqrt(dx * dx + dy * dy + dz * dz);
        }
        R.total_distance = tot;
        if (r->w.desc.save_all_positions) {   // kept for the report's pos and init_pos fields
            r->final_pos = std::move(p);
            r->final_init_pos = std::move(ip);
        }
        R.submit_s = r->submit_s;
        R.start_s = r->start_s;
        r->finish_s = now_s() - t0_;
        R.finish_s = r->finish_s;
        r->status = R.status;
        r->retired = true;
        return 0;
    }

    // ---------------------------------------------------------------- serving
    int submit(int64_t id, int64_t horizon, std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        r->horizon = horizon;
        r->submit_s = now_s() - t0_;
        queue_.push_back(id);
        return 0;
    }
    int pending() const override { return (int)(queue_.size() + active_.size()); }

    // Serving policy: the order queued requests are admitted in (first come first served; the
    // least work — voxels x horizon steps — first; or the least work first beside one lane for
    // the most work queued) and the voxels the running batch may hold (0: as many as the HBM
    // budget allows; the first request is always admitted; the lane's request is not counted).
    int serve_order_ = 0;
    int64_t serve_max_voxels_ = 0;
    int64_t lane_id_ = -1;   // the request running in the lane of order 2, or -1
    int set_serving(int order, int64_t max_active_voxels) override {
        if (order < 0 || order > 2 || max_active_voxels < 0) return -6;
        serve_order_ = order;
        serve_max_voxels_ = max_active_voxels;
        return 0;
    }
    double serve_work(int64_t id) {
        SimRec* a = find(id);
        return a ? (double)a->w.nv * (double)(a->horizon > 0 ? a->horizon : 1000000) : 0;
    }

    int poll(SimResult* out, int max, int chunk, std::string* err) override {
        // admit while the HBM budget (and the voxel cap) allows, in the policy's order; the
        // uploads of everything admitted now are finished together
        std::vector<SimRec*> begun, admitted;
        if (serve_order_ != 2 || (lane_id_ >= 0 && std::find(active_.begin(), active_.end(), lane_id_) == active_.end()))
            lane_id_ = -1;
        int64_t active_voxels = 0;   // of the running batch, the lane's request left out
        for (int64_t id : active_)
            if (SimRec* a = find(id)) active_voxels += id == lane_id_ ? 0 : a->w.nv;
        bool lane_first = false;
        if (serve_order_ >= 1 && queue_.size() > 1) {
            // least work first; ties keep their arrival order
            std::stable_sort(queue_.begin(), queue_.end(), [&](int64_t x, int64_t y) { return serve_work(x) < serve_work(y); });
        }
        if (serve_order_ == 2 && lane_id_ < 0 && !queue_.empty()) {
            // the lane is free: the request with the most work goes first, so that the longest
            // runs overlap the short ones instead of running alone at the end
            const int64_t big = queue_.back();
            queue_.pop_back();
            queue_.push_front(big);
            lane_first = true;
        }
        while (!queue_.empty()) {
            SimRec* r = find(queue_.front());
            if (!r) { queue_.pop_front(); lane_first = false; continue; }
            const bool in_lane = lane_first && admitted.empty();
            if (!in_lane && serve_max_voxels_ > 0 && !(active_.empty() && admitted.empty()) &&
                active_voxels + r->w.nv > serve_max_voxels_)
                break;
            std::string e2;
            const bool fresh = !r->resident;
            int e = fresh ? upload_begin(r, &e2) : 0;
            if (e == -2) {
                if (active_.empty() && admitted.empty()) { *err = "simulation larger than the HBM budget"; return -2; }
                break;
            }
            if (e) { upload_finish(begun, err); *err = e2; return e; }
            if (fresh) begun.push_back(r);
            admitted.push_back(r);
            if (in_lane) lane_id_ = r->id;
            else active_voxels += r->w.nv;
            queue_.pop_front();
            r->start_s = now_s() - t0_;
            active_.push_back(r->id);
        }
        if (int e = upload_finish(begun, err)) return e;
        if (!admitted.empty()) {
            std::vector<int> slots;
            std::vector<int64_t> tg;
            for (SimRec* r : admitted) {
                slots.push_back(r->slot);
                tg.push_back(r->horizon > 0 ? r->horizon : 1000000);
            }
            if (int e3 = set_running(slots, tg, err)) return e3;
            batch_dirty_ = true;
        }
        if (active_.empty()) return 0;
        std::vector<int> slots;
        for (int64_t id : active_) slots.push_back(find(id)->slot);
        if (batch_dirty_ || slots != batch_slots_) {
            if (int e = build_items(slots, err)) return e;
            batch_slots_ = slots;
            if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
            batch_dirty_ = false;
        }
        int k = std::max(1, chunk);
        if (!graph_ || graph_len_ != k) {
            if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
            bins_dirty_ = true;
            graph_launches_ = 0;
            for (int s = 0; s < k; s++) graph_launches_ += launch_step(stream_, false);
            CK(cudaStreamEndCapture(stream_, &g));
            bins_dirty_ = true;   // captured kernels have not run: the next eager step regroups
            CK(cudaGraphInstantiate(&graph_, g, 0));
            cudaGraphDestroy(g);
            graph_len_ = k;
        }
        CK(cudaGraphLaunch(graph_, stream_));
        timing_.launches += graph_launches_;
        std::vector<int32_t> st(active_.size());
        {
            int lo = INT32_MAX, hi = -1;
            for (int s : slots) { lo = std::min(lo, s); hi = std::max(hi, s); }
            std::vector<dev::Ctl> cs;
            if (int e = read_ctls(lo, hi, &cs, err)) return e;
            for (size_t i = 0; i < active_.size(); i++) st[i] = cs[(size_t)(slots[i] - lo)].status;
        }
        int nout = 0;
        std::vector<int64_t> still;
        for (size_t i = 0; i < active_.size(); i++) {
            SimRec* r = find(active_[i]);
            if (st[i] == SIM_RUNNING) { still.push_back(active_[i]); continue; }
            if (int e = finish(r, st[i], err)) return e;
            if (nout < max) out[nout++] = r->result;
            release(r);
        }
        active_ = still;
        return nout;
    }

    int result(int64_t id, SimResult* out, std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        if (!r->retired) {
            if (!r->resident) { *err = "simulation has not run"; return -7; }
            if (int e = finish(r, r->status, err)) return e;
            r->retired = false;
        }
        *out = r->result;
        return 0;
    }

    int info(int64_t id, int* nv, int* nl, double* dt, double* t, int64_t* steps, int* status) override {
        SimRec* r = find(id);
        if (!r) return -6;
        *nv = r->w.nv; *nl = r->w.nl;
        *dt = r->dt; *t = 0; *steps = 0; *status = r->status;
        if (r->resident) {
            dev::Ctl c;
            std::string e;
            if (read_ctl(r->slot, &c, &e)) return -5;
            *t = c.t; *steps = c.steps; *status = c.status; *dt = c.dt;
        }
        return 0;
    }

    int voxel_state(int64_t id, double* d13, float* f4, int32_t* flags, std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        if (!r->resident) if (int e = upload(r, err)) return e;
        const int nv = r->w.nv;
        std::vector<double> buf(13 * (size_t)nv);
        double* srcs[13] = {r->dsim.px, r->dsim.py, r->dsim.pz, r->dsim.mx, r->dsim.my, r->dsim.mz, r->dsim.qw, r->dsim.qx,
                            r->dsim.qy, r->dsim.qz, r->dsim.ax, r->dsim.ay, r->dsim.az};
        for (int k = 0; k < 13; k++) CK(copy_async(buf.data() + (size_t)k * nv, srcs[k], 8 * nv, cudaMemcpyDeviceToHost, stream_));
        std::vector<float> tb((size_t)nv), ps(3 * (size_t)nv);
        std::vector<uint32_t> fl((size_t)nv);
        CK(copy_async(tb.data(), r->dsim.temp, 4 * nv, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(ps.data(), r->dsim.ps, 12 * nv, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(fl.data(), r->dsim.vfl, 4 * nv, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (int i = 0; i < nv; i++) {
            if (d13) for (int k = 0; k < 13; k++) d13[13 * (size_t)i + k] = buf[(size_t)k * nv + i];
            if (f4) { f4[4 * (size_t)i] = tb[i]; for (int k = 0; k < 3; k++) f4[4 * (size_t)i + 1 + k] = ps[(size_t)k * nv + i]; }
            if (flags) flags[i] = (int32_t)fl[i];
        }
        return 0;
    }

    int links(int64_t id, int32_t* n_links, int32_t* ends4, int max, std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        if (!r->resident) if (int e = upload(r, err)) return e;
        dev::Ctl c;
        if (int e = read_ctl(r->slot, &c, err)) return e;
        *n_links = c.n_links;
        const int n = std::min(c.n_links, max);
        if (n <= 0 || !ends4) return 0;
        std::vector<int32_t> ln((size_t)n), lp((size_t)n);
        std::vector<uint8_t> la((size_t)n), lf((size_t)n);
        CK(copy_async(ln.data(), r->dsim.lneg, 4 * (size_t)n, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(lp.data(), r->dsim.lpos, 4 * (size_t)n, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(la.data(), r->dsim.lax, (size_t)n, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(lf.data(), r->dsim.lfl, (size_t)n, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (int i = 0; i < n; i++) {
            ends4[4 * i] = ln[i]; ends4[4 * i + 1] = lp[i]; ends4[4 * i + 2] = la[i]; ends4[4 * i + 3] = lf[i];
        }
        return 0;
    }

    int extras(int64_t id, double* measures4, double* sig6, std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        if (!r->resident) if (int e = upload(r, err)) return e;
        const size_t nv = r->w.nv;
        dev::Ctl c;
        if (int e = read_ctl(r->slot, &c, err)) return e;
        if (measures4) {
            measures4[0] = c.closeness; measures4[1] = c.num_close_pairs; measures4[2] = c.hit_count; measures4[3] = c.recent_angle;
        }
        if (sig6) {
            if (!r->dsim.sig) { std::fill(sig6, sig6 + 6 * nv, 0.0); return 0; }
            std::vector<double> g(6 * nv);
            CK(copy_async(g.data(), r->dsim.sig, 8 * 6 * nv, cudaMemcpyDeviceToHost, stream_));
            CK(cudaStreamSynchronize(stream_));
            for (size_t i = 0; i < nv; i++)
                for (int k = 0; k < 6; k++) sig6[6 * i + k] = g[(size_t)k * nv + i];
        }
        return 0;
    }

    int link_state(int64_t id, double* d9, float* f3, int32_t* flags, std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        if (!r->resident) if (int e = upload(r, err)) return e;
        const int nl = r->w.nl;                 // the loaded links (links made at run time follow them)
        const size_t stride = r->dsim.nl;       // link capacity: the blocks' stride
        if (nl == 0) return 0;
        std::vector<double> st(9 * stride);
        std::vector<float> sf(3 * stride);
        std::vector<uint8_t> fl((size_t)nl);
        CK(copy_async(st.data(), r->dsim.lst, 72 * stride, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(sf.data(), r->dsim.lsf, 12 * stride, cudaMemcpyDeviceToHost, stream_));
        CK(copy_async(fl.data(), r->dsim.lfl, nl, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (int i = 0; i < nl; i++) {
            if (d9) for (int k = 0; k < 9; k++) d9[9 * (size_t)i + k] = st[(size_t)k * stride + i];
            if (f3) for (int k = 0; k < 3; k++) f3[3 * (size_t)i + k] = sf[(size_t)k * stride + i];
            if (flags) flags[i] = fl[i];
        }
        return 0;
    }

    int gather_states(const int64_t* ids, int n, double* pos3, double* q4, uint8_t* flags, std::string* err) override {
        std::vector<int> slots((size_t)n);
        std::vector<int64_t> offs((size_t)n);
        int64_t total = 0;
        for (int k = 0; k < n; k++) {
            SimRec* r = find(ids[k]);
            if (!r) { *err = "unknown simulation id"; return -6; }
            if (!r->resident) if (int e = upload(r, err)) return e;
            slots[k] = r->slot;
            offs[k] = total;
            total += r->w.nv;
        }
        if (total == 0) return 0;
        const size_t b_pos = 24 * (size_t)total, b_q = 32 * (size_t)total, b_fl = (size_t)total;
        const size_t b_idx = 4 * (size_t)n + 8 * (size_t)n;
        const size_t need = b_pos + b_q + b_fl + 16 + b_idx + 16;
        // the packing area: the context's scratch, or for large read-backs a temporary region
        // of the arena (given back below, after the copy has finished), else a larger scratch
        char* dg = d_gather_;
        size_t tmp_off = 0;
        bool tmp = false;
        if (need > cap_gather_) {
            if (arena_.alloc(need, &tmp_off)) {
                tmp = true;
                dg = arena_base_ + tmp_off;
            } else {
                CK(cudaStreamSynchronize(stream_));
                cudaFree(d_gather_);
                d_gather_ = nullptr;
                cap_gather_ = 0;
                CK(cudaMalloc(&d_gather_, need));
                cap_gather_ = need;
                dg = d_gather_;
            }
        }
        struct ArenaTemp {   // gives the temporary region back on every way out
            EngineImpl* e; bool on; size_t off, n;
            ~ArenaTemp() { if (on) { cudaStreamSynchronize(e->stream_); e->arena_.release(off, n); } }
        } arena_temp{this, tmp, tmp_off, need};
        if (int e = pinned(&rb_, b_idx, err)) return e;
        // the index tables go through the pinned buffer
        const size_t o_idx = (b_pos + b_q + b_fl + 15) & ~(size_t)15;
        char* h = rb_.p;
        memcpy(h, offs.data(), 8 * (size_t)n);
        memcpy(h + 8 * (size_t)n, slots.data(), 4 * (size_t)n);
        CK(copy_async(dg + o_idx, h, b_idx, cudaMemcpyHostToDevice, stream_));
        double* dpos = (double*)dg;
        double* dq = (double*)(dg + b_pos);
        uint8_t* dfl = (uint8_t*)(dg + b_pos + b_q);
        const int64_t* doff = (const int64_t*)(dg + o_idx);
        const int* dslot = (const int*)(dg + o_idx + 8 * (size_t)n);
        for (int k0 = 0; k0 < n; k0 += 65535)
            ks_.gather(stream_, d_sims_, dslot + k0, doff + k0, std::min(65535, n - k0), dpos, dq, dfl);
        CK(cudaGetLastError());
        const size_t b_all = b_pos + b_q + b_fl;
        if (b_all <= kPinnedUploadMax) {
            // one copy into the pinned generation buffer (grown if need be; pinned buffers are
            // cached across contexts), then host threads copy into the caller's arrays (and take
            // their first-touch faults): a copy straight into pageable memory took up to 38 ms
            TraceClock tg;
            if (int e = pinned(&gen_, b_all, err)) return e;   // waits for the buffer's last use
            tg.mark("gather: pinned buffer");
            char* hs = gen_.p;
            if (pos3 && q4 && flags) {
                CK(copy_async(hs, dpos, b_all, cudaMemcpyDeviceToHost, stream_));
            } else {
                if (pos3) CK(copy_async(hs, dpos, b_pos, cudaMemcpyDeviceToHost, stream_));
                if (q4) CK(copy_async(hs + b_pos, dq, b_q, cudaMemcpyDeviceToHost, stream_));
                if (flags) CK(copy_async(hs + b_pos + b_q, dfl, b_fl, cudaMemcpyDeviceToHost, stream_));
            }
            CK(cudaEventRecord(gen_.done, stream_));
            CK(cudaEventSynchronize(gen_.done));
            tg.mark("gather: kernel and copy");
            struct Piece { char* dst; const char* src; size_t n; };
            std::vector<Piece> pieces;
            auto cut = [&](void* dst, const char* src, size_t n) {
                if (!dst) return;
                for (size_t o = 0; o < n; o += kReadPiece)
                    pieces.push_back(Piece{(char*)dst + o, src + o, std::min(kReadPiece, n - o)});
            };
            cut(pos3, hs, b_pos);
            cut(q4, hs + b_pos, b_q);
            cut(flags, hs + b_pos + b_q, b_fl);
            std::atomic<size_t> next{0};
            auto work = [&]() {
                for (size_t i = next++; i < pieces.size(); i = next++) memcpy(pieces[i].dst, pieces[i].src, pieces[i].n);
            };
            const int nt = (int)std::max<size_t>(1, std::min<size_t>(pieces.size(), std::max(1u, std::thread::hardware_concurrency())));
            std::vector<std::thread> pool;
            for (int t = 1; t < nt; t++) pool.emplace_back(work);
            work();
            for (auto& t : pool) t.join();
            tg.mark("gather: host copies");
            return 0;
        }
        // straight into the caller's buffers: no pinned buffer grown to the size of a whole
        // generation just for this
        if (pos3) CK(copy_async(pos3, dpos, b_pos, cudaMemcpyDeviceToHost, stream_));
        if (q4) CK(copy_async(q4, dq, b_q, cudaMemcpyDeviceToHost, stream_));
        if (flags) CK(copy_async(flags, dfl, b_fl, cudaMemcpyDeviceToHost, stream_));
        CK(cudaEventRecord(rb_.done, stream_));
        CK(cudaEventSynchronize(rb_.done));
        return 0;
    }
    static constexpr size_t kReadPiece = 1u << 20;   // bytes per host copy task of a staged read-back

    const SimWorld* world(int64_t id) override {
        SimRec* r = find(id);
        return r ? &r->w : nullptr;
    }

    double optimal_dt(int64_t id) override {
        SimRec* r = find(id);
        return r ? (double)r->optdt : 0.0;
    }

    int saved_positions(int64_t id, int* save, std::vector<double>* init, std::vector<double>* cur, std::vector<int>* matid,
                        std::string* err) override {
        SimRec* r = find(id);
        if (!r) { *err = "unknown simulation id"; return -6; }
        *save = r->w.desc.save_all_positions;
        if (!*save) return 0;
        const int nv = r->w.nv;
        // positions at finish for retired simulations, else the current device state (x block, y block, z block)
        std::vector<double> p = r->final_pos;
        if (p.empty()) {
            if (!r->resident) if (int e = upload(r, err)) return e;
            p.resize(3 * (size_t)nv);
            CK(copy_async(p.data(), r->dsim.px, 8 * (size_t)nv, cudaMemcpyDeviceToHost, stream_));
            CK(copy_async(p.data() + nv, r->dsim.py, 8 * (size_t)nv, cudaMemcpyDeviceToHost, stream_));
            CK(copy_async(p.data() + 2 * (size_t)nv, r->dsim.pz, 8 * (size_t)nv, cudaMemcpyDeviceToHost, stream_));
            CK(cudaStreamSynchronize(stream_));
        }
        init->resize(3 * (size_t)nv);
        cur->resize(3 * (size_t)nv);
        matid->resize((size_t)nv);
        for (int i = 0; i < nv; i++) {
            const int mi = r->w.desc.voxels[4 * i + 3];
            const double nom = r->w.vmats[mi].nom;
            for (int k = 0; k < 3; k++) {
                (*init)[3 * (size_t)i + k] = r->final_init_pos.empty() ? r->w.desc.voxels[4 * i + k] * nom
                                                                       : r->final_init_pos[(size_t)k * nv + i];
                (*cur)[3 * (size_t)i + k] = p[(size_t)k * nv + i];
            }
            (*matid)[i] = mi + 1;   // palette index 0 is the empty material (VX_Object.cpp:149-158, 486)
        }
        return 0;
    }

    int free_sim(int64_t id) override {
        SimRec* r = find(id);
        if (!r) return -6;
        for (auto it = queue_.begin(); it != queue_.end(); ++it) if (*it == id) { queue_.erase(it); break; }
        for (auto it = active_.begin(); it != active_.end(); ++it) if (*it == id) { active_.erase(it); break; }
        release(r);
        sims_.erase(id);
        return 0;
    }

    const Timing& timing() const override { return timing_; }
    void set_profiling(int on) override { profiling_ = on; }
    size_t bytes_in_use() const override { return arena_.used; }
    int device_check(std::string* err) override {
        CK(cudaStreamSynchronize(stream_));
        CK(cudaGetLastError());
        return 0;
    }
    int set_tuning(int bl, int bv, int il, int iv, int gs) override {
        if (bl > 0) block_links_ = std::min(256, std::max(32, bl & ~31));   // whole warps (the link ordering uses ballots)
        if (bv > 0) block_voxels_ = std::min(256, std::max(32, bv & ~31));
        if (il > 0) items_links_ = il;
        if (iv > 0) items_voxels_ = iv;
        if (gs > 0) graph_steps_ = gs;
        batch_dirty_ = true;
        return 0;
    }
    int set_claims(int cl, int cv) override {
        if (cl > 0) claim_links_ = std::min(1024, std::max(32, cl & ~31));   // whole warps' worth
        if (cv > 0) claim_voxels_ = std::min(1024, std::max(32, cv & ~31));
        batch_dirty_ = true;
        return 0;
    }
    int set_contact_slots(int n) override {
        if (n < 1 || n > dev::kContactInline) return -6;
        contact_inline_ = n;
        return 0;
    }
    void get_tuning(int32_t* out8) const override {
        out8[0] = block_links_; out8[1] = block_voxels_; out8[2] = items_links_; out8[3] = items_voxels_;
        out8[4] = graph_steps_; out8[5] = claim_links_; out8[6] = claim_voxels_; out8[7] = contact_inline_;
    }
    // Project autotuner: a coordinate search over the launch shape on the live batch.  From
    // the current shape it tries, one axis at a time, threads per block (128, 256), elements
    // per link and per voxel work item (256, 512, 1024: the grouping window) and elements a
    // warp claims from the link and voxel queues at a time (32, 64, 128), keeping a value
    // when the median of three timed runs beats the best so far by more than 1%.  The
    // simulations' device regions and control blocks are copied aside first and put back
    // afterwards, so tuning leaves their state as it found it.
    struct TuneShape { int bl, bv, il, iv, cl, cv; };
    int autotune(const int64_t* ids, int n, std::string* err) override {
        std::vector<SimRec*> rs;
        if (int e = prepare(ids, n, &rs, err)) return e;
        std::vector<int> slots;
        for (auto* r : rs) slots.push_back(r->slot);
        if (slots.empty()) return 0;
        // copy the simulations' device regions aside (on the device when there is room)
        size_t total = 0;
        for (auto* r : rs) total += r->bytes;
        char* d_snap = nullptr;
        std::vector<std::vector<char>> snap;
        if (cudaMalloc(&d_snap, total) != cudaSuccess) {
            cudaGetLastError();   // the failed allocation is not an error of the engine
            d_snap = nullptr;
            snap.resize(rs.size());
        }
        std::vector<dev::Ctl> csnap(rs.size());
        size_t at = 0;
        for (size_t i = 0; i < rs.size(); i++) {
            if (d_snap) CK(copy_async(d_snap + at, arena_base_ + rs[i]->off, rs[i]->bytes, cudaMemcpyDeviceToDevice, stream_));
            else {
                snap[i].resize(rs[i]->bytes);
                CK(copy_async(snap[i].data(), arena_base_ + rs[i]->off, rs[i]->bytes, cudaMemcpyDeviceToHost, stream_));
            }
            at += rs[i]->bytes;
            CK(copy_async(&csnap[i], d_ctl_ + rs[i]->slot, sizeof(dev::Ctl), cudaMemcpyDeviceToHost, stream_));
        }
        CK(cudaStreamSynchronize(stream_));
        std::vector<int64_t> tg(slots.size(), (int64_t)1 << 40);
        int steps = 4;   // timed steps per run, sized below to about 10 ms
        int rc = 0;
        auto time_shape = [&](const TuneShape& c, double* ms_per_step) -> int {
            block_links_ = c.bl; block_voxels_ = c.bv; items_links_ = c.il; items_voxels_ = c.iv;
            claim_links_ = c.cl; claim_voxels_ = c.cv;
            if (int e = build_items(slots, err)) return e;
            if (int e = set_running(slots, tg, err)) return e;
            for (int w = 0; w < 2; w++) launch_step(stream_, false);
            float runs[3];
            for (int k = 0; k < 3; k++) {
                CK(cudaEventRecord(ev0_, stream_));
                for (int q = 0; q < steps; q++) launch_step(stream_, false);
                CK(cudaEventRecord(ev1_, stream_));
                CK(cudaEventSynchronize(ev1_));
                cudaEventElapsedTime(&runs[k], ev0_, ev1_);
            }
            std::sort(runs, runs + 3);
            *ms_per_step = runs[1] / steps;
            return 0;
        };
        TuneShape best{block_links_, block_voxels_, items_links_, items_voxels_, claim_links_, claim_voxels_};
        double bt = 0;
        if ((rc = time_shape(best, &bt)) == 0) {
            steps = std::max(2, std::min(16, (int)std::ceil(10.0 / std::max(bt, 1e-3))));
            rc = time_shape(best, &bt);
        }
        auto try_axis = [&](int TuneShape::*f1, int TuneShape::*f2, std::initializer_list<int> vals) {
            for (int v : vals) {
                if (rc) return;
                if (best.*f1 == v && (!f2 || best.*f2 == v)) continue;
                TuneShape c = best;
                c.*f1 = v;
                if (f2) c.*f2 = v;
                double t = 0;
                if ((rc = time_shape(c, &t))) return;
                if (t < 0.99 * bt) { best = c; bt = t; }
            }
        };
        try_axis(&TuneShape::bl, &TuneShape::bv, {128, 256});
        try_axis(&TuneShape::il, nullptr, {256, 512, 1024});
        try_axis(&TuneShape::iv, nullptr, {256, 512, 1024});
        try_axis(&TuneShape::cl, nullptr, {32, 64, 128});
        try_axis(&TuneShape::cv, nullptr, {32, 64, 128});
        at = 0;
        for (size_t i = 0; i < rs.size(); i++) {
            if (d_snap) CK(copy_async(arena_base_ + rs[i]->off, d_snap + at, rs[i]->bytes, cudaMemcpyDeviceToDevice, stream_));
            else CK(copy_async(arena_base_ + rs[i]->off, snap[i].data(), rs[i]->bytes, cudaMemcpyHostToDevice, stream_));
            at += rs[i]->bytes;
            CK(copy_async(d_ctl_ + rs[i]->slot, &csnap[i], sizeof(dev::Ctl), cudaMemcpyHostToDevice, stream_));
        }
        CK(cudaStreamSynchronize(stream_));
        cudaFree(d_snap);
        block_links_ = best.bl; block_voxels_ = best.bv; items_links_ = best.il; items_voxels_ = best.iv;
        claim_links_ = best.cl; claim_voxels_ = best.cv;
        tuned_ms_ = bt;
        batch_dirty_ = true;
        if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
        return rc;
    }
    double tuned_ms_ = 0;

    int eval_formula(const MathTree& m, const double* vars9, int n, double* out, std::string* err) override {
        if (n <= 0) return 0;
        char* d = nullptr;
        const size_t o_vars = align256(sizeof(MathTree)), o_out = o_vars + align256(72 * (size_t)n);
        CK(cudaMalloc(&d, o_out + 8 * (size_t)n));
        auto fail = [&](cudaError_t e) { cudaFree(d); if (err) *err = cudaGetErrorString(e); return -5; };
        cudaError_t e;
        if ((e = copy_async(d, &m, sizeof(MathTree), cudaMemcpyHostToDevice, stream_)) != cudaSuccess) return fail(e);
        if ((e = copy_async(d + o_vars, vars9, 72 * (size_t)n, cudaMemcpyHostToDevice, stream_)) != cudaSuccess) return fail(e);
        k_eval_formula<<<(unsigned)((n + 127) / 128), 128, 0, stream_>>>((const MathTree*)d, (const double*)(d + o_vars), n,
                                                                         (double*)(d + o_out));
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
        if ((e = copy_async(out, d + o_out, 8 * (size_t)n, cudaMemcpyDeviceToHost, stream_)) != cudaSuccess) return fail(e);
        if ((e = cudaStreamSynchronize(stream_)) != cudaSuccess) return fail(e);
        cudaFree(d);
        return 0;
    }
};

}  // namespace

Engine* engine_create(int device, size_t budget, std::string* err) {
    auto* e = new EngineImpl();
    if (e->init(device, budget, err)) { delete e; return nullptr; }
    return e;
}
void engine_destroy(Engine* e) { delete e; }

}  // namespace gvx
