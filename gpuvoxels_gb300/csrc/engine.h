// GB300 step engine: device layout, batching and serving.  Host-side interface.
#pragma once
#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "mathtree.h"
#include "world.h"

namespace gvx {

enum SimStatus : int32_t {
    SIM_IDLE = 0,       // loaded, not scheduled
    SIM_RUNNING = 1,
    SIM_DONE = 2,       // stop condition or horizon reached
    SIM_DIVERGED = 3,   // a link strain exceeded 100 (Voxelyze3/src/old/Voxelyze.cpp:263-269)
    SIM_ERROR = 4,      // contact list overflow or other device-detected error
};

enum RunMode : int32_t { MODE_PLAIN = 0, MODE_BATCHED = 1 };

struct SimResult {
    int64_t id;
    int32_t status;
    int32_t num_voxel;
    int32_t num_measured_voxel;
    int32_t num_close_pairs;
    int64_t steps;
    double current_time;
    double fitness;
    double vox_size;
    double initial_com[3];
    double current_com[3];
    double total_distance;
    double submit_s, start_s, finish_s;   // host wall clock (seconds since context creation)
};

struct Timing {
    double device_ms = 0;        // CUDA-event time of the last run/step call on the context stream
    double wall_ms = 0;
    int64_t voxel_steps = 0;     // voxels x steps actually advanced
    int64_t launches = 0;        // kernel launches issued by the last call (graph nodes counted)
    double link_kernel_ms = 0;   // per-kernel CUDA-event times (profiling mode only)
    double voxel_kernel_ms = 0;
    double contact_kernel_ms = 0;
};

class Engine;
Engine* engine_create(int device, size_t budget_bytes, std::string* err);
void engine_destroy(Engine* e);

class Engine {
public:
    virtual ~Engine() = default;
    virtual int add_sim(const SimDesc& d, int64_t* id, std::string* err) = 0;
    // Many at once: topology and materials are built on host threads; ids[i] = -1 and
    // errs[i] set where descs[i] is rejected.  Returns the number rejected.
    virtual int add_sims(const SimDesc* const* descs, int n, int64_t* ids, std::string* errs) = 0;
    // The same, with each description made on the host thread that builds it: read(i, &d,
    // &err) fills simulation i's description or returns false with the reason.
    virtual int add_sims_read(int n, const std::function<bool(int, SimDesc*, std::string*)>& read, int64_t* ids,
                              std::string* errs) = 0;
    virtual int set_external(int64_t id, const External& x, std::string* err) = 0;
    // Advance the given simulations by exactly `steps` steps each (fewer if they stop).
    virtual int step(const int64_t* ids, int n, int mode, int64_t steps, std::string* err) = 0;
    // Run the given simulations until their stop condition (or max_steps).
    virtual int run(const int64_t* ids, int n, int mode, int64_t max_steps, std::string* err) = 0;
    // Serving: queue a simulation with a step horizon; admitted as memory frees up.
    virtual int submit(int64_t id, int64_t horizon_steps, std::string* err) = 0;
    // Serving: advance everything admitted by one chunk, admit/retire; returns finished results.
    virtual int poll(SimResult* out, int max, int chunk_steps, std::string* err) = 0;
    virtual int pending() const = 0;
    // Serving policy: admission order (0 first come first served, 1 least voxels x horizon first)
    // and the most voxels the running batch may hold (0 = as the HBM budget allows).
    virtual int set_serving(int order, int64_t max_active_voxels) = 0;
    virtual int result(int64_t id, SimResult* out, std::string* err) = 0;
    virtual int info(int64_t id, int* nv, int* nl, double* dt, double* t, int64_t* steps, int* status) = 0;
    virtual int voxel_state(int64_t id, double* d13, float* f4, int32_t* flags, std::string* err) = 0;
    // VX3 extras: measures4 = targetCloseness, numClosePairs, collisionCount, recentAngle;
    // sig6 = per voxel localSignal, next decay time, refractory-until, pending signal, its time,
    // next pacemaker pulse (zeros without signals).  Either pointer may be null.
    virtual int extras(int64_t id, double* measures4, double* sig6, std::string* err) = 0;
    // Every link in use (the loaded ones, then those VX3 attachment made): *n_links, and for
    // the first `max` of them negative end, positive end, axis and flag byte.
    virtual int links(int64_t id, int32_t* n_links, int32_t* ends4, int max, std::string* err) = 0;
    // Bytes the context has copied host->device and device->host since it was created.
    virtual void transfer_bytes(int64_t* h2d, int64_t* d2h) const = 0;
    // Poses of many simulations in one device pass and one copy: pos3/q4/flags hold the
    // simulations' voxels one after another in the order of ids (any pointer may be null).
    virtual int gather_states(const int64_t* ids, int n, double* pos3, double* q4, uint8_t* flags, std::string* err) = 0;
    virtual int link_state(int64_t id, double* d9, float* f3, int32_t* flags, std::string* err) = 0;
    // Report extras of VXA Simulator/SavePositionOfAllVoxels: initial and current voxel positions
    // (x,y,z per voxel) and palette material ids (1-based); *save = the VXA flag (vectors untouched if 0).
    virtual int saved_positions(int64_t id, int* save, std::vector<double>* init, std::vector<double>* cur,
                                std::vector<int>* matid, std::string* err) = 0;
    virtual int free_sim(int64_t id) = 0;
    // Host-side description of a loaded simulation (topology, materials, VXA settings); null if unknown.
    virtual const SimWorld* world(int64_t id) = 0;
    // recommendedTimeStep of the simulation (0 until its first step).
    virtual double optimal_dt(int64_t id) = 0;
    virtual const Timing& timing() const = 0;
    virtual void set_profiling(int on) = 0;
    virtual size_t bytes_in_use() const = 0;
    virtual int device_check(std::string* err) = 0;
    virtual int set_tuning(int block_links, int block_voxels, int items_links, int items_voxels, int graph_steps) = 0;
    virtual int autotune(const int64_t* ids, int n, std::string* err) = 0;
    // Elements a warp claims from the link / voxel queues at a time (multiples of 32; 0 keeps).
    virtual int set_claims(int claim_links, int claim_voxels) = 0;
    // Contacts kept in each voxel's own slots (1..kContactInline) for simulations uploaded later.
    virtual int set_contact_slots(int n) = 0;
    // block_links, block_voxels, items_links, items_voxels, graph_steps, claim_links,
    // claim_voxels, contact slots
    virtual void get_tuning(int32_t* out8) const = 0;
    // A formula evaluated on the device for n variable sets of 9 (x, y, z, hit, t, angle,
    // closeness, numClosePairs, num_voxel): the step kernels' evaluator.
    virtual int eval_formula(const MathTree& m, const double* vars9, int n, double* out, std::string* err) = 0;
    virtual int64_t sim_bytes(const SimDesc& d) const = 0;
    virtual int64_t sim_bytes_id(int64_t id) = 0;
    // 0: exact build (no contraction, the reference's rounding); 1: FMA build
    virtual int set_precision(int fma) = 0;
    virtual int precision() const = 0;
};

}  // namespace gvx
