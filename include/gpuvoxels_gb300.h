/* gpuvoxels_gb300: GB300-native Voxelyze3 soft-body step engine, C ABI.
 *
 * Drop-in boundary for the reference's simulation path.  The reference has no
 * plugin API; its boundary is the batch manager and per-simulation kernel object
 * (reference paths relative to the liusida/gpuVoxels root):
 *   - VX3_SimulationManager(sub_batches, base, input_dir, nDevices).start() -> h_results
 *       Voxelyze3/src/VX3/VX3_SimulationManager.cuh:15-46, .cu:123-155
 *   - VX3_VoxelyzeKernel(CVX_Sim*) + __device__ doTimeStep(float dt = -1)
 *       Voxelyze3/src/VX3/VX3_VoxelyzeKernel.cuh:24-30, .cu:237-359
 *   - the worker's report writer  Voxelyze3/src/Executables/vx3_node_worker.cu:98-141
 * Each entry point below names the reference interface it replaces.
 *
 * Conventions: status codes are 0 (OK) or negative (VX3_E_*); the caller owns
 * every buffer it passes; one context per host thread; calls on one context are
 * not re-entrant; all device work of a context is ordered on its own stream.
 * vx3_last_error() returns the message of the context's most recent failure.
 */
#ifndef GPUVOXELS_GB300_H
#define GPUVOXELS_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VX3_OK 0
#define VX3_E_PARSE (-1)      /* malformed VXA/VXD, unsupported feature */
#define VX3_E_OOM_BUDGET (-2) /* the HBM budget of the context cannot hold the simulation */
#define VX3_E_DIVERGED (-3)   /* reported in vx3_result.status, not returned */
#define VX3_E_TIMEOUT (-4)
#define VX3_E_CUDA (-5)
#define VX3_E_ARG (-6)
#define VX3_E_STATE (-7)
#define VX3_E_LIMIT (-8)      /* a size beyond a fixed, documented limit */

/* vx3_result.status / vx3_sim_info.status */
#define VX3_SIM_IDLE 0
#define VX3_SIM_RUNNING 1
#define VX3_SIM_DONE 2
#define VX3_SIM_DIVERGED 3
#define VX3_SIM_ERROR 4

/* run modes */
#define VX3_PLAIN 0   /* one simulation per launch, step by step (the reference's per-simulation form) */
#define VX3_BATCHED 1 /* all listed simulations packed into shared launches, CUDA-graph captured */

typedef struct vx3_ctx vx3_ctx;
typedef int64_t vx3_sim_id;

/* One finished simulation: the fields of VX3_SimulationResult
 * (Voxelyze3/src/VX3/VX3_SimulationResult.h:4-33) plus serving timestamps. */
typedef struct {
    vx3_sim_id id;
    int32_t status;
    int32_t num_voxel;
    int32_t num_measured_voxel;
    int32_t num_close_pairs;
    int64_t steps;
    double current_time;
    double fitness_score;
    double vox_size;
    double initial_center_of_mass[3];
    double current_center_of_mass[3];
    double total_distance_of_all_voxels;
    double submit_time_s, start_time_s, finish_time_s;
} vx3_result;

typedef struct {
    int32_t num_voxel;
    int32_t num_link;
    int32_t status;
    int32_t pad;
    double dt;
    double current_time;
    int64_t steps;
} vx3_sim_info;

/* Replaces VX3_SimulationManager construction (VX3_SimulationManager.cu:123-130) and its
 * heap sizing (:384-396): reserves `hbm_budget_bytes` of device memory (0 = half of free). */
vx3_ctx* vx3_create(int device, size_t hbm_budget_bytes);
/* Replaces ~VX3_SimulationManager (VX3_SimulationManager.cu:131-136). */
void vx3_destroy(vx3_ctx* ctx);
const char* vx3_last_error(vx3_ctx* ctx);

/* Replaces VX3_SimulationManager::readVXD for one file (VX3_SimulationManager.cu:277-380):
 * merges the VXD into the base VXA (Utils/ctool.h:49-57), reads it, builds the
 * voxel/link topology.  Host only; device memory is taken when the simulation first runs. */
int vx3_load_vxa(vx3_ctx* ctx, const char* base_vxa_xml, const char* vxd_xml_or_null, const char* name, vx3_sim_id* out);
/* A whole generation at once (the loop of VX3_SimulationManager::readVXD over its files,
 * VX3_SimulationManager.cu:285-380): n VXDs merged into the base (vxds NULL or an entry NULL =
 * the base alone; base NULL = every entry is a whole VXA), parsed and built on host threads.
 * ids[i] = -1 and status[i] (optional) = the error code where file i is rejected; the others
 * load.  Returns VX3_OK, or the first error code with its message in vx3_last_error. */
int vx3_load_vxa_many(vx3_ctx* ctx, const char* base_vxa_xml_or_null, const char* const* vxds, const char* const* names, int n,
                      vx3_sim_id* ids, int* status_or_null);

/* Replaces CVX_Voxel::external() fixes/forces (Voxelyze3/src/old/VX_External.h:58-79):
 * dof_fixed bits 0-2 fix x/y/z translation, 3-5 fix x/y/z rotation.  Before the first step only. */
int vx3_set_external(vx3_ctx* ctx, vx3_sim_id id, int voxel, int dof_fixed, const float force[3], const float moment[3],
                     const double translate[3], const double rotate[3]);

/* Replaces VX3_SimulationManager::start() for a batch (VX3_SimulationManager.cu:138-155):
 * runs every listed simulation until its StopConditionFormula holds (or max_steps, 0 = 1e6). */
int vx3_run(vx3_ctx* ctx, const vx3_sim_id* ids, int n, int mode, int64_t max_steps);
/* Replaces n calls of VX3_VoxelyzeKernel::doTimeStep() (VX3_VoxelyzeKernel.cu:237-359). */
int vx3_step(vx3_ctx* ctx, const vx3_sim_id* ids, int n, int mode, int64_t steps);

/* Serving pair (no reference counterpart beyond the dir-watch daemon, Executables/vx3_node_daemon.cu:16-66):
 * submit queues a loaded simulation with a horizon in steps; poll admits queued simulations as
 * the HBM budget allows, advances all admitted ones by `chunk_steps`, retires finished ones and
 * returns up to `max` results (the count, or a negative status). */
int vx3_submit(vx3_ctx* ctx, vx3_sim_id id, int64_t horizon_steps);
int vx3_poll(vx3_ctx* ctx, vx3_result* out, int max, int chunk_steps);
int vx3_pending(vx3_ctx* ctx);
/* Serving policy of vx3_poll's admission (no reference counterpart): order 0 admits queued
 * simulations first come first served (the default), 1 the least work first (voxels x horizon
 * steps; ties in arrival order; under a never-ending stream long requests may wait indefinitely),
 * 2 the least work first beside one lane: whenever no request is running in the lane, the queued
 * request with the most work is admitted into it first, so that the longest requests overlap the
 * short ones rather than run alone at the end; max_active_voxels caps the voxels the running
 * batch holds (0 = as the HBM budget allows; a request is always admitted into an empty batch;
 * the lane's request is not counted). */
#define VX3_SERVE_FCFS 0
#define VX3_SERVE_LEAST_WORK 1
#define VX3_SERVE_LONG_LANE 2
int vx3_set_serving(vx3_ctx* ctx, int order, int64_t max_active_voxels);

/* Replaces VX3_SimulationManager::collectResults for one simulation (VX3_SimulationManager.cu:416-458). */
int vx3_get_result(vx3_ctx* ctx, vx3_sim_id id, vx3_result* out);
int vx3_sim_info_get(vx3_ctx* ctx, vx3_sim_id id, vx3_sim_info* out);
/* Voxel and link counts of many simulations, from the host-side description only (no
 * device read): what VX3_VoxelyzeKernel keeps as num_d_voxels / num_d_links
 * (Voxelyze3/src/VX3/VX3_VoxelyzeKernel.cuh:72,79).  Either output may be NULL.
 * num_link is the number of links loaded from the VXA: links that VX3 attachment (EnableAttach)
 * creates during the run are not in it; vx3_get_links reports the live count. */
int vx3_sim_sizes(vx3_ctx* ctx, const vx3_sim_id* ids, int n, int32_t* num_voxel, int32_t* num_link);

/* Voxel state in the reference's CVX_Voxel member layout (Voxelyze3/src/old/VX_Voxel.h:166-182):
 * pos[3*nv], orient[4*nv] (w,x,y,z) and flags[nv]; any pointer may be NULL. */
int vx3_get_state(vx3_ctx* ctx, vx3_sim_id id, double* pos, double* orient, uint8_t* flags);
/* The same for a whole generation in one device pass and one copy (the read-back loop of
 * VX3_SimulationManager::collectResults, VX3_SimulationManager.cu:416-455): the voxels of
 * ids[0], ids[1], ... follow one another in pos / orient / flags, each simulation's block
 * sized by its num_voxel.  Any output pointer may be NULL. */
int vx3_get_states(vx3_ctx* ctx, const vx3_sim_id* ids, int n, double* pos, double* orient, uint8_t* flags);
/* Full voxel state: d13 = pos3 linMom3 orient4 angMom3, f4 = temperature, poisson strain3, flags. */
int vx3_get_voxel_state(vx3_ctx* ctx, vx3_sim_id id, double* d13, float* f4, int32_t* flags);
/* Link state (CVX_Link, VX_Link.h:68-99): d9 = pos2 angle1v angle2v, f3 = strain maxStrain strainOffset, flags. */
int vx3_get_link_state(vx3_ctx* ctx, vx3_sim_id id, double* d9, float* f3, int32_t* flags);
/* VX3 extras of one simulation: measures4 = targetCloseness, numClosePairs, collisionCount and
 * recentAngle (VX3_VoxelyzeKernel members, VX3/VX3_VoxelyzeKernel.cuh); signals6 = per voxel
 * localSignal, localSignaldt, inactiveUntil, d_signal.value, d_signal.activeTime and
 * packmakerNextPulse (VX3_Voxel members, VX3/VX3_Voxel.h:304-309; zeros without EnableSignals).
 * Either pointer may be NULL. */
int vx3_get_extras(vx3_ctx* ctx, vx3_sim_id id, double* measures4, double* signals6);
/* Every link in use, the loaded ones first, then those VX3 attachment created during the run
 * (VX3_VoxelyzeKernel::d_v_links, VX3/VX3_VoxelyzeKernel.cuh): *n_links, and for the first
 * `max` links negative-end voxel, positive-end voxel, axis and flag byte (ends4, may be NULL). */
int vx3_get_links(vx3_ctx* ctx, vx3_sim_id id, int32_t* n_links, int32_t* ends4, int max);

/* Replaces the .history stream the reference prints from its simulation loop when the VXA
 * sets Simulator/RecordHistory/RecordStepSize (VX3/VX3_SimulationManager.cu:40-114): settings
 * header, then every int(RecordStepSize/(10000*recommendedTimeStep*DtFrac))+1 loop steps a
 * line with the surface voxels (RecordVoxel, default 1) and links (RecordLink).  Writes to
 * `path` during the following vx3_run / vx3_step calls (which then advance in chunks that end
 * on recorded steps); NULL stops recording.  VX3_E_ARG if the VXA has no RecordStepSize. */
int vx3_record_history(vx3_ctx* ctx, vx3_sim_id id, const char* path_or_null);

/* Replaces the worker's report (Executables/vx3_node_worker.cu:98-141): report.inputdir,
 * report.bestfit.{filename,fitness_score}, report.detail.<name>.{...}; results sorted by
 * fitness with NaN last (VX3_SimulationResult.h:26-33).  A simulation whose VXA sets
 * Simulator/SavePositionOfAllVoxels also gets init_pos, pos and mats (vx3_node_worker.cu:123-139). */
int vx3_write_report(vx3_ctx* ctx, const vx3_sim_id* ids, int n, const char* input_dir, const char* path);
/* One report over the simulations of several contexts (one per GPU), as the worker writes a
 * single report after dealing files across devices (vx3_node_worker.cu:88-98).  ids[k] lists
 * counts[k] simulations of ctxs[k]; errors are left in ctxs[0]. */
int vx3_write_report_multi(vx3_ctx* const* ctxs, const vx3_sim_id* const* ids, const int* counts, int nctx,
                           const char* input_dir, const char* path);

/* Releases a simulation's device memory and host state. */
int vx3_free_sim(vx3_ctx* ctx, vx3_sim_id id);

/* Timing of the last vx3_run/vx3_step call on the context stream:
 * out[0] device ms (CUDA events), out[1] wall ms, out[2] voxel-steps, out[3] kernel launches,
 * out[4..6] link/contact/voxel kernel ms of the last profiled step. */
int vx3_last_timing(vx3_ctx* ctx, double* out7);
/* Bytes the context has copied host->device and device->host since vx3_create (uploads,
 * control blocks, read-backs): what a caller's data movement costs. */
int vx3_transfer_bytes(vx3_ctx* ctx, int64_t* h2d, int64_t* d2h);
/* Tuning: threads per block and elements per work item for the link and voxel
 * launches, and steps per captured graph; 0 keeps the current value. */
int vx3_set_tuning(vx3_ctx* ctx, int block_links, int block_voxels, int items_links, int items_voxels, int graph_steps);
/* Elements (links, voxels) a warp claims from the step kernels' work queues at a time: multiples of 32
 * (0 keeps the current value).  No reference counterpart: the reference launches one thread per element. */
int vx3_set_claim_sizes(vx3_ctx* ctx, int claim_links, int claim_voxels);
/* Searches the launch shape on the given simulations and keeps the fastest found: threads per block
 * (128, 256), elements per link and per voxel work item (256, 512, 1024: the grouping window) and elements
 * a warp claims from the link and voxel queues at a time (32, 64, 128), one axis at a time from the
 * current shape, each candidate timed as the median of three runs.  The simulations' device state is
 * copied aside before and put back after, so their results are those of an untuned run.
 * No reference counterpart (the reference's launch shapes are fixed, VX3_VoxelyzeKernel.cu:237-359). */
int vx3_autotune(vx3_ctx* ctx, const vx3_sim_id* ids, int n);
/* The launch shape in use: out8 = threads per block (links, voxels), elements per work item (links,
 * voxels), steps per captured graph, elements per claim (links, voxels), contact slots per voxel. */
int vx3_get_tuning(vx3_ctx* ctx, int32_t* out8);
/* Contacts kept in each voxel's own slots (1..16, default 16) for simulations uploaded afterwards; a voxel
 * with more contacts in a step takes records of the context's spill pool (1/64 of the HBM budget), so the
 * contact list has no per-voxel limit, like the reference's CVX_Voxel::colWatch vector
 * (Voxelyze3/src/old/Voxelyze.cpp:726-751).  A memory/speed knob only: results do not depend on it.
 * A step whose contacts overflow the whole pool stops the simulations concerned with VX3_SIM_ERROR. */
int vx3_set_contact_slots(vx3_ctx* ctx, int slots);
int vx3_set_profiling(vx3_ctx* ctx, int on);
/* Kernel build used by the context (no reference counterpart: the reference has one GPU build).
 * VX3_EXACT (default): every FP64/FP32 multiply and add rounded separately, as the reference's CPU path.
 * VX3_FMA: multiply-add pairs contracted into FMAs; fewer FP64 instructions, results within the
 * parity tolerance of the reference rather than bit-faithful to its rounding. */
#define VX3_EXACT 0
#define VX3_FMA 1
int vx3_set_precision(vx3_ctx* ctx, int mode);

/* Mass-weighted centre of mass of n points already on the device, for callers that cannot
 * allocate device memory: a plugin inside another framework whose caching allocator or pool owns
 * the device memory, a real-time loop that cannot take cudaMalloc's implicit synchronisation and
 * latency, a service whose HBM budget must account for every allocation.
 * This entry point has no counterpart in the reference.  It is the engine's centre-of-mass
 * reduction (per-block partial sums, then one fixed-order fold) with its scratch in a fixed
 * array compiled into the library, so it calls no cudaMalloc, cudaFree or allocating routine.
 *   x, y, z[n] (double), mass[n] (float): device inputs; out4: device output (cx, cy, cz, total mass;
 *   zeros for n = 0 or a total mass of 0);
 *   stream: a cudaStream_t, or NULL for the legacy default stream; the work is only enqueued.
 * Limit: n <= VX3_NOALLOC_MAX_POINTS; larger n returns VX3_E_LIMIT without launching anything.
 * A CUDA error already pending on the calling thread makes it return VX3_E_CUDA without launching
 * and leaves that error pending for the caller.
 * The scratch (64 KiB) stays resident on every GPU that loads the library until the process exits.
 * The first call on a device resolves the scratch array's device address with that device current
 * (kept for the life of the process; a cudaDeviceReset of the device invalidates it); make that first
 * call before any stream capture.  All calls share the scratch and it keeps the last call's contents
 * (each call overwrites everything it reads); calls that overlap on the GPU race, so serialise them
 * (one stream, or events between streams). */
#define VX3_NOALLOC_MAX_POINTS 4194304
int vx3_center_of_mass_noalloc(const double* x, const double* y, const double* z, const float* mass, int64_t n, double* out4,
                               void* stream);
/* Device bytes a loaded simulation needs when resident (for HBM-budget admission). */
int64_t vx3_sim_bytes(vx3_ctx* ctx, vx3_sim_id id);
size_t vx3_bytes_in_use(vx3_ctx* ctx);

/* Host-only inspection (no device, no context): reads a VXA (+VXD) the way vx3_load_vxa does and
 * reports what the engine would simulate.  Replaces reading CVX_Sim/CVoxelyze members after
 * CVX_Sim::Import (Voxelyze3/src/VXA/VX_Sim.cpp:59-153).
 *   counts[6] = voxels, links, voxel materials, link materials, surface voxels, externals
 *   env[12]   = voxel size, DtFrac, gravity (g), floor, collisions, vary temperature, amplitude,
 *               period, expansion, initial temperature, bounding radius, watch distance
 * Returns VX3_OK or VX3_E_PARSE (message in err, up to err_len bytes). */
int vx3_inspect_vxa(const char* base_vxa_xml, const char* vxd_xml_or_null, int32_t* counts, double* env, char* err, int err_len);
/* Topology and derived constants, sized from vx3_inspect_vxa counts; any pointer may be NULL.
 *   vox4[4*nv]  = ix, iy, iz, material;  lnk4[4*nl] = negative voxel, positive voxel, axis, link material
 *   phase[nv]; vmat18[18*nvm] and vnom[nvm] in CVX_MaterialVoxel order (E, nu, rho, cte, muStatic, muKinetic,
 *   zetaInternal, zetaGlobal, zetaCollision, eHat, mass, 1/mass, sqrt(mass), inertia, 1/inertia,
 *   2sqrt(mEs), 2sqrt(IEs^3), gravity); lidx2[2*nlm] constituent voxel materials;
 *   lmat20[20*nlm] = E, nu, eHat, a1, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp,
 *   sigmaYield, sigmaFail, epsYield, epsFail, linear, nomSize, rho. */
/* Host-only: the externals the VXA's boundary-condition regions put on each voxel, as
 * CVX_Sim::Import applies them (VXA/VX_Sim.cpp:109-144): dof[nv] fixed-DOF bits (1,2,4 translate
 * x,y,z; 8,16,32 rotate), fm6[6*nv] force xyz + moment xyz, tr6[6*nv] prescribed translation xyz +
 * rotation xyz; zeros for voxels no region touches. */
int vx3_inspect_externals(const char* base_vxa_xml, const char* vxd_xml_or_null, int32_t* dof, float* fm6, double* tr6);
int vx3_inspect_topology(const char* base_vxa_xml, const char* vxd_xml_or_null, int32_t* vox4, int32_t* lnk4, double* phase,
                         float* vmat18, double* vnom, int32_t* lidx2, float* lmat20);
/* Stop/fitness formula evaluation as the engine performs it (Utils/VX3_MathTree.h:50-192);
 * which: 0 stop condition, 1 fitness.  vars = x, y, z, hit, t, angle, closeness, numClosePairs, num_voxel. */
int vx3_inspect_formula(const char* base_vxa_xml, const char* vxd_xml_or_null, int which, const double* vars9, double* out);
/* The same formulas evaluated on the context's device by the evaluator the step kernels use
 * (VX3_MathTree::eval run on the GPU, Utils/VX3_MathTree.h:50-192; stop condition in the step loop,
 * VX3_VoxelyzeKernel.cu:162-182; force field in the voxel update, VX3_Voxel.cu:178-184), for n
 * variable sets of 9 doubles (vars9[9*n]); which: 0 stop condition, 1 fitness, 2/3/4 force field
 * x/y/z.  out[n]; absent formulas give NaN (0 for an absent force-field component). */
int vx3_eval_formula(vx3_ctx* ctx, const char* base_vxa_xml, const char* vxd_xml_or_null, int which, const double* vars9, int n,
                     double* out);

#ifdef __cplusplus
}
#endif
#endif
