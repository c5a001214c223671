// Device data layout shared by the host engine and both kernel builds.

#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mathtree.h"

namespace gvx {
namespace dev {

// ---------------------------------------------------------------- layouts
// Contact list of one voxel in one step: up to kContactInline contacts sit in the voxel's
// own slots; a voxel with more takes a run of records from the context's spill pool, so the
// list is unbounded like the reference's (only the pool's size, a fraction of the HBM
// budget, limits the contacts of a whole step).
constexpr int kContactInline = 16;
constexpr int kReachWords = 8;        // 231 offsets of the L1 ball of radius 5 -> 8 x 32 bits
constexpr int kOrderKeysBins = 10;    // link ordering keys (the step kernels' kOrderKeys)

// voxel flag bits
constexpr uint32_t VF_LINKS = 0x3Fu;      // bits 0..5: link present in direction d
constexpr uint32_t VF_STATIC = 1u << 6;   // FLOOR_STATIC_FRICTION
constexpr uint32_t VF_INTERIOR = 1u << 7; // all 6 links present
constexpr uint32_t VF_EXT = 1u << 8;      // has an external
constexpr uint32_t VF_MEASURED = 1u << 9;
// link flag bits
constexpr uint8_t LF_SMALL = 1;           // small-angle mode
constexpr uint8_t LF_LVV = 2;             // LOCAL_VELOCITY_VALID
constexpr uint8_t LF_WIDE1 = 4;           // last step: angle1 came from FromAngleToPosX's general (acos/sincos) branch
constexpr uint8_t LF_WIDE2 = 8;           // last step: angle2's rotation vector took the acos branch
constexpr uint8_t LF_ACOS1 = 16;          // last step: angle1's rotation vector took the acos branch
constexpr uint8_t LF_GONE = 32;           // VX3: detached (failed) or removed with a voxel: no longer updated
constexpr uint8_t LF_REMOVED = 64;        // VX3: removed with a voxel (left out of the history's link records)
constexpr uint32_t VF_FLOORC = 1u << 10;  // last step: the voxel touched the floor
constexpr uint32_t VF_REMOVED = 1u << 11; // VX3: removed from the simulation (frozen, no links, no contacts)
constexpr uint32_t VF_TGTHIT = 1u << 12;  // VX3: this step's contacts include a target voxel (non-target voxel)
constexpr uint32_t VF_ATTACH = 1u << 13;  // VX3: enableAttach (every attach condition holds at the voxel)
constexpr uint32_t VF_WROT = 1u << 14;    // last step: the orientation update took the sin/cos branch (grouping key only)

// sim flag bits
constexpr int SF_FLOOR = 1, SF_COLLIDE = 2, SF_VARY = 4, SF_EXPAND = 8;
constexpr int SF_CILIA = 16, SF_FFIELD = 32;   // VX3 extras: cilia forces, force-field formulas
constexpr int SF_SIGNALS = 64;                 // VX3 signals
constexpr int SF_TARGETS = 128;                // target materials present (contact count, closeness)
constexpr int SF_DETACH = 256;                 // failed links detach from their voxels
constexpr int SF_REMOVE = 512;                 // secondary experiment: material removal, initial position reset
constexpr int SF_FIXEDMAT = 1024;              // materials marked Fixed (their voxels never move)
constexpr int SF_ATTACH = 2048;                // touching sticky voxels may be joined by new links
constexpr int SF_DYNSURF = SF_DETACH | SF_REMOVE | SF_ATTACH;   // the surface set can change during the run
constexpr int SF_WATCH = 4096;                 // contacts from watch lists regenerated as the reference does

// VMat::vx3 bits
constexpr int VM_TARGET = 1, VM_PACEMAKER = 2, VM_FIXED = 4, VM_STICKY = 8;

struct VMat {
    float E, nu, cte, mus, muk, eHat;
    float mass, massInv, Iinv;
    float dampNum;      // 2*sqrtMass*zetaInternal   (numerator of dampingMultiplier)
    float gDampT, gDampR, cDampT;   // zg*c2m, zg*c2i, zc*c2m
    float gravForce;    // -mass*9.80665f*gravMult
    float penStiff;     // (float)(2*E*nom)
    float sizef;        // (float)nom
    double nom;
    int32_t measured;
    int32_t vx3;        // VM_* bits
    // the float constants above that enter FP64 expressions, widened once (exact)
    double massInvD, IinvD, gDampTD, gDampRD, cDampTD, gravForceD;
    double halfNom;       // nom/2
    double halfMassInv;   // 0.5*(double)massInv
    // VX3 material extras: cilia force scale and start time, thermal actuation start time
    double cilia, ciliaOn, thermalOn;
    // signals: pacemaker period, relayed fraction, relay delay, refractory period; removal time
    double pmPeriod, sigDecay, sigDelay, sigInactive, removeAfter;
    int32_t attachLmat;   // link material of a new link between two voxels of this material (-1: not sticky)
    int32_t pad_vm;
    // powf(x, -nu) of the host's C library for every float x in [0.5, 2) (index: bits(x) - kPowTabFirst),
    // the Poisson power of the reference's CPU path; null when nu is 0
    const float* powtab;
};
constexpr uint32_t kPowTabFirst = 0x3F000000u;   // bits of 0.5f
constexpr uint32_t kPowTabSize = 0x01000000u;    // floats in [0.5, 2)

// VX3 per-voxel signal state (SF_SIGNALS), one block of nv doubles each
enum SigField {
    SG_LOCAL = 0,     // localSignal
    SG_LOCAL_DT,      // localSignaldt: next decay time
    SG_INACTIVE,      // inactiveUntil
    SG_VALUE,         // d_signal.value: pending signal to relay
    SG_ACTIVE,        // d_signal.activeTime
    SG_PULSE,         // packmakerNextPulse
    SG_OUT,           // this step's relayed value (0: none)
    SG_OUT_T,         // its arrival time at the neighbours
    SG_FIELDS
};

struct LMat {
    float E, nu, eHat, a1, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp, epsFail;
    int32_t linear, n;
    float strain[18], stress[18];
    // beam and damping constants widened once (exact float -> double)
    double a2D, b1D, b2D, b3D, sqA1D, sqA2xIpD, sqB1D, sqB2xFMpD, sqB3xIpD;
};

struct Ext {
    int32_t dof;
    float f[3], m[3];
    double tr[3];
    double rq[4];       // rotationQuat (w,x,y,z)
};

// Per-simulation device descriptor: pointers into the simulation's region.
struct Sim {
    int32_t nv, nl, nsurf, flags;
    double temp_amp, temp_period;
    double cell_size;           // spatial hash cell edge (m)
    int32_t hash_size;          // buckets per table (power of two)
    float env_radius;           // 0.625
    const VMat* vm;
    const LMat* lm;
    const Ext* ext;
    // voxel SoA (state)
    double *px, *py, *pz, *mx, *my, *mz, *qw, *qx, *qy, *qz, *ax, *ay, *az;
    float* temp;
    float* ps;                  // poisson strain, 3 blocks of nv
    uint32_t* vfl;
    const uint8_t* vmat;
    const int32_t* vext;
    const double* phase;
    // link -> voxel slots (direction d of voxel v): force (18 x nv), moment (18 x nv), axial strain (6 x nv)
    double* sf;
    double* sm;
    float* ss;
    // links (written during the run only by VX3 attachment)
    int32_t *lneg, *lpos;
    uint8_t *lax, *lmt;
    double* lst;                // 9 blocks of nl: pos2 xyz, angle1v xyz, angle2v xyz
    float* lsf;                 // 3 blocks of nl: strain, maxStrain, strainOffset
    uint8_t* lfl;
    // collisions
    const int32_t* surf;        // surface voxel ids (sorted)
    const int16_t* ijk;         // lattice indices, 3 blocks of nv
    const uint32_t* reach;      // kReachWords per voxel
    int32_t* ccount;            // per voxel
    float* cforce;              // 3*kContactInline per voxel
    int32_t* cspill;            // per voxel: first spill record when ccount > kContactInline
    // the context's spill pool (shared by every simulation of a step): partner and force
    // records, the records taken this step (reset by k_links) and the pool's capacity
    int32_t* spill_p;
    float* spill_f;
    int32_t* spill_used;
    int32_t spill_cap;
    int32_t contact_inline;     // contacts kept in the voxel's own slots (1..kContactInline); more spill
    int32_t* hash_head;         // 2 tables of hash_size
    int32_t* hash_next;         // per voxel
    float4* cpos;               // per hashed voxel: position rounded to float, float base size (broadphase only)
    // watch lists (SF_WATCH), the reference's collision list (Voxelyze.cpp:671-751): per voxel the
    // position at the last regeneration (lastColWatchPosition, float), per surface index the
    // offset of its partners in wlist (nsurf + 1 entries), the list's capacity, the squared watch
    // radius and re-check distance (float, as the reference forms them), and the hash cells the
    // regeneration scans on each side of a voxel's own
    float4* watch;
    int32_t* woff;
    int32_t* wlist;
    int32_t wcap;
    int32_t wcells;
    float watch_r2, recalc2;
    float inv_cell;             // 1 / cell_size, for the float cell index
    // VX3 extras
    const double* cilia;        // BaseCiliaForce, 3 blocks of nv (SF_CILIA)
    const MathTree* ffield;     // x, y, z force-field formulas (SF_FFIELD)
    const double* shift_cilia;  // ShiftCiliaForce, 3 blocks of nv (SF_CILIA with SF_SIGNALS)
    double* sig;                // SG_FIELDS blocks of nv (SF_SIGNALS)
    int32_t* vlink;             // link per voxel direction, 6 per voxel, -1 if none (SF_SIGNALS, SF_REMOVE, SF_ATTACH)
    const int32_t* targets;     // target voxel ids in index order (SF_TARGETS)
    int32_t n_targets;
    int32_t n_mats;
    double close_r;             // MaxDistInVoxelLengthsToCountAsPair * voxel size (0: closeness off)
    double reinit_after;        // ReinitializeInitialPositionAfterThisManySeconds (SF_REMOVE set: secondary experiment)
    double* init_pos;           // initial positions, 3 blocks of nv (secondary experiment)
    // VX3 attachment (SF_ATTACH): link capacity (links nl..nl_cap-1 are created at run time),
    // new-link damping counters, candidate pairs of this step, the attach conditions
    int32_t nl_cap;
    int32_t cand_cap;           // pairs
    int32_t safety_guard;
    int32_t attach_mask;        // bit k: AttachCondition k given (a missing one holds)
    int32_t* lnew;              // per link: steps left with forces scaled by 0.01
    int32_t* cand;              // 2 per candidate pair
    int32_t* cpart;             // contact partners, kContactInline per voxel
    const MathTree* attach_cond;   // 5 formulas
};

// Mutable per-simulation control block.
struct Ctl {
    double t;
    float dt, optdt;
    int32_t status, diverged, error, cycle_step;
    int64_t steps, target;
    int32_t done_items, n_vox_items, item_begin, angle_samples;
    uint32_t maxf2_bits;
    int32_t hash_parity;
    int32_t no_stop;            // set while vx3_step advances a fixed count: the stop formula is not applied
    int32_t sig_done_items;     // signal-phase items finished this step (SF_SIGNALS)
    double com[3], com_hist[2][3];
    double recent_angle;
    double t_cycles;            // (t + dt) / TempPeriod for the coming step (actuation phase)
    // VX3 measures: target closeness and close pairs (at CoM samples), target contacts so far
    double closeness;
    int32_t num_close_pairs, hit_count;
    int32_t sig_pending;        // 1 between a completed voxel update and its signal phase
    int32_t removed_mats;       // materials already removed (bit per palette index)
    int32_t reinit_done;        // initial centre of mass reset (secondary experiment)
    int32_t n_links;            // links in use (VX3 attachment appends)
    int32_t n_cand;             // attachment candidates found this step
    int32_t col_stale;          // SF_WATCH: regenerate the watch lists at this step's contact pass
    int32_t col_moved;          // SF_WATCH: a surface voxel moved beyond the re-check distance this step
    int32_t watch_ok;           // SF_WATCH: the lists hold the current regeneration (else the hash search runs)
    int32_t watch_regens;       // regenerations so far
    int32_t c_item_begin;       // the simulation's contact items in the batch's contact item list
    int32_t c_item_count;
    int32_t watch_used;         // SF_WATCH: list entries taken by this regeneration's runs
    int32_t pad_watch;
    double init_com[3];         // initial centre of mass (host value, reset by the secondary experiment)
    MathTree stop;
};

struct Item {
    int32_t sim, begin, end, seq;
};

// One list to group by key (k_bin_*): its work items, the element kind (0 links,
// 1 voxels), the window in items, and the per-item counts / offsets, the listed
// count and the (simulation, element) list.
struct BinList {
    const Item* items;
    int32_t n_items, kind, win, pad;
    int32_t* hist;
    int32_t* base;
    int32_t* total;
    int2* perm;
};

}  // namespace dev
}  // namespace gvx
