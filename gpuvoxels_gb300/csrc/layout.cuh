// Device data layout shared by the host engine and both kernel builds.

#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mathtree.h"

namespace gvx {
namespace dev {

// ---------------------------------------------------------------- layouts
constexpr int kContactCap = 32;       // contacts kept per voxel per step
constexpr int kReachWords = 8;        // 231 offsets of the L1 ball of radius 5 -> 8 x 32 bits

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
constexpr uint32_t VF_FLOORC = 1u << 10;  // last step: the voxel touched the floor

// sim flag bits
constexpr int SF_FLOOR = 1, SF_COLLIDE = 2, SF_VARY = 4, SF_EXPAND = 8;
constexpr int SF_CILIA = 16, SF_FFIELD = 32;   // VX3 extras: cilia forces, force-field formulas

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
    int32_t pad;
    // the float constants above that enter FP64 expressions, widened once (exact)
    double massInvD, IinvD, gDampTD, gDampRD, cDampTD, gravForceD;
    double halfNom;       // nom/2
    double halfMassInv;   // 0.5*(double)massInv
    // VX3 material extras: cilia force scale and start time, thermal actuation start time
    double cilia, ciliaOn, thermalOn;
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
    // links
    const int32_t *lneg, *lpos;
    const uint8_t *lax, *lmt;
    double* lst;                // 9 blocks of nl: pos2 xyz, angle1v xyz, angle2v xyz
    float* lsf;                 // 3 blocks of nl: strain, maxStrain, strainOffset
    uint8_t* lfl;
    // collisions
    const int32_t* surf;        // surface voxel ids (sorted)
    const int16_t* ijk;         // lattice indices, 3 blocks of nv
    const uint32_t* reach;      // kReachWords per voxel
    int32_t* ccount;            // per voxel
    float* cforce;              // 3*kContactCap per voxel
    int32_t* hash_head;         // 2 tables of hash_size
    int32_t* hash_next;         // per voxel
    float4* cpos;               // per hashed voxel: position rounded to float, float base size (broadphase only)
    float inv_cell;             // 1 / cell_size, for the float cell index
    // VX3 extras
    const double* cilia;        // BaseCiliaForce, 3 blocks of nv (SF_CILIA)
    const MathTree* ffield;     // x, y, z force-field formulas (SF_FFIELD)
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
    int32_t pad_ctl;
    double com[3], com_hist[2][3];
    double recent_angle;
    MathTree stop;
};

struct Item {
    int32_t sim, begin, end, seq;
};

}  // namespace dev
}  // namespace gvx
