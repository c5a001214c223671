/* CPU oracle for the Voxelyze soft-body step: TEST INFRASTRUCTURE ONLY.
 *
 * A sequential C restatement of the reference's CPU Voxelyze step
 * (Voxelyze3/src/old/{Voxelyze,VX_Voxel,VX_Link,VX_Material*,VX_Collision,
 * VX_External}.cpp) with the VX3 step-driver semantics (per-voxel
 * temperature actuation, dt = float(DtFrac*OptimalDt), double time).  It is
 * pinned against the reference itself (oracle/_ref, built from the reference
 * sources by oracle/Makefile) and against the golden vectors under
 * tests/golden/.  Only tests, __graft_entry__.smoke() and bench.py's CPU
 * baseline load it; the product never links, loads or calls it.
 */
#ifndef VX_ORACLE_H
#define VX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VXO_MAX_DATA 16

/* One palette material as the VXA reader leaves it (CVXC_Material after
 * CVX_Sim::CopyMat, Voxelyze3/src/VXA/VX_Sim.cpp:368-420): values already
 * converted to float where the reference stores float. */
typedef struct {
    int model;              /* 0 linear, 1 linear+fail, 2 bilinear, 3 data points */
    float E, plastic_mod, yield_stress, fail_stress;
    int ndata;              /* model 3 only */
    float strain_data[VXO_MAX_DATA], stress_data[VXO_MAX_DATA];
    float rho, nu, cte, mu_static, mu_kinetic;
    float zeta_internal, zeta_global, zeta_collision;
    int is_measured;
} vxo_material;

typedef struct {
    double vox_size;        /* Lattice_Dim */
    double dt_frac;
    float gravity_mult;     /* CVoxelyze::grav, in g */
    int floor_enabled;
    int collisions_enabled;
    float bounding_radius, watch_distance;
    int vary_temp;          /* per-step actuation on */
    double temp_amplitude, temp_period;
    int enable_expansion;
    float initial_temp;     /* temperature every voxel starts at */
} vxo_env;

/* External influence on one voxel (CVX_External). */
typedef struct {
    int voxel;
    int dof_fixed;          /* bit0..2 translate xyz, bit3..5 rotate xyz */
    float force[3], moment[3];
    double translate[3], rotate[3];
} vxo_external;

typedef struct vxo_sim vxo_sim;

/* Build a simulation.  voxels[4*i] = ix, iy, iz, material index (0-based into
 * mats); voxels are added in the given order (structure order). */
vxo_sim* vxo_create(const vxo_env* env, const vxo_material* mats, int nmat,
                    const int* voxels, const double* phase, int nvox,
                    const vxo_external* ext, int next);
void vxo_free(vxo_sim* s);

/* Advance n steps; returns the steps taken (fewer when the run diverged). */
int vxo_step(vxo_sim* s, int n);

void vxo_counts(const vxo_sim* s, int* out4);        /* nvox, nlink, nvoxmat, nlinkmat */
void vxo_scalars(const vxo_sim* s, double* out5);    /* t, optimal_dt, dt, diverged, steps */
void vxo_voxel_state(const vxo_sim* s, double* d13, float* f4, int* flags);
void vxo_link_state(const vxo_sim* s, double* d22, float* f6, int* i2);
void vxo_topology(const vxo_sim* s, int* vox4, int* lnk4);
void vxo_voxmats(const vxo_sim* s, float* f18, double* nom);
void vxo_linkmats(const vxo_sim* s, int* idx2, float* f20);
/* mass-weighted centre of mass over measured voxels (VX3 semantics) */
void vxo_center_of_mass(const vxo_sim* s, double* out3);

#ifdef __cplusplus
}
#endif
#endif
