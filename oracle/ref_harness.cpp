// Test infrastructure only: a small driver around the reference's own CPU
// Voxelyze (CVX_Sim + CVoxelyze), compiled together with the reference
// sources by oracle/Makefile into oracle/_ref/libvxref.so.  Nothing in the
// product links or loads this; tests and bench.py use it as the checker and
// as the CPU baseline where the reference sources are available.
//
// It reproduces the VX3 step-driver semantics around CVoxelyze::doTimeStep
// (Voxelyze3/src/old/Voxelyze.cpp:251-284):
//   * per-voxel temperature T_v = A*sin(2*pi_f*(t/P + phase_v)), clamped to
//     <= 0 unless expansion is enabled, applied before each step
//     (Voxelyze3/src/VX3/VX3_VoxelyzeKernel.cu:625-650, :240);
//   * OptimalDt = recommendedTimeStep() once, after the first temperature
//     update; dt = float(DtFrac*OptimalDt)  (VX3_VoxelyzeKernel.cu:244-254);
//   * currentTime is a double accumulating the float dt (:352).
// The CPU path's own OptimalDt (Voxelyze3/src/old/Voxelyze.cpp:286-311) is
// computed in float; that value is used.
#include "VX_Sim.h"
#include "VX_Environment.h"
#include "VX_Object.h"
#include "XML_Rip.h"
#include "Voxelyze.h"
#include "VX_Voxel.h"
#include "VX_Link.h"
#include "VX_MaterialVoxel.h"
#include "VX_MaterialLink.h"
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {
struct RefSim {
    CVX_Environment env;
    CVX_Object obj;
    CVX_Sim sim;
    double t = 0.0;
    float optimal_dt = 0.0f;
    bool have_dt = false;
    int expansion = 0;
    int diverged = 0;
    long steps = 0;
    std::map<CVX_Voxel*, int> vindex;
    std::map<CVX_MaterialVoxel*, int> mindex;
    std::vector<CVX_MaterialLink*> linkmats;
};
}

extern "C" {

void* vxref_load(const char* merged_vxa, int enable_collision, int enable_expansion,
                 float bounding_radius, float watch_distance) {
    RefSim* r = new RefSim();
    r->env.pObj = &r->obj;
    r->sim.pEnv = &r->env;
    std::string txt(merged_vxa);
    CXML_Rip xml;
    xml.fromXMLText(&txt);
    std::string msg;
    r->sim.ReadVXA(&xml, &msg);
    r->sim.Import(NULL, NULL, &msg);
    r->expansion = enable_expansion;
    r->sim.Vx.boundingRadius = bounding_radius;
    r->sim.Vx.watchDistance = watch_distance;
    r->sim.Vx.enableCollisions(enable_collision != 0);
    for (int i = 0; i < r->sim.Vx.voxelCount(); i++) r->vindex[r->sim.Vx.voxel(i)] = i;
    for (int i = 0; i < (int)r->sim.Vx.voxelMats.size(); i++) r->mindex[r->sim.Vx.voxelMats[i]] = i;
    for (auto* m : r->sim.Vx.linkMats) r->linkmats.push_back(m);
    return r;
}

void vxref_free(void* h) { delete (RefSim*)h; }

// counts: [nvox, nlink, nvoxmat, nlinkmat]
void vxref_counts(void* h, int* out) {
    RefSim* r = (RefSim*)h;
    out[0] = r->sim.Vx.voxelCount();
    out[1] = r->sim.Vx.linkCount();
    out[2] = (int)r->sim.Vx.voxelMats.size();
    out[3] = (int)r->linkmats.size();
}

// env: [voxSize, DtFrac, TempAmplitude, TempPeriod, VaryTempEnabled, TempEnabled, gravity multiplier, floor, collisions]
void vxref_env(void* h, double* out) {
    RefSim* r = (RefSim*)h;
    out[0] = r->sim.Vx.voxSize;
    out[1] = r->sim.DtFrac;
    out[2] = r->env.GetTempAmplitude();
    out[3] = r->env.GetTempPeriod();
    out[4] = r->env.IsTempVaryEnabled() ? 1 : 0;
    out[5] = r->env.IsTempEnabled() ? 1 : 0;
    out[6] = r->sim.Vx.gravity();
    out[7] = r->sim.Vx.isFloorEnabled() ? 1 : 0;
    out[8] = r->sim.Vx.isCollisionsEnabled() ? 1 : 0;
}

// per voxel-material float constants (18 floats each) + nomSize (double)
void vxref_voxmats(void* h, float* f, double* nom) {
    RefSim* r = (RefSim*)h;
    int k = 0;
    for (auto* m : r->sim.Vx.voxelMats) {
        float v[18] = {m->E, m->nu, m->rho, m->alphaCTE, m->muStatic, m->muKinetic,
                       m->zetaInternal, m->zetaGlobal, m->zetaCollision, m->_eHat,
                       m->_mass, m->_massInverse, m->_sqrtMass, m->_momentInertia,
                       m->_momentInertiaInverse, m->_2xSqMxExS, m->_2xSqIxExSxSxS, m->gravMult};
        memcpy(f + 18 * k, v, sizeof(v));
        nom[k] = m->nomSize;
        k++;
    }
}

// per link-material: [vox1 idx, vox2 idx] + 20 floats
void vxref_linkmats(void* h, int* idx, float* f) {
    RefSim* r = (RefSim*)h;
    int k = 0;
    for (auto* m : r->linkmats) {
        idx[2 * k] = r->mindex[m->vox1Mat];
        idx[2 * k + 1] = r->mindex[m->vox2Mat];
        float v[20] = {m->E, m->nu, m->_eHat, m->_a1, m->_a2, m->_b1, m->_b2, m->_b3,
                       m->_sqA1, m->_sqA2xIp, m->_sqB1, m->_sqB2xFMp, m->_sqB3xIp,
                       m->sigmaYield, m->sigmaFail, m->epsilonYield, m->epsilonFail,
                       m->linear ? 1.0f : 0.0f, (float)m->nomSize, m->rho};
        memcpy(f + 20 * k, v, sizeof(v));
        k++;
    }
}

// topology: voxels [ix,iy,iz,mat] ; links [neg, pos, axis, linkmat]
void vxref_topology(void* h, int* vox, int* lnk, double* phase) {
    RefSim* r = (RefSim*)h;
    for (int i = 0; i < r->sim.Vx.voxelCount(); i++) {
        CVX_Voxel* v = r->sim.Vx.voxel(i);
        vox[4 * i] = v->ix; vox[4 * i + 1] = v->iy; vox[4 * i + 2] = v->iz;
        vox[4 * i + 3] = r->mindex[v->mat];
        phase[i] = v->phaseOffset;
    }
    for (int i = 0; i < r->sim.Vx.linkCount(); i++) {
        CVX_Link* l = r->sim.Vx.link(i);
        lnk[4 * i] = r->vindex[l->pVNeg];
        lnk[4 * i + 1] = r->vindex[l->pVPos];
        lnk[4 * i + 2] = (int)l->axis;
        int lm = -1;
        for (int k = 0; k < (int)r->linkmats.size(); k++) if (r->linkmats[k] == l->mat) lm = k;
        lnk[4 * i + 3] = lm;
    }
}

// externals: per voxel [dofFixed] + 12 doubles (force3, moment3, translate3, rotate3)
void vxref_externals(void* h, int* dof, double* vals) {
    RefSim* r = (RefSim*)h;
    for (int i = 0; i < r->sim.Vx.voxelCount(); i++) {
        CVX_Voxel* v = r->sim.Vx.voxel(i);
        dof[i] = 0;
        for (int k = 0; k < 12; k++) vals[12 * i + k] = 0.0;
        if (!v->externalExists()) continue;
        CVX_External* e = v->external();
        dof[i] = e->dofFixed;
        for (int k = 0; k < 3; k++) {
            vals[12 * i + k] = e->extForce[k];
            vals[12 * i + 3 + k] = e->extMoment[k];
            vals[12 * i + 6 + k] = e->extTranslation[k];
            vals[12 * i + 9 + k] = e->extRotation[k];
        }
    }
}

// Fixes / forces one voxel through the reference's own CVX_External API (VX_External.cpp:53-66).
void vxref_set_external(void* h, int voxel, int dof, const float* force, const float* moment, const double* translate,
                        const double* rotate) {
    RefSim* r = (RefSim*)h;
    CVX_External* e = r->sim.Vx.voxel(voxel)->external();
    const double disp[6] = {translate[0], translate[1], translate[2], rotate[0], rotate[1], rotate[2]};
    for (int k = 0; k < 6; k++) if (dof & (1 << k)) e->setDisplacement((dofComponent)(1 << k), disp[k]);
    e->addForce(Vec3D<float>(force[0], force[1], force[2]));
    e->addMoment(Vec3D<float>(moment[0], moment[1], moment[2]));
}

// Advance n steps with VX3 step-driver semantics.  Returns steps done; stops at divergence.
int vxref_step(void* h, int n) {
    RefSim* r = (RefSim*)h;
    CVoxelyze& Vx = r->sim.Vx;
    int done = 0;
    for (int s = 0; s < n && !r->diverged; s++) {
        if (r->env.IsTempVaryEnabled() && r->env.GetTempPeriod() > 0) {
            for (int i = 0; i < Vx.voxelCount(); i++) {
                CVX_Voxel* v = Vx.voxel(i);
                double T = r->env.GetTempAmplitude() * sin(2 * 3.1415926f * (r->t / r->env.GetTempPeriod() + v->phaseOffset));
                if (!r->expansion && T > 0) T = 0;
                v->setTemperature((float)T);
            }
        }
        if (!r->have_dt) {
            r->optimal_dt = Vx.recommendedTimeStep();
            if (r->optimal_dt < 1e-10f) r->optimal_dt = 1e-10f;
            r->have_dt = true;
        }
        float dt = (float)(r->sim.DtFrac * (double)r->optimal_dt);
        if (!Vx.doTimeStep(dt)) { r->diverged = 1; break; }
        r->t += dt;
        r->steps++;
        done++;
    }
    return done;
}

// scalars: [t, optimal_dt, dt, diverged, steps]
void vxref_scalars(void* h, double* out) {
    RefSim* r = (RefSim*)h;
    out[0] = r->t;
    out[1] = r->optimal_dt;
    out[2] = (float)(r->sim.DtFrac * (double)r->optimal_dt);
    out[3] = r->diverged;
    out[4] = (double)r->steps;
}

// voxel state: pos3 linMom3 orient4 angMom3 (13 doubles), temp, pStrain3 (floats), boolStates (int)
void vxref_voxel_state(void* h, double* d13, float* f4, int* flags) {
    RefSim* r = (RefSim*)h;
    for (int i = 0; i < r->sim.Vx.voxelCount(); i++) {
        CVX_Voxel* v = r->sim.Vx.voxel(i);
        double* d = d13 + 13 * i;
        d[0] = v->pos.x; d[1] = v->pos.y; d[2] = v->pos.z;
        d[3] = v->linMom.x; d[4] = v->linMom.y; d[5] = v->linMom.z;
        d[6] = v->orient.w; d[7] = v->orient.x; d[8] = v->orient.y; d[9] = v->orient.z;
        d[10] = v->angMom.x; d[11] = v->angMom.y; d[12] = v->angMom.z;
        f4[4 * i] = v->temp;
        f4[4 * i + 1] = v->pStrain.x; f4[4 * i + 2] = v->pStrain.y; f4[4 * i + 3] = v->pStrain.z;
        flags[i] = v->boolStates;
    }
}

// link state: pos2 angle1v angle2v (9 doubles), forceNeg forcePos momentNeg momentPos (12 doubles),
// restLength (1 double); floats: strain maxStrain strainOffset stress A_t strainSum; ints: smallAngle, boolStates
void vxref_link_state(void* h, double* d22, float* f6, int* i2) {
    RefSim* r = (RefSim*)h;
    for (int i = 0; i < r->sim.Vx.linkCount(); i++) {
        CVX_Link* l = r->sim.Vx.link(i);
        double* d = d22 + 22 * i;
        Vec3D<double> vs[7] = {l->pos2, l->angle1v, l->angle2v, l->forceNeg, l->forcePos, l->momentNeg, l->momentPos};
        for (int k = 0; k < 7; k++) { d[3 * k] = vs[k].x; d[3 * k + 1] = vs[k].y; d[3 * k + 2] = vs[k].z; }
        d[21] = l->currentRestLength;
        float* f = f6 + 6 * i;
        f[0] = l->strain; f[1] = l->maxStrain; f[2] = l->strainOffset; f[3] = l->_stress;
        f[4] = l->currentTransverseArea; f[5] = l->currentTransverseStrainSum;
        i2[2 * i] = l->smallAngle ? 1 : 0;
        i2[2 * i + 1] = l->boolStates;
    }
}

// collision pairs currently tracked by the CPU path (pairs [i,j]); returns the count
int vxref_collisions(void* h, int* pairs, int max_pairs) {
    RefSim* r = (RefSim*)h;
    const std::vector<CVX_Collision*>* cl = r->sim.Vx.collisionList();
    int n = (int)cl->size();
    for (int i = 0; i < n && i < max_pairs; i++) {
        pairs[2 * i] = r->vindex[(*cl)[i]->voxel1()];
        pairs[2 * i + 1] = r->vindex[(*cl)[i]->voxel2()];
    }
    return n;
}

}  // extern "C"
