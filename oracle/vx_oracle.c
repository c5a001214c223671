/* CPU oracle for the Voxelyze soft-body step: TEST INFRASTRUCTURE ONLY.
 *
 * Sequential C restatement of the reference's CPU Voxelyze step.  Every
 * function cites the reference file:line it follows; paths are relative to the
 * reference project root.  Floating-point expressions keep the reference's
 * operand types (float vs double) and association order, and the build
 * disables contraction (-ffp-contract=off), so results are bit-identical to the
 * reference compiled the same way, up to libm differences between platforms.
 *
 * Only tests, __graft_entry__.smoke() and bench.py's CPU baseline use this
 * file.  The product path never links, loads or calls it.
 */
#include "vx_oracle.h"
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* constants: Voxelyze3/src/old/types.h:57-59, Quat3D.h:21-31               */
#define HYSTERESIS_FACTOR 1.2f
#define SA_BOND_BEND_RAD 0.05f
#define SA_BOND_EXT_PERC 0.50f
#define Q_PI 3.14159265358979
#define DISCARD_ANGLE_RAD 1e-7
#define SMALL_ANGLE_RAD 1.732e-2
#define DBL_EPSILONx24 5.328e-15
#define SLTHRESH_ACOS2SQRT 2.4e-3
#define ENVELOPE_RADIUS 0.625f            /* VX_Collision.cpp:15 */

/* voxel flag bits, Voxelyze3/src/old/VX_Voxel.h:145-150 */
#define VF_INTERIOR 2                     /* named SURFACE in the reference; set when all 6 links exist */
#define VF_FLOOR 4
#define VF_STATIC 8
#define VF_COLLIDE 32
#define LF_LOCAL_VEL_VALID 1              /* VX_Link.h:73-75 */

typedef struct { double x, y, z; } v3;
typedef struct { float x, y, z; } v3f;
typedef struct { double w, x, y, z; } qd;

static v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
/* Vec3D::operator*(f): (f*x, f*y, f*z)  (Vec3D.h:57,67) */
static v3 vscale(v3 a, double f) { return V(f * a.x, f * a.y, f * a.z); }
static double vlen2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static qd Q(double w, double x, double y, double z) { qd r = {w, x, y, z}; return r; }
static qd qident(void) { return Q(1, 0, 0, 0); }

/* Quat3D::operator*(Quat3D)  Quat3D.h:87 */
static qd qmul(qd a, qd f) {
    return Q(a.w * f.w - a.x * f.x - a.y * f.y - a.z * f.z,
             a.w * f.x + a.x * f.w + a.y * f.z - a.z * f.y,
             a.w * f.y - a.x * f.z + a.y * f.w + a.z * f.x,
             a.w * f.z + a.x * f.y - a.y * f.x + a.z * f.w);
}
static qd qconj(qd a) { return Q(a.w, -a.x, -a.y, -a.z); }

/* Quat3D::RotateVec3D  Quat3D.h:174-181 */
static v3 qrot(qd q, v3 f) {
    double fx = f.x, fy = f.y, fz = f.z;
    double tw = fx * q.x + fy * q.y + fz * q.z;
    double tx = fx * q.w - fy * q.z + fz * q.y;
    double ty = fx * q.z + fy * q.w - fz * q.x;
    double tz = -fx * q.y + fy * q.x + fz * q.w;
    return V(q.w * tx + q.x * tw + q.y * tz - q.z * ty,
             q.w * ty - q.x * tz + q.y * tw + q.z * tx,
             q.w * tz + q.x * ty - q.y * tx + q.z * tw);
}
/* Quat3D::RotateVec3DInv  Quat3D.h:192-199 */
static v3 qrotinv(qd q, v3 f) {
    double fx = f.x, fy = f.y, fz = f.z;
    double tw = q.x * fx + q.y * fy + q.z * fz;
    double tx = q.w * fx - q.y * fz + q.z * fy;
    double ty = q.w * fy + q.x * fz - q.z * fx;
    double tz = q.w * fz - q.x * fy + q.y * fx;
    return V(tw * q.x + tx * q.w + ty * q.z - tz * q.y,
             tw * q.y - tx * q.z + ty * q.w + tz * q.x,
             tw * q.z + tx * q.y - ty * q.x + tz * q.w);
}
/* Quat3D::ToRotationVector  Quat3D.h:121-126 */
static v3 q_to_rotvec(qd q) {
    if (q.w >= 1.0 || q.w <= -1.0) return V(0, 0, 0);
    double sl = 1.0 - q.w * q.w;
    if (sl < SLTHRESH_ACOS2SQRT) {
        double s = sqrt((2 - 2 * q.w) / sl);
        return V((q.x * 2.0) * s, (q.y * 2.0) * s, (q.z * 2.0) * s);
    } else {
        double a = acos(q.w);
        double inv = 1.0 / sqrt(sl);     /* Vec3D::operator/ multiplies by 1/f (Vec3D.h:69) */
        return V(((q.x * 2.0) * a) * inv, ((q.y * 2.0) * a) * inv, ((q.z * 2.0) * a) * inv);
    }
}
/* Quat3D::FromRotationVector  Quat3D.h:128-143 */
static qd q_from_rotvec(v3 vin) {
    v3 th = V(0.5 * vin.x, 0.5 * vin.y, 0.5 * vin.z);   /* VecIn/2 == VecIn*(1.0/2) */
    double m2 = th.x * th.x + th.y * th.y + th.z * th.z;
    double w, s;
    if (m2 * m2 < DBL_EPSILONx24) {
        w = 1.0 - 0.5 * m2;
        s = 1.0 - m2 / 6.0;
    } else {
        double m = sqrt(m2);
        w = cos(m);
        s = sin(m) / m;
    }
    return Q(w, th.x * s, th.y * s, th.z * s);
}
/* Quat3D::FromAngleToPosX  Quat3D.h:145-170 (caller passes the current value, returned unchanged for a zero vector) */
static qd q_from_angle_to_posx(qd cur, v3 r) {
    if (r.x == 0 && r.y == 0 && r.z == 0) return cur;
    double yox = r.y / r.x, zox = r.z / r.x;
    if (yox < SMALL_ANGLE_RAD && yox > -SMALL_ANGLE_RAD && zox < SMALL_ANGLE_RAD && zox > -SMALL_ANGLE_RAD) {
        double y = 0.5 * zox, z = -0.5 * yox;
        return Q(1 + 0.5 * (-y * y - z * z), 0, y, z);
    }
    double l = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    v3 n = r;
    if (l > 0) { double li = 1.0 / l; n.x *= li; n.y *= li; n.z *= li; }
    double theta = acos(n.x);
    if (theta > Q_PI - DISCARD_ANGLE_RAD) return Q(0, 0, 1, 0);
    double ami = 1.0 / sqrt(n.z * n.z + n.y * n.y);
    double a = 0.5 * theta;
    double s = sin(a);
    return Q(cos(a), 0, n.z * ami * s, -n.y * ami * s);
}

/* CVX_Link::toAxisX / toAxisOriginal  Voxelyze3/src/old/VX_Link.h:106-111 */
static v3 to_axis_x(int axis, v3 v) {
    if (axis == 1) return V(v.y, -v.x, v.z);
    if (axis == 2) return V(v.z, v.y, -v.x);
    return v;
}
static qd q_to_axis_x(int axis, qd q) {
    if (axis == 1) return Q(q.w, q.y, -q.x, q.z);
    if (axis == 2) return Q(q.w, q.z, q.y, -q.x);
    return q;
}
static v3 to_axis_orig(int axis, v3 v) {
    if (axis == 1) return V(-v.y, v.x, v.z);
    if (axis == 2) return V(-v.z, v.y, v.x);
    return v;
}

/* ------------------------------------------------------------------------ */
/* Materials: Voxelyze3/src/old/VX_Material.cpp, VX_MaterialVoxel.cpp,      */
/* VX_MaterialLink.cpp                                                      */
typedef struct {
    int linear;
    float E, nu, rho, cte, mus, muk, zi, zg, zc, eHat;
    float sigmaYield, sigmaFail, epsYield, epsFail;
    int n;                                  /* data points including the (0,0) point */
    float strain[VXO_MAX_DATA + 2], stress[VXO_MAX_DATA + 2];
    double nom;
    float grav;
    float mass, massInv, sqrtMass, I, Iinv, c2m, c2i;
    int is_measured;
    /* link-only */
    int v1, v2;
    float a1, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp;
} mat_t;

/* CVX_Material::updateDerived + CVX_MaterialVoxel::updateDerived
 * (VX_Material.cpp:542-549, VX_MaterialVoxel.cpp:57-79) */
static void mat_update_derived(mat_t* m) {
    m->eHat = m->E / ((1 - 2 * m->nu) * (1 + m->nu));
    double volume = m->nom * m->nom * m->nom;
    m->mass = (float)(volume * m->rho);
    m->I = (float)(m->mass * m->nom * m->nom / 6.0f);
    if (volume == 0 || m->mass == 0 || m->I == 0) {
        m->massInv = m->sqrtMass = m->Iinv = m->c2m = m->c2i = 0.0f;
        return;
    }
    m->massInv = 1.0f / m->mass;
    m->sqrtMass = sqrtf(m->mass);
    m->Iinv = 1.0f / m->I;
    m->c2m = (float)(2.0f * sqrt(m->mass * m->E * m->nom));
    m->c2i = (float)(2.0f * sqrt(m->I * m->E * m->nom * m->nom * m->nom));
}
/* CVX_MaterialLink::updateDerived  VX_MaterialLink.cpp:121-141 */
static void linkmat_update_derived(mat_t* m) {
    mat_update_derived(m);
    float L = (float)m->nom;
    m->a1 = m->E * L;
    m->a2 = m->E * L * L * L / (12.0f * (1 + m->nu));
    m->b1 = m->E * L;
    m->b2 = m->E * L * L / 2.0f;
    m->b3 = m->E * L * L * L / 6.0f;
    m->sqA1 = sqrtf(m->a1);
    m->sqA2xIp = sqrtf(m->a2 * L * L / 6.0f);
    m->sqB1 = sqrtf(m->b1);
    m->sqB2xFMp = sqrtf(m->b2 * L / 2.0f);
    m->sqB3xIp = sqrtf(m->b3 * L * L / 6.0f);
}

/* CVX_Material::setModelLinear  VX_Material.cpp:372-401 */
static void mat_set_linear(mat_t* m, float E, float failStress) {
    if (E <= 0) return;
    if (failStress != -1.0f && failStress <= 0) return;
    float tmpfail = failStress;
    if (tmpfail == -1) tmpfail = 1000000;
    float tmpfailStrain = tmpfail / E;
    m->n = 2;
    m->strain[0] = 0; m->stress[0] = 0;
    m->strain[1] = tmpfailStrain; m->stress[1] = tmpfail;
    m->linear = 1;
    m->E = E;
    m->sigmaYield = failStress;
    m->sigmaFail = failStress;
    m->epsYield = (failStress == -1) ? -1 : tmpfailStrain;
    m->epsFail = (failStress == -1) ? -1 : tmpfailStrain;
}

/* CVX_Material::setYieldFromData  VX_Material.cpp:454-487 */
static void mat_yield_from_data(mat_t* m, float pct) {
    m->sigmaYield = -1.0f;
    m->epsYield = -1.0f;
    float oM = m->E;
    float oB = (-pct / 100 * oM);
    int dp = m->n - 1;
    for (int i = 1; i < dp - 1; i++) {
        float x1 = m->strain[i], x2 = m->strain[i + 1], y1 = m->stress[i], y2 = m->stress[i + 1];
        float tM = (y2 - y1) / (x2 - x1);
        float tB = y1 - tM * x1;
        if (oM != tM) {
            float xi = (tB - oB) / (oM - tM);
            if (xi > x1 && xi < x2) {
                float p = (xi - x1) / (x2 - x1);
                m->sigmaYield = y1 + p * (y2 - y1);
                m->epsYield = xi;
                return;
            }
        }
    }
    m->sigmaYield = m->sigmaFail;
    m->epsYield = m->epsFail;
}

/* CVX_Material::setModel  VX_Material.cpp:300-367 */
static int mat_set_model(mat_t* m, int count, const float* se, const float* ss) {
    if (*se == 0 && *ss == 0) { se++; ss++; count--; }
    if (count <= 0) return 0;
    if (*se <= 0 || *ss <= 0) return 0;
    float ts[VXO_MAX_DATA + 2], tt[VXO_MAX_DATA + 2];
    ts[0] = 0; tt[0] = 0;
    float sweepE = 0.0f, sweepS = 0.0f;
    for (int i = 0; i < count; i++) {
        float e = se[i], s = ss[i];
        if (e <= sweepE) return 0;
        if (i > 0 && (s - sweepS) / (e - sweepE) > tt[0] / ts[0]) return 0;
        sweepE = e; sweepS = s;
        ts[i + 1] = e; tt[i + 1] = s;
    }
    m->n = count + 1;
    for (int i = 0; i < m->n; i++) { m->strain[i] = ts[i]; m->stress[i] = tt[i]; }
    m->E = m->stress[1] / m->strain[1];
    m->sigmaFail = m->stress[m->n - 1];
    m->epsFail = m->strain[m->n - 1];
    m->linear = (count == 1);
    if (count == 1 || count == 2) { m->sigmaYield = m->stress[1]; m->epsYield = m->strain[1]; }
    else mat_yield_from_data(m, 0.2f);
    return 1;
}

/* CVX_Material::setModelBilinear  VX_Material.cpp:406-451 */
static void mat_set_bilinear(mat_t* m, float E, float pE, float ys, float fs) {
    if (E <= 0 || pE <= 0 || pE >= E || ys <= 0) return;
    if (fs != -1.0f && fs <= ys) return;
    float yieldStrain = ys / E;
    float tmpfs = fs;
    if (tmpfs == -1) tmpfs = 3 * ys;
    float tM = pE;
    float tB = ys - tM * yieldStrain;
    float tmpfailStrain = (tmpfs - tB) / tM;
    m->n = 3;
    m->strain[0] = 0; m->strain[1] = yieldStrain; m->strain[2] = tmpfailStrain;
    m->stress[0] = 0; m->stress[1] = ys; m->stress[2] = tmpfs;
    m->linear = 0;
    m->E = E;
    m->sigmaYield = ys;
    m->sigmaFail = fs;
    m->epsYield = yieldStrain;
    m->epsFail = fs == -1.0f ? -1.0f : tmpfailStrain;
}

static int mat_is_failed(const mat_t* m, float strain) { return m->epsFail != -1.0f && strain > m->epsFail; }

/* CVX_Material::stress  VX_Material.cpp:182-212 */
static float mat_stress(const mat_t* m, float strain, float tss, int forceLinear) {
    if (mat_is_failed(m, strain)) return 0.0f;
    if (strain <= m->strain[1] || m->linear || forceLinear) {
        if (m->nu == 0.0f) return m->E * strain;
        else return m->eHat * ((1 - m->nu) * strain + m->nu * tss);
    }
    int dc = m->n;
    for (int i = 2; i < dc; i++) {
        if (strain <= m->strain[i] || i == dc - 1) {
            float perc = (strain - m->strain[i - 1]) / (m->strain[i] - m->strain[i - 1]);
            float basic = m->stress[i - 1] + perc * (m->stress[i] - m->stress[i - 1]);
            if (m->nu == 0.0f) return basic;
            float mod = (m->stress[i] - m->stress[i - 1]) / (m->strain[i] - m->strain[i - 1]);
            float modHat = mod / ((1 - 2 * m->nu) * (1 + m->nu));
            float effS = basic / mod;
            float effT = tss * (effS / strain);
            return modHat * ((1 - m->nu) * effS + m->nu * effT);
        }
    }
    return 0.0f;
}
/* CVX_Material::strain  VX_Material.cpp:214-228 */
static float mat_strain_of(const mat_t* m, float stress) {
    if (stress <= m->stress[1] || m->linear) return stress / m->E;
    for (int i = 2; i < m->n; i++) {
        if (stress <= m->stress[i] || i == m->n - 1) {
            float p = (stress - m->stress[i - 1]) / (m->stress[i] - m->stress[i - 1]);
            return m->strain[i - 1] + p * (m->strain[i] - m->strain[i - 1]);
        }
    }
    return 0.0f;
}
/* CVX_Material::modulus  VX_Material.cpp:231-243 */
static float mat_modulus(const mat_t* m, float strain) {
    if (mat_is_failed(m, strain)) return 0.0f;
    if (strain <= m->strain[1] || m->linear) return m->E;
    for (int i = 2; i < m->n; i++)
        if (strain <= m->strain[i] || i == m->n - 1)
            return (m->stress[i] - m->stress[i - 1]) / (m->strain[i] - m->strain[i - 1]);
    return 0.0f;
}

/* Palette material -> CVX_MaterialVoxel: CVX_Material::CVX_Material(1e6, 1e3) (VX_Material.cpp:15-22, 71-90),
 * CVX_Sim::CopyMat (Voxelyze3/src/VXA/VX_Sim.cpp:368-420) and the damping setters
 * applied in CVX_Sim::Import (VX_Sim.cpp:80-83). */
static void vmat_from_palette(mat_t* m, const vxo_material* p, double nom, float grav) {
    memset(m, 0, sizeof(*m));
    m->nu = 0.0f; m->rho = 1.0f; m->cte = 0.0f; m->mus = 0.0f; m->muk = 0.0f;
    m->zi = 1.0f; m->zg = 0.0f; m->zc = 0.0f;
    /* CVoxelyze::addMaterial() builds CVX_MaterialVoxel(1e6, 1e3): a model setter that rejects
       its arguments leaves this linear 1e6 Pa model in place (VX_Material.cpp:15-22) */
    mat_set_linear(m, 1e6f, -1.0f);
    switch (p->model) {
    case 0: mat_set_linear(m, p->E, -1.0f); break;
    case 1: mat_set_linear(m, p->E, p->fail_stress); break;
    case 2: mat_set_bilinear(m, p->E, p->plastic_mod, p->yield_stress, p->fail_stress); break;
    case 3: mat_set_model(m, p->ndata, p->strain_data, p->stress_data); break;
    }
    float nu = p->nu;                                   /* setPoissonsRatio, VX_Material.cpp:489-495 */
    if (nu < 0) nu = 0;
    if (nu >= 0.5) nu = (float)(0.5 - FLT_EPSILON * 2);
    m->nu = nu;
    float rho = p->rho;                                 /* setDensity, :497-502 */
    if (rho <= 0) rho = FLT_MIN;
    m->rho = rho;
    m->cte = p->cte;
    m->mus = p->mu_static <= 0 ? 0 : p->mu_static;
    m->muk = p->mu_kinetic <= 0 ? 0 : p->mu_kinetic;
    m->zi = p->zeta_internal <= 0 ? 0 : p->zeta_internal;
    m->zg = p->zeta_global <= 0 ? 0 : p->zeta_global;
    m->zc = p->zeta_collision <= 0 ? 0 : p->zeta_collision;
    m->nom = nom;
    m->grav = grav;
    m->is_measured = p->is_measured;
    mat_update_derived(m);
}

/* CVX_MaterialLink::updateAll  VX_MaterialLink.cpp:45-119 */
static void linkmat_build(mat_t* lm, const mat_t* a, const mat_t* b, int ia, int ib) {
    memset(lm, 0, sizeof(*lm));
    lm->v1 = ia; lm->v2 = ib;
    lm->nom = 0.5 * (a->nom + b->nom);
    lm->rho = 0.5f * (a->rho + b->rho);
    lm->cte = 0.5f * (a->cte + b->cte);
    lm->mus = 0.5f * (a->mus + b->mus);
    lm->muk = 0.5f * (a->muk + b->muk);
    lm->zi = 0.5f * (a->zi + b->zi);
    lm->zg = 0.5f * (a->zg + b->zg);
    lm->zc = 0.5f * (a->zc + b->zc);
    float f1 = a->sigmaFail, f2 = b->sigmaFail, sf;
    if (f1 == -1.0f) sf = f2;
    else if (f2 == -1.0f) sf = f1;
    else sf = f1 < f2 ? f1 : f2;
    if (a->linear && b->linear) {
        mat_set_linear(lm, 2.0f * a->E * b->E / (a->E + b->E), sf);
    } else {
        float ns[2 * VXO_MAX_DATA + 4], ne[2 * VXO_MAX_DATA + 4];
        int cnt = 1;
        ns[0] = 0.0f; ne[0] = 0.0f;
        int i1 = 1, i2 = 1;
        while (i1 < a->n && i2 < b->n) {
            float s = FLT_MAX;
            if (i1 < a->n) s = a->strain[i1];
            if (i2 < b->n && b->strain[i2] < s) s = b->strain[i2];
            if (s == a->strain[i1]) i1++;
            if (s == b->strain[i2]) i2++;
            float m1 = mat_modulus(a, s - FLT_EPSILON);
            float m2 = mat_modulus(b, s - FLT_EPSILON);
            float tm = 2.0f * m1 * m2 / (m1 + m2);
            int last = cnt - 1;
            ne[cnt] = s;
            ns[cnt] = ns[last] + tm * (s - ne[last]);
            cnt++;
        }
        mat_set_model(lm, cnt, ne, ns);
        lm->sigmaFail = sf;
        lm->epsFail = sf == -1.0f ? -1.0f : mat_strain_of(lm, sf);
    }
    if (a->nu == 0 && b->nu == 0) lm->nu = 0;
    else {
        float tmpEHat = 2 * a->eHat * b->eHat / (a->eHat + b->eHat);
        float tmpE = lm->E;
        float c2 = (float)((tmpEHat - tmpE) / (2 * tmpEHat) + 0.0625);
        lm->nu = (float)(sqrtf(c2) - 0.25);
    }
    linkmat_update_derived(lm);
}

/* ------------------------------------------------------------------------ */
typedef struct {
    int ix, iy, iz, mat, links[6], ext, flags;
    v3 pos, linMom, angMom;
    qd orient;
    float temp, prevDt;
    v3f pStrain;
    int pStrainInvalid;
    double phase;
    /* collision bookkeeping (VX_Voxel.h:193-195) */
    v3f lastColWatch;
    int* nearby; int n_nearby;
    int* colWatch; int n_col, cap_col;
} vox_t;

typedef struct {
    int neg, pos, axis, mat, flags, smallAngle;
    v3 fN, fP, mN, mP, pos2, a1v, a2v;
    qd angle1, angle2;
    float strain, maxStrain, strainOffset, stress, strainRatio, A, tss;
    double restLen;
} link_t;

typedef struct {
    vxo_external e;
    qd rotQ;
} ext_t;

typedef struct { int v1, v2; float k, c; v3f force; } col_t;

struct vxo_sim {
    vxo_env env;
    mat_t* vm; int nvm;
    mat_t* lm; int nlm, caplm;
    vox_t* v; int nv;
    link_t* l; int nl, capl;
    ext_t* ext; int next;
    int minx, miny, minz, dx, dy, dz;
    int* grid;                      /* voxel index per lattice cell, -1 empty */
    int* lgrid[3];                  /* link index per link-lattice cell */
    double t; float optdt; int have_dt; int diverged; long steps;
    /* collisions, Voxelyze.h:181-182 */
    col_t* col; int ncol, capcol;
    int collisionsStale, nearbyStale;
};

static int cell(const vxo_sim* s, int x, int y, int z) {
    x -= s->minx; y -= s->miny; z -= s->minz;
    if (x < 0 || y < 0 || z < 0 || x >= s->dx || y >= s->dy || z >= s->dz) return -1;
    return (z * s->dy + y) * s->dx + x;
}
static int lcell(const vxo_sim* s, int x, int y, int z) {   /* link lattice is one larger on the low side */
    x -= s->minx - 1; y -= s->miny - 1; z -= s->minz - 1;
    if (x < 0 || y < 0 || z < 0 || x >= s->dx + 1 || y >= s->dy + 1 || z >= s->dz + 1) return -1;
    return (z * (s->dy + 1) + y) * (s->dx + 1) + x;
}
static int voxel_at(const vxo_sim* s, int x, int y, int z) { int c = cell(s, x, y, z); return c < 0 ? -1 : s->grid[c]; }

static const int DOFF[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
static int is_neg_dir(int d) { return d % 2 == 1; }
static int opposite(int d) { return d - d % 2 + (d + 1) % 2; }

/* CVX_Voxel::baseSize(axis)  VX_Voxel.h:91 (extScale is 1 for palette materials) */
static double base_size(const vxo_sim* s, const vox_t* v) {
    const mat_t* m = &s->vm[v->mat];
    return (m->nom * 1.0) * (1 + v->temp * m->cte);
}
/* CVX_Voxel::baseSizeAverage  VX_Voxel.h:92 */
static double base_size_avg(const vxo_sim* s, const vox_t* v) {
    double b = base_size(s, v);
    return (b + b + b) / 3.0f;
}
/* CVX_Link::updateRestLength  VX_Link.cpp:131-134 */
static void link_update_rest(vxo_sim* s, link_t* l) {
    l->restLen = 0.5 * (base_size(s, &s->v[l->neg]) + base_size(s, &s->v[l->pos]));
}
/* CVX_Link::axialStrain(positiveEnd)  VX_Link.cpp:115-118 */
static float link_axial_strain(const link_t* l, int positiveEnd) {
    return positiveEnd ? 2.0f * l->strain * l->strainRatio / (1.0f + l->strainRatio)
                       : 2.0f * l->strain / (1.0f + l->strainRatio);
}
/* CVX_Voxel::strain(true)  VX_Voxel.cpp:299-333 */
static v3f voxel_poisson_strain_calc(const vxo_sim* s, const vox_t* v) {
    float st[3] = {0, 0, 0};
    int nb[3] = {0, 0, 0};
    int tension[3] = {0, 0, 0};
    for (int i = 0; i < 6; i++) {
        if (v->links[i] >= 0) {
            int ax = i / 2;
            st[ax] += link_axial_strain(&s->l[v->links[i]], is_neg_dir(i));
            nb[ax]++;
        }
    }
    const ext_t* e = v->ext >= 0 ? &s->ext[v->ext] : NULL;
    for (int i = 0; i < 3; i++) {
        if (nb[i] == 2) st[i] *= 0.5f;
        tension[i] = (nb[i] == 2) || (e && (nb[i] == 1 && ((e->e.dof_fixed & (1 << i)) || e->e.force[i] != 0)));
    }
    if (!(tension[0] && tension[1] && tension[2])) {
        float add = 0;
        for (int i = 0; i < 3; i++) if (tension[i]) add += st[i];
        float value = powf(1.0f + add, -s->vm[v->mat].nu) - 1.0f;
        for (int i = 0; i < 3; i++) if (!tension[i]) st[i] = value;
    }
    v3f r = {st[0], st[1], st[2]};
    return r;
}
/* CVX_Voxel::poissonsStrain  VX_Voxel.cpp:335-342 */
static v3f voxel_pstrain(vxo_sim* s, vox_t* v) {
    if (v->pStrainInvalid) { v->pStrain = voxel_poisson_strain_calc(s, v); v->pStrainInvalid = 0; }
    return v->pStrain;
}
/* CVX_Voxel::transverseStrainSum  VX_Voxel.cpp:345-358 */
static float voxel_tss(vxo_sim* s, vox_t* v, int axis) {
    if (s->vm[v->mat].nu == 0) return 0;
    v3f p = voxel_pstrain(s, v);
    if (axis == 0) return p.y + p.z;
    if (axis == 1) return p.x + p.z;
    return p.x + p.y;
}
/* CVX_Voxel::transverseArea  VX_Voxel.cpp:360-373 */
static float voxel_tarea(vxo_sim* s, vox_t* v, int axis) {
    float size = (float)s->vm[v->mat].nom;
    if (s->vm[v->mat].nu == 0) return size * size;
    v3f pf = voxel_pstrain(s, v);
    double px = pf.x, py = pf.y, pz = pf.z;
    if (axis == 0) return (float)(size * size * (1 + py) * (1 + pz));
    if (axis == 1) return (float)(size * size * (1 + px) * (1 + pz));
    return (float)(size * size * (1 + px) * (1 + py));
}
/* CVX_Link::updateTransverseInfo  VX_Link.cpp:136-141 */
static void link_update_transverse(vxo_sim* s, link_t* l) {
    vox_t* n = &s->v[l->neg]; vox_t* p = &s->v[l->pos];
    l->A = 0.5f * (voxel_tarea(s, n, l->axis) + voxel_tarea(s, p, l->axis));
    l->tss = 0.5f * (voxel_tss(s, n, l->axis) + voxel_tss(s, p, l->axis));
}
/* CVX_Link::reset  VX_Link.cpp:56-70 */
static void link_reset(vxo_sim* s, link_t* l) {
    l->pos2 = l->a1v = l->a2v = V(0, 0, 0);
    l->angle1 = l->angle2 = qident();
    l->fN = l->fP = l->mN = l->mP = V(0, 0, 0);
    l->strain = l->maxStrain = l->strainOffset = l->stress = 0.0f;
    l->strainRatio = s->vm[s->v[l->pos].mat].E / s->vm[s->v[l->neg].mat].E;
    l->smallAngle = 1;
    l->flags &= ~LF_LOCAL_VEL_VALID;
    link_update_rest(s, l);
    link_update_transverse(s, l);
}

/* CVoxelyze::combinedMaterial  Voxelyze3/src/old/Voxelyze.cpp:626-641 */
static int combined_material(vxo_sim* s, int m1, int m2) {
    for (int i = 0; i < s->nlm; i++)
        if ((s->lm[i].v1 == m1 && s->lm[i].v2 == m2) || (s->lm[i].v1 == m2 && s->lm[i].v2 == m1)) return i;
    if (s->nlm == s->caplm) { s->caplm = s->caplm ? 2 * s->caplm : 8; s->lm = realloc(s->lm, s->caplm * sizeof(mat_t)); }
    linkmat_build(&s->lm[s->nlm], &s->vm[m1], &s->vm[m2], m1, m2);
    return s->nlm++;
}

/* CVoxelyze::addLink  Voxelyze.cpp:508-539 with the CVX_Link constructor VX_Link.cpp:21-54 */
static void add_link(vxo_sim* s, int x, int y, int z, int dir) {
    int axis = dir / 2;
    int lx = x + (dir == 1 ? -1 : 0), ly = y + (dir == 3 ? -1 : 0), lz = z + (dir == 5 ? -1 : 0);
    int lc = lcell(s, lx, ly, lz);
    if (lc < 0 || s->lgrid[axis][lc] >= 0) return;
    int a = voxel_at(s, x, y, z);
    int b = voxel_at(s, x + DOFF[dir][0], y + DOFF[dir][1], z + DOFF[dir][2]);
    if (a < 0 || b < 0) return;
    int lmat = combined_material(s, s->v[a].mat, s->v[b].mat);
    if (s->nl == s->capl) { s->capl = s->capl ? 2 * s->capl : 64; s->l = realloc(s->l, s->capl * sizeof(link_t)); }
    link_t* l = &s->l[s->nl];
    memset(l, 0, sizeof(*l));
    /* voxel1 = a, voxel2 = b: the lower-index voxel along the axis is the negative end */
    int rev = is_neg_dir(dir);
    l->neg = rev ? b : a;
    l->pos = rev ? a : b;
    l->axis = axis;
    l->mat = lmat;
    l->flags = 0;
    link_reset(s, l);
    s->lgrid[axis][lc] = s->nl;
    s->v[a].links[dir] = s->nl;
    s->v[b].links[opposite(dir)] = s->nl;
    s->nl++;
    /* CVX_Voxel::addLinkInfo -> updateSurface (VX_Voxel.cpp:66-70, 375-380) */
    int ends[2] = {a, b};
    for (int k = 0; k < 2; k++) {
        vox_t* v = &s->v[ends[k]];
        int interior = 1;
        for (int i = 0; i < 6; i++) if (v->links[i] < 0) interior = 0;
        if (interior) v->flags |= VF_INTERIOR; else v->flags &= ~VF_INTERIOR;
    }
}

vxo_sim* vxo_create(const vxo_env* env, const vxo_material* mats, int nmat,
                    const int* voxels, const double* phase, int nvox,
                    const vxo_external* ext, int next) {
    vxo_sim* s = calloc(1, sizeof(vxo_sim));
    s->env = *env;
    s->nvm = nmat;
    s->vm = calloc(nmat > 0 ? nmat : 1, sizeof(mat_t));
    for (int i = 0; i < nmat; i++) vmat_from_palette(&s->vm[i], &mats[i], env->vox_size, env->gravity_mult);
    int mn[3] = {1 << 30, 1 << 30, 1 << 30}, mx[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int i = 0; i < nvox; i++)
        for (int k = 0; k < 3; k++) {
            if (voxels[4 * i + k] < mn[k]) mn[k] = voxels[4 * i + k];
            if (voxels[4 * i + k] > mx[k]) mx[k] = voxels[4 * i + k];
        }
    if (nvox == 0) { mn[0] = mn[1] = mn[2] = 0; mx[0] = mx[1] = mx[2] = 0; }
    s->minx = mn[0]; s->miny = mn[1]; s->minz = mn[2];
    s->dx = mx[0] - mn[0] + 1; s->dy = mx[1] - mn[1] + 1; s->dz = mx[2] - mn[2] + 1;
    size_t ncell = (size_t)s->dx * s->dy * s->dz, nlcell = (size_t)(s->dx + 1) * (s->dy + 1) * (s->dz + 1);
    s->grid = malloc(ncell * sizeof(int));
    for (size_t i = 0; i < ncell; i++) s->grid[i] = -1;
    for (int a = 0; a < 3; a++) {
        s->lgrid[a] = malloc(nlcell * sizeof(int));
        for (size_t i = 0; i < nlcell; i++) s->lgrid[a][i] = -1;
    }
    s->ext = calloc(next > 0 ? next : 1, sizeof(ext_t));
    s->next = next;
    s->v = calloc(nvox > 0 ? nvox : 1, sizeof(vox_t));
    /* CVoxelyze::addVoxel  Voxelyze.cpp:439-461 (voxel ctor + reset: VX_Voxel.cpp:23-57) */
    for (int i = 0; i < nvox; i++) {
        vox_t* v = &s->v[i];
        v->ix = voxels[4 * i]; v->iy = voxels[4 * i + 1]; v->iz = voxels[4 * i + 2]; v->mat = voxels[4 * i + 3];
        for (int k = 0; k < 6; k++) v->links[k] = -1;
        v->ext = -1;
        double sz = s->vm[v->mat].nom;
        v->pos = V(v->ix * sz, v->iy * sz, v->iz * sz);
        v->orient = qident();
        v->linMom = v->angMom = V(0, 0, 0);
        v->flags = VF_STATIC;
        v->temp = 0.0f;
        v->prevDt = 0.0f;
        v->pStrainInvalid = 1;
        v->phase = phase ? phase[i] : 0.0;
        if (env->floor_enabled) v->flags |= VF_FLOOR;
        s->grid[cell(s, v->ix, v->iy, v->iz)] = i;
        s->nv = i + 1;
        for (int d = 0; d < 6; d++) add_link(s, v->ix, v->iy, v->iz, d);
    }
    for (int k = 0; k < next; k++) {
        s->ext[k].e = ext[k];
        v3 r = V(ext[k].rotate[0], ext[k].rotate[1], ext[k].rotate[2]);
        /* CVX_External::rotationChanged  VX_External.cpp:100-109 */
        s->ext[k].rotQ = (r.x != 0 || r.y != 0 || r.z != 0) ? q_from_rotvec(r) : qident();
        if (ext[k].voxel >= 0 && ext[k].voxel < nvox) s->v[ext[k].voxel].ext = k;
    }
    /* initial temperature (CVX_Sim::UpdateMatTemps, VX_Sim.cpp:467-483) */
    for (int i = 0; i < nvox; i++) {
        vox_t* v = &s->v[i];
        v->temp = env->initial_temp;
        for (int d = 0; d < 6; d++) if (v->links[d] >= 0) link_update_rest(s, &s->l[v->links[d]]);
    }
    if (env->collisions_enabled) for (int i = 0; i < nvox; i++) s->v[i].flags |= VF_COLLIDE;
    s->collisionsStale = 1;
    s->nearbyStale = 1;
    return s;
}

void vxo_free(vxo_sim* s) {
    if (!s) return;
    for (int i = 0; i < s->nv; i++) { free(s->v[i].nearby); free(s->v[i].colWatch); }
    free(s->vm); free(s->lm); free(s->v); free(s->l); free(s->ext); free(s->grid);
    for (int a = 0; a < 3; a++) free(s->lgrid[a]);
    free(s->col);
    free(s);
}

/* CVX_Link::updateStrain  VX_Link.cpp:212-241 */
static float link_update_strain(link_t* l, const mat_t* m, float axialStrain) {
    l->strain = axialStrain;
    if (m->linear) {
        if (axialStrain > l->maxStrain) l->maxStrain = axialStrain;
        return mat_stress(m, axialStrain, l->tss, 0);
    }
    float rs;
    if (axialStrain > l->maxStrain) {
        l->maxStrain = axialStrain;
        rs = mat_stress(m, axialStrain, l->tss, 0);
        if (m->nu != 0.0f) l->strainOffset = l->maxStrain - mat_stress(m, axialStrain, 0.0f, 0) / (m->eHat * (1 - m->nu));
        else l->strainOffset = l->maxStrain - rs / m->E;
    } else {
        float rel = axialStrain - l->strainOffset;
        if (m->nu != 0.0f) rs = mat_stress(m, rel, l->tss, 1);
        else rs = m->E * rel;
    }
    return rs;
}

/* CVX_Voxel::dampingMultiplier  VX_Voxel.h:132 */
static float damping_mult(const vxo_sim* s, const vox_t* v) {
    const mat_t* m = &s->vm[v->mat];
    return 2 * m->sqrtMass * m->zi / v->prevDt;
}

/* CVX_Link::orientLink + updateForces  VX_Link.cpp:72-113, 143-209 */
static void link_update_forces(vxo_sim* s, link_t* l) {
    v3 oldPos2 = l->pos2, oldA1 = l->a1v, oldA2 = l->a2v;
    const vox_t* vn = &s->v[l->neg];
    const vox_t* vp = &s->v[l->pos];
    const mat_t* m = &s->lm[l->mat];
    /* orientLink */
    l->pos2 = to_axis_x(l->axis, vsub(vp->pos, vn->pos));
    qd angle1 = q_to_axis_x(l->axis, vn->orient);
    qd angle2 = q_to_axis_x(l->axis, vp->orient);
    qd totalRot = qconj(angle1);
    l->pos2 = qrot(totalRot, l->pos2);
    angle2 = qmul(totalRot, angle2);
    angle1 = qident();
    float smallTurn = (float)((fabs(l->pos2.z) + fabs(l->pos2.y)) / l->pos2.x);
    float extendPerc = (float)(fabs(1 - l->pos2.x / l->restLen));
    if (!l->smallAngle && smallTurn < SA_BOND_BEND_RAD && extendPerc < SA_BOND_EXT_PERC) {
        l->smallAngle = 1;
        l->flags &= ~LF_LOCAL_VEL_VALID;
    } else if (l->smallAngle && (smallTurn > HYSTERESIS_FACTOR * SA_BOND_BEND_RAD || extendPerc > HYSTERESIS_FACTOR * SA_BOND_EXT_PERC)) {
        l->smallAngle = 0;
        l->flags &= ~LF_LOCAL_VEL_VALID;
    }
    if (l->smallAngle) {
        l->pos2.x -= l->restLen;
    } else {
        angle1 = q_from_angle_to_posx(angle1, l->pos2);
        angle2 = qmul(angle1, angle2);
        l->pos2 = V(sqrt(vlen2(l->pos2)) - l->restLen, 0, 0);
    }
    l->a1v = q_to_rotvec(angle1);
    l->a2v = q_to_rotvec(angle2);
    l->angle1 = angle1;
    l->angle2 = angle2;
    /* updateForces */
    v3 dPos2 = vscale(vsub(l->pos2, oldPos2), 0.5);
    v3 dA1 = vscale(vsub(l->a1v, oldA1), 0.5);
    v3 dA2 = vscale(vsub(l->a2v, oldA2), 0.5);
    if (!(m->nu == 0.0f) || l->tss != 0) link_update_transverse(s, l);
    l->stress = link_update_strain(l, m, (float)(l->pos2.x / l->restLen));
    if (mat_is_failed(m, l->maxStrain)) { l->fN = l->fP = l->mN = l->mP = V(0, 0, 0); return; }
    float b1 = m->b1, b2 = m->b2, b3 = m->b3, a2 = m->a2;
    v3 p2 = l->pos2, a1v = l->a1v, a2v = l->a2v;
    l->fN = V(l->stress * l->A, b1 * p2.y - b2 * (a1v.z + a2v.z), b1 * p2.z + b2 * (a1v.y + a2v.y));
    l->fP = V(-l->fN.x, -l->fN.y, -l->fN.z);
    l->mN = V(a2 * (a2v.x - a1v.x), -b2 * p2.z - b3 * (2 * a1v.y + a2v.y), b2 * p2.y - b3 * (2 * a1v.z + a2v.z));
    l->mP = V(a2 * (a1v.x - a2v.x), -b2 * p2.z - b3 * (a1v.y + 2 * a2v.y), b2 * p2.y - b3 * (a1v.z + 2 * a2v.z));
    if (l->flags & LF_LOCAL_VEL_VALID) {
        float sqA1 = m->sqA1, sqA2xIp = m->sqA2xIp, sqB1 = m->sqB1, sqB2xFMp = m->sqB2xFMp, sqB3xIp = m->sqB3xIp;
        v3 pc = V(sqA1 * dPos2.x, sqB1 * dPos2.y - sqB2xFMp * (dA1.z + dA2.z), sqB1 * dPos2.z + sqB2xFMp * (dA1.y + dA2.y));
        float dmN = damping_mult(s, vn), dmP = damping_mult(s, vp);
        l->fN = vadd(l->fN, vscale(pc, dmN));
        l->fP = vsub(l->fP, vscale(pc, dmP));
        double hN = 0.5 * dmN, hP = 0.5 * dmP;
        v3 tN = V(-sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (2 * dA1.y + dA2.y), -sqB2xFMp * dPos2.y + sqB3xIp * (2 * dA1.z + dA2.z));
        v3 tP = V(sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (dA1.y + 2 * dA2.y), -sqB2xFMp * dPos2.y + sqB3xIp * (dA1.z + 2 * dA2.z));
        l->mN = vsub(l->mN, vscale(tN, hN));
        l->mP = vsub(l->mP, vscale(tP, hP));
    } else {
        l->flags |= LF_LOCAL_VEL_VALID;
    }
    if (!l->smallAngle) {
        l->fN = qrotinv(angle1, l->fN);
        l->mN = qrotinv(angle1, l->mN);
    }
    l->fP = qrotinv(angle2, l->fP);
    l->mP = qrotinv(angle2, l->mP);
    l->fN = to_axis_orig(l->axis, l->fN);
    l->fP = to_axis_orig(l->axis, l->fP);
    l->mN = to_axis_orig(l->axis, l->mN);
    l->mP = to_axis_orig(l->axis, l->mP);
}

/* CVX_Link::axialStiffness  VX_Link.cpp:251-259 */
static float link_axial_stiffness(vxo_sim* s, link_t* l) {
    const mat_t* m = &s->lm[l->mat];
    if (m->nu == 0.0f) return m->a1;
    link_update_rest(s, l);
    link_update_transverse(s, l);
    return (float)(m->eHat * l->A / ((l->strain + 1) * l->restLen));
}

/* CVoxelyze::recommendedTimeStep  Voxelyze.cpp:286-311 */
static float recommended_dt(vxo_sim* s) {
    float maxf2 = 0.0f;
    for (int i = 0; i < s->nl; i++) {
        link_t* l = &s->l[i];
        float m1 = s->vm[s->v[l->neg].mat].mass, m2 = s->vm[s->v[l->pos].mat].mass;
        float f2 = link_axial_stiffness(s, l) / (m1 < m2 ? m1 : m2);
        if (f2 > maxf2) maxf2 = f2;
    }
    if (maxf2 <= 0.0f) {
        for (int i = 0; i < s->nv; i++) {
            const mat_t* m = &s->vm[s->v[i].mat];
            float f2 = (float)(m->E * m->nom / m->mass);
            if (f2 > maxf2) maxf2 = f2;
        }
    }
    if (maxf2 <= 0.0f) return 0.0f;
    return 1.0f / (6.283185f * sqrtf(maxf2));
}

/* CVX_Collision::updateContactForce  VX_Collision.cpp:42-56 */
static void col_update(vxo_sim* s, col_t* c) {
    const vox_t* a = &s->v[c->v1];
    const vox_t* b = &s->v[c->v2];
    v3 d = vsub(b->pos, a->pos);
    v3f off = {(float)d.x, (float)d.y, (float)d.z};
    float nomDist = (float)((base_size_avg(s, a) + base_size_avg(s, b)) * ENVELOPE_RADIUS);
    float relDist = nomDist - sqrtf(off.x * off.x + off.y * off.y + off.z * off.z);
    if (relDist > 0) {
        float l = sqrtf(off.x * off.x + off.y * off.y + off.z * off.z);
        v3f u = off;
        if (l > 0) { float inv = 1.0f / l; u.x = inv * off.x; u.y = inv * off.y; u.z = inv * off.z; }
        const mat_t* ma = &s->vm[a->mat];
        const mat_t* mb = &s->vm[b->mat];
        v3 va = vscale(a->linMom, ma->massInv), vb = vscale(b->linMom, mb->massInv);
        float rv = (float)((va.x * (double)u.x + va.y * (double)u.y + va.z * (double)u.z) -
                           (vb.x * (double)u.x + vb.y * (double)u.y + vb.z * (double)u.z));
        float f = c->k * relDist + c->c * rv;
        c->force.x = f * u.x; c->force.y = f * u.y; c->force.z = f * u.z;
    } else {
        c->force.x = c->force.y = c->force.z = 0;
    }
}

/* CVX_Voxel::generateNearby  VX_Voxel.cpp:394-417 (breadth-first over links) */
static void gen_nearby(vxo_sim* s, int vi, int depth) {
    int cap = 64, n = 0;
    int* all = malloc(cap * sizeof(int));
    char* seen = calloc(s->nv, 1);
    all[n++] = vi; seen[vi] = 1;
    int cur = 0;
    for (int k = 0; k < depth; k++) {
        int end = n;
        while (cur != end) {
            const vox_t* v = &s->v[all[cur++]];
            for (int d = 0; d < 6; d++) {
                int li = v->links[d];
                if (li < 0) continue;
                int o = s->l[li].neg == (int)(v - s->v) ? s->l[li].pos : s->l[li].neg;
                if (!seen[o]) {
                    if (n == cap) { cap *= 2; all = realloc(all, cap * sizeof(int)); }
                    all[n++] = o; seen[o] = 1;
                }
            }
        }
    }
    vox_t* v = &s->v[vi];
    free(v->nearby);
    v->nearby = malloc((n > 0 ? n : 1) * sizeof(int));
    v->n_nearby = 0;
    for (int i = 0; i < n; i++)
        if (!(s->v[all[i]].flags & VF_INTERIOR) && all[i] != vi) v->nearby[v->n_nearby++] = all[i];
    free(all); free(seen);
}
static int in_nearby(const vox_t* v, int o) {
    for (int i = 0; i < v->n_nearby; i++) if (v->nearby[i] == o) return 1;
    return 0;
}
static void colwatch_push(vox_t* v, int ci) {
    if (v->n_col == v->cap_col) { v->cap_col = v->cap_col ? 2 * v->cap_col : 8; v->colWatch = realloc(v->colWatch, v->cap_col * sizeof(int)); }
    v->colWatch[v->n_col++] = ci;
}
/* CVoxelyze::regenerateCollisions  Voxelyze.cpp:726-751 */
static void regen_collisions(vxo_sim* s, float threshSq) {
    s->ncol = 0;
    for (int i = 0; i < s->nv; i++) s->v[i].n_col = 0;
    for (int i = 0; i < s->nv; i++) {
        vox_t* a = &s->v[i];
        if (a->flags & VF_INTERIOR) continue;
        a->lastColWatch.x = (float)a->pos.x; a->lastColWatch.y = (float)a->pos.y; a->lastColWatch.z = (float)a->pos.z;
        for (int j = i + 1; j < s->nv; j++) {
            vox_t* b = &s->v[j];
            if ((b->flags & VF_INTERIOR) || vlen2(vsub(a->pos, b->pos)) > threshSq || in_nearby(a, j)) continue;
            if (s->ncol == s->capcol) { s->capcol = s->capcol ? 2 * s->capcol : 64; s->col = realloc(s->col, s->capcol * sizeof(col_t)); }
            col_t* c = &s->col[s->ncol];
            const mat_t* ma = &s->vm[a->mat];
            const mat_t* mb = &s->vm[b->mat];
            float ka = (float)(2 * ma->E * ma->nom), kb = (float)(2 * mb->E * mb->nom);
            c->v1 = i; c->v2 = j;
            c->k = 2.0f / (1.0f / ka + 1.0f / kb);
            c->c = 0.5f * (ma->zc * ma->c2m + mb->zc * mb->c2m);
            c->force.x = c->force.y = c->force.z = 0;
            colwatch_push(a, s->ncol);
            colwatch_push(b, s->ncol);
            s->ncol++;
        }
    }
    s->collisionsStale = 0;
}
/* CVoxelyze::updateCollisions  Voxelyze.cpp:671-711 */
static void update_collisions(vxo_sim* s) {
    float watchVx = 2 * s->env.bounding_radius + s->env.watch_distance;
    float watchMm = (float)(s->env.vox_size * watchVx);
    float recalc = (float)(s->env.vox_size * s->env.watch_distance / 2);
    if (s->nearbyStale) {
        for (int i = 0; i < s->nv; i++) gen_nearby(s, i, (int)(watchVx * 2));
        s->nearbyStale = 0;
        s->collisionsStale = 1;
    }
    for (int i = 0; i < s->nv; i++) {
        vox_t* v = &s->v[i];
        if (v->flags & VF_INTERIOR) continue;
        v3 d = V(v->pos.x - v->lastColWatch.x, v->pos.y - v->lastColWatch.y, v->pos.z - v->lastColWatch.z);
        if (vlen2(d) > recalc * recalc) s->collisionsStale = 1;
    }
    if (s->collisionsStale) regen_collisions(s, watchMm * watchMm);
    for (int i = 0; i < s->ncol; i++) col_update(s, &s->col[i]);
}

/* CVX_Voxel::force  VX_Voxel.cpp:232-251 */
static v3 voxel_force(vxo_sim* s, vox_t* v) {
    const mat_t* m = &s->vm[v->mat];
    v3 f = V(0, 0, 0);
    for (int i = 0; i < 6; i++) {
        if (v->links[i] < 0) continue;
        const link_t* l = &s->l[v->links[i]];
        f = vadd(f, is_neg_dir(i) ? l->fP : l->fN);
    }
    f = qrot(v->orient, f);
    if (v->ext >= 0) { const float* ef = s->ext[v->ext].e.force; f.x += ef[0]; f.y += ef[1]; f.z += ef[2]; }
    v3 vel = vscale(v->linMom, m->massInv);
    f = vsub(f, vscale(vel, m->zg * m->c2m));
    f.z += -m->mass * 9.80665f * m->grav;
    if (v->flags & VF_COLLIDE) {
        int self = (int)(v - s->v);
        for (int k = 0; k < v->n_col; k++) {
            const col_t* c = &s->col[v->colWatch[k]];
            v3f cf = c->force;
            if (c->v2 == self) { cf.x = -cf.x; cf.y = -cf.y; cf.z = -cf.z; }
            f.x -= cf.x; f.y -= cf.y; f.z -= cf.z;
        }
    }
    return f;
}
/* CVX_Voxel::moment  VX_Voxel.cpp:253-269 */
static v3 voxel_moment(vxo_sim* s, vox_t* v) {
    const mat_t* m = &s->vm[v->mat];
    v3 t = V(0, 0, 0);
    for (int i = 0; i < 6; i++) {
        if (v->links[i] < 0) continue;
        const link_t* l = &s->l[v->links[i]];
        t = vadd(t, is_neg_dir(i) ? l->mP : l->mN);
    }
    t = qrot(v->orient, t);
    if (v->ext >= 0) { const float* em = s->ext[v->ext].e.moment; t.x += em[0]; t.y += em[1]; t.z += em[2]; }
    v3 w = vscale(v->angMom, m->Iinv);
    return vsub(t, vscale(w, m->zg * m->c2i));
}
/* CVX_Voxel::floorPenetration  VX_Voxel.h:124 */
static float floor_pen(const vxo_sim* s, const vox_t* v) {
    return (float)(base_size_avg(s, v) / 2 - s->vm[v->mat].nom / 2 - v->pos.z);
}
/* CVX_Voxel::floorForce  VX_Voxel.cpp:272-297 */
static void floor_force(vxo_sim* s, vox_t* v, v3* F) {
    const mat_t* m = &s->vm[v->mat];
    float pen = floor_pen(s, v);
    if (pen >= 0) {
        v3 vel = vscale(v->linMom, m->massInv);
        v3 hv = V(vel.x, vel.y, 0);
        float normal = (float)(2 * m->E * m->nom) * pen;
        F->z += normal - (m->zc * m->c2m) * vel.z;
        if (v->flags & VF_STATIC) {
            float surf = (float)(F->x * F->x + F->y * F->y);
            float fric = (m->mus * normal) * (m->mus * normal);
            if (surf > fric) v->flags &= ~VF_STATIC;
        } else {
            double l = sqrt(hv.x * hv.x + hv.y * hv.y + hv.z * hv.z);
            v3 n = hv;
            if (l > 0) { double inv = 1.0 / l; n = V(inv * hv.x, inv * hv.y, inv * hv.z); }
            float k = m->muk * normal;
            F->x -= k * n.x; F->y -= k * n.y; F->z -= k * n.z;
        }
    } else {
        v->flags &= ~VF_STATIC;
    }
}

/* CVX_Voxel::timeStep  VX_Voxel.cpp:163-230 */
static void voxel_step(vxo_sim* s, vox_t* v, float dt) {
    const mat_t* m = &s->vm[v->mat];
    v->prevDt = dt;
    if (dt == 0.0f) return;
    const ext_t* e = v->ext >= 0 ? &s->ext[v->ext] : NULL;
    if (e && (e->e.dof_fixed & 0x3F) == 0x3F) {
        double sz = m->nom;
        v->pos = V(v->ix * sz + e->e.translate[0], v->iy * sz + e->e.translate[1], v->iz * sz + e->e.translate[2]);
        v->orient = e->rotQ;
        v->linMom = v->angMom = V(0, 0, 0);
        return;
    }
    v3 F = voxel_force(s, v);
    v3 fric = F;
    if (v->flags & VF_FLOOR) floor_force(s, v, &F);
    fric = vsub(F, fric);
    v->linMom = vadd(v->linMom, vscale(F, dt));
    v3 tr = vscale(v->linMom, dt * m->massInv);
    if ((v->flags & VF_FLOOR) && floor_pen(s, v) >= 0) {
        double work = fric.x * tr.x + fric.y * tr.y;
        double hKe = 0.5 * m->massInv * (v->linMom.x * v->linMom.x + v->linMom.y * v->linMom.y);
        if (hKe + work <= 0) v->flags |= VF_STATIC;
        if (v->flags & VF_STATIC) { v->linMom.x = v->linMom.y = 0; tr.x = tr.y = 0; }
    } else {
        v->flags &= ~VF_STATIC;
    }
    v->pos = vadd(v->pos, tr);
    v3 M = voxel_moment(s, v);
    v->angMom = vadd(v->angMom, vscale(M, dt));
    v->orient = qmul(q_from_rotvec(vscale(v->angMom, dt * m->Iinv)), v->orient);
    if (e) {
        double sz = m->nom;
        int d = e->e.dof_fixed;
        if (d & 1) { v->pos.x = v->ix * sz + e->e.translate[0]; v->linMom.x = 0; }
        if (d & 2) { v->pos.y = v->iy * sz + e->e.translate[1]; v->linMom.y = 0; }
        if (d & 4) { v->pos.z = v->iz * sz + e->e.translate[2]; v->linMom.z = 0; }
        if (d & 0x38) {
            if ((d & 0x38) == 0x38) {
                v->orient = e->rotQ;
                v->angMom = V(0, 0, 0);
            } else {
                v3 rv = q_to_rotvec(v->orient);
                if (d & 8) { rv.x = 0; v->angMom.x = 0; }
                if (d & 16) { rv.y = 0; v->angMom.y = 0; }
                if (d & 32) { rv.z = 0; v->angMom.z = 0; }
                v->orient = q_from_rotvec(rv);
            }
        }
    }
    v->pStrainInvalid = 1;
}

/* one step: VX3 driver (Voxelyze3/src/VX3/VX3_VoxelyzeKernel.cu:237-359, 625-650)
 * around CVoxelyze::doTimeStep (Voxelyze3/src/old/Voxelyze.cpp:251-284) */
int vxo_step(vxo_sim* s, int n) {
    int done = 0;
    for (int k = 0; k < n && !s->diverged; k++) {
        if (s->env.vary_temp && s->env.temp_period > 0) {
            for (int i = 0; i < s->nv; i++) {
                vox_t* v = &s->v[i];
                double T = s->env.temp_amplitude * sin(2 * 3.1415926f * (s->t / s->env.temp_period + v->phase));
                if (!s->env.enable_expansion && T > 0) T = 0;
                v->temp = (float)T;
                for (int d = 0; d < 6; d++) if (v->links[d] >= 0) link_update_rest(s, &s->l[v->links[d]]);
            }
        }
        if (!s->have_dt) {
            s->optdt = recommended_dt(s);
            if (s->optdt < 1e-10f) s->optdt = 1e-10f;
            s->have_dt = 1;
        }
        float dt = (float)(s->env.dt_frac * (double)s->optdt);
        if (dt == 0) { done++; continue; }
        int diverged = 0;
        for (int i = 0; i < s->nl; i++) {
            link_update_forces(s, &s->l[i]);
            if (s->l[i].strain > 100) diverged = 1;
        }
        if (diverged) { s->diverged = 1; break; }
        if (s->env.collisions_enabled) update_collisions(s);
        for (int i = 0; i < s->nv; i++) voxel_step(s, &s->v[i], dt);
        s->t += dt;
        s->steps++;
        done++;
    }
    return done;
}

void vxo_counts(const vxo_sim* s, int* o) { o[0] = s->nv; o[1] = s->nl; o[2] = s->nvm; o[3] = s->nlm; }
void vxo_scalars(const vxo_sim* s, double* o) {
    o[0] = s->t; o[1] = s->optdt; o[2] = (float)(s->env.dt_frac * (double)s->optdt); o[3] = s->diverged; o[4] = (double)s->steps;
}
void vxo_voxel_state(const vxo_sim* s, double* d13, float* f4, int* flags) {
    for (int i = 0; i < s->nv; i++) {
        const vox_t* v = &s->v[i];
        double* d = d13 + 13 * i;
        d[0] = v->pos.x; d[1] = v->pos.y; d[2] = v->pos.z;
        d[3] = v->linMom.x; d[4] = v->linMom.y; d[5] = v->linMom.z;
        d[6] = v->orient.w; d[7] = v->orient.x; d[8] = v->orient.y; d[9] = v->orient.z;
        d[10] = v->angMom.x; d[11] = v->angMom.y; d[12] = v->angMom.z;
        f4[4 * i] = v->temp; f4[4 * i + 1] = v->pStrain.x; f4[4 * i + 2] = v->pStrain.y; f4[4 * i + 3] = v->pStrain.z;
        flags[i] = v->flags | (v->flags & VF_COLLIDE ? 0 : 0);
    }
}
void vxo_link_state(const vxo_sim* s, double* d22, float* f6, int* i2) {
    for (int i = 0; i < s->nl; i++) {
        const link_t* l = &s->l[i];
        double* d = d22 + 22 * i;
        v3 vs[7] = {l->pos2, l->a1v, l->a2v, l->fN, l->fP, l->mN, l->mP};
        for (int k = 0; k < 7; k++) { d[3 * k] = vs[k].x; d[3 * k + 1] = vs[k].y; d[3 * k + 2] = vs[k].z; }
        d[21] = l->restLen;
        float* f = f6 + 6 * i;
        f[0] = l->strain; f[1] = l->maxStrain; f[2] = l->strainOffset; f[3] = l->stress; f[4] = l->A; f[5] = l->tss;
        i2[2 * i] = l->smallAngle; i2[2 * i + 1] = l->flags;
    }
}
void vxo_topology(const vxo_sim* s, int* vox4, int* lnk4) {
    for (int i = 0; i < s->nv; i++) {
        vox4[4 * i] = s->v[i].ix; vox4[4 * i + 1] = s->v[i].iy; vox4[4 * i + 2] = s->v[i].iz; vox4[4 * i + 3] = s->v[i].mat;
    }
    for (int i = 0; i < s->nl; i++) {
        lnk4[4 * i] = s->l[i].neg; lnk4[4 * i + 1] = s->l[i].pos; lnk4[4 * i + 2] = s->l[i].axis; lnk4[4 * i + 3] = s->l[i].mat;
    }
}
void vxo_voxmats(const vxo_sim* s, float* f, double* nom) {
    for (int k = 0; k < s->nvm; k++) {
        const mat_t* m = &s->vm[k];
        float v[18] = {m->E, m->nu, m->rho, m->cte, m->mus, m->muk, m->zi, m->zg, m->zc, m->eHat,
                       m->mass, m->massInv, m->sqrtMass, m->I, m->Iinv, m->c2m, m->c2i, m->grav};
        memcpy(f + 18 * k, v, sizeof(v));
        nom[k] = m->nom;
    }
}
void vxo_linkmats(const vxo_sim* s, int* idx, float* f) {
    for (int k = 0; k < s->nlm; k++) {
        const mat_t* m = &s->lm[k];
        idx[2 * k] = m->v1; idx[2 * k + 1] = m->v2;
        float v[20] = {m->E, m->nu, m->eHat, m->a1, m->a2, m->b1, m->b2, m->b3, m->sqA1, m->sqA2xIp, m->sqB1,
                       m->sqB2xFMp, m->sqB3xIp, m->sigmaYield, m->sigmaFail, m->epsYield, m->epsFail,
                       m->linear ? 1.0f : 0.0f, (float)m->nom, m->rho};
        memcpy(f + 20 * k, v, sizeof(v));
    }
}
/* VX3_VoxelyzeKernel::updateCurrentCenterOfMass  Voxelyze3/src/VX3/VX3_VoxelyzeKernel.cu:477-493 */
void vxo_center_of_mass(const vxo_sim* s, double* out) {
    double tm = 0, sx = 0, sy = 0, sz = 0;
    for (int i = 0; i < s->nv; i++) {
        const mat_t* m = &s->vm[s->v[i].mat];
        if (!m->is_measured) continue;
        double w = m->mass;
        sx += s->v[i].pos.x * w; sy += s->v[i].pos.y * w; sz += s->v[i].pos.z * w;
        tm += w;
    }
    if (tm == 0) { out[0] = out[1] = out[2] = 0; return; }
    out[0] = sx / tm; out[1] = sy / tm; out[2] = sz / tm;
}
