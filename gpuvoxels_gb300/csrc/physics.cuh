// Device physics for the Voxelyze step, written for sm_103a.
//
// Each function restates one routine of the reference CPU Voxelyze
// (Voxelyze3/src/old/*.cpp, cited per function) with the same operand types
// (float vs double) and the same association order.  This header is compiled
// twice, into namespace GVX_KNS: the exact build (-fmad=false, every multiply
// and add rounds on its own, as in the reference built without contraction)
// and the FMA build (-fmad=true, fewer FP64 instructions).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "fp64_int.cuh"
#include "layout.cuh"

#ifndef GVX_KNS
#error "GVX_KNS (the kernel build namespace) must be defined"
#endif

namespace gvx {
namespace GVX_KNS {
using namespace gvx::dev;

// ------------------------------------------------------------ small vector math
struct d3 { double x, y, z; };
struct q4 { double w, x, y, z; };

__device__ __forceinline__ d3 D3(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ q4 Q4(double w, double x, double y, double z) { q4 r; r.w = w; r.x = x; r.y = y; r.z = z; return r; }

// ---------------------------------------------------- exact FP64 shortcuts
// Scaling by 2 or 1/2, float<->double conversions and FP64 comparisons run on the
// integer pipes (fp64_int.cuh); results are bit-identical to the FP64 instructions.
using fp64i::mul2;
using fp64i::half;
using fp64i::f2d;
using fp64i::d2f;
using fp64i::zero_plus;
using fp64i::zero_minus;
using fp64i::minus_zero;
using fp64i::times_zero;

// (float)(n/d) compared with a float threshold T, deciding with one multiply
// unless n/d lies within 2^-20 (relative) of T, where the quotient is formed
// exactly.  Outside that band the rounded float quotient cannot reach T, so the
// decision equals the reference's (float)(n/d) < T (or > T).
__device__ __forceinline__ bool quot_lt(double n, double d, float T) {
    const double t = T;
    if (fp64i::gt0(d)) {
        if (fp64i::lt(n, (t * (1.0 - 0x1p-20)) * d)) return true;
        if (fp64i::gt(n, (t * (1.0 + 0x1p-20)) * d)) return false;
    }
    return d2f(n / d) < T;
}
__device__ __forceinline__ bool quot_gt(double n, double d, float T) {
    const double t = T;
    if (fp64i::gt0(d)) {
        if (fp64i::gt(n, (t * (1.0 + 0x1p-20)) * d)) return true;
        if (fp64i::lt(n, (t * (1.0 - 0x1p-20)) * d)) return false;
    }
    return d2f(n / d) > T;
}
// (float)fabs(1 - x/r) < T and > T for r > 0, with the same band rule (T < 1).
__device__ __forceinline__ bool ext_lt(double x, double r, float T) {
    const double t = T;
    if (fp64i::gt(x, ((1.0 - t) * (1.0 + 0x1p-20)) * r) && fp64i::lt(x, ((1.0 + t) * (1.0 - 0x1p-20)) * r)) return true;
    if (fp64i::lt(x, ((1.0 - t) * (1.0 - 0x1p-20)) * r) || fp64i::gt(x, ((1.0 + t) * (1.0 + 0x1p-20)) * r)) return false;
    return d2f(fabs(1 - x / r)) < T;
}
__device__ __forceinline__ bool ext_gt(double x, double r, float T) {
    const double t = T;
    if (fp64i::gt(x, ((1.0 - t) * (1.0 + 0x1p-20)) * r) && fp64i::lt(x, ((1.0 + t) * (1.0 - 0x1p-20)) * r)) return false;
    if (fp64i::lt(x, ((1.0 - t) * (1.0 - 0x1p-20)) * r) || fp64i::gt(x, ((1.0 + t) * (1.0 + 0x1p-20)) * r)) return true;
    return d2f(fabs(1 - x / r)) > T;
}

// Quat3D::operator*  Voxelyze3/src/old/Quat3D.h:87
__device__ __forceinline__ q4 qmul(const q4& a, const q4& f) {
    return Q4(a.w * f.w - a.x * f.x - a.y * f.y - a.z * f.z,
              a.w * f.x + a.x * f.w + a.y * f.z - a.z * f.y,
              a.w * f.y - a.x * f.z + a.y * f.w + a.z * f.x,
              a.w * f.z + a.x * f.y - a.y * f.x + a.z * f.w);
}
// Quat3D::RotateVec3D  Quat3D.h:174-181
__device__ __forceinline__ d3 qrot(const q4& q, const d3& f) {
    double tw = f.x * q.x + f.y * q.y + f.z * q.z;
    double tx = f.x * q.w - f.y * q.z + f.z * q.y;
    double ty = f.x * q.z + f.y * q.w - f.z * q.x;
    double tz = -f.x * q.y + f.y * q.x + f.z * q.w;
    return D3(q.w * tx + q.x * tw + q.y * tz - q.z * ty,
              q.w * ty - q.x * tz + q.y * tw + q.z * tx,
              q.w * tz + q.x * ty - q.y * tx + q.z * tw);
}
// Quat3D::RotateVec3DInv  Quat3D.h:192-199
__device__ __forceinline__ d3 qrotinv(const q4& q, const d3& f) {
    double tw = q.x * f.x + q.y * f.y + q.z * f.z;
    double tx = q.w * f.x - q.y * f.z + q.z * f.y;
    double ty = q.w * f.y + q.x * f.z - q.z * f.x;
    double tz = q.w * f.z - q.x * f.y + q.y * f.x;
    return D3(tw * q.x + tx * q.w + ty * q.z - tz * q.y,
              tw * q.y - tx * q.z + ty * q.w + tz * q.x,
              tw * q.z + tx * q.y - ty * q.x + tz * q.w);
}
// The same two operations for a quaternion whose x component is the exact zero
// FromAngleToPosX always leaves there (finite operands): the q.x terms are settled on
// the integer pipes (times_zero, zero_plus, minus_zero), with bit-identical results.
__device__ __forceinline__ q4 qmul_x0(const q4& a, const q4& f) {
    return Q4(minus_zero(a.w * f.w, times_zero(f.x, a.x)) - a.y * f.y - a.z * f.z,
              zero_plus(times_zero(f.w, a.x), a.w * f.x) + a.y * f.z - a.z * f.y,
              minus_zero(a.w * f.y, times_zero(f.z, a.x)) + a.y * f.w + a.z * f.x,
              zero_plus(times_zero(f.y, a.x), a.w * f.z) - a.y * f.x + a.z * f.w);
}
__device__ __forceinline__ d3 qrotinv_x0(const q4& q, const d3& f) {
    double tw = zero_plus(times_zero(f.x, q.x), q.y * f.y) + q.z * f.z;
    double tx = q.w * f.x - q.y * f.z + q.z * f.y;
    double ty = zero_plus(times_zero(f.z, q.x), q.w * f.y) - q.z * f.x;
    double tz = minus_zero(q.w * f.z, times_zero(f.y, q.x)) + q.y * f.x;
    return D3(zero_plus(times_zero(tw, q.x), tx * q.w) + ty * q.z - tz * q.y,
              zero_plus(times_zero(tz, q.x), tw * q.y - tx * q.z + ty * q.w),
              minus_zero(tw * q.z + tx * q.y, times_zero(ty, q.x)) + tz * q.w);
}
// Quat3D::ToRotationVector  Quat3D.h:121-126; *wide = the acos branch was taken.
// kX0: q.x is the exact zero of a FromAngleToPosX result (the x component then too).
template <bool kX0 = false>
__device__ __forceinline__ d3 q_to_rotvec(const q4& q, bool* wide = nullptr) {
    if (fp64i::ge(fabs(q.w), 1.0)) return D3(0, 0, 0);   // q.w >= 1 || q.w <= -1
    double sl = 1.0 - q.w * q.w;
    if (fp64i::lt(sl, 2.4e-3)) {
        double s = sqrt((2 - mul2(q.w)) / sl);
        return D3(kX0 ? times_zero(s, q.x) : mul2(q.x) * s, mul2(q.y) * s, mul2(q.z) * s);
    }
    if (wide) *wide = true;
    double a = acos(q.w);
    double inv = 1.0 / sqrt(sl);
    return D3(kX0 ? times_zero(inv, times_zero(a, q.x)) : (mul2(q.x) * a) * inv, (mul2(q.y) * a) * inv, (mul2(q.z) * a) * inv);
}
// Quat3D::FromRotationVector  Quat3D.h:128-143
// *wide = the sin/cos branch was taken
__device__ __forceinline__ q4 q_from_rotvec(const d3& v, bool* wide = nullptr) {
    double tx = half(v.x), ty = half(v.y), tz = half(v.z);
    double m2 = tx * tx + ty * ty + tz * tz;
    double w, s;
    if (fp64i::lt(m2 * m2, 5.328e-15)) {
        w = 1.0 - half(m2);
        s = 1.0 - m2 / 6.0;
    } else {
        if (wide) *wide = true;
        double m = sqrt(m2);
        double sn, cs;
        sincos(m, &sn, &cs);
        w = cs;
        s = sn / m;
    }
    return Q4(w, tx * s, ty * s, tz * s);
}
// Quat3D::FromAngleToPosX  Quat3D.h:145-170; `cur` is returned for a zero vector;
// *wide = the general (acos, sincos) branch was taken.  len = r.Length() (sqrt(x*x + y*y + z*z)),
// which the caller needs too: the general branch's normalisation takes it from there.
// Whether |RN(n/d)| < T for T = SMALL_ANGLE_RAD (1.732e-2), decided with one multiply
// where n/d lies outside [T(1 - 2^-20), T(1 + 2^-20)]: 1 (yes), 0 (no), -1 (undecided:
// near the threshold, or d zero, tiny, huge or not finite; the quotient decides).
__device__ __forceinline__ int quot_small_band(double n, double d) {
    const uint64_t ua = fp64i::bits(n) & fp64i::kAbs, ub = fp64i::bits(d) & fp64i::kAbs;
    const uint32_t eb = (uint32_t)(ub >> 52);
    if (eb - 64u >= 1918u || ua >= fp64i::kInf) return -1;
    const double a = fp64i::from_bits(ua), b = fp64i::from_bits(ub);
    if (fp64i::lt(a, (1.732e-2 * (1.0 - 0x1p-20)) * b)) return 1;
    if (fp64i::gt(a, (1.732e-2 * (1.0 + 0x1p-20)) * b)) return 0;
    return -1;
}
__device__ __forceinline__ q4 q_from_angle_to_posx(const q4& cur, const d3& r, double len, bool* wide = nullptr) {
    if (fp64i::eq0(r.x) && fp64i::eq0(r.y) && fp64i::eq0(r.z)) return cur;
    // YoverX, ZoverX within +-SMALL_ANGLE_RAD: the general branch below does not use the
    // quotients, so they are formed only when the small-angle branch needs them or the
    // band test cannot decide
    const int by = quot_small_band(r.y, r.x);
    const int bz = by == 0 ? 0 : quot_small_band(r.z, r.x);
    bool small_turn = by == 1 && bz == 1;
    double yox = 0, zox = 0;
    if (by != 0 && bz != 0) {
        yox = r.y / r.x;
        zox = r.z / r.x;
        small_turn = fp64i::lt(fabs(yox), 1.732e-2) && fp64i::lt(fabs(zox), 1.732e-2);   // |yox|, |zox| < 1.732e-2
    }
    if (small_turn) {
        double y = half(zox), z = -half(yox);
        return Q4(1 + half(-y * y - z * z), 0, y, z);
    }
    if (wide) *wide = true;
    const double l = len;
    double nx = r.x, ny = r.y, nz = r.z;
    if (fp64i::gt0(l)) { double li = 1.0 / l; nx *= li; ny *= li; nz *= li; }
    double theta = acos(nx);
    if (fp64i::gt(theta, 3.14159265358979 - 1e-7)) return Q4(0, 0, 1, 0);
    double ami = 1.0 / sqrt(nz * nz + ny * ny);
    double a = half(theta);
    double sn, cs;
    sincos(a, &sn, &cs);
    return Q4(cs, 0, nz * ami * sn, -ny * ami * sn);
}
// CVX_Link::toAxisX / toAxisOriginal  Voxelyze3/src/old/VX_Link.h:106-111
__device__ __forceinline__ d3 to_axis_x(int axis, const d3& v) {
    if (axis == 1) return D3(v.y, -v.x, v.z);
    if (axis == 2) return D3(v.z, v.y, -v.x);
    return v;
}
__device__ __forceinline__ q4 q_to_axis_x(int axis, const q4& q) {
    if (axis == 1) return Q4(q.w, q.y, -q.x, q.z);
    if (axis == 2) return Q4(q.w, q.z, q.y, -q.x);
    return q;
}
__device__ __forceinline__ d3 to_axis_orig(int axis, const d3& v) {
    if (axis == 1) return D3(-v.y, v.x, v.z);
    if (axis == 2) return D3(-v.z, v.y, v.x);
    return v;
}

// CVX_Material::stress  Voxelyze3/src/old/VX_Material.cpp:182-212
__device__ __forceinline__ float mat_stress(const LMat& m, float strain, float tss, bool forceLinear) {
    if (m.epsFail != -1.0f && strain > m.epsFail) return 0.0f;
    if (strain <= m.strain[1] || m.linear || forceLinear) {
        if (m.nu == 0.0f) return m.E * strain;
        return m.eHat * ((1 - m.nu) * strain + m.nu * tss);
    }
    int dc = m.n;
    for (int i = 2; i < dc; i++) {
        if (strain <= m.strain[i] || i == dc - 1) {
            float perc = (strain - m.strain[i - 1]) / (m.strain[i] - m.strain[i - 1]);
            float basic = m.stress[i - 1] + perc * (m.stress[i] - m.stress[i - 1]);
            if (m.nu == 0.0f) return basic;
            float mod = (m.stress[i] - m.stress[i - 1]) / (m.strain[i] - m.strain[i - 1]);
            float modHat = mod / ((1 - 2 * m.nu) * (1 + m.nu));
            float effS = basic / mod;
            float effT = tss * (effS / strain);
            return modHat * ((1 - m.nu) * effS + m.nu * effT);
        }
    }
    return 0.0f;
}

// (float)pow(x, y) for the Poisson strain of CVX_Voxel::strain (VX_Voxel.cpp:327), where
// x = 1 + the summed axial strains and y = -poissonsRatio.  For |x - 1| <= 1/2 (all but
// about 1e-3 of the calls in actuated soft creatures) it is exp(y * log x) from two
// series summed far enough for a double within about one unit in the last place:
// log(1+a) = 2 atanh(s), s = a/(2+a), to the s^33 term (s^2 <= 1/9), and exp(z) to the
// z^17 term (|z| <= ln 2); the float rounding of that double equals the rounded
// library result on every one of 5e7 random inputs checked on the host.  Other inputs
// take the library pow, out of line so that its instructions never run for the rest.
__device__ __noinline__ float pow_library(float x, float y) { return d2f(pow(f2d(x), f2d(y))); }
__device__ __forceinline__ float poisson_pow(float x, float y) {
    const double a = f2d(x) - 1.0;
    if (!fp64i::le(fabs(a), 0.5) || !(y <= 0.0f && y >= -1.0f)) return pow_library(x, y);
    const double s = a / (2.0 + a);
    const double w = s * s;
    double p = 1.0 / 33;
    p = fma(p, w, 1.0 / 31); p = fma(p, w, 1.0 / 29); p = fma(p, w, 1.0 / 27); p = fma(p, w, 1.0 / 25);
    p = fma(p, w, 1.0 / 23); p = fma(p, w, 1.0 / 21); p = fma(p, w, 1.0 / 19); p = fma(p, w, 1.0 / 17);
    p = fma(p, w, 1.0 / 15); p = fma(p, w, 1.0 / 13); p = fma(p, w, 1.0 / 11); p = fma(p, w, 1.0 / 9);
    p = fma(p, w, 1.0 / 7); p = fma(p, w, 1.0 / 5); p = fma(p, w, 1.0 / 3); p = fma(p, w, 1.0);
    const double z = f2d(y) * (mul2(s) * p);
    double e = 1.0 / 355687428096000.0;                               // 1/17!
    e = fma(e, z, 1.0 / 20922789888000.0); e = fma(e, z, 1.0 / 1307674368000.0);
    e = fma(e, z, 1.0 / 87178291200.0); e = fma(e, z, 1.0 / 6227020800.0); e = fma(e, z, 1.0 / 479001600.0);
    e = fma(e, z, 1.0 / 39916800.0); e = fma(e, z, 1.0 / 3628800.0); e = fma(e, z, 1.0 / 362880.0);
    e = fma(e, z, 1.0 / 40320.0); e = fma(e, z, 1.0 / 5040.0); e = fma(e, z, 1.0 / 720.0); e = fma(e, z, 1.0 / 120.0);
    e = fma(e, z, 1.0 / 24.0); e = fma(e, z, 1.0 / 6.0); e = fma(e, z, 0.5); e = fma(e, z, 1.0); e = fma(e, z, 1.0);
    return d2f(e);
}

// The Poisson power of CVX_Voxel::strain (VX_Voxel.cpp:327): pow(float, float), i.e. the C
// library's powf, which is not correctly rounded (about 6e-4 of its results are the other
// neighbour of the exact power).  The engine tabulates the host C library's powf(x, -nu)
// for every float x in [0.5, 2) per Poisson ratio, so the step reads the reference's value
// itself; other x (strains beyond -50% / +100%) take the series above.
__device__ __forceinline__ float poisson_power(const VMat& m, float x) {
    const uint32_t k = fp64i::fbits(x) - kPowTabFirst;
    if (m.powtab && k < kPowTabSize) return __ldg(m.powtab + k);
    return poisson_pow(x, -m.nu);
}

// CVX_Voxel::baseSize(axis) and baseSizeAverage  Voxelyze3/src/old/VX_Voxel.h:91-92
__device__ __forceinline__ double base_size(const VMat& m, float temp) { return m.nom * f2d(1 + temp * m.cte); }
__device__ __forceinline__ double base_size_avg(const VMat& m, float temp) {
    double b = base_size(m, temp);
    return (b + b + b) / 3.0f;
}
// CVX_Voxel::transverseArea  VX_Voxel.cpp:360-373  (psa, psb: the two transverse Poisson strains)
__device__ __forceinline__ float voxel_tarea(const VMat& m, float psa, float psb) {
    float size = m.sizef;
    if (m.nu == 0) return size * size;
    return d2f(f2d(size * size) * (1 + f2d(psa)) * (1 + f2d(psb)));
}
// CVX_Voxel::transverseStrainSum  VX_Voxel.cpp:345-358
__device__ __forceinline__ float voxel_tss(const VMat& m, float psa, float psb) {
    if (m.nu == 0) return 0;
    return psa + psb;
}

}  // namespace GVX_KNS
}  // namespace gvx
