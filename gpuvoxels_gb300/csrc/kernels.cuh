// Step kernels.  One step of every running simulation is three launches
// (links, contacts when any simulation collides, voxels).  Each launch is a
// persistent-style grid whose blocks pull work items (simulation, element
// range) from a queue with an atomic ticket, so thousands of uneven
// simulations share one launch with no per-simulation launch overhead.
#pragma once
#include "physics.cuh"

namespace gvx {
namespace GVX_KNS {

constexpr float HB_TURN = 1.2f * 0.05f;   // HYSTERESIS_FACTOR*SA_BOND_BEND_RAD (types.h:57-58)
constexpr float HB_EXT = 1.2f * 0.50f;    // HYSTERESIS_FACTOR*SA_BOND_EXT_PERC (types.h:57-59)

__device__ __forceinline__ int claim(int* ticket, int* s_item) {
    __syncthreads();
    if (threadIdx.x == 0) *s_item = atomicAdd(ticket, 1);
    __syncthreads();
    return *s_item;
}

// Beam forces and moments of both ends in the link frame, with the local damping
// when the previous state is valid (VX_Link.cpp:167-215).  The float beam constants
// enter as exactly widened doubles (b1*pos2.y is float*double in the reference).
//
// The two angle modes leave exact zeros in the operands, and the terms they meet are
// settled on the integer pipes with bit-identical results (zero_plus, zero_minus,
// minus_zero, times_zero):
//  * small angle (kSmall): angle1v is (0,0,0); with a valid previous state the
//    previous step was small too, so its angle1v and the difference d1 are zero;
//  * large angle: pos2.y, pos2.z and angle1v.x are zero (the relative position was
//    rotated onto +x by an angle whose x component is 0); with a valid previous
//    state the same holds for the previous step, so dP.y, dP.z and d1.x are zero.
// (A mode switch clears the valid-previous-state flag, VX_Link.cpp:85-94.)
template <bool kSmall>
__device__ __forceinline__ void beam_forces(const LMat& m, double fx, const d3& pos2, const d3& a1v, const d3& a2v, const d3& o2,
                                            const d3& oa1, const d3& oa2, bool lvv, double dmN, double dmP, d3* fN_, d3* fP_, d3* mN_,
                                            d3* mP_) {
    const double b1 = m.b1D, b2 = m.b2D, b3 = m.b3D, a2 = m.a2D;
    d3 fN, fP, mN, mP;
    if (kSmall) {
        // a1v + x = zero_plus(a1v, x);  x - a1v.x = x;  a1v.x - x = zero_minus(a1v.x, x)
        fN = D3(fx, b1 * pos2.y - b2 * zero_plus(a1v.z, a2v.z), b1 * pos2.z + b2 * zero_plus(a1v.y, a2v.y));
        mN = D3(a2 * minus_zero(a2v.x, a1v.x), -b2 * pos2.z - b3 * zero_plus(mul2(a1v.y), a2v.y),
                b2 * pos2.y - b3 * zero_plus(mul2(a1v.z), a2v.z));
        mP = D3(a2 * zero_minus(a1v.x, a2v.x), -b2 * pos2.z - b3 * zero_plus(a1v.y, mul2(a2v.y)),
                b2 * pos2.y - b3 * zero_plus(a1v.z, mul2(a2v.z)));
    } else {
        // b*pos2.y and b*pos2.z are zeros; so is a1v.x
        const double zy1 = times_zero(b1, pos2.y), zz1 = times_zero(b1, pos2.z);
        const double zz2 = times_zero(-b2, pos2.z), zy2 = times_zero(b2, pos2.y);
        fN = D3(fx, zero_minus(zy1, b2 * (a1v.z + a2v.z)), zero_plus(zz1, b2 * (a1v.y + a2v.y)));
        mN = D3(a2 * minus_zero(a2v.x, a1v.x), zero_minus(zz2, b3 * (mul2(a1v.y) + a2v.y)), zero_minus(zy2, b3 * (mul2(a1v.z) + a2v.z)));
        mP = D3(a2 * zero_minus(a1v.x, a2v.x), zero_minus(zz2, b3 * (a1v.y + mul2(a2v.y))), zero_minus(zy2, b3 * (a1v.z + mul2(a2v.z))));
    }
    fP = D3(-fN.x, -fN.y, -fN.z);
    if (lvv) {
        const double sqA1 = m.sqA1D, sqA2xIp = m.sqA2xIpD, sqB1 = m.sqB1D, sqB2xFMp = m.sqB2xFMpD, sqB3xIp = m.sqB3xIpD;
        const d3 d2 = D3(half(a2v.x - oa2.x), half(a2v.y - oa2.y), half(a2v.z - oa2.z));
        d3 dP, d1, pc, tN, tP;
        if (kSmall) {
            dP = D3(half(pos2.x - o2.x), half(pos2.y - o2.y), half(pos2.z - o2.z));
            d1 = D3(half(minus_zero(a1v.x, oa1.x)), half(minus_zero(a1v.y, oa1.y)), half(minus_zero(a1v.z, oa1.z)));   // zeros
            pc = D3(sqA1 * dP.x, sqB1 * dP.y - sqB2xFMp * zero_plus(d1.z, d2.z), sqB1 * dP.z + sqB2xFMp * zero_plus(d1.y, d2.y));
            const double ddx = minus_zero(d2.x, d1.x);
            tN = D3(-sqA2xIp * ddx, sqB2xFMp * dP.z + sqB3xIp * zero_plus(mul2(d1.y), d2.y), -sqB2xFMp * dP.y + sqB3xIp * zero_plus(mul2(d1.z), d2.z));
            tP = D3(sqA2xIp * ddx, sqB2xFMp * dP.z + sqB3xIp * zero_plus(d1.y, mul2(d2.y)), -sqB2xFMp * dP.y + sqB3xIp * zero_plus(d1.z, mul2(d2.z)));
        } else {
            dP = D3(half(pos2.x - o2.x), half(minus_zero(pos2.y, o2.y)), half(minus_zero(pos2.z, o2.z)));   // y, z zeros
            d1 = D3(half(minus_zero(a1v.x, oa1.x)), half(a1v.y - oa1.y), half(a1v.z - oa1.z));                  // x zero
            pc = D3(sqA1 * dP.x, zero_minus(times_zero(sqB1, dP.y), sqB2xFMp * (d1.z + d2.z)),
                    zero_plus(times_zero(sqB1, dP.z), sqB2xFMp * (d1.y + d2.y)));
            const double ddx = minus_zero(d2.x, d1.x);
            const double sz = times_zero(sqB2xFMp, dP.z), sy = times_zero(-sqB2xFMp, dP.y);
            tN = D3(-sqA2xIp * ddx, zero_plus(sz, sqB3xIp * (mul2(d1.y) + d2.y)), zero_plus(sy, sqB3xIp * (mul2(d1.z) + d2.z)));
            tP = D3(sqA2xIp * ddx, zero_plus(sz, sqB3xIp * (d1.y + mul2(d2.y))), zero_plus(sy, sqB3xIp * (d1.z + mul2(d2.z))));
        }
        fN = D3(fN.x + dmN * pc.x, fN.y + dmN * pc.y, fN.z + dmN * pc.z);
        fP = D3(fP.x - dmP * pc.x, fP.y - dmP * pc.y, fP.z - dmP * pc.z);
        const double hN = half(dmN), hP = half(dmP);
        mN = D3(mN.x - hN * tN.x, mN.y - hN * tN.y, mN.z - hN * tN.z);
        mP = D3(mP.x - hP * tP.x, mP.y - hP * tP.y, mP.z - hP * tP.z);
    }
    *fN_ = fN; *fP_ = fP; *mN_ = mN; *mP_ = mP;
}

// CVX_Link::updateForces with orientLink, updateStrain and updateTransverseInfo
// (Voxelyze3/src/old/VX_Link.cpp:72-113, 136-141, 143-241), in two parts: link_orient
// (orientLink up to the small/large-angle hysteresis test) and link_finish (the rest),
// which writes the two end forces/moments and axial strains into the voxels' direction
// slots.  A link's pose in its own frame and its mode for this step:
struct LinkOrient {
    d3 pos2;          // positive end relative to the negative end, in the negative end's frame on +x
    q4 angle2;        // positive end's orientation in that frame
    double restLen;   // CVX_Link::updateRestLength
    bool small, lvv;  // small-angle mode and valid previous state for this step
    bool switched;    // the mode differs from the previous step's
};

// False for a link that is not updated (detached or removed, or between two Fixed voxels).
__device__ __forceinline__ bool link_orient(const Sim& S, int l, LinkOrient* out) {
    const int ng = __ldg(S.lneg + l), pv = __ldg(S.lpos + l);
    const int axis = __ldg(S.lax + l);
    const VMat& vN = S.vm[__ldg(S.vmat + ng)];
    const VMat& vP = S.vm[__ldg(S.vmat + pv)];
    const uint8_t fl = S.lfl[l];
    // VX3 extras: detached and removed links are no longer updated (VX3_VoxelyzeKernel.cu:565-575),
    // nor are links between two voxels of Fixed materials
    if (fl & LF_GONE) return false;
    if ((S.flags & SF_FIXEDMAT) && (vN.vx3 & vP.vx3 & VM_FIXED)) return false;
    const float tN = S.temp[ng], tP = S.temp[pv];
    const double restLen = half(base_size(vN, tN) + base_size(vP, tP));   // CVX_Link::updateRestLength
    bool small = fl & LF_SMALL, lvv = fl & LF_LVV;

    // orientLink
    d3 pos2 = to_axis_x(axis, D3(S.px[pv] - S.px[ng], S.py[pv] - S.py[ng], S.pz[pv] - S.pz[ng]));
    q4 angle1 = q_to_axis_x(axis, Q4(S.qw[ng], S.qx[ng], S.qy[ng], S.qz[ng]));
    q4 angle2 = q_to_axis_x(axis, Q4(S.qw[pv], S.qx[pv], S.qy[pv], S.qz[pv]));
    const q4 tr = Q4(angle1.w, -angle1.x, -angle1.y, -angle1.z);
    pos2 = qrot(tr, pos2);
    angle2 = qmul(tr, angle2);
    // SmallTurn = (float)((|z|+|y|)/x), ExtendPerc = (float)|1 - x/restLength|, compared with the
    // hysteresis thresholds (VX_Link.cpp:85-94); decided without dividing unless near a threshold
    const double turnNum = fabs(pos2.z) + fabs(pos2.y);
    if (!small) {
        if (quot_lt(turnNum, pos2.x, 0.05f) && ext_lt(pos2.x, restLen, 0.50f)) { small = true; lvv = false; }
    } else if (quot_gt(turnNum, pos2.x, HB_TURN) || ext_gt(pos2.x, restLen, HB_EXT)) {
        small = false;
        lvv = false;
    }
    out->pos2 = pos2; out->angle2 = angle2; out->restLen = restLen; out->small = small; out->lvv = lvv;
    out->switched = small != ((fl & LF_SMALL) != 0);
    return true;
}

// The rest of CVX_Link::updateForces for a link oriented by link_orient.
__device__ __forceinline__ void link_finish(const Sim& S, int l, float dt, const LinkOrient& lo, bool* diverged) {
    const int ng = __ldg(S.lneg + l), pv = __ldg(S.lpos + l);
    const int axis = __ldg(S.lax + l);
    const LMat& m = S.lm[__ldg(S.lmt + l)];
    const VMat& vN = S.vm[__ldg(S.vmat + ng)];
    const VMat& vP = S.vm[__ldg(S.vmat + pv)];
    const double restLen = lo.restLen;
    const int nl = S.nl;
    double* st = S.lst;
    const d3 o2 = D3(st[l], st[nl + l], st[2 * nl + l]);
    const d3 oa1 = D3(st[3 * nl + l], st[4 * nl + l], st[5 * nl + l]);
    const d3 oa2 = D3(st[6 * nl + l], st[7 * nl + l], st[8 * nl + l]);
    float strain = S.lsf[l], maxStrain = S.lsf[nl + l], strainOffset = S.lsf[2 * nl + l];
    bool small = lo.small, lvv = lo.lvv;
    d3 pos2 = lo.pos2;
    q4 angle2 = lo.angle2;
    q4 angle1 = Q4(1, 0, 0, 0);
    d3 a1v;
    bool wide1 = false, acos1 = false, wide2 = false;   // branches taken, kept as the next step's ordering key
    if (small) {
        pos2.x -= restLen;
        a1v = D3(0, 0, 0);                  // ToRotationVector of the identity
    } else {
        // pos2.Length(), used by FromAngleToPosX's general branch and for the axial position
        const double len = sqrt(pos2.x * pos2.x + pos2.y * pos2.y + pos2.z * pos2.z);
        angle1 = q_from_angle_to_posx(angle1, pos2, len, &wide1);
        angle2 = qmul_x0(angle1, angle2);
        pos2 = D3(len - restLen, 0, 0);
        a1v = q_to_rotvec<true>(angle1, &acos1);
    }
    const d3 a2v = q_to_rotvec(angle2, &wide2);
    st[l] = pos2.x; st[nl + l] = pos2.y; st[2 * nl + l] = pos2.z;
    st[3 * nl + l] = a1v.x; st[4 * nl + l] = a1v.y; st[5 * nl + l] = a1v.z;
    st[6 * nl + l] = a2v.x; st[7 * nl + l] = a2v.y; st[8 * nl + l] = a2v.z;

    // updateTransverseInfo (the CPU path refreshes it every step when nu != 0)
    float A, tss;
    if (m.nu != 0.0f) {
        const int nv = S.nv;
        float nx = S.ps[ng], ny = S.ps[nv + ng], nz = S.ps[2 * nv + ng];
        float px_ = S.ps[pv], py_ = S.ps[nv + pv], pz_ = S.ps[2 * nv + pv];
        float na, nb, pa, pb;
        if (axis == 0) { na = ny; nb = nz; pa = py_; pb = pz_; }
        else if (axis == 1) { na = nx; nb = nz; pa = px_; pb = pz_; }
        else { na = nx; nb = ny; pa = px_; pb = py_; }
        A = 0.5f * (voxel_tarea(vN, na, nb) + voxel_tarea(vP, pa, pb));
        tss = 0.5f * (voxel_tss(vN, na, nb) + voxel_tss(vP, pa, pb));
    } else {
        A = 0.5f * (voxel_tarea(vN, 0.f, 0.f) + voxel_tarea(vP, 0.f, 0.f));
        tss = 0.0f;
    }

    // updateStrain
    const float axial = d2f(pos2.x / restLen);
    float stress;
    strain = axial;
    if (m.linear) {
        if (axial > maxStrain) maxStrain = axial;
        stress = mat_stress(m, axial, tss, false);
    } else if (axial > maxStrain) {
        maxStrain = axial;
        stress = mat_stress(m, axial, tss, false);
        if (m.nu != 0.0f) strainOffset = maxStrain - mat_stress(m, axial, 0.0f, false) / (m.eHat * (1 - m.nu));
        else strainOffset = maxStrain - stress / m.E;
    } else {
        const float rel = axial - strainOffset;
        stress = (m.nu != 0.0f) ? mat_stress(m, rel, tss, true) : m.E * rel;
    }
    if (strain > 100) *diverged = true;
    S.lsf[l] = strain; S.lsf[nl + l] = maxStrain; S.lsf[2 * nl + l] = strainOffset;

    d3 fN, fP, mN, mP;
    const bool failed = m.epsFail != -1.0f && maxStrain > m.epsFail;
    if (failed) {
        fN = fP = mN = mP = D3(0, 0, 0);
    } else {
        const float dmNf = vN.dampNum / dt, dmPf = vP.dampNum / dt;   // CVX_Voxel::dampingMultiplier
        if (small) {
            beam_forces<true>(m, f2d(stress * A), pos2, a1v, a2v, o2, oa1, oa2, lvv, f2d(dmNf), f2d(dmPf), &fN, &fP, &mN, &mP);
        } else {
            beam_forces<false>(m, f2d(stress * A), pos2, a1v, a2v, o2, oa1, oa2, lvv, f2d(dmNf), f2d(dmPf), &fN, &fP, &mN, &mP);
            fN = qrotinv_x0(angle1, fN);
            mN = qrotinv_x0(angle1, mN);
        }
        lvv = true;
        fP = qrotinv(angle2, fP);
        mP = qrotinv(angle2, mP);
        fN = to_axis_orig(axis, fN); fP = to_axis_orig(axis, fP);
        mN = to_axis_orig(axis, mN); mP = to_axis_orig(axis, mP);
        if (S.lnew && S.lnew[l] > 0) {
            // VX3 attachment: a new link acts at 1% for its first SafetyGuard updates (VX3_Link.cu:206-213)
            fN = D3(fN.x * 0.01, fN.y * 0.01, fN.z * 0.01); fP = D3(fP.x * 0.01, fP.y * 0.01, fP.z * 0.01);
            mN = D3(mN.x * 0.01, mN.y * 0.01, mN.z * 0.01); mP = D3(mP.x * 0.01, mP.y * 0.01, mP.z * 0.01);
            S.lnew[l] -= 1;
        }
    }
    uint8_t gone = 0;
    if (failed && (S.flags & SF_DETACH)) {
        // VX3 updateDetach (VX3_VoxelyzeKernel.cu:946-968): the failed link leaves both voxels'
        // link lists (before this step's voxel update) and both become surface voxels
        atomicAnd(&S.vfl[ng], ~((1u << (2 * axis)) | VF_INTERIOR));
        atomicAnd(&S.vfl[pv], ~((1u << (2 * axis + 1)) | VF_INTERIOR));
        gone = LF_GONE;
    }
    S.lfl[l] = (uint8_t)((small ? LF_SMALL : 0) | (lvv ? LF_LVV : 0) | (wide1 ? LF_WIDE1 : 0) | (wide2 ? LF_WIDE2 : 0) |
                         (acos1 ? LF_ACOS1 : 0) | gone);

    // direction slots: the negative-end voxel sees this link in direction 2*axis,
    // the positive-end voxel in direction 2*axis+1 (CVX_Voxel::force, VX_Voxel.cpp:236-238)
    const int nv = S.nv;
    const int dn = 2 * axis, dp = 2 * axis + 1;
    double* sf = S.sf;
    double* sm = S.sm;
    sf[(dn * 3 + 0) * nv + ng] = fN.x; sf[(dn * 3 + 1) * nv + ng] = fN.y; sf[(dn * 3 + 2) * nv + ng] = fN.z;
    sm[(dn * 3 + 0) * nv + ng] = mN.x; sm[(dn * 3 + 1) * nv + ng] = mN.y; sm[(dn * 3 + 2) * nv + ng] = mN.z;
    sf[(dp * 3 + 0) * nv + pv] = fP.x; sf[(dp * 3 + 1) * nv + pv] = fP.y; sf[(dp * 3 + 2) * nv + pv] = fP.z;
    sm[(dp * 3 + 0) * nv + pv] = mP.x; sm[(dp * 3 + 1) * nv + pv] = mP.y; sm[(dp * 3 + 2) * nv + pv] = mP.z;
    // CVX_Link::axialStrain(positiveEnd)  VX_Link.cpp:115-118
    const float ratio = vP.E / vN.E;
    S.ss[dn * nv + ng] = 2.0f * strain / (1.0f + ratio);
    S.ss[dp * nv + pv] = 2.0f * strain * ratio / (1.0f + ratio);
}

// Work-item elements in an order that keeps warps on one code path.  GB300's FP64
// pipe spends the same cycles on a warp instruction whatever its active lanes, so a
// warp whose lanes take different branches pays for every branch.  Elements are
// grouped by a small key describing the branches they took in the previous step
// (paths change rarely from one step to the next); the partition is stable and
// deterministic.  The order never changes results: every link writes only its own
// state and its two direction slots, and voxel work is per voxel.
constexpr int kOrderMax = 1024;   // elements per item that are reordered (larger items run in index order)
constexpr int kOrderKeys = kOrderKeysBins;

// perm[0..n) = element indices grouped by key(j) in increasing key order; wc holds
// kOrderKeys x 8 warp counts.  Every thread of the block must call it.
template <typename KeyFn>
__device__ __forceinline__ void order_by_key(int n, KeyFn key, int* perm, int* wc) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    int start[kOrderKeys];
    for (int k = 0; k < kOrderKeys; k++) start[k] = 0;
    // pass 1: group sizes
    for (int j0 = 0; j0 < n; j0 += blockDim.x) {
        const int j = j0 + threadIdx.x;
        const int kj = j < n ? key(j) : -1;
#pragma unroll
        for (int k = 0; k < kOrderKeys; k++) {
            const unsigned b = __ballot_sync(0xffffffffu, kj == k);
            if (lane == 0) wc[k * 8 + wid] = __popc(b);
        }
        __syncthreads();
        for (int k = 0; k < kOrderKeys; k++)
            for (int q = 0; q < nw; q++) start[k] += wc[k * 8 + q];
        __syncthreads();
    }
    // group starts
    int acc = 0;
    for (int k = 0; k < kOrderKeys; k++) { const int c = start[k]; start[k] = acc; acc += c; }
    // pass 2: place
    for (int j0 = 0; j0 < n; j0 += blockDim.x) {
        const int j = j0 + threadIdx.x;
        const int kj = j < n ? key(j) : -1;
        unsigned mine = 0;
#pragma unroll
        for (int k = 0; k < kOrderKeys; k++) {
            const unsigned b = __ballot_sync(0xffffffffu, kj == k);
            if (kj == k) mine = b;
            if (lane == 0) wc[k * 8 + wid] = __popc(b);
        }
        __syncthreads();
        if (kj >= 0) {
            int p = start[kj] + __popc(mine & below);
            for (int q = 0; q < wid; q++) p += wc[kj * 8 + q];
            perm[p] = j;
        }
        for (int k = 0; k < kOrderKeys; k++)
            for (int q = 0; q < nw; q++) start[k] += wc[k * 8 + q];
        __syncthreads();
    }
}

// Link key: small-angle mode, then within each mode which rotation branches were taken
// (small links: angle2's rotation-vector branch; large links: that, angle1's, and
// FromAngleToPosX's).  10 groups, the costliest first (large links taking every
// acos/sincos branch are key 0, plain small links key 9).
struct LinkKey {
    const uint8_t* lfl;
    int begin;
    __device__ int operator()(int j) const {
        const uint8_t f = lfl[begin + j];
        if (f & LF_SMALL) return (f & LF_WIDE2) ? 8 : 9;
        return 7 - (((f & LF_WIDE1) ? 4 : 0) | ((f & LF_ACOS1) ? 2 : 0) | ((f & LF_WIDE2) ? 1 : 0));
    }
};

// Voxel key: touched the floor last step (contact and friction branches) and, if so,
// held by static friction (the kinetic branch forms the sliding direction), then
// surface voxels (Poisson strain by pow) apart from interior ones.
// Voxel key: floor contact with kinetic (0, 1) or static (2, 3) friction, else surface
// (4, 6) or interior (5, 7) voxel; the lower key of each pair when the last orientation
// update took the sin/cos branch.  (Voxels touching the floor are not told apart by
// interior: they are almost always surface voxels.)
struct VoxelKey {
    const uint32_t* vfl;
    int begin;
    __device__ int operator()(int j) const {
        const uint32_t f = vfl[begin + j];
        const int narrow = (f & VF_WROT) ? 0 : 1;
        if (f & VF_FLOORC) return ((f & VF_STATIC) ? 2 : 0) + narrow;
        return 4 + 2 * narrow + ((f & VF_INTERIOR) ? 1 : 0);
    }
};

// Grouping key of element j of a work item starting at `begin`: links (kind 0) or voxels (kind 1).
__device__ __forceinline__ int bin_key(const Sim& S, int kind, int begin, int j) {
    return kind == 0 ? LinkKey{S.lfl, begin}(j) : VoxelKey{S.vfl, begin}(j);
}

// Resident blocks per SM the register allocation of k_links / k_voxels is sized for
// (a build-time tuning knob: -DGVX_LINKS_MIN_BLOCKS=3 trades registers for warps).
#ifndef GVX_STEP_BLOCK
#define GVX_STEP_BLOCK 256   // largest block of k_links / k_voxels (the register budget is sized for it)
#endif
#ifndef GVX_LINKS_MIN_BLOCKS
#define GVX_LINKS_MIN_BLOCKS 2
#endif
#ifndef GVX_VOXELS_MIN_BLOCKS
#define GVX_VOXELS_MIN_BLOCKS 2
#endif

// ---------------------------------------------------------------- link binning
// Every few steps the links of every running simulation are grouped by key within
// windows of consecutive work items (three small passes: key counts per item, their
// exclusive scan, a stable scatter of (simulation, link) pairs); keys change slowly,
// so the grouping is reused for the steps in between.  Every
// warp of k_links then runs one code path, and warps take 32-link chunks from one
// queue in window order: no block barriers, no tail of uneven work items, and the
// link state of a window (a few MB) stays in L2 while its key groups are processed.
// (Earlier forms ordered each 256-link item inside its block, between block
// barriers: warps of cheap small-angle links waited for warps of costly large-angle
// ones.  Grouping across the whole batch at once made every key group a separate
// pass over all link state and tripled k_links' DRAM traffic.)
__global__ void __launch_bounds__(256) k_bin_hist(const Sim* __restrict__ sims, const Ctl* __restrict__ ctl, BinList la, BinList lb) {
    __shared__ int wc[kOrderKeys * 8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int g = blockIdx.x; g < la.n_items + lb.n_items; g += gridDim.x) {
        const bool first = g < la.n_items;       // the two lists' items share the grid
        const int it = first ? g : g - la.n_items;
        const int kind = first ? la.kind : lb.kind;
        int* hist = first ? la.hist : lb.hist;
        const Item w = (first ? la.items : lb.items)[it];
        const bool run = ctl[w.sim].status == 1;
        const Sim& S = sims[w.sim];
        const int n = w.end - w.begin;
        int cnt = 0;   // thread k < kOrderKeys: elements of key k
        for (int j0 = 0; j0 < n; j0 += blockDim.x) {
            const int j = j0 + threadIdx.x;
            const int kj = (run && j < n) ? bin_key(S, kind, w.begin, j) : -1;
#pragma unroll
            for (int k = 0; k < kOrderKeys; k++) {
                const unsigned b = __ballot_sync(0xffffffffu, kj == k);
                if (lane == 0) wc[k * 8 + wid] = __popc(b);
            }
            __syncthreads();
            if (threadIdx.x < kOrderKeys)
                for (int q = 0; q < nw; q++) cnt += wc[threadIdx.x * 8 + q];
            __syncthreads();
        }
        if (threadIdx.x < kOrderKeys) hist[(size_t)it * kOrderKeys + threadIdx.x] = cnt;
    }
}

// One block: an exclusive scan of the per-item key counts taken window by window, key
// by key, item by item, so base[item][key] = links of earlier windows + links of
// smaller keys in the window + links of that key in earlier items of the window.
// Each thread scans a contiguous run of that order; the runs are joined by a block scan.
__global__ void __launch_bounds__(1024) k_bin_scan(BinList la, BinList lb) {
    __shared__ int s_sum[1024];
    const BinList& L = blockIdx.x == 0 ? la : lb;   // one block per list
    const int* hist = L.hist;
    int* base = L.base;
    const int n_items = L.n_items, win = L.win;
    int* total = L.total;
    const int n_win = (n_items + win - 1) / win;
    const int N = n_win * win * kOrderKeys;
    const int per = (N + blockDim.x - 1) / blockDim.x;
    const int e0 = min(N, (int)threadIdx.x * per), e1 = min(N, e0 + per);
    auto item_of = [win](int e, int* k) {
        const int w = e / (win * kOrderKeys), r = e - w * (win * kOrderKeys);
        *k = r / win;
        return w * win + (r - *k * win);
    };
    int sum = 0;
    for (int e = e0; e < e1; e++) {
        int k;
        const int it = item_of(e, &k);
        if (it < n_items) sum += hist[(size_t)it * kOrderKeys + k];
    }
    s_sum[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {   // inclusive scan of the runs' sums
        const int v = (int)threadIdx.x >= off ? s_sum[threadIdx.x - off] : 0;
        __syncthreads();
        s_sum[threadIdx.x] += v;
        __syncthreads();
    }
    int run = threadIdx.x ? s_sum[threadIdx.x - 1] : 0;
    for (int e = e0; e < e1; e++) {
        int k;
        const int it = item_of(e, &k);
        if (it < n_items) {
            base[(size_t)it * kOrderKeys + k] = run;
            run += hist[(size_t)it * kOrderKeys + k];
        }
    }
    if (threadIdx.x == blockDim.x - 1) *total = s_sum[blockDim.x - 1];
}

__global__ void __launch_bounds__(256) k_bin_scatter(const Sim* __restrict__ sims, const Ctl* __restrict__ ctl, BinList la, BinList lb) {
    __shared__ int wc[kOrderKeys * 8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    for (int g = blockIdx.x; g < la.n_items + lb.n_items; g += gridDim.x) {
        const bool first = g < la.n_items;
        const int it = first ? g : g - la.n_items;
        const int kind = first ? la.kind : lb.kind;
        const int* base = first ? la.base : lb.base;
        int2* perm = first ? la.perm : lb.perm;
        const Item w = (first ? la.items : lb.items)[it];
        if (ctl[w.sim].status != 1) continue;   // the same for the whole block
        const Sim& S = sims[w.sim];
        int start[kOrderKeys];
        for (int k = 0; k < kOrderKeys; k++) start[k] = base[(size_t)it * kOrderKeys + k];
        const int n = w.end - w.begin;
        for (int j0 = 0; j0 < n; j0 += blockDim.x) {
            const int j = j0 + threadIdx.x;
            const int kj = j < n ? bin_key(S, kind, w.begin, j) : -1;
            unsigned mine = 0;
#pragma unroll
            for (int k = 0; k < kOrderKeys; k++) {
                const unsigned b = __ballot_sync(0xffffffffu, kj == k);
                if (kj == k) mine = b;
                if (lane == 0) wc[k * 8 + wid] = __popc(b);
            }
            __syncthreads();
            if (kj >= 0) {
                int p = start[kj] + __popc(mine & below);
                for (int q = 0; q < wid; q++) p += wc[kj * 8 + q];
                perm[p] = make_int2(w.sim, w.begin + j);
            }
            for (int k = 0; k < kOrderKeys; k++)
                for (int q = 0; q < nw; q++) start[k] += wc[k * 8 + q];
            __syncthreads();
        }
    }
}

// Warps take chunks of `claim` consecutive links of the binned list (one atomic per
// chunk; claim is a multiple of 32) and update them 32 at a time, one per lane.
// The grouping keys come from the previous step, so a link that changes between small-
// and large-angle mode this step sits among links of the other mode, and its warp would
// run both paths (on GB300 the FP64 pipe spends the same cycles on a warp instruction
// whatever its active lanes).  While many links change mode (a fresh batch's first tens of
// steps: more than 1 in 256 links did in the previous step) and every warp has many rounds
// to fill its queues with (at least 256 links per resident warp), each round first orients
// the 32 links and decides their modes; the minority mode waits in
// the warp's queue for that mode (its links' ids only) while the majority finishes, and a
// queue that holds 32 links is run as one full round of a single mode: its links are
// oriented again (the same inputs give the same pose and mode) and finished.  What is
// left in the queues at the end runs in one last round per mode.  When few links change
// mode, or a warp has few rounds, the queues would rarely fill and the last rounds would
// run nearly empty, so every link is finished in its own round.  Every link still writes only its own state and its
// two direction slots, so the order changes no result.  tickets[5] counts this launch's
// mode changes; k_voxels moves the count to tickets[6] for the next step's decision.
constexpr int kLinkDefer = 48;          // a queue holds at most 31 + 16 links between rounds
constexpr int kDeferPerWarp = 256;      // queues only with at least this many links per resident warp
constexpr int kDeferRate = 256;         // queues while more than 1 link in kDeferRate changed mode
__global__ void __launch_bounds__(GVX_STEP_BLOCK, GVX_LINKS_MIN_BLOCKS) k_links(const Sim* __restrict__ sims, Ctl* ctl, const int2* __restrict__ perm,
                                                                     const int* __restrict__ total, int cap, int n_slots, int* tickets,
                                                                     int claim) {
    __shared__ int2 s_defer[GVX_STEP_BLOCK / 32][2][kLinkDefer];   // per warp: large-angle (0), small-angle (1)
    // this step's queues of the kernels that follow, and the contact spill pool's records
    if (blockIdx.x == 0 && threadIdx.x == 0) { tickets[1] = 0; tickets[2] = 0; tickets[3] = 0; tickets[4] = 0; }
    const int n = min(*total, cap);
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    int2* q0 = s_defer[threadIdx.x >> 5][0];
    int2* q1 = s_defer[threadIdx.x >> 5][1];
    int qn0 = 0, qn1 = 0;        // links waiting in each queue (the same in every lane)
    const bool queues = (long long)n >= (long long)kDeferPerWarp * (gridDim.x * (blockDim.x / 32)) &&
                        (long long)tickets[6] * kDeferRate > (long long)n;
    int switched = 0;            // mode changes seen by this warp
    int kb = 0, k1 = 0;          // the claimed chunk: next round's first link, its end
    bool more = true;            // chunks may remain
    for (;;) {
        // this round's links: a full queue, else the claimed chunk (claiming one when it is
        // used up), else what the queues hold at the end
        int src, cnt = 32;       // src: -1 the chunk, 0 / 1 a queue
        if (qn0 >= 32) src = 0;
        else if (qn1 >= 32) src = 1;
        else {
            if (kb >= k1 && more) {
                int chunk = 0;
                if (lane == 0) chunk = atomicAdd(&tickets[0], 1);
                chunk = __shfl_sync(0xffffffffu, chunk, 0);
                kb = chunk * claim;
                k1 = min(n, kb + claim);
                if (kb >= n) more = false;
            }
            if (kb < k1) src = -1;
            else if (qn0 > 0) { src = 0; cnt = qn0; }
            else if (qn1 > 0) { src = 1; cnt = qn1; }
            else break;
        }
        int2 e = make_int2(-1, -1);
        if (src < 0) {
            if (kb + lane < k1) e = __ldg(perm + kb + lane);
            kb += 32;
        } else {
            int2* q = src ? q1 : q0;
            const int left = (src ? qn1 : qn0) - cnt;   // at most 15 after a full round, else 0
            if (lane < cnt) e = q[lane];
            __syncwarp();
            if (lane < left) q[lane] = q[cnt + lane];
            __syncwarp();
            if (src) qn1 = left; else qn0 = left;
        }
        // e.x >= n_slots never happens (the grouping lists running slots); a simulation may
        // have stopped since the grouping was made
        bool act = e.x >= 0 && (unsigned)e.x < (unsigned)n_slots && ctl[e.x].status == 1 && (unsigned)e.y < (unsigned)sims[e.x].nl;
        LinkOrient o;
        act = act && link_orient(sims[e.x], e.y, &o);
        if (src < 0) {
            const unsigned am = __ballot_sync(0xffffffffu, act), sm = __ballot_sync(0xffffffffu, act && o.small);
            switched += __popc(__ballot_sync(0xffffffffu, act && o.switched));
            const bool major_small = 2 * __popc(sm) >= __popc(am);
            const bool defer = queues && act && o.small != major_small;
            const unsigned dm = __ballot_sync(0xffffffffu, defer);
            if (dm) {
                // the deferred lanes' mode is the other one: small when the majority is large
                int2* q = major_small ? q0 : q1;
                const int at = major_small ? qn0 : qn1;
                if (defer) q[at + __popc(dm & below)] = e;
                if (major_small) qn0 += __popc(dm); else qn1 += __popc(dm);
                __syncwarp();
            }
            act = act && !defer;
        }
        if (act) {
            Ctl& c = ctl[e.x];
            bool div = false;
            link_finish(sims[e.x], e.y, c.dt, o, &div);
            if (div) c.diverged = 1;
        }
    }
    if (lane == 0 && switched) atomicAdd(&tickets[5], switched);
}

// Overlap test and repelling force for one voxel pair (CVX_Collision::updateContactForce,
// Voxelyze3/src/old/VX_Collision.cpp:17-23, 42-56).  a < b; returns false when apart.
__device__ __forceinline__ bool pair_force(const Sim& S, int a, int b, float* f3) {
    const VMat& ma = S.vm[__ldg(S.vmat + a)];
    const VMat& mb = S.vm[__ldg(S.vmat + b)];
    const float ox = d2f(S.px[b] - S.px[a]), oy = d2f(S.py[b] - S.py[a]), oz = d2f(S.pz[b] - S.pz[a]);
    const float nomDist = d2f((base_size_avg(ma, S.temp[a]) + base_size_avg(mb, S.temp[b])) * S.env_radius);
    const float len = sqrtf(ox * ox + oy * oy + oz * oz);
    const float relDist = nomDist - len;
    if (!(relDist > 0)) return false;
    float ux = ox, uy = oy, uz = oz;
    if (len > 0) { const float inv = 1.0f / len; ux = inv * ox; uy = inv * oy; uz = inv * oz; }
    const double vax = S.mx[a] * ma.massInv, vay = S.my[a] * ma.massInv, vaz = S.mz[a] * ma.massInv;
    const double vbx = S.mx[b] * mb.massInv, vby = S.my[b] * mb.massInv, vbz = S.mz[b] * mb.massInv;
    const double dux = f2d(ux), duy = f2d(uy), duz = f2d(uz);
    const float rv = d2f((vax * dux + vay * duy + vaz * duz) - (vbx * dux + vby * duy + vbz * duz));
    const float k = 2.0f / (1.0f / ma.penStiff + 1.0f / mb.penStiff);
    const float cd = 0.5f * (ma.cDampT + mb.cDampT);
    const float f = k * relDist + cd * rv;
    f3[0] = f * ux; f3[1] = f * uy; f3[2] = f * uz;
    return true;
}

__device__ __forceinline__ uint32_t cell_hash(int cx, int cy, int cz, int mask) {
    return ((uint32_t)cx * 73856093u ^ (uint32_t)cy * 19349663u ^ (uint32_t)cz * 83492791u) & (uint32_t)mask;
}
// The broadphase runs in FP32 on positions rounded to float: it only has to be
// conservative (every pair the exact FP64 test accepts must be found), and the
// same float values give the same cell at insertion and lookup.
__device__ __forceinline__ int cell_of(float p, float inv_cell) { return (int)floorf(p * inv_cell); }

// Records voxel v (position pos, temperature temp) in hash table `head` and its
// float position and base size in cpos for the next contact pass.
__device__ __forceinline__ void hash_insert(const Sim& S, int v, const d3& pos, float temp, int* head) {
    const VMat& m = S.vm[__ldg(S.vmat + v)];
    const float4 p = make_float4(d2f(pos.x), d2f(pos.y), d2f(pos.z), m.sizef * (1.0f + temp * m.cte));
    S.cpos[v] = p;
    const uint32_t h = cell_hash(cell_of(p.x, S.inv_cell), cell_of(p.y, S.inv_cell), cell_of(p.z, S.inv_cell), S.hash_size - 1);
    S.hash_next[v] = atomicExch(head + h, v);
}

// Conservative FP32 overlap test: false only when the exact test (pair_force) cannot
// accept the pair.  2% of the contact distance plus 4 float ulps of every coordinate
// cover the float rounding of positions and base sizes.
__device__ __forceinline__ bool maybe_touching(float4 a, float4 b, float env_radius) {
    const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    const float lim = env_radius * (a.w + b.w) * 1.02f +
                      2.4e-7f * (fabsf(a.x) + fabsf(a.y) + fabsf(a.z) + fabsf(b.x) + fabsf(b.y) + fabsf(b.z));
    return dx * dx + dy * dy + dz * dz <= lim * lim;
}

// First index of each (oz, oy) row of the radius-5 L1 ball enumerated z-major, then y, then
// x (the order of the reach masks, world.cpp l1_ball_offsets); rows outside the ball unused.
struct BallRows {
    int r[11][11];
    constexpr BallRows() : r() {
        int k = 0;
        for (int z = -5; z <= 5; z++) {
            const int rz = 5 - (z < 0 ? -z : z);
            for (int y = -5; y <= 5; y++) {
                const int ay = y < 0 ? -y : y;
                r[z + 5][y + 5] = k;
                if (ay <= rz) k += 2 * (rz - ay) + 1;
            }
        }
    }
};
__constant__ const BallRows kBallRowTable{};
#define kBallRow kBallRowTable.r

// Whether hashed voxel q, found in cell (tx, ty, tz) of the table, is a partner of surface
// voxel v (float position pv, lattice indices vx, vy, vz) in this step's contact list: q
// lies in that cell, is not within 5 lattice links of v (nor linked to it by a link made
// at run time) and overlaps v by the exact test.
__device__ __forceinline__ bool is_contact(const Sim& S, int v, int q, float4 pv, int vx, int vy, int vz, int tx, int ty, int tz) {
    const float ic = S.inv_cell;
    const float4 pq = S.cpos[q];
    if (q == v || cell_of(pq.x, ic) != tx || cell_of(pq.y, ic) != ty || cell_of(pq.z, ic) != tz || !maybe_touching(pv, pq, S.env_radius))
        return false;
    const int nv = S.nv;
    // lattice exclusion: within 5 links of each other
    const int ox = S.ijk[q] - vx, oy = S.ijk[nv + q] - vy, oz = S.ijk[2 * nv + q] - vz;
    const int l1 = abs(ox) + abs(oy) + abs(oz);
    if (l1 == 1) return false;   // lattice neighbours are always linked to each other
    if (l1 <= 5) {
        // index of (ox,oy,oz) in the L1 ball enumerated z-major, then y, then x: the row of
        // (oz, oy) starts at kBallRow, the row spans ox in [-(5-|oz|-|oy|), 5-|oz|-|oy|]
        const int k = kBallRow[oz + 5][oy + 5] + ox + (5 - abs(oz) - abs(oy));
        if ((S.reach[(size_t)v * kReachWords + (k >> 5)] >> (k & 31)) & 1u) return false;
    }
    if (S.flags & SF_ATTACH) {
        // links made at run time join voxels the loaded topology kept apart: voxels linked to
        // each other do not collide (is_neighbor depth 1, VX3_VoxelyzeKernel.cu:697-700)
        const uint32_t fv = S.vfl[v];
        for (int d = 0; d < 6; d++)
            if ((fv >> d) & 1) {
                const int l = S.vlink[6 * v + d];
                if (S.lneg[l] == q || S.lpos[l] == q) return false;
            }
    }
    float f3[3];
    return pair_force(S, v < q ? v : q, v < q ? q : v, f3);
}

// Calls fn(q) for every partner q of surface voxel v in this step's contact list, in no
// particular order: hashed voxels in the 27 cells around v that pass is_contact.
template <typename Fn>
__device__ __forceinline__ void for_each_contact(const Sim& S, int v, int parity, Fn fn) {
    const float4 pv = S.cpos[v];
    const float ic = S.inv_cell;
    const int cx = cell_of(pv.x, ic), cy = cell_of(pv.y, ic), cz = cell_of(pv.z, ic);
    const int nv = S.nv;
    const int vx = S.ijk[v], vy = S.ijk[nv + v], vz = S.ijk[2 * nv + v];
    const int* head = S.hash_head + (size_t)parity * S.hash_size;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int tx = cx + dx, ty = cy + dy, tz = cz + dz;
                int q = head[cell_hash(tx, ty, tz, S.hash_size - 1)];
                int guard = 0;
                while (q >= 0 && guard++ < nv) {
                    const int nq = S.hash_next[q];
                    if (is_contact(S, v, q, pv, vx, vy, vz, tx, ty, tz)) fn(q);
                    q = nq;
                }
            }
}

// Spatial-hash broadphase + exact contact forces for one surface voxel.  The
// reference keeps a conservative pair list of surface voxels that are not
// within 5 lattice links of each other (Voxelyze3/src/old/Voxelyze.cpp:671-751,
// VX_Voxel.cpp:394-417) and sums the pair forces in increasing partner order;
// pairs that do not overlap contribute exactly zero, so summing the
// overlapping pairs in partner order reproduces it.  The list has no length
// limit: up to S.contact_inline (at most kContactInline) contacts go to the
// voxel's own slots; a voxel with more takes a run of records of the spill pool, fills it with its
// partners in a second pass over the hash and sorts them there.
__device__ void voxel_contacts(const Sim& S, int v, int parity, Ctl& c) {
    if (S.flags & SF_DYNSURF) {
        // the surface set changes during the run: every voxel is listed, interior and
        // removed ones have no contacts
        const uint32_t f = S.vfl[v];
        if (f & (VF_INTERIOR | VF_REMOVED)) { S.ccount[v] = 0; return; }
    }
    // the `cap` smallest partners in increasing order, and the number of partners
    const int cap = min(max(S.contact_inline, 1), kContactInline);
    int partners[kContactInline] = {};
    int np = 0, ntot = 0;
    for_each_contact(S, v, parity, [&](int q) {
        ntot++;
        if (np == cap) {
            if (q > partners[cap - 1]) return;
            np--;   // the largest kept partner gives way
        }
        int k = np++;
        while (k > 0 && partners[k - 1] > q) { partners[k] = partners[k - 1]; k--; }
        partners[k] = q;
    });
    int32_t* sp = nullptr;   // the spill run of a voxel with more than kContactInline partners
    float* out = S.cforce + (size_t)v * 3 * kContactInline;
    if (ntot > cap) {
        const int off = atomicAdd(S.spill_used, ntot);
        if (off < 0 || (unsigned)off > (unsigned)(S.spill_cap - ntot)) {
            // the pool's records for this step are used up: the simulation stops with an error
            atomicOr(&c.error, 2);
            S.ccount[v] = 0;
            return;
        }
        sp = S.spill_p + off;
        int k = 0;
        for_each_contact(S, v, parity, [&](int q) { if (k < ntot) sp[k++] = q; });
        for (int i = 1; i < k; i++) {   // insertion sort by partner index (runs are short)
            const int q = sp[i];
            int j = i;
            while (j > 0 && sp[j - 1] > q) { sp[j] = sp[j - 1]; j--; }
            sp[j] = q;
        }
        np = k;
        out = S.spill_f + 3 * (size_t)off;
        S.cspill[v] = off;
    } else if (S.cpart) {   // partner ids, kept where attachment may drop a pair's force
        for (int k = 0; k < np; k++) S.cpart[(size_t)v * kContactInline + k] = partners[k];
    }
    auto partner = [&](int k) { return sp ? sp[k] : partners[k]; };
    for (int k = 0; k < np; k++) {
        const int q = partner(k);
        float f3[3];
        pair_force(S, v < q ? v : q, v < q ? q : v, f3);
        const float sgn = v < q ? 1.0f : -1.0f;   // contactForce(): +force on voxel1, -force on voxel2
        out[3 * k] = sgn * f3[0]; out[3 * k + 1] = sgn * f3[1]; out[3 * k + 2] = sgn * f3[2];
    }
    S.ccount[v] = np;
    if (S.flags & SF_ATTACH) {
        // VX3 attachment candidates (handle_collision_attachment, VX3_VoxelyzeKernel.cu:729-742):
        // touching voxels that both allow attachment, of one sticky material that is not Fixed;
        // the rest of the test and the link creation run in k_attach, in pair order
        const uint32_t fv = S.vfl[v];
        const int mv = __ldg(S.vmat + v);
        const VMat& mm = S.vm[mv];
        if ((fv & VF_ATTACH) && (mm.vx3 & VM_STICKY) && !(mm.vx3 & VM_FIXED)) {
            for (int k = 0; k < np; k++) {
                const int q = partner(k);
                if (q < v || __ldg(S.vmat + q) != mv || !(S.vfl[q] & VF_ATTACH)) continue;
                const int slot = atomicAdd(&c.n_cand, 1);
                if (slot < S.cand_cap) { S.cand[2 * slot] = v; S.cand[2 * slot + 1] = q; }
            }
        }
    }
    if (S.flags & SF_TARGETS) {
        // VX3 target contacts (VX3_VoxelyzeKernel.cu:713-724): each touching pair of a target and
        // a non-target voxel counts once (collisionCount, the formulas' `hit`), and with signals
        // the non-target voxel receives a forced signal in its step
        const bool tv = S.vm[__ldg(S.vmat + v)].vx3 & VM_TARGET;
        int pairs = 0;
        bool hit = false;
        for (int k = 0; k < np; k++) {
            const int q = partner(k);
            const bool tq = S.vm[__ldg(S.vmat + q)].vx3 & VM_TARGET;
            if (tv != tq) { hit = true; if (q > v) pairs++; }
        }
        if (pairs) atomicAdd(&c.hit_count, pairs);
        if (hit && !tv && (S.flags & SF_SIGNALS)) S.vfl[v] |= VF_TGTHIT;
    }
}

// ---------------------------------------------------------------- watch lists
// The reference regenerates its collision list (CVoxelyze::regenerateCollisions,
// Voxelyze3/src/old/Voxelyze.cpp:726-751) when a surface voxel has moved more than half
// the watch distance since the last regeneration (updateCollisions, :671-711): the list
// holds every pair of surface voxels not within 5 links of each other whose centres lie
// within the watch radius, (2 boundingRadius + watchDistance) voxel sizes, and each step
// sums the forces of the pairs on it.  SF_WATCH simulations keep the same lists: per
// surface voxel its partners in increasing order, found through the spatial hash (cells on
// each side enough to cover the radius, those farther than the radius skipped), in one pass
// that runs only in the steps that regenerate.

// Calls fn(q) for every partner q of surface voxel v on its regenerated watch list found in
// the hash cells c0, c0 + cstep, ... of the (2R+1)^3 cells around v (the lanes of a warp
// share a voxel's cells), in no particular order; the exact test is the reference's:
// squared centre distance (double) not above the squared watch radius (float).
template <typename Fn>
__device__ __forceinline__ void for_each_watch_partner(const Sim& S, int v, int parity, int c0, int cstep, Fn fn) {
    const float4 pv = S.cpos[v];
    const float ic = S.inv_cell;
    const int cx = cell_of(pv.x, ic), cy = cell_of(pv.y, ic), cz = cell_of(pv.z, ic);
    const int nv = S.nv;
    const int vx = S.ijk[v], vy = S.ijk[nv + v], vz = S.ijk[2 * nv + v];
    const int* head = S.hash_head + (size_t)parity * S.hash_size;
    const double wr2 = (double)S.watch_r2;
    const float lim = sqrtf(S.watch_r2) * 1.02f + 2.4e-7f * (fabsf(pv.x) + fabsf(pv.y) + fabsf(pv.z)) * 2.0f;
    const int R = S.wcells, side = 2 * R + 1, ncell = side * side * side;
    const double ax = S.px[v], ay = S.py[v], az = S.pz[v];
    // a cell whose box lies farther than lim from v holds no partner: its voxels' float
    // positions have that cell's index, so they lie in the box up to rounding (the box is
    // taken a thousandth of a cell, and a few ulps of the coordinates, larger on each side)
    const float cs = 1.0f / ic, pad = 1e-3f * cs + 4.8e-7f * (fabsf(pv.x) + fabsf(pv.y) + fabsf(pv.z));
    auto gap = [&](int t, float p) { return fmaxf(0.0f, fmaxf(t * cs - pad - p, p - (t + 1) * cs - pad)); };
    for (int cc = c0; cc < ncell; cc += cstep) {
                const int dx = cc % side - R, dy = (cc / side) % side - R, dz = cc / (side * side) - R;
                const int tx = cx + dx, ty = cy + dy, tz = cz + dz;
                const float gx = gap(tx, pv.x), gy = gap(ty, pv.y), gz = gap(tz, pv.z);
                if (gx * gx + gy * gy + gz * gz > lim * lim) continue;
                int q = head[cell_hash(tx, ty, tz, S.hash_size - 1)];
                int guard = 0;
                while (q >= 0 && guard++ < nv) {
                    const int nq = S.hash_next[q];
                    const float4 pq = S.cpos[q];
                    const float fx = pq.x - pv.x, fy = pq.y - pv.y, fz = pq.z - pv.z;
                    if (q != v && cell_of(pq.x, ic) == tx && cell_of(pq.y, ic) == ty && cell_of(pq.z, ic) == tz &&
                        fx * fx + fy * fy + fz * fz <= lim * lim) {
                        const int ox = S.ijk[q] - vx, oy = S.ijk[nv + q] - vy, oz = S.ijk[2 * nv + q] - vz;
                        const int l1 = abs(ox) + abs(oy) + abs(oz);
                        bool near = l1 == 1;   // lattice neighbours are always linked to each other
                        if (!near && l1 <= 5) {
                            const int k = kBallRow[oz + 5][oy + 5] + ox + (5 - abs(oz) - abs(oy));
                            near = (S.reach[(size_t)v * kReachWords + (k >> 5)] >> (k & 31)) & 1u;
                        }
                        if (!near) {
                            const double ex = ax - S.px[q], ey = ay - S.py[q], ez = az - S.pz[q];
                            if (!(ex * ex + ey * ey + ez * ez > wr2)) fn(q);
                        }
                    }
                    q = nq;
                }
    }
}

// The watch-list pass runs over the contact items of the simulations that regenerate this
// step (listed by the previous step's k_sim_end, or every item after the batch changed or
// simulations were restarted), in units of 4 surface voxels, one warp per voxel with its
// lanes splitting the hash cells: a regeneration of one creature spreads over the whole GPU,
// and a step without one costs a launch.
constexpr int kWatchUnit = 4;                 // surface voxels per work unit
constexpr int kWatchUnitsPerItem = 128 / kWatchUnit;   // contact items hold at most 128 surface voxels
template <typename Fn>
__device__ __forceinline__ void for_each_watch_voxel(const Sim* sims, Ctl* ctl, const Item* items, int n_items,
                                                     const int* stale_items, const int* tickets, Fn fn) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int n = min(tickets[7], n_items);
    for (int u = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n * kWatchUnitsPerItem; u += warps) {
        const int it = stale_items[u / kWatchUnitsPerItem];
        if ((unsigned)it >= (unsigned)n_items) continue;
        const Item w = items[it];
        Ctl& c = ctl[w.sim];
        const Sim& S = sims[w.sim];
        if (c.status != 1 || c.diverged || !(S.flags & SF_WATCH) || !c.col_stale) continue;
        const int b = w.begin + (u % kWatchUnitsPerItem) * kWatchUnit, e = min(w.end, b + kWatchUnit);
        for (int i = b; i < e; i++) fn(S, c, i, lane);
    }
}

// One pass: every surface voxel of a regenerating simulation finds its partners (one warp per
// voxel, its lanes splitting the hash cells) into a per-warp buffer, takes a run of the
// simulation's list for them (one atomic on the simulation's count) and writes them in the
// reference's increasing partner order (each lane ranks up to four entries against the
// buffer: partners are distinct, so the ranks are a permutation); it records its position
// as the regeneration's (lastColWatchPosition).  More partners than the buffer or the list
// holds leave the simulation on the per-step hash search until the next regeneration.
constexpr int kWatchBuf = 128;   // partners one surface voxel may have in a list
__global__ void __launch_bounds__(256) k_watch_build(const Sim* __restrict__ sims, Ctl* ctl, const Item* __restrict__ items,
                                                     int n_items, const int* __restrict__ stale_items, const int* tickets) {
    __shared__ int s_found[8];
    __shared__ int s_buf[8][kWatchBuf];
    const int wid = threadIdx.x >> 5;
    for_each_watch_voxel(sims, ctl, items, n_items, stale_items, tickets, [&](const Sim& S, Ctl& c, int i, int lane) {
        const int v = S.surf[i];
        if (lane == 0) {
            S.watch[v] = make_float4(d2f(S.px[v]), d2f(S.py[v]), d2f(S.pz[v]), 0.0f);
            s_found[wid] = 0;
        }
        __syncwarp();
        for_each_watch_partner(S, v, c.hash_parity, lane, 32, [&](int q) {
            const int k = atomicAdd(&s_found[wid], 1);
            if (k < kWatchBuf) s_buf[wid][k] = q;
        });
        __syncwarp();
        const int k = s_found[wid];
        int base = 0;
        if (lane == 0) {
            base = k <= kWatchBuf ? atomicAdd(&c.watch_used, k) : -1;
            if (base < 0 || base > S.wcap - k) { c.watch_ok = 0; base = -1; }
            S.woff[2 * i] = base < 0 ? 0 : base;
            S.woff[2 * i + 1] = base < 0 ? 0 : k;
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= 0 && k > 0) {
            int e[4], r[4];
#pragma unroll
            for (int t = 0; t < 4; t++) { e[t] = lane + 32 * t < k ? s_buf[wid][lane + 32 * t] : 0; r[t] = 0; }
            for (int j = 0; j < k; j++) {
                const int x = s_buf[wid][j];
#pragma unroll
                for (int t = 0; t < 4; t++) r[t] += x < e[t] ? 1 : 0;
            }
#pragma unroll
            for (int t = 0; t < 4; t++)
                if (lane + 32 * t < k) S.wlist[base + r[t]] = e[t];
        }
        __syncwarp();
    });
}

// The contact pass of surface voxel v (surface index si) from its watch list: the list is in
// increasing partner order, so the overlapping pairs (float envelope test, then the exact
// test) are the reference's colWatch terms in order; their forces go straight to the voxel's
// slots, and a voxel with more than its slots walks the list again into a spill run.
__device__ void voxel_contacts_watch(const Sim& S, int v, int si, Ctl& c) {
    const int cap = min(max(S.contact_inline, 1), kContactInline);
    float* out = S.cforce + (size_t)v * 3 * kContactInline;
    const float4 pv = S.cpos[v];
    int b = S.woff[2 * si], e = b + S.woff[2 * si + 1];
    if (b < 0 || e > S.wcap || b > e) {   // never: a run outside the lists is read as empty
        atomicOr(&c.error, 4);
        b = e = 0;
    }
    const bool targets = S.flags & SF_TARGETS;
    const bool tv = targets && (S.vm[__ldg(S.vmat + v)].vx3 & VM_TARGET);
    int n = 0, pairs = 0;
    bool hit = false;
    for (int k = b; k < e; k++) {
        const int q = S.wlist[k];
        if ((unsigned)q >= (unsigned)S.nv) { atomicOr(&c.error, 4); continue; }   // never: not a voxel
        if (!maybe_touching(pv, S.cpos[q], S.env_radius)) continue;
        float f3[3];
        if (!pair_force(S, v < q ? v : q, v < q ? q : v, f3)) continue;
        if (n < cap) {
            const float sgn = v < q ? 1.0f : -1.0f;   // contactForce(): +force on voxel1, -force on voxel2
            out[3 * n] = sgn * f3[0]; out[3 * n + 1] = sgn * f3[1]; out[3 * n + 2] = sgn * f3[2];
        }
        n++;
        if (targets && (bool)(S.vm[__ldg(S.vmat + q)].vx3 & VM_TARGET) != tv) { hit = true; if (q > v) pairs++; }
    }
    if (n > cap) {
        const int off = atomicAdd(S.spill_used, n);
        if (off < 0 || (unsigned)off > (unsigned)(S.spill_cap - n)) {
            atomicOr(&c.error, 2);   // the pool's records for this step are used up
            S.ccount[v] = 0;
            return;
        }
        int j = 0;
        for (int k = b; k < e && j < n; k++) {
            const int q = S.wlist[k];
            if ((unsigned)q >= (unsigned)S.nv) continue;
            if (!maybe_touching(pv, S.cpos[q], S.env_radius)) continue;
            float f3[3];
            if (!pair_force(S, v < q ? v : q, v < q ? q : v, f3)) continue;
            const float sgn = v < q ? 1.0f : -1.0f;
            S.spill_p[off + j] = q;
            float* o = S.spill_f + 3 * (size_t)(off + j);
            o[0] = sgn * f3[0]; o[1] = sgn * f3[1]; o[2] = sgn * f3[2];
            j++;
        }
        S.cspill[v] = off;
    }
    S.ccount[v] = n;
    if (targets) {   // VX3 target contacts, as in voxel_contacts
        if (pairs) atomicAdd(&c.hit_count, pairs);
        if (hit && !tv && (S.flags & SF_SIGNALS)) S.vfl[v] |= VF_TGTHIT;
    }
}

__global__ void __launch_bounds__(128) k_contacts(const Sim* __restrict__ sims, Ctl* ctl, const Item* __restrict__ items, int n_items, int* tickets) {
    __shared__ int s_item;
    for (;;) {
        const int it = claim(&tickets[1], &s_item);
        if (it >= n_items) break;
        const Item w = items[it];
        Ctl& c = ctl[w.sim];
        if (c.status != 1 || c.diverged) continue;
        const Sim& S = sims[w.sim];
        const int parity = c.hash_parity;
        // clear the other table for the insertions made by this step's voxel update
        int* other = S.hash_head + (size_t)(parity ^ 1) * S.hash_size;
        const int per = (S.hash_size + S.nsurf - 1) / (S.nsurf > 0 ? S.nsurf : 1);
        const int cb = w.begin * per, ce = min(S.hash_size, (w.end == S.nsurf) ? S.hash_size : w.end * per);
        for (int h = cb + threadIdx.x; h < ce; h += blockDim.x) other[h] = -1;
        if ((S.flags & SF_WATCH) && c.watch_ok) {
            for (int i = w.begin + threadIdx.x; i < w.end; i += blockDim.x) voxel_contacts_watch(S, S.surf[i], i, c);
        } else {
            for (int i = w.begin + threadIdx.x; i < w.end; i += blockDim.x) voxel_contacts(S, S.surf[i], parity, c);
        }
    }
}


// CVX_Voxel::timeStep with force(), moment() and floorForce()
// (Voxelyze3/src/old/VX_Voxel.cpp:163-297), then the Poisson strain the next
// step's links will read (CVX_Voxel::strain(true), :299-333) and the next
// step's actuation temperature (VX3_VoxelyzeKernel.cu:625-650).
// Per-step values shared by every voxel of a simulation.
struct StepTimes {
    double t_now;      // currentTime during this step
    double t_next;     // after it
    double t_cycles;   // t_next / TempPeriod
    double angle;      // recentAngle (force-field variable)
    double closeness;  // targetCloseness, numClosePairs and collisionCount (force-field variables)
    int close_pairs, hits;
};

// ---------------------------------------------------------------- VX3 signals
// VX3_Voxel::receiveSignal (VX3/VX3_Voxel.cu:301-322): a signal arriving at `active`
// is taken unless the voxel is refractory (a forced one always is); the voxel shows
// it as its local signal and will relay value*signalValueDecay at that time.
__device__ __forceinline__ void sig_receive(const Sim& S, int v, const VMat& m, double value, double active, bool force) {
    double* G = S.sig;
    const size_t nv = S.nv;
    if (!force && G[SG_INACTIVE * nv + v] > active) return;
    if (value < 0.1) return;
    G[SG_INACTIVE * nv + v] = active + m.sigInactive;
    G[SG_LOCAL * nv + v] = value;
    double relay = value * m.sigDecay;
    if (relay < 0.1) relay = 0;
    G[SG_VALUE * nv + v] = relay;
    G[SG_ACTIVE * nv + v] = active;
}

// A voxel's own signal work at the end of its time step (VX3_Voxel.cu:271-276):
// propagateSignal (:323-347) relays a due signal (recorded in SG_OUT / SG_OUT_T for
// the neighbours, which take it in k_signals), then packMaker (:291-299) and
// localSignalDecay (:279-289).  The reference writes into the neighbours from this
// thread while they run their own step, so its outcome depends on thread timing;
// here every voxel first finishes its own work and the neighbours then take the
// relayed signals in direction order, which is deterministic.
__device__ __forceinline__ void sig_own_step(const Sim& S, int v, const VMat& m, double t) {
    double* G = S.sig;
    const size_t nv = S.nv;
    double out = 0, out_t = 0;
    if (!(G[SG_ACTIVE * nv + v] > t) && !(G[SG_VALUE * nv + v] < 0.1)) {
        out = G[SG_VALUE * nv + v];
        out_t = t + m.sigDelay;
        G[SG_VALUE * nv + v] = 0;
        G[SG_ACTIVE * nv + v] = 0;
        G[SG_INACTIVE * nv + v] = t + 2 * m.sigDelay + m.sigInactive;
    }
    G[SG_OUT * nv + v] = out;
    G[SG_OUT_T * nv + v] = out_t;
    if ((m.vx3 & VM_PACEMAKER) && !(G[SG_PULSE * nv + v] > t)) {
        sig_receive(S, v, m, 100, t, true);
        G[SG_PULSE * nv + v] = t + m.pmPeriod;
    }
    if (!(G[SG_LOCAL_DT * nv + v] > t)) {
        if (G[SG_LOCAL * nv + v] < 0.1) {
            G[SG_LOCAL * nv + v] = 0;
        } else {
            G[SG_LOCAL * nv + v] = G[SG_LOCAL * nv + v] * 0.9;
            G[SG_LOCAL_DT * nv + v] = t + 0.01;
        }
    }
}

// Voxels of Fixed materials and removed voxels do not move (gpu_update_voxels,
// VX3_VoxelyzeKernel.cu:582-588), keep their temperature (gpu_update_temperature
// skips them) and run no signal step of their own; they count in the centre of
// mass, and a fixed voxel stays in the contact search (a removed one leaves it).
__device__ void frozen_voxel(const Sim& S, int v, uint32_t fl, const VMat& m, const StepTimes& st, int flags, double* com4,
                             int* hash_next_table) {
    if (flags & SF_SIGNALS) {
        if ((fl & VF_TGTHIT) && !(fl & VF_REMOVED)) sig_receive(S, v, m, 100, st.t_now, true);
        S.sig[SG_OUT * (size_t)S.nv + v] = 0;
    }
    if (fl & VF_TGTHIT) S.vfl[v] = fl & ~VF_TGTHIT;
    const d3 pos = D3(S.px[v], S.py[v], S.pz[v]);
    if (com4 && (fl & VF_MEASURED)) {
        const double w = m.mass;
        com4[0] += pos.x * w; com4[1] += pos.y * w; com4[2] += pos.z * w; com4[3] += w;
    }
    if ((flags & SF_COLLIDE) && !(fl & (VF_INTERIOR | VF_REMOVED))) hash_insert(S, v, pos, S.temp[v], hash_next_table);
}

__device__ __forceinline__ void voxel_update(const Sim& S, int v, float dt, const StepTimes& st, int flags, double* com4, int* hash_next_table,
                                             int* watch_moved = nullptr) {
    const double t_cycles = st.t_cycles;
    const int nv = S.nv;
    const VMat& m = S.vm[__ldg(S.vmat + v)];
    uint32_t fl = S.vfl[v];
    if ((flags & (SF_REMOVE | SF_FIXEDMAT)) && ((fl & VF_REMOVED) || (m.vx3 & VM_FIXED))) {
        frozen_voxel(S, v, fl, m, st, flags, com4, hash_next_table);
        return;
    }
    // VX3: a contact with a target voxel this step hands a forced signal to a non-target
    // voxel (handle_collision_attachment, VX3_VoxelyzeKernel.cu:709-724), before the cilia
    // forces and the voxel's own step
    if ((flags & SF_SIGNALS) && (fl & VF_TGTHIT)) sig_receive(S, v, m, 100, st.t_now, true);
    fl &= ~VF_TGTHIT;
    const Ext* e = (fl & VF_EXT) ? &S.ext[__ldg(S.vext + v)] : nullptr;
    d3 pos = D3(S.px[v], S.py[v], S.pz[v]);
    d3 lm = D3(S.mx[v], S.my[v], S.mz[v]);
    q4 q = Q4(S.qw[v], S.qx[v], S.qy[v], S.qz[v]);
    d3 am = D3(S.ax[v], S.ay[v], S.az[v]);
    const float temp = S.temp[v];
    bool fixed_all = false;
    if (e && (e->dof & 0x3F) == 0x3F) {
        fixed_all = true;
        pos = D3(S.ijk[v] * m.nom + e->tr[0], S.ijk[nv + v] * m.nom + e->tr[1], S.ijk[2 * nv + v] * m.nom + e->tr[2]);
        q = Q4(e->rq[0], e->rq[1], e->rq[2], e->rq[3]);
        lm = am = D3(0, 0, 0);
    } else {
        // force()
        // the sum starts at +0, so its first term (direction 0) adds exactly as plus_zero
        const double* sf = S.sf;
        d3 F = (fl & 1u) ? D3(fp64i::plus_zero(sf[v]), fp64i::plus_zero(sf[nv + v]), fp64i::plus_zero(sf[2 * nv + v])) : D3(0, 0, 0);
#pragma unroll
        for (int d = 1; d < 6; d++)
            if (fl & (1u << d)) F = D3(F.x + sf[(d * 3) * nv + v], F.y + sf[(d * 3 + 1) * nv + v], F.z + sf[(d * 3 + 2) * nv + v]);
        F = qrot(q, F);
        if (e) { F.x += e->f[0]; F.y += e->f[1]; F.z += e->f[2]; }
        const double vx = m.massInvD * lm.x, vy = m.massInvD * lm.y, vz = m.massInvD * lm.z;
        F = D3(F.x - m.gDampTD * vx, F.y - m.gDampTD * vy, F.z - m.gDampTD * vz);
        F.z += m.gravForceD;
        if (flags & SF_COLLIDE) {
            const int nc = S.ccount[v];
            const float* cf = nc <= S.contact_inline ? S.cforce + (size_t)v * 3 * kContactInline : S.spill_f + 3 * (size_t)S.cspill[v];
            for (int k = 0; k < nc; k++) { F.x -= cf[3 * k]; F.y -= cf[3 * k + 1]; F.z -= cf[3 * k + 2]; }
        }
        // VX3 cilia (gpu_update_cilia_force, VX3_VoxelyzeKernel.cu:846-859; VX3_Voxel::force,
        // VX3_Voxel.cu:376): surface voxels of a cilia material, once it is switched on, are
        // pushed along baseCiliaForce + localSignal * shiftCiliaForce rotated into the world
        // frame (without signals the shift term is zero)
        if ((flags & SF_CILIA) && !(fl & VF_INTERIOR) && m.cilia != 0 && !fp64i::gt(m.ciliaOn, st.t_now)) {
            d3 base = D3(S.cilia[v], S.cilia[nv + v], S.cilia[2 * nv + v]);
            if (S.shift_cilia) {
                const double ls = S.sig[SG_LOCAL * (size_t)nv + v];
                base = D3(base.x + ls * S.shift_cilia[v], base.y + ls * S.shift_cilia[nv + v], base.z + ls * S.shift_cilia[2 * nv + v]);
            }
            const d3 cf = qrot(q, base);
            F = D3(F.x + cf.x * m.cilia, F.y + cf.y * m.cilia, F.z + cf.z * m.cilia);
        }
        // VX3 force field (VX3_Voxel::timeStep, VX3_Voxel.cu:178-184): formulas of the voxel's
        // position and the simulation's time, recent angle and voxel count
        if (flags & SF_FFIELD) {
            MathVars mv;
            mv.x = pos.x; mv.y = pos.y; mv.z = pos.z; mv.hit = st.hits; mv.t = st.t_now; mv.angle = st.angle;
            mv.closeness = st.closeness; mv.num_close_pairs = st.close_pairs; mv.num_voxel = nv;
            F.x += mathtree_eval(S.ffield[0], mv);
            F.y += mathtree_eval(S.ffield[1], mv);
            F.z += mathtree_eval(S.ffield[2], mv);
        }
        // floorForce()
        const d3 F0 = F;
        const bool floor = flags & SF_FLOOR;
        // CVX_Voxel::floorPenetration; pos is unchanged until the translation below, so the
        // reference's second evaluation (VX_Voxel.cpp:188) yields this same value
        const float pen = floor ? d2f(half(base_size_avg(m, temp)) - m.halfNom - pos.z) : -1.0f;
        if (floor) {
            fl = (pen >= 0) ? (fl | VF_FLOORC) : (fl & ~VF_FLOORC);
            if (pen >= 0) {
                const float normal = m.penStiff * pen;
                F.z += f2d(normal) - m.cDampTD * vz;
                if (fl & VF_STATIC) {
                    const float surf = d2f(F.x * F.x + F.y * F.y);
                    const float fr = (m.mus * normal) * (m.mus * normal);
                    if (surf > fr) fl &= ~VF_STATIC;
                } else {
                    const double hl = sqrt(fp64i::plus_zero(vx * vx + vy * vy));   // + 0.0 * 0.0
                    double nx = vx, ny = vy, nz = 0.0;
                    if (fp64i::gt0(hl)) { const double inv = 1.0 / hl; nx = inv * vx; ny = inv * vy; nz = inv * 0.0; }
                    const double k = f2d(m.muk * normal);
                    F = D3(F.x - k * nx, F.y - k * ny, F.z - k * nz);
                }
            } else {
                fl &= ~VF_STATIC;
            }
        }
        const d3 fric = D3(F.x - F0.x, F.y - F0.y, F.z - F0.z);
        const double dtd = f2d(dt);
        lm = D3(lm.x + dtd * F.x, lm.y + dtd * F.y, lm.z + dtd * F.z);
        const double sdt = f2d(dt * m.massInv);
        d3 tr = D3(sdt * lm.x, sdt * lm.y, sdt * lm.z);
        if (floor && pen >= 0) {
            const double work = fric.x * tr.x + fric.y * tr.y;
            const double hKe = m.halfMassInv * (lm.x * lm.x + lm.y * lm.y);
            if (fp64i::le(hKe + work, 0.0)) fl |= VF_STATIC;
            if (fl & VF_STATIC) { lm.x = lm.y = 0; tr.x = tr.y = 0; }
        } else {
            fl &= ~VF_STATIC;
        }
        pos = D3(pos.x + tr.x, pos.y + tr.y, pos.z + tr.z);
        // moment()
        const double* sm = S.sm;
        d3 M = (fl & 1u) ? D3(fp64i::plus_zero(sm[v]), fp64i::plus_zero(sm[nv + v]), fp64i::plus_zero(sm[2 * nv + v])) : D3(0, 0, 0);
#pragma unroll
        for (int d = 1; d < 6; d++)
            if (fl & (1u << d)) M = D3(M.x + sm[(d * 3) * nv + v], M.y + sm[(d * 3 + 1) * nv + v], M.z + sm[(d * 3 + 2) * nv + v]);
        M = qrot(q, M);
        if (e) { M.x += e->m[0]; M.y += e->m[1]; M.z += e->m[2]; }
        const double wx = m.IinvD * am.x, wy = m.IinvD * am.y, wz = m.IinvD * am.z;
        M = D3(M.x - m.gDampRD * wx, M.y - m.gDampRD * wy, M.z - m.gDampRD * wz);
        am = D3(am.x + dtd * M.x, am.y + dtd * M.y, am.z + dtd * M.z);
        const double sI = f2d(dt * m.Iinv);
        bool wrot = false;
        q = qmul(q_from_rotvec(D3(sI * am.x, sI * am.y, sI * am.z), &wrot), q);
        fl = wrot ? (fl | VF_WROT) : (fl & ~VF_WROT);
        if (e) {
            const int d = e->dof;
            if (d & 1) { pos.x = S.ijk[v] * m.nom + e->tr[0]; lm.x = 0; }
            if (d & 2) { pos.y = S.ijk[nv + v] * m.nom + e->tr[1]; lm.y = 0; }
            if (d & 4) { pos.z = S.ijk[2 * nv + v] * m.nom + e->tr[2]; lm.z = 0; }
            if (d & 0x38) {
                if ((d & 0x38) == 0x38) {
                    q = Q4(e->rq[0], e->rq[1], e->rq[2], e->rq[3]);
                    am = D3(0, 0, 0);
                } else {
                    d3 rv = q_to_rotvec(q);
                    if (d & 8) { rv.x = 0; am.x = 0; }
                    if (d & 16) { rv.y = 0; am.y = 0; }
                    if (d & 32) { rv.z = 0; am.z = 0; }
                    q = q_from_rotvec(rv);
                }
            }
        }
    }
    S.px[v] = pos.x; S.py[v] = pos.y; S.pz[v] = pos.z;
    S.mx[v] = lm.x; S.my[v] = lm.y; S.mz[v] = lm.z;
    S.qw[v] = q.w; S.qx[v] = q.x; S.qy[v] = q.y; S.qz[v] = q.z;
    S.ax[v] = am.x; S.ay[v] = am.y; S.az[v] = am.z;
    if (flags & SF_ATTACH) {
        // enableAttach (gpu_update_voxels, VX3_VoxelyzeKernel.cu:608-620): every given attach
        // condition is positive at the voxel's new position
        MathVars mv;
        mv.x = pos.x; mv.y = pos.y; mv.z = pos.z; mv.hit = st.hits; mv.t = st.t_now; mv.angle = st.angle;
        mv.closeness = st.closeness; mv.num_close_pairs = st.close_pairs; mv.num_voxel = nv;
        bool ok = true;
        for (int k = 0; k < 5 && ok; k++)
            if ((S.attach_mask >> k) & 1) ok = mathtree_eval(S.attach_cond[k], mv) > 0;
        fl = ok ? (fl | VF_ATTACH) : (fl & ~VF_ATTACH);
    }
    S.vfl[v] = fl;
    if (com4 && (fl & VF_MEASURED)) {
        const double w = m.mass;
        com4[0] += pos.x * w; com4[1] += pos.y * w; com4[2] += pos.z * w; com4[3] += w;
    }
    // CVX_Voxel::strain(true) for the next step (fully fixed voxels keep their cached value)
    if (!fixed_all && m.nu != 0.0f) {
        float s[3] = {0, 0, 0};
        int nb[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < 6; d++)
            if (fl & (1u << d)) { s[d >> 1] += S.ss[d * nv + v]; nb[d >> 1]++; }
        bool ten[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            if (nb[i] == 2) s[i] *= 0.5f;
            ten[i] = (nb[i] == 2) || (e && nb[i] == 1 && ((e->dof & (1 << i)) || e->f[i] != 0));
        }
        if (!(ten[0] && ten[1] && ten[2])) {
            float add = 0;
            for (int i = 0; i < 3; i++) if (ten[i]) add += s[i];
            const float value = poisson_power(m, 1.0f + add) - 1.0f;
            for (int i = 0; i < 3; i++) if (!ten[i]) s[i] = value;
        }
        S.ps[v] = s[0]; S.ps[nv + v] = s[1]; S.ps[2 * nv + v] = s[2];
    }
    // VX3 signals: the voxel's own signal work at the end of its step (a voxel fixed in all
    // degrees of freedom returns from VX3_Voxel::timeStep before it, VX3_Voxel.cu:166-173)
    if (flags & SF_SIGNALS) {
        if (!fixed_all) sig_own_step(S, v, m, st.t_now);
        else S.sig[SG_OUT * (size_t)nv + v] = 0;
    }
    // actuation temperature for the next step
    float temp_next = temp;
    // (VX3: no update before the material's TurnOnThermalExpansionAfterThisManySeconds)
    if ((flags & SF_VARY) && !fp64i::gt(m.thermalOn, st.t_next)) {
        const float two_pi = 2 * 3.1415926f;
        double T = S.temp_amp * sin((double)two_pi * (t_cycles + __ldg(S.phase + v)));
        if (!(flags & SF_EXPAND) && fp64i::gt0(T)) T = 0;
        temp_next = d2f(T);
        S.temp[v] = temp_next;
    }
    // insert into the table the next step's contact pass reads
    if ((flags & SF_COLLIDE) && !(fl & VF_INTERIOR)) hash_insert(S, v, pos, temp_next, hash_next_table);
    // watch lists: a surface voxel further than the re-check distance from where the last
    // regeneration saw it makes the next step regenerate (CVoxelyze::updateCollisions,
    // Voxelyze.cpp:689-697: (pos - lastColWatchPosition).Length2() > recalcDist*recalcDist)
    if (watch_moved && !(fl & VF_INTERIOR)) {
        const float4 wp = S.watch[v];
        const double dx = pos.x - (double)wp.x, dy = pos.y - (double)wp.y, dz = pos.z - (double)wp.z;
        if (dx * dx + dy * dy + dz * dz > (double)S.recalc2) *watch_moved = 1;
    }
}

__device__ __forceinline__ double block_sum(double x, double* red) {
    // fixed-order reduction (deterministic): a shuffle tree inside each warp, then the warps'
    // sums folded in warp order by the first warp (blockDim.x a multiple of 32, at most 1024)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) x = x + __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[wid] = x;
    __syncthreads();
    if (wid == 0) {
        double y = lane < nw ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) y = y + __shfl_down_sync(0xffffffffu, y, o);
        if (lane == 0) red[32] = y;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

// VX3 secondary experiment (VX3_VoxelyzeKernel.cu:336-349, 365-397), after the CoM
// sample: every material whose RemoveFromSimulationAfterThisManySeconds has passed
// loses its voxels (frozen, unlinked from their neighbours, off the surface), and once
// ReinitializeInitialPositionAfterThisManySeconds has passed the initial centre of
// mass becomes the last sampled one and the initial positions the current ones.  One
// thread; each of these happens once per run.
__device__ __noinline__ void secondary_experiment(const Sim& S, Ctl& c, double t_now) {
    const int nv = S.nv;
    for (int i = 0; i < S.n_mats && i < 32; i++) {
        const VMat& m = S.vm[i];
        if ((c.removed_mats >> i) & 1) continue;
        if (!(m.removeAfter > 0 && m.removeAfter < t_now)) continue;
        for (int v = 0; v < nv; v++) {
            if (S.vmat[v] != i) continue;
            const uint32_t f = S.vfl[v];
            if (f & VF_REMOVED) continue;
            for (int d = 0; d < 6; d++) {
                if (!(f & (1u << d))) continue;
                const int l = S.vlink[6 * v + d];
                S.lfl[l] |= LF_GONE | LF_REMOVED;
                const int u = S.lneg[l] == v ? S.lpos[l] : S.lneg[l];
                S.vfl[u] &= ~((1u << (d ^ 1)) | VF_INTERIOR);   // the neighbour holds the link in the opposite direction
            }
            S.vfl[v] = (f & ~(VF_LINKS | VF_INTERIOR)) | VF_REMOVED;
        }
        c.removed_mats |= 1 << i;
    }
    if (!c.reinit_done && S.reinit_after < t_now) {
        c.reinit_done = 1;
        for (int k = 0; k < 3; k++) c.init_com[k] = c.com[k];
        for (int v = 0; v < nv; v++) {
            S.init_pos[v] = S.px[v]; S.init_pos[nv + v] = S.py[v]; S.init_pos[2 * (size_t)nv + v] = S.pz[v];
        }
    }
}

// Per-simulation bookkeeping after its last voxel item of the step (one thread):
// status on divergence/error, time and step count, cycle CoM sampling and the
// recent-angle measure (VX3_VoxelyzeKernel.cu:314-334, 352), stop condition.
// Kept out of line so the voxel loop does not carry its registers and stack.
__device__ __noinline__ void sim_control(const Sim& S, Ctl& c, bool div, double t_next, int64_t stepno, bool com_step, int flags,
                                         int nv, const double* s4) {
    if (div) { c.status = 3; return; }
    if (c.error) { c.status = 4; return; }
    const double t_now = c.t;
    if (flags & SF_SIGNALS) c.sig_pending = 1;   // k_signals completes this step's signals
    c.t = t_next;
    c.steps = stepno;
    if (flags & SF_VARY) c.t_cycles = (c.t + c.dt) / S.temp_period;   // the next step's actuation phase
    if (flags & SF_COLLIDE) c.hash_parity ^= 1;
    if (flags & SF_WATCH) {
        c.col_stale = c.col_moved;
        c.col_moved = 0;
        if (c.col_stale) { c.watch_used = 0; c.watch_ok = 1; c.watch_regens += 1; }   // the next step regenerates
    }
    if (com_step) {
        c.angle_samples++;
        for (int j = 0; j < 3; j++) { c.com_hist[0][j] = c.com_hist[1][j]; c.com_hist[1][j] = c.com[j]; }
        if (s4[3] == 0) { c.com[0] = c.com[1] = c.com[2] = 0; }
        else for (int j = 0; j < 3; j++) c.com[j] = s4[j] / s4[3];
        const double* A = c.com_hist[0];
        const double* B = c.com_hist[1];
        const double* C = c.com;
        const bool eqBC = B[0] == C[0] && B[1] == C[1] && B[2] == C[2];
        const bool eqAB = A[0] == B[0] && A[1] == B[1] && A[2] == B[2];
        if (eqBC || eqAB || c.angle_samples < 3) c.recent_angle = 0;
        else {
            const double bax = B[0] - A[0], bay = B[1] - A[1], baz = B[2] - A[2];
            const double cbx = C[0] - B[0], cby = C[1] - B[1], cbz = C[2] - B[2];
            c.recent_angle = acos((bax * cbx + bay * cby + baz * cbz) /
                                  (sqrt(bax * bax + bay * bay + baz * baz) * sqrt(cbx * cbx + cby * cby + cbz * cbz)));
        }
        // VX3 computeTargetCloseness (VX3_VoxelyzeKernel.cu:545-563): over the target voxels in
        // index order, pairs closer than MaxDistInVoxelLengthsToCountAsPair voxel sizes and the
        // sum of inverse distances
        if ((flags & SF_TARGETS) && S.close_r != 0) {
            double ret = 0;
            int pairs = 0;
            for (int i = 0; i < S.n_targets; i++) {
                const int a = S.targets[i];
                for (int j = i + 1; j < S.n_targets; j++) {
                    const int b = S.targets[j];
                    const double dx = S.px[b] - S.px[a], dy = S.py[b] - S.py[a], dz = S.pz[b] - S.pz[a];
                    const double dist = sqrt(dx * dx + dy * dy + dz * dz);
                    if (dist < S.close_r) pairs++;
                    ret += 1 / dist;
                }
            }
            c.closeness = ret;
            c.num_close_pairs = pairs;
        }
    }
    if (flags & SF_REMOVE) secondary_experiment(S, c, t_now);
    bool stop = c.target > 0 && stepno >= c.target;
    if (c.stop.n > 0 && !c.no_stop) {
        MathVars mv;
        mv.x = c.com[0]; mv.y = c.com[1]; mv.z = c.com[2]; mv.hit = c.hit_count; mv.t = c.t; mv.angle = c.recent_angle;
        mv.closeness = c.closeness; mv.num_close_pairs = c.num_close_pairs; mv.num_voxel = nv;
        if (mathtree_eval(c.stop, mv) > 0) stop = true;
    }
    if (stop) c.status = 2;
}

__global__ void __launch_bounds__(GVX_STEP_BLOCK, GVX_VOXELS_MIN_BLOCKS) k_voxels(const Sim* __restrict__ sims, Ctl* ctl, const int2* __restrict__ perm,
                                                                       const int* __restrict__ total, int cap, int n_slots, int* tickets,
                                                                       int claim) {
    // the voxels of the running simulations, grouped by key like the links (k_bin_*); warps
    // take chunks of `claim` voxels (a multiple of 32), so no warp waits at a block barrier
    // for a costlier one
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        tickets[0] = 0;
        tickets[6] = tickets[5];   // the last k_links launch's mode changes, for the next one
        tickets[5] = 0;
        tickets[7] = 0;            // this step's watch-list passes are done: k_sim_end lists the next
    }
    const int n = min(*total, cap);
    const int lane = threadIdx.x & 31;
    for (;;) {
        int chunk = 0;
        if (lane == 0) chunk = atomicAdd(&tickets[2], 1);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        const int k0 = chunk * claim;
        if (k0 >= n) break;
        const int k1 = min(n, k0 + claim);
        for (int k = k0 + lane; k < k1; k += 32) {
            const int2 e = __ldg(perm + k);
            if ((unsigned)e.x >= (unsigned)n_slots) continue;   // never: the grouping lists running slots
            const Ctl& c = ctl[e.x];
            const float dt = c.dt;
            if (c.status == 1 && !c.diverged && dt != 0.0f && (unsigned)e.y < (unsigned)sims[e.x].nv) {
                const Sim& S = sims[e.x];
                StepTimes st;
                st.t_now = c.t; st.t_next = c.t + dt; st.t_cycles = c.t_cycles; st.angle = c.recent_angle;
                st.closeness = c.closeness; st.close_pairs = c.num_close_pairs; st.hits = c.hit_count;
                int* hnext = (S.flags & SF_COLLIDE) ? S.hash_head + (size_t)(c.hash_parity ^ 1) * S.hash_size : nullptr;
                voxel_update(S, e.y, dt, st, S.flags, nullptr, hnext, (S.flags & SF_WATCH) ? &ctl[e.x].col_moved : nullptr);
            }
        }
    }
}

// The end of a step for each simulation of the batch, one block each: on cycle steps the
// centre of mass of the measured voxels (the fixed-order sum of k_com), then sim_control.
__global__ void __launch_bounds__(256) k_sim_end(const Sim* __restrict__ sims, Ctl* ctl, const int* __restrict__ slots, int n, int* tickets,
                                                 int* stale_items) {
    __shared__ double red[256];
    __shared__ int s_base;
    if ((int)blockIdx.x >= n) return;
    const int sim = slots[blockIdx.x];
    Ctl& c = ctl[sim];
    if (c.status != 1) return;
    const Sim& S = sims[sim];
    const bool div = c.diverged;
    const double t_next = c.t + c.dt;
    const int64_t stepno = c.steps + 1;
    const bool com_step = c.cycle_step > 0 && (stepno % c.cycle_step) == 0;
    double s4[4] = {0, 0, 0, 0};
    if (com_step && !div) {
        double a[4] = {0, 0, 0, 0};
        for (int v = threadIdx.x; v < S.nv; v += blockDim.x) {
            if (!(S.vfl[v] & VF_MEASURED)) continue;
            const double w = S.vm[S.vmat[v]].mass;
            a[0] += S.px[v] * w; a[1] += S.py[v] * w; a[2] += S.pz[v] * w; a[3] += w;
        }
        for (int k = 0; k < 4; k++) s4[k] = block_sum(a[k], red);
    }
    if (threadIdx.x == 0) {
        sim_control(S, c, div, t_next, stepno, com_step, S.flags, S.nv, s4);
        // the next step's watch-list passes go over the items of the simulations that regenerate
        s_base = (c.status == 1 && (S.flags & SF_WATCH) && c.col_stale && c.c_item_count > 0) ? atomicAdd(&tickets[7], c.c_item_count) : -1;
    }
    __syncthreads();
    if (s_base >= 0)
        for (int k = threadIdx.x; k < c.c_item_count; k += blockDim.x) stale_items[s_base + k] = c.c_item_begin + k;
}

// VX3 attachment (handle_collision_attachment, VX3_VoxelyzeKernel.cu:729-827) for one
// simulation, after its contact pass and before its voxel update: the candidate pairs
// (touching voxels of one sticky material that both allow attachment) in increasing
// pair order; a pair not within 5 links of each other gets a new link along the axis
// on which the other voxel lies in the first voxel's frame, if both voxels have that
// link slot free.  The reference creates links from many threads at once with no
// synchronisation; here one thread creates them in pair order, which is deterministic.
// The new link starts from the reset state (VX3_Link::reset, VX3_Link.cu:58-70), acts
// at 1% for SafetyGuard updates, and the pair's contact forces of this step are dropped.
__device__ bool linked_within(const Sim& S, int from, int target, int depth) {
    // VX3's is_neighbor (VX3_VoxelyzeKernel.cu:651-680): a path of at most `depth` links that
    // never steps straight back over the link it arrived by (depth-first, explicit stack)
    constexpr int kStack = 1 + 5 * 5;
    int sv[kStack], sl[kStack], sd[kStack];
    int sp = 0;
    sv[0] = from; sl[0] = -1; sd[0] = 0;
    sp = 1;
    while (sp > 0) {
        --sp;
        const int v = sv[sp], in = sl[sp], dd = sd[sp];
        if (v == target) return true;
        if (dd >= depth) continue;
        const uint32_t f = S.vfl[v];
        for (int d = 5; d >= 0; d--) {
            if (!((f >> d) & 1)) continue;
            const int l = S.vlink[6 * v + d];
            if (l == in || sp >= kStack) continue;
            sv[sp] = S.lneg[l] == v ? S.lpos[l] : S.lneg[l];
            sl[sp] = l;
            sd[sp] = dd + 1;
            sp++;
        }
    }
    return false;
}

// Drops voxel v's contact force from partner q for this step (a zero force adds nothing).
__device__ void drop_pair_contact(const Sim& S, int v, int q) {
    const int n = S.ccount[v];
    const bool spilled = n > S.contact_inline;
    const int32_t* part = spilled ? S.spill_p + S.cspill[v] : S.cpart + (size_t)v * kContactInline;
    float* f = spilled ? S.spill_f + 3 * (size_t)S.cspill[v] : S.cforce + (size_t)v * 3 * kContactInline;
    for (int k = 0; k < n; k++)
        if (part[k] == q) { f[3 * k] = 0.0f; f[3 * k + 1] = 0.0f; f[3 * k + 2] = 0.0f; }
}

__global__ void k_attach(const Sim* __restrict__ sims, Ctl* ctl, const int* __restrict__ slots, int n) {
    if ((int)blockIdx.x >= n || threadIdx.x != 0) return;
    const int sim = slots[blockIdx.x];
    Ctl& c = ctl[sim];
    const Sim& S = sims[sim];
    if (c.status != 1 || c.diverged || !(S.flags & SF_ATTACH)) { c.n_cand = 0; return; }
    const int nc = min(c.n_cand, S.cand_cap);
    c.n_cand = 0;
    int* cand = S.cand;
    // insertion sort of the pairs (few per step)
    for (int i = 1; i < nc; i++) {
        const int a = cand[2 * i], b = cand[2 * i + 1];
        int j = i;
        while (j > 0 && (cand[2 * j - 2] > a || (cand[2 * j - 2] == a && cand[2 * j - 1] > b))) {
            cand[2 * j] = cand[2 * j - 2]; cand[2 * j + 1] = cand[2 * j - 1];
            j--;
        }
        cand[2 * j] = a; cand[2 * j + 1] = b;
    }
    const int nv = S.nv;
    for (int i = 0; i < nc; i++) {
        // voxel1 is the later voxel of the pair in the surface list (gpu_update_attach takes
        // first > second, VX3_VoxelyzeKernel.cu:833-843)
        const int v2 = cand[2 * i], v1 = cand[2 * i + 1];
        if ((S.vfl[v1] | S.vfl[v2]) & VF_REMOVED) continue;
        if (linked_within(S, v1, v2, 5)) continue;
        // relative position of voxel2 in voxel1's frame: orientation1.RotateVec3DInv(-(pos1 - pos2))
        const q4 a = Q4(S.qw[v1], S.qx[v1], S.qy[v1], S.qz[v1]);
        const d3 e = D3(S.px[v1] - S.px[v2], S.py[v1] - S.py[v2], S.pz[v1] - S.pz[v2]);
        const d3 ea = qrotinv(a, D3(-e.x, -e.y, -e.z));
        const double fx = fabs(ea.x), fy = fabs(ea.y), fz = fabs(ea.z);
        int axis;
        bool reverse;
        if (fx >= fy && fx >= fz) { axis = 0; reverse = ea.x < 0; }
        else if (fy >= fx && fy >= fz) { axis = 1; reverse = ea.y < 0; }
        else { axis = 2; reverse = ea.z < 0; }
        // the negative-end voxel holds the link in direction 2*axis, the positive end in 2*axis+1
        const int vneg = reverse ? v2 : v1, vpos = reverse ? v1 : v2;
        const int dn = 2 * axis, dp = 2 * axis + 1;
        if (((S.vfl[vneg] >> dn) & 1) || ((S.vfl[vpos] >> dp) & 1)) continue;
        if (c.n_links >= S.nl_cap) continue;
        const int l = c.n_links++;
        const int nl = S.nl_cap;
        S.lneg[l] = vneg; S.lpos[l] = vpos; S.lax[l] = (uint8_t)axis;
        S.lmt[l] = (uint8_t)S.vm[S.vmat[v1]].attachLmat;
        for (int k = 0; k < 9; k++) S.lst[(size_t)k * nl + l] = 0.0;
        S.lsf[l] = 0.0f; S.lsf[nl + l] = 0.0f; S.lsf[2 * nl + l] = 0.0f;
        S.lfl[l] = LF_SMALL;
        S.lnew[l] = S.safety_guard;
        S.vlink[6 * vneg + dn] = l;
        S.vlink[6 * vpos + dp] = l;
        // the new link's slots hold no force yet
        for (int k = 0; k < 3; k++) {
            S.sf[(size_t)(dn * 3 + k) * nv + vneg] = 0.0; S.sm[(size_t)(dn * 3 + k) * nv + vneg] = 0.0;
            S.sf[(size_t)(dp * 3 + k) * nv + vpos] = 0.0; S.sm[(size_t)(dp * 3 + k) * nv + vpos] = 0.0;
        }
        S.ss[(size_t)dn * nv + vneg] = 0.0f;
        S.ss[(size_t)dp * nv + vpos] = 0.0f;
        uint32_t fa = S.vfl[vneg] | (1u << dn), fb = S.vfl[vpos] | (1u << dp);
        if ((fa & VF_LINKS) == VF_LINKS) fa |= VF_INTERIOR;
        if ((fb & VF_LINKS) == VF_LINKS) fb |= VF_INTERIOR;
        S.vfl[vneg] = fa;
        S.vfl[vpos] = fb;
        drop_pair_contact(S, v1, v2);
        drop_pair_contact(S, v2, v1);
    }
}

// Second half of a step's VX3 signals, after every voxel's own signal work: each
// voxel takes the signals its linked neighbours relayed this step, in direction order
// (VX3_Voxel::propagateSignal, VX3_Voxel.cu:323-347, run from the receiving side).
// Runs over the voxel items of simulations whose step completed; the last block of a
// simulation closes its signal phase.
__global__ void __launch_bounds__(256) k_signals(const Sim* __restrict__ sims, Ctl* ctl, const Item* __restrict__ items, int n_items,
                                                 int* tickets) {
    __shared__ int s_item, s_last;
    for (;;) {
        const int it = claim(&tickets[3], &s_item);
        if (it >= n_items) break;
        const Item w = items[it];
        Ctl& c = ctl[w.sim];
        if (!c.sig_pending) continue;
        const Sim& S = sims[w.sim];
        const size_t nv = S.nv;
        for (int v = w.begin + threadIdx.x; v < w.end; v += blockDim.x) {
            const uint32_t f = S.vfl[v];
            if (!(f & VF_LINKS)) continue;
            const VMat& m = S.vm[S.vmat[v]];
            for (int d = 0; d < 6; d++) {
                if (!(f & (1u << d))) continue;
                const int l = S.vlink[6 * v + d];
                const int u = S.lneg[l] == v ? S.lpos[l] : S.lneg[l];
                const double out = S.sig[SG_OUT * nv + u];
                if (out > 0) sig_receive(S, v, m, out, S.sig[SG_OUT_T * nv + u], false);
            }
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) s_last = (atomicAdd(&c.sig_done_items, 1) == c.n_vox_items - 1);
        __syncthreads();
        if (s_last && threadIdx.x == 0) { c.sig_done_items = 0; c.sig_pending = 0; }
    }
}

// Stable time step (CVoxelyze::recommendedTimeStep, Voxelyze3/src/old/Voxelyze.cpp:286-311,
// with CVX_Link::axialStiffness, VX_Link.cpp:251-259): a warp-shuffle max over links.
// The three set-up kernels run for a whole list of newly uploaded simulations at once:
// blockIdx.y picks the simulation (slots[y]), the blocks along x stride over its elements.
__global__ void k_dt(const Sim* __restrict__ sims, Ctl* ctl, const int* __restrict__ slots, int n) {
    if ((int)blockIdx.y >= n) return;
    const int sim = slots[blockIdx.y];
    const Sim& S = sims[sim];
    float best = 0.0f;
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < S.nl; l += gridDim.x * blockDim.x) {
        if (S.lfl[l] & LF_GONE) continue;   // free slots for links made at run time
        const int ng = S.lneg[l], pv = S.lpos[l];
        const LMat& m = S.lm[S.lmt[l]];
        const VMat& vN = S.vm[S.vmat[ng]];
        const VMat& vP = S.vm[S.vmat[pv]];
        float k;
        if (m.nu == 0.0f) k = m.a1;
        else {
            const double rl = 0.5 * (base_size(vN, S.temp[ng]) + base_size(vP, S.temp[pv]));
            const float A = 0.5f * (voxel_tarea(vN, 0.f, 0.f) + voxel_tarea(vP, 0.f, 0.f));
            k = (float)(m.eHat * A / ((S.lsf[l] + 1) * rl));
        }
        const float m1 = vN.mass, m2 = vP.mass;
        const float f2 = k / (m1 < m2 ? m1 : m2);
        if (f2 > best) best = f2;
    }
    for (int o = 16; o > 0; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(&ctl[sim].maxf2_bits, __float_as_uint(best));
}

// Set-up of newly uploaded simulations: initial positions and orientations, and the first
// actuation temperature.
__global__ void k_init_temp(const Sim* __restrict__ sims, const int* __restrict__ slots, const float* __restrict__ initials, int n) {
    if ((int)blockIdx.y >= n) return;
    const Sim& S = sims[slots[blockIdx.y]];
    const float initial = initials[blockIdx.y];
    const float two_pi = 2 * 3.1415926f;
    const int nv = S.nv;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const VMat& m = S.vm[S.vmat[v]];
        // the lattice position and the identity orientation (CVoxelyze::addVoxel places a voxel
        // at its index times the voxel size, Voxelyze3/src/old/Voxelyze.cpp:439-470)
        S.px[v] = (double)S.ijk[v] * m.nom;
        S.py[v] = (double)S.ijk[nv + v] * m.nom;
        S.pz[v] = (double)S.ijk[2 * nv + v] * m.nom;
        S.qw[v] = 1.0;
        if ((S.flags & SF_VARY) && !fp64i::gt(m.thermalOn, 0.0) && !(m.vx3 & VM_FIXED)) {
            double T = S.temp_amp * sin((double)two_pi * (0.0 / S.temp_period + S.phase[v]));
            if (!(S.flags & SF_EXPAND) && T > 0) T = 0;
            S.temp[v] = (float)T;
        } else {
            S.temp[v] = initial;
        }
    }
}

__global__ void k_hash_build(const Sim* __restrict__ sims, Ctl* ctl, const int* __restrict__ slots, int n) {
    if ((int)blockIdx.y >= n) return;
    const int sim = slots[blockIdx.y];
    const Sim& S = sims[sim];
    if (!(S.flags & SF_COLLIDE) || S.nsurf == 0) return;
    int* head = S.hash_head + (size_t)ctl[sim].hash_parity * S.hash_size;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.nsurf; i += gridDim.x * blockDim.x) {
        const int v = S.surf[i];
        if (S.vfl[v] & (VF_INTERIOR | VF_REMOVED)) continue;   // listed only while the surface can change
        hash_insert(S, v, D3(S.px[v], S.py[v], S.pz[v]), S.temp[v], head);
    }
}

// Poses of many simulations packed for one device-to-host copy: blockIdx.y picks the
// simulation, the blocks along x stride over its voxels.  Flags are the voxel flag word
// shifted to the reference's CVX_Voxel bit order (static friction first).
__global__ void k_gather(const Sim* __restrict__ sims, const int* __restrict__ slot, const int64_t* __restrict__ off, int n, double* pos3,
                         double* q4, uint8_t* flags) {
    const int k = blockIdx.y;
    if (k >= n) return;
    const Sim& S = sims[slot[k]];
    const int64_t o = off[k];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < S.nv; v += gridDim.x * blockDim.x) {
        const int64_t i = o + v;
        pos3[3 * i] = S.px[v]; pos3[3 * i + 1] = S.py[v]; pos3[3 * i + 2] = S.pz[v];
        q4[4 * i] = S.qw[v]; q4[4 * i + 1] = S.qx[v]; q4[4 * i + 2] = S.qy[v]; q4[4 * i + 3] = S.qz[v];
        flags[i] = (uint8_t)(S.vfl[v] >> 6);
    }
}

// Mass-weighted centre of mass of measured voxels (VX3_VoxelyzeKernel::updateCurrentCenterOfMass,
// VX3_VoxelyzeKernel.cu:477-493); one block, fixed order.
__global__ void k_com(const Sim* __restrict__ sims, int sim, double* out4) {
    __shared__ double red[256];
    const Sim& S = sims[sim];
    double a[4] = {0, 0, 0, 0};
    for (int v = threadIdx.x; v < S.nv; v += blockDim.x) {
        if (!(S.vfl[v] & VF_MEASURED)) continue;
        const double w = S.vm[S.vmat[v]].mass;
        a[0] += S.px[v] * w; a[1] += S.py[v] * w; a[2] += S.pz[v] * w; a[3] += w;
    }
    for (int k = 0; k < 4; k++) {
        const double r = block_sum(a[k], red);
        if (threadIdx.x == 0) out4[k] = r;
    }
}

}  // namespace GVX_KNS
}  // namespace gvx

// ---------------------------------------------------------------- launch table
namespace gvx {
namespace GVX_KNS {
inline void l_bins(int g, cudaStream_t s, const Sim* sims, Ctl* ctl, BinList la, BinList lb) {
    k_bin_hist<<<g, 256, 0, s>>>(sims, ctl, la, lb);
    k_bin_scan<<<2, 1024, 0, s>>>(la, lb);
    k_bin_scatter<<<g, 256, 0, s>>>(sims, ctl, la, lb);
}
inline void l_links(int g, int b, cudaStream_t s, const Sim* sims, Ctl* ctl, const int2* perm, const int* total, int cap, int n_slots,
                    int* tk, int claim) {
    k_links<<<g, b, 0, s>>>(sims, ctl, perm, total, cap, n_slots, tk, claim);
}
inline void l_contacts(int g, int b, cudaStream_t s, const Sim* sims, Ctl* ctl, const Item* it, int n, int* tk) { k_contacts<<<g, b, 0, s>>>(sims, ctl, it, n, tk); }
inline void l_watch(int g, cudaStream_t s, const Sim* sims, Ctl* ctl, const Item* it, int n_items, const int* stale, const int* tk,
                    const int* slots, int n_sims) {
    (void)slots; (void)n_sims;
    k_watch_build<<<g, 256, 0, s>>>(sims, ctl, it, n_items, stale, tk);
}
inline void l_voxels(int g, int b, cudaStream_t s, const Sim* sims, Ctl* ctl, const int2* perm, const int* total, int cap, int n_slots,
                     int* tk, int claim) {
    k_voxels<<<g, b, 0, s>>>(sims, ctl, perm, total, cap, n_slots, tk, claim);
}
inline void l_sim_end(cudaStream_t s, const Sim* sims, Ctl* ctl, const int* slots, int n, int* tk, int* stale) {
    if (n > 0) k_sim_end<<<n, 256, 0, s>>>(sims, ctl, slots, n, tk, stale);
}
inline void l_signals(int g, int b, cudaStream_t s, const Sim* sims, Ctl* ctl, const Item* it, int n, int* tk) {
    k_signals<<<g, b, 0, s>>>(sims, ctl, it, n, tk);
}
inline void l_attach(cudaStream_t s, const Sim* sims, Ctl* ctl, const int* slots, int n) {
    if (n > 0) k_attach<<<n, 32, 0, s>>>(sims, ctl, slots, n);
}
inline void l_dt(int g, cudaStream_t s, const Sim* sims, Ctl* ctl, const int* slots, int n) {
    for (int k0 = 0; k0 < n; k0 += 65535) k_dt<<<dim3(g, (unsigned)std::min(65535, n - k0)), 256, 0, s>>>(sims, ctl, slots + k0, n - k0);
}
inline void l_init_temp(int g, cudaStream_t s, const Sim* sims, const int* slots, const float* t0, int n) {
    for (int k0 = 0; k0 < n; k0 += 65535)
        k_init_temp<<<dim3(g, (unsigned)std::min(65535, n - k0)), 256, 0, s>>>(sims, slots + k0, t0 + k0, n - k0);
}
inline void l_hash_build(int g, cudaStream_t s, const Sim* sims, Ctl* ctl, const int* slots, int n) {
    for (int k0 = 0; k0 < n; k0 += 65535)
        k_hash_build<<<dim3(g, (unsigned)std::min(65535, n - k0)), 256, 0, s>>>(sims, ctl, slots + k0, n - k0);
}
inline void l_com(cudaStream_t s, const Sim* sims, int sim, double* out4) { k_com<<<1, 256, 0, s>>>(sims, sim, out4); }
inline void l_gather(cudaStream_t s, const Sim* sims, const int* slot, const int64_t* off, int n, double* pos3, double* q4, uint8_t* fl) {
    if (n > 0) k_gather<<<dim3(8, (unsigned)n), 256, 0, s>>>(sims, slot, off, n, pos3, q4, fl);
}
// Resident blocks per SM of the persistent grids at a block size (what the register use allows).
inline int l_resident_blocks(int which, int block) {
    static int cached[2][33] = {};
    block = block < 32 ? 32 : (block > 1024 ? 1024 : block & ~31);
    int& n = cached[which ? 1 : 0][block >> 5];
    if (n == 0) {
        int r = 0;
        if (which == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_links, block, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_voxels, block, 0);
        n = r > 0 ? r : 1;
    }
    return n;
}
inline KernelSet make_kernelset(const char* name) {
    return KernelSet{name, l_bins, l_links, l_contacts, l_voxels, l_sim_end, l_signals, l_attach, l_dt, l_init_temp, l_hash_build, l_com,
                     l_gather, l_resident_blocks, GVX_STEP_BLOCK, l_watch};
}
}  // namespace GVX_KNS
}  // namespace gvx
