// Formula trees of the VXA file (stop condition, fitness): the token format
// and evaluation rule of Voxelyze3/src/Utils/VX3_MathTree.h:4-192, parsed as in
// VX3_SimulationManager::ParseMathTree (Voxelyze3/src/VX3/VX3_SimulationManager.cu:157-275):
// the XML subtree is walked breadth-first, and the reversed walk is evaluated
// with a value queue, each operator consuming the oldest unconsumed values.
#pragma once
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define GVX_HD __host__ __device__
#else
#define GVX_HD
#endif

namespace gvx {

enum MathOp : int32_t {
    mtEND, mtCONST, mtE, mtPI, mtVAR, mtADD, mtSUB, mtMUL, mtDIV, mtPOW, mtSQRT, mtSIN, mtCOS, mtTAN,
    mtATAN, mtLOG, mtINT, mtABS, mtNOT, mtGREATERTHAN, mtLESSTHAN, mtAND, mtOR, mtNORMALCDF
};

constexpr int kMaxMathTokens = 64;

struct MathToken {
    int32_t op;
    int32_t pad;
    double value;
};

// A parsed formula.  n == 0 means "absent" (the reference evaluates an
// all-mtEND buffer, whose value is undefined; absent formulas are reported as NaN).
struct MathTree {
    int32_t n = 0;
    int32_t valid = 1;
    MathToken tok[kMaxMathTokens];
};

struct MathVars {
    double x, y, z, hit, t, angle, closeness;
    int num_close_pairs, num_voxel;
};

GVX_HD inline double mathtree_eval(const MathTree& m, const MathVars& v) {
    if (m.n == 0 || !m.valid) return NAN;
    double vals[kMaxMathTokens];
    int vc = 0, pc = 0;
    for (int i = 0; i < m.n && i < kMaxMathTokens; i++) {
        const MathToken& k = m.tok[i];
        double r = 0;
        switch (k.op) {
        case mtEND: return vals[pc];
        case mtCONST: r = k.value; break;
        case mtE: r = 2.71828182845904523536; break;
        case mtPI: r = 3.14159265358979323846; break;
        case mtVAR:
            if (k.value < 0.5) r = v.x;
            else if (k.value < 1.5) r = v.y;
            else if (k.value < 2.5) r = v.z;
            else if (k.value < 3.5) r = v.hit;
            else if (k.value < 4.5) r = v.t;
            else if (k.value < 5.5) r = v.angle;
            else if (k.value < 6.5) r = v.closeness;
            else if (k.value < 7.5) r = v.num_close_pairs;
            else r = v.num_voxel;
            break;
        case mtSIN: r = sin(vals[pc++]); break;
        case mtCOS: r = cos(vals[pc++]); break;
        case mtTAN: r = tan(vals[pc++]); break;
        case mtATAN: r = atan(vals[pc++]); break;
        case mtLOG: r = log(vals[pc++]); break;
        case mtINT: r = rint(vals[pc++]); break;
        case mtNORMALCDF: r = 0.5 * erfc(-vals[pc] / 1.41421356237309504880); pc++; break;
        case mtSQRT: r = sqrt(vals[pc++]); break;
        case mtABS: r = fabs(vals[pc++]); break;
        case mtNOT: r = !vals[pc]; pc++; break;
        case mtADD: r = vals[pc + 1] + vals[pc]; pc += 2; break;
        case mtSUB: r = vals[pc + 1] - vals[pc]; pc += 2; break;
        case mtMUL: r = vals[pc + 1] * vals[pc]; pc += 2; break;
        case mtDIV: r = vals[pc + 1] / vals[pc]; pc += 2; break;
        case mtPOW: r = pow(vals[pc + 1], vals[pc]); pc += 2; break;
        case mtGREATERTHAN: r = vals[pc + 1] > vals[pc]; pc += 2; break;
        case mtLESSTHAN: r = vals[pc + 1] < vals[pc]; pc += 2; break;
        case mtAND: r = vals[pc + 1] && vals[pc]; pc += 2; break;
        case mtOR: r = vals[pc + 1] || vals[pc]; pc += 2; break;
        default: return NAN;
        }
        if (pc > vc) return NAN;
        vals[vc++] = r;
    }
    return NAN;
}

}  // namespace gvx
