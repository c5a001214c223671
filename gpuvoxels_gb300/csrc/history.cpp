// .history stream writer (see history.h).  Number formats are the reference's printf
// formats; values are formed in the reference's types (float corner offsets, double
// positions).
#include "history.h"
#include "layout.cuh"

#include <cmath>
#include <cstdio>

namespace gvx {

namespace {

void appendf(std::string* s, const char* fmt, double a) {
    char b[64];
    snprintf(b, sizeof(b), fmt, a);
    *s += b;
}

// (int)(colour * 255) clamped to 0..255 (CVXC_Material::GetRedi, VXA/VX_Object.h:419;
// CVX_Material::setRed, old/VX_Material.cpp:253-258)
int color_byte(float c) {
    int v = (int)(c * 255);
    return v > 255 ? 255 : (v < 0 ? 0 : v);
}

// VX3_Link::axialStrain(positiveEnd), VX3/VX3_Link.cu:72-74
float axial_strain(const SimWorld& w, int l, float strain, bool positive_end) {
    const float ratio = w.vmats[w.desc.voxels[4 * w.link_pos[l] + 3]].E / w.vmats[w.desc.voxels[4 * w.link_neg[l] + 3]].E;
    return positive_end ? 2.0f * strain * ratio / (1.0f + ratio) : 2.0f * strain / (1.0f + ratio);
}

}  // namespace

int history_step_interval(const SimWorld& w, double optimal_dt) {
    return (int)(w.desc.record_step_size / (10000 * optimal_dt * w.desc.dt_frac)) + 1;
}

std::string history_header(const SimWorld& w, double optimal_dt) {
    std::string s = "\n{{{setting}}}<rescale>0.001</rescale>\n";
    for (size_t i = 0; i < w.desc.mats.size(); i++) {
        const float* c = w.desc.mats[i].rgba;
        char b[256];
        snprintf(b, sizeof(b), "{{{setting}}}<matcolor><id>%d</id><r>%.2f</r><g>%.2f</g><b>%.2f</b><a>%.2f</a></matcolor>\n",
                 (int)i + 1, color_byte(c[0]) / 255., color_byte(c[1]) / 255., color_byte(c[2]) / 255., color_byte(c[3]) / 255.);
        s += b;
    }
    appendf(&s, "\n{{{setting}}}<voxel_size>%f</voxel_size>\n", w.desc.vox_size);
    char b[256];
    snprintf(b, sizeof(b), "real_stepsize: %d ; recommendedTimeStep %f; d_v3->DtFrac %f . \n", history_step_interval(w, optimal_dt),
             optimal_dt, w.desc.dt_frac);
    s += b;
    return s;
}

// Temperature voxel v had during the step that ended at time t: the reference sets it from the
// time at the start of the step (VX3_VoxelyzeKernel.cu:625-650).  The engine already holds the
// next step's value, so varying temperatures are formed again from t - dt.
float step_temperature(const SimWorld& w, int v, double t, float dt, const float* f4) {
    const SimDesc& d = w.desc;
    if (!(d.vary_temp && d.temp_period > 0)) return f4[4 * (size_t)v];
    const float two_pi = 2 * 3.1415926f;
    double T = d.temp_amplitude * sin((double)two_pi * ((t - dt) / d.temp_period + d.phase[v]));
    if (!d.enable_expansion && T > 0) T = 0;
    return (float)T;
}

std::string history_record(const SimWorld& w, int64_t j, double t, float dt, const double* d13, const float* f4, const float* lsf3,
                           const int32_t* vflags, const int32_t* lflags, const double* local_signal, const int32_t* links4,
                           int n_links) {
    const double vs = 1 / 0.001;
    std::string s;
    char b[512];
    const int nl = w.nl;
    if (w.desc.record_voxel) {
        snprintf(b, sizeof(b), "<<<Step%lld Time:%f>>>", (long long)j, t);
        s += b;
        for (int v = 0; v < w.nv; v++) {
            // surface voxels only, in voxel order; removed voxels are left out
            if (vflags ? (vflags[v] & (dev::VF_INTERIOR | dev::VF_REMOVED)) != 0 : w.vox_interior[v] != 0) continue;
            const double* p = d13 + 13 * (size_t)v;
            const double qw = p[6], qx = p[7], qy = p[8], qz = p[9];
            snprintf(b, sizeof(b), "%.1f,%.1f,%.1f,", p[0] * vs, p[1] * vs, p[2] * vs);
            s += b;
            const double angle = 2.0 * acos(qw > 1 ? 1 : qw) * 57.29577951308232;   // Quat3D::AngleDegrees
            snprintf(b, sizeof(b), "%.1f,%.2f,%.2f,%.2f,", angle, qx, qy, qz);
            s += b;
            // VX3_Voxel::cornerOffset(NNN) and (PPP), VX3/VX3_Voxel.cu:147-159
            const int mi = w.desc.voxels[4 * v + 3];
            const VoxelMaterial& m = w.vmats[mi];
            const double half_size = 0.5 * (m.nom * (1 + step_temperature(w, v, t, dt, f4) * m.cte));
            float nnn[3], ppp[3];
            for (int i = 0; i < 3; i++) {
                for (int corner = 0; corner < 2; corner++) {
                    const bool pos_link = corner == 1;
                    const int d = 2 * i + (pos_link ? 0 : 1);
                    const int l = w.vox_links[6 * (size_t)v + d];
                    double st = pos_link ? 1.0 : -1.0;
                    if (l >= 0 && (!vflags || (vflags[v] >> d) & 1)) {   // a detached link is no longer the voxel's
                        const LinkMaterial& lm = w.lmats[w.link_mat[l]];
                        const bool failed = lm.epsFail != -1.0f && lsf3[3 * (size_t)l + 1] > lm.epsFail;
                        if (!failed) st = (1 + axial_strain(w, l, lsf3[3 * (size_t)l], pos_link)) * (pos_link ? 1 : -1);
                    }
                    (pos_link ? ppp : nnn)[i] = (float)(half_size * st);
                }
            }
            snprintf(b, sizeof(b), "%.1f,%.1f,%.1f,%.1f,%.1f,%.1f,", nnn[0] * vs, nnn[1] * vs, nnn[2] * vs, ppp[0] * vs, ppp[1] * vs,
                     ppp[2] * vs);
            s += b;
            snprintf(b, sizeof(b), "%d,", mi + 1);
            s += b;
            snprintf(b, sizeof(b), "%.1f,;", local_signal ? local_signal[v] : 0.0);   // localSignal (for colouring)
            s += b;
        }
        s += "<<<>>>";
    }
    if (w.desc.record_link) {
        snprintf(b, sizeof(b), "|[[[%lld]]]", (long long)j);
        s += b;
        const int n = links4 ? n_links : nl;
        for (int l = 0; l < n; l++) {
            const int fl = links4 ? links4[4 * l + 3] : (lflags ? lflags[l] : 0);
            if (fl & dev::LF_REMOVED) continue;   // links removed with their voxels
            const int lp = links4 ? links4[4 * l + 1] : w.link_pos[l], ln = links4 ? links4[4 * l] : w.link_neg[l];
            const double* a = d13 + 13 * (size_t)lp;
            const double* c = d13 + 13 * (size_t)ln;
            snprintf(b, sizeof(b), "%.4f,%.4f,%.4f,%.4f,%.4f,%.4f,;", a[0], a[1], a[2], c[0], c[1], c[2]);
            s += b;
        }
        s += "[[[]]]";
    }
    s += "\n";
    return s;
}

}  // namespace gvx
