// C ABI over the engine (declarations and reference citations in include/gpuvoxels_gb300.h).
#include "../../include/gpuvoxels_gb300.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"
#include "history.h"
#include "world.h"

// A simulation whose steps are written to a .history file.
struct HistoryState {
    FILE* f = nullptr;
    bool header = false;
    int interval = 1;
    int64_t last_j = -1;
};

struct vx3_ctx {
    gvx::Engine* eng = nullptr;
    std::string err;
    std::map<int64_t, std::string> names;
    std::map<int64_t, HistoryState> hist;
};

namespace {
int fail(vx3_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    return code;
}
void to_c(const gvx::SimResult& r, vx3_result* o) {
    o->id = r.id;
    o->status = r.status;
    o->num_voxel = r.num_voxel;
    o->num_measured_voxel = r.num_measured_voxel;
    o->num_close_pairs = r.num_close_pairs;
    o->steps = r.steps;
    o->current_time = r.current_time;
    o->fitness_score = r.fitness;
    o->vox_size = r.vox_size;
    for (int k = 0; k < 3; k++) { o->initial_center_of_mass[k] = r.initial_com[k]; o->current_center_of_mass[k] = r.current_com[k]; }
    o->total_distance_of_all_voxels = r.total_distance;
    o->submit_time_s = r.submit_s;
    o->start_time_s = r.start_s;
    o->finish_time_s = r.finish_s;
}
std::string num(double v) {
    char b[64];
    snprintf(b, sizeof(b), "%.17g", v);
    return b;
}
}  // namespace

extern "C" {

vx3_ctx* vx3_create(int device, size_t budget) {
    std::string err;
    gvx::Engine* e = gvx::engine_create(device, budget, &err);
    if (!e) {
        fprintf(stderr, "vx3_create: %s\n", err.c_str());
        return nullptr;
    }
    vx3_ctx* c = new vx3_ctx();
    c->eng = e;
    return c;
}

void vx3_destroy(vx3_ctx* c) {
    if (!c) return;
    for (auto& kv : c->hist)
        if (kv.second.f) fclose(kv.second.f);
    gvx::engine_destroy(c->eng);
    delete c;
}

const char* vx3_last_error(vx3_ctx* c) { return c ? c->err.c_str() : "null context"; }

int vx3_load_vxa(vx3_ctx* c, const char* base, const char* vxd, const char* name, vx3_sim_id* out) {
    if (!c || !base || !out) return fail(c, VX3_E_ARG, "null argument");
    gvx::SimDesc d;
    std::string err;
    if (!gvx::parse_vxa(base, vxd, &d, &err)) return fail(c, VX3_E_PARSE, err);
    d.name = name ? name : "";
    int64_t id;
    if (c->eng->add_sim(d, &id, &err)) return fail(c, VX3_E_PARSE, err);
    c->names[id] = d.name;
    *out = id;
    return VX3_OK;
}

int vx3_load_vxa_many(vx3_ctx* c, const char* base, const char* const* vxds, const char* const* names, int n, vx3_sim_id* ids,
                      int* status) {
    if (!c || !ids || n < 0 || (!base && !vxds)) return fail(c, VX3_E_ARG, "null argument");
    if (!base)
        for (int i = 0; i < n; i++)
            if (!vxds[i]) return fail(c, VX3_E_ARG, "without a base every entry must be a whole VXA");
    // each VXD merged into its own copy of the base, read and built on the engine's host threads
    std::vector<std::string> errs((size_t)n);
    std::vector<int> rc((size_t)n, VX3_OK);
    std::vector<int64_t> got((size_t)n, -1);
    c->eng->add_sims_read(n, [&](int i, gvx::SimDesc* d, std::string* e) {
        const bool ok = base ? gvx::parse_vxa(base, vxds ? vxds[i] : nullptr, d, e) : gvx::parse_vxa(vxds[i], nullptr, d, e);
        d->name = (names && names[i]) ? names[i] : "";
        return ok;
    }, got.data(), errs.data());
    for (int i = 0; i < n; i++) {
        if (got[i] < 0) { rc[i] = VX3_E_PARSE; continue; }
        ids[i] = got[i];
        c->names[got[i]] = (names && names[i]) ? names[i] : "";
    }
    int first = VX3_OK;
    for (int i = 0; i < n; i++) {
        if (rc[i] != VX3_OK) {
            ids[i] = -1;
            if (first == VX3_OK) { first = rc[i]; c->err = "simulation " + std::to_string(i) + ": " + errs[i]; }
        }
        if (status) status[i] = rc[i];
    }
    return first;
}

int vx3_set_external(vx3_ctx* c, vx3_sim_id id, int voxel, int dof, const float force[3], const float moment[3],
                     const double translate[3], const double rotate[3]) {
    if (!c) return VX3_E_ARG;
    gvx::External x;
    x.voxel = voxel;
    x.dof_fixed = dof;
    for (int k = 0; k < 3; k++) {
        x.force[k] = force ? force[k] : 0.0f;
        x.moment[k] = moment ? moment[k] : 0.0f;
        x.translate[k] = translate ? translate[k] : 0.0;
        x.rotate[k] = rotate ? rotate[k] : 0.0;
    }
    std::string err;
    int e = c->eng->set_external(id, x, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

}  // extern "C"

namespace {
bool any_history(vx3_ctx* c, const vx3_sim_id* ids, int n) {
    for (int i = 0; i < n; i++)
        if (c->hist.count(ids[i])) return true;
    return false;
}

// Writes the header (once the first step has fixed the time step) and a record for every
// recording simulation that has just completed a recorded loop step.
int history_after_chunk(vx3_ctx* c, const vx3_sim_id* ids, int n) {
    for (int i = 0; i < n; i++) {
        auto it = c->hist.find(ids[i]);
        if (it == c->hist.end()) continue;
        HistoryState& h = it->second;
        int nv, nl, status;
        double dt, t;
        int64_t steps;
        if (c->eng->info(ids[i], &nv, &nl, &dt, &t, &steps, &status)) continue;
        const gvx::SimWorld* w = c->eng->world(ids[i]);
        if (!w || steps == 0) continue;
        if (!h.header) {
            const double opt = c->eng->optimal_dt(ids[i]);
            h.interval = gvx::history_step_interval(*w, opt);
            const std::string hd = gvx::history_header(*w, opt);
            fwrite(hd.data(), 1, hd.size(), h.f);
            h.header = true;
        }
        const int64_t j = steps - 1;                 // the reference's loop index of the last step
        if (j % h.interval != 0 || j == h.last_j) continue;
        std::vector<double> d13(13 * (size_t)nv);
        std::vector<float> f4(4 * (size_t)nv), lsf(3 * (size_t)std::max(nl, 1));
        std::vector<int32_t> vf((size_t)nv), lf((size_t)std::max(nl, 1));
        std::string err;
        if (int e = c->eng->voxel_state(ids[i], d13.data(), f4.data(), vf.data(), &err)) return fail(c, e, err);
        std::vector<double> ld(9 * (size_t)std::max(nl, 1));
        if (nl > 0)
            if (int e = c->eng->link_state(ids[i], ld.data(), lsf.data(), lf.data(), &err)) return fail(c, e, err);
        std::vector<double> sig;
        if (w->desc.enable_signals) {
            sig.resize(6 * (size_t)nv);
            if (int e = c->eng->extras(ids[i], nullptr, sig.data(), &err)) return fail(c, e, err);
            for (int v = 0; v < nv; v++) sig[v] = sig[6 * (size_t)v];   // localSignal of each voxel
        }
        std::vector<int32_t> l4;
        int32_t n_links = 0;
        if (w->desc.enable_attach) {   // links made during the run are recorded too
            if (int e = c->eng->links(ids[i], &n_links, nullptr, 0, &err)) return fail(c, e, err);
            l4.resize(4 * (size_t)std::max(n_links, 1));
            if (int e = c->eng->links(ids[i], &n_links, l4.data(), n_links, &err)) return fail(c, e, err);
        }
        const std::string rec = gvx::history_record(*w, j, t, (float)dt, d13.data(), f4.data(), lsf.data(), vf.data(),
                                                    nl > 0 ? lf.data() : nullptr, sig.empty() ? nullptr : sig.data(),
                                                    l4.empty() ? nullptr : l4.data(), n_links);
        fwrite(rec.data(), 1, rec.size(), h.f);
        fflush(h.f);
        h.last_j = j;
    }
    return VX3_OK;
}

// Steps in chunks that end on every recorded step of every recording simulation.
// steps < 0: until every listed simulation has stopped (or max_steps).
int drive_with_history(vx3_ctx* c, const vx3_sim_id* ids, int n, int mode, int64_t steps, int64_t max_steps) {
    int64_t done = 0;
    const int64_t limit = steps >= 0 ? steps : (max_steps > 0 ? max_steps : INT64_MAX);
    while (done < limit) {
        int64_t chunk = std::min<int64_t>(limit - done, 4096);
        bool running = false;
        for (int i = 0; i < n; i++) {
            int nv, nl, status;
            double dt, t;
            int64_t s;
            if (c->eng->info(ids[i], &nv, &nl, &dt, &t, &s, &status)) continue;
            if (status == gvx::SIM_IDLE || status == gvx::SIM_RUNNING) running = true;
            else continue;
            auto it = c->hist.find(ids[i]);
            if (it == c->hist.end()) continue;
            const HistoryState& h = it->second;
            if (!h.header) { chunk = 1; continue; }
            // next loop index j > s - 1 with j % interval == 0, completed after step j + 1
            const int64_t jn = ((s - 1) / h.interval + 1) * h.interval;
            chunk = std::min(chunk, std::max<int64_t>(1, jn + 1 - s));
        }
        if (!running) break;
        std::string err;
        if (int e = c->eng->step(ids, n, mode, chunk, &err)) return fail(c, e, err);
        done += chunk;
        if (int e = history_after_chunk(c, ids, n)) return e;
    }
    return VX3_OK;
}
}  // namespace

extern "C" {

int vx3_run(vx3_ctx* c, const vx3_sim_id* ids, int n, int mode, int64_t max_steps) {
    if (!c || (!ids && n > 0) || n < 0) return fail(c, VX3_E_ARG, "bad arguments");
    if (any_history(c, ids, n)) return drive_with_history(c, ids, n, mode, -1, max_steps);
    std::string err;
    int e = c->eng->run(ids, n, mode, max_steps, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_step(vx3_ctx* c, const vx3_sim_id* ids, int n, int mode, int64_t steps) {
    if (!c || (!ids && n > 0) || n < 0 || steps < 0) return fail(c, VX3_E_ARG, "bad arguments");
    if (any_history(c, ids, n)) return drive_with_history(c, ids, n, mode, steps, 0);
    std::string err;
    int e = c->eng->step(ids, n, mode, steps, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_record_history(vx3_ctx* c, vx3_sim_id id, const char* path) {
    if (!c) return VX3_E_ARG;
    auto it = c->hist.find(id);
    if (it != c->hist.end()) {
        if (it->second.f) fclose(it->second.f);
        c->hist.erase(it);
    }
    if (!path) return VX3_OK;
    const gvx::SimWorld* w = c->eng->world(id);
    if (!w) return fail(c, VX3_E_ARG, "unknown simulation id");
    if (w->desc.record_step_size <= 0) return fail(c, VX3_E_ARG, "the VXA sets no Simulator/RecordHistory/RecordStepSize");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(c, VX3_E_ARG, std::string("cannot open ") + path);
    HistoryState h;
    h.f = f;
    c->hist[id] = h;
    return VX3_OK;
}

int vx3_submit(vx3_ctx* c, vx3_sim_id id, int64_t horizon) {
    if (!c) return VX3_E_ARG;
    std::string err;
    int e = c->eng->submit(id, horizon, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_poll(vx3_ctx* c, vx3_result* out, int max, int chunk) {
    if (!c || (max > 0 && !out)) return VX3_E_ARG;
    std::vector<gvx::SimResult> rs((size_t)std::max(1, max));
    std::string err;
    int n = c->eng->poll(rs.data(), max, chunk, &err);
    if (n < 0) return fail(c, n, err);
    for (int i = 0; i < n; i++) to_c(rs[i], &out[i]);
    return n;
}

int vx3_pending(vx3_ctx* c) { return c ? c->eng->pending() : VX3_E_ARG; }

int vx3_get_result(vx3_ctx* c, vx3_sim_id id, vx3_result* out) {
    if (!c || !out) return VX3_E_ARG;
    gvx::SimResult r;
    std::string err;
    int e = c->eng->result(id, &r, &err);
    if (e) return fail(c, e, err);
    to_c(r, out);
    return VX3_OK;
}

int vx3_sim_sizes(vx3_ctx* c, const vx3_sim_id* ids, int n, int32_t* num_voxel, int32_t* num_link) {
    if (!c || (!ids && n > 0) || n < 0) return VX3_E_ARG;
    for (int k = 0; k < n; k++) {
        const gvx::SimWorld* w = c->eng->world(ids[k]);
        if (!w) return fail(c, VX3_E_ARG, "unknown simulation id");
        if (num_voxel) num_voxel[k] = w->nv;
        if (num_link) num_link[k] = w->nl;
    }
    return VX3_OK;
}

int vx3_sim_info_get(vx3_ctx* c, vx3_sim_id id, vx3_sim_info* out) {
    if (!c || !out) return VX3_E_ARG;
    int nv, nl, st;
    double dt, t;
    int64_t steps;
    int e = c->eng->info(id, &nv, &nl, &dt, &t, &steps, &st);
    if (e) return fail(c, e, "unknown simulation id");
    out->num_voxel = nv;
    out->num_link = nl;
    out->status = st;
    out->pad = 0;
    out->dt = dt;
    out->current_time = t;
    out->steps = steps;
    return VX3_OK;
}

int vx3_get_state(vx3_ctx* c, vx3_sim_id id, double* pos, double* orient, uint8_t* flags) {
    if (!c) return VX3_E_ARG;
    vx3_sim_info info;
    if (int e = vx3_sim_info_get(c, id, &info)) return e;
    std::vector<double> d13((size_t)info.num_voxel * 13);
    std::vector<int32_t> fl((size_t)info.num_voxel);
    std::string err;
    int e = c->eng->voxel_state(id, d13.data(), nullptr, fl.data(), &err);
    if (e) return fail(c, e, err);
    for (int i = 0; i < info.num_voxel; i++) {
        if (pos) for (int k = 0; k < 3; k++) pos[3 * (size_t)i + k] = d13[13 * (size_t)i + k];
        if (orient) for (int k = 0; k < 4; k++) orient[4 * (size_t)i + k] = d13[13 * (size_t)i + 6 + k];
        if (flags) flags[i] = (uint8_t)(fl[i] >> 6);
    }
    return VX3_OK;
}

int vx3_get_states(vx3_ctx* c, const vx3_sim_id* ids, int n, double* pos, double* orient, uint8_t* flags) {
    if (!c || n < 0 || (n > 0 && !ids)) return VX3_E_ARG;
    std::string err;
    int e = c->eng->gather_states(ids, n, pos, orient, flags, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_get_voxel_state(vx3_ctx* c, vx3_sim_id id, double* d13, float* f4, int32_t* flags) {
    if (!c) return VX3_E_ARG;
    std::string err;
    int e = c->eng->voxel_state(id, d13, f4, flags, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_get_link_state(vx3_ctx* c, vx3_sim_id id, double* d9, float* f3, int32_t* flags) {
    if (!c) return VX3_E_ARG;
    std::string err;
    int e = c->eng->link_state(id, d9, f3, flags, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_get_links(vx3_ctx* c, vx3_sim_id id, int32_t* n_links, int32_t* ends4, int max) {
    if (!c || !n_links || max < 0) return VX3_E_ARG;
    std::string err;
    int e = c->eng->links(id, n_links, ends4, max, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_transfer_bytes(vx3_ctx* c, int64_t* h2d, int64_t* d2h) {
    if (!c || !h2d || !d2h) return VX3_E_ARG;
    c->eng->transfer_bytes(h2d, d2h);
    return VX3_OK;
}

int vx3_get_extras(vx3_ctx* c, vx3_sim_id id, double* measures4, double* signals6) {
    if (!c) return VX3_E_ARG;
    std::string err;
    int e = c->eng->extras(id, measures4, signals6, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

}  // extern "C"

namespace {
// One simulation's report entry: its result, file name and (SavePositionOfAllVoxels) positions.
struct ReportEntry {
    vx3_result r;
    std::string name;
    int save = 0;
    std::vector<double> init, cur;
    std::vector<int> mats;
};

int collect_entries(vx3_ctx* c, const vx3_sim_id* ids, int n, std::vector<ReportEntry>* out) {
    for (int i = 0; i < n; i++) {
        ReportEntry e;
        if (int rc = vx3_get_result(c, ids[i], &e.r)) return rc;
        e.name = c->names[ids[i]];
        if (int rc = c->eng->saved_positions(ids[i], &e.save, &e.init, &e.cur, &e.mats, &c->err)) return rc;
        out->push_back(std::move(e));
    }
    return VX3_OK;
}

// Positions as the worker prints them: std::to_string per coordinate, "x,y,z;" per voxel.
std::string pos_list(const std::vector<double>& p) {
    std::string s;
    for (size_t i = 0; i + 2 < p.size(); i += 3)
        s += std::to_string(p[i]) + "," + std::to_string(p[i + 1]) + "," + std::to_string(p[i + 2]) + ";";
    return s;
}

// The worker's report (vx3_node_worker.cu:98-141), results sorted by VX3_SimulationResult::compareFitnessScore.
int write_report_file(std::vector<ReportEntry>& rs, const char* input_dir, const char* path, std::string* err) {
    // diverged (NaN) last, then descending fitness
    std::stable_sort(rs.begin(), rs.end(), [](const ReportEntry& a, const ReportEntry& b) {
        if (std::isnan(b.r.fitness_score)) return !std::isnan(a.r.fitness_score);
        if (std::isnan(a.r.fitness_score)) return false;
        return a.r.fitness_score > b.r.fitness_score;
    });
    std::string dir = input_dir ? input_dir : "";
    while (!dir.empty() && dir.back() == '/') dir.pop_back();
    size_t slash = dir.rfind('/');
    if (slash != std::string::npos) dir = dir.substr(slash + 1);
    std::string o = "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n<report><inputdir>" + gvx::xml_escape(dir) + "</inputdir>";
    if (!rs.empty())
        o += "<bestfit><filename>" + gvx::xml_escape(rs[0].name) + "</filename><fitness_score>" + num(rs[0].r.fitness_score) +
             "</fitness_score></bestfit>";
    o += "<detail>";
    for (auto& p : rs) {
        std::string nm = p.name.substr(0, p.name.find('.'));
        if (nm.empty()) nm = "sim" + std::to_string(p.r.id);
        const vx3_result& r = p.r;
        o += "<" + nm + ">";
        o += "<currentTime>" + num(r.current_time) + "</currentTime>";
        o += "<fitness_score>" + num(r.fitness_score) + "</fitness_score>";
        o += "<num_voxel>" + std::to_string(r.num_voxel) + "</num_voxel>";
        o += "<num_measured_voxel>" + std::to_string(r.num_measured_voxel) + "</num_measured_voxel>";
        o += "<voxSize>" + num(r.vox_size) + "</voxSize>";
        o += "<numClosePairs>" + std::to_string(r.num_close_pairs) + "</numClosePairs>";
        o += "<initialCenterOfMass><x>" + num(r.initial_center_of_mass[0]) + "</x><y>" + num(r.initial_center_of_mass[1]) + "</y><z>" +
             num(r.initial_center_of_mass[2]) + "</z></initialCenterOfMass>";
        o += "<currentCenterOfMass><x>" + num(r.current_center_of_mass[0]) + "</x><y>" + num(r.current_center_of_mass[1]) + "</y><z>" +
             num(r.current_center_of_mass[2]) + "</z></currentCenterOfMass>";
        o += "<total_distance_of_all_voxels>" + num(r.total_distance_of_all_voxels) + "</total_distance_of_all_voxels>";
        if (p.save) {
            o += "<init_pos>" + pos_list(p.init) + "</init_pos>";
            o += "<pos>" + pos_list(p.cur) + "</pos>";
            std::string m;
            for (int id : p.mats) m += std::to_string(id) + ";";
            o += "<mats>" + m + "</mats>";
        }
        o += "</" + nm + ">";
    }
    o += "</detail></report>\n";
    FILE* f = fopen(path, "wb");
    if (!f) { *err = std::string("cannot open ") + path; return VX3_E_ARG; }
    fwrite(o.data(), 1, o.size(), f);
    fclose(f);
    return VX3_OK;
}
}  // namespace

extern "C" {

int vx3_write_report(vx3_ctx* c, const vx3_sim_id* ids, int n, const char* input_dir, const char* path) {
    if (!c || !path || (n > 0 && !ids)) return VX3_E_ARG;
    std::vector<ReportEntry> rs;
    if (int e = collect_entries(c, ids, n, &rs)) return e;
    return write_report_file(rs, input_dir, path, &c->err);
}

int vx3_write_report_multi(vx3_ctx* const* ctxs, const vx3_sim_id* const* ids, const int* counts, int nctx, const char* input_dir,
                           const char* path) {
    if (!ctxs || !ids || !counts || nctx <= 0 || !path) return VX3_E_ARG;
    std::vector<ReportEntry> rs;
    for (int k = 0; k < nctx; k++) {
        if (!ctxs[k] || (counts[k] > 0 && !ids[k])) return VX3_E_ARG;
        if (int e = collect_entries(ctxs[k], ids[k], counts[k], &rs)) return e;
    }
    return write_report_file(rs, input_dir, path, &ctxs[0]->err);
}

int vx3_free_sim(vx3_ctx* c, vx3_sim_id id) {
    if (!c) return VX3_E_ARG;
    c->names.erase(id);
    auto h = c->hist.find(id);
    if (h != c->hist.end()) {
        if (h->second.f) fclose(h->second.f);
        c->hist.erase(h);
    }
    return c->eng->free_sim(id) ? fail(c, VX3_E_ARG, "unknown simulation id") : VX3_OK;
}

int vx3_last_timing(vx3_ctx* c, double* out) {
    if (!c || !out) return VX3_E_ARG;
    const gvx::Timing& t = c->eng->timing();
    out[0] = t.device_ms;
    out[1] = t.wall_ms;
    out[2] = (double)t.voxel_steps;
    out[3] = (double)t.launches;
    out[4] = t.link_kernel_ms;
    out[5] = t.contact_kernel_ms;
    out[6] = t.voxel_kernel_ms;
    return VX3_OK;
}

int vx3_set_tuning(vx3_ctx* c, int bl, int bv, int il, int iv, int gs) {
    if (!c) return VX3_E_ARG;
    return c->eng->set_tuning(bl, bv, il, iv, gs);
}

int vx3_autotune(vx3_ctx* c, const vx3_sim_id* ids, int n) {
    if (!c) return VX3_E_ARG;
    std::string err;
    int e = c->eng->autotune(ids, n, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_set_serving(vx3_ctx* c, int order, int64_t max_active_voxels) {
    if (!c) return VX3_E_ARG;
    return c->eng->set_serving(order, max_active_voxels) ? fail(c, VX3_E_ARG, "order must be 0, 1 or 2, the voxel cap >= 0") : VX3_OK;
}

int vx3_set_claim_sizes(vx3_ctx* c, int claim_links, int claim_voxels) {
    if (!c || claim_links < 0 || claim_voxels < 0) return VX3_E_ARG;
    return c->eng->set_claims(claim_links, claim_voxels);
}

int vx3_set_contact_slots(vx3_ctx* c, int slots) {
    if (!c) return VX3_E_ARG;
    return c->eng->set_contact_slots(slots) ? fail(c, VX3_E_ARG, "contact slots must be 1..16") : VX3_OK;
}

int vx3_get_tuning(vx3_ctx* c, int32_t* out8) {
    if (!c || !out8) return VX3_E_ARG;
    c->eng->get_tuning(out8);
    return VX3_OK;
}

int vx3_set_profiling(vx3_ctx* c, int on) {
    if (!c) return VX3_E_ARG;
    c->eng->set_profiling(on);
    return VX3_OK;
}

int64_t vx3_sim_bytes(vx3_ctx* c, vx3_sim_id id) {
    if (!c) return VX3_E_ARG;
    int64_t b = c->eng->sim_bytes_id(id);
    return b < 0 ? fail(c, VX3_E_ARG, "unknown simulation id") : b;
}

int vx3_set_precision(vx3_ctx* c, int mode) {
    if (!c || (mode != VX3_EXACT && mode != VX3_FMA)) return fail(c, VX3_E_ARG, "precision must be VX3_EXACT or VX3_FMA");
    return c->eng->set_precision(mode == VX3_FMA);
}

size_t vx3_bytes_in_use(vx3_ctx* c) { return c ? c->eng->bytes_in_use() : 0; }

static int inspect_world(const char* base, const char* vxd, gvx::SimWorld* w, std::string* err) {
    if (!base) { *err = "null VXA"; return VX3_E_ARG; }
    gvx::SimDesc d;
    if (!gvx::parse_vxa(base, vxd, &d, err)) return VX3_E_PARSE;
    if (!gvx::build_world(d, w, err)) return VX3_E_PARSE;
    return VX3_OK;
}

int vx3_inspect_vxa(const char* base, const char* vxd, int32_t* counts, double* env, char* errbuf, int err_len) {
    gvx::SimWorld w;
    std::string err;
    int e = inspect_world(base, vxd, &w, &err);
    if (e) {
        if (errbuf && err_len > 0) { strncpy(errbuf, err.c_str(), (size_t)err_len - 1); errbuf[err_len - 1] = 0; }
        return e;
    }
    if (counts) {
        counts[0] = w.nv; counts[1] = w.nl; counts[2] = (int32_t)w.vmats.size(); counts[3] = (int32_t)w.loaded_lmats;
        counts[4] = w.surface_count; counts[5] = (int32_t)w.desc.externals.size();
    }
    if (env) {
        const gvx::SimDesc& d = w.desc;
        double v[12] = {d.vox_size, d.dt_frac, d.gravity_mult, (double)d.floor, (double)d.collisions, (double)d.vary_temp,
                        d.temp_amplitude, d.temp_period, (double)d.enable_expansion, d.initial_temp, d.bounding_radius, d.watch_distance};
        memcpy(env, v, sizeof(v));
    }
    return VX3_OK;
}

int vx3_inspect_topology(const char* base, const char* vxd, int32_t* vox4, int32_t* lnk4, double* phase, float* vmat18, double* vnom,
                         int32_t* lidx2, float* lmat20) {
    gvx::SimWorld w;
    std::string err;
    if (int e = inspect_world(base, vxd, &w, &err)) return e;
    for (int i = 0; i < w.nv; i++) {
        if (vox4) for (int k = 0; k < 4; k++) vox4[4 * i + k] = w.desc.voxels[4 * i + k];
        if (phase) phase[i] = w.desc.phase.empty() ? 0.0 : w.desc.phase[i];
    }
    for (int i = 0; i < w.nl; i++)
        if (lnk4) { lnk4[4 * i] = w.link_neg[i]; lnk4[4 * i + 1] = w.link_pos[i]; lnk4[4 * i + 2] = w.link_axis[i]; lnk4[4 * i + 3] = w.link_mat[i]; }
    for (size_t k = 0; k < w.vmats.size(); k++) {
        const gvx::VoxelMaterial& m = w.vmats[k];
        float v[18] = {m.E, m.nu, m.rho, m.cte, m.mus, m.muk, m.zi, m.zg, m.zc, m.eHat, m.mass, m.massInv, m.sqrtMass, m.I, m.Iinv, m.c2m, m.c2i, m.grav};
        if (vmat18) memcpy(vmat18 + 18 * k, v, sizeof(v));
        if (vnom) vnom[k] = m.nom;
    }
    for (size_t k = 0; k < (size_t)w.loaded_lmats; k++) {
        const gvx::LinkMaterial& m = w.lmats[k];
        if (lidx2) { lidx2[2 * k] = m.vox1; lidx2[2 * k + 1] = m.vox2; }
        float v[20] = {m.E, m.nu, m.eHat, m.a1, m.a2, m.b1, m.b2, m.b3, m.sqA1, m.sqA2xIp, m.sqB1, m.sqB2xFMp, m.sqB3xIp,
                       m.sigmaYield, m.sigmaFail, m.epsYield, m.epsFail, m.linear ? 1.0f : 0.0f, (float)m.nom, m.rho};
        if (lmat20) memcpy(lmat20 + 20 * k, v, sizeof(v));
    }
    return VX3_OK;
}

int vx3_inspect_externals(const char* base, const char* vxd, int32_t* dof, float* fm6, double* tr6) {
    gvx::SimWorld w;
    std::string err;
    if (int e = inspect_world(base, vxd, &w, &err)) return e;
    for (int i = 0; i < w.nv; i++) {
        if (dof) dof[i] = 0;
        for (int k = 0; k < 6; k++) {
            if (fm6) fm6[6 * i + k] = 0.0f;
            if (tr6) tr6[6 * i + k] = 0.0;
        }
    }
    for (const gvx::External& x : w.desc.externals) {
        const int i = x.voxel;
        if (dof) dof[i] = x.dof_fixed;
        for (int k = 0; k < 3; k++) {
            if (fm6) { fm6[6 * i + k] = x.force[k]; fm6[6 * i + 3 + k] = x.moment[k]; }
            if (tr6) { tr6[6 * i + k] = x.translate[k]; tr6[6 * i + 3 + k] = x.rotate[k]; }
        }
    }
    return VX3_OK;
}

int vx3_eval_formula(vx3_ctx* c, const char* base, const char* vxd, int which, const double* vars9, int n, double* out) {
    if (!c || !base || (n > 0 && (!vars9 || !out)) || n < 0 || which < 0 || which > 4) return VX3_E_ARG;
    gvx::SimDesc d;
    std::string err;
    if (!gvx::parse_vxa(base, vxd, &d, &err)) return fail(c, VX3_E_PARSE, err);
    const gvx::MathTree& m = which == 0 ? d.stop_formula : which == 1 ? d.fitness : d.force_field[which - 2];
    int e = c->eng->eval_formula(m, vars9, n, out, &err);
    return e ? fail(c, e, err) : VX3_OK;
}

int vx3_inspect_formula(const char* base, const char* vxd, int which, const double* vars, double* out) {
    if (!base || !vars || !out) return VX3_E_ARG;
    gvx::SimDesc d;
    std::string err;
    if (!gvx::parse_vxa(base, vxd, &d, &err)) return VX3_E_PARSE;
    const gvx::MathTree& m = which == 0 ? d.stop_formula : d.fitness;
    gvx::MathVars mv{vars[0], vars[1], vars[2], vars[3], vars[4], vars[5], vars[6], (int)vars[7], (int)vars[8]};
    *out = gvx::mathtree_eval(m, mv);
    return VX3_OK;
}

}  // extern "C"
