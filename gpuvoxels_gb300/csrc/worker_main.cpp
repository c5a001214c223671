// vx3_node_worker: the reference worker's process contract over the GB300 engine.
//
//     vx3_node_worker -i <job.vxt> -o <report.vxr> [-f]
//
// Same flags, input and output as Voxelyze3/src/Executables/vx3_node_worker.cu:32-141:
// the .vxt names the base VXA (<vxa>), the directory of the VXD files (<input_dir>) and
// the VXD file names (children of <vxd>); the files are dealt round-robin to the GPUs
// (:88-93), each GPU runs its share as one batch through the C ABI, and one report is
// written with the worker's keys.  Exit status 1 on a usage error, a missing input, an
// existing output without -f, or no GPU, as the reference does.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include "../../include/gpuvoxels_gb300.h"
#include "xml_dom.h"

namespace {

const char* kUsage =
    "vx3_node_worker: runs a generation of VXD files against a base VXA on every GPU and writes a report.\n"
    "Usage:\n  vx3_node_worker -i <job.vxt> -o <report.vxr> [-f]\n"
    "Allowed options:\n"
    "  -h [ --help ]          produce help message\n"
    "  -i [ --input ] arg     Set input .vxt file (base vxa, input_dir and the vxd file list).\n"
    "  -o [ --output ] arg    Set output file path for report. (e.g. report_1.xml)\n"
    "  -f [ --force ]         Overwrite output file if exists.\n";

bool is_file(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

bool slurp(const std::string& p, std::string* out) {
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    *out = ss.str();
    return true;
}

std::string join(const std::string& dir, const std::string& file) {
    if (dir.empty() || (!file.empty() && file[0] == '/')) return file;
    return dir.back() == '/' ? dir + file : dir + "/" + file;
}

std::string base_name(const std::string& p) {
    size_t s = p.find_last_of('/');
    return s == std::string::npos ? p : p.substr(s + 1);
}

struct DeviceJob {
    int device = 0;
    std::vector<std::string> files;
    vx3_ctx* ctx = nullptr;
    std::vector<vx3_sim_id> ids;
    int rc = 0;
};

void run_device(DeviceJob* job, const std::string* base_xml, const std::string* input_dir) {
    job->ctx = vx3_create(job->device, 0);
    if (!job->ctx) { job->rc = VX3_E_CUDA; return; }
    std::vector<std::string> texts, names;
    for (const std::string& f : job->files) {
        std::string vxd;
        if (!slurp(join(*input_dir, f), &vxd)) {
            fprintf(stderr, "%s: cannot read\n", f.c_str());
            continue;
        }
        texts.push_back(std::move(vxd));
        names.push_back(base_name(f));
    }
    std::vector<const char*> tp, np;
    for (size_t i = 0; i < texts.size(); i++) { tp.push_back(texts[i].c_str()); np.push_back(names[i].c_str()); }
    std::vector<vx3_sim_id> ids(texts.size());
    std::vector<int> st(texts.size());
    vx3_load_vxa_many(job->ctx, base_xml->c_str(), tp.data(), np.data(), (int)texts.size(), ids.data(), st.data());
    for (size_t i = 0; i < ids.size(); i++) {
        if (st[i] != VX3_OK) fprintf(stderr, "%s: rejected (error %d)\n", names[i].c_str(), st[i]);
        else job->ids.push_back(ids[i]);
    }
    if (!job->ids.empty()) {
        job->rc = vx3_run(job->ctx, job->ids.data(), (int)job->ids.size(), VX3_BATCHED, 0);
        if (job->rc) fprintf(stderr, "device %d: %s\n", job->device, vx3_last_error(job->ctx));
    }
}

}  // namespace

int main(int argc, char** argv) {
    std::string input, output;
    bool force = false, help = false;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto value = [&](const char* shortf, const char* longf, std::string* dst) {
            const std::string lf = std::string(longf) + "=";
            if (a == shortf || a == longf) {
                if (i + 1 < argc) *dst = argv[++i];
                return true;
            }
            if (a.compare(0, lf.size(), lf) == 0) { *dst = a.substr(lf.size()); return true; }
            if (a.size() > 2 && a.compare(0, 2, shortf) == 0) { *dst = a.substr(2); return true; }
            return false;
        };
        if (a == "-h" || a == "--help") help = true;
        else if (a == "-f" || a == "--force") force = true;
        else if (value("-i", "--input", &input) || value("-o", "--output", &output)) {}
        else { fprintf(stderr, "unrecognised option '%s'\n", a.c_str()); help = true; }
    }
    if (help || input.empty() || output.empty()) {
        printf("%s\n", kUsage);
        return 1;
    }
    if (is_file(output) && !force) {
        printf("Error: output file exists.\n\n%s\n", kUsage);
        return 1;
    }
    if (!is_file(input)) {
        printf("Error: input file not found.\n\n%s\n", kUsage);
        return 1;
    }
    std::string vxt_text, err;
    slurp(input, &vxt_text);
    // Boost's write_xml emits the .vxt's elements side by side at top level (no single root):
    // drop the declaration and parse them inside one wrapper element.
    if (vxt_text.compare(0, 5, "<?xml") == 0) {
        const size_t e = vxt_text.find("?>");
        vxt_text = e == std::string::npos ? std::string() : vxt_text.substr(e + 2);
    }
    std::unique_ptr<gvx::XmlNode> vxt = gvx::xml_parse("<vxt>" + vxt_text + "</vxt>", &err);
    if (!vxt) {
        fprintf(stderr, "%s: %s\n", input.c_str(), err.c_str());
        return 1;
    }
    // a file that already has one wrapper element around <vxa>, <input_dir> and <vxd> is accepted too
    const gvx::XmlNode* root = vxt.get();
    if (!root->child("vxa") && root->children.size() == 1) root = root->children[0].get();
    const gvx::XmlNode* n_vxa = root->child("vxa");
    const gvx::XmlNode* n_dir = root->child("input_dir");
    const gvx::XmlNode* n_vxd = root->child("vxd");
    if (!n_vxa || !n_dir) {
        fprintf(stderr, "%s: needs <vxa> and <input_dir>\n", input.c_str());
        return 1;
    }
    const std::string base_path = n_vxa->text, input_dir = n_dir->text;
    std::vector<std::string> files;
    if (n_vxd)
        for (const auto& c : n_vxd->children) files.push_back(c->text);
    std::string base_xml;
    if (!slurp(base_path, &base_xml)) {
        fprintf(stderr, "%s: cannot read base VXA\n", base_path.c_str());
        return 1;
    }

    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev <= 0) {
        printf("ERROR: No GPU found.\n");
        return 1;
    }
    printf("%d GPU found.\n", n_dev);

    std::vector<DeviceJob> jobs((size_t)n_dev);
    for (int d = 0; d < n_dev; d++) jobs[d].device = d;
    for (size_t i = 0; i < files.size(); i++) jobs[i % n_dev].files.push_back(files[i]);
    std::vector<std::thread> threads;
    for (auto& j : jobs)
        if (!j.files.empty()) threads.emplace_back(run_device, &j, &base_xml, &input_dir);
    for (auto& t : threads) t.join();

    std::vector<vx3_ctx*> ctxs;
    std::vector<const vx3_sim_id*> idp;
    std::vector<int> counts;
    int rc = 0;
    for (auto& j : jobs) {
        if (!j.ctx) continue;
        if (j.rc) rc = 1;
        ctxs.push_back(j.ctx);
        idp.push_back(j.ids.data());
        counts.push_back((int)j.ids.size());
    }
    if (ctxs.empty()) {
        printf("ERROR: no simulation ran.\n");
        return 1;
    }
    if (vx3_write_report_multi(ctxs.data(), idp.data(), counts.data(), (int)ctxs.size(), input_dir.c_str(), output.c_str()) != VX3_OK) {
        fprintf(stderr, "report: %s\n", vx3_last_error(ctxs[0]));
        rc = 1;
    }
    for (vx3_ctx* c : ctxs) vx3_destroy(c);
    return rc;
}
