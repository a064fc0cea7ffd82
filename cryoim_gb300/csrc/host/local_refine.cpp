// local_refine — drop-in for the reference's `local_refine` (its refine_PR path):
// `local_refine local_ort0=... local_newort=... model3d=... key=value ...`.
//
// The 22 keys of local_refine/SRC/0input_parameters.f90:5-26 with the code's defaults
// (apix 1, maxRes 10, minRes 200, Ncycle 12, convF 0.8, vol 200, Cs 2.7, ampwg 0.1,
// applyCTF y, sym c1, first 1, refine_angle / refine_shift derived from maxRes).  The
// local map (model3d) fixes FFTsize, the whole-particle stacks (or imgstck) FFTsize0.
// Reads the 23-column local orientation file (load_original_ort.f90), refines every
// sub-particle on the GPU and writes the 28-column rows of refine_PR.f90:236-253.
// Not on this path: particle_df=y / Zhigh_df=y (refine_particle_df.f90,
// refine_PR_Zhigh.f90) and sym other than cN (asym, c180, c360, i2, i5): the run stops
// with a message.  Extension keys: device, batch (sub-particles per device call).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "cryoim.h"

namespace {

const char* kKeys[] = {"local_ort0", "local_newort", "model3d", "imgstck", "minRes", "apix", "first", "last",
                       "imgmask", "applyCTF", "Ncycle", "vol", "Cs", "refine_angle", "refine_shift", "maxRes",
                       "convF", "particle_df", "Zhigh_df", "sym", "sign", "ampwg"};
const char* kExt[] = {"device", "batch"};

void usage() {
    std::puts("local_refine (cryoim_gb300): refinement of sub-particles against a local map on a GB300 GPU\n"
              "usage: local_refine local_ort0=<ort> local_newort=<out> model3d=<map> [apix= maxRes= imgmask= "
              "applyCTF= Ncycle= convF= refine_angle= refine_shift= sym=cN vol= Cs= ampwg= first= last= imgstck=]\n"
              "  GPU extensions: device batch");
}

std::string first_token(const std::string& v) {
    size_t a = v.find_first_not_of(" \t'\"");
    if (a == std::string::npos) return "";
    size_t b = v.find_first_of(" \t,'\"", a);
    return v.substr(a, b == std::string::npos ? std::string::npos : b - a);
}

bool yes(const std::string& v) { return !v.empty() && (v[0] == 'y' || v[0] == 'Y'); }

int die(const char* what) {
    std::fprintf(stderr, "local_refine: %s (%s)\n", what, cryoim_last_error());
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc - 1 < 3) { usage(); return 0; }
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        size_t e = a.find('=');
        std::string k = e == std::string::npos ? a : a.substr(0, e);
        bool known = false;
        for (const char* x : kKeys) known |= (k == x);
        for (const char* x : kExt) known |= (k == x);
        if (!known || e == std::string::npos) { usage(); return 0; }
        kv[k] = first_token(a.substr(e + 1));
    }
    auto has = [&](const char* k) { return kv.count(k) > 0; };
    auto sval = [&](const char* k, const char* d) { return has(k) ? kv[k] : std::string(d); };
    auto fval = [&](const char* k, float d) { return has(k) ? (float)std::atof(kv[k].c_str()) : d; };
    auto ival = [&](const char* k, int d) { return has(k) ? std::atoi(kv[k].c_str()) : d; };
    if (yes(sval("particle_df", "n")) || yes(sval("Zhigh_df", "n")))
        return die("particle_df / Zhigh_df refinement is not on this path");
    const std::string sym = sval("sym", "c1");
    if (sym.size() < 2 || (sym[0] != 'c' && sym[0] != 'C') || std::atoi(sym.c_str() + 1) < 1 ||
        std::atoi(sym.c_str() + 1) > 60)
        return die("only sym=cN (N <= 60) is on this path");
    const std::string ort = sval("local_ort0", ""), out = sval("local_newort", ""), model = sval("model3d", "");
    if (ort.empty() || out.empty() || model.empty()) { usage(); return 0; }
    // 0calc_initialvalue.f90:9-52
    cryoim_mrc_header mh;
    if (cryoim_mrc_read_header(model.c_str(), &mh)) return die("cannot read model3d");
    const int nx = mh.nx;
    int32_t rows = 0;
    if (cryoim_ort_count(ort.c_str(), &rows) || rows < 1) return die("cannot read local_ort0");
    std::vector<cryoim_local_particle> all(rows);
    std::vector<char> names((size_t)rows * 256);
    if (cryoim_local_ort_read(ort.c_str(), 1, rows, all.data(), names.data(), 256)) return die("malformed local_ort0");
    const std::string imgstck = sval("imgstck", "");
    cryoim_mrc_header ih;
    if (cryoim_mrc_read_header(imgstck.empty() ? &names[0] : imgstck.c_str(), &ih)) return die("cannot read a stack");
    const int nx0 = ih.nx;
    const int first = ival("first", 1);
    int last = ival("last", rows);
    if (last > rows) last = rows;
    if (first < 1 || last < first) return die("first/last out of range");
    cryoim_local_params p;
    if (cryoim_local_params_default(&p, nx, nx0)) return die("box sizes");
    p.nsym = std::atoi(sym.c_str() + 1);
    p.apix = fval("apix", 1.0f);
    p.max_res = fval("maxRes", 10.0f);
    p.imgmask = has("imgmask") ? fval("imgmask", 0.0f) : 0.0f;
    p.apply_ctf = yes(sval("applyCTF", "y"));
    p.ncycle = ival("Ncycle", 12);
    p.vol = fval("vol", 200.0f);
    p.cs = fval("Cs", 2.7f);
    p.ampwg = fval("ampwg", 0.1f);
    p.convf = fval("convF", 0.8f);
    p.refine_angle = has("refine_angle") ? fval("refine_angle", 1.0f) : 0.0f;
    p.refine_shift = has("refine_shift") ? fval("refine_shift", 1.0f) : 0.0f;
    p.normalize = imgstck.empty() ? 1 : 0;  // refine_PR.f90:73-88: only stack-file images are normalised
    if (cryoim_local_params_derive(&p)) return die("parameters");
    std::printf(" FFTsize0,FFTsize,maxRes,Ncycle,convF,refine_angle,refine_shift:\n %d %d %f %d %f %f %f\n", nx0, nx,
                p.max_r, p.ncycle, p.convf, p.refine_angle, p.refine_shift);
    std::vector<float> map((size_t)nx * nx * nx);
    if (cryoim_mrc_read_sections(model.c_str(), 1, nx, map.data())) return die("model3d data");
    void* ctx = nullptr;
    if (cryoim_ctx_create(ival("device", 0), &ctx)) return die("device");
    const int chunk = std::max(1, ival("batch", 512));
    const size_t nn0 = (size_t)nx0 * nx0;
    std::FILE* trunc = std::fopen(out.c_str(), "w");
    if (!trunc) return die("cannot write local_newort");
    std::fclose(trunc);
    for (int i0 = first - 1; i0 < last; i0 += chunk) {
        const int n = std::min(chunk, last - i0);
        std::vector<float> imgs((size_t)n * nn0);
        for (int i = 0; i < n; ++i) {
            const int row = i0 + i;
            int r;
            // with imgstck the reference reads the stack in sequence from its start: its
            // seek past first-1 images goes to another unit (refine_PR.f90:59-64)
            if (!imgstck.empty()) r = cryoim_mrc_read_sections(imgstck.c_str(), row - (first - 1) + 1, 1, &imgs[i * nn0]);
            else r = cryoim_mrc_read_sections(&names[(size_t)row * 256], all[row].img_particle_id, 1, &imgs[i * nn0]);
            if (r) return die("particle stack read");
        }
        if (cryoim_local_refine(ctx, &p, map.data(), imgs.data(), &all[i0], n)) return die("refinement");
        std::vector<char> nm((size_t)n * 64, 0);
        for (int i = 0; i < n; ++i) std::strncpy(&nm[(size_t)i * 64], &names[(size_t)(i0 + i) * 256], 63);
        if (cryoim_local_ort_write(out.c_str(), &all[i0], nm.data(), 64, n, 28, 1)) return die("cannot write local_newort");
    }
    cryoim_ctx_destroy(ctx);
    return 0;
}
