// local_box — drop-in for the reference's `local_box`:
//   `local_box icos_ort=... local_ort=... local_x= local_y= local_z= ...` (coordinate
//   mode, loc_box_coordinate.f90) or, with local_imgstck=<out.mrc>, the sub-image stack
//   mode (loc_box.f90) on the GPU.
//
// The keys of local_box/SRC/0input_parameters.f90:5-34 with the code's defaults (first 1,
// apix 1, PR_threshold 90, sub_FFTsize 256, sym i2, boundX 100).  Reads the
// whole-particle orientation file (13 list-directed columns, load_ort.f90), takes
// FFTsize from the first particle's stack.  Coordinate mode: one 23-column row (format
// 900 of loc_box_coordinate.f90:46) per selected particle and symmetry rotation.  Stack
// mode: the whole images come from icos_imgstck (images first..last in order) or from
// each particle's own stack (imgparticleID); the sub-images go to local_imgstck behind
// the header of local_maphead.f90 with nz = Nsym x (rows of icos_ort), as
// loc_box.f90:29 writes it, and one 14-column row (format 900 of loc_box.f90:93) per
// sub-image to local_ort.  sym: cN, i2, i3, i5, or sym_matrix=<file> (3 rows of 3 per
// rotation, each row one column of the matrix, read_sym_matrix.f90).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "cryoim.h"

namespace {

const char* kKeys[] = {"icos_ort", "local_ort", "local_imgstck", "local_x", "local_y", "local_z",
                       "apix",     "PR_threshold", "sub_FFTsize", "icos_imgstck", "Nsym", "sym_matrix",
                       "sym",      "first",     "last",          "boundX"};

void usage() {
    std::puts("local_box (cryoim_gb300): sub-particle coordinates for localized reconstruction\n"
              "usage: local_box icos_ort=<ort> local_ort=<out> local_x= local_y= local_z= [apix= sym=cN|i2|i3|i5 "
              "sym_matrix=<file> PR_threshold= boundX= first= last=]\n"
              "       with local_imgstck=<out.mrc> [sub_FFTsize= icos_imgstck=<stack>]: the sub-image stack");
}

std::string first_token(const std::string& v) {
    size_t a = v.find_first_not_of(" \t'\"");
    if (a == std::string::npos) return "";
    size_t b = v.find_first_of(" \t,'\"", a);
    return v.substr(a, b == std::string::npos ? std::string::npos : b - a);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc - 1 < 4) { usage(); return 0; }
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        size_t e = a.find('=');
        std::string k = e == std::string::npos ? a : a.substr(0, e);
        bool known = false;
        for (const char* x : kKeys) known |= (k == x);
        if (!known || e == std::string::npos) { usage(); return 0; }
        kv[k] = first_token(a.substr(e + 1));
    }
    auto has = [&](const char* k) { return kv.count(k) > 0; };
    auto sval = [&](const char* k, const char* d) { return has(k) ? kv[k] : std::string(d); };
    auto fval = [&](const char* k, float d) { return has(k) ? (float)std::atof(kv[k].c_str()) : d; };
    const std::string ort = sval("icos_ort", ""), out = sval("local_ort", "");
    if (ort.empty() || out.empty()) { usage(); return 0; }
    int32_t rows = 0;
    if (cryoim_ort_count(ort.c_str(), &rows) || rows < 1) { std::fprintf(stderr, "cannot read %s\n", ort.c_str()); return 2; }
    const int first = has("first") ? std::atoi(kv["first"].c_str()) : 1;
    int last = has("last") ? std::atoi(kv["last"].c_str()) : rows;
    if (last > rows) { std::puts(" last should smaller than totalparticle"); return 1; }  // load_ort.f90:21-24
    std::vector<cryoim_particle> parts(rows);
    std::vector<char> names((size_t)rows * 256);
    if (cryoim_ort_read(ort.c_str(), 1, rows, parts.data(), names.data(), 256)) {
        std::fprintf(stderr, "malformed %s\n", ort.c_str());
        return 2;
    }
    cryoim_mrc_header h;  // load_ort.f90:37-40: FFTsize from the first particle's stack
    if (cryoim_mrc_read_header(&names[0], &h)) { std::fprintf(stderr, "cannot read %s\n", &names[0]); return 2; }
    std::vector<float> sym(9 * 4096);
    int32_t nsym = 0;
    if (has("sym_matrix")) {
        std::FILE* f = std::fopen(kv["sym_matrix"].c_str(), "r");
        if (!f) { std::fprintf(stderr, "cannot read %s\n", kv["sym_matrix"].c_str()); return 2; }
        float a, b, c;
        int line = 0;
        while (nsym < 4096 && std::fscanf(f, "%f %f %f", &a, &b, &c) == 3) {
            const int col = line % 3;
            float* m = &sym[9 * (size_t)nsym];
            m[col] = a; m[3 + col] = b; m[6 + col] = c;
            if (++line % 3 == 0) ++nsym;
        }
        std::fclose(f);
    } else if (cryoim_local_sym_matrices(sval("sym", "i2").c_str(), sym.data(), &nsym)) {
        std::fprintf(stderr, "local_box: sym=%s is not on this path (cN, i2, i3, i5 or sym_matrix)\n",
                     sval("sym", "i2").c_str());
        return 2;
    }
    const int P = last - first + 1;
    if (has("local_imgstck")) {
        // loc_box.f90:14-27: whole images of particles first..last
        const int nx0 = h.nx, sub = has("sub_FFTsize") ? std::atoi(kv["sub_FFTsize"].c_str()) : 256;
        const size_t nn0 = (size_t)nx0 * nx0, ns = (size_t)sub * sub;
        std::vector<float> imgs((size_t)P * nn0);
        for (int i = 0; i < P; ++i) {
            const int r = has("icos_imgstck")
                              ? cryoim_mrc_read_sections(kv["icos_imgstck"].c_str(), first + i, 1, &imgs[i * nn0])
                              : cryoim_mrc_read_sections(&names[(size_t)(first - 1 + i) * 256],
                                                         parts[first - 1 + i].img_particle_id, 1, &imgs[i * nn0]);
            if (r) { std::fprintf(stderr, "cannot read the image of particle %d\n", first + i); return 2; }
        }
        void* ctx = nullptr;
        if (cryoim_ctx_create(0, &ctx)) { std::fprintf(stderr, "local_box: %s\n", cryoim_last_error()); return 2; }
        std::vector<float> subs((size_t)P * nsym * ns);
        std::vector<cryoim_local_particle> rec((size_t)P * nsym);
        int32_t nout = 0;
        const int rc = cryoim_local_box_extract(ctx, imgs.data(), &parts[first - 1], P, nx0, sym.data(), nsym,
                                                fval("local_x", 0.f), fval("local_y", 0.f), fval("local_z", 0.f),
                                                fval("apix", 1.0f), sub, fval("PR_threshold", 90.0f),
                                                fval("boundX", 100.0f), subs.data(), rec.data(), &nout);
        cryoim_ctx_destroy(ctx);
        if (rc) { std::fprintf(stderr, "local_box: %s\n", cryoim_last_error()); return 2; }
        cryoim_mrc_header mh;
        cryoim_map_header(&mh, sub, sub, sub, fval("apix", 1.0f));  // local_maphead.f90
        mh.nz = nsym * rows;
        if (cryoim_mrc_write(kv["local_imgstck"].c_str(), &mh, subs.data(), (int64_t)nout * (int64_t)ns)) {
            std::fprintf(stderr, "cannot write %s\n", kv["local_imgstck"].c_str());
            return 2;
        }
        // each record's stack name: records come nsym per selected particle, in order
        std::vector<int> sel;
        for (int i = first - 1; i < last; ++i) {
            const cryoim_particle& q = parts[i];
            if (q.pr <= fval("PR_threshold", 90.0f) && std::fabs(q.x) <= fval("boundX", 100.0f) &&
                std::fabs(q.y) <= fval("boundX", 100.0f))
                sel.push_back(i);
        }
        std::vector<char> lnames((size_t)nout * 64, 0);
        for (int k = 0; k < nout && k / nsym < (int)sel.size(); ++k)
            std::strncpy(&lnames[(size_t)k * 64], &names[(size_t)sel[k / nsym] * 256], 63);
        if (cryoim_local_ort_write(out.c_str(), rec.data(), lnames.data(), 64, nout, 14, 0)) {
            std::fprintf(stderr, "cannot write %s\n", out.c_str());
            return 2;
        }
        return 0;
    }
    std::vector<cryoim_local_particle> loc((size_t)P * nsym);
    int32_t nout = 0;
    if (cryoim_local_box_coordinates(&parts[first - 1], P, sym.data(), nsym, fval("local_x", 0.f), fval("local_y", 0.f),
                                     fval("local_z", 0.f), fval("apix", 1.0f), h.nx, fval("PR_threshold", 90.0f),
                                     fval("boundX", 100.0f), loc.data(), &nout)) {
        std::fprintf(stderr, "local_box: %s\n", cryoim_last_error());
        return 2;
    }
    // each output row carries its particle's stack name: the records come nsym per
    // selected particle, in particle order (the selection of load_ort.f90:30-34)
    std::vector<char> lnames((size_t)nout * 64, 0);
    const float prt = fval("PR_threshold", 90.0f), bx = fval("boundX", 100.0f);
    for (int i = first - 1, k = 0; i < last && k < nout; ++i) {
        const cryoim_particle& q = parts[i];
        if (!(q.pr <= prt && std::fabs(q.x) <= bx && std::fabs(q.y) <= bx)) continue;
        for (int s = 0; s < nsym && k < nout; ++s, ++k) std::strncpy(&lnames[(size_t)k * 64], &names[(size_t)i * 256], 63);
    }
    if (cryoim_local_ort_write(out.c_str(), loc.data(), lnames.data(), 64, nout, 23, 0)) {
        std::fprintf(stderr, "cannot write %s\n", out.c_str());
        return 2;
    }
    return 0;
}
