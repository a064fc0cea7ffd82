// merge_icosprocess_subrec — drop-in for the reference's merge of partial
// reconstructions: `merge_icosprocess_subrec part_1 ... part_n map.mrc`.
//
// main.f90:16-28: the header of part_1//'oddtnf' (else part_1) decides the mode.
//   * flag FSC = 0 (merge_reconstruct.f90): sum the tnf partials part_i, fold with an
//     integer radius, invert, icosahedral average when the avg flag is set, and write
//     the central (nx-8)^3 voxels taken with that routine's index (lz = i/(nx-8)^2 + 4
//     instead of (i-1)/(nx-8)^2 + 4: the last voxel of every section comes from the
//     next section), under a header for nx-8.
//   * flag FSC = 1 (merge_reconstruct_FSC.f90): sum part_i//'oddtnf' and part_i//'evetnf',
//     FSC.txt, FSC weighting, fold, forward-signed transform, shift, cut at imgmask; then
//     the header for nx-8 and the first (nx-8)^3 values of the nx^3 array (the routine
//     shrinks FFTsize before it writes and averages), averaged as an (nx-8)^3 box when
//     the avg flag is set.
// The merging runs through the library on the GPU.  Extension key: device=<n> may appear
// anywhere in the argument list.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cryoim.h"

namespace {

bool exists(const std::string& p) {
    std::FILE* f = std::fopen(p.c_str(), "rb");
    if (f) std::fclose(f);
    return f != nullptr;
}

int die(const char* what) {
    std::fprintf(stderr, "merge_icosprocess_subrec: %s (%s)\n", what, cryoim_last_error());
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    std::vector<std::string> files;
    int device = 0;
    for (int i = 1; i < argc; ++i) {
        if (!std::strncmp(argv[i], "device=", 7)) device = std::atoi(argv[i] + 7);
        else files.push_back(argv[i]);
    }
    if (files.size() < 2) {
        std::puts("usage: merge_icosprocess_subrec part_1 [part_2 ...] map.mrc [device=0]\n"
                  "  parts are tnf partials (subrec=y), or the result3d prefixes of FSC=y subrec=y\n"
                  "  runs (prefix//'oddtnf', prefix//'evetnf')");
        return 0;
    }
    const std::string first = exists(files[0] + "oddtnf") ? files[0] + "oddtnf" : files[0];
    int32_t ih[4];
    float fh[2];
    if (cryoim_tnf_read(first.c_str(), ih, fh, nullptr, nullptr, nullptr)) {
        std::fprintf(stderr, "cannot read %s\n", first.c_str());
        return 2;
    }
    const int nx = ih[0], R = ih[1], with_fsc = ih[2] == 1, avg = ih[3] == 1;
    std::printf("%12d%12d%14.7f%14.7f%12d%12d\n", nx, R, fh[0], fh[1], ih[2], ih[3]);
    cryoim_params p;
    if (cryoim_params_default(&p, nx)) return 2;
    p.apix = fh[0];
    cryoim_params_derive(&p);
    p.max_r = R;  // the partials fix the band
    p.min_r = 0;
    p.imgmask_px = fh[1];
    p.realspaceavg = 0;
    void* ctx = nullptr;
    if (cryoim_ctx_create(device, &ctx) || cryoim_set_params(ctx, &p)) return die("device");
    const size_t n = (size_t)(2 * R + 1) * (2 * R + 1) * (R + 1);
    const size_t n3 = (size_t)nx * nx * nx;
    const int m = nx - 8;
    const size_t m3 = (size_t)m * m * m;
    std::vector<float> map(n3), out(m3);
    auto read_part = [&](const std::string& f, std::vector<float>* acc) {
        int32_t h2[4];
        float f2[2];
        std::vector<float> a(n), b(n), w(n);
        if (cryoim_tnf_read(f.c_str(), h2, f2, a.data(), b.data(), w.data()) || h2[0] != nx || h2[1] != R) {
            std::fprintf(stderr, "cannot read %s or its box differs\n", f.c_str());
            return false;
        }
        for (size_t i = 0; i < n; ++i) { acc[0][i] += a[i]; acc[1][i] += b[i]; acc[2][i] += w[i]; }
        return true;
    };
    if (!with_fsc) {
        if (cryoim_rec_begin(ctx)) return die("reconstruction");
        std::vector<float> part[3] = {std::vector<float>(n), std::vector<float>(n), std::vector<float>(n)};
        for (size_t i = 0; i + 1 < files.size(); ++i) {
            std::printf(" reading data form %s\n", files[i].c_str());
            for (auto& v : part) std::fill(v.begin(), v.end(), 0.0f);
            if (!read_part(files[i], part)) return 2;
            if (cryoim_rec_add_partial(ctx, part[0].data(), part[1].data(), part[2].data())) return die("partial");
        }
        if (cryoim_rec_finish_merge(ctx, map.data())) return die("merge");
        if (avg && cryoim_icosavg(ctx, map.data(), nx, fh[1])) return die("icosavg");
        // merge_reconstruct.f90:144-150
        for (size_t i = 1; i <= m3; ++i) {
            const size_t lz = i / ((size_t)m * m) + 4, ky = ((i - 1) % ((size_t)m * m)) / m + 4,
                         hx = ((i - 1) % ((size_t)m * m)) % m + 4;
            out[i - 1] = map[(lz * nx + ky) * nx + hx];
        }
    } else {
        std::vector<float> odd[3], eve[3];
        for (int k = 0; k < 3; ++k) { odd[k].assign(n, 0.0f); eve[k].assign(n, 0.0f); }
        for (size_t i = 0; i + 1 < files.size(); ++i)
            if (!read_part(files[i] + "oddtnf", odd) || !read_part(files[i] + "evetnf", eve)) return 2;
        std::vector<float> fsc(R + 1);
        if (cryoim_merge_fsc_combine(ctx, odd[0].data(), odd[1].data(), odd[2].data(), eve[0].data(),
                                     eve[1].data(), eve[2].data(), fsc.data(), map.data()))
            return die("FSC merge");
        std::FILE* f = std::fopen("FSC.txt", "w");  // merge_reconstruct_FSC.f90:8, 63
        if (!f) return die("cannot write FSC.txt");
        for (int ir = 0; ir <= R; ++ir) {
            const float F = fsc[ir], w = std::sqrt(2.0f * F / (1.0f + F));
            std::fprintf(f, "%12d %15.7f ", ir, F);
            if (w == w) std::fprintf(f, "%15.7f\n", w);
            else std::fprintf(f, "%15s\n", "NaN");
        }
        std::fclose(f);
        std::memcpy(out.data(), map.data(), sizeof(float) * m3);
        if (avg && cryoim_icosavg(ctx, out.data(), m, fh[1])) return die("icosavg");
    }
    cryoim_mrc_header h;
    cryoim_map_header(&h, m, m, m, p.apix);
    if (cryoim_mrc_write(files.back().c_str(), &h, out.data(), (int64_t)out.size())) return die("cannot write map");
    cryoim_ctx_destroy(ctx);
    return 0;
}
