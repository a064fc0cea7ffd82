// merge_icosprocess_subrec — drop-in for the reference's merge of partial
// reconstructions: `merge_icosprocess_subrec part_1.tnf ... part_n.tnf map.mrc`.
// Sums the tnf half boxes (merge_reconstruct.f90:20-34), then folds, divides by the
// CTF^2 weights, inverse-transforms and writes the map (merge_reconstruct.f90:37-159),
// through the library's reconstruction finish on the GPU.  Extension key: device=<n>
// may appear anywhere in the argument list.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cryoim.h"

int main(int argc, char** argv) {
    std::vector<std::string> files;
    int device = 0;
    for (int i = 1; i < argc; ++i) {
        if (!std::strncmp(argv[i], "device=", 7)) device = std::atoi(argv[i] + 7);
        else files.push_back(argv[i]);
    }
    if (files.size() < 2) {
        std::puts("usage: merge_icosprocess_subrec part_1.tnf [part_2.tnf ...] map.mrc [device=0]");
        return 0;
    }
    int32_t ih[4];
    float fh[2];
    if (cryoim_tnf_read(files[0].c_str(), ih, fh, nullptr, nullptr, nullptr)) {
        std::fprintf(stderr, "cannot read %s\n", files[0].c_str());
        return 2;
    }
    const int nx = ih[0], R = ih[1];
    cryoim_params p;
    if (cryoim_params_default(&p, nx)) return 2;
    p.apix = fh[0];
    cryoim_params_derive(&p);
    p.max_r = R;  // the partials fix the band
    p.min_r = 0;
    void* ctx = nullptr;
    if (cryoim_ctx_create(device, &ctx) || cryoim_set_params(ctx, &p) || cryoim_rec_begin(ctx)) {
        std::fprintf(stderr, "device: %s\n", cryoim_last_error());
        return 2;
    }
    const size_t n = (size_t)(2 * R + 1) * (2 * R + 1) * (R + 1);
    std::vector<float> fa(n), fb(n), wg(n);
    for (size_t i = 0; i + 1 < files.size(); ++i) {
        int32_t h2[4];
        float f2[2];
        std::printf(" reading data form %s\n", files[i].c_str());
        if (cryoim_tnf_read(files[i].c_str(), h2, f2, fa.data(), fb.data(), wg.data()) || h2[0] != nx ||
            h2[1] != R) {
            std::fprintf(stderr, "cannot read %s or its box differs\n", files[i].c_str());
            return 2;
        }
        if (cryoim_rec_add_partial(ctx, fa.data(), fb.data(), wg.data())) {
            std::fprintf(stderr, "%s\n", cryoim_last_error());
            return 2;
        }
    }
    std::vector<float> map((size_t)nx * nx * nx);
    if (cryoim_rec_finish(ctx, map.data())) {
        std::fprintf(stderr, "%s\n", cryoim_last_error());
        return 2;
    }
    cryoim_mrc_header h;
    cryoim_map_header(&h, nx, nx, nx, p.apix);
    if (cryoim_mrc_write(files.back().c_str(), &h, map.data(), (int64_t)map.size())) return 2;
    cryoim_ctx_destroy(ctx);
    return 0;
}
