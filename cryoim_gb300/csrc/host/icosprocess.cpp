// icosprocess — drop-in for the reference's `icosprocess` executable on the GPU path.
//
// Same `key=value` command line (the 32 keys of icosprocess/SRC/0input_parameters.f90:
// 6-37, matched exactly, unknown keys print the usage and stop), same defaults
// (0initialvalue.f90, 0calc_initialvalues.f90), same files: particle stacks and maps in
// MRC, orientation files read as 13 list-directed columns and written as the 19-column
// row of format 900, tnf partial reconstructions.  Modes:
//   0  project the model along every template orientation into templatestck
//   1  symmetrised reconstruction into result3d (map, or tnf partial with subrec=y;
//      FSC=y: gold-standard half maps, FSC.txt and the FSC-weighted map)
//   3  origin centring (calc_center.f90 / calc_center_selfrot180.f90) -> newortfile
//   4  global orientation search (ort_globesearch.f90) -> newortfile
//   5  local refinement (ort_refinement.f90) -> newortfile
// Extension keys without a reference counterpart: device, batch (particles per device
// call), contract=y (mode 4 through the tensor-core contraction), originmax,
// originstep, topk, precision=bf16|fp8 (contraction operands), nbr (rescoring
// neighbourhood in grid steps), nbrbest (rescore only the neighbourhoods of the best k
// candidates), coarse=k (coarse-contraction proposals), learned=k (proposals of the
// learned proposer: loaded from learnmodel=file if it exists, else trained on
// learnsamples projections of model3d and saved there), proposalnbr (the proposals'
// fine neighbourhood in grid steps), localrange / localstep (the local form: each
// particle's own grid around its input orientation, picked by FP64 correlation, on
// sections of the twice-oversampled transform).  Output rows are appended after
// every chunk, so a run can resume with first=k as with the reference's per-particle
// writes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "cryoim.h"

namespace {

const char* kKeys[] = {"apix",         "minRes",       "maxRes",     "imgmask",    "first",
                       "last",         "applyCTF",     "Ncycle",     "templatestck", "vol",
                       "Cs",           "Bfactor",      "ampwg",      "PR_threshold", "result3d",
                       "mode",         "newortfile",   "model3d",    "templateort", "searchstep",
                       "realspaceavg", "ortfile",      "recISAF",    "subrec",     "FSC",
                       "imgstck",      "sym",          "maxcentshift", "corrCTF",  "boundX",
                       "loc_box",      "check"};
const char* kExt[] = {"device", "batch", "contract", "originmax", "originstep", "topk", "precision", "nbr",
                      "coarse", "nbrbest", "learned", "learnmodel", "learnsamples", "localrange",
                      "localstep", "proposalnbr"};

void usage() {
    std::puts(
        "icosprocess (cryoim_gb300): icosahedral projection matching on a GB300 GPU\n"
        "usage: icosprocess mode=<0|1|3|4|5> ortfile=<ort> key=value ...\n"
        "  mode=0 project model3d along templateort into templatestck\n"
        "  mode=1 reconstruct into result3d      (PR_threshold, boundX, subrec, applyCTF;\n"
        "         FSC=y: odd/even half maps oddtnf, evetnf, FSC.txt, FSC-weighted result3d)\n"
        "  mode=3 origin centring into newortfile (against model3d, or the 180-degree self-rotation)\n"
        "  mode=4 global search into newortfile  (templateort + templatestck or model3d,\n"
        "         searchstep, minRes, maxRes, applyCTF, vol, Cs, ampwg)\n"
        "  mode=5 local refinement into newortfile (Ncycle, templateort, ...)\n"
        "  common: apix imgmask first last imgstck\n"
        "  GPU extensions: device batch contract=y originmax originstep topk precision=bf16|fp8 nbr nbrbest\n"
        "                  coarse learned learnmodel learnsamples proposalnbr localrange localstep");
}

bool yes(const std::string& v) { return !v.empty() && (v[0] == 'y' || v[0] == 'Y'); }

// list-directed read of the first value of a key
std::string first_token(const std::string& v) {
    size_t a = v.find_first_not_of(" \t'\"");
    if (a == std::string::npos) return "";
    size_t b = v.find_first_of(" \t,'\"", a);
    return v.substr(a, b == std::string::npos ? std::string::npos : b - a);
}

int die(const char* what, int code) {
    std::fprintf(stderr, "icosprocess: %s (%s)\n", what, cryoim_last_error());
    return code;
}

struct Stack {
    std::string name;
    cryoim_mrc_header h;
};

// Images of particles [i0, i0+n) from their stacks (stack name + imgparticleID).
int gather(const std::vector<cryoim_particle>& parts, const std::vector<std::string>& stck, int i0, int n,
           int nx, const std::string& imgstck, int first, std::vector<float>& out) {
    const size_t nn = (size_t)nx * nx;
    out.resize((size_t)n * nn);
    for (int i = 0; i < n; ++i) {
        int r;
        if (!imgstck.empty())  // one stack in particle order (reconstruct.f90:45-50, 63-64)
            r = cryoim_mrc_read_sections(imgstck.c_str(), first + i0 + i, 1, &out[(size_t)i * nn]);
        else
            r = cryoim_mrc_read_sections(stck[i0 + i].c_str(), parts[i0 + i].img_particle_id, 1,
                                         &out[(size_t)i * nn]);
        if (r) return r;
    }
    return CRYOIM_OK;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc - 1 < 2) { usage(); return 0; }
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        size_t e = a.find('=');
        std::string k = e == std::string::npos ? a : a.substr(0, e);
        bool known = false;
        for (const char* x : kKeys) known |= (k == x);
        for (const char* x : kExt) known |= (k == x);
        if (!known || e == std::string::npos) { usage(); return 0; }
        kv[k] = a.substr(e + 1);
    }
    auto has = [&](const char* k) { return kv.count(k) > 0; };
    auto sval = [&](const char* k, const char* d) { return has(k) ? first_token(kv[k]) : std::string(d); };
    auto fval = [&](const char* k, float d) { return has(k) ? (float)std::atof(first_token(kv[k]).c_str()) : d; };
    auto ival = [&](const char* k, int d) { return has(k) ? std::atoi(first_token(kv[k]).c_str()) : d; };
    const int mode = ival("mode", 0);
    const int device = ival("device", 0);
    void* ctx = nullptr;

    if (mode == 0) {  // 0main.f90:70-86
        if (!has("model3d")) { std::puts(" should input model3d."); return 1; }
        if (!has("templateort")) { std::puts(" should input templateort."); return 1; }
        if (!has("templatestck")) { std::puts(" should input templatestck."); return 1; }
        cryoim_mrc_header mh;
        if (cryoim_mrc_read_header(sval("model3d", "").c_str(), &mh)) return die("cannot read model3d", 2);
        const int nx = mh.nx;
        int T = 0;
        if (cryoim_template_ort_read(sval("templateort", "").c_str(), nullptr, 0, &T)) return die("templateort", 2);
        std::vector<cryoim_template> t(T);
        cryoim_template_ort_read(sval("templateort", "").c_str(), t.data(), T, &T);
        std::vector<float> map((size_t)nx * nx * nx), out((size_t)T * nx * nx);
        if (cryoim_mrc_read_sections(sval("model3d", "").c_str(), 1, nx, map.data())) return die("model3d data", 2);
        cryoim_params p;
        cryoim_params_default(&p, nx);
        p.apix = fval("apix", 1.0f);
        cryoim_params_derive(&p);
        // projection uses no Fourier band: keep the derived radii inside the box
        if (p.max_r > nx / 2 - 2) p.max_r = nx / 2 - 2;
        if (p.min_r > p.max_r) p.min_r = p.max_r;
        if (cryoim_ctx_create(device, &ctx) || cryoim_set_params(ctx, &p)) return die("device", 2);
        if (cryoim_project_templates(ctx, map.data(), t.data(), T, out.data())) return die("projection", 2);
        cryoim_mrc_header oh;
        cryoim_map_header(&oh, nx, nx, T, p.apix);
        if (cryoim_mrc_write(sval("templatestck", "").c_str(), &oh, out.data(), (int64_t)out.size()))
            return die("cannot write templatestck", 2);
        cryoim_ctx_destroy(ctx);
        return 0;
    }

    // initialvalue (0initialvalue.f90:7-45): FFTsize from the first stack, last = rows
    const std::string ortfile = sval("ortfile", "");
    const std::string imgstck = sval("imgstck", "");
    int32_t nrows = 0;
    if (ortfile.empty() || cryoim_ort_count(ortfile.c_str(), &nrows) || nrows < 1)
        return die("cannot read ortfile", 2);
    std::string stack0 = imgstck;
    if (stack0.empty()) {
        std::vector<cryoim_particle> one(1);
        std::vector<char> nm(256);
        if (cryoim_ort_read(ortfile.c_str(), 1, 1, one.data(), nm.data(), 256)) return die("ortfile row 1", 2);
        stack0 = nm.data();
    }
    cryoim_mrc_header h0;
    if (cryoim_mrc_read_header(stack0.c_str(), &h0)) return die("cannot read the first stack", 2);
    cryoim_params p;
    if (cryoim_params_default(&p, h0.nx)) return die("FFTsize", 2);
    p.mode = mode;
    p.last = nrows;
    // keys read after initialvalue (0main.f90:90-184)
    p.min_res = fval("minRes", p.min_res);
    p.max_res = fval("maxRes", p.max_res);
    if (has("imgmask")) { p.imgmask = fval("imgmask", p.imgmask); if (p.imgmask > 0) p.use_imgmask = 1; }
    if (has("applyCTF")) p.apply_ctf = yes(sval("applyCTF", "y"));
    p.apix = fval("apix", p.apix);
    p.vol = fval("vol", p.vol);
    p.cs = fval("Cs", p.cs);
    p.ampwg = fval("ampwg", p.ampwg);
    p.bfactor = fval("Bfactor", p.bfactor);
    p.first = ival("first", p.first);
    p.last = ival("last", p.last);
    p.pr_threshold = fval("PR_threshold", p.pr_threshold);
    p.ncycle = ival("Ncycle", p.ncycle);
    p.searchstep = fval("searchstep", p.searchstep);
    p.realspaceavg = yes(sval("realspaceavg", "n"));
    p.subrec = yes(sval("subrec", "n"));
    p.fsc = yes(sval("FSC", "n"));
    p.imgstck = !imgstck.empty();
    p.maxcentshift = fval("maxcentshift", p.maxcentshift);
    p.boundx = fval("boundX", p.boundx);
    if (sval("sym", "icos") != "icos") return die("only sym=icos is on this path", 2);
    if (has("corrCTF") || has("recISAF") || has("loc_box"))
        return die("corrCTF / recISAF / loc_box modes are not on this path", 2);
    if (cryoim_params_derive(&p)) return die("parameters", 2);
    if (p.first < 1 || p.last < p.first || p.last > nrows) return die("first/last out of range", 2);

    // load_original_ortcent + checkstckfile (checkstckfile.f90:7-24)
    const int P = p.last - p.first + 1;
    std::vector<cryoim_particle> parts(P);
    std::vector<char> names((size_t)P * 256);
    if (cryoim_ort_read(ortfile.c_str(), p.first, p.last, parts.data(), names.data(), 256))
        return die("malformed or short ortfile", 2);
    std::vector<std::string> stck(P);
    int bad = 0;
    std::map<std::string, int> nz;
    for (int i = 0; i < P; ++i) {
        stck[i] = &names[(size_t)i * 256];
        if (!imgstck.empty()) continue;
        auto it = nz.find(stck[i]);
        if (it == nz.end()) {
            cryoim_mrc_header h;
            int z = cryoim_mrc_read_header(stck[i].c_str(), &h) ? -1 : h.nz;
            if (z < 0) std::printf(" the stck file %s is not exist.\n", stck[i].c_str());
            it = nz.emplace(stck[i], z).first;
        }
        if (it->second < 0) { ++bad; continue; }
        if (it->second < parts[i].img_particle_id) {
            std::printf(" the particle number between ortfile and %s is not match.\n", stck[i].c_str());
            ++bad;
        }
    }
    if (bad) { std::puts(" please check the ortfile and stckfiles."); return 3; }
    std::puts(" the ortfile and stckfiles are match each other.");

    if (cryoim_ctx_create(device, &ctx) || cryoim_set_params(ctx, &p)) return die("device", 2);
    const int chunk = std::max(1, ival("batch", 256));
    const int nx = p.fftsize;
    std::vector<float> imgs;

    if (mode == 4 || mode == 5) {
        // templates (load_template.f90): templatestck, else projections of model3d
        const std::string tort = sval("templateort", "");
        int T = 0;
        if (tort.empty() || cryoim_template_ort_read(tort.c_str(), nullptr, 0, &T) || T < 1)
            return die("templateort is required", 2);
        std::vector<cryoim_template> t(T);
        cryoim_template_ort_read(tort.c_str(), t.data(), T, &T);
        std::vector<float> timg((size_t)T * nx * nx), map;
        if (has("model3d")) {
            map.resize((size_t)nx * nx * nx);
            if (cryoim_mrc_read_sections(sval("model3d", "").c_str(), 1, nx, map.data())) return die("model3d", 2);
        }
        if (has("templatestck")) {
            if (cryoim_mrc_read_sections(sval("templatestck", "").c_str(), 1, T, timg.data()))
                return die("templatestck", 2);
        } else if (!map.empty()) {
            if (cryoim_project_templates(ctx, map.data(), t.data(), T, timg.data())) return die("projection", 2);
        } else {
            return die("mode 4/5 needs templatestck or model3d", 2);
        }
        if (cryoim_load_templates(ctx, timg.data(), t.data(), T)) return die("templates", 2);
        const bool contract = mode == 4 && yes(sval("contract", "n"));
        cryoim_contract_opts co{fval("originmax", 6.0f), fval("originstep", 0.5f), ival("topk", 16), 0,
                                sval("precision", "bf16") == "fp8" ? 1 : 0, ival("nbr", 1), ival("coarse", 0),
                                ival("learned", 0), ival("nbrbest", 0), fval("localrange", 0.0f),
                                fval("localstep", 0.25f)};
        co.proposal_nbr = ival("proposalnbr", 0);
        if (co.local_range > 0.0f) co.pick = 1;  // the local form picks by FP64 correlation
        if (contract) {
            if (map.empty()) return die("contract=y needs model3d", 2);
            if (cryoim_set_reference_map(ctx, map.data())) return die("reference map", 2);
            if (co.local_range > 0.0f && cryoim_set_interpolation(ctx, 2, 0.0f)) return die("interpolation", 2);
            if (co.learned > 0) {
                const std::string model = sval("learnmodel", "proposer.bin");
                std::FILE* f = std::fopen(model.c_str(), "rb");
                if (f) {
                    std::fclose(f);
                    if (cryoim_learn_load(ctx, model.c_str())) return die("learnmodel", 2);
                } else {
                    cryoim_learn_opts lo;
                    cryoim_learn_opts_default(&lo);
                    lo.samples = ival("learnsamples", 25600);
                    lo.origin_max = co.origin_max;
                    float st[4];
                    if (cryoim_learn_train(ctx, map.data(), &lo, st)) return die("proposer training", 2);
                    std::printf("proposer: %d views, trained on %d projections in %.1f s (loss %.3f)\n",
                                (int)st[3], lo.samples, st[1], st[0]);
                    if (cryoim_learn_save(ctx, model.c_str())) return die("learnmodel write", 2);
                }
            }
        }
        const std::string out = sval("newortfile", "newort.dat");
        std::FILE* trunc = std::fopen(out.c_str(), "w");
        if (!trunc) return die("cannot write newortfile", 2);
        std::fclose(trunc);
        for (int i0 = 0; i0 < P; i0 += chunk) {
            const int n = std::min(chunk, P - i0);
            if (gather(parts, stck, i0, n, nx, imgstck, p.first, imgs)) return die("particle stack read", 2);
            int r = mode == 5 ? cryoim_refine(ctx, imgs.data(), &parts[i0], n)
                              : contract ? cryoim_contract_search(ctx, imgs.data(), &parts[i0], n, &co, nullptr)
                                         : cryoim_globesearch(ctx, imgs.data(), &parts[i0], n, nullptr);
            if (r) return die("search", 2);
            for (int i = 0; i < n; ++i) {
                const cryoim_particle& q = parts[i0 + i];
                std::printf("%12d %14.7f %14.7f %14.7f %14.7f %14.7f %14.7f\n", p.first + i0 + i, q.theta, q.phi,
                            q.omega, q.x, q.y, q.pr);
            }
            if (cryoim_ort_write(out.c_str(), &parts[i0], &names[(size_t)i0 * 256], 256, n, 54, 1))
                return die("cannot write newortfile", 2);
        }
    } else if (mode == 3) {
        // 0main.f90:237-241: calc_center with model3d, else calc_center_selfrot180; then
        // output_ort.f90 writes every particle of first..last to newortfile
        std::vector<float> map;
        if (has("model3d")) {
            map.resize((size_t)nx * nx * nx);
            if (cryoim_mrc_read_sections(sval("model3d", "").c_str(), 1, nx, map.data())) return die("model3d", 2);
        }
        // calc_center.f90:40-53 reads the particles' own stacks even with imgstck
        const std::string src = map.empty() ? imgstck : std::string();
        for (int i0 = 0; i0 < P; i0 += chunk) {
            const int n = std::min(chunk, P - i0);
            if (gather(parts, stck, i0, n, nx, src, p.first, imgs)) return die("particle stack read", 2);
            if (cryoim_center(ctx, map.empty() ? nullptr : map.data(), imgs.data(), &parts[i0], n))
                return die("centring", 2);
            for (int i = 0; i < n; ++i) {
                const cryoim_particle& q = parts[i0 + i];
                std::printf("%12d %14.7f %14.7f %14.7f\n", p.first + i0 + i, q.x, q.y, q.pr);
            }
        }
        const std::string out = sval("newortfile", "newort.dat");
        if (cryoim_ort_write(out.c_str(), parts.data(), names.data(), 256, P, 54, 0))
            return die("cannot write newortfile", 2);
    } else if (mode == 1 && p.fsc) {
        // 0main.f90:207-222: odd half (first, first+2, ...) into oddtnf, even half
        // (first+1, ...) into evetnf, both masked at particle(first)'s origin; without
        // subrec, reconstruct_FSC combines them into FSC.txt and result3d.
        const std::string res = sval("result3d", "map3d.mrc");
        const size_t t = (size_t)(2 * p.max_r + 1), tnf = t * t * (p.max_r + 1);
        std::vector<float> half[2][3];
        std::string last_stack = imgstck;
        for (int parity = 0; parity < 2; ++parity) {
            std::vector<cryoim_particle> hp;
            std::vector<std::string> hs;
            for (int i = parity; i < P; i += 2) { hp.push_back(parts[i]); hs.push_back(stck[i]); }
            if (cryoim_rec_begin_half(ctx, parts[0].x, parts[0].y)) return die("half map", 2);
            const int H = (int)hp.size();
            int used = 0;
            for (int i0 = 0; i0 < H; i0 += chunk) {
                const int n = std::min(chunk, H - i0);
                // with imgstck the reference reads the stack in sequence from image first
                // of the half, one image per step of two particles (reconstruct_half.f90:
                // 32-36, 53): particle first+2k meets image first+k
                if (gather(hp, hs, i0, n, nx, imgstck, p.first + parity, imgs)) return die("particle stack read", 2);
                int u = 0;
                if (cryoim_rec_insert(ctx, imgs.data(), &hp[i0], n, &u)) return die("insertion", 2);
                used += u;
            }
            if (H > 0 && imgstck.empty()) last_stack = hs[H - 1];
            std::printf(" half %s: used particles: %d of %d\n", parity ? "even" : "odd", used, H);
            for (auto& v : half[parity]) v.resize(tnf);
            if (cryoim_rec_get_partial(ctx, half[parity][0].data(), half[parity][1].data(), half[parity][2].data()))
                return die("partial", 2);
            const std::string name = (p.subrec ? res : std::string()) + (parity ? "evetnf" : "oddtnf");
            // reconstruct_half.f90:140-144: the header flag is subrec
            if (cryoim_tnf_write(name.c_str(), nx, p.max_r, p.apix, p.imgmask_px, p.subrec, p.realspaceavg,
                                 half[parity][0].data(), half[parity][1].data(), half[parity][2].data()))
                return die("cannot write the half-map tnf", 2);
        }
        if (!p.subrec) {
            std::vector<float> fsc(p.max_r + 1), map((size_t)nx * nx * nx);
            if (cryoim_fsc_combine(ctx, half[0][0].data(), half[0][1].data(), half[0][2].data(), half[1][0].data(),
                                   half[1][1].data(), half[1][2].data(), fsc.data(), map.data()))
                return die("FSC", 2);
            std::FILE* f = std::fopen("FSC.txt", "w");  // reconstruct_FSC.f90:14, 56
            if (!f) return die("cannot write FSC.txt", 2);
            for (int ir = 0; ir <= p.max_r; ++ir) {
                const float F = fsc[ir], w = std::sqrt(2.0f * F / (1.0f + F));
                std::fprintf(f, "%12d %15.7f ", ir, F);
                if (w == w) std::fprintf(f, "%15.7f\n", w);
                else std::fprintf(f, "%15s\n", "NaN");
            }
            std::fclose(f);
            // reconstruct_FSC.f90:181-182 writes the header it last read: that of the
            // particle stack the even half read last
            cryoim_mrc_header oh;
            if (cryoim_mrc_read_header(last_stack.c_str(), &oh)) cryoim_map_header(&oh, nx, nx, nx, p.apix);
            if (cryoim_mrc_write(res.c_str(), &oh, map.data(), (int64_t)map.size())) return die("cannot write result3d", 2);
        }
    } else if (mode == 1) {
        if (cryoim_rec_begin(ctx)) return die("reconstruction", 2);
        int used = 0;
        for (int i0 = 0; i0 < P; i0 += chunk) {
            const int n = std::min(chunk, P - i0);
            if (gather(parts, stck, i0, n, nx, imgstck, p.first, imgs)) return die("particle stack read", 2);
            int u = 0;
            if (cryoim_rec_insert(ctx, imgs.data(), &parts[i0], n, &u)) return die("insertion", 2);
            used += u;
        }
        std::printf(" used particles: %d of %d\n", used, P);
        const std::string out = sval("result3d", "map3d.mrc");
        if (p.subrec) {
            const size_t t = (size_t)(2 * p.max_r + 1);
            std::vector<float> fa(t * t * (p.max_r + 1)), fb(fa.size()), wg(fa.size());
            if (cryoim_rec_get_partial(ctx, fa.data(), fb.data(), wg.data())) return die("partial", 2);
            if (cryoim_tnf_write(out.c_str(), nx, p.max_r, p.apix, p.imgmask_px, p.fsc, p.realspaceavg, fa.data(),
                                 fb.data(), wg.data()))
                return die("cannot write result3d", 2);
        } else {
            std::vector<float> map((size_t)nx * nx * nx);
            if (cryoim_rec_finish(ctx, map.data())) return die("reconstruction finish", 2);
            cryoim_mrc_header oh;
            cryoim_map_header(&oh, nx, nx, nx, p.apix);
            if (cryoim_mrc_write(out.c_str(), &oh, map.data(), (int64_t)map.size())) return die("cannot write result3d", 2);
        }
    } else {
        return die("mode must be 0, 1, 3, 4 or 5 on this path", 2);
    }
    cryoim_ctx_destroy(ctx);
    return 0;
}
