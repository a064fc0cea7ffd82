// api.cu — context, drivers and the C ABI of libcryoim_gb300.so (include/cryoim.h).
//
// Host-side logic mirrors the reference drivers: ort_globesearch.f90 (mode 4),
// ort_refinement.f90 (mode 5), reconstruct.f90 / reconstruct_substep.f90 (mode 1),
// load_template.f90, and proc_icos's orientation transforms.  Device work runs on one
// CUDA stream per context; particles are processed in batches of `batch` images.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <iterator>
#include <map>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cryoim.h"
#include "geom.cuh"
#include "kernels.h"

using namespace cryoim;

namespace {

thread_local std::string g_err = "";

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e__ = (x);                                                                  \
        if (e__ != cudaSuccess)                                                                 \
            return fail(CRYOIM_ERR_CUDA, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e__), \
                        __FILE__, __LINE__);                                                    \
    } while (0)
#define CKF(x)                                                                                \
    do {                                                                                      \
        cufftResult r__ = (x);                                                                \
        if (r__ != CUFFT_SUCCESS)                                                             \
            return fail(CRYOIM_ERR_CUDA, "%s failed: cufft %d (%s:%d)", #x, (int)r__, __FILE__, \
                        __LINE__);                                                            \
    } while (0)

// ---------------------------------------------------------------------------
// host geometry
// ---------------------------------------------------------------------------

// The 60 operators, generated from the group generators of
// proc_icos/SRC/icos2f_operation_matrix.f90:13-55 (in R), generator order.
template <class R> void gen_ops(R* r) {
    const R d2r = R(4) * std::atan2(R(1), R(1)) / R(180);
    R a5 = R(72) * d2r;
    R v = std::acos(std::cos(R(60) * d2r) / std::sin(R(36) * d2r));
    R rz5[9] = {std::cos(a5), -std::sin(a5), 0, std::sin(a5), std::cos(a5), 0, 0, 0, 1};
    R ryv[9] = {std::cos(v), 0, std::sin(v), 0, 1, 0, -std::sin(v), 0, std::cos(v)};
    R ryvt[9] = {ryv[0], ryv[3], ryv[6], ryv[1], ryv[4], ryv[7], ryv[2], ryv[5], ryv[8]};
    auto mm = [](const R* a, const R* b, R* c) {
        R t[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                R s = a[i * 3] * b[j];
                s = s + a[i * 3 + 1] * b[3 + j];
                s = s + a[i * 3 + 2] * b[6 + j];
                t[i * 3 + j] = s;
            }
        std::memcpy(c, t, sizeof(t));
    };
    R t[9];
    mm(rz5, ryvt, t);
    mm(ryv, t, rz5);
    const R rx2[9] = {1, 0, 0, 0, -1, 0, 0, 0, -1};
    const R ry2[9] = {-1, 0, 0, 0, 1, 0, 0, 0, -1};
    const R r3[9] = {0, 0, 1, 1, 0, 0, 0, 1, 0};
    for (int k = 0; k < 9; ++k) r[k] = (k % 4 == 0) ? R(1) : R(0);
    for (int i = 1; i < 5; ++i) mm(r + (i - 1) * 9, rz5, r + i * 9);
    for (int i = 5; i < 10; ++i) mm(rx2, r + (i - 5) * 9, r + i * 9);
    for (int i = 10; i < 20; ++i) mm(ry2, r + (i - 10) * 9, r + i * 9);
    for (int i = 20; i < 60; ++i) mm(r3, r + (i - 20) * 9, r + i * 9);
}

// icosprocess/SRC/icos2f_sym_mat.f90:5-243 holds the same 60 matrices in another order;
// entry k of that table is generator element TABLE_FROM_GEN[k].
const int TABLE_FROM_GEN[60] = {
    0, 26, 34, 48, 42, 24, 56, 28, 17, 23, 6, 52, 49, 41, 58, 9, 37, 18, 32, 54,
    36, 1, 2, 3, 4, 8, 29, 35, 45, 40, 20, 31, 7, 38, 22, 55, 30, 59, 51, 25,
    50, 19, 47, 43, 16, 27, 13, 12, 33, 15, 44, 14, 5, 11, 46, 57, 53, 21, 10, 39};

const float* table_ops() {
    static float tab[540];
    static bool init = false;
    if (!init) {
        double g[540];
        gen_ops<double>(g);
        const double cand[5] = {0.0, 0.5, 1.0, 0.80901699437494742, 0.30901699437494742};
        for (int k = 0; k < 60; ++k)
            for (int e = 0; e < 9; ++e) {
                double x = g[TABLE_FROM_GEN[k] * 9 + e], ax = std::fabs(x), best = 0.0;
                for (double c : cand)
                    if (std::fabs(ax - c) < std::fabs(ax - best)) best = c;
                tab[k * 9 + e] = (float)(x < 0 ? -best : best);
            }
        init = true;
    }
    return tab;
}

// proc_icos/SRC/Eularmatrix.f90:1-15
void eular_matrix(float theta0, float phi0, float omega0, float* r) {
    const float d2r = 4.0f * std::atan2(1.0f, 1.0f) / 180.0f;
    float theta = theta0 * d2r, phi = phi0 * d2r, omega = omega0 * d2r;
    r[0] = cosf(phi) * cosf(theta) * cosf(omega) - sinf(phi) * sinf(omega);
    r[1] = -cosf(phi) * cosf(theta) * sinf(omega) - sinf(phi) * cosf(omega);
    r[2] = cosf(phi) * sinf(theta);
    r[3] = sinf(phi) * cosf(theta) * cosf(omega) + cosf(phi) * sinf(omega);
    r[4] = -sinf(phi) * cosf(theta) * sinf(omega) + cosf(phi) * cosf(omega);
    r[5] = sinf(phi) * sinf(theta);
    r[6] = -sinf(theta) * cosf(omega);
    r[7] = sinf(theta) * sinf(omega);
    r[8] = cosf(theta);
}

// equalort.f90:13-21 / transform_ort_2fTo5f.f90:19-27
void euler_from(const float* r, float* th, float* ph, float* om) {
    const float r2d = 45.0f / std::atan2(1.0f, 1.0f);
    if (r[8] >= 1.0f) *th = 0.0f;
    else if (r[8] < -1.0f) *th = 180.0f;
    else *th = acosf(r[8]) * r2d;
    *ph = atan2f(r[5], r[2]) * r2d;
    *om = atan2f(r[7], -r[6]) * r2d;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
template <class T> struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    bool own = true;  // false: another context's buffer, used read-only and never freed here
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    int ensure(size_t want) {
        if (want <= n) return 0;
        release();
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(CRYOIM_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", want * sizeof(T),
                        cudaGetErrorString(e));
        }
        n = want;
        return 0;
    }
    void borrow(const DBuf& o) {
        release();
        p = o.p;
        n = o.n;
        own = false;
    }
    void release() {
        if (p && own) cudaFree(p);
        p = nullptr;
        n = 0;
        own = true;
    }
};

// accumulation kinds: full box (reconstruct.f90), tnf partial (reconstruct_substep.f90),
// tnf half map (reconstruct_half.f90)
enum { REC_FULL = 0, REC_SUBSTEP = 1, REC_HALF = 2 };

// The ASU view grid of ort_globesearch.f90:68-101 at a given step: views (theta, phi,
// slot bits, 0), with the slot <-> view maps used for grid neighbours.
struct ViewGrid {
    float step = 0.0f;
    int nth = 0, nph = 0, nom = 0, V = 0;
    std::vector<float> views;
    std::vector<int> view_slot, slot_view;
};

static void build_view_grid(float step, ViewGrid* g) {
    g->step = step;
    g->nth = (int)(21.0f / step);
    g->nph = (int)(32.0f / step);
    g->nom = (int)(360.0f / step);
    const Angles an = host_angles();
    const float d2r = an.deg2rad;
    const AsuPlanes pl = asu_planes(d2r);
    g->views.clear();
    for (int it = 0; it <= g->nth; ++it) {
        const float theta = 69.0f + step * (float)it;
        const float z = cosf(theta * d2r), z0 = sinf(theta * d2r);
        for (int iph = 0; iph <= g->nph; ++iph) {
            const float phi = step * (float)iph;
            const float x = z0 * cosf(phi * d2r), y = z0 * sinf(phi * d2r);
            if (!asu_inside(pl, x, y, z)) continue;
            for (int sgn = (iph == 0 ? -1 : 1); sgn >= -1; sgn -= 2) {
                const int slot = it * (2 * g->nph + 1) + (sgn * iph + g->nph);
                float v[4] = {theta, sgn > 0 ? phi : -phi, 0.0f, 0.0f};
                std::memcpy(&v[2], &slot, 4);
                g->views.insert(g->views.end(), v, v + 4);
            }
        }
    }
    g->V = (int)(g->views.size() / 4);
    g->view_slot.assign(g->V, -1);
    g->slot_view.assign((size_t)(g->nth + 1) * (2 * g->nph + 1), -1);
    for (int v = 0; v < g->V; ++v) {
        int slot;
        std::memcpy(&slot, &g->views[4 * v + 2], 4);
        g->view_slot[v] = slot;
        g->slot_view[slot] = v;
    }
}

// The learned proposer's weights, Adam state and activations (learn.cu has the layers).
struct LearnModel {
    bool ready = false;
    int V = 0;          // classes: views of the twice-the-step grid
    int sign = 1;       // +1: an in-plane rotation by w shifts the features by +w
    float step = 0.0f;  // search step the view grid belongs to
    long nparam = 0;
    long oW[5] = {0}, ob[5] = {0}, oT = 0;  // parameter offsets (conv 1-4, mix)
    int steps = 0;      // Adam steps taken
    int cap = 0, capV = 0;  // batch capacity of the activations, views they were sized for
    DBuf<float> w, gr, m, v, vview, wflip;
    DBuf<float> feat, a1, a2, p2, a3, p3, a4, p4, g, sc, dsc, dg, dp4, da4, dp3, da3, dp2, da2, da1, loss, truth;
    DBuf<int> cell;
    DBuf<float> cellv;
    DBuf<float2> hscr;  // the head's frequency-domain scratch
    bool conv_tc = true;  // convolutions on the tensor cores (TF32) or on the CUDA cores (FP32)
    DBuf<int> cerr;       // set by a tensor-core convolution whose wait timed out
    void release() {
        for (DBuf<float>* b : {&w, &gr, &m, &v, &vview, &wflip, &feat, &a1, &a2, &p2, &a3, &p3, &a4, &p4, &g, &sc,
                               &dsc, &dg, &dp4, &da4, &dp3, &da3, &dp2, &da2, &da1, &loss, &truth, &cellv})
            b->release();
        cell.release();
        hscr.release();
        cerr.release();
        ready = false;
        cap = 0;
    }
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // CUDA-event timing of the hot kernel launches (off by default)
    bool prof = false;
    cudaEvent_t pe0 = nullptr, pe1 = nullptr;
    double prof_ms = 0.0;
    long long prof_launches = 0;
    cryoim_params p{};
    bool have_params = false;
    Band bd{};
    int batch = 64;
    DBuf<float> ops;  // 540, table order
    // templates
    int T = 0;
    std::vector<cryoim_template> tmpl;
    DBuf<float2> tband;
    DBuf<float> tfcut0, tort;
    // search grid
    bool grid_ready = false;
    int nth = 0, nph = 0, nom = 0, V = 0;
    std::vector<float> views;  // V x 4
    DBuf<float> d_views;
    DBuf<float2> alpha;
    // per-batch scratch
    DBuf<float> imgs, par, fcut0, ctf, tfcut, state, cand, rpr, rot, prbuf;
    DBuf<float2> fft, band, ralpha;
    DBuf<unsigned long long> best;
    DBuf<int> flag, sel;
    std::map<int, cufftHandle> plans;
    // reconstruction
    DBuf<float4> acc;
    DBuf<int2> samples;
    DBuf<float2> vol;
    bool rec_active = false;
    int rec_kind = 0;  // REC_FULL, REC_SUBSTEP or REC_HALF
    int nsamples = 0, rec_used = 0, rec_img_id0 = -100;
    float rec_src_df[3] = {0, 0, 0};
    bool rec_have_first = false;
    float rec_ox = 0, rec_oy = 0;
    float rec_off_xy = 0, rec_off_z = 0;
    int rec_base_xy = 0, rec_base_z = 0;
    // contraction form: map band cube, samples, orientation sections (operand B)
    DBuf<float2> mapcube;
    bool map_ready = false;
    DBuf<int2> csamples;
    int cS = 0, cKpad = 0;
    DBuf<uint16_t> bmat;
    long n_orient = 0;
    bool bmat_ready = false;
    double bmat_ms = 0.0;
    DBuf<uint16_t> amat;
    // FP8-e4m3 operands: B8 (n_orient x cKpad8 bytes), per-sample band scales, A8
    DBuf<uint8_t> bmat8, amat8;
    bool bmat8_ready = false;
    double bmat8_ms = 0.0;
    int cKpad8 = 0, last_kpad = 0;
    double last_slice_ms = 0.0;
    int last_fallbacks = 0;   // particles of the last contraction call re-searched exhaustively
    float interp_sigma = 0.0f;  // sections: 0 trilinear, > 0 Gaussian kernel of this width (voxels)
    // band cube of the reference map: of the map itself (ovs 1) or of the map zero-padded
    // to twice its side (ovs 2, trilinear on a twice-oversampled transform); its radius
    // cube_r (side 2 cube_r + 3); the map kept on the device to rebuild it
    int ovs = 1, cube_r = 0;
    DBuf<float> mapreal;
    DBuf<float> poff;         // per-pass particle origins (x, y) of the centred origin grid
    DBuf<float> mulA, mulB;
    DBuf<unsigned> bandmax;
    DBuf<int> fexp;
    // coarse-to-fine proposals: a 2x-step grid, the half-radius band, a 2x-step origin
    // grid; its BF16 sections; the proposal forms' per-pass row lists (gidx) and the local
    // form's cut sections (bgather)
    ViewGrid cgrid;
    DBuf<int2> csamples_c;
    int cS_c = 0, cKpad_c = 0, n_origin_c = 0;
    float orig_max_c = -1.0f, orig_step_c = -1.0f;
    DBuf<uint16_t> bmat_c, amat_c;
    bool bmat_c_ready = false;
    long n_orient_c = 0;
    DBuf<float> corigins_c, topv_c, tilev_c, kcc_c;
    DBuf<int> topi_c, tileo_c, tileorig_c, kor_c, korig_c, gidx;
    DBuf<double> pnorm_c;
    DBuf<uint8_t> bgather;
    DBuf<float> corigins, topv, kcc, kcand;
    DBuf<int> topi, gerr, kor, korig;
    DBuf<double> pnorm, kcc64;
    DBuf<double2> pcband;  // per particle of a pass: CTF x (a, b) per band sample, FP64
    // the local form's unbiased score: per particle of a pass sum |P|^2 and the CTF per sample
    DBuf<double> pnorm0;
    DBuf<float> pctf;
    DBuf<int> xorient;  // rescoring: each candidate's grid orientation (view * nom + omega index)
    int n_origin = 0;
    float orig_max = -1.0f, orig_step = -1.0f;
    DBuf<float> tilev, xcand, xpr;
    DBuf<int> tileo, tileorig;
    DBuf<float2> xalpha;
    DBuf<float4> sband;
    DBuf<int> xcount;
    DBuf<double> kpart;
    DBuf<float4> tbandc;
    DBuf<int4> xgroups;
    DBuf<float> lcentre;  // local form: (theta, phi, omega) grid centre per particle of a group
    DBuf<GemmGroup> ggroups;
    DBuf<int2> gseg;
    LearnModel lm;
    // view <-> grid slot (itheta * (2 Nphi + 1) + iphi + Nphi) maps for neighbours
    std::vector<int> view_slot, slot_view;
    std::vector<uint8_t> list_mark;  // one byte per fine-grid orientation (expand_seeds)
    int num_sms = 0;
    // CUDA-event timing of the contraction launches (with prof)
    double prof_gemm_ms = 0.0;
    long long prof_gemm_launches = 0;
    double prof_gemm_flops = 0.0;
    // phase-residual rescoring launches of the contraction forms (profiling on)
    double prof_pr_ms = 0.0;
    long long prof_pr_launches = 0;
    double prof_pr_cands = 0.0;

    // pass lanes of the contraction search: this context and xlanes (refresh_lane), each
    // extra lane with its own stream and per-pass buffers, this context's read-only
    // state borrowed
    int lanes = 6;
    std::vector<Ctx*> xlanes;

    ~Ctx() {
        for (Ctx* x : xlanes) delete x;
        cudaSetDevice(device);
        for (auto& kv : plans) cufftDestroy(kv.second);
        ops.release(); tband.release(); tfcut0.release(); tort.release(); d_views.release();
        alpha.release(); imgs.release(); par.release(); fcut0.release(); ctf.release();
        tfcut.release(); state.release(); cand.release(); rpr.release(); rot.release();
        prbuf.release(); fft.release(); band.release(); ralpha.release(); best.release();
        flag.release(); sel.release(); acc.release(); samples.release(); vol.release();
        mapcube.release(); mapreal.release(); csamples.release(); bmat.release(); amat.release(); corigins.release();
        topv.release(); kcc.release(); kcand.release(); topi.release(); gerr.release();
        kor.release(); korig.release(); pnorm.release(); kcc64.release(); pnorm0.release(); pctf.release();
        xorient.release();
        tilev.release(); xcand.release(); xpr.release(); tileo.release(); tileorig.release();
        xalpha.release(); bmat8.release(); amat8.release(); mulA.release(); mulB.release();
        bandmax.release(); fexp.release();
        csamples_c.release(); bmat_c.release(); amat_c.release(); corigins_c.release(); topv_c.release();
        tilev_c.release(); kcc_c.release(); topi_c.release(); tileo_c.release(); tileorig_c.release();
        kor_c.release(); korig_c.release(); gidx.release(); pnorm_c.release(); bgather.release();
        sband.release(); xcount.release(); kpart.release(); ggroups.release(); gseg.release(); tbandc.release(); xgroups.release(); lcentre.release();
        lm.release();
        if (pe0) cudaEventDestroy(pe0);
        if (pe1) cudaEventDestroy(pe1);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

Ctx* as_ctx(void* c) { return reinterpret_cast<Ctx*>(c); }

int refresh_lane(Ctx* c, int i);

int plan2d(Ctx* c, int nb, cufftHandle* out) {
    auto it = c->plans.find(nb);
    if (it != c->plans.end()) {
        *out = it->second;
        return CRYOIM_OK;
    }
    cufftHandle h;
    int n[2] = {c->p.fftsize, c->p.fftsize};
    CKF(cufftPlanMany(&h, 2, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_C2C, nb));
    CKF(cufftSetStream(h, c->stream));
    c->plans[nb] = h;
    *out = h;
    return CRYOIM_OK;
}

int check_ready(Ctx* c, bool need_templates) {
    if (!c) return fail(CRYOIM_ERR_ARG, "null context");
    if (!c->have_params) return fail(CRYOIM_ERR_STATE, "cryoim_set_params has not been called");
    if (need_templates && c->T <= 0)
        return fail(CRYOIM_ERR_STATE, "cryoim_load_templates has not been called");
    CK(cudaSetDevice(c->device));
    return CRYOIM_OK;
}

int ensure_batch(Ctx* c, int B) {
    const long nn = (long)c->p.fftsize * c->p.fftsize;
    const Band& bd = c->bd;
    const long w2 = (long)bd.W * bd.W;
    int r;
    if ((r = c->imgs.ensure((size_t)B * nn))) return r;
    if ((r = c->fft.ensure((size_t)B * nn))) return r;
    if ((r = c->band.ensure((size_t)B * w2))) return r;
    if ((r = c->fcut0.ensure((size_t)B * bd.nr))) return r;
    if ((r = c->ctf.ensure((size_t)B * w2))) return r;
    if ((r = c->par.ensure((size_t)B * 8))) return r;
    if ((r = c->best.ensure((size_t)B))) return r;
    if ((r = c->flag.ensure(4))) return r;
    if ((r = c->sel.ensure((size_t)B))) return r;
    if ((r = c->rot.ensure((size_t)B * 9))) return r;
    if (c->T > 0 && (r = c->tfcut.ensure((size_t)B * c->T * bd.nr))) return r;
    return CRYOIM_OK;
}

// Per-image parameter block on the device: [ox | oy | sx | sy | df(3) ...] of B each.
struct ParView {
    float *ox, *oy, *sx, *sy, *dfs;
};
ParView par_view(Ctx* c, int B) {
    float* b = c->par.p;
    return ParView{b, b + B, b + 2 * B, b + 3 * B, b + 4 * B};
}

// Mask / checkerboard / FFT / band of nb images already on the device.
// keep_flag: leave the non-finite-input flag as it is (a caller that checks it once
// after several batches) instead of clearing it first.  need_fcut = false: the band only,
// without the particle's amplitude cuts (FT_amp_expfit).
int transform_batch(Ctx* c, const float* d_src, int nb, int B, const std::vector<float>& hpar,
                    int use_mask, int normalize, bool shift, bool keep_flag = false, bool need_fcut = true) {
    ParView pv = par_view(c, B);
    CK(cudaMemcpyAsync(c->par.p, hpar.data(), sizeof(float) * 8 * B, cudaMemcpyHostToDevice,
                       c->stream));
    if (!keep_flag) CK(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
    launch_prep_images(d_src, nb, c->p.fftsize, pv.ox, pv.oy, use_mask, c->p.imgmask_px, normalize,
                       c->fft.p, c->flag.p, c->stream);
    CK(cudaGetLastError());
    cufftHandle h;
    int r = plan2d(c, nb, &h);
    if (r) return r;
    CKF(cufftExecC2C(h, (cufftComplex*)c->fft.p, (cufftComplex*)c->fft.p, CUFFT_FORWARD));
    launch_post_fft(c->fft.p, nb, c->bd, shift ? pv.sx : nullptr, shift ? pv.sy : nullptr,
                    c->band.p, need_fcut ? c->fcut0.p : nullptr, c->stream);
    CK(cudaGetLastError());
    return CRYOIM_OK;
}

int check_flag(Ctx* c) {
    int f = 0;
    CK(cudaMemcpyAsync(&f, c->flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (f) return fail(CRYOIM_ERR_INPUT, "non-finite pixel (NaN/Inf) in an input image");
    return CRYOIM_OK;
}

// Views of ort_globesearch.f90:68-101.  For iphi = 0 the reference evaluates (theta, 0)
// and then (theta, -0) into the same slot; only the second survives, so only it is run.
int ensure_grid(Ctx* c) {
    if (c->grid_ready) return CRYOIM_OK;
    const float step = c->p.searchstep;
    c->nth = (int)(21.0f / step);
    c->nph = (int)(32.0f / step);
    c->nom = (int)(360.0f / step);
    if (c->nom < 1 || c->nom > 768)
        return fail(CRYOIM_ERR_SIZE, "searchstep %g gives Nomega=%d (supported 1..768)", step, c->nom);
    Angles an = host_angles();
    const float d2r = an.deg2rad;
    AsuPlanes pl = asu_planes(d2r);
    c->views.clear();
    for (int it = 0; it <= c->nth; ++it) {
        float theta = 69.0f + step * (float)it;
        float tmp = theta * d2r;
        float z = cosf(tmp), z0 = sinf(tmp);
        for (int iph = 0; iph <= c->nph; ++iph) {
            float phi = step * (float)iph;
            tmp = phi * d2r;
            float x = z0 * cosf(tmp), y = z0 * sinf(tmp);
            if (!asu_inside(pl, x, y, z)) continue;
            for (int sgn = (iph == 0 ? -1 : 1); sgn >= -1; sgn -= 2) {
                int slot = (it * (2 * c->nph + 1) + (sgn * iph + c->nph)) * c->nom;
                float v[4];
                v[0] = theta;
                v[1] = (sgn > 0) ? phi : -phi;
                std::memcpy(&v[2], &slot, 4);
                v[3] = 0.0f;
                c->views.insert(c->views.end(), v, v + 4);
            }
        }
    }
    c->V = (int)(c->views.size() / 4);
    c->view_slot.assign(c->V, -1);
    c->slot_view.assign((size_t)(c->nth + 1) * (2 * c->nph + 1), -1);
    for (int v = 0; v < c->V; ++v) {
        int base;
        std::memcpy(&base, &c->views[4 * v + 2], 4);
        c->view_slot[v] = base / c->nom;
        c->slot_view[base / c->nom] = v;
    }
    int r;
    if ((r = c->d_views.ensure(c->views.size() + 4))) return r;
    CK(cudaMemcpyAsync(c->d_views.p, c->views.data(), sizeof(float) * c->views.size(),
                       cudaMemcpyHostToDevice, c->stream));
    if (c->V > 0 && c->T > 0) {  // common-line angles of the phase-residual search
        std::vector<float> v2(2 * c->V);
        for (int v = 0; v < c->V; ++v) { v2[2 * v] = c->views[4 * v]; v2[2 * v + 1] = c->views[4 * v + 1]; }
        DBuf<float> tmp;
        if ((r = tmp.ensure(v2.size()))) return r;
        CK(cudaMemcpyAsync(tmp.p, v2.data(), sizeof(float) * v2.size(), cudaMemcpyHostToDevice,
                           c->stream));
        if ((r = c->alpha.ensure((size_t)c->V * c->T * 60))) return r;
        launch_alpha_table(tmp.p, c->V, c->tort.p, c->T, c->ops.p, c->alpha.p, c->stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
        tmp.release();
    }
    c->grid_ready = true;
    return CRYOIM_OK;
}

unsigned long long key_of(float pr, unsigned idx) {
    unsigned bits;
    std::memcpy(&bits, &pr, 4);
    return ((unsigned long long)bits << 32) | idx;
}

int globesearch_impl(Ctx* c, const float* imgs, bool on_device, cryoim_particle* parts, int P,
                     float* pr_array) {
    int r = check_ready(c, true);
    if (r) return r;
    if (!imgs || !parts || P < 0) return fail(CRYOIM_ERR_ARG, "null input or negative count");
    if (P == 0) return CRYOIM_OK;
    if ((r = ensure_grid(c))) return r;
    const int B = c->batch, nx = c->p.fftsize;
    const long nn = (long)nx * nx;
    if ((r = ensure_batch(c, B))) return r;
    const long per = (long)c->nom * (2 * c->nph + 1) * (c->nth + 1);
    if (pr_array && (r = c->prbuf.ensure((size_t)B * per))) return r;
    // CTF cache of ort_globesearch.f90:60-66
    std::vector<int> src(P);
    {
        int id0 = -100, cur = -1;
        for (int i = 0; i < P; ++i) {
            if (parts[i].img_id != id0) { cur = i; id0 = parts[i].img_id; }
            src[i] = cur;
        }
    }
    std::vector<float> hpar(8 * B);
    std::vector<unsigned long long> hbest(B);
    for (int b0 = 0; b0 < P; b0 += B) {
        const int nb = std::min(B, P - b0);
        const float* d_src;
        if (on_device) {
            d_src = imgs + b0 * nn;
        } else {
            CK(cudaMemcpyAsync(c->imgs.p, imgs + b0 * nn, sizeof(float) * nb * nn,
                               cudaMemcpyHostToDevice, c->stream));
            d_src = c->imgs.p;
        }
        std::fill(hpar.begin(), hpar.end(), 0.0f);
        for (int i = 0; i < nb; ++i) {
            const cryoim_particle& q = parts[b0 + i];
            const cryoim_particle& s = parts[src[b0 + i]];
            hpar[i] = q.x; hpar[B + i] = q.y; hpar[2 * B + i] = q.x; hpar[3 * B + i] = q.y;
            hpar[4 * B + 3 * i] = s.df1; hpar[4 * B + 3 * i + 1] = s.df2; hpar[4 * B + 3 * i + 2] = s.astigang;
        }
        // ort_globesearch.f90:50 masks unconditionally
        if ((r = transform_batch(c, d_src, nb, B, hpar, 1, 0, true))) return r;
        ParView pv = par_view(c, B);
        const float* ctfp = nullptr;
        const float* tfc = c->tfcut0.p;
        long tfs = 0;
        if (c->p.apply_ctf) {
            launch_ctf_band(nb, c->bd, pv.dfs, c->p.apix, c->p.vol, c->p.cs, c->p.ampwg, c->ctf.p,
                            c->stream);
            launch_tmpl_fcut(c->tband.p, c->T, c->ctf.p, nb, c->bd, c->tfcut.p, c->stream);
            CK(cudaGetLastError());
            ctfp = c->ctf.p;
            tfc = c->tfcut.p;
            tfs = (long)c->T * c->bd.nr;
        }
        for (int i = 0; i < nb; ++i) hbest[i] = key_of(1000.0f, 0u);
        CK(cudaMemcpyAsync(c->best.p, hbest.data(), sizeof(unsigned long long) * nb,
                           cudaMemcpyHostToDevice, c->stream));
        if (pr_array) {
            std::vector<float> init((size_t)nb * per, 1000.0f);
            CK(cudaMemcpyAsync(c->prbuf.p, init.data(), sizeof(float) * init.size(),
                               cudaMemcpyHostToDevice, c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
        if (c->V > 0) {
            PrOmegaArgs a{};
            a.band = c->band.p; a.fcut0 = c->fcut0.p; a.tband = c->tband.p;
            a.tfcut = tfc; a.tfcut_pstride = tfs; a.ctf = ctfp; a.alpha = c->alpha.p;
            a.views = c->d_views.p; a.V = c->V; a.T = c->T; a.nomega = c->nom;
            a.step = c->p.searchstep; a.bd = c->bd; a.best = c->best.p;
            a.pr_array = pr_array ? c->prbuf.p : nullptr; a.per = per;
            if (c->prof) CK(cudaEventRecord(c->pe0, c->stream));
            CK(launch_pr_omega(a, nb, c->stream));
            if (c->prof) CK(cudaEventRecord(c->pe1, c->stream));
        }
        CK(cudaMemcpyAsync(hbest.data(), c->best.p, sizeof(unsigned long long) * nb,
                           cudaMemcpyDeviceToHost, c->stream));
        if (pr_array)
            CK(cudaMemcpyAsync(pr_array + (long)b0 * per, c->prbuf.p, sizeof(float) * nb * per,
                               cudaMemcpyDeviceToHost, c->stream));
        if ((r = check_flag(c))) return r;
        if (c->prof && c->V > 0) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, c->pe0, c->pe1));
            c->prof_ms += ms;
            c->prof_launches += 1;
        }
        for (int i = 0; i < nb; ++i) {
            cryoim_particle& q = parts[b0 + i];
            unsigned idx = (unsigned)(hbest[i] & 0xffffffffu);
            unsigned bits = (unsigned)(hbest[i] >> 32);
            float pr;
            std::memcpy(&pr, &bits, 4);
            int iom = (int)(idx % c->nom);
            int iph = (int)((idx / c->nom) % (2 * c->nph + 1));
            int it = (int)(idx / ((unsigned)c->nom * (2 * c->nph + 1)));
            // ort_globesearch.f90:102-126
            q.theta0 = q.theta; q.phi0 = q.phi; q.omega0 = q.omega; q.x0 = q.x; q.y0 = q.y;
            q.pr0 = q.pr;
            q.theta = 69.0f + c->p.searchstep * (float)it;
            q.phi = c->p.searchstep * (float)(iph - c->nph);
            q.omega = c->p.searchstep * (float)iom;
            q.pr = pr;
            q.dtheta = q.theta - q.theta0; q.dphi = q.phi - q.phi0; q.domega = q.omega - q.omega0;
            q.dx = q.x - q.x0; q.dy = q.y - q.y0; q.dpr = q.pr - q.pr0;
        }
    }
    return CRYOIM_OK;
}

int refine_impl(Ctx* c, const float* imgs, bool on_device, cryoim_particle* parts, int P) {
    int r = check_ready(c, true);
    if (r) return r;
    if (!imgs || !parts || P < 0) return fail(CRYOIM_ERR_ARG, "null input or negative count");
    if (P == 0) return CRYOIM_OK;
    const int B = c->batch, nx = c->p.fftsize, T = c->T;
    const long nn = (long)nx * nx;
    if ((r = ensure_batch(c, B))) return r;
    if ((r = c->state.ensure((size_t)B * 6))) return r;
    if ((r = c->cand.ensure((size_t)B * 55))) return r;
    if ((r = c->rpr.ensure((size_t)B * 11))) return r;
    if ((r = c->ralpha.ensure((size_t)B * 11 * T * 60))) return r;
    std::vector<float> hpar(8 * B), hstate(6 * B);
    for (int b0 = 0; b0 < P; b0 += B) {
        const int nb = std::min(B, P - b0);
        const float* d_src;
        if (on_device) {
            d_src = imgs + b0 * nn;
        } else {
            CK(cudaMemcpyAsync(c->imgs.p, imgs + b0 * nn, sizeof(float) * nb * nn,
                               cudaMemcpyHostToDevice, c->stream));
            d_src = c->imgs.p;
        }
        std::fill(hpar.begin(), hpar.end(), 0.0f);
        for (int i = 0; i < nb; ++i) {
            const cryoim_particle& q = parts[b0 + i];
            hpar[i] = q.x; hpar[B + i] = q.y;
            // ort_refinement.f90:61-67: CTF per particle (no imgID cache)
            hpar[4 * B + 3 * i] = q.df1; hpar[4 * B + 3 * i + 1] = q.df2; hpar[4 * B + 3 * i + 2] = q.astigang;
            hstate[6 * i] = q.theta; hstate[6 * i + 1] = q.phi; hstate[6 * i + 2] = q.omega;
            hstate[6 * i + 3] = q.x; hstate[6 * i + 4] = q.y; hstate[6 * i + 5] = q.pr;
        }
        // ort_refinement.f90:46-54: no origin shift at this point
        if ((r = transform_batch(c, d_src, nb, B, hpar, c->p.use_imgmask, 0, false))) return r;
        ParView pv = par_view(c, B);
        const float* ctfp = nullptr;
        const float* tfc = c->tfcut0.p;
        long tfs = 0;
        if (c->p.apply_ctf) {
            launch_ctf_band(nb, c->bd, pv.dfs, c->p.apix, c->p.vol, c->p.cs, c->p.ampwg, c->ctf.p,
                            c->stream);
            launch_tmpl_fcut(c->tband.p, T, c->ctf.p, nb, c->bd, c->tfcut.p, c->stream);
            ctfp = c->ctf.p;
            tfc = c->tfcut.p;
            tfs = (long)T * c->bd.nr;
        }
        CK(cudaMemcpyAsync(c->state.p, hstate.data(), sizeof(float) * 6 * nb, cudaMemcpyHostToDevice,
                           c->stream));
        float fac = 1.0f;
        for (int cyc = 1; cyc <= c->p.ncycle; ++cyc) {
            float dang = c->p.delta_angle * fac, dtran = c->p.delta_trans * fac;
            fac = fac * 0.8f;
            launch_refine_candidates(c->state.p, nb, dang, dtran, c->ops.p, c->cand.p, c->stream);
            launch_refine_alpha(c->cand.p, nb, c->tort.p, T, c->ops.p, c->ralpha.p, c->stream);
            PrSingleArgs a{};
            a.band = c->band.p; a.fcut0 = c->fcut0.p; a.tband = c->tband.p; a.tfcut = tfc;
            a.tfcut_pstride = tfs; a.ctf = ctfp; a.cand = c->cand.p; a.alpha = c->ralpha.p;
            a.T = T; a.bd = c->bd; a.pr = c->rpr.p;
            CK(launch_pr_single(a, nb, c->stream));
            launch_refine_select(c->cand.p, c->rpr.p, nb, c->state.p, c->stream);
            CK(cudaGetLastError());
        }
        CK(cudaMemcpyAsync(hstate.data(), c->state.p, sizeof(float) * 6 * nb, cudaMemcpyDeviceToHost,
                           c->stream));
        if ((r = check_flag(c))) return r;
        for (int i = 0; i < nb; ++i) {
            cryoim_particle& q = parts[b0 + i];
            const float* st = &hstate[6 * i];
            q.theta0 = q.theta; q.phi0 = q.phi; q.omega0 = q.omega; q.x0 = q.x; q.y0 = q.y;
            q.pr0 = q.pr;
            q.theta = st[0]; q.phi = st[1]; q.omega = st[2]; q.x = st[3]; q.y = st[4]; q.pr = st[5];
            q.dtheta = q.theta - q.theta0; q.dphi = q.phi - q.phi0; q.domega = q.omega - q.omega0;
            q.dx = q.x - q.x0; q.dy = q.y - q.y0; q.dpr = q.pr - q.pr0;
        }
    }
    return CRYOIM_OK;
}

int rec_insert_impl(Ctx* c, const float* imgs, bool on_device, const cryoim_particle* parts, int P,
                    int32_t* used) {
    int r = check_ready(c, false);
    if (r) return r;
    if (!c->rec_active) return fail(CRYOIM_ERR_STATE, "cryoim_rec_begin has not been called");
    if (!imgs || !parts || P < 0) return fail(CRYOIM_ERR_ARG, "null input or negative count");
    const int B = c->batch, nx = c->p.fftsize;
    const long nn = (long)nx * nx;
    if ((r = ensure_batch(c, B))) return r;
    // reconstruct_substep.f90:22 sets boundX = FFTsize/4; reconstruct_half.f90:17 keeps it
    const float boundx = c->rec_kind == REC_SUBSTEP ? (float)nx / 4.0f : c->p.boundx;
    const Angles an = host_angles();
    std::vector<float> hpar(8 * B), hrot(9 * B);
    std::vector<int> hsel(B);
    int nused = 0;
    for (int b0 = 0; b0 < P; b0 += B) {
        const int nb = std::min(B, P - b0);
        std::fill(hpar.begin(), hpar.end(), 0.0f);
        for (int i = 0; i < nb; ++i) {
            const cryoim_particle& q = parts[b0 + i];
            if (!c->rec_have_first) {  // reconstruct.f90:92 masks every image at particle(first)'s origin
                c->rec_ox = q.x; c->rec_oy = q.y; c->rec_have_first = true;
            }
            int s = (q.pr <= c->p.pr_threshold && std::fabs(q.x) <= boundx && std::fabs(q.y) <= boundx);
            hsel[i] = s;
            hpar[i] = c->rec_ox; hpar[B + i] = c->rec_oy;
            hpar[2 * B + i] = q.x; hpar[3 * B + i] = q.y;
            if (s) {
                ++nused;
                // reconstruct.f90:80-91: CTF per particle for imgstck, else cached per imgID
                if (c->p.imgstck || q.img_id != c->rec_img_id0) {
                    c->rec_src_df[0] = q.df1; c->rec_src_df[1] = q.df2; c->rec_src_df[2] = q.astigang;
                    if (!c->p.imgstck) c->rec_img_id0 = q.img_id;
                }
                hpar[4 * B + 3 * i] = c->rec_src_df[0];
                hpar[4 * B + 3 * i + 1] = c->rec_src_df[1];
                hpar[4 * B + 3 * i + 2] = c->rec_src_df[2];
                euler_mat(q.theta, q.phi, q.omega, an.deg2rad, &hrot[9 * i]);
            }
        }
        const float* d_src;
        if (on_device) {
            d_src = imgs + b0 * nn;
        } else {
            CK(cudaMemcpyAsync(c->imgs.p, imgs + b0 * nn, sizeof(float) * nb * nn,
                               cudaMemcpyHostToDevice, c->stream));
            d_src = c->imgs.p;
        }
        if ((r = transform_batch(c, d_src, nb, B, hpar, c->p.use_imgmask, 1, true))) return r;
        ParView pv = par_view(c, B);
        const float* ctfp = nullptr;
        if (c->p.apply_ctf || c->p.imgstck) {
            launch_ctf_band(nb, c->bd, pv.dfs, c->p.apix, c->p.vol, c->p.cs, c->p.ampwg, c->ctf.p,
                            c->stream);
            ctfp = c->ctf.p;
        }
        CK(cudaMemcpyAsync(c->rot.p, hrot.data(), sizeof(float) * 9 * nb, cudaMemcpyHostToDevice,
                           c->stream));
        CK(cudaMemcpyAsync(c->sel.p, hsel.data(), sizeof(int) * nb, cudaMemcpyHostToDevice,
                           c->stream));
        InsertArgs a{};
        a.band = c->band.p; a.ctf = ctfp; a.rot = c->rot.p; a.ops = c->ops.p;
        a.samples = c->samples.p; a.nsamples = c->nsamples; a.nsym = c->p.nsym; a.sel = c->sel.p;
        a.off_xy = c->rec_off_xy; a.off_z = c->rec_off_z; a.base_xy = c->rec_base_xy;
        a.base_z = c->rec_base_z; a.bd = c->bd; a.acc = c->acc.p;
        if (c->nsamples > 0) CK(launch_insert(a, nb, c->stream));
        if ((r = check_flag(c))) return r;
    }
    c->rec_used += nused;
    if (used) *used = nused;
    return CRYOIM_OK;
}

// ---------------------------------------------------------------------------
// contraction form
// ---------------------------------------------------------------------------

// Half-plane band samples (hx > 0, or hx == 0 and ky > 0) with minR <= |h| <= maxR.
int ensure_samples(Ctx* c) {
    if (c->cS > 0) return CRYOIM_OK;
    const int R = c->p.max_r, r0 = c->p.min_r;
    std::vector<int2> s;
    for (int ky = -R; ky <= R; ++ky)
        for (int hx = 0; hx <= R; ++hx) {
            if (hx == 0 && ky <= 0) continue;
            const int d2 = hx * hx + ky * ky;
            if (d2 >= r0 * r0 && d2 <= R * R) s.push_back(make_int2(hx, ky));
        }
    int r;
    if ((r = c->csamples.ensure(s.size()))) return r;
    CK(cudaMemcpyAsync(c->csamples.p, s.data(), sizeof(int2) * s.size(), cudaMemcpyHostToDevice, c->stream));
    c->cS = (int)s.size();
    c->cKpad = (2 * c->cS + 63) / 64 * 64;
    c->cKpad8 = (2 * c->cS + 127) / 128 * 128;
    return CRYOIM_OK;
}

int ensure_bmat(Ctx* c) {
    int r;
    if ((r = ensure_grid(c))) return r;
    if ((r = ensure_samples(c))) return r;
    const long n = (long)c->V * c->nom;
    if (c->bmat_ready && c->n_orient == n) return CRYOIM_OK;
    if ((r = c->bmat.ensure((size_t)n * c->cKpad))) return r;
    std::vector<float> v2(2 * (size_t)c->V);
    for (int v = 0; v < c->V; ++v) { v2[2 * v] = c->views[4 * v]; v2[2 * v + 1] = c->views[4 * v + 1]; }
    DBuf<float> dv;
    if ((r = dv.ensure(v2.size() + 2))) return r;
    CK(cudaMemcpyAsync(dv.p, v2.data(), sizeof(float) * v2.size(), cudaMemcpyHostToDevice, c->stream));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    cudaError_t te = make_cube_texture(c->mapcube.p, c->cube_r, c->stream, &arr, &tex);
    if (te == cudaSuccess) te = cudaEventRecord(e0, c->stream);
    if (te == cudaSuccess)
        te = launch_slice_bf16(tex, c->cube_r, c->csamples.p, c->cS, c->cKpad, dv.p, c->nom, c->p.searchstep, 0,
                               n, c->bmat.p, c->stream, c->mapcube.p, c->interp_sigma, (float)c->ovs);
    if (te == cudaSuccess) te = cudaEventRecord(e1, c->stream);
    if (te == cudaSuccess) te = cudaEventSynchronize(e1);
    free_cube_texture(arr, tex);
    if (te != cudaSuccess) return fail(CRYOIM_ERR_CUDA, "section build: %s", cudaGetErrorString(te));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->bmat_ms = ms;
    c->n_orient = n;
    c->bmat_ready = true;
    return CRYOIM_OK;
}

// The coarse level of the proposal form: views at twice the search step, the band
// minR <= |h| <= maxR/2, BF16 unit-norm sections (built as the fine ones), origins at
// twice the origin step over the same range.
int ensure_coarse(Ctx* c, float omax, float ostep) {
    int r;
    if ((r = ensure_grid(c))) return r;
    if (!c->bmat_c_ready) {
        build_view_grid(2.0f * c->p.searchstep, &c->cgrid);
        const ViewGrid& g = c->cgrid;
        if (g.nom < 1 || g.V < 1) return fail(CRYOIM_ERR_SIZE, "coarse grid is empty");
        const int R = c->p.max_r, r0 = c->p.min_r, Rc = std::max(r0 + 1, R / 2);
        std::vector<int2> s;
        for (int ky = -Rc; ky <= Rc; ++ky)
            for (int hx = 0; hx <= Rc; ++hx) {
                if (hx == 0 && ky <= 0) continue;
                const int d2 = hx * hx + ky * ky;
                if (d2 >= r0 * r0 && d2 <= Rc * Rc) s.push_back(make_int2(hx, ky));
            }
        if ((r = c->csamples_c.ensure(s.size()))) return r;
        CK(cudaMemcpyAsync(c->csamples_c.p, s.data(), sizeof(int2) * s.size(), cudaMemcpyHostToDevice, c->stream));
        c->cS_c = (int)s.size();
        c->cKpad_c = (2 * c->cS_c + 63) / 64 * 64;
        const long n = (long)g.V * g.nom;
        if ((r = c->bmat_c.ensure((size_t)n * c->cKpad_c))) return r;
        std::vector<float> v2(2 * (size_t)g.V);
        for (int v = 0; v < g.V; ++v) { v2[2 * v] = g.views[4 * v]; v2[2 * v + 1] = g.views[4 * v + 1]; }
        DBuf<float> dv;
        if ((r = dv.ensure(v2.size()))) return r;
        CK(cudaMemcpyAsync(dv.p, v2.data(), sizeof(float) * v2.size(), cudaMemcpyHostToDevice, c->stream));
        cudaArray_t arr = nullptr;
        cudaTextureObject_t tex = 0;
        cudaError_t te = make_cube_texture(c->mapcube.p, c->cube_r, c->stream, &arr, &tex);
        if (te == cudaSuccess)
            te = launch_slice_bf16(tex, c->cube_r, c->csamples_c.p, c->cS_c, c->cKpad_c, dv.p, g.nom, g.step, 0, n,
                                   c->bmat_c.p, c->stream, c->mapcube.p, c->interp_sigma, (float)c->ovs);
        if (te == cudaSuccess) te = cudaStreamSynchronize(c->stream);
        free_cube_texture(arr, tex);
        if (te != cudaSuccess) return fail(CRYOIM_ERR_CUDA, "coarse sections: %s", cudaGetErrorString(te));
        c->n_orient_c = n;
        c->bmat_c_ready = true;
    }
    if (omax != c->orig_max_c || 2.0f * ostep != c->orig_step_c) {
        const float st = 2.0f * ostep;
        const int n1 = (int)(2.0f * omax / st + 0.5f) + 1;
        std::vector<float> og;
        for (int iy = 0; iy < n1; ++iy)
            for (int ix = 0; ix < n1; ++ix) {
                og.push_back(-omax + st * (float)ix);
                og.push_back(-omax + st * (float)iy);
            }
        if ((r = c->corigins_c.ensure(og.size()))) return r;
        CK(cudaMemcpyAsync(c->corigins_c.p, og.data(), sizeof(float) * og.size(), cudaMemcpyHostToDevice,
                           c->stream));
        c->n_origin_c = n1 * n1;
        c->orig_max_c = omax;
        c->orig_step_c = st;
    }
    return CRYOIM_OK;
}

// The fine-grid orientations within nbf steps (theta, phi, omega) of each seed (fine
// grid theta index, signed phi index, omega index), each once, in the order first
// reached: lists[i] for seeds[i].  One byte per grid orientation marks what a list
// already holds (cleared after each list), so the cost is linear in the seeds.
void expand_seeds(Ctx* c, const std::vector<std::vector<int3>>& seeds, int nbf,
                  std::vector<std::vector<int>>& lists) {
    const int span = 2 * c->nph + 1;
    std::vector<uint8_t>& mark = c->list_mark;
    if (mark.size() < (size_t)c->n_orient) mark.assign((size_t)c->n_orient, 0);
    lists.assign(seeds.size(), std::vector<int>());
    for (size_t i = 0; i < seeds.size(); ++i) {
        std::vector<int>& lst = lists[i];
        lst.reserve(seeds[i].size() * (2 * nbf + 1) * (2 * nbf + 1) * (2 * nbf + 1));
        for (const int3& sd : seeds[i])
            for (int dt = -nbf; dt <= nbf; ++dt)
                for (int dp = -nbf; dp <= nbf; ++dp) {
                    const int it2 = sd.x + dt, ips2 = sd.y + dp;
                    if (it2 < 0 || it2 > c->nth || ips2 < -c->nph || ips2 > c->nph) continue;
                    const int v2 = c->slot_view[(size_t)it2 * span + ips2 + c->nph];
                    if (v2 < 0) continue;
                    for (int dw = -nbf; dw <= nbf; ++dw) {
                        const int n = v2 * c->nom + ((sd.z + dw) % c->nom + c->nom) % c->nom;
                        if (!mark[n]) {
                            mark[n] = 1;
                            lst.push_back(n);
                        }
                    }
                }
        for (int n : lst) mark[n] = 0;
        if (lst.empty()) lst.push_back(0);
    }
}

// Coarse level for nb prepared particles (c->band, ctfp): the best kc distinct coarse
// orientations of each, mapped onto the fine grid (twice the coarse indices) with their
// fine neighbours within nbf steps in theta, phi and omega -> lists[i].
int coarse_lists(Ctx* c, int nb, const float* ctfp, int kc, int nbf, std::vector<std::vector<int>>& lists) {
    const ViewGrid& g = c->cgrid;
    const int Oc = c->n_origin_c;
    const int ntc = (int)((c->n_orient_c + gemm_tile_n() - 1) / gemm_tile_n());
    int r;
    if ((r = c->amat_c.ensure((size_t)nb * Oc * c->cKpad_c)) || (r = c->topv_c.ensure((size_t)nb * Oc * ntc)) ||
        (r = c->topi_c.ensure((size_t)nb * Oc * ntc)) || (r = c->tilev_c.ensure((size_t)nb * ntc)) ||
        (r = c->tileo_c.ensure((size_t)nb * ntc)) || (r = c->tileorig_c.ensure((size_t)nb * ntc)) ||
        (r = c->kor_c.ensure((size_t)nb * kc)) || (r = c->korig_c.ensure((size_t)nb * kc)) ||
        (r = c->kcc_c.ensure((size_t)nb * kc)) || (r = c->pnorm_c.ensure(nb)))
        return r;
    launch_particle_norm(c->band.p, ctfp, c->bd, c->csamples_c.p, c->cS_c, nb, c->pnorm_c.p, c->stream);
    launch_build_a(c->band.p, ctfp, c->bd, c->csamples_c.p, c->cS_c, c->cKpad_c, c->corigins_c.p, Oc, c->pnorm_c.p,
                   nb, c->amat_c.p, c->stream);
    GemmArgmaxArgs ga{};
    ga.b_mode = 1;  // the coarse bank's rows are pre-swizzled
    ga.topv = c->topv_c.p;
    ga.topi = c->topi_c.p;
    ga.err = c->gerr.p;
    CK(cudaMemsetAsync(c->gerr.p, 0, sizeof(int), c->stream));
    CK(launch_gemm_argmax(c->amat_c.p, c->bmat_c.p, nb * Oc, (int)c->n_orient_c, c->cKpad_c, false, ga, c->num_sms,
                          c->stream));
    launch_select_topk(c->topv_c.p, c->topi_c.p, Oc, ntc, kc, nb, c->tilev_c.p, c->tileo_c.p, c->tileorig_c.p,
                       c->kor_c.p, c->korig_c.p, c->kcc_c.p, c->stream);
    CK(cudaGetLastError());
    std::vector<int> kor((size_t)nb * kc);
    int gerr = 0;
    CK(cudaMemcpyAsync(&gerr, c->gerr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(kor.data(), c->kor_c.p, sizeof(int) * nb * kc, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (gerr) return fail(CRYOIM_ERR_CUDA, "coarse contraction wait timed out");
    const int span_c = 2 * g.nph + 1;
    std::vector<std::vector<int3>> seeds(nb);
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < kc; ++j) {
            const int n = kor[(size_t)i * kc + j];
            if (n < 0) continue;
            const int vc = n / g.nom, ioc = n % g.nom, slot = g.view_slot[vc];
            seeds[i].push_back(make_int3(2 * (slot / span_c), 2 * (slot % span_c - g.nph), 2 * ioc));
        }
    expand_seeds(c, seeds, nbf, lists);
    return CRYOIM_OK;
}

// ---- learned orientation proposer: host side -------------------------------------
constexpr int LP_CIN[4] = {1, LP_C1, LP_C2, LP_C3}, LP_COUT[4] = {LP_C1, LP_C2, LP_C3, LP_C4};

int ensure_cgrid(Ctx* c) {
    if (c->cgrid.V > 0 && c->cgrid.step == 2.0f * c->p.searchstep) return CRYOIM_OK;
    build_view_grid(2.0f * c->p.searchstep, &c->cgrid);
    if (c->cgrid.V < 1) return fail(CRYOIM_ERR_SIZE, "coarse view grid is empty");
    return CRYOIM_OK;
}

// parameter layout and view vectors for V views; weights not initialised
int learn_layout(Ctx* c, int V) {
    LearnModel& L = c->lm;
    long off = 0;
    for (int l = 0; l < 4; ++l) {
        L.oW[l] = off;
        off += (long)LP_COUT[l] * LP_CIN[l] * 9;
        L.ob[l] = off;
        off += LP_COUT[l];
    }
    L.oW[4] = off;
    off += (long)LP_CM * LP_MIXK;
    L.ob[4] = off;
    off += LP_CM;
    L.oT = off;
    off += (long)V * LP_CM * LP_NT;
    L.nparam = off;
    L.V = V;
    int r;
    if ((r = L.w.ensure(off)) || (r = L.gr.ensure(off)) || (r = L.m.ensure(off)) || (r = L.v.ensure(off)) ||
        (r = L.vview.ensure(3 * (size_t)V)) || (r = L.wflip.ensure((size_t)LP_C2 * LP_C3 * 9)) ||
        (r = L.cerr.ensure(1)))
        return r;
    CK(cudaMemsetAsync(L.cerr.p, 0, sizeof(int), c->stream));
    std::vector<float> vv(3 * (size_t)V);
    const float d2r = host_angles().deg2rad;
    for (int i = 0; i < V; ++i) {
        const float th = c->cgrid.views[4 * i] * d2r, ph = c->cgrid.views[4 * i + 1] * d2r;
        vv[3 * i] = sinf(th) * cosf(ph);
        vv[3 * i + 1] = sinf(th) * sinf(ph);
        vv[3 * i + 2] = cosf(th);
    }
    CK(cudaMemcpyAsync(L.vview.p, vv.data(), sizeof(float) * vv.size(), cudaMemcpyHostToDevice, c->stream));
    return CRYOIM_OK;
}

int learn_activations(Ctx* c, int B) {
    LearnModel& L = c->lm;
    if (B <= L.cap && L.V == L.capV) return CRYOIM_OK;
    B = std::max(B, L.cap);
    const size_t b = (size_t)B, P = LP_NT;
    int r;
    if ((r = L.feat.ensure(b * LP_NR * P)) || (r = L.a1.ensure(b * LP_C1 * LP_NR * P)) ||
        (r = L.a2.ensure(b * LP_C2 * LP_NR * P)) || (r = L.p2.ensure(b * LP_C2 * (LP_NR / 2) * P)) ||
        (r = L.a3.ensure(b * LP_C3 * (LP_NR / 2) * P)) || (r = L.p3.ensure(b * LP_C3 * (LP_NR / 4) * P)) ||
        (r = L.a4.ensure(b * LP_C4 * (LP_NR / 4) * P)) || (r = L.p4.ensure(b * LP_MIXK * P)) ||
        (r = L.g.ensure(b * LP_CM * P)) || (r = L.sc.ensure(b * L.V * P)) || (r = L.dsc.ensure(b * L.V * P)) ||
        (r = L.dg.ensure(b * LP_CM * P)) || (r = L.dp4.ensure(b * LP_MIXK * P)) ||
        (r = L.da4.ensure(b * LP_C4 * (LP_NR / 4) * P)) || (r = L.dp3.ensure(b * LP_C3 * (LP_NR / 4) * P)) ||
        (r = L.da3.ensure(b * LP_C3 * (LP_NR / 2) * P)) || (r = L.dp2.ensure(b * LP_C2 * (LP_NR / 2) * P)) ||
        (r = L.da2.ensure(b * LP_C2 * LP_NR * P)) || (r = L.da1.ensure(b * LP_C1 * LP_NR * P)) ||
        (r = L.loss.ensure(b)) || (r = L.truth.ensure(4 * b)) || (r = L.cell.ensure(b * 64)) ||
        (r = L.cellv.ensure(b * 64)) || (r = L.hscr.ensure((size_t)lp_head_scratch(B, L.V))))
        return r;
    L.cap = B;
    L.capV = L.V;
    return CRYOIM_OK;
}

// The proposer's 3x3 convolutions: TF32 on the tensor cores (conv_tc.cu, the default) or
// FP32 on the CUDA cores (learn.cu).
cudaError_t lp_conv(Ctx* c, const float* in, int B, int Cin, int H, const float* W, const float* bias, int Cout,
                    bool relu, float* out) {
    LearnModel& L = c->lm;
    if (L.conv_tc) return launch_lp_conv3_tc(in, B, Cin, H, W, bias, Cout, relu, out, L.cerr.p, c->stream);
    return launch_lp_conv3(in, B, Cin, H, W, bias, Cout, relu, out, c->stream);
}
cudaError_t lp_wgrad(Ctx* c, const float* in, const float* dpre, int B, int Cin, int H, int Cout, float* dW,
                     float* db) {
    LearnModel& L = c->lm;
    if (L.conv_tc) return launch_lp_conv3_wgrad_tc(in, dpre, B, Cin, H, Cout, dW, db, L.cerr.p, c->stream);
    return launch_lp_conv3_wgrad(in, dpre, B, Cin, H, Cout, dW, db, c->stream);
}
// After the stream has drained: did a tensor-core convolution give up waiting?
int learn_conv_status(Ctx* c) {
    LearnModel& L = c->lm;
    if (!L.cerr.p) return CRYOIM_OK;
    int e = 0;
    CK(cudaMemcpyAsync(&e, L.cerr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (e) return fail(CRYOIM_ERR_CUDA, "proposer convolution: tensor-core wait timed out");
    return CRYOIM_OK;
}

// scores L.sc [B][V][NT] of the features in L.feat
int learn_forward(Ctx* c, int B) {
    LearnModel& L = c->lm;
    const float* w = L.w.p;
    cudaStream_t st = c->stream;
    CK(lp_conv(c, L.feat.p, B, 1, LP_NR, w + L.oW[0], w + L.ob[0], LP_C1, true, L.a1.p));
    CK(lp_conv(c, L.a1.p, B, LP_C1, LP_NR, w + L.oW[1], w + L.ob[1], LP_C2, true, L.a2.p));
    launch_lp_pool(L.a2.p, B, LP_C2, LP_NR / 2, L.p2.p, st);
    CK(lp_conv(c, L.p2.p, B, LP_C2, LP_NR / 2, w + L.oW[2], w + L.ob[2], LP_C3, true, L.a3.p));
    launch_lp_pool(L.a3.p, B, LP_C3, LP_NR / 4, L.p3.p, st);
    CK(lp_conv(c, L.p3.p, B, LP_C3, LP_NR / 4, w + L.oW[3], w + L.ob[3], LP_C4, true, L.a4.p));
    launch_lp_pool(L.a4.p, B, LP_C4, LP_NR / 8, L.p4.p, st);
    launch_lp_mix(L.p4.p, B, w + L.oW[4], w + L.ob[4], L.g.p, st);
    CK(launch_lp_head(L.g.p, w + L.oT, B, L.V, L.sc.p, L.hscr.p, st));
    return CRYOIM_OK;
}

// loss (L.loss [B]) and parameter gradients (L.gr) of the last forward, targets in L.truth
int learn_backward(Ctx* c, int B) {
    LearnModel& L = c->lm;
    const float* w = L.w.p;
    float* gr = L.gr.p;
    cudaStream_t st = c->stream;
    const long nt = LP_NT;
    CK(cudaMemsetAsync(gr, 0, sizeof(float) * L.nparam, st));
    launch_lp_loss(L.sc.p, B, L.V, L.vview.p, L.truth.p, 2.0f * c->p.searchstep, 1.0f, L.dsc.p, L.loss.p, st);
    launch_lp_head_grad(L.g.p, w + L.oT, L.dsc.p, B, L.V, L.dg.p, gr + L.oT, L.hscr.p, st);
    launch_lp_mix_grad(L.p4.p, L.dg.p, B, w + L.oW[4], L.dp4.p, gr + L.oW[4], gr + L.ob[4], st);
    // layer 4
    launch_lp_pool_grad(L.dp4.p, B, LP_C4, LP_NR / 8, L.a4.p, L.da4.p, st);
    CK(lp_wgrad(c, L.p3.p, L.da4.p, B, LP_C3, LP_NR / 4, LP_C4, gr + L.oW[3], gr + L.ob[3]));
    launch_lp_flip(w + L.oW[3], LP_C4, LP_C3, L.wflip.p, st);
    CK(lp_conv(c, L.da4.p, B, LP_C4, LP_NR / 4, L.wflip.p, nullptr, LP_C3, false, L.dp3.p));
    // layer 3
    launch_lp_pool_grad(L.dp3.p, B, LP_C3, LP_NR / 4, L.a3.p, L.da3.p, st);
    CK(lp_wgrad(c, L.p2.p, L.da3.p, B, LP_C2, LP_NR / 2, LP_C3, gr + L.oW[2], gr + L.ob[2]));
    launch_lp_flip(w + L.oW[2], LP_C3, LP_C2, L.wflip.p, st);
    CK(lp_conv(c, L.da3.p, B, LP_C3, LP_NR / 2, L.wflip.p, nullptr, LP_C2, false, L.dp2.p));
    // layer 2
    launch_lp_pool_grad(L.dp2.p, B, LP_C2, LP_NR / 2, L.a2.p, L.da2.p, st);
    CK(lp_wgrad(c, L.a1.p, L.da2.p, B, LP_C1, LP_NR, LP_C2, gr + L.oW[1], gr + L.ob[1]));
    launch_lp_flip(w + L.oW[1], LP_C2, LP_C1, L.wflip.p, st);
    CK(lp_conv(c, L.da2.p, B, LP_C2, LP_NR, L.wflip.p, nullptr, LP_C1, false, L.da1.p));
    // layer 1
    launch_lp_relu_grad(L.a1.p, L.da1.p, (long)B * LP_C1 * LP_NR * nt, L.da1.p, st);
    CK(lp_wgrad(c, L.feat.p, L.da1.p, B, 1, LP_NR, LP_C1, gr + L.oW[0], gr + L.ob[0]));
    return CRYOIM_OK;
}

// Haar-uniform rotation (unit quaternion) as ZYZ Euler angles in degrees
template <class RNG> void random_euler(RNG& rng, float* e) {
    std::normal_distribution<double> nd(0.0, 1.0);
    double q[4], s = 0.0;
    for (double& x : q) { x = nd(rng); s += x * x; }
    s = 1.0 / std::sqrt(s);
    const double w = q[0] * s, x = q[1] * s, y = q[2] * s, z = q[3] * s;
    const double r02 = 2 * (x * z + y * w), r12 = 2 * (y * z - x * w), r20 = 2 * (x * z - y * w),
                 r21 = 2 * (y * z + x * w), r22 = 1 - 2 * (x * x + y * y);
    const double r2d = 180.0 / 3.14159265358979323846;
    e[0] = (float)(std::acos(std::min(1.0, std::max(-1.0, r22))) * r2d);
    e[1] = (float)(std::atan2(r12, r02) * r2d);
    e[2] = (float)(std::atan2(r21, -r20) * r2d);
}

// Renders B particles into img (device, B x nx^2) from the band cube texture: Fourier
// slice at eul, CTF (if ctf) and origin shift from par, inverse transform, white noise
// at snr (signal variance inside the 0.4 nx disc / noise variance; 0: none).
int learn_render(Ctx* c, cudaTextureObject_t tex, const float* deul, const float* dpar, int B, float snr,
                 unsigned long long seed, bool ctf, float* img, float2* ft, float* var) {
    const int nx = c->p.fftsize;
    launch_lp_render(tex, 2 * c->p.max_r + 3, c->p.max_r + 1, 2, nx, deul, dpar, B, c->p.apix,
                     ctf ? c->p.vol : -1.0f, c->p.cs, c->p.ampwg, host_angles().deg2rad, ft, c->stream);
    cufftHandle h;
    int r;
    if ((r = plan2d(c, B, &h))) return r;
    CKF(cufftExecC2C(h, (cufftComplex*)ft, (cufftComplex*)ft, CUFFT_INVERSE));
    launch_lp_cplx_to_real(ft, nx, B, img, var, c->stream);
    if (snr > 0.0f) launch_lp_add_noise(img, nx, B, var, snr, seed, c->stream);
    CK(cudaGetLastError());
    return CRYOIM_OK;
}

// the band cube as a texture for the lifetime of a scope
struct CubeTexture {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    ~CubeTexture() { if (arr || tex) free_cube_texture(arr, tex); }
};

// The renderer's band cube: the map padded to (2n)^3, its transform, frequencies up to
// 2 (maxR + 1) + 1 of the padded grid (maxR + 1 of the map's, twice oversampled), as a
// texture.
int render_cube(Ctx* c, const float* map3d, CubeTexture* ct) {
    const int n = c->p.fftsize, m = 2 * n, Rc = 2 * c->p.max_r + 3;
    const long m3 = (long)m * m * m, c3 = (long)(2 * Rc + 3) * (2 * Rc + 3) * (2 * Rc + 3);
    DBuf<float> dmap;
    DBuf<float2> work, cube;
    int r;
    if ((r = dmap.ensure((size_t)n * n * n)) || (r = work.ensure(m3)) || (r = cube.ensure(c3))) return r;
    CK(cudaMemcpyAsync(dmap.p, map3d, sizeof(float) * n * n * n, cudaMemcpyHostToDevice, c->stream));
    launch_lp_pad_checker(dmap.p, n, work.p, c->stream);
    CK(cudaGetLastError());
    cufftHandle h;
    CKF(cufftPlan3d(&h, m, m, m, CUFFT_C2C));
    cufftResult fr = cufftSetStream(h, c->stream);
    if (fr == CUFFT_SUCCESS) fr = cufftExecC2C(h, (cufftComplex*)work.p, (cufftComplex*)work.p, CUFFT_FORWARD);
    if (fr != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return fail(CRYOIM_ERR_CUDA, "padded 3D transform failed: cufft %d", (int)fr);
    }
    launch_map_band(work.p, m, Rc, cube.p, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cufftDestroy(h);
    if (e != cudaSuccess) return fail(CRYOIM_ERR_CUDA, "render cube: %s", cudaGetErrorString(e));
    CK(make_cube_texture(cube.p, Rc, c->stream, &ct->arr, &ct->tex));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

// mask at (x, y), transform, polar features of nb images on the device -> L.feat
int learn_features_dev(Ctx* c, const float* d_img, int nb, const float* ox, const float* oy,
                       bool keep_flag = false) {
    std::vector<float> hpar(8 * (size_t)nb, 0.0f);
    for (int i = 0; i < nb; ++i) { hpar[i] = ox[i]; hpar[nb + i] = oy[i]; }
    int r;
    if ((r = ensure_batch(c, nb))) return r;
    if ((r = transform_batch(c, d_img, nb, nb, hpar, 1, 0, false, keep_flag, false))) return r;
    launch_lp_features(c->band.p, c->bd, nb, c->lm.feat.p, c->stream);
    CK(cudaGetLastError());
    return CRYOIM_OK;
}

int learn_train_impl(Ctx* c, const float* map3d, const cryoim_learn_opts* o, float* stats) {
    int r = check_ready(c, false);
    if (r) return r;
    if (!map3d || !o) return fail(CRYOIM_ERR_ARG, "null input");
    if (o->batch < 8 || o->batch > 1024 || o->samples < o->batch || !(o->lr > 0) || o->snr < 0 ||
        o->df_max < o->df_min || o->origin_max < 0 || o->astig_max < 0)
        return fail(CRYOIM_ERR_ARG, "bad learn options");
    const auto t0 = std::chrono::steady_clock::now();
    if ((r = ensure_cgrid(c))) return r;
    LearnModel& L = c->lm;
    L.ready = false;
    const int V = c->cgrid.V, B = o->batch, nx = c->p.fftsize;
    const long nn = (long)nx * nx;
    if ((r = learn_layout(c, V)) || (r = learn_activations(c, B))) return r;
    // initial weights: He-normal convolutions, 1/sqrt(fan-in) mix, small templates
    std::mt19937_64 rng((uint64_t)o->seed * 0x9E3779B97F4A7C15ull + 12345u);
    {
        std::vector<float> hw(L.nparam, 0.0f);
        std::normal_distribution<float> nd(0.0f, 1.0f);
        for (int l = 0; l < 4; ++l) {
            const float sd = std::sqrt(2.0f / (9.0f * LP_CIN[l]));
            for (long q = 0; q < (long)LP_COUT[l] * LP_CIN[l] * 9; ++q) hw[L.oW[l] + q] = sd * nd(rng);
        }
        for (long q = 0; q < (long)LP_CM * LP_MIXK; ++q) hw[L.oW[4] + q] = nd(rng) / std::sqrt((float)LP_MIXK);
        for (long q = 0; q < (long)V * LP_CM * LP_NT; ++q) hw[L.oT + q] = 0.01f * nd(rng);
        CK(cudaMemcpyAsync(L.w.p, hw.data(), sizeof(float) * L.nparam, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemsetAsync(L.m.p, 0, sizeof(float) * L.nparam, c->stream));
        CK(cudaMemsetAsync(L.v.p, 0, sizeof(float) * L.nparam, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    L.steps = 0;
    CubeTexture ct;
    if ((r = render_cube(c, map3d, &ct))) return r;
    DBuf<float> img, deul, dpar, var;
    DBuf<float2> ft;
    if ((r = img.ensure((size_t)B * nn)) || (r = ft.ensure((size_t)B * nn)) || (r = deul.ensure(3 * (size_t)B)) ||
        (r = dpar.ensure(5 * (size_t)B)) || (r = var.ensure(B)))
        return r;
    // direction of the feature shift under an in-plane rotation: two clean projections
    // 30 degrees apart, features, circular correlation
    {
        const float e2[6] = {80.0f, 5.0f, 0.0f, 80.0f, 5.0f, 30.0f};
        const float p2[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        CK(cudaMemcpyAsync(deul.p, e2, sizeof(e2), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(dpar.p, p2, sizeof(p2), cudaMemcpyHostToDevice, c->stream));
        if ((r = learn_render(c, ct.tex, deul.p, dpar.p, 2, 0.0f, 0, false, img.p, ft.p, var.p))) return r;
        const float z2[2] = {0.0f, 0.0f};
        if ((r = learn_features_dev(c, img.p, 2, z2, z2))) return r;
        std::vector<float> f(2 * LP_NR * LP_NT);
        CK(cudaMemcpyAsync(f.data(), L.feat.p, sizeof(float) * f.size(), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        int best = 0;
        double bv = -1e300;
        for (int s = 0; s < LP_NT; ++s) {
            double acc = 0.0;
            for (int ir = 0; ir < LP_NR; ++ir)
                for (int t = 0; t < LP_NT; ++t)
                    acc += (double)f[ir * LP_NT + t] * f[LP_NR * LP_NT + ir * LP_NT + (t + s) % LP_NT];
            if (acc > bv) { bv = acc; best = s; }
        }
        // the best s has f1(t + s) ~ f0(t): a rotation by +30 degrees moves the features
        // by +s bins; the head then peaks at shift sign * omega / (180 / NT)
        const float dw = 180.0f / LP_NT;
        const float sdeg = best * dw;
        L.sign = std::fabs(sdeg - 30.0f) < std::fabs(sdeg - 150.0f) ? 1 : -1;
    }
    const int nsteps = o->samples / B;
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    std::vector<float> heul(3 * B), hpar(5 * B), hox(B), hoy(B);
    std::vector<float> htruth[2] = {std::vector<float>(4 * B), std::vector<float>(4 * B)};
    const float* ops = table_ops();
    const float d2r = host_angles().deg2rad, dw = 180.0f / LP_NT;
    // step s's orientations, CTF and origins (heul, hpar, hox, hoy) and targets (htruth[s & 1])
    auto draw = [&](int sidx) {
        std::vector<float>& ht = htruth[sidx & 1];
        for (int b = 0; b < B; ++b) {
            float e[3];
            random_euler(rng, e);
            heul[3 * b] = e[0]; heul[3 * b + 1] = e[1]; heul[3 * b + 2] = e[2];
            const float df = o->df_min + (o->df_max - o->df_min) * U(rng);
            const float da = o->astig_max * U(rng), ang = 180.0f * U(rng);
            const float ox = o->origin_max * (2.0f * U(rng) - 1.0f), oy = o->origin_max * (2.0f * U(rng) - 1.0f);
            hpar[5 * b] = df; hpar[5 * b + 1] = df + da; hpar[5 * b + 2] = ang; hpar[5 * b + 3] = ox;
            hpar[5 * b + 4] = oy;
            hox[b] = ox;
            hoy[b] = oy;
            float th = e[0], ph = e[1], om = e[2];
            asu_fold(&th, &ph, &om, ops, d2r);
            ht[4 * b] = sinf(th * d2r) * cosf(ph * d2r);
            ht[4 * b + 1] = sinf(th * d2r) * sinf(ph * d2r);
            ht[4 * b + 2] = cosf(th * d2r);
            float wv = std::fmod((float)L.sign * om, 180.0f);
            if (wv < 0.0f) wv += 180.0f;
            ht[4 * b + 3] = (float)(((int)std::lround(wv / dw)) % LP_NT);
        }
    };
    // The training data of step s + 1 (projections, transforms, features) are made on a
    // second lane (its own stream and buffers) while the network runs step s; events order
    // the hand-over of the features.  No host wait inside the loop: the host draws step
    // s + 1 while the GPU works.  The non-finite-input flags are checked once at the end
    // (cleared once here, kept by every step) and the losses of the last 10 % of steps
    // land in pinned host memory, read after the final wait.
    if ((r = refresh_lane(c, 0))) return r;
    Ctx* G = c->xlanes[0];
    DBuf<float> gimg, gdeul, gdpar, gvar;
    DBuf<float2> gft;
    if ((r = gimg.ensure((size_t)B * nn)) || (r = gft.ensure((size_t)B * nn)) || (r = gdeul.ensure(3 * (size_t)B)) ||
        (r = gdpar.ensure(5 * (size_t)B)) || (r = gvar.ensure(B)) || (r = ensure_batch(G, B)) ||
        (r = G->lm.feat.ensure((size_t)B * LP_NR * LP_NT)))
        return r;
    struct Events {
        cudaEvent_t ready = nullptr, copied = nullptr;
        ~Events() {
            if (ready) cudaEventDestroy(ready);
            if (copied) cudaEventDestroy(copied);
        }
    } ev;
    CK(cudaEventCreateWithFlags(&ev.ready, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev.copied, cudaEventDisableTiming));
    const int ntail_steps = std::max(1, nsteps / 10);
    float* hloss = nullptr;
    CK(cudaHostAlloc((void**)&hloss, sizeof(float) * (size_t)ntail_steps * B, cudaHostAllocDefault));
    struct PinnedFree {
        float* p;
        ~PinnedFree() { if (p) cudaFreeHost(p); }
    } hloss_free{hloss};
    CK(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));  // weights, sign and flag set before the lane starts
    CK(cudaMemsetAsync(G->flag.p, 0, sizeof(int), G->stream));
    // step sidx's features into G->lm.feat, once the network has taken the previous ones
    auto generate = [&](int sidx) -> int {
        if (sidx > 0) CK(cudaStreamWaitEvent(G->stream, ev.copied, 0));
        CK(cudaMemcpyAsync(gdeul.p, heul.data(), sizeof(float) * 3 * B, cudaMemcpyHostToDevice, G->stream));
        CK(cudaMemcpyAsync(gdpar.p, hpar.data(), sizeof(float) * 5 * B, cudaMemcpyHostToDevice, G->stream));
        int rr;
        if ((rr = learn_render(G, ct.tex, gdeul.p, gdpar.p, B, o->snr,
                               (unsigned long long)o->seed * 1000003ull + (unsigned long long)sidx,
                               G->p.apply_ctf != 0, gimg.p, gft.p, gvar.p)))
            return rr;
        if ((rr = learn_features_dev(G, gimg.p, B, hox.data(), hoy.data(), true))) return rr;
        CK(cudaEventRecord(ev.ready, G->stream));
        return CRYOIM_OK;
    };
    draw(0);
    if ((r = generate(0))) return r;
    for (int sidx = 0; sidx < nsteps; ++sidx) {
        CK(cudaMemcpyAsync(L.truth.p, htruth[sidx & 1].data(), sizeof(float) * 4 * B, cudaMemcpyHostToDevice,
                           c->stream));
        CK(cudaStreamWaitEvent(c->stream, ev.ready, 0));
        CK(cudaMemcpyAsync(L.feat.p, G->lm.feat.p, sizeof(float) * (size_t)B * LP_NR * LP_NT,
                           cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaEventRecord(ev.copied, c->stream));
        if (sidx + 1 < nsteps) {
            draw(sidx + 1);
            if ((r = generate(sidx + 1))) return r;
        }
        if ((r = learn_forward(c, B)) || (r = learn_backward(c, B))) return r;
        // the learning rate ramps up linearly over the first tenth of the steps (from 10 %),
        // then stays at o->lr: Adam's first steps at the full rate sent some seeds' runs
        // to a poor minimum (the proposals' agreement with the exhaustive search ranged over
        // 83-99 % across seeds at 8,192 samples)
        const int nwarm = std::max(1, nsteps / 10);
        const float lr_s = sidx < nwarm ? o->lr * (0.1f + 0.9f * (float)sidx / (float)nwarm) : o->lr;
        launch_lp_adam(L.w.p, L.gr.p, L.m.p, L.v.p, L.nparam, lr_s, ++L.steps, c->stream);
        CK(cudaGetLastError());
        const int tail_slot = sidx - (nsteps - ntail_steps);
        if (tail_slot >= 0)
            CK(cudaMemcpyAsync(hloss + (size_t)tail_slot * B, L.loss.p, sizeof(float) * B, cudaMemcpyDeviceToHost,
                               c->stream));
    }
    CK(cudaStreamSynchronize(G->stream));
    if ((r = check_flag(G))) return r;
    CK(cudaStreamSynchronize(c->stream));
    if ((r = check_flag(c)) || (r = learn_conv_status(c))) return r;
    double tail = 0.0;
    const int ntail = ntail_steps * B;
    for (int q = 0; q < ntail; ++q) tail += hloss[q];
    L.step = c->p.searchstep;
    L.ready = true;
    if (stats) {
        stats[0] = ntail ? (float)(tail / ntail) : 0.0f;
        stats[1] = (float)std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats[2] = (float)L.sign;
        stats[3] = (float)V;
    }
    return CRYOIM_OK;
}

// Proposals of the trained model for the nb particles whose band is in c->band: the
// top kl cells, each as two fine-grid seeds (angle, angle + 180 degrees), expanded to
// their fine neighbourhoods within nbf steps -> lists[i].
int learned_lists(Ctx* c, int nb, int kl, int nbf, std::vector<std::vector<int>>& lists) {
    LearnModel& L = c->lm;
    int r;
    if ((r = learn_activations(c, nb))) return r;
    launch_lp_features(c->band.p, c->bd, nb, L.feat.p, c->stream);
    if ((r = learn_forward(c, nb))) return r;
    launch_lp_topk(L.sc.p, nb, L.V, kl, L.cell.p, L.cellv.p, c->stream);
    CK(cudaGetLastError());
    std::vector<int> cell((size_t)nb * kl);
    CK(cudaMemcpyAsync(cell.data(), L.cell.p, sizeof(int) * cell.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if ((r = learn_conv_status(c))) return r;
    const ViewGrid& g = c->cgrid;
    const int span_c = 2 * g.nph + 1;
    const float dw = 180.0f / LP_NT, step = c->p.searchstep;
    std::vector<std::vector<int3>> seeds(nb);
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < kl; ++j) {
            const int q = cell[(size_t)i * kl + j];
            if (q < 0) continue;
            const int vc = q / LP_NT, s = q % LP_NT, slot = g.view_slot[vc];
            for (int half = 0; half < 2; ++half) {
                float om = (float)L.sign * dw * (float)s + 180.0f * (float)half;
                om = std::fmod(om, 360.0f);
                if (om < 0.0f) om += 360.0f;
                const int io = ((int)std::lround(om / step)) % c->nom;
                seeds[i].push_back(make_int3(2 * (slot / span_c), 2 * (slot % span_c - g.nph), io));
            }
        }
    expand_seeds(c, seeds, nbf, lists);
    return CRYOIM_OK;
}

// FP8-e4m3 copy of operand B with per-band power-of-two scales (contract.cu explains the
// scaling): band maxima of the BF16 rows (every 4th orientation), e_b = floor(log2(224 /
// max_b)), mulB = 2^e_b and mulA = 2^-e_b per sample, then the conversion.
int ensure_bmat8(Ctx* c) {
    int r;
    if ((r = ensure_bmat(c))) return r;
    if (c->bmat8_ready) return CRYOIM_OK;
    const int S = c->cS, nband = c->p.max_r + 2;
    const long n = c->n_orient;
    if ((r = c->bmat8.ensure((size_t)n * c->cKpad8)) || (r = c->bandmax.ensure(nband)) ||
        (r = c->mulA.ensure(S)) || (r = c->mulB.ensure(S)))
        return r;
    if (c->num_sms == 0) CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    CK(launch_band_absmax(c->bmat.p, n, c->cKpad, c->csamples.p, S, nband, 4, c->bandmax.p, c->num_sms,
                          c->stream));
    std::vector<unsigned> hm(nband);
    std::vector<int2> hs(S);
    CK(cudaMemcpyAsync(hm.data(), c->bandmax.p, sizeof(unsigned) * nband, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(hs.data(), c->csamples.p, sizeof(int2) * S, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::vector<int> eb(nband, 0);
    for (int b = 0; b < nband; ++b) {
        float m;
        std::memcpy(&m, &hm[b], 4);
        if (m > 0.0f) eb[b] = std::max(-30, std::min(30, (int)std::floor(std::log2(224.0f / m))));
    }
    std::vector<float> ma(S), mb(S);
    for (int i = 0; i < S; ++i) {
        const int b = std::min(nband - 1, (int)std::sqrt((float)(hs[i].x * hs[i].x + hs[i].y * hs[i].y)));
        mb[i] = std::ldexp(1.0f, eb[b]);
        ma[i] = std::ldexp(1.0f, -eb[b]);
    }
    CK(cudaMemcpyAsync(c->mulA.p, ma.data(), sizeof(float) * S, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->mulB.p, mb.data(), sizeof(float) * S, cudaMemcpyHostToDevice, c->stream));
    CK(launch_b_to_e4m3(c->bmat.p, n, c->cKpad, S, c->mulB.p, c->cKpad8, c->bmat8.p, c->stream));
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->bmat8_ms = ms;
    c->bmat8_ready = true;
    return CRYOIM_OK;
}

// Extra pass lane i of the contraction search: a context with its own stream, cuFFT
// plans, per-pass buffers and proposer activations, and c's read-only state borrowed
// (parameters, templates, search grids, origin grids, reference-map sections, proposer
// weights).  Refreshed at every multi-pass call, after c's state is complete.
int refresh_lane(Ctx* c, int i) {
    while ((int)c->xlanes.size() <= i) {
        Ctx* h = new (std::nothrow) Ctx();
        if (!h) return fail(CRYOIM_ERR_NOMEM, "lane context");
        h->device = c->device;
        c->xlanes.push_back(h);
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    Ctx* h = c->xlanes[i];
    h->p = c->p;
    h->have_params = c->have_params;
    h->bd = c->bd;
    h->batch = c->batch;
    h->ops.borrow(c->ops);
    h->T = c->T;
    h->tmpl = c->tmpl;
    h->tband.borrow(c->tband);
    h->tfcut0.borrow(c->tfcut0);
    h->tort.borrow(c->tort);
    h->grid_ready = c->grid_ready;
    h->nth = c->nth; h->nph = c->nph; h->nom = c->nom; h->V = c->V;
    h->views = c->views;
    h->d_views.borrow(c->d_views);
    h->alpha.borrow(c->alpha);
    h->mapcube.borrow(c->mapcube);
    h->map_ready = c->map_ready;
    h->ovs = c->ovs;
    h->cube_r = c->cube_r;
    h->csamples.borrow(c->csamples);
    h->cS = c->cS; h->cKpad = c->cKpad;
    h->bmat.borrow(c->bmat);
    h->n_orient = c->n_orient;
    h->bmat_ready = c->bmat_ready; h->bmat_ms = c->bmat_ms;
    h->bmat8.borrow(c->bmat8);
    h->bmat8_ready = c->bmat8_ready; h->bmat8_ms = c->bmat8_ms; h->cKpad8 = c->cKpad8;
    h->mulA.borrow(c->mulA);
    h->mulB.borrow(c->mulB);
    h->cgrid = c->cgrid;
    h->csamples_c.borrow(c->csamples_c);
    h->cS_c = c->cS_c; h->cKpad_c = c->cKpad_c; h->n_origin_c = c->n_origin_c;
    h->orig_max_c = c->orig_max_c; h->orig_step_c = c->orig_step_c;
    h->bmat_c.borrow(c->bmat_c);
    h->bmat_c_ready = c->bmat_c_ready; h->n_orient_c = c->n_orient_c;
    h->corigins_c.borrow(c->corigins_c);
    h->corigins.borrow(c->corigins);
    h->n_origin = c->n_origin; h->orig_max = c->orig_max; h->orig_step = c->orig_step;
    h->view_slot = c->view_slot;
    h->slot_view = c->slot_view;
    h->num_sms = c->num_sms;
    h->prof = c->prof;
    LearnModel& a = h->lm;
    const LearnModel& b = c->lm;
    a.ready = b.ready; a.V = b.V; a.sign = b.sign; a.step = b.step; a.nparam = b.nparam;
    for (int i = 0; i < 5; ++i) { a.oW[i] = b.oW[i]; a.ob[i] = b.ob[i]; }
    a.oT = b.oT; a.steps = b.steps; a.conv_tc = b.conv_tc;
    a.w.borrow(b.w);
    a.vview.borrow(b.vview);
    int r;
    if ((r = a.cerr.ensure(1))) return r;
    CK(cudaMemsetAsync(a.cerr.p, 0, sizeof(int), h->stream));
    return CRYOIM_OK;
}

int contract_impl(Ctx* c, const float* imgs, bool on_device, cryoim_particle* parts, int P,
                  const cryoim_contract_opts* opts, float* cands) {
    int r = check_ready(c, false);
    if (r) return r;
    if (!imgs || !parts || !opts || P < 0) return fail(CRYOIM_ERR_ARG, "null input or negative count");
    if (!c->map_ready) return fail(CRYOIM_ERR_STATE, "cryoim_set_reference_map has not been called");
    const int k = opts->topk;
    if (k < 1 || k > 64) return fail(CRYOIM_ERR_ARG, "topk must be 1..64");
    if (!(opts->origin_step > 0) || opts->origin_max < 0) return fail(CRYOIM_ERR_ARG, "bad origin grid");
    if (opts->precision != 0 && opts->precision != 1) return fail(CRYOIM_ERR_ARG, "precision must be 0 or 1");
    const bool f8 = opts->precision == 1;
    const bool centred = opts->centred_origins != 0;
    const int nbr = opts->nbr <= 0 ? 1 : opts->nbr;
    const int nbest = opts->nbr_best;  // 0: neighbourhoods of every candidate
    if (nbest < 0) return fail(CRYOIM_ERR_ARG, "nbr_best must be >= 0");
    const int nbox = (2 * nbr + 1) * (2 * nbr + 1) * (2 * nbr + 1);
    if (nbr > 3 || (long)nbox * k > 4096) return fail(CRYOIM_ERR_ARG, "(2 nbr + 1)^3 x topk must be <= 4096");
    const int kc = opts->coarse;  // 0: exhaustive; else coarse proposals per particle
    // fine neighbourhood of a proposal, in fine steps
    const int nbf = opts->proposal_nbr == 0 ? 2 : opts->proposal_nbr;
    if (kc < 0 || kc > 64) return fail(CRYOIM_ERR_ARG, "coarse must be 0..64");
    if (nbf < 1 || nbf > 4) return fail(CRYOIM_ERR_ARG, "proposal_nbr must be 0..4");
    const int kl = opts->learned;  // 0: off; else learned proposals per particle
    if (kl < 0 || kl > 64 || (kl > 0 && kc > 0)) return fail(CRYOIM_ERR_ARG, "learned must be 0..64, not with coarse");
    if (kl > 0 && !(c->lm.ready && c->lm.step == c->p.searchstep && c->cgrid.V == c->lm.V))
        return fail(CRYOIM_ERR_STATE, "no trained proposer for this search step (cryoim_learn_train / _load)");
    // local form: each particle's own grid of (2 lm + 1)^3 orientations, cut from the band
    // cube per pass instead of gathered from the global sections
    const bool local = opts->local_range > 0.0f;
    int lm = 0;
    long nloc = 0;
    if (local) {
        if (!(opts->local_step > 0.0f)) return fail(CRYOIM_ERR_ARG, "local_step must be > 0");
        lm = (int)std::lround(opts->local_range / opts->local_step);
        if (lm < 1 || lm > 64) return fail(CRYOIM_ERR_ARG, "local_range / local_step must round to 1..64");
        if (opts->pick != 1 || f8 || kc > 0 || kl > 0)
            return fail(CRYOIM_ERR_ARG, "the local form needs pick = 1, BF16, no coarse or learned proposals");
        nloc = (long)(2 * lm + 1) * (2 * lm + 1) * (2 * lm + 1);
    } else if (opts->pick == 0 && c->T <= 0) {
        return fail(CRYOIM_ERR_STATE, "PR rescoring needs cryoim_load_templates");
    }
    if (P == 0) return CRYOIM_OK;
    if ((r = local ? ensure_samples(c) : (f8 ? ensure_bmat8(c) : ensure_bmat(c)))) return r;
    if (kc > 0 && (r = ensure_coarse(c, opts->origin_max, opts->origin_step))) return r;
    const int kpad = f8 ? c->cKpad8 : c->cKpad;
    c->last_kpad = kpad;
    c->last_slice_ms = c->bmat_ms + (f8 ? c->bmat8_ms : 0.0);
    if (c->n_orient > 0x7fffffffL) return fail(CRYOIM_ERR_SIZE, "too many orientations");
    // origin grid
    if (opts->origin_max != c->orig_max || opts->origin_step != c->orig_step) {
        const int n1 = (int)(2.0f * opts->origin_max / opts->origin_step + 0.5f) + 1;
        std::vector<float> og;
        for (int iy = 0; iy < n1; ++iy)
            for (int ix = 0; ix < n1; ++ix) {
                og.push_back(-opts->origin_max + opts->origin_step * (float)ix);
                og.push_back(-opts->origin_max + opts->origin_step * (float)iy);
            }
        if ((r = c->corigins.ensure(og.size()))) return r;
        CK(cudaMemcpyAsync(c->corigins.p, og.data(), sizeof(float) * og.size(), cudaMemcpyHostToDevice,
                           c->stream));
        c->n_origin = n1 * n1;
        c->orig_max = opts->origin_max;
        c->orig_step = opts->origin_step;
    }
    const int O = c->n_origin, T = c->T, nx = c->p.fftsize;
    const long nn = (long)nx * nx, w2 = (long)c->bd.W * c->bd.W;
    // Particles per pass (transform, rescoring: large grids, two host waits per pass) and
    // per exhaustive contraction launch (operand A of about 2400 rows stays L2-resident
    // while the sections stream).  The proposal form builds A for the whole pass: its
    // grouped launch reads each particle's A against that particle's own few tiles.
    const int PB = std::max(1, c->batch);
    const int pb = std::max(1, std::min(PB, 2400 / std::max(O, 1)));
    const int arows = (kc > 0 || kl > 0 || local) ? PB : pb;
    const int ntiles = (int)(((local ? nloc : c->n_orient) + gemm_tile_n() - 1) / gemm_tile_n());
    // the band cube as a filtering texture for the local form's sections (shared by the lanes)
    struct LocalTexture {
        cudaArray_t arr = nullptr;
        cudaTextureObject_t tex = 0;
        ~LocalTexture() { free_cube_texture(arr, tex); }
    } ltex;
    if (local) CK(make_cube_texture(c->mapcube.p, c->cube_r, c->stream, &ltex.arr, &ltex.tex));
    // rescoring set: each selected orientation and its grid neighbours within nbr steps
    const int maxx = nbox * k;
    if (c->num_sms == 0) CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
    std::vector<int> src(P);
    {
        int id0 = -100, cur = -1;
        for (int i = 0; i < P; ++i) {
            if (parts[i].img_id != id0) { cur = i; id0 = parts[i].img_id; }
            src[i] = cur;
        }
    }
    std::vector<float> ohost(2 * (size_t)O);
    CK(cudaMemcpyAsync(ohost.data(), c->corigins.p, sizeof(float) * 2 * O, cudaMemcpyDeviceToHost, c->stream));
    const long row_bytes = f8 ? (long)c->cKpad8 : 2L * c->cKpad;
    // Passes are dealt round-robin to lanes (this context and c->xlanes, each with its own
    // stream, per-pass buffers and host thread), so that one lane's host work between
    // its waits overlaps the other lanes' kernels.
    const int nlanes = std::max(1, std::min(c->lanes, (P + PB - 1) / PB));
    auto alloc = [&](Ctx* L) -> int {
        int r;
        if ((r = ensure_batch(L, PB))) return r;
        if (f8 ? ((r = L->amat8.ensure((size_t)arows * O * L->cKpad8)) || (r = L->fexp.ensure(PB)))
               : (r = L->amat.ensure((size_t)arows * O * L->cKpad)))
            return r;
        if ((r = L->topv.ensure((size_t)arows * O * ntiles)) || (r = L->topi.ensure((size_t)arows * O * ntiles)))
            return r;
        if ((r = L->gerr.ensure(1)) || (r = L->pnorm.ensure(PB)) || (r = L->pcband.ensure((size_t)PB * L->cS)) ||
            (r = L->kor.ensure((size_t)PB * k)) ||
            (r = L->korig.ensure((size_t)PB * k)) || (r = L->kcc.ensure((size_t)PB * k)) ||
            (r = L->kcand.ensure((size_t)PB * k * 5)) || (r = L->kcc64.ensure((size_t)PB * k)) ||
            (r = L->kpart.ensure((size_t)cc_fp64_scratch(k, PB))))
            return r;
        if (local && ((r = L->pnorm0.ensure(PB)) || (r = L->pctf.ensure((size_t)PB * L->cS)))) return r;
        if ((r = L->tilev.ensure((size_t)pb * ntiles)) || (r = L->tileo.ensure((size_t)pb * ntiles)) ||
            (r = L->tileorig.ensure((size_t)pb * ntiles)) || (r = L->xcand.ensure((size_t)PB * maxx * 5)) ||
            (r = L->xpr.ensure((size_t)PB * maxx)))
            return r;
        if (local && (r = L->lcentre.ensure(3 * (size_t)PB))) return r;
        if (centred && (r = L->poff.ensure(2 * (size_t)PB))) return r;
        if (T > 0 && !local &&
            ((r = L->xalpha.ensure((size_t)PB * maxx * T * 60)) || (r = L->sband.ensure((size_t)PB * w2)) ||
                      (r = L->xcount.ensure(PB)) || (L->p.apply_ctf && (r = L->tbandc.ensure((size_t)PB * T * w2)))))
            return r;
        return CRYOIM_OK;
    };
    auto run = [&](Ctx* L, int lane) -> int {
        int r;
        std::vector<float> hpar(8 * PB), hcand((size_t)PB * k * 5), hcc((size_t)PB * k);
        std::vector<int> hor((size_t)PB * k), horig((size_t)PB * k);
        std::vector<double> hcc64((size_t)PB * k);
        // profiling: an event pair around every contraction launch of a pass
        std::vector<cudaEvent_t> gev;
        auto gmark = [&](size_t i) -> int {
            while (gev.size() <= i) {
                cudaEvent_t e;
                CK(cudaEventCreate(&e));
                gev.push_back(e);
            }
            CK(cudaEventRecord(gev[i], L->stream));
            return CRYOIM_OK;
        };
        size_t ngev = 0;
        for (int b0 = lane * PB; b0 < P; b0 += nlanes * PB) {
            const int nb = std::min(PB, P - b0);
            const float* d_src;
            if (on_device) {
                d_src = imgs + b0 * nn;
            } else {
                CK(cudaMemcpyAsync(L->imgs.p, imgs + b0 * nn, sizeof(float) * nb * nn, cudaMemcpyHostToDevice,
                                   L->stream));
                d_src = L->imgs.p;
            }
            std::fill(hpar.begin(), hpar.end(), 0.0f);
            for (int i = 0; i < nb; ++i) {
                const cryoim_particle& q = parts[b0 + i];
                const cryoim_particle& s = parts[src[b0 + i]];
                hpar[i] = q.x; hpar[PB + i] = q.y;
                hpar[4 * PB + 3 * i] = s.df1; hpar[4 * PB + 3 * i + 1] = s.df2; hpar[4 * PB + 3 * i + 2] = s.astigang;
            }
            // mask at the input origin as ort_globesearch.f90:50 does; the transform stays unshifted
            if ((r = transform_batch(L, d_src, nb, PB, hpar, 1, 0, false))) return r;
            ParView pv = par_view(L, PB);
            const float* ctfp = nullptr;
            const float* tfc = L->tfcut0.p;
            long tfs = 0;
            if (L->p.apply_ctf) {
                launch_ctf_band(nb, L->bd, pv.dfs, L->p.apix, L->p.vol, L->p.cs, L->p.ampwg, L->ctf.p, L->stream);
                ctfp = L->ctf.p;
                if (T > 0 && !local) {
                    launch_tmpl_fcut(L->tband.p, T, L->ctf.p, nb, L->bd, L->tfcut.p, L->stream);
                    tfc = L->tfcut.p;
                    tfs = (long)T * L->bd.nr;
                }
            }
            launch_particle_norm(L->band.p, ctfp, L->bd, L->csamples.p, L->cS, nb, L->pnorm.p, L->stream,
                                 L->pcband.p, local ? L->pnorm0.p : nullptr, local ? L->pctf.p : nullptr);
            if (centred) {  // the origin grid around each particle's own origin
                std::vector<float> po(2 * (size_t)nb);
                for (int i = 0; i < nb; ++i) { po[2 * i] = parts[b0 + i].x; po[2 * i + 1] = parts[b0 + i].y; }
                CK(cudaMemcpyAsync(L->poff.p, po.data(), sizeof(float) * po.size(), cudaMemcpyHostToDevice, L->stream));
            }
            // operand A rows (particle, origin) of particles [s0, s0 + ns) at row (s0 - a0) O
            auto build_rows = [&](int s0, int ns, int a0) {
                const float2* bb = L->band.p + (long)s0 * w2;
                const float* cc = ctfp ? ctfp + (long)s0 * w2 : nullptr;
                const float* po = centred ? L->poff.p + 2 * (size_t)s0 : nullptr;
                if (f8)
                    launch_build_a8(bb, cc, L->bd, L->csamples.p, L->cS, L->cKpad8, L->corigins.p, O, L->pnorm.p + s0,
                                    L->mulA.p, L->fexp.p + s0, ns, L->amat8.p + (size_t)(s0 - a0) * O * L->cKpad8,
                                    L->stream, po);
                else  // the local form's rows are normalised by |P| (its sections by |CTF S|)
                    launch_build_a(bb, cc, L->bd, L->csamples.p, L->cS, L->cKpad, L->corigins.p, O,
                                   (local ? L->pnorm0.p : L->pnorm.p) + s0, ns,
                                   L->amat.p + (size_t)(s0 - a0) * O * L->cKpad, L->stream, po);
            };
            GemmArgmaxArgs g{};
            g.b_mode = 1;  // section rows are stored pre-swizzled (exhaustive and local tiles)
            g.topv = L->topv.p;
            g.topi = L->topi.p;
            g.cfull = nullptr;
            g.err = L->gerr.p;
            CK(cudaMemsetAsync(L->gerr.p, 0, sizeof(int), L->stream));
            std::vector<std::vector<int>> lists, slots;
            ngev = 0;
            if (kc > 0 || kl > 0 || local) {
                // proposal forms: the coarse contraction or the learned proposer names each
                // particle's candidate orientations, the fine contraction runs on their
                // sections only; the local form cuts each particle's local grid
                if (!local &&
                    (r = kc > 0 ? coarse_lists(L, nb, ctfp, kc, nbf, lists) : learned_lists(L, nb, kl, nbf, lists)))
                    return r;
                CK(cudaMemsetAsync(L->gerr.p, 0, sizeof(int), L->stream));
                const void* bsrc = f8 ? (const void*)L->bmat8.p : (const void*)L->bmat.p;
                const char* abase = f8 ? (const char*)L->amat8.p : (const char*)L->amat.p;
                build_rows(0, nb, 0);
                CK(cudaGetLastError());
                // the proposal forms read their sections from the bank by index: the
                // contraction's producer copies each listed row into its tile (the rows are
                // stored pre-swizzled; the copy re-swizzles a row for its tile row).  The
                // local form cuts each particle's grid into the pass buffer at a start that
                // is a multiple of 8.
                const long lpitch = (nloc + 7) / 8 * 8;
                if (!local) slots = lists;
                auto rows_of = [&](int i) -> long { return local ? lpitch : (long)slots[i].size(); };
                // particles in groups (the local form's cut sections under 8 GB per group): one
                // grouped contraction per group (each particle's origin rows against its own
                // sections), then the k distinct best orientations of each particle
                for (int i0 = 0; i0 < nb;) {
                    int i1 = i0;
                    long rows = 0;
                    while (i1 < nb && (i1 == i0 || !local || (rows + rows_of(i1)) * row_bytes <= (8L << 30)))
                        rows += rows_of(i1++);
                    GemmArgmaxArgs gg = g;
                    if (local) {
                        if ((r = L->bgather.ensure((size_t)rows * row_bytes))) return r;
                        std::vector<float> cen(3 * (size_t)(i1 - i0));
                        for (int i = i0; i < i1; ++i) {
                            cen[3 * (i - i0)] = parts[b0 + i].theta;
                            cen[3 * (i - i0) + 1] = parts[b0 + i].phi;
                            cen[3 * (i - i0) + 2] = parts[b0 + i].omega;
                        }
                        CK(cudaMemcpyAsync(L->lcentre.p, cen.data(), sizeof(float) * cen.size(), cudaMemcpyHostToDevice,
                                           L->stream));
                        CK(launch_slice_bf16_local(ltex.tex, c->cube_r, L->csamples.p, L->cS, L->cKpad, L->lcentre.p,
                                                   lm, opts->local_step, rows, L->bgather.p, L->stream,
                                                   c->mapcube.p, c->interp_sigma, lpitch,
                                                   L->pctf.p + (size_t)i0 * L->cS, (float)c->ovs));
                    } else {
                        std::vector<int> idx;
                        idx.reserve(rows);
                        for (int i = i0; i < i1; ++i) idx.insert(idx.end(), slots[i].begin(), slots[i].end());
                        for (int n : idx)
                            if (n < 0 || n >= L->n_orient) return fail(CRYOIM_ERR_STATE, "proposal row %d", n);
                        if ((r = L->gidx.ensure(rows))) return r;
                        CK(cudaMemcpyAsync(L->gidx.p, idx.data(), sizeof(int) * rows, cudaMemcpyHostToDevice,
                                           L->stream));
                        gg.b_mode = 2;
                        gg.b_index = L->gidx.p;
                        gg.b_rows = (const unsigned char*)bsrc;
                        gg.b_row_bytes = row_bytes;
                    }
                    std::vector<GemmGroup> hg(i1 - i0);
                    std::vector<int2> seg(i1 - i0);
                    long roff = 0, toff = 0;
                    for (int i = i0; i < i1; ++i) {
                        const int nl = (int)(local ? nloc : (long)slots[i].size());
                        const int ntp = (nl + gemm_tile_n() - 1) / gemm_tile_n();
                        GemmGroup& q = hg[i - i0];
                        q.a_row0 = i * O;
                        q.m_valid = O;
                        q.b_row0 = (int)roff;
                        q.n_valid = nl;
                        q.topv_off = (int)toff;
                        seg[i - i0] = make_int2((int)toff, ntp);
                        roff += local ? lpitch : nl;
                        toff += (long)O * ntp;
                        // the useful work: the particle's listed orientations (not padding slots)
                        if (L->prof)
                            L->prof_gemm_flops += 2.0 * (double)O * (double)(local ? nloc : (long)lists[i].size()) *
                                                  (double)kpad;
                    }
                    if ((r = L->ggroups.ensure(i1 - i0)) || (r = L->gseg.ensure(i1 - i0))) return r;
                    if (L->prof && (r = gmark(ngev++))) return r;
                    CK(launch_gemm_argmax_grouped(abase, (long)nb * O, local ? (const void*)L->bgather.p : bsrc, rows,
                                                  kpad, f8, hg.data(), i1 - i0, L->ggroups.p, gg, L->num_sms,
                                                  L->stream));
                    if (L->prof && (r = gmark(ngev++))) return r;
                    CK(cudaMemcpyAsync(L->gseg.p, seg.data(), sizeof(int2) * seg.size(), cudaMemcpyHostToDevice,
                                       L->stream));
                    launch_select_distinct(L->topv.p, L->topi.p, O, L->gseg.p, i1 - i0, k, L->kor.p + (size_t)i0 * k,
                                           L->korig.p + (size_t)i0 * k, L->kcc.p + (size_t)i0 * k, L->stream);
                    CK(cudaGetLastError());
                    // the cut-section buffer and the row lists are reused by the next group
                    if (i1 < nb) CK(cudaStreamSynchronize(L->stream));
                    i0 = i1;
                }
            } else {
                // exhaustive: sub-batches of pb particles against every section, queued back to back
                for (int s0 = 0; s0 < nb; s0 += pb) {
                    const int ns = std::min(pb, nb - s0);
                    build_rows(s0, ns, s0);
                    CK(cudaGetLastError());
                    if (L->prof && (r = gmark(ngev++))) return r;
                    if (f8)
                        CK(launch_gemm_argmax(L->amat8.p, L->bmat8.p, ns * O, (int)L->n_orient, kpad, true, g,
                                              L->num_sms, L->stream));
                    else
                        CK(launch_gemm_argmax(L->amat.p, L->bmat.p, ns * O, (int)L->n_orient, kpad, false, g,
                                              L->num_sms, L->stream));
                    if (L->prof && (r = gmark(ngev++))) return r;
                    launch_select_topk(L->topv.p, L->topi.p, O, ntiles, k, ns, L->tilev.p, L->tileo.p, L->tileorig.p,
                                       L->kor.p + (size_t)s0 * k, L->korig.p + (size_t)s0 * k,
                                       L->kcc.p + (size_t)s0 * k, L->stream);
                    CK(cudaGetLastError());
                    if (L->prof) L->prof_gemm_flops += 2.0 * (double)ns * O * (double)L->n_orient * (double)kpad;
                }
            }
            int gerr = 0;
            CK(cudaMemcpyAsync(&gerr, L->gerr.p, sizeof(int), cudaMemcpyDeviceToHost, L->stream));
            CK(cudaMemcpyAsync(hor.data(), L->kor.p, sizeof(int) * nb * k, cudaMemcpyDeviceToHost, L->stream));
            CK(cudaMemcpyAsync(horig.data(), L->korig.p, sizeof(int) * nb * k, cudaMemcpyDeviceToHost, L->stream));
            CK(cudaMemcpyAsync(hcc.data(), L->kcc.p, sizeof(float) * nb * k, cudaMemcpyDeviceToHost, L->stream));
            std::vector<int> hfe(nb, 0);
            if (f8) CK(cudaMemcpyAsync(hfe.data(), L->fexp.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, L->stream));
            if ((r = check_flag(L))) return r;
            if (gerr) return fail(CRYOIM_ERR_CUDA, "contraction pipeline wait timed out");
            if (f8)  // remove the per-particle exponent: the CC of the unit-norm rows
                for (int i = 0; i < nb * k; ++i) hcc[i] = std::ldexp(hcc[i], -hfe[i / k]);
            if (kc > 0 || kl > 0)  // list position -> fine orientation index
                for (int i = 0; i < nb * k; ++i)
                    if (hor[i] >= 0) hor[i] = slots[i / k][hor[i]];
            if (L->prof)
                for (size_t e = 0; e + 1 < ngev; e += 2) {
                    float ms = 0.f;
                    CK(cudaEventElapsedTime(&ms, gev[e], gev[e + 1]));
                    L->prof_gemm_ms += ms;
                    L->prof_gemm_launches += 1;
                }
            // candidates (theta, phi, omega, x, y) of the selected (orientation, origin) pairs
            for (int i = 0; i < nb * k; ++i) {
                int n = hor[i] < 0 ? 0 : hor[i];
                int o = horig[i];
                if (local) {  // the local grid index of the particle's own grid, as k_slice_bf16_local
                    const cryoim_particle& q = parts[b0 + i / k];
                    const int ln = 2 * lm + 1, li = n / (ln * ln), lj = (n / ln) % ln, lk = n % ln;
                    hcand[5 * i] = q.theta + opts->local_step * (float)(li - lm);
                    hcand[5 * i + 1] = q.phi + opts->local_step * (float)(lj - lm);
                    hcand[5 * i + 2] = q.omega + opts->local_step * (float)(lk - lm);
                } else {
                    int v = n / L->nom, io = n % L->nom;
                    hcand[5 * i] = L->views[4 * v];
                    hcand[5 * i + 1] = L->views[4 * v + 1];
                    hcand[5 * i + 2] = L->p.searchstep * (float)io;
                }
                hcand[5 * i + 3] = ohost[2 * o] + (centred ? parts[b0 + i / k].x : 0.0f);
                hcand[5 * i + 4] = ohost[2 * o + 1] + (centred ? parts[b0 + i / k].y : 0.0f);
            }
            CK(cudaMemcpyAsync(L->kcand.p, hcand.data(), sizeof(float) * nb * k * 5, cudaMemcpyHostToDevice,
                               L->stream));
            // the FP64 correlations decide the pick (pick = 1) or are returned with the
            // candidates; a phase-residual pick without candidate output does not read them
            const bool need_cc64 = opts->pick != 0 || cands != nullptr;
            if (need_cc64)
                launch_cc_fp64(L->mapcube.p, L->pcband.p, L->bd, L->csamples.p, L->cS, L->kcand.p, k, nb,
                               local ? L->pnorm0.p : L->pnorm.p, L->kpart.p, L->kcc64.p, L->stream, c->interp_sigma,
                               local ? L->pctf.p : nullptr, c->cube_r, (float)c->ovs);
            // Phase-residual rescoring at the particle's own origin (ort_globesearch.f90 scores
            // every view at particle(i)%x, %y) over each selected orientation and its grid
            // neighbours within nbr steps (all of them, or, with nbr_best = m, only those of
            // the m candidates of least phase residual, scored first); the result equals the
            // exhaustive search wherever its minimum lies in the scored set.  Sets are sorted
            // by orientation index, without repeats.
            std::vector<std::vector<int>> xs(nb);
            std::vector<std::vector<float>> xp(nb);
            const int span = 2 * L->nph + 1;
            auto neighbourhood = [&](int n, std::vector<int>& lst) {
                const int v = n / L->nom, io = n % L->nom, slot = L->view_slot[v];
                const int it = slot / span, ips = slot % span - L->nph;
                for (int dt = -nbr; dt <= nbr; ++dt)
                    for (int dp = -nbr; dp <= nbr; ++dp) {
                        const int it2 = it + dt, ips2 = ips + dp;
                        if (it2 < 0 || it2 > L->nth || ips2 < -L->nph || ips2 > L->nph) continue;
                        const int v2 = L->slot_view[(size_t)it2 * span + ips2 + L->nph];
                        if (v2 < 0) continue;
                        for (int dw = -nbr; dw <= nbr; ++dw)
                            lst.push_back(v2 * L->nom + ((io + dw) % L->nom + L->nom) % L->nom);
                    }
            };
            // phase residuals of per-particle orientation sets (empty sets score nothing)
            auto score = [&](const std::vector<std::vector<int>>& sets, std::vector<std::vector<float>>& out) -> int {
                int maxc = 1;
                for (int i = 0; i < nb; ++i) maxc = std::max(maxc, (int)sets[i].size());
                if (maxc > maxx) return fail(CRYOIM_ERR_SIZE, "rescoring set of %d orientations", maxc);
                std::vector<float> hx((size_t)nb * maxc * 5, 0.0f);
                std::vector<int> hcount(nb);
                for (int i = 0; i < nb; ++i) {
                    hcount[i] = (int)sets[i].size();
                    for (int j = 0; j < maxc; ++j) {
                        const int n = sets[i].empty() ? 0 : sets[i][std::min<size_t>(j, sets[i].size() - 1)];
                        float* o = &hx[((size_t)i * maxc + j) * 5];
                        o[0] = L->views[4 * (n / L->nom)];
                        o[1] = L->views[4 * (n / L->nom) + 1];
                        o[2] = L->p.searchstep * (float)(n % L->nom);
                        o[3] = parts[b0 + i].x;
                        o[4] = parts[b0 + i].y;
                    }
                }
                CK(cudaMemcpyAsync(L->xcand.p, hx.data(), sizeof(float) * hx.size(), cudaMemcpyHostToDevice,
                                   L->stream));
                CK(cudaMemcpyAsync(L->xcount.p, hcount.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, L->stream));
                // the shared-band kernel takes its line angles from the search grid's view table
                // (the exhaustive search's own); the other kernel from per-candidate tables
                const bool shared = pr_rescore_shared_band(L->bd, T);
                if (shared) {
                    std::vector<int> ho((size_t)nb * maxc, 0);
                    for (int i = 0; i < nb; ++i)
                        for (int j = 0; j < maxc; ++j)
                            ho[(size_t)i * maxc + j] =
                                sets[i].empty() ? 0 : sets[i][std::min<size_t>(j, sets[i].size() - 1)];
                    if ((r = L->xorient.ensure(ho.size()))) return r;
                    CK(cudaMemcpyAsync(L->xorient.p, ho.data(), sizeof(int) * ho.size(), cudaMemcpyHostToDevice,
                                       L->stream));
                } else {
                    launch_refine_alpha(L->xcand.p, nb, L->tort.p, T, L->ops.p, L->xalpha.p, L->stream, maxc);
                }
                // every candidate of a particle sits at the particle's origin: shift its band once
                CK(launch_shift_band(L->band.p, L->xcand.p, maxc, L->bd, nb, L->sband.p, L->stream));
                PrSingleArgs a{};
                a.band = L->band.p; a.fcut0 = L->fcut0.p; a.tband = L->tband.p; a.tfcut = tfc;
                a.tfcut_pstride = tfs; a.ctf = ctfp; a.cand = L->xcand.p; a.alpha = L->xalpha.p; a.T = T;
                a.bd = L->bd; a.pr = L->xpr.p; a.ncand = maxc; a.sband = L->sband.p; a.ncount = L->xcount.p;
                a.tbandc = ctfp ? L->tbandc.p : nullptr;
                if (shared) {
                    a.valpha = L->alpha.p;
                    a.corient = L->xorient.p;
                    a.nom = L->nom;
                    a.step = L->p.searchstep;
                }
                // candidates of a particle sharing a view, in groups (the sets are sorted by
                // orientation index, so a view's omegas are adjacent)
                std::vector<int4> grp;
                const int rg = pr_rescore_group_size();
                for (int i = 0; i < nb; ++i)
                    for (size_t j = 0; j < sets[i].size();) {
                        size_t e = j + 1;
                        while (e < sets[i].size() && (int)(e - j) < rg && sets[i][e] / L->nom == sets[i][j] / L->nom) ++e;
                        grp.push_back(make_int4(i, (int)j, (int)(e - j), 0));
                        j = e;
                    }
                // larger groups first: a block's time grows with its candidates, so the last
                // wave of blocks is filled with the short ones (the results do not depend on
                // the order: each group writes its own candidates' scores)
                std::stable_sort(grp.begin(), grp.end(), [](const int4& x, const int4& y) { return x.z > y.z; });
                if (!grp.empty()) {
                    if ((r = L->xgroups.ensure(grp.size()))) return r;
                    CK(cudaMemcpyAsync(L->xgroups.p, grp.data(), sizeof(int4) * grp.size(), cudaMemcpyHostToDevice,
                                       L->stream));
                    if (L->prof && (r = gmark(ngev++))) return r;
                    CK(launch_pr_rescore_groups(a, L->xgroups.p, (int)grp.size(), L->stream));
                    if (L->prof) {
                        if ((r = gmark(ngev++))) return r;
                        for (int i = 0; i < nb; ++i) L->prof_pr_cands += (double)sets[i].size();
                    }
                }
                std::vector<float> h((size_t)nb * maxc);
                CK(cudaMemcpyAsync(h.data(), L->xpr.p, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, L->stream));
                CK(cudaStreamSynchronize(L->stream));
                if (L->prof && !grp.empty() && ngev >= 2) {
                    float ms = 0.f;
                    CK(cudaEventElapsedTime(&ms, gev[ngev - 2], gev[ngev - 1]));
                    L->prof_pr_ms += ms;
                    L->prof_pr_launches += 1;
                    ngev -= 2;
                }
                out.assign(nb, std::vector<float>());
                for (int i = 0; i < nb; ++i) out[i].assign(h.begin() + (size_t)i * maxc, h.begin() + (size_t)i * maxc + sets[i].size());
                return CRYOIM_OK;
            };
            if (T > 0 && !local) {
                // the templates under each particle's CTF, once per pass
                if (ctfp) CK(launch_tband_ctf(L->tband.p, T, ctfp, L->bd, nb, L->tbandc.p, L->stream));
                if (nbest <= 0 || nbest >= k) {
                    for (int i = 0; i < nb; ++i) {
                        for (int rr = 0; rr < k; ++rr)
                            if (hor[i * k + rr] >= 0) neighbourhood(hor[i * k + rr], xs[i]);
                        std::sort(xs[i].begin(), xs[i].end());
                        xs[i].erase(std::unique(xs[i].begin(), xs[i].end()), xs[i].end());
                        if (xs[i].empty()) xs[i].push_back(0);
                    }
                    if ((r = score(xs, xp))) return r;
                } else {
                    // the candidates first, then the neighbourhoods of the nbest best of them
                    std::vector<std::vector<int>> xa(nb), xb(nb);
                    std::vector<std::vector<float>> pa, pb;
                    for (int i = 0; i < nb; ++i) {
                        for (int rr = 0; rr < k; ++rr)
                            if (hor[i * k + rr] >= 0) xa[i].push_back(hor[i * k + rr]);
                        std::sort(xa[i].begin(), xa[i].end());
                        xa[i].erase(std::unique(xa[i].begin(), xa[i].end()), xa[i].end());
                        if (xa[i].empty()) xa[i].push_back(0);
                    }
                    if ((r = score(xa, pa))) return r;
                    for (int i = 0; i < nb; ++i) {
                        std::vector<int> ord(xa[i].size());
                        for (size_t j = 0; j < ord.size(); ++j) ord[j] = (int)j;
                        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return pa[i][x] < pa[i][y]; });
                        std::vector<int> nb_set;
                        for (int j = 0; j < std::min<int>(nbest, (int)ord.size()); ++j) neighbourhood(xa[i][ord[j]], nb_set);
                        std::sort(nb_set.begin(), nb_set.end());
                        nb_set.erase(std::unique(nb_set.begin(), nb_set.end()), nb_set.end());
                        std::set_difference(nb_set.begin(), nb_set.end(), xa[i].begin(), xa[i].end(),
                                            std::back_inserter(xb[i]));
                    }
                    if ((r = score(xb, pb))) return r;
                    for (int i = 0; i < nb; ++i) {  // merge, sorted by orientation index
                        size_t ia = 0, ib = 0;
                        while (ia < xa[i].size() || ib < xb[i].size()) {
                            if (ib >= xb[i].size() || (ia < xa[i].size() && xa[i][ia] < xb[i][ib])) {
                                xs[i].push_back(xa[i][ia]);
                                xp[i].push_back(pa[i][ia++]);
                            } else {
                                xs[i].push_back(xb[i][ib]);
                                xp[i].push_back(pb[i][ib++]);
                            }
                        }
                    }
                }
            }
            if (need_cc64)
                CK(cudaMemcpyAsync(hcc64.data(), L->kcc64.p, sizeof(double) * nb * k, cudaMemcpyDeviceToHost,
                               L->stream));
            CK(cudaStreamSynchronize(L->stream));
            for (int i = 0; i < nb; ++i) {
                cryoim_particle& q = parts[b0 + i];
                q.theta0 = q.theta; q.phi0 = q.phi; q.omega0 = q.omega; q.x0 = q.x; q.y0 = q.y; q.pr0 = q.pr;
                if (opts->pick == 0) {
                    int best = 0;
                    for (int j = 1; j < (int)xs[i].size(); ++j)
                        if (xp[i][j] < xp[i][best]) best = j;
                    const int n = xs[i][best];
                    q.theta = L->views[4 * (n / L->nom)];
                    q.phi = L->views[4 * (n / L->nom) + 1];
                    q.omega = L->p.searchstep * (float)(n % L->nom);
                    q.pr = xp[i][best];
                } else {
                    int best = 0;
                    for (int j = 1; j < k; ++j)
                        if (hcc64[i * k + j] > hcc64[i * k + best]) best = j;
                    const int sidx = i * k + best;
                    q.theta = hcand[5 * sidx]; q.phi = hcand[5 * sidx + 1]; q.omega = hcand[5 * sidx + 2];
                    q.x = hcand[5 * sidx + 3]; q.y = hcand[5 * sidx + 4];
                    q.pr = (float)hcc64[sidx];
                }
                q.dtheta = q.theta - q.theta0; q.dphi = q.phi - q.phi0; q.domega = q.omega - q.omega0;
                q.dx = q.x - q.x0; q.dy = q.y - q.y0; q.dpr = q.pr - q.pr0;
                if (cands)
                    for (int j = 0; j < k; ++j) {
                        const int a = i * k + j;
                        float* o = cands + ((size_t)(b0 + i) * k + j) * 8;
                        for (int e = 0; e < 5; ++e) o[e] = hcand[5 * a + e];
                        o[5] = hcc[a];
                        o[6] = (float)hcc64[a];
                        o[7] = 0.0f;
                        if (T > 0)
                            for (size_t m = 0; m < xs[i].size(); ++m)
                                if (xs[i][m] == hor[a]) { o[7] = xp[i][m]; break; }
                    }
            }
        }
        for (cudaEvent_t e : gev) cudaEventDestroy(e);
        return CRYOIM_OK;
    };
    if ((r = alloc(c))) return r;
    for (int i = 0; i + 1 < nlanes; ++i)
        if ((r = refresh_lane(c, i)) || (r = alloc(c->xlanes[i]))) return r;
    CK(cudaStreamSynchronize(c->stream));  // origins, sections and proposer ready for every lane
    if (nlanes == 1) return run(c, 0);
    std::vector<int> rx(nlanes - 1, CRYOIM_OK);
    std::vector<std::string> ex(nlanes - 1);
    std::vector<std::thread> th;
    for (int i = 0; i + 1 < nlanes; ++i) {
        Ctx* X = c->xlanes[i];
        X->prof_gemm_ms = 0.0;
        X->prof_gemm_launches = 0;
        X->prof_gemm_flops = 0.0;
        X->prof_pr_ms = 0.0;
        X->prof_pr_launches = 0;
        X->prof_pr_cands = 0.0;
        th.emplace_back([&, X, i] {
            if (cudaSetDevice(X->device) != cudaSuccess) {
                rx[i] = CRYOIM_ERR_CUDA;
                ex[i] = "cudaSetDevice failed in a pass lane";
                return;
            }
            rx[i] = run(X, i + 1);
            if (rx[i]) ex[i] = g_err;
        });
    }
    const int r0 = run(c, 0);
    for (std::thread& t : th) t.join();
    for (int i = 0; i + 1 < nlanes; ++i) {
        c->prof_gemm_ms += c->xlanes[i]->prof_gemm_ms;
        c->prof_gemm_launches += c->xlanes[i]->prof_gemm_launches;
        c->prof_gemm_flops += c->xlanes[i]->prof_gemm_flops;
        c->prof_pr_ms += c->xlanes[i]->prof_pr_ms;
        c->prof_pr_launches += c->xlanes[i]->prof_pr_launches;
        c->prof_pr_cands += c->xlanes[i]->prof_pr_cands;
    }
    if (r0) return r0;
    for (int i = 0; i + 1 < nlanes; ++i)
        if (rx[i]) return fail(rx[i], "%s", ex[i].c_str());
    return CRYOIM_OK;
}

// The learned form with its run-time fallback (cryoim_contract_opts.fallback): the
// particles whose phase residual lies more than t robust standard deviations above the
// call's median are searched again by the exhaustive contraction (same options, no
// proposals) and keep whichever result has the lower phase residual.
int contract_search_impl(Ctx* c, const float* imgs, bool on_device, cryoim_particle* parts, int P,
                         const cryoim_contract_opts* opts, float* cands) {
    if (c) c->last_fallbacks = 0;
    if (!c || !opts || !(opts->fallback >= 0.0f)) return contract_impl(c, imgs, on_device, parts, P, opts, cands);
    const bool fb = opts->fallback > 0.0f;
    if (fb && (opts->learned <= 0 || opts->pick != 0))
        return fail(CRYOIM_ERR_ARG, "fallback applies to the learned form with pick = 0");
    if (!fb || !parts || P < 1) return contract_impl(c, imgs, on_device, parts, P, opts, cands);
    std::vector<cryoim_particle> in(parts, parts + P);
    int r = contract_impl(c, imgs, on_device, parts, P, opts, cands);
    if (r) return r;
    std::vector<float> v(P);
    for (int i = 0; i < P; ++i) v[i] = parts[i].pr;
    auto median = [](std::vector<float> x) {
        const size_t m = x.size() / 2;
        std::nth_element(x.begin(), x.begin() + m, x.end());
        return x[m];
    };
    const float med = median(v);
    std::vector<float> dev(P);
    for (int i = 0; i < P; ++i) dev[i] = std::fabs(v[i] - med);
    const float thr = med + opts->fallback * 1.4826f * median(dev);
    std::vector<int> sel;
    for (int i = 0; i < P; ++i)
        if (v[i] > thr) sel.push_back(i);
    if (sel.empty()) return CRYOIM_OK;
    const int ns = (int)sel.size(), k = opts->topk;
    const long nn = (long)c->p.fftsize * c->p.fftsize;
    std::vector<cryoim_particle> sub(ns);
    for (int j = 0; j < ns; ++j) sub[j] = in[sel[j]];
    cryoim_contract_opts o2 = *opts;
    o2.learned = 0;
    o2.fallback = 0.0f;
    std::vector<float> c2(cands ? (size_t)ns * k * 8 : 0);
    if (on_device) {
        DBuf<float> d;
        if ((r = d.ensure((size_t)ns * nn))) return r;
        for (int j = 0; j < ns; ++j)
            CK(cudaMemcpyAsync(d.p + (size_t)j * nn, imgs + (size_t)sel[j] * nn, sizeof(float) * nn,
                               cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        r = contract_impl(c, d.p, true, sub.data(), ns, &o2, cands ? c2.data() : nullptr);
    } else {
        std::vector<float> h((size_t)ns * nn);
        for (int j = 0; j < ns; ++j) std::memcpy(&h[(size_t)j * nn], imgs + (size_t)sel[j] * nn, sizeof(float) * nn);
        r = contract_impl(c, h.data(), false, sub.data(), ns, &o2, cands ? c2.data() : nullptr);
    }
    if (r) return r;
    for (int j = 0; j < ns; ++j)
        if (sub[j].pr < parts[sel[j]].pr) {
            parts[sel[j]] = sub[j];
            if (cands) std::memcpy(cands + (size_t)sel[j] * k * 8, &c2[(size_t)j * k * 8], sizeof(float) * k * 8);
        }
    c->last_fallbacks = ns;
    return CRYOIM_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int32_t cryoim_version(void) { return 100; }

const char* cryoim_last_error(void) { return g_err.c_str(); }

int cryoim_params_default(cryoim_params* p, int32_t fftsize) {
    if (!p) return fail(CRYOIM_ERR_ARG, "null params");
    if (fftsize < 8 || (fftsize & 1)) return fail(CRYOIM_ERR_SIZE, "fftsize %d must be even and >= 8", fftsize);
    std::memset(p, 0, sizeof(*p));
    p->fftsize = fftsize;
    p->mode = 0;
    p->first = 1;
    p->last = 0;
    p->ncycle = 6;
    p->apply_ctf = 1;
    p->use_imgmask = 1;
    p->apix = 1.0f;
    p->min_res = 300.0f;
    p->max_res = 8.0f;
    p->imgmask = (float)(fftsize / 2 - 2);
    p->vol = 300.0f;
    p->cs = 2.7f;
    p->ampwg = 0.1f;
    p->bfactor = 0.0f;
    p->pr_threshold = 90.0f;
    p->searchstep = 2.0f;
    p->maxcentshift = 100.0f;
    p->boundx = (float)(fftsize / 2 - 2);
    p->nsym = 60;
    p->nlin = 60;
    return CRYOIM_OK;
}

int cryoim_params_derive(cryoim_params* p) {
    if (!p) return fail(CRYOIM_ERR_ARG, "null params");
    if (!(p->apix > 0) || !(p->min_res > 0) || !(p->max_res > 0))
        return fail(CRYOIM_ERR_ARG, "apix, minRes and maxRes must be positive");
    // 0calc_initialvalues.f90:6-21 (mode != 6)
    float minres = p->apix * (float)p->fftsize / p->min_res;
    float maxres = p->apix * (float)p->fftsize / p->max_res;
    p->min_r = (int)minres;
    p->max_r = (int)maxres;
    if (p->max_r % 2 != 0) p->max_r = p->max_r + 1;
    p->imgmask_px = p->use_imgmask ? p->imgmask / p->apix : p->imgmask;
    p->delta_angle = 360.0f / (maxres * sqrtf(5.0f) * 3.14159f);
    p->delta_trans = (float)p->fftsize / (maxres * sqrtf(5.0f));
    p->nsym = 60;
    p->nlin = 60;
    return CRYOIM_OK;
}

int cryoim_ctx_create(int32_t device, void** out) {
    if (!out) return fail(CRYOIM_ERR_ARG, "null output pointer");
    *out = nullptr;
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(CRYOIM_ERR_ARG, "device %d of %d", device, ndev);
    CK(cudaSetDevice(device));
    Ctx* c = new Ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(CRYOIM_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    c->own_stream = true;
    int r = c->ops.ensure(540);
    if (r) { delete c; return r; }
    e = cudaMemcpy(c->ops.p, table_ops(), sizeof(float) * 540, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete c;
        return fail(CRYOIM_ERR_CUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
    }
    *out = c;
    return CRYOIM_OK;
}

int cryoim_ctx_destroy(void* ctx) {
    if (!ctx) return CRYOIM_OK;
    delete as_ctx(ctx);
    return CRYOIM_OK;
}

int cryoim_ctx_set_stream(void* ctx, void* stream) {
    Ctx* c = as_ctx(ctx);
    if (!c) return fail(CRYOIM_ERR_ARG, "null context");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    if (stream) {
        c->stream = (cudaStream_t)stream;
        c->own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    for (auto& kv : c->plans) CKF(cufftSetStream(kv.second, c->stream));
    return CRYOIM_OK;
}

int cryoim_ctx_set_batch(void* ctx, int32_t batch) {
    Ctx* c = as_ctx(ctx);
    if (!c) return fail(CRYOIM_ERR_ARG, "null context");
    if (batch < 1 || batch > 65535) return fail(CRYOIM_ERR_ARG, "batch %d out of range", batch);
    c->batch = batch;
    return CRYOIM_OK;
}

int cryoim_ctx_set_lanes(void* ctx, int32_t lanes) {
    Ctx* c = as_ctx(ctx);
    if (!c) return fail(CRYOIM_ERR_ARG, "null context");
    if (lanes < 1 || lanes > 8) return fail(CRYOIM_ERR_ARG, "lanes %d out of range 1..8", lanes);
    c->lanes = lanes;
    return CRYOIM_OK;
}

int cryoim_ctx_set_profiling(void* ctx, int32_t on) {
    Ctx* c = as_ctx(ctx);
    if (!c) return fail(CRYOIM_ERR_ARG, "null context");
    CK(cudaSetDevice(c->device));
    if (on && !c->pe0) {
        CK(cudaEventCreate(&c->pe0));
        CK(cudaEventCreate(&c->pe1));
    }
    c->prof = on != 0;
    c->prof_ms = 0.0;
    c->prof_launches = 0;
    return CRYOIM_OK;
}

int cryoim_ctx_kernel_time(void* ctx, double* ms, int64_t* launches) {
    Ctx* c = as_ctx(ctx);
    if (!c || !ms || !launches) return fail(CRYOIM_ERR_ARG, "null argument");
    *ms = c->prof_ms;
    *launches = c->prof_launches;
    c->prof_ms = 0.0;
    c->prof_launches = 0;
    return CRYOIM_OK;
}

int cryoim_set_params(void* ctx, const cryoim_params* p) {
    Ctx* c = as_ctx(ctx);
    if (!c || !p) return fail(CRYOIM_ERR_ARG, "null argument");
    if (p->fftsize < 8 || (p->fftsize & 1) || p->fftsize > 2048)
        return fail(CRYOIM_ERR_SIZE, "fftsize %d unsupported (even, 8..2048)", p->fftsize);
    if (p->min_r < 0 || p->max_r < p->min_r)
        return fail(CRYOIM_ERR_ARG, "minR=%d maxR=%d (derive the parameters first)", p->min_r, p->max_r);
    if (p->max_r > p->fftsize / 2 - 2)
        return fail(CRYOIM_ERR_SIZE, "maxR=%d exceeds FFTsize/2-2=%d", p->max_r, p->fftsize / 2 - 2);
    if (!(p->searchstep > 0)) return fail(CRYOIM_ERR_ARG, "searchstep must be positive");
    if (p->nsym != 60) return fail(CRYOIM_ERR_ARG, "only sym=icos (nsym=60) is on this path");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    bool geom_changed = !c->have_params || c->p.fftsize != p->fftsize || c->p.min_r != p->min_r ||
                        c->p.max_r != p->max_r;
    bool step_changed = !c->have_params || c->p.searchstep != p->searchstep;
    c->p = *p;
    c->bd = make_band(p->fftsize, p->min_r, p->max_r);
    c->have_params = true;
    if (geom_changed) {
        for (auto& kv : c->plans) cufftDestroy(kv.second);
        c->plans.clear();
        c->T = 0;  // templates depend on the band geometry
        c->grid_ready = false;
        c->rec_active = false;
        c->map_ready = false;
        c->cS = 0;
        c->bmat_ready = false;
        c->bmat8_ready = false;
        c->cS_c = 0;
        c->bmat_c_ready = false;
    }
    if (step_changed) {
        c->grid_ready = false;
        c->bmat_ready = false;
        c->bmat8_ready = false;
        c->bmat_c_ready = false;
    }
    long nn = (long)p->fftsize * p->fftsize;
    c->batch = (int)std::max(1L, std::min(64L, (long)(16L * 1024 * 1024) / nn));
    return CRYOIM_OK;
}

int cryoim_load_templates(void* ctx, const float* tmpl_real, const cryoim_template* t, int32_t T) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!tmpl_real || !t || T < 1) return fail(CRYOIM_ERR_ARG, "templates: null input or T < 1");
    const int nx = c->p.fftsize;
    const long nn = (long)nx * nx, w2 = (long)c->bd.W * c->bd.W;
    c->T = 0;
    c->grid_ready = false;
    c->tmpl.assign(t, t + T);
    if ((r = c->tband.ensure((size_t)T * w2))) return r;
    if ((r = c->tfcut0.ensure((size_t)T * c->bd.nr))) return r;
    if ((r = c->tort.ensure((size_t)T * 3))) return r;
    std::vector<float> tort(3 * T);
    for (int i = 0; i < T; ++i) { tort[3 * i] = t[i].theta; tort[3 * i + 1] = t[i].phi; tort[3 * i + 2] = t[i].omega; }
    CK(cudaMemcpyAsync(c->tort.p, tort.data(), sizeof(float) * 3 * T, cudaMemcpyHostToDevice, c->stream));
    const int B = c->batch;
    if ((r = ensure_batch(c, B))) return r;
    std::vector<float> hpar(8 * B);
    for (int b0 = 0; b0 < T; b0 += B) {
        const int nb = std::min(B, T - b0);
        CK(cudaMemcpyAsync(c->imgs.p, tmpl_real + b0 * nn, sizeof(float) * nb * nn,
                           cudaMemcpyHostToDevice, c->stream));
        std::fill(hpar.begin(), hpar.end(), 0.0f);
        for (int i = 0; i < nb; ++i) {
            hpar[i] = t[b0 + i].x; hpar[B + i] = t[b0 + i].y;
            hpar[2 * B + i] = t[b0 + i].x; hpar[3 * B + i] = t[b0 + i].y;
        }
        // load_template.f90:36-47
        if ((r = transform_batch(c, c->imgs.p, nb, B, hpar, c->p.use_imgmask, 0, true))) return r;
        CK(cudaMemcpyAsync(c->tband.p + b0 * w2, c->band.p, sizeof(float2) * nb * w2,
                           cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(c->tfcut0.p + (long)b0 * c->bd.nr, c->fcut0.p,
                           sizeof(float) * nb * c->bd.nr, cudaMemcpyDeviceToDevice, c->stream));
        if ((r = check_flag(c))) return r;
    }
    c->T = T;
    if ((r = ensure_batch(c, B))) return r;  // tfcut sized for T
    return CRYOIM_OK;
}

int cryoim_project_templates(void* ctx, const float* map3d, const cryoim_template* t, int32_t T,
                             float* out) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!map3d || !t || !out || T < 1) return fail(CRYOIM_ERR_ARG, "null input or T < 1");
    const int nx = c->p.fftsize;
    const long nn = (long)nx * nx, n3 = nn * nx;
    DBuf<float> dmap, deul, dout;
    if ((r = dmap.ensure(n3)) || (r = deul.ensure(3 * T)) || (r = dout.ensure((size_t)T * nn))) return r;
    std::vector<float> eul(3 * T);
    for (int i = 0; i < T; ++i) { eul[3 * i] = t[i].theta; eul[3 * i + 1] = t[i].phi; eul[3 * i + 2] = t[i].omega; }
    CK(cudaMemcpyAsync(dmap.p, map3d, sizeof(float) * n3, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(deul.p, eul.data(), sizeof(float) * 3 * T, cudaMemcpyHostToDevice, c->stream));
    launch_project(dmap.p, nx, deul.p, T, dout.p, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout.p, sizeof(float) * T * nn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

int cryoim_search_grid(void* ctx, int32_t* ntheta, int32_t* nphi, int32_t* nomega, int32_t* nviews) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, true);
    if (r) return r;
    if ((r = ensure_grid(c))) return r;
    if (ntheta) *ntheta = c->nth;
    if (nphi) *nphi = c->nph;
    if (nomega) *nomega = c->nom;
    if (nviews) *nviews = c->V;
    return CRYOIM_OK;
}

int cryoim_search_terms(void* ctx, double* terms) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, true);
    if (r) return r;
    if (!terms) return fail(CRYOIM_ERR_ARG, "null output");
    if ((r = ensure_grid(c))) return r;
    std::vector<float2> al((size_t)c->V * c->T * 60);
    if (!al.empty()) {
        CK(cudaMemcpyAsync(al.data(), c->alpha.p, sizeof(float2) * al.size(), cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    long long lines = 0;
    for (const float2& a : al) lines += (a.x < 999.0f && a.y < 999.0f);
    *terms = (double)lines * c->bd.nr * c->nom;
    return CRYOIM_OK;
}

int cryoim_globesearch(void* ctx, const float* imgs, cryoim_particle* parts, int32_t P,
                       float* pr_array) {
    return globesearch_impl(as_ctx(ctx), imgs, false, parts, P, pr_array);
}

int cryoim_globesearch_device(void* ctx, const float* d_imgs, cryoim_particle* parts, int32_t P,
                              float* pr_array) {
    return globesearch_impl(as_ctx(ctx), d_imgs, true, parts, P, pr_array);
}

int cryoim_prscore_omega(void* ctx, const float* ft_a, const float* ft_b, const float* fcut0,
                         const float* ctf, float theta, float phi, float* pr_omega) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, true);
    if (r) return r;
    if (!ft_a || !ft_b || !fcut0 || !pr_omega) return fail(CRYOIM_ERR_ARG, "null argument");
    const int nx = c->p.fftsize, W = c->bd.W, off = c->bd.off, nr = c->bd.nr, T = c->T;
    const float step = c->p.searchstep;
    const int nom = (int)(360.0f / step);
    if (nom < 1 || nom > 768) return fail(CRYOIM_ERR_SIZE, "Nomega=%d unsupported", nom);
    if ((r = ensure_batch(c, c->batch))) return r;
    std::vector<float2> band((size_t)W * W);
    std::vector<float> cband(ctf ? (size_t)W * W : 0);
    for (int y = 0; y < W; ++y)
        for (int x = 0; x < W; ++x) {
            long i = (long)(off + y) * nx + (off + x);
            band[(size_t)y * W + x] = make_float2(ft_a[i], ft_b[i]);
            if (ctf) cband[(size_t)y * W + x] = ctf[i];
        }
    CK(cudaMemcpyAsync(c->band.p, band.data(), sizeof(float2) * W * W, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->fcut0.p, fcut0, sizeof(float) * nr, cudaMemcpyHostToDevice, c->stream));
    float hv[4] = {theta, phi, 0.f, 0.f};
    int zero = 0;
    std::memcpy(&hv[2], &zero, 4);
    DBuf<float> dv;
    DBuf<float2> dal;
    DBuf<float> dprs;
    if ((r = dv.ensure(4)) || (r = dal.ensure((size_t)T * 60)) || (r = dprs.ensure(nom))) return r;
    CK(cudaMemcpyAsync(dv.p, hv, sizeof(hv), cudaMemcpyHostToDevice, c->stream));
    launch_alpha_table(dv.p, 1, c->tort.p, T, c->ops.p, dal.p, c->stream);
    // the view array of launch_alpha_table is (theta, phi) pairs: pass hv's first two
    const float* tfc = c->tfcut0.p;
    long tfs = 0;
    const float* ctfp = nullptr;
    if (ctf) {
        CK(cudaMemcpyAsync(c->ctf.p, cband.data(), sizeof(float) * W * W, cudaMemcpyHostToDevice, c->stream));
        launch_tmpl_fcut(c->tband.p, T, c->ctf.p, 1, c->bd, c->tfcut.p, c->stream);
        ctfp = c->ctf.p;
        tfc = c->tfcut.p;
        tfs = (long)T * nr;
    }
    unsigned long long k0 = key_of(1000.0f, 0u);
    CK(cudaMemcpyAsync(c->best.p, &k0, sizeof(k0), cudaMemcpyHostToDevice, c->stream));
    PrOmegaArgs a{};
    a.band = c->band.p; a.fcut0 = c->fcut0.p; a.tband = c->tband.p; a.tfcut = tfc;
    a.tfcut_pstride = tfs; a.ctf = ctfp; a.alpha = dal.p; a.views = dv.p; a.V = 1; a.T = T;
    a.nomega = nom; a.step = step; a.bd = c->bd; a.best = c->best.p; a.pr_array = dprs.p; a.per = nom;
    CK(launch_pr_omega(a, 1, c->stream));
    CK(cudaMemcpyAsync(pr_omega, dprs.p, sizeof(float) * nom, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

int cryoim_refine(void* ctx, const float* imgs, cryoim_particle* parts, int32_t P) {
    return refine_impl(as_ctx(ctx), imgs, false, parts, P);
}

int cryoim_refine_device(void* ctx, const float* d_imgs, cryoim_particle* parts, int32_t P) {
    return refine_impl(as_ctx(ctx), d_imgs, true, parts, P);
}

int cryoim_prscore(void* ctx, const float* ft_a, const float* ft_b, const float* fcut0,
                   const float* ctf, float theta, float phi, float omega, float x, float y,
                   float* pr) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, true);
    if (r) return r;
    if (!ft_a || !ft_b || !fcut0 || !pr) return fail(CRYOIM_ERR_ARG, "null argument");
    const int nx = c->p.fftsize, W = c->bd.W, off = c->bd.off, nr = c->bd.nr, T = c->T;
    if ((r = ensure_batch(c, c->batch))) return r;
    if ((r = c->cand.ensure(55)) || (r = c->rpr.ensure(11)) || (r = c->ralpha.ensure((size_t)11 * T * 60)))
        return r;
    std::vector<float2> band((size_t)W * W);
    std::vector<float> cband(ctf ? (size_t)W * W : 0);
    for (int yy = 0; yy < W; ++yy)
        for (int xx = 0; xx < W; ++xx) {
            long i = (long)(off + yy) * nx + (off + xx);
            band[(size_t)yy * W + xx] = make_float2(ft_a[i], ft_b[i]);
            if (ctf) cband[(size_t)yy * W + xx] = ctf[i];
        }
    CK(cudaMemcpyAsync(c->band.p, band.data(), sizeof(float2) * W * W, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->fcut0.p, fcut0, sizeof(float) * nr, cudaMemcpyHostToDevice, c->stream));
    std::vector<float> hc(55);
    for (int j = 0; j < 11; ++j) { hc[5 * j] = theta; hc[5 * j + 1] = phi; hc[5 * j + 2] = omega; hc[5 * j + 3] = x; hc[5 * j + 4] = y; }
    CK(cudaMemcpyAsync(c->cand.p, hc.data(), sizeof(float) * 55, cudaMemcpyHostToDevice, c->stream));
    launch_refine_alpha(c->cand.p, 1, c->tort.p, T, c->ops.p, c->ralpha.p, c->stream);
    const float* tfc = c->tfcut0.p;
    long tfs = 0;
    const float* ctfp = nullptr;
    if (ctf) {
        CK(cudaMemcpyAsync(c->ctf.p, cband.data(), sizeof(float) * W * W, cudaMemcpyHostToDevice, c->stream));
        launch_tmpl_fcut(c->tband.p, T, c->ctf.p, 1, c->bd, c->tfcut.p, c->stream);
        ctfp = c->ctf.p;
        tfc = c->tfcut.p;
        tfs = (long)T * nr;
    }
    PrSingleArgs a{};
    a.band = c->band.p; a.fcut0 = c->fcut0.p; a.tband = c->tband.p; a.tfcut = tfc;
    a.tfcut_pstride = tfs; a.ctf = ctfp; a.cand = c->cand.p; a.alpha = c->ralpha.p; a.T = T;
    a.bd = c->bd; a.pr = c->rpr.p;
    CK(launch_pr_single(a, 1, c->stream));
    float out[11];
    CK(cudaMemcpyAsync(out, c->rpr.p, sizeof(float) * 11, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *pr = out[0];
    return CRYOIM_OK;
}

// The end of every map-producing routine, on c->vol (nx^3 complex, filled by a fold):
// 3D FFT in direction dir (cuFFT unnormalised, as FFTW's backward and Singleton's
// isn = -1 transforms are), then either shift3dComplex + real part (reconstruct.f90:
// 246-247) or the masked real part of merge_reconstruct_FSC.f90:190-198 (merge_mask),
// then the real-space icosahedral average at imgmask when avg is set, into host map.
static int finish_volume(Ctx* c, int dir, bool merge_mask, bool avg, float* map) {
    const int nx = c->p.fftsize;
    const long n3 = (long)nx * nx * nx;
    cufftHandle h;
    CKF(cufftPlan3d(&h, nx, nx, nx, CUFFT_C2C));
    cufftResult fr = cufftSetStream(h, c->stream);
    if (fr == CUFFT_SUCCESS) fr = cufftExecC2C(h, (cufftComplex*)c->vol.p, (cufftComplex*)c->vol.p, dir);
    if (fr != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return fail(CRYOIM_ERR_CUDA, "3D FFT failed: cufft %d", (int)fr);
    }
    DBuf<float> dmap, davg;
    int r;
    if ((r = dmap.ensure(n3)) || (avg && (r = davg.ensure(n3)))) { cufftDestroy(h); return r; }
    cudaError_t e = merge_mask ? launch_merge_real(c->vol.p, nx, c->p.imgmask_px, dmap.p, c->stream)
                               : (launch_rec_real(c->vol.p, nx, dmap.p, c->stream), cudaGetLastError());
    if (e == cudaSuccess && avg) e = launch_icosavg(dmap.p, nx, c->p.imgmask_px, c->ops.p, 60, davg.p, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(map, avg ? davg.p : dmap.p, sizeof(float) * n3, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cufftDestroy(h);
    if (e != cudaSuccess) return fail(CRYOIM_ERR_CUDA, "map finish: %s", cudaGetErrorString(e));
    return CRYOIM_OK;
}

// kind: REC_FULL (reconstruct.f90), REC_SUBSTEP (reconstruct_substep.f90) or REC_HALF
// (reconstruct_half.f90, mask origin given by the caller).
static int rec_begin_impl(Ctx* c, int kind, const float* mask_origin) {
    int r = check_ready(c, false);
    if (r) return r;
    const Band& bd = c->bd;
    const int R = bd.max_r, nx = c->p.fftsize;
    const long nacc = (long)bd.AW * bd.AW * (R + 2);
    if ((r = c->acc.ensure(nacc))) return r;
    // reconstruct.f90:26-28 (wg = 0.01), reconstruct_substep.f90:23-25 and
    // reconstruct_half.f90:17 (wg = 0)
    const float wg0 = kind == REC_FULL ? 0.01f : 0.0f;
    std::vector<float4> init(nacc, make_float4(0.f, 0.f, wg0, 0.f));
    CK(cudaMemcpyAsync(c->acc.p, init.data(), sizeof(float4) * nacc, cudaMemcpyHostToDevice, c->stream));
    // insertion samples: reconstruct.f90:103-106 and reconstruct_half.f90:95-96 (r <= maxR),
    // reconstruct_substep.f90:101-104 (r <= maxR-2)
    const float lim = kind == REC_SUBSTEP ? (float)(R - 2) : (float)R;
    std::vector<int2> smp;
    for (int ky = -R; ky <= R; ++ky)
        for (int hx = 0; hx <= R; ++hx) {
            float dr = sqrtf((float)(hx * hx + ky * ky));
            if (dr <= lim) smp.push_back(make_int2(hx, ky));
        }
    c->nsamples = (int)smp.size();
    if ((r = c->samples.ensure(smp.size() + 1))) return r;
    CK(cudaMemcpyAsync(c->samples.p, smp.data(), sizeof(int2) * smp.size(), cudaMemcpyHostToDevice, c->stream));
    if (kind != REC_FULL) {
        // reconstruct_substep.f90:121, reconstruct_half.f90:114: x0(1:2) += maxR, z
        // unshifted; tnf cell lx -> box lx+1
        c->rec_off_xy = (float)R; c->rec_off_z = 0.0f; c->rec_base_xy = -1; c->rec_base_z = 0;
    } else {
        c->rec_off_xy = (float)(nx / 2); c->rec_off_z = (float)(nx / 2);
        c->rec_base_xy = nx / 2 - R - 1; c->rec_base_z = nx / 2;
    }
    CK(cudaStreamSynchronize(c->stream));
    c->rec_kind = kind;
    c->rec_active = true;
    c->rec_used = 0;
    c->rec_img_id0 = -100;
    c->rec_have_first = mask_origin != nullptr;
    if (mask_origin) { c->rec_ox = mask_origin[0]; c->rec_oy = mask_origin[1]; }
    return CRYOIM_OK;
}

int cryoim_rec_begin(void* ctx) {
    Ctx* c = as_ctx(ctx);
    return rec_begin_impl(c, c->p.subrec ? REC_SUBSTEP : REC_FULL, nullptr);
}

int cryoim_rec_begin_half(void* ctx, float mask_x, float mask_y) {
    const float o[2] = {mask_x, mask_y};
    return rec_begin_impl(as_ctx(ctx), REC_HALF, o);
}

int cryoim_rec_insert(void* ctx, const float* imgs, const cryoim_particle* parts, int32_t P,
                      int32_t* used) {
    return rec_insert_impl(as_ctx(ctx), imgs, false, parts, P, used);
}

int cryoim_rec_insert_device(void* ctx, const float* d_imgs, const cryoim_particle* parts,
                             int32_t P, int32_t* used) {
    return rec_insert_impl(as_ctx(ctx), d_imgs, true, parts, P, used);
}

int cryoim_rec_finish(void* ctx, float* map) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!c->rec_active) return fail(CRYOIM_ERR_STATE, "cryoim_rec_begin has not been called");
    if (!map) return fail(CRYOIM_ERR_ARG, "null map");
    if (c->rec_kind != REC_FULL)
        return fail(CRYOIM_ERR_STATE, "tnf accumulation (subrec or half map) has no map: use "
                                      "cryoim_rec_get_partial (and cryoim_fsc_combine for half maps)");
    const int nx = c->p.fftsize;
    const long n3 = (long)nx * nx * nx;
    if ((r = c->vol.ensure(n3))) return r;
    CK(cudaMemsetAsync(c->vol.p, 0, sizeof(float2) * n3, c->stream));
    launch_rec_fold(c->acc.p, c->bd, 0, c->vol.p, c->stream);
    CK(cudaGetLastError());
    // reconstruct.f90:243-255: backward FFT, shift, real part, icosavg if realspaceavg
    return finish_volume(c, CUFFT_INVERSE, false, c->p.realspaceavg != 0, map);
}

int cryoim_rec_finish_merge(void* ctx, float* map) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!c->rec_active) return fail(CRYOIM_ERR_STATE, "cryoim_rec_begin has not been called");
    if (!map) return fail(CRYOIM_ERR_ARG, "null map");
    if (c->rec_kind != REC_FULL) return fail(CRYOIM_ERR_STATE, "merge sums into a full accumulation");
    const int nx = c->p.fftsize;
    const long n3 = (long)nx * nx * nx;
    if ((r = c->vol.ensure(n3))) return r;
    CK(cudaMemsetAsync(c->vol.p, 0, sizeof(float2) * n3, c->stream));
    launch_rec_fold(c->acc.p, c->bd, 1, c->vol.p, c->stream);
    CK(cudaGetLastError());
    return finish_volume(c, CUFFT_INVERSE, false, false, map);
}

int cryoim_icosavg(void* ctx, float* map, int32_t n, float r0) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!map || n < 2) return fail(CRYOIM_ERR_ARG, "null map or n < 2");
    const long n3 = (long)n * n * n;
    DBuf<float> a, b;
    if ((r = a.ensure(n3)) || (r = b.ensure(n3))) return r;
    CK(cudaMemcpyAsync(a.p, map, sizeof(float) * n3, cudaMemcpyHostToDevice, c->stream));
    CK(launch_icosavg(a.p, n, r0, c->ops.p, 60, b.p, c->stream));
    CK(cudaMemcpyAsync(map, b.p, sizeof(float) * n3, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

int cryoim_rec_get_partial(void* ctx, float* fa, float* fb, float* wg) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!c->rec_active) return fail(CRYOIM_ERR_STATE, "cryoim_rec_begin has not been called");
    if (!fa || !fb || !wg) return fail(CRYOIM_ERR_ARG, "null output");
    const Band& bd = c->bd;
    const int R = bd.max_r, AW = bd.AW, t = 2 * R + 1;
    const long nacc = (long)AW * AW * (R + 2);
    std::vector<float4> h(nacc);
    CK(cudaMemcpyAsync(h.data(), c->acc.p, sizeof(float4) * nacc, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // tnf cell (x, y, z), x = hx + maxR, is box cell (hx, ky, lz) = acc_cell(x - R, y - R, z)
    for (int z = 0; z <= R; ++z)
        for (int y = 0; y < t; ++y)
            for (int x = 0; x < t; ++x) {
                const float4& v = h[acc_cell(bd, x - R, y - R, z)];
                long o = ((long)z * t + y) * t + x;
                fa[o] = v.x; fb[o] = v.y; wg[o] = v.z;
            }
    if (c->rec_kind != REC_FULL) {
        // The reference indexes its tnf box linearly (cubID = lz t^2 + ly t + lx + 1,
        // reconstruct_half.f90:127-130): a trilinear corner at x = t (or y = t) lands on
        // the next row (plane).  Corners at z = maxR+1 fall past its array: dropped.
        const long tnf = (long)(R + 1) * t * t;
        for (int z = 0; z <= R + 1; ++z)
            for (int y = 0; y <= t; ++y)
                for (int x = 0; x <= t; ++x) {
                    if (x < t && y < t && z <= R) continue;
                    const long o = ((long)z * t + y) * t + x;
                    if (o >= tnf) continue;
                    const float4& v = h[acc_cell(bd, x - R, y - R, z)];
                    fa[o] += v.x; fb[o] += v.y; wg[o] += v.z;
                }
    }
    return CRYOIM_OK;
}

// reconstruct_FSC.f90:25-187 (merge = false) or merge_reconstruct_FSC.f90:37-198 (merge =
// true; the same FSC, weighting and fold, a different transform and output step).
static int fsc_impl(Ctx* c, const float* const src[6], float* fsc, float* map, bool merge) {
    int r = check_ready(c, false);
    if (r) return r;
    for (int i = 0; i < 6; ++i)
        if (!src[i]) return fail(CRYOIM_ERR_ARG, "null tnf input");
    const int nx = c->p.fftsize, R = c->p.max_r, t = 2 * R + 1, ns = R + 1;
    const long tnf = (long)ns * t * t, n3 = (long)nx * nx * nx;
    DBuf<float> d;
    DBuf<double> sums;
    DBuf<float> wt;
    if ((r = d.ensure(6 * tnf)) || (r = sums.ensure(3 * ns)) || (r = wt.ensure(ns))) return r;
    for (int i = 0; i < 6; ++i)
        CK(cudaMemcpyAsync(d.p + i * tnf, src[i], sizeof(float) * tnf, cudaMemcpyHostToDevice, c->stream));
    FscArgs a{};
    a.fa1 = d.p; a.fb1 = d.p + tnf; a.wg1 = d.p + 2 * tnf;
    a.fa2 = d.p + 3 * tnf; a.fb2 = d.p + 4 * tnf; a.wg2 = d.p + 5 * tnf;
    a.nx = nx; a.max_r = R;
    if (c->num_sms == 0) CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
    CK(launch_fsc_shells(a, sums.p, c->num_sms, c->stream));
    std::vector<double> hs(3 * ns);
    CK(cudaMemcpyAsync(hs.data(), sums.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // reconstruct_FSC.f90:43-62: FSC1 = FSC2 = 1e-10 at start; weight sqrt(2F/(1+F)), 0 if F <= 0
    std::vector<float> hw(ns);
    for (int i = 0; i < ns; ++i) {
        const float F = (float)(hs[i] / std::sqrt((1e-10 + hs[ns + i]) * (1e-10 + hs[2 * ns + i])));
        if (fsc) fsc[i] = F;
        hw[i] = F <= 0.0f ? 0.0f : std::sqrt(2.0f * F / (1.0f + F));
    }
    if (!map) return CRYOIM_OK;
    CK(cudaMemcpyAsync(wt.p, hw.data(), sizeof(float) * ns, cudaMemcpyHostToDevice, c->stream));
    if ((r = c->vol.ensure(n3))) return r;
    CK(launch_fsc_fold(a, wt.p, c->vol.p, c->stream));
    if (merge)  // merge_reconstruct_FSC.f90:184-198: Singleton isn = -1 transform, masked real part
        return finish_volume(c, CUFFT_FORWARD, true, false, map);
    // reconstruct_FSC.f90:177-187: backward FFT, shift, real part, icosavg if realspaceavg
    return finish_volume(c, CUFFT_INVERSE, false, c->p.realspaceavg != 0, map);
}

int cryoim_fsc_combine(void* ctx, const float* fa1, const float* fb1, const float* wg1, const float* fa2,
                       const float* fb2, const float* wg2, float* fsc, float* map) {
    const float* in[6] = {fa1, fb1, wg1, fa2, fb2, wg2};
    return fsc_impl(as_ctx(ctx), in, fsc, map, false);
}

int cryoim_merge_fsc_combine(void* ctx, const float* fa1, const float* fb1, const float* wg1,
                             const float* fa2, const float* fb2, const float* wg2, float* fsc, float* map) {
    const float* in[6] = {fa1, fb1, wg1, fa2, fb2, wg2};
    return fsc_impl(as_ctx(ctx), in, fsc, map, true);
}

int cryoim_rec_add_partial(void* ctx, const float* fa, const float* fb, const float* wg) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!c->rec_active) return fail(CRYOIM_ERR_STATE, "cryoim_rec_begin has not been called");
    if (!fa || !fb || !wg) return fail(CRYOIM_ERR_ARG, "null input");
    const Band& bd = c->bd;
    const int R = bd.max_r, t = 2 * R + 1;
    const long nacc = (long)bd.AW * bd.AW * (R + 2);
    std::vector<float4> h(nacc);
    CK(cudaMemcpyAsync(h.data(), c->acc.p, sizeof(float4) * nacc, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int z = 0; z <= R; ++z)
        for (int y = 0; y < t; ++y)
            for (int x = 0; x < t; ++x) {
                const long i = ((long)z * t + y) * t + x;
                float4& v = h[acc_cell(bd, x - R, y - R, z)];
                v.x += fa[i];
                v.y += fb[i];
                v.z += wg[i];
            }
    CK(cudaMemcpyAsync(c->acc.p, h.data(), sizeof(float4) * nacc, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

// icosprocess mode 3.  With map3d: calc_center.f90:22-105 (the map masked by img3d_mask
// and transformed once; per particle the image masked at its origin and low-passed, the
// model's projection at its orientation with the CTF, masked at the centre and
// low-passed, both normalised, cross-correlated, Gaussian fit of the peak).  Without:
// calc_center_selfrot180.f90:22-86 (the image against itself rotated by 180 degrees,
// half the peak offset).
int cryoim_center(void* ctx, const float* map3d, const float* imgs, cryoim_particle* parts, int32_t P) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!imgs || !parts || P < 0) return fail(CRYOIM_ERR_ARG, "null input or negative count");
    if (P == 0) return CRYOIM_OK;
    const int nx = c->p.fftsize, B = c->batch, R = c->p.max_r;
    const long nn = (long)nx * nx, n3 = nn * nx;
    const bool model = map3d != nullptr, mask = c->p.use_imgmask != 0;
    if ((r = ensure_batch(c, B))) return r;
    DBuf<float2> f2;
    DBuf<float> a1, a2, ore, oim, ctfb, eul, out, fr, fi;
    DBuf<double> acc2;
    if ((r = f2.ensure((size_t)B * nn)) || (r = a1.ensure((size_t)B * nn)) || (r = a2.ensure((size_t)B * nn)) ||
        (r = out.ensure((size_t)3 * B)) || (r = acc2.ensure(2)))
        return r;
    if (model && ((r = ore.ensure((size_t)B * nn)) || (r = oim.ensure((size_t)B * nn)) ||
                  (r = ctfb.ensure((size_t)B * nn)) || (r = eul.ensure((size_t)3 * B)) || (r = fr.ensure(n3)) ||
                  (r = fi.ensure(n3))))
        return r;
    if (model) {  // calc_center.f90:24-38
        DBuf<float> dmap;
        DBuf<float2> work;
        if ((r = dmap.ensure(n3)) || (r = work.ensure(n3))) return r;
        CK(cudaMemcpyAsync(dmap.p, map3d, sizeof(float) * n3, cudaMemcpyHostToDevice, c->stream));
        if (mask) CK(launch_mask3d(dmap.p, nx, c->p.imgmask_px, acc2.p, c->stream));
        launch_map_checker(dmap.p, nx, work.p, c->stream);
        cufftHandle h3;
        CKF(cufftPlan3d(&h3, nx, nx, nx, CUFFT_C2C));
        cufftResult fr3 = cufftSetStream(h3, c->stream);
        if (fr3 == CUFFT_SUCCESS) fr3 = cufftExecC2C(h3, (cufftComplex*)work.p, (cufftComplex*)work.p, CUFFT_FORWARD);
        cudaError_t e = fr3 == CUFFT_SUCCESS ? launch_center_ft(work.p, nx, fr.p, fi.p, c->stream) : cudaSuccess;
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cufftDestroy(h3);
        if (fr3 != CUFFT_SUCCESS) return fail(CRYOIM_ERR_CUDA, "3D forward FFT failed: cufft %d", (int)fr3);
        if (e != cudaSuccess) return fail(CRYOIM_ERR_CUDA, "centring map: %s", cudaGetErrorString(e));
    }
    // a forward or backward transform of the first nb images of buf, img2d_FFT-style
    auto xform = [&](float2* buf, int nb, bool fwd) -> int {
        cufftHandle h;
        if ((r = plan2d(c, nb, &h))) return r;
        CKF(cufftExecC2C(h, (cufftComplex*)buf, (cufftComplex*)buf, fwd ? CUFFT_FORWARD : CUFFT_INVERSE));
        launch_ref_post(buf, (long)nb * nn, fwd ? (float)nn : 1.0f, c->stream);
        return CRYOIM_OK;
    };
    // img2d_lowpass of the shifted complex images in buf (from prep or pack), into real dst
    auto lowpass = [&](float2* buf, int nb, float* dst) -> int {
        if ((r = xform(buf, nb, true))) return r;
        launch_lowpass(buf, nx, (long)nb * nn, R, c->stream);
        if ((r = xform(buf, nb, false))) return r;
        launch_real_shift(buf, nx, (long)nb * nn, dst, c->stream);
        return CRYOIM_OK;
    };
    Band bf{};  // the full nx x nx CTF through the band kernel: window = whole image
    bf.nx = nx; bf.max_r = nx / 2; bf.W = nx;
    const ParView pv = par_view(c, B);
    std::vector<float> hpar(8 * B), heul(3 * B), hout(3 * B);
    int id0 = -100;
    float sdf[3] = {0, 0, 0};
    for (int b0 = 0; b0 < P; b0 += B) {
        const int nb = std::min(B, P - b0);
        const long m = (long)nb * nn;
        CK(cudaMemcpyAsync(c->imgs.p, imgs + b0 * nn, sizeof(float) * m, cudaMemcpyHostToDevice, c->stream));
        std::fill(hpar.begin(), hpar.end(), 0.0f);
        for (int i = 0; i < nb; ++i) {
            const cryoim_particle& q = parts[b0 + i];
            if (model) { hpar[i] = q.x; hpar[B + i] = q.y; }
            if (q.img_id != id0) { sdf[0] = q.df1; sdf[1] = q.df2; sdf[2] = q.astigang; id0 = q.img_id; }
            hpar[4 * B + 3 * i] = sdf[0]; hpar[4 * B + 3 * i + 1] = sdf[1]; hpar[4 * B + 3 * i + 2] = sdf[2];
            heul[3 * i] = q.theta; heul[3 * i + 1] = q.phi; heul[3 * i + 2] = q.omega;
        }
        CK(cudaMemcpyAsync(c->par.p, hpar.data(), sizeof(float) * 8 * B, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
        if (model) {
            // a1: mask at the particle's origin, low pass (calc_center.f90:55-56)
            if (mask) launch_prep_images(c->imgs.p, nb, nx, pv.ox, pv.oy, 1, c->p.imgmask_px, 0, c->fft.p, c->flag.p,
                                         c->stream);
            else launch_pack_shift(c->imgs.p, nullptr, nx, m, c->fft.p, c->stream);
            if ((r = lowpass(c->fft.p, nb, a1.p))) return r;
            // a2: projection of the model (project2d_FT3dTo2d.f90), CTF, mask, low pass (:57-67)
            CK(cudaMemcpyAsync(eul.p, heul.data(), sizeof(float) * 3 * nb, cudaMemcpyHostToDevice, c->stream));
            launch_sections(fr.p, fi.p, nx, eul.p, nb, ore.p, oim.p, c->stream);
            launch_pack_shift(ore.p, oim.p, nx, m, f2.p, c->stream);
            if ((r = xform(f2.p, nb, false))) return r;
            launch_real_shift(f2.p, nx, m, a2.p, c->stream);
            if (c->p.apply_ctf) {  // img2d_applyCTF.f90
                launch_ctf_band(nb, bf, pv.dfs, c->p.apix, c->p.vol, c->p.cs, c->p.ampwg, ctfb.p, c->stream);
                launch_pack_shift(a2.p, nullptr, nx, m, f2.p, c->stream);
                if ((r = xform(f2.p, nb, true))) return r;
                launch_ctf_mul(f2.p, ctfb.p, m, c->stream);
                if ((r = xform(f2.p, nb, false))) return r;
                launch_real_shift(f2.p, nx, m, a2.p, c->stream);
            }
            if (mask) launch_prep_images(a2.p, nb, nx, pv.sx, pv.sy, 1, c->p.imgmask_px, 0, f2.p, c->flag.p,
                                         c->stream);  // sx, sy are zero here: the centre
            else launch_pack_shift(a2.p, nullptr, nx, m, f2.p, c->stream);
            if ((r = lowpass(f2.p, nb, a2.p))) return r;
            launch_norm(a1.p, nx, nb, c->stream);
            launch_norm(a2.p, nx, nb, c->stream);
        } else {
            // calc_center_selfrot180.f90:39-52: low pass, mask at the centre, norm, rotate
            launch_pack_shift(c->imgs.p, nullptr, nx, m, c->fft.p, c->stream);
            if ((r = lowpass(c->fft.p, nb, a1.p))) return r;
            if (mask) {
                launch_prep_images(a1.p, nb, nx, pv.ox, pv.oy, 1, c->p.imgmask_px, 0, c->fft.p, c->flag.p, c->stream);
                launch_real_shift(c->fft.p, nx, m, a1.p, c->stream);
            }
            launch_norm(a1.p, nx, nb, c->stream);
            launch_rot180(a1.p, a2.p, nx, m, c->stream);
        }
        // cross_correlation.f90 and the peak (calc_center.f90:71-86)
        launch_pack(a1.p, m, c->fft.p, c->stream);
        launch_pack(a2.p, m, f2.p, c->stream);
        if ((r = xform(c->fft.p, nb, true)) || (r = xform(f2.p, nb, true))) return r;
        launch_cross_power(c->fft.p, f2.p, nx, m, c->stream);
        if ((r = xform(c->fft.p, nb, false))) return r;
        launch_peak(c->fft.p, nx, nb, model ? 0 : 1, out.p, c->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(hout.data(), out.p, sizeof(float) * 3 * nb, cudaMemcpyDeviceToHost, c->stream));
        if ((r = check_flag(c))) return r;
        for (int i = 0; i < nb; ++i) {  // calc_center.f90:87-99
            cryoim_particle& q = parts[b0 + i];
            float cc = hout[3 * i + 2];
            if (cc >= 1.0f) cc = 1.0f;
            if (cc <= -1.0f) cc = -1.0f;
            q.x0 = q.x; q.y0 = q.y; q.pr0 = q.pr;
            q.x = hout[3 * i];
            q.y = hout[3 * i + 1];
            q.pr = std::acos(cc) * 45.0f / std::atan2(1.0f, 1.0f);
            q.dx = q.x - q.x0; q.dy = q.y - q.y0; q.dpr = q.pr - q.pr0;
        }
    }
    return CRYOIM_OK;
}

// local_refine/SRC/icos_equalort.f90:1-23 with icos2f_sym_matc.f90's C_N rotations: the
// nsym orientations equivalent to (theta, phi, omega), FP32 as the reference.
static void local_equalort(float th0, float ph0, float om0, const float* sym, int nsym, float d2r, float* out) {
    const float r2d = 45.0f / std::atan2(1.0f, 1.0f);
    float e[9];
    euler_mat(th0, -ph0, 180.0f - om0, d2r, e);
    for (int s = 0; s < nsym; ++s) {
        const float* S = sym + 9 * s;
        float m[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                float t = S[3 * i] * e[j];
                t = t + S[3 * i + 1] * e[3 + j];
                t = t + S[3 * i + 2] * e[6 + j];
                m[3 * i + j] = t;
            }
        out[3 * s] = std::acos(m[8]) * r2d;
        out[3 * s + 1] = -std::atan2(m[5], m[2]) * r2d;
        out[3 * s + 2] = std::atan2(m[7], m[6]) * r2d;
    }
}

// local_refine/SRC/ort_cent_11.f90: centre, -/+ x, -/+ y, then -/+ theta, phi, omega
static void local_cent11(const float* s, float dang, float dtran, float* c) {
    for (int j = 0; j < 11; ++j)
        for (int k = 0; k < 5; ++k) c[5 * j + k] = s[k];
    c[5 * 1 + 3] = s[3] - dtran; c[5 * 2 + 3] = s[3] + dtran;
    c[5 * 3 + 4] = s[4] - dtran; c[5 * 4 + 4] = s[4] + dtran;
    c[5 * 5 + 0] = s[0] - dang;  c[5 * 6 + 0] = s[0] + dang;
    c[5 * 7 + 1] = s[1] - dang;  c[5 * 8 + 1] = s[1] + dang;
    c[5 * 9 + 2] = s[2] - dang;  c[5 * 10 + 2] = s[2] + dang;
}

// loc_box.f90:34-91: whole images shifted to centre on the GPU (checkerboard, batched
// cuFFT, phase ramp, inverse), sub-images cut and normalised by k_lb_cut; the geometry
// (equivalent orientations, box corners) on the host in the reference's FP32 order.
static int local_box_extract_impl(Ctx* c, const float* imgs, bool dev_in, const cryoim_particle* parts, int P,
                                  int nx0, const float* sym, int nsym, float lx, float ly, float lz, float apix,
                                  int sub, float prt, float bx, float* sub_out, bool dev_out,
                                  cryoim_local_particle* out, int32_t* nout) {
    if (!c || !imgs || !parts || !sym || !sub_out || !out || !nout || P < 0)
        return fail(CRYOIM_ERR_ARG, "null input or negative count");
    if (nx0 < 8 || (nx0 & 1) || nx0 > 8192 || sub < 2 || sub > nx0 || nsym < 1 || nsym > 4096)
        return fail(CRYOIM_ERR_SIZE, "fftsize %d, sub_FFTsize %d, nsym %d unsupported", nx0, sub, nsym);
    *nout = 0;
    if (P == 0) return CRYOIM_OK;
    CK(cudaSetDevice(c->device));
    std::vector<cryoim_local_particle> rec((size_t)P * nsym);
    std::vector<int> src((size_t)P * nsym);
    const int K = local_box_stack_geometry(parts, P, sym, nsym, lx, ly, lz, apix, nx0, sub, prt, bx, rec.data(),
                                           src.data());
    if (K == 0) return CRYOIM_OK;
    const long nn0 = (long)nx0 * nx0, ns = (long)sub * sub;
    // chunks of B selected particles: complex work rows and (host paths) staging within
    // about 512 MB each
    const long cap = 512L << 20;
    const int B = (int)std::max(1L, std::min(64L, std::min(cap / (nn0 * 8), cap / (std::max(1L, ns * nsym) * 4))));
    DBuf<float2> work;
    DBuf<float> dimg, dsub, dxy;
    DBuf<int> dsrc, dhk;
    int r;
    if ((r = work.ensure((size_t)B * nn0)) || (r = dxy.ensure(2 * (size_t)B)) || (r = dsrc.ensure(B)) ||
        (r = dhk.ensure(3 * (size_t)B * nsym)))
        return r;
    if (!dev_in && (r = dimg.ensure((size_t)B * nn0))) return r;
    if (!dev_out && (r = dsub.ensure((size_t)B * nsym * ns))) return r;
    cufftHandle plan = 0;
    int plan_n = 0;
    std::vector<int> hsrc(B), hhk(3 * (size_t)B * nsym);
    std::vector<float> hxy(2 * (size_t)B);
    int k = 0;
    int rc = CRYOIM_OK;
    while (k < K && rc == CRYOIM_OK) {
        // the records of the next nb selected particles: k .. k1
        int nb = 0, k1 = k;
        while (k1 < K && nb < B) {
            const int i = src[k1];
            hsrc[nb] = dev_in ? i : nb;
            hxy[2 * nb] = -parts[i].x;
            hxy[2 * nb + 1] = -parts[i].y;
            for (; k1 < K && src[k1] == i; ++k1) {
                hhk[3 * (k1 - k)] = rec[k1].local_hx0;
                hhk[3 * (k1 - k) + 1] = rec[k1].local_ky0;
                hhk[3 * (k1 - k) + 2] = nb;
            }
            if (!dev_in)
                CK(cudaMemcpyAsync(dimg.p + (size_t)nb * nn0, imgs + (size_t)i * nn0, sizeof(float) * nn0,
                                   cudaMemcpyHostToDevice, c->stream));
            ++nb;
        }
        const int nk = k1 - k;
        CK(cudaMemcpyAsync(dsrc.p, hsrc.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(dxy.p, hxy.data(), sizeof(float) * 2 * nb, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(dhk.p, hhk.data(), sizeof(int) * 3 * nk, cudaMemcpyHostToDevice, c->stream));
        if (plan_n != nb) {
            if (plan) cufftDestroy(plan);
            plan = 0;
            int dims[2] = {nx0, nx0};
            cufftResult fr = cufftPlanMany(&plan, 2, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_C2C, nb);
            if (fr == CUFFT_SUCCESS) fr = cufftSetStream(plan, c->stream);
            if (fr != CUFFT_SUCCESS) { rc = fail(CRYOIM_ERR_CUDA, "2D FFT plan: cufft %d", (int)fr); break; }
            plan_n = nb;
        }
        launch_lb_checker(dev_in ? imgs : dimg.p, nx0, dsrc.p, nb, work.p, c->stream);
        cufftResult fr = cufftExecC2C(plan, (cufftComplex*)work.p, (cufftComplex*)work.p, CUFFT_FORWARD);
        if (fr == CUFFT_SUCCESS) {
            launch_lb_phase(work.p, nx0, dxy.p, nb, c->stream);
            fr = cufftExecC2C(plan, (cufftComplex*)work.p, (cufftComplex*)work.p, CUFFT_INVERSE);
        }
        if (fr != CUFFT_SUCCESS) { rc = fail(CRYOIM_ERR_CUDA, "2D FFT: cufft %d", (int)fr); break; }
        float* dst = dev_out ? sub_out + (size_t)k * ns : dsub.p;
        launch_lb_cut(work.p, nx0, dhk.p, nk, sub, dst, c->stream);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && !dev_out)
            e = cudaMemcpyAsync(sub_out + (size_t)k * ns, dsub.p, sizeof(float) * nk * ns, cudaMemcpyDeviceToHost,
                                c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { rc = fail(CRYOIM_ERR_CUDA, "local_box extraction: %s", cudaGetErrorString(e)); break; }
        k = k1;
    }
    if (plan) cufftDestroy(plan);
    if (rc != CRYOIM_OK) return rc;
    std::memcpy(out, rec.data(), sizeof(cryoim_local_particle) * K);
    *nout = K;
    return CRYOIM_OK;
}

int cryoim_local_box_extract(void* ctx, const float* imgs, const cryoim_particle* parts, int32_t P, int32_t fftsize,
                             const float* sym, int32_t nsym, float loc_x, float loc_y, float loc_z, float apix,
                             int32_t sub_fftsize, float pr_threshold, float boundx, float* sub_imgs,
                             cryoim_local_particle* out, int32_t* nout) {
    return local_box_extract_impl(as_ctx(ctx), imgs, false, parts, P, fftsize, sym, nsym, loc_x, loc_y, loc_z,
                                  apix, sub_fftsize, pr_threshold, boundx, sub_imgs, false, out, nout);
}

int cryoim_local_box_extract_device(void* ctx, const float* d_imgs, const cryoim_particle* parts, int32_t P,
                                    int32_t fftsize, const float* sym, int32_t nsym, float loc_x, float loc_y,
                                    float loc_z, float apix, int32_t sub_fftsize, float pr_threshold, float boundx,
                                    float* d_sub_imgs, cryoim_local_particle* out, int32_t* nout) {
    return local_box_extract_impl(as_ctx(ctx), d_imgs, true, parts, P, fftsize, sym, nsym, loc_x, loc_y, loc_z,
                                  apix, sub_fftsize, pr_threshold, boundx, d_sub_imgs, true, out, nout);
}

int cryoim_local_refine(void* ctx, const cryoim_local_params* lp, const float* map3d, const float* imgs,
                        cryoim_local_particle* parts, int32_t P) {
    Ctx* c = as_ctx(ctx);
    if (!c || !lp || !map3d || !imgs || !parts || P < 0) return fail(CRYOIM_ERR_ARG, "null input or negative count");
    const int nx = lp->fftsize, nx0 = lp->fftsize0, nsym = lp->nsym;
    if (nx < 8 || (nx & 1) || nx > 1024 || nx0 < nx || nx0 > 4096)
        return fail(CRYOIM_ERR_SIZE, "fftsize %d / fftsize0 %d unsupported", nx, nx0);
    if (nsym < 1 || nsym > 360 || lp->ncycle < 0 || !(lp->max_r > 0) || !(lp->imgmask_px >= 0))
        return fail(CRYOIM_ERR_ARG, "local parameters (derive them first)");
    if (P == 0) return CRYOIM_OK;
    CK(cudaSetDevice(c->device));
    const long nn = (long)nx * nx, nn0 = (long)nx0 * nx0, n3 = nn * nx;
    const int B = (int)std::max(1L, std::min(64L, (256L << 20) / (nn0 * 4)));
    const int C = std::max(nsym, 11);
    DBuf<float> dmap, fr, fi, dimg, boxed, ctf, dfs, cand, prs, oxy;
    DBuf<float2> work, spec;
    DBuf<double> acc2;
    DBuf<int> hk, flag;
    int r;
    if ((r = dmap.ensure(n3)) || (r = fr.ensure(n3)) || (r = fi.ensure(n3)) || (r = work.ensure(n3)) ||
        (r = acc2.ensure(2)) || (r = dimg.ensure((size_t)B * nn0)) || (r = boxed.ensure((size_t)B * nn)) ||
        (r = spec.ensure((size_t)B * nn)) || (r = ctf.ensure((size_t)B * nn)) || (r = dfs.ensure(3 * B)) ||
        (r = cand.ensure((size_t)B * C * 5)) || (r = prs.ensure((size_t)B * C)) || (r = oxy.ensure(2 * B)) ||
        (r = hk.ensure(2 * B)) || (r = flag.ensure(1)))
        return r;
    // refine_PR.f90:24-52: the soft-masked local map and its transform
    CK(cudaMemcpyAsync(dmap.p, map3d, sizeof(float) * n3, cudaMemcpyHostToDevice, c->stream));
    CK(launch_local_softmask(dmap.p, nx, lp->imgmask_px, acc2.p, c->stream));
    launch_map_checker(dmap.p, nx, work.p, c->stream);
    cufftHandle h3;
    CKF(cufftPlan3d(&h3, nx, nx, nx, CUFFT_C2C));
    cufftResult fr3 = cufftSetStream(h3, c->stream);
    if (fr3 == CUFFT_SUCCESS) fr3 = cufftExecC2C(h3, (cufftComplex*)work.p, (cufftComplex*)work.p, CUFFT_FORWARD);
    cudaError_t e3 = fr3 == CUFFT_SUCCESS ? launch_local_ft(work.p, nx, fr.p, fi.p, c->stream) : cudaSuccess;
    if (e3 == cudaSuccess) e3 = cudaStreamSynchronize(c->stream);
    cufftDestroy(h3);
    if (fr3 != CUFFT_SUCCESS) return fail(CRYOIM_ERR_CUDA, "3D forward FFT failed: cufft %d", (int)fr3);
    if (e3 != cudaSuccess) return fail(CRYOIM_ERR_CUDA, "local map: %s", cudaGetErrorString(e3));
    std::vector<float> sym(9 * (size_t)nsym);
    {
        const std::string name = "c" + std::to_string(nsym);
        int32_t ns = 0;
        if (nsym <= 60) {
            if (cryoim_local_sym_matrices(name.c_str(), sym.data(), &ns) != CRYOIM_OK || ns != nsym)
                return fail(CRYOIM_ERR_ARG, "symmetry c%d", nsym);
        } else {
            return fail(CRYOIM_ERR_ARG, "sym c%d: at most c60", nsym);
        }
    }
    const Angles an = host_angles();
    std::vector<float> hcand((size_t)B * C * 5), hpr((size_t)B * C), hdf(3 * B), hxy(2 * B), st(5 * (size_t)B),
        best(B);
    std::vector<int> hhk(2 * B);
    for (int b0 = 0; b0 < P; b0 += B) {
        const int nb = std::min(B, P - b0);
        const long m = (long)nb * nn;
        cufftHandle h2;
        int dims[2] = {nx, nx};
        CKF(cufftPlanMany(&h2, 2, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_C2C, nb));
        cufftResult f2 = cufftSetStream(h2, c->stream);
        for (int i = 0; i < nb; ++i) {
            const cryoim_local_particle& q = parts[b0 + i];
            hhk[2 * i] = q.local_hx0; hhk[2 * i + 1] = q.local_ky0;
            hxy[i] = q.local_x0; hxy[B + i] = q.local_y0;
            hdf[3 * i] = q.df1; hdf[3 * i + 1] = q.df2; hdf[3 * i + 2] = q.astigang;
        }
        CK(cudaMemcpyAsync(dimg.p, imgs + (size_t)b0 * nn0, sizeof(float) * nb * nn0, cudaMemcpyHostToDevice,
                           c->stream));
        CK(cudaMemcpyAsync(hk.p, hhk.data(), sizeof(int) * 2 * nb, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(oxy.p, hxy.data(), sizeof(float) * 2 * B, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(dfs.p, hdf.data(), sizeof(float) * 3 * nb, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemsetAsync(flag.p, 0, sizeof(int), c->stream));
        // refine_PR.f90:116-120: window, mask at the local origin, transform, weight
        launch_local_box(dimg.p, nx0, hk.p, nx, lp->normalize, nb, boxed.p, c->stream);
        launch_prep_images(boxed.p, nb, nx, oxy.p, oxy.p + B, 1, lp->imgmask_px, 0, spec.p, flag.p, c->stream);
        if (f2 == CUFFT_SUCCESS) f2 = cufftExecC2C(h2, (cufftComplex*)spec.p, (cufftComplex*)spec.p, CUFFT_FORWARD);
        if (f2 != CUFFT_SUCCESS) { cufftDestroy(h2); return fail(CRYOIM_ERR_CUDA, "2D FFT failed: cufft %d", (int)f2); }
        cufftDestroy(h2);
        launch_ref_post(spec.p, m, (float)nn, c->stream);
        launch_wlp(spec.p, nx, m, lp->max_r, c->stream);
        const float* ctfp = nullptr;
        if (lp->apply_ctf) {
            launch_local_ctf(dfs.p, nx, lp->apix, lp->vol, lp->cs, lp->ampwg, nb, ctf.p, c->stream);
            ctfp = ctf.p;
        }
        CK(cudaGetLastError());
        for (int i = 0; i < nb; ++i) {
            const cryoim_local_particle& q = parts[b0 + i];
            float* s = &st[5 * i];
            s[0] = q.local_theta0; s[1] = q.local_phi0; s[2] = q.local_omega0; s[3] = q.local_x0; s[4] = q.local_y0;
            best[i] = 0.0f;  // refine_PR.f90 leaves maxCC unset when there is nothing to score
        }
        // score nc candidates per particle (already in hcand) and move to the first minimum
        auto score_round = [&](int nc) -> int {
            CK(cudaMemcpyAsync(cand.p, hcand.data(), sizeof(float) * nb * nc * 5, cudaMemcpyHostToDevice, c->stream));
            launch_local_pr(cand.p, nc, fr.p, fi.p, nx, spec.p, ctfp, lp->max_r, nb, prs.p, c->stream);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(hpr.data(), prs.p, sizeof(float) * nb * nc, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            for (int i = 0; i < nb; ++i) {
                int k = 0;
                for (int j = 1; j < nc; ++j)
                    if (hpr[(size_t)i * nc + j] < hpr[(size_t)i * nc + k]) k = j;
                for (int v = 0; v < 5; ++v) st[5 * i + v] = hcand[((size_t)i * nc + k) * 5 + v];
                best[i] = hpr[(size_t)i * nc + k];
            }
            return CRYOIM_OK;
        };
        if (nsym > 1) {  // refine_PR.f90:122-145: the equivalent orientations at the local origin
            std::vector<float> eq(3 * (size_t)nsym);
            for (int i = 0; i < nb; ++i) {
                local_equalort(st[5 * i], st[5 * i + 1], st[5 * i + 2], sym.data(), nsym, an.deg2rad, eq.data());
                for (int s = 0; s < nsym; ++s) {
                    float* o = &hcand[((size_t)i * nsym + s) * 5];
                    o[0] = eq[3 * s]; o[1] = eq[3 * s + 1]; o[2] = eq[3 * s + 2];
                    o[3] = st[5 * i + 3]; o[4] = st[5 * i + 4];
                }
            }
            if ((r = score_round(nsym))) return r;
        }
        // refine_PR.f90:146-168 / 180-202: Ncycle rounds of the 11-candidate descent
        float fac = 1.0f;
        for (int cyc = 1; cyc <= lp->ncycle; ++cyc) {
            const float dang = lp->refine_angle * fac, dtran = lp->refine_shift * fac;
            fac = fac * lp->convf;
            for (int i = 0; i < nb; ++i) local_cent11(&st[5 * i], dang, dtran, &hcand[(size_t)i * 11 * 5]);
            if ((r = score_round(11))) return r;
        }
        int bad = 0;
        CK(cudaMemcpyAsync(&bad, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (bad) return fail(CRYOIM_ERR_INPUT, "non-finite pixel (NaN/Inf) in a sub-particle window");
        for (int i = 0; i < nb; ++i) {  // refine_PR.f90:220-231
            cryoim_local_particle& q = parts[b0 + i];
            const float* s = &st[5 * i];
            q.local_dtheta = s[0] - q.local_theta0;
            q.local_dphi = s[1] - q.local_phi0;
            q.local_domega = s[2] - q.local_omega0;
            q.local_dx = s[3] - q.local_x0;
            q.local_dy = s[4] - q.local_y0;
            q.local_theta = s[0]; q.local_phi = s[1]; q.local_omega = s[2];
            q.local_x = s[3]; q.local_y = s[4];
            q.local_z = q.local_z0;
            q.local_pr = best[i];
        }
    }
    return CRYOIM_OK;
}

int cryoim_central_sections(void* ctx, const float* ft_re, const float* ft_im, const float* eulers,
                            int32_t n, float* out_re, float* out_im) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!ft_re || !ft_im || !eulers || !out_re || !out_im || n < 1)
        return fail(CRYOIM_ERR_ARG, "null input or n < 1");
    const int nx = c->p.fftsize;
    const long nn = (long)nx * nx, n3 = nn * nx;
    DBuf<float> dre, dim, deul, ore, oim;
    if ((r = dre.ensure(n3)) || (r = dim.ensure(n3)) || (r = deul.ensure(3 * n)) ||
        (r = ore.ensure((size_t)n * nn)) || (r = oim.ensure((size_t)n * nn)))
        return r;
    CK(cudaMemcpyAsync(dre.p, ft_re, sizeof(float) * n3, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dim.p, ft_im, sizeof(float) * n3, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(deul.p, eulers, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    launch_sections(dre.p, dim.p, nx, deul.p, n, ore.p, oim.p, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out_re, ore.p, sizeof(float) * n * nn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(out_im, oim.p, sizeof(float) * n * nn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

// The band cube of c->mapreal: frequencies -(cube_r + 1) .. cube_r + 1 of the map's
// centred transform (ovs 1), or of the map zero-padded to (2 n)^3 (ovs 2: the samples of
// a section at frequency h sit at 2 h, cube_r = 2 maxR + 1).  Trilinear interpolation of
// the twice-oversampled transform matches the map's projections far better (noise-free
// correlation 0.998 against 0.96 at box 128); it removes the bias the interpolation error
// puts on the local searches' maxima.
int build_map_cube(Ctx* c) {
    const int nx = c->p.fftsize, R = c->p.max_r, ovs = c->ovs, m = ovs * nx;
    const int Rq = ovs == 1 ? R : 2 * R + 1;
    const long m3 = (long)m * m * m, c3 = (long)(2 * Rq + 3) * (2 * Rq + 3) * (2 * Rq + 3);
    DBuf<float2> work;
    int r;
    if ((r = work.ensure(m3)) || (r = c->mapcube.ensure(c3))) return r;
    if (ovs == 1)
        launch_map_checker(c->mapreal.p, nx, work.p, c->stream);
    else
        launch_lp_pad_checker(c->mapreal.p, nx, work.p, c->stream);
    CK(cudaGetLastError());
    cufftHandle h;
    CKF(cufftPlan3d(&h, m, m, m, CUFFT_C2C));
    cufftResult fr = cufftSetStream(h, c->stream);
    if (fr == CUFFT_SUCCESS) fr = cufftExecC2C(h, (cufftComplex*)work.p, (cufftComplex*)work.p, CUFFT_FORWARD);
    if (fr != CUFFT_SUCCESS) {
        cufftDestroy(h);
        return fail(CRYOIM_ERR_CUDA, "3D forward FFT failed: cufft %d", (int)fr);
    }
    launch_map_band(work.p, m, Rq, c->mapcube.p, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cufftDestroy(h);
    if (e != cudaSuccess) return fail(CRYOIM_ERR_CUDA, "reference map: %s", cudaGetErrorString(e));
    c->cube_r = Rq;
    c->map_ready = true;
    c->bmat_ready = false;
    c->bmat8_ready = false;
    c->bmat_c_ready = false;
    return CRYOIM_OK;
}

int cryoim_set_reference_map(void* ctx, const float* map3d) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!map3d) return fail(CRYOIM_ERR_ARG, "null map");
    const int nx = c->p.fftsize;
    const long n3 = (long)nx * nx * nx;
    if ((r = c->mapreal.ensure(n3))) return r;
    CK(cudaMemcpyAsync(c->mapreal.p, map3d, sizeof(float) * n3, cudaMemcpyHostToDevice, c->stream));
    return build_map_cube(c);
}

int cryoim_contract_search(void* ctx, const float* imgs, cryoim_particle* parts, int32_t P,
                           const cryoim_contract_opts* opts, float* cands) {
    return contract_search_impl(as_ctx(ctx), imgs, false, parts, P, opts, cands);
}

int cryoim_contract_search_device(void* ctx, const float* d_imgs, cryoim_particle* parts, int32_t P,
                                  const cryoim_contract_opts* opts, float* cands) {
    return contract_search_impl(as_ctx(ctx), d_imgs, true, parts, P, opts, cands);
}

int cryoim_set_interpolation(void* ctx, int32_t kind, float sigma) {
    Ctx* c = as_ctx(ctx);
    if (!c) return fail(CRYOIM_ERR_ARG, "null context");
    if (kind == 0 || kind == 2) {
        sigma = 0.0f;
    } else if (kind != 1 || !(sigma >= 0.25f && sigma <= 2.0f)) {
        return fail(CRYOIM_ERR_ARG,
                    "interpolation: kind 0 (trilinear), 1 (Gaussian, sigma 0.25..2 voxels) or 2 (trilinear, "
                    "twice-oversampled transform)");
    }
    const int ovs = kind == 2 ? 2 : 1;
    if (sigma != c->interp_sigma || ovs != c->ovs) {
        c->interp_sigma = sigma;
        c->bmat_ready = false;
        c->bmat8_ready = false;
        c->bmat_c_ready = false;
        if (ovs != c->ovs) {
            c->ovs = ovs;
            int r;
            if (c->map_ready && (r = build_map_cube(c))) return r;
        }
    }
    return CRYOIM_OK;
}

int cryoim_contract_fallbacks(void* ctx, int32_t* n) {
    Ctx* c = as_ctx(ctx);
    if (!c || !n) return fail(CRYOIM_ERR_ARG, "null argument");
    *n = c->last_fallbacks;
    return CRYOIM_OK;
}

int cryoim_learn_opts_default(cryoim_learn_opts* o) {
    if (!o) return fail(CRYOIM_ERR_ARG, "null options");
    o->samples = 200000;
    o->batch = 256;
    o->seed = 1;
    o->lr = 2.0e-3f;
    o->snr = 0.1f;
    o->df_min = 1.0f;
    o->df_max = 3.0f;
    o->astig_max = 0.0f;
    o->origin_max = 3.0f;
    return CRYOIM_OK;
}

int cryoim_learn_train(void* ctx, const float* map3d, const cryoim_learn_opts* o, float* stats) {
    return learn_train_impl(as_ctx(ctx), map3d, o, stats);
}

int cryoim_learn_save(void* ctx, const char* path) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!path) return fail(CRYOIM_ERR_ARG, "null path");
    const LearnModel& L = c->lm;
    if (!L.ready) return fail(CRYOIM_ERR_STATE, "no trained proposer");
    std::vector<float> w(L.nparam);
    CK(cudaMemcpyAsync(w.data(), L.w.p, sizeof(float) * L.nparam, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(CRYOIM_ERR_IO, "cannot write %s", path);
    const int32_t hdr[3] = {1, L.V, L.sign};
    const int64_t np = L.nparam;
    bool ok = std::fwrite("CRYOIMLP", 1, 8, f) == 8 && std::fwrite(hdr, 4, 3, f) == 3 &&
              std::fwrite(&L.step, 4, 1, f) == 1 && std::fwrite(&np, 8, 1, f) == 1 &&
              std::fwrite(w.data(), 4, w.size(), f) == w.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? CRYOIM_OK : fail(CRYOIM_ERR_IO, "short write to %s", path);
}

int cryoim_learn_load(void* ctx, const char* path) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!path) return fail(CRYOIM_ERR_ARG, "null path");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(CRYOIM_ERR_IO, "cannot read %s", path);
    char magic[8];
    int32_t hdr[3];
    float step = 0.0f;
    int64_t np = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "CRYOIMLP", 8) == 0 &&
              std::fread(hdr, 4, 3, f) == 3 && std::fread(&step, 4, 1, f) == 1 && std::fread(&np, 8, 1, f) == 1;
    if (!ok || hdr[0] != 1) {
        std::fclose(f);
        return fail(CRYOIM_ERR_INPUT, "%s is not a proposer file", path);
    }
    if ((r = ensure_cgrid(c))) { std::fclose(f); return r; }
    if (step != c->p.searchstep || hdr[1] != c->cgrid.V) {
        std::fclose(f);
        return fail(CRYOIM_ERR_MISMATCH, "%s was trained for step %g (%d views), not %g (%d views)", path,
                    (double)step, hdr[1], (double)c->p.searchstep, c->cgrid.V);
    }
    LearnModel& L = c->lm;
    if ((r = learn_layout(c, hdr[1]))) { std::fclose(f); return r; }
    if (np != L.nparam) {
        std::fclose(f);
        return fail(CRYOIM_ERR_MISMATCH, "%s holds %lld parameters, expected %ld", path, (long long)np, L.nparam);
    }
    std::vector<float> w(np);
    ok = std::fread(w.data(), 4, w.size(), f) == w.size();
    std::fclose(f);
    if (!ok) return fail(CRYOIM_ERR_IO, "short read from %s", path);
    CK(cudaMemcpyAsync(L.w.p, w.data(), sizeof(float) * np, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    L.sign = hdr[2];
    L.step = step;
    L.steps = 0;
    L.ready = true;
    return CRYOIM_OK;
}

int cryoim_learn_params(void* ctx, float* get, const float* set, int64_t* n) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if ((r = ensure_cgrid(c))) return r;
    LearnModel& L = c->lm;
    if (L.nparam == 0 || L.V != c->cgrid.V) {
        if ((r = learn_layout(c, c->cgrid.V))) return r;
        CK(cudaMemsetAsync(L.w.p, 0, sizeof(float) * L.nparam, c->stream));
        L.step = c->p.searchstep;
    }
    if (n) *n = L.nparam;
    if (set) CK(cudaMemcpyAsync(L.w.p, set, sizeof(float) * L.nparam, cudaMemcpyHostToDevice, c->stream));
    if (get) CK(cudaMemcpyAsync(get, L.w.p, sizeof(float) * L.nparam, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

int cryoim_learn_forward(void* ctx, const float* feat, const float* truth, int32_t B, float* scores, float* loss,
                         float* grads) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    LearnModel& L = c->lm;
    if (L.nparam == 0) return fail(CRYOIM_ERR_STATE, "no proposer parameters (cryoim_learn_params)");
    if (!feat || B < 1 || ((loss || grads) && !truth)) return fail(CRYOIM_ERR_ARG, "bad arguments");
    if ((r = learn_activations(c, B))) return r;
    CK(cudaMemcpyAsync(L.feat.p, feat, sizeof(float) * B * LP_NR * LP_NT, cudaMemcpyHostToDevice, c->stream));
    if ((r = learn_forward(c, B))) return r;
    if (scores)
        CK(cudaMemcpyAsync(scores, L.sc.p, sizeof(float) * B * L.V * LP_NT, cudaMemcpyDeviceToHost, c->stream));
    if (truth) {
        CK(cudaMemcpyAsync(L.truth.p, truth, sizeof(float) * 4 * B, cudaMemcpyHostToDevice, c->stream));
        if ((r = learn_backward(c, B))) return r;
        if (loss) CK(cudaMemcpyAsync(loss, L.loss.p, sizeof(float) * B, cudaMemcpyDeviceToHost, c->stream));
        if (grads) CK(cudaMemcpyAsync(grads, L.gr.p, sizeof(float) * L.nparam, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return learn_conv_status(c);
}

// Test hook of the proposer's convolution kernels on host arrays (current device, its
// default stream): out = conv(x) (+ bias, ReLU) and, when dpre is given, the weight and
// bias gradients dW, db of dpre.  tensor_cores: 1 = conv_tc.cu (TF32), 0 = learn.cu (FP32).
int cryoim_conv3_check(int32_t tensor_cores, const float* x, int32_t B, int32_t Cin, int32_t H, const float* W,
                       const float* bias, int32_t Cout, int32_t relu, float* out, const float* dpre, float* dW,
                       float* db) {
    if (!x || !W || !out || B < 1 || H < 1 || Cin < 1 || Cin > 32 || (Cout != 16 && Cout != 32) ||
        (dpre && (!dW || !db)))
        return fail(CRYOIM_ERR_ARG, "bad arguments");
    const size_t nx = (size_t)B * Cin * H * LP_NT, ny = (size_t)B * Cout * H * LP_NT, nw = (size_t)Cout * Cin * 9;
    DBuf<float> dx, dy, dwt, dbias, dg, dgw, dgb;
    DBuf<int> derr;
    int r;
    if ((r = dx.ensure(nx)) || (r = dy.ensure(ny)) || (r = dwt.ensure(nw)) || (r = dbias.ensure(Cout)) ||
        (r = derr.ensure(1)) || (dpre && ((r = dg.ensure(ny)) || (r = dgw.ensure(nw)) || (r = dgb.ensure(Cout)))))
        return r;
    auto done = [&](int code) {
        for (DBuf<float>* b : {&dx, &dy, &dwt, &dbias, &dg, &dgw, &dgb}) b->release();
        derr.release();
        return code;
    };
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    ok(cudaMemcpy(dx.p, x, nx * 4, cudaMemcpyHostToDevice));
    ok(cudaMemcpy(dwt.p, W, nw * 4, cudaMemcpyHostToDevice));
    ok(cudaMemset(dbias.p, 0, Cout * 4));
    if (bias) ok(cudaMemcpy(dbias.p, bias, Cout * 4, cudaMemcpyHostToDevice));
    ok(cudaMemset(derr.p, 0, sizeof(int)));
    if (e == cudaSuccess)
        ok(tensor_cores ? launch_lp_conv3_tc(dx.p, B, Cin, H, dwt.p, bias ? dbias.p : nullptr, Cout, relu != 0, dy.p,
                                             derr.p, 0)
                        : launch_lp_conv3(dx.p, B, Cin, H, dwt.p, bias ? dbias.p : nullptr, Cout, relu != 0, dy.p, 0));
    if (dpre && e == cudaSuccess) {
        ok(cudaMemcpy(dg.p, dpre, ny * 4, cudaMemcpyHostToDevice));
        ok(cudaMemset(dgw.p, 0, nw * 4));
        ok(cudaMemset(dgb.p, 0, Cout * 4));
        if (e == cudaSuccess)
            ok(tensor_cores ? launch_lp_conv3_wgrad_tc(dx.p, dg.p, B, Cin, H, Cout, dgw.p, dgb.p, derr.p, 0)
                            : launch_lp_conv3_wgrad(dx.p, dg.p, B, Cin, H, Cout, dgw.p, dgb.p, 0));
    }
    ok(cudaDeviceSynchronize());
    int flag = 0;
    ok(cudaMemcpy(&flag, derr.p, sizeof(int), cudaMemcpyDeviceToHost));
    ok(cudaMemcpy(out, dy.p, ny * 4, cudaMemcpyDeviceToHost));
    if (dpre) {
        ok(cudaMemcpy(dW, dgw.p, nw * 4, cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(db, dgb.p, Cout * 4, cudaMemcpyDeviceToHost));
    }
    if (e != cudaSuccess) return done(fail(CRYOIM_ERR_CUDA, "%s", cudaGetErrorString(e)));
    if (flag) return done(fail(CRYOIM_ERR_CUDA, "tensor-core convolution wait timed out"));
    return done(CRYOIM_OK);
}

int cryoim_learn_set_conv(void* ctx, int32_t tensor_cores) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (tensor_cores != 0 && tensor_cores != 1) return fail(CRYOIM_ERR_ARG, "tensor_cores must be 0 or 1");
    c->lm.conv_tc = tensor_cores != 0;
    return CRYOIM_OK;
}

int cryoim_learn_render(void* ctx, const float* map3d, const float* eul, const float* par, int32_t B, float snr,
                        int32_t seed, float* imgs) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!map3d || !eul || !par || !imgs || B < 1 || snr < 0) return fail(CRYOIM_ERR_ARG, "bad arguments");
    const long nn = (long)c->p.fftsize * c->p.fftsize;
    CubeTexture ct;
    if ((r = render_cube(c, map3d, &ct))) return r;
    DBuf<float> img, deul, dpar, var;
    DBuf<float2> ft;
    if ((r = img.ensure((size_t)B * nn)) || (r = ft.ensure((size_t)B * nn)) || (r = deul.ensure(3 * (size_t)B)) ||
        (r = dpar.ensure(5 * (size_t)B)) || (r = var.ensure(B)))
        return r;
    CK(cudaMemcpyAsync(deul.p, eul, sizeof(float) * 3 * B, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dpar.p, par, sizeof(float) * 5 * B, cudaMemcpyHostToDevice, c->stream));
    if ((r = learn_render(c, ct.tex, deul.p, dpar.p, B, snr, (unsigned long long)seed, c->p.apply_ctf != 0, img.p,
                          ft.p, var.p)))
        return r;
    CK(cudaMemcpyAsync(imgs, img.p, sizeof(float) * B * nn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CRYOIM_OK;
}

int cryoim_learn_views(void* ctx, float* out, int32_t* V) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!V) return fail(CRYOIM_ERR_ARG, "null count");
    if ((r = ensure_cgrid(c))) return r;
    *V = c->cgrid.V;
    if (out)
        for (int i = 0; i < c->cgrid.V; ++i) {
            out[2 * i] = c->cgrid.views[4 * i];
            out[2 * i + 1] = c->cgrid.views[4 * i + 1];
        }
    return CRYOIM_OK;
}

int cryoim_learn_features(void* ctx, const float* imgs, const cryoim_particle* parts, int32_t P, float* feat) {
    Ctx* c = as_ctx(ctx);
    int r = check_ready(c, false);
    if (r) return r;
    if (!imgs || !parts || !feat || P < 1) return fail(CRYOIM_ERR_ARG, "bad arguments");
    const long nn = (long)c->p.fftsize * c->p.fftsize;
    const int B = std::min(P, 64);
    if ((r = ensure_cgrid(c))) return r;
    if (c->lm.V == 0) c->lm.V = c->cgrid.V;
    if ((r = learn_activations(c, B)) || (r = ensure_batch(c, B))) return r;
    DBuf<float> d;
    if ((r = d.ensure((size_t)B * nn))) return r;
    std::vector<float> ox(B), oy(B);
    for (int b0 = 0; b0 < P; b0 += B) {
        const int nb = std::min(B, P - b0);
        for (int i = 0; i < nb; ++i) { ox[i] = parts[b0 + i].x; oy[i] = parts[b0 + i].y; }
        CK(cudaMemcpyAsync(d.p, imgs + b0 * nn, sizeof(float) * nb * nn, cudaMemcpyHostToDevice, c->stream));
        if ((r = learn_features_dev(c, d.p, nb, ox.data(), oy.data()))) return r;
        CK(cudaMemcpyAsync(feat + (long)b0 * LP_NR * LP_NT, c->lm.feat.p, sizeof(float) * nb * LP_NR * LP_NT,
                           cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    if ((r = check_flag(c))) return r;
    return CRYOIM_OK;
}

int cryoim_contract_stats(void* ctx, double* out /* 6 */) {
    Ctx* c = as_ctx(ctx);
    if (!c || !out) return fail(CRYOIM_ERR_ARG, "null argument");
    int r;
    if (c->map_ready && c->have_params && c->T >= 0) {
        if ((r = ensure_grid(c)) || (r = ensure_samples(c))) return r;
    }
    out[0] = c->last_slice_ms > 0.0 ? c->last_slice_ms : c->bmat_ms;
    out[1] = c->prof_gemm_ms;
    out[2] = (double)c->prof_gemm_launches;
    out[3] = c->prof_gemm_flops;
    out[4] = (double)((long)c->V * c->nom);
    out[5] = (double)(c->last_kpad > 0 ? c->last_kpad : c->cKpad);
    c->prof_gemm_ms = 0.0;
    c->prof_gemm_launches = 0;
    c->prof_gemm_flops = 0.0;
    return CRYOIM_OK;
}

int cryoim_rescore_stats(void* ctx, double* out /* 3 */) {
    Ctx* c = as_ctx(ctx);
    if (!c || !out) return fail(CRYOIM_ERR_ARG, "null argument");
    out[0] = c->prof_pr_ms;
    out[1] = (double)c->prof_pr_launches;
    out[2] = c->prof_pr_cands;
    c->prof_pr_ms = 0.0;
    c->prof_pr_launches = 0;
    c->prof_pr_cands = 0.0;
    return CRYOIM_OK;
}

int cryoim_icos_ops(float* rot) {
    if (!rot) return fail(CRYOIM_ERR_ARG, "null output");
    std::memcpy(rot, table_ops(), sizeof(float) * 540);
    return CRYOIM_OK;
}

int cryoim_asu_fold(float* theta, float* phi, float* omega) {
    if (!theta || !phi || !omega) return fail(CRYOIM_ERR_ARG, "null argument");
    asu_fold(theta, phi, omega, table_ops(), host_angles().deg2rad);
    return CRYOIM_OK;
}

int cryoim_equalort(float theta, float phi, float omega, float* out) {
    if (!out) return fail(CRYOIM_ERR_ARG, "null output");
    float e[9], g[540];
    eular_matrix(theta, phi, omega, e);
    gen_ops<float>(g);
    for (int i = 0; i < 60; ++i) {
        float r[9];
        mm3(g + i * 9, e, r);
        euler_from(r, out + 3 * i, out + 3 * i + 1, out + 3 * i + 2);
    }
    return CRYOIM_OK;
}

int cryoim_transform_ort(int32_t to, float* theta, float* phi, float* omega, int32_t n) {
    if (!theta || !phi || !omega || n < 0) return fail(CRYOIM_ERR_ARG, "null argument");
    if (to != 5 && to != 3) return fail(CRYOIM_ERR_ARG, "to must be 5 or 3");
    const float d2r = 4.0f * std::atan2(1.0f, 1.0f) / 180.0f;
    float rot0[9];
    if (to == 5) {
        float v = acosf(cosf(60.0f * d2r) / sinf(36.0f * d2r));
        float t[9] = {cosf(v), 0, sinf(v), 0, 1, 0, -sinf(v), 0, cosf(v)};
        std::memcpy(rot0, t, sizeof(t));
    } else {
        float w = acosf(cosf(36.0f * d2r) / sinf(60.0f * d2r));
        float t[9] = {1, 0, 0, 0, cosf(-w), sinf(-w), 0, -sinf(-w), cosf(-w)};
        std::memcpy(rot0, t, sizeof(t));
    }
    for (int i = 0; i < n; ++i) {
        float e[9], r[9];
        eular_matrix(theta[i], phi[i], omega[i], e);
        mm3(rot0, e, r);
        euler_from(r, theta + i, phi + i, omega + i);
    }
    return CRYOIM_OK;
}

}  // extern "C"
