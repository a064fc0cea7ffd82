// kernels.h — launchers shared by the translation units of libcryoim_gb300.so.
//
// Device data layout (all buffers live in HBM, owned by the context):
//   * particle / template Fourier "band": the (W x W) window of the centred nx*nx
//     transform that the common-line sampler can touch, W = 2*maxR + 2, window
//     origin at pixel (off, off), off = nx/2 - maxR.  float2 = (a, b) with b = -Im.
//   * amplitude cuts (Fcut): nr = maxR - minR + 1 floats per image.
//   * reconstruction accumulator: float4 (fa, fb, wg, 0) over a half box of
//     AW x AW x (maxR + 2) voxels, AW = 2*maxR + 3, covering frequencies
//     -maxR-1 .. maxR+1 in x and y and 0 .. maxR+1 in z (z >= 0 after the Friedel
//     fold).  The extra low cell absorbs FP32 rotations that put a radius-maxR
//     sample a hair beyond -maxR (the reference writes that cell in its full grid).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/cryoim.h"

namespace cryoim {

struct Band {
    int nx, min_r, max_r, nr, W, off, AW;
};
inline Band make_band(int nx, int min_r, int max_r) {
    Band b;
    b.nx = nx; b.min_r = min_r; b.max_r = max_r; b.nr = max_r - min_r + 1;
    b.W = 2 * max_r + 2; b.off = nx / 2 - max_r;
    b.AW = 2 * max_r + 3;
    return b;
}
// accumulator index of frequency (hx, ky, lz)
__host__ __device__ inline long acc_cell(const Band& b, int hx, int ky, int lz) {
    return ((long)lz * b.AW + (ky + b.max_r + 1)) * b.AW + (hx + b.max_r + 1);
}

// ---- prep.cu (FP32 in the reference's operation order, -fmad=false) -------
// mask (+ optional img2d_norm), checkerboard, real -> complex; nonfinite -> *flag |= 1
void launch_prep_images(const float* imgs, int B, int nx, const float* ox, const float* oy,
                        int use_mask, float mask_px, int normalize, float2* fft, int* flag,
                        cudaStream_t st);
// scale 1/nx^2, b = -Im, Fcut fit, optional origin shift (sx/sy per image, may be null),
// band extraction.
void launch_post_fft(const float2* fft, int B, Band bd, const float* sx, const float* sy,
                     float2* band, float* fcut, cudaStream_t st);
// getCTF2d over the band for B images (per-image defocus triples in dfs: df1, df2, astig)
void launch_ctf_band(int B, Band bd, const float* dfs, float apix, float vol, float cs,
                     float ampwg, float* ctf, cudaStream_t st);
// Fcut of template x CTF for every (image, template)
void launch_tmpl_fcut(const float2* tband, int T, const float* ctf, int B, Band bd, float* tfcut,
                      cudaStream_t st);
// common-line angle pairs for every (view, template, operator); views: V x 2 (theta, phi)
void launch_alpha_table(const float* views, int V, const float* tort, int T, const float* ops,
                        float2* alpha, cudaStream_t st);
// refinement: the 11 candidates of every image (ort_cent_11) and their angle pairs
void launch_refine_candidates(float* state, int B, float dang, float dtran, const float* ops,
                              float* cand, cudaStream_t st);
void launch_refine_alpha(const float* cand, int B, const float* tort, int T, const float* ops,
                         float2* alpha, cudaStream_t st, int ncand = 11);
void launch_refine_select(const float* cand, const float* pr, int B, float* state,
                          cudaStream_t st);
// reconstruction finish: fold / divide / sign into the full complex grid
// int_shell: 0 keeps |h| <= maxR (reconstruct.f90), 1 keeps int(|h|) <= maxR
// (merge_reconstruct.f90)
void launch_rec_fold(const float4* acc, Band bd, int int_shell, float2* vol, cudaStream_t st);
void launch_rec_real(const float2* vol, int nx, float* map, cudaStream_t st);
// real-space template projection and central sections
void launch_project(const float* map, int nx, const float* eul, int n, float* out,
                    cudaStream_t st);
void launch_sections(const float* fre, const float* fim, int nx, const float* eul, int n,
                     float* ore, float* oim, cudaStream_t st);

// ---- score.cu (phase-residual scoring and insertion) ------------------------
struct PrOmegaArgs {
    const float2* band;      // [B][W*W]
    const float* fcut0;      // [B][nr]
    const float2* tband;     // [T][W*W]
    const float* tfcut;      // [B][T][nr] (CTF) or [T][nr] (no CTF, tfcut_pstride = 0)
    long tfcut_pstride;
    const float* ctf;        // [B][W*W] or nullptr
    const float2* alpha;     // [V][T][60]
    const float* views;      // [V][4]: theta, phi, slot base (int bits), pad
    int V, T, nomega;
    float step;
    Band bd;
    unsigned long long* best;  // [B]
    float* pr_array;           // [B][per] or nullptr
    long per;
};
int pr_omega_smem_bytes(const Band& bd, int nomega, int* threads);
cudaError_t launch_pr_omega(const PrOmegaArgs& a, int B, cudaStream_t st);

struct PrSingleArgs {
    const float2* band;      // [B][W*W] unshifted particle FT
    const float* fcut0;      // [B][nr]
    const float2* tband;     // [T][W*W]
    const float* tfcut;
    long tfcut_pstride;
    const float* ctf;        // [B][W*W] or nullptr
    const float* cand;       // [B][ncand][5]
    const float2* alpha;     // [B][ncand][T][60]
    int T;
    Band bd;
    float* pr;               // [B][ncand]
    int ncand = 11;          // 11 for the refinement step (ort_cent_11.f90)
    // rescoring by groups (launch_pr_rescore_groups) only:
    const float4* sband = nullptr;  // [B][W*W] band shifted to the candidates' common origin, in
                                    // (pixel, right neighbour) pairs (launch_shift_band)
    const int* ncount = nullptr;    // [B] candidates in use (later slots are skipped), or nullptr
    const float4* tbandc = nullptr; // [B][T][W*W] templates x CTF as (pixel, right neighbour) pairs
                                    // (launch_tband_ctf), or nullptr
    // the view table of the search grid ([V][T][60], launch_alpha_table) and each candidate's
    // grid orientation (view * nom + omega index, [B][ncand]): the shared-band rescoring then
    // takes its line angles from the table and subtracts omega as k_pr_omega does, so that
    // its terms are the exhaustive search's (alpha is not read)
    const float2* valpha = nullptr;
    const int* corient = nullptr;
    int nom = 0;
    float step = 0.0f;
};
// cal_crosslin_PR for each candidate, its origin shift applied to every tap (k_pr_single)
cudaError_t launch_pr_single(const PrSingleArgs& a, int B, cudaStream_t st);
// rescoring by groups of candidates sharing a view: groups[g] = (particle, first
// candidate slot, count <= pr_rescore_group_size(), 0); requires sband
cudaError_t launch_pr_rescore_groups(const PrSingleArgs& a, const int4* groups, int ngroups, cudaStream_t st);
int pr_rescore_group_size();
// whether launch_pr_rescore_groups runs the shared-band kernel (which reads valpha and
// corient) for this band and template count, rather than the one that reads alpha
bool pr_rescore_shared_band(const Band& bd, int T);
// the templates x each particle's CTF, each pixel stored with its right neighbour (zero
// past the row's end), so a bilinear sample reads two 16-byte pairs
cudaError_t launch_tband_ctf(const float2* tband, int T, const float* ctf, const Band& bd, int B, float4* out,
                             cudaStream_t st);
// sband for PrSingleArgs: the band of each particle shifted to cand[p][0]'s origin, each
// pixel stored with its right neighbour
cudaError_t launch_shift_band(const float2* band, const float* cand, int ncand, const Band& bd, int B,
                              float4* out, cudaStream_t st);

struct InsertArgs {
    const float2* band;      // [B][W*W] shifted particle FT
    const float* ctf;        // [B][W*W] or nullptr (CTF = 1)
    const float* rot;        // [B][9] particle rotation matrices
    const float* ops;        // [60][9]
    const int2* samples;     // (hx, ky) insertion samples
    int nsamples, nsym;
    const int* sel;          // [B] 1 = insert
    float off_xy, off_z;     // coordinate offsets added before int()
    int base_xy, base_z;     // accumulator index origin
    Band bd;
    float4* acc;             // half box
};
cudaError_t launch_insert(const InsertArgs& a, int B, cudaStream_t st);

// ---- gemm_tc.cu (tcgen05 BF16 contraction with fused per-tile argmax) --------
// One independent product of a grouped launch: rows [a_row0, a_row0 + m_valid) of A
// against rows [b_row0, b_row0 + n_valid) of B; its (row, tile) maxima go to
// topv/topi + topv_off as [m_valid][n_tiles], columns counted from b_row0.
struct GemmGroup {
    int tile_start, m_tiles, a_row0, m_valid, b_row0, n_valid, n_tiles, topv_off;
};
struct GemmArgmaxArgs {
    int m_tiles, n_tiles, kblocks, m_valid, n_valid;  // set by the launcher
    float* topv;   // [M][n_tiles] max of each row over each 256-column tile
    int* topi;     // [M][n_tiles] its column
    float* cfull;  // optional full C [M][ldc] (tests; not with groups)
    long ldc;
    int* err;      // set to 1 when a wait times out (zero it before the launch)
    const GemmGroup* groups = nullptr;  // device array, or nullptr for one product
    int ngroups = 0, total_tiles = 0;   // set by the grouped launcher
    // tests of the failure path: a wait limit other than the default 2 s, and (withhold
    // = s + 1) CTA 0's producer leaving k-stage s of its first tile unloaded, so that the
    // issuer's wait for it runs out
    unsigned long long wait_ns = 0;
    int withhold = 0;
    // operand B: 0 plain rows (the TMA load applies the 128-byte swizzle); 1 pre-swizzled
    // rows (contract.cu's section rows) loaded by TMA tiles without swizzle, every tile
    // starting at a multiple of 8 rows (so a row's residue mod 8 is its slot's); 2 (grouped
    // launches only) pre-swizzled rows by index: row j of a group's B is row
    // b_index[b_row0 + j] of b_rows (b_row_bytes apart), copied into the tile by the
    // producer warp's 16-byte cp.async with the chunks re-swizzled for the tile row
    int b_mode = 0;
    const int* b_index = nullptr;
    const unsigned char* b_rows = nullptr;
    long b_row_bytes = 0;
};
int gemm_tile_n();
int gemm_tile_m();
// A: M x K, B: N x K, BF16 row-major (K contiguous, K % 64 == 0, 16-byte aligned)
cudaError_t launch_gemm_bf16_argmax(const void* a, const void* b, int M, int N, int K,
                                    const GemmArgmaxArgs& g, int num_sms, cudaStream_t st);
// f8: both operands FP8-e4m3 bytes (K % 128 == 0), else BF16
cudaError_t launch_gemm_argmax(const void* a, const void* b, int M, int N, int K, bool f8,
                               const GemmArgmaxArgs& g, int num_sms, cudaStream_t st);
// Several products in one persistent launch (A: Mtot x K, B: Ntot x K).  hgroups
// (host, a_row0/m_valid/b_row0/n_valid/topv_off filled) is completed and copied to
// dgroups (device, ngroups entries) on st; the host array must stay alive until then.
cudaError_t launch_gemm_argmax_grouped(const void* a, long Mtot, const void* b, long Ntot, int K, bool f8,
                                       GemmGroup* hgroups, int ngroups, GemmGroup* dgroups,
                                       const GemmArgmaxArgs& g, int num_sms, cudaStream_t st);

// ---- contract.cu (operands of the contraction, selection, FP64 rescoring) ------
// Fourier band cube of the reference map: (2R+3)^3 float2, frequencies -(R+1)..R+1.
void launch_map_checker(const float* map, int nx, float2* work, cudaStream_t st);
void launch_map_band(const float2* ft, int nx, int R, float2* cube, cudaStream_t st);
// The band cube as a linear-filtering 3D texture (for the section build).
cudaError_t make_cube_texture(const float2* cube, int R, cudaStream_t st, cudaArray_t* arr,
                              cudaTextureObject_t* tex);
void free_cube_texture(cudaArray_t arr, cudaTextureObject_t tex);
// Rows n0 .. n0+count-1 of B (orientation n = view * nom + iomega), unit norm, BF16.
// sigma > 0 (with lin = the band cube in memory): Gaussian-kernel interpolation of
// width sigma voxels over the 27 voxels around the nearest one instead of the texture's
// trilinear filtering
cudaError_t launch_slice_bf16(cudaTextureObject_t cube, int R, const int2* samples, int S, int Kpad,
                              const float* views, int nom, float step, long n0, long count, void* B,
                              cudaStream_t st, const float2* lin = nullptr, float sigma = 0.0f, float sc = 1.0f);
// (R: the band cube's radius, its side 2 R + 3; sc: cube voxels per frequency unit, 2 for
// the cube of the map zero-padded to twice its side)
// Rows of each particle's local grid (k_slice_bf16_local): count = particles x (2 m + 1)^3;
// pctf (particles x S, launch_particle_norm): rows normalised by |CTF S| (the unbiased
// projection-matching score, A rows normalised by |P|), else by |S|
cudaError_t launch_slice_bf16_local(cudaTextureObject_t cube, int R, const int2* samples, int S, int Kpad,
                                    const float* centre, int m, float step, long count, void* B, cudaStream_t st,
                                    const float2* lin = nullptr, float sigma = 0.0f, long lpitch = 0,
                                    const float* pctf = nullptr, float sc = 1.0f);
// norm: sum |CTF P|^2 per particle; pc: CTF P per sample (FP64); norm0: sum |P|^2; pctf:
// the CTF at each sample
void launch_particle_norm(const float2* band, const float* ctf, Band bd, const int2* samples, int S,
                          int B, double* norm, cudaStream_t st, double2* pc = nullptr, double* norm0 = nullptr,
                          float* pctf = nullptr);
// Rows (p, o) of A, p < B, o < O; origins: O x 2 (x, y) pixels, absolute, or relative to
// each particle's own origin poff[p] = (x, y) when poff is given.
void launch_build_a(const float2* band, const float* ctf, Band bd, const int2* samples, int S, int Kpad,
                    const float* origins, int O, const double* norm, int B, void* A, cudaStream_t st,
                    const float* poff = nullptr);
// Best origin per (particle, tile) (tile_*: B x ntiles scratch), then the k best tiles
// per particle: distinct orientations with their best origin and CC.
void launch_select_topk(const float* topv, const int* topi, int O, int ntiles, int k, int B,
                        float* tile_v, int* tile_o, int* tile_orig, int* orient, int* origin, float* cc,
                        cudaStream_t st);
// cand: B x k x (theta, phi, omega, x, y); out: B x k FP64 cross-correlations
// scratch: cc_fp64_scratch(k, B) doubles
long cc_fp64_scratch(int k, int B);
// FP64 CC of k candidates per particle; pcband: each particle's CTF x (a, b) per sample in
// FP64 and pnorm its FP64 norm (launch_particle_norm).  With pctf and pnorm = sum |P|^2
// (norm0): the unbiased score sum Re(P conj(CTF S)) / (|P| |CTF S|)
void launch_cc_fp64(const float2* cube, const double2* pcband, Band bd, const int2* samples, int S,
                    const float* cand, int k, int B, const double* pnorm, double* scratch, double* out,
                    cudaStream_t st, float sigma = 0.0f, const float* pctf = nullptr, int cube_r = -1,
                    float sc = 1.0f);

// ---- learned orientation proposer (learn.cu) ----
constexpr int LP_NR = 64, LP_NT = 128;   // polar feature: radii over [minR, maxR] x angles over [0, 180)
constexpr int LP_C1 = 16, LP_C2 = 32, LP_C3 = 32, LP_C4 = 32, LP_CM = 16;
constexpr int LP_MIXK = LP_C4 * (LP_NR / 8);  // (channel, radius) inputs of the mix
// the n^3 map zero-padded to (2n)^3, checkerboarded, complex
void launch_lp_pad_checker(const float* map, int n, float2* out, cudaStream_t st);
// transforms of B rendered particles (Fourier slice of the band cube texture of the
// map padded scale times, CTF, origin shift) over |h| <= R1; par[b] = (df1, df2,
// astig, ox, oy), volt <= 0: no CTF
void launch_lp_render(cudaTextureObject_t cube, int Rc, int R1, int scale, int nx, const float* eul, const float* par,
                      int B, float apix, float volt, float cs, float ampwg, float d2r, float2* ft, cudaStream_t st);
void launch_lp_cplx_to_real(const float2* in, int nx, int B, float* out, float* var, cudaStream_t st);
void launch_lp_add_noise(float* img, int nx, int B, const float* var, float snr, unsigned long long seed,
                         cudaStream_t st);
void launch_lp_features(const float2* band, const Band& bd, int B, float* feat, cudaStream_t st);
cudaError_t launch_lp_conv3(const float* in, int B, int Cin, int H, const float* W, const float* bias, int Cout,
                            bool relu, float* out, cudaStream_t st);
// accumulates into dW, db (zero them first)
cudaError_t launch_lp_conv3_wgrad(const float* in, const float* dpre, int B, int Cin, int H, int Cout, float* dW,
                                  float* db, cudaStream_t st);
// The same two convolutions on the tensor cores (conv_tc.cu, tcgen05 kind::tf32): Cin <= 32
// (wgrad: 1 or a multiple of 8), Cout 16 or 32; *err is set if a wait timed out.
cudaError_t launch_lp_conv3_tc(const float* in, int B, int Cin, int H, const float* W, const float* bias, int Cout,
                               bool relu, float* out, int* err, cudaStream_t st);
cudaError_t launch_lp_conv3_wgrad_tc(const float* in, const float* dpre, int B, int Cin, int H, int Cout, float* dW,
                                     float* db, int* err, cudaStream_t st);
void launch_lp_relu_grad(const float* out, const float* dout, long n, float* dpre, cudaStream_t st);
void launch_lp_flip(const float* W, int Cout, int Cin, float* Wf, cudaStream_t st);
void launch_lp_pool(const float* a, int B, int C, int Hout, float* p, cudaStream_t st);
// with a (the pooled layer's ReLU output, or nullptr): the ReLU gate applied too
void launch_lp_pool_grad(const float* dp, int B, int C, int Hout, const float* a, float* da, cudaStream_t st);
void launch_lp_mix(const float* x, int B, const float* W5, const float* b5, float* g, cudaStream_t st);
void launch_lp_mix_grad(const float* x, const float* dg, int B, const float* W5, float* dx, float* dW5, float* db5,
                        cudaStream_t st);
// the head through 128-point real transforms; scratch of lp_head_scratch(B, V) float2,
// kept between a forward and its backward
long lp_head_scratch(int B, int V);
cudaError_t launch_lp_head(const float* g, const float* T, int B, int V, float* sc, float2* scratch, cudaStream_t st);
void launch_lp_head_grad(const float* g, const float* T, const float* dsc, int B, int V, float* dg, float* dT,
                         float2* scratch, cudaStream_t st);
// truth[b] = (view unit vector x, y, z, shift); sv degrees, ss shifts
void launch_lp_loss(const float* sc, int B, int V, const float* vview, const float* truth, float sv, float ss,
                    float* dsc, float* loss, cudaStream_t st);
void launch_lp_adam(float* w, const float* g, float* m, float* v, long n, float lr, int step, cudaStream_t st);
// sc is overwritten (taken cells set to -inf)
void launch_lp_topk(float* sc, int B, int V, int k, int* cell, float* val, cudaStream_t st);

// dst row r = src row idx[r] (row_bytes a multiple of 16), n rows
// per particle b of B: the k best of its O x seg[b].y (value, column) entries at
// topv/topi + seg[b].x with distinct columns -> col, origin, cc [B][k]
void launch_select_distinct(float* topv, const int* topi, int O, const int2* seg, int B, int k, int* col,
                            int* origin, float* cc, cudaStream_t st);
// FP8-e4m3 operands (contract.cu): per-band max |B| (R+1 bands, float bits) over every
// stride-th row; B8 = e4m3(B x mulB) with rows of Kpad8 bytes; A8 rows with mulA and the
// per-particle exponent fexp (written by launch_build_a8).
cudaError_t launch_band_absmax(const void* B, long n, int Kpad, const int2* samples, int S, int nband, int stride,
                               unsigned* out, int sms, cudaStream_t st);
cudaError_t launch_b_to_e4m3(const void* B, long n, int Kpad, int S, const float* mulB, int Kpad8, void* B8,
                             cudaStream_t st);
void launch_build_a8(const float2* band, const float* ctf, Band bd, const int2* samples, int S, int Kpad8,
                     const float* origins, int O, const double* norm, const float* mulA, int* fexp, int B, void* A8,
                     cudaStream_t st, const float* poff = nullptr);

// ---- fsc.cu: half-map FSC and the FSC-weighted map ---------------------------
struct FscArgs {
    const float *fa1, *fb1, *wg1;  // odd tnf partial, (maxR+1)(2maxR+1)^2 each
    const float *fa2, *fb2, *wg2;  // even tnf partial
    int nx, max_r;
};
// sums: 3 x (maxR+1) FP64 (cross, |odd|^2, |even|^2 per shell)
cudaError_t launch_fsc_shells(const FscArgs& a, double* sums, int sms, cudaStream_t st);
// wt: maxR+1 shell weights; vol: nx^3 complex, zeroed and filled with cmplx(fa, fb)
cudaError_t launch_fsc_fold(const FscArgs& a, const float* wt, float2* vol, cudaStream_t st);

// ---- center.cu: mode-3 origin centring (buffers of B x nx^2, float2 = (a, b) in the
// img2d_FFT convention b = -Im) -------------------------------------------------
cudaError_t launch_mask3d(float* map, int nx, float mask, double* acc2, cudaStream_t st);
cudaError_t launch_center_ft(const float2* ft, int nx, float* fr, float* fi, cudaStream_t st);
void launch_ref_post(float2* b, long n, float s, cudaStream_t st);
void launch_lowpass(float2* b, int nx, long n, int lp, cudaStream_t st);
void launch_ctf_mul(float2* b, const float* ctf, long n, cudaStream_t st);
void launch_real_shift(const float2* b, int nx, long n, float* out, cudaStream_t st);
void launch_pack_shift(const float* re, const float* im, int nx, long n, float2* b, cudaStream_t st);
void launch_pack(const float* re, long n, float2* b, cudaStream_t st);
void launch_norm(float* img, int nx, int B, cudaStream_t st);
void launch_cross_power(float2* f1, const float2* f2, int nx, long n, cudaStream_t st);
void launch_rot180(float* a1, float* a2, int nx, long n, cudaStream_t st);
void launch_peak(const float2* cc, int nx, int B, int half, float* out, cudaStream_t st);

// ---- local.cu: local_box's sub-image stack mode (loc_box.f90) -----------------
// work[b] = checkerboard x imgs[src[b]] as complex rows (B whole images of nx0^2)
void launch_lb_checker(const float* imgs, int nx0, const int* src, int B, float2* work, cudaStream_t st);
// the forward transform's 1/N^2 and the phase ramp of the shift xy[b] = (x, y)
void launch_lb_phase(float2* work, int nx0, const float* xy, int B, cudaStream_t st);
// n sub-images: hk[k] = (hx0, ky0, slot of the inverse-transformed image), normalised
void launch_lb_cut(const float2* work, int nx0, const int* hk, int n, int sub, float* out, cudaStream_t st);
// host geometry (local_host.cpp): records and source particle per (particle, rotation)
int local_box_stack_geometry(const cryoim_particle* parts, int P, const float* sym, int nsym, float loc_x,
                             float loc_y, float loc_z, float apix, int nx0, int sub, float pr_threshold,
                             float boundx, cryoim_local_particle* out, int* src);

// ---- local.cu: local_refine's sub-particle refinement ------------------------
cudaError_t launch_local_softmask(float* map, int nx, float mask, double* acc2, cudaStream_t st);
cudaError_t launch_local_ft(const float2* ft, int nx, float* fr, float* fi, cudaStream_t st);
// hk: B x (hx0, ky0); out: B x nx^2 windows of the B whole images (nx0^2 each)
void launch_local_box(const float* imgs, int nx0, const int* hk, int nx, int normalize, int B, float* out,
                      cudaStream_t st);
// dfs: B x (df1, df2, astig) with defocus in Angstrom; ctf: B x nx^2
void launch_local_ctf(const float* dfs, int nx, float apix, float vol, float cs, float ampwg, int B, float* ctf,
                      cudaStream_t st);
void launch_wlp(float2* b, int nx, long n, float max_r, cudaStream_t st);
void launch_local_pr(const float* cand, int C, const float* fr, const float* fi, int nx, const float2* part,
                     const float* ctf, float max_r, int B, float* out, cudaStream_t st);

// ---- mapops.cu: whole-map real-space operations ------------------------------
// real-space icosahedral average of an nx^3 map (in != out), radius r0 pixels
cudaError_t launch_icosavg(const float* in, int nx, float r0, const float* ops, int nsym, float* out,
                           cudaStream_t st);
// real part with the (-1)^(x+y+z) origin shift, zero beyond r0 (merge_reconstruct_FSC.f90)
cudaError_t launch_merge_real(const float2* vol, int nx, float r0, float* map, cudaStream_t st);

}  // namespace cryoim
