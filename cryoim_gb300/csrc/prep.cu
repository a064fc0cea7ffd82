// prep.cu — per-image preprocessing, CTF, amplitude-cut fit, orientation tables,
// reconstruction fold and projections.
//
// Compiled with -fmad=false: every FP32 expression rounds where the Fortran's does
// (icosprocess is built without fused multiply-add), so these kernels reproduce the
// reference's preprocessing to the last bit of its expression order.  Reductions the
// reference does sequentially in FP32 are done here in FP64 (then rounded), which is
// closer to the exact value than the reference and independent of thread order.
#include <cstdio>

#include "geom.cuh"
#include "kernels.h"

namespace cryoim {
namespace {

struct HostAngles {
    float pi, d2r, r2d;
};
HostAngles angles() {
    Angles a = host_angles();
    return HostAngles{a.pi, a.deg2rad, a.rad2deg};
}

__device__ double block_sum_d(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    double r = 0;
    if (threadIdx.x < 32) {
        r = (l < nw) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        if (l == 0) sh[0] = r;
    }
    __syncthreads();
    r = sh[0];
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------
// mask / normalise / checkerboard: img2d_norm.f90:1-22, img2d_mask.f90:2-49,
// and the (-1)^(hx+ky) multiply of ort_globesearch.f90:51
// ---------------------------------------------------------------------------
// h + l += x with Knuth's TwoSum: the pair holds the running sum to ~2^-48 relative in
// FP32 arithmetic (GB300's FP64 pipe is far slower than its FP32 pipe)
__device__ __forceinline__ void two_sum_acc(float& h, float& l, float x) {
    const float s2 = h + x, bb = s2 - h;
    l += (h - (s2 - bb)) + (x - bb);
    h = s2;
}

// One block of 1024 threads per image; warp w walks rows w, w + 32, ..., its lanes the
// columns, so no pixel index is split by a division.  The image sums the reference takes
// in FP64 are FP32 TwoSum pairs per thread (exact to far below FP32 rounding), combined
// in FP64 across the block.
__global__ void k_prep_images(const float* __restrict__ imgs, int nx,
                              const float* __restrict__ ox, const float* __restrict__ oy,
                              int use_mask, float mask, int normalize, float pi,
                              float2* __restrict__ out, int* flag) {
    __shared__ double sh[32];
    const int p = blockIdx.x;
    const long nn = (long)nx * nx;
    const float* img = imgs + p * nn;
    float2* o = out + p * nn;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int bad = 0;
    float avg = 0.f, nd = 1.f;
    if (normalize) {
        float h = 0.f, l = 0.f;
        for (int iy = warp; iy < nx; iy += nw)
            for (int ix = lane; ix < nx; ix += 32) two_sum_acc(h, l, img[(long)iy * nx + ix]);
        const double s = block_sum_d((double)h + (double)l, sh);
        avg = (float)s / (float)nn;
        h = 0.f, l = 0.f;
        for (int iy = warp; iy < nx; iy += nw)
            for (int ix = lane; ix < nx; ix += 32) {
                const float d = img[(long)iy * nx + ix] - avg;
                two_sum_acc(h, l, __fmul_rn(d, d));  // the square rounded to FP32, as the reference
            }
        const double s2 = block_sum_d((double)h + (double)l, sh);
        nd = sqrtf((float)s2 / (float)nn);
    }
    const int hh = nx / 2;
    float R1 = mask - 3.0f;
    if (R1 <= 0.0f) R1 = 0.0f;
    float R2 = mask + 3.0f;
    if (R2 > (float)hh) R2 = (float)hh;
    const float x0 = ox[p] + (float)hh, y0 = oy[p] + (float)hh;
    double summ = 0;
    if (use_mask) {
        float h = 0.f, l = 0.f;
        int cnt = 0;
        for (int iy = warp; iy < nx; iy += nw) {
            const float yy = (-y0 + (float)iy) * (-y0 + (float)iy);
            for (int ix = lane; ix < nx; ix += 32) {
                const float xx = (-x0 + (float)ix) * (-x0 + (float)ix);
                const float ra = sqrtf(yy + xx);
                if (ra > R1 && ra <= R2) {
                    float v = img[(long)iy * nx + ix];
                    if (normalize) v = (v - avg) / nd;
                    two_sum_acc(h, l, v);
                    ++cnt;
                }
            }
        }
        summ = block_sum_d((double)h + (double)l, sh);
        const double c = block_sum_d((double)cnt, sh);
        if (c != 0.0) summ = summ / (double)(float)c;
    }
    for (int iy = warp; iy < nx; iy += nw) {
        const float yy = (-y0 + (float)iy) * (-y0 + (float)iy);
        for (int ix = lane; ix < nx; ix += 32) {
            const long i = (long)iy * nx + ix;
            float v = img[i];
            if (!isfinite(v)) bad = 1;
            if (normalize) v = (v - avg) / nd;
            if (use_mask) {
                const float xx = (-x0 + (float)ix) * (-x0 + (float)ix);
                const float ra = sqrtf(yy + xx);
                if (ra > R1 && ra <= R2) {
                    float edge = (1.0f + cosf(pi * (ra - R1) / 6.0f)) / 2.0f;
                    v = (float)((double)(v * edge) + (double)(1.0f - edge) * summ);
                }
                if (ra > R2) v = (float)summ;
            }
            if ((ix + iy) & 1) v = -v;
            o[i] = make_float2(v, 0.0f);
        }
    }
    if (bad) atomicOr(flag, 1);
}

// floor(sqrt(v)) and ceil(sqrt(v)) of a non-negative integer, exactly
__device__ __forceinline__ int isqrt_floor(int v) {
    int s = (int)sqrtf((float)v);
    while (s > 0 && s * s > v) --s;
    while ((s + 1) * (s + 1) <= v) ++s;
    return s;
}
__device__ __forceinline__ int isqrt_ceil(int v) {
    const int s = isqrt_floor(v);
    return s * s < v ? s + 1 : s;
}

// FT_amp_expfit.f90:27-46: per-ring means, log, 2x2 least squares, Fcut.
__device__ void expfit_finish(const double* sfav, const double* sres, const int* snum, int nr,
                              float* out) {
    float aa11 = 0.f, aa12 = 0.f, aa22 = 0.f, bb1 = 0.f, bb2 = 0.f;
    for (int k = 0; k < nr; ++k) {
        float fa = (float)sfav[k], rl = (float)sres[k];
        int num = snum[k];
        float fl;
        if (num > 0 && fa > 0.0f) {
            rl = rl / (float)num;
            fl = logf(fa / (float)num);
        } else {
            fl = 0.0f;
        }
        aa11 = aa11 + rl * rl;
        aa12 = aa12 + rl * 1.0f;
        aa22 = aa22 + 1.0f * 1.0f;
        bb1 = bb1 + rl * fl;
        bb2 = bb2 + 1.0f * fl;
    }
    float aa21 = aa12;
    float x2 = (bb2 - bb1 * aa21 / aa11) / (aa22 - aa12 * aa21 / aa11);
    float x1 = (bb1 - aa12 * x2) / aa11;
    for (int k = 0; k < nr; ++k) {
        float rl = (float)sres[k];
        int num = snum[k];
        if (num > 0 && (float)sfav[k] > 0.0f) rl = rl / (float)num;
        out[k] = expf(rl * x1 + x2) * 0.8f;
    }
}

// ---------------------------------------------------------------------------
// after the forward FFT: 1/nx^2, b = -Im (img2d_FFT.f90:18-19, FFTW.f90:185),
// Fcut fit (FT_amp_expfit.f90:13-25), optional origin shift (img2d_FT_centshift.f90:8-16)
// and extraction of the band window.
// ---------------------------------------------------------------------------
__global__ void k_post_fft(const float2* __restrict__ fft, Band bd, const float* __restrict__ sx,
                           const float* __restrict__ sy, float pi, float2* __restrict__ band,
                           float* __restrict__ fcut) {
    extern __shared__ double dsm[];
    const int nr = bd.nr, R = bd.max_r, nx = bd.nx, h = nx / 2;
    double* sfav = dsm;
    double* sres = dsm + nr;
    int* snum = (int*)(dsm + 2 * nr);
    const int p = blockIdx.x;
    const long nn = (long)nx * nx;
    const float2* f = fft + p * nn;
    const float s = (float)nn;
    if (fcut) {  // (no amplitude cut asked: the band only)
        // ring sums over the ky >= 0 half plane, one warp per ring as in k_tmpl_fcut
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        for (int ir = bd.min_r + warp; ir <= R; ir += nw) {
            float fh = 0.f, fl = 0.f, rh = 0.f, rl = 0.f;
            int n = 0;
            const int lo = ir * ir - ir + 1, hi = ir * ir + ir;
            for (int ky = lane; ky <= ir; ky += 32) {
                const int k2 = ky * ky;
                if (k2 > hi) continue;
                const int hmax = isqrt_floor(hi - k2);
                const int hmin = lo - k2 <= 0 ? 0 : isqrt_ceil(lo - k2);
                for (int hx = hmin; hx <= hmax; ++hx) {
                    const float rad = sqrtf((float)(hx * hx + k2));
                    for (int sgn = (hx == 0 ? 1 : -1); sgn <= 1; sgn += 2) {
                        const float2 v = f[(long)(ky + h) * nx + (sgn * hx + h)];
                        const float a = v.x / s, b = -(v.y / s);
                        two_sum_acc(fh, fl, sqrtf(a * a + b * b));
                        two_sum_acc(rh, rl, rad);
                        ++n;
                    }
                }
            }
            double fa = (double)fh + (double)fl, rs = (double)rh + (double)rl;
            for (int o = 16; o > 0; o >>= 1) {
                fa += __shfl_xor_sync(0xffffffffu, fa, o);
                rs += __shfl_xor_sync(0xffffffffu, rs, o);
                n += __shfl_xor_sync(0xffffffffu, n, o);
            }
            if (lane == 0) {
                sfav[ir - bd.min_r] = fa;
                sres[ir - bd.min_r] = rs;
                snum[ir - bd.min_r] = n;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) expfit_finish(sfav, sres, snum, nr, fcut + (long)p * nr);
    }
    const int W = bd.W;
    const bool shift = (sx != nullptr);
    const float xs = shift ? sx[p] + (float)h : 0.f, ys = shift ? sy[p] + (float)h : 0.f;
    float2* ob = band + (long)p * W * W;
    for (int q = threadIdx.x; q < W * W; q += blockDim.x) {
        int by = q / W, bx = q % W;
        int hi = bd.off + bx, ki = bd.off + by;
        float2 v = f[(long)ki * nx + hi];
        float a = v.x / s, b = -(v.y / s);
        if (shift) {
            int hx = hi - h, ky = ki - h;
            float phase = 2.0f * pi * (xs * (float)hx + ys * (float)ky) / (float)nx;
            float c = cosf(phase), sn = sinf(phase);
            float fr = (a * c + b * sn);
            float fi = (-a * sn + b * c);
            a = fr;
            b = fi;
        }
        ob[q] = make_float2(a, b);
    }
}

// getCTF2d.f90:2-29 evaluated over the band window.
__global__ void k_ctf_band(Band bd, const float* __restrict__ dfs, float apix, float vol, float cs0,
                           float ampwg, float pi, float* __restrict__ ctf) {
    const int p = blockIdx.y;
    const int W = bd.W, R = bd.max_r;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= W * W) return;
    const float d2r = pi / 180.0f;
    float lam = 0.387818f / sqrtf(1.0f * vol * (1.0f + 0.978459E-3f * vol));
    float cs = cs0 * 1.0e7f, df1 = dfs[p * 3] * 1.0e4f, df2 = dfs[p * 3 + 1] * 1.0e4f;
    float astig = dfs[p * 3 + 2] * d2r;
    int ky = q / W - R, hx = q % W - R;
    float phi = atan2f((float)ky, (float)hx);
    if (phi < 0.0f) phi = phi + 2.0f * pi;
    phi = phi - astig;
    float c = cosf(phi), s = sinf(phi);
    float df = df1 * (c * c) + df2 * (s * s);
    float res = sqrtf((float)(hx * hx + ky * ky)) / (float)bd.nx / apix;
    float r2 = res * res, r4 = r2 * r2, lam3 = lam * lam * lam;
    float phase = 2.0f * pi * (-(cs * lam3 * r4 / 4.0f) + df * lam * r2 / 2.0f);
    float sq = sqrtf(1.0f - ampwg * ampwg);
    ctf[(long)p * W * W + q] = -(sq * sinf(phase) + ampwg * cosf(phase));
}

// Fcut of (template x CTF): cal_crosslin_PR_omega.f90:34-38, hoisted per particle.
// Template amplitude cuts under each particle's CTF (FT_amp_expfit.f90 on template x
// CTF over the ky >= 0 half plane): one block per (template, particle), one warp per
// ring at a time.  Ring ir holds the pixels with int(|h| + 1/2) = ir, i.e. the integer
// range ir^2 - ir + 1 <= hx^2 + ky^2 <= ir^2 + ir; lane l takes rows ky = l, l + 32, ...
// and the ring's hx on them, summing |t c|, the radius and the count in FP64 (then a
// warp reduction: no atomics, a fixed order).
__global__ void k_tmpl_fcut(const float2* __restrict__ tband, int T, const float* __restrict__ ctf,
                            Band bd, float* __restrict__ tfcut) {
    extern __shared__ double dsm[];
    const int nr = bd.nr, R = bd.max_r, W = bd.W;
    double* sfav = dsm;
    double* sres = dsm + nr;
    int* snum = (int*)(dsm + 2 * nr);
    const int i = blockIdx.x, p = blockIdx.y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const float2* tb = tband + (long)i * W * W;
    const float* cb = ctf + (long)p * W * W;
    for (int ir = bd.min_r + warp; ir <= R; ir += nw) {
        // per lane an FP32 pair (two_sum_acc), to FP64 once per lane
        float fh = 0.f, fl = 0.f, rh = 0.f, rl = 0.f;
        int n = 0;
        const int lo = ir * ir - ir + 1, hi = ir * ir + ir;
        for (int ky = lane; ky <= ir; ky += 32) {
            const int k2 = ky * ky;
            if (k2 > hi) continue;
            const int hmax = isqrt_floor(hi - k2);
            const int hmin = lo - k2 <= 0 ? 0 : isqrt_ceil(lo - k2);
            for (int hx = hmin; hx <= hmax; ++hx) {
                const float rad = sqrtf((float)(hx * hx + k2));
                for (int sgn = (hx == 0 ? 1 : -1); sgn <= 1; sgn += 2) {
                    const int b = (ky + R) * W + (sgn * hx + R);
                    const float c = cb[b];
                    const float2 t = tb[b];
                    const float a2 = t.x * c, b2 = t.y * c;
                    two_sum_acc(fh, fl, sqrtf(a2 * a2 + b2 * b2));
                    two_sum_acc(rh, rl, rad);
                    ++n;
                }
            }
        }
        double fa = (double)fh + (double)fl, rs = (double)rh + (double)rl;
        for (int o = 16; o > 0; o >>= 1) {
            fa += __shfl_xor_sync(0xffffffffu, fa, o);
            rs += __shfl_xor_sync(0xffffffffu, rs, o);
            n += __shfl_xor_sync(0xffffffffu, n, o);
        }
        if (lane == 0) {
            sfav[ir - bd.min_r] = fa;
            sres[ir - bd.min_r] = rs;
            snum[ir - bd.min_r] = n;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) expfit_finish(sfav, sres, snum, nr, tfcut + ((long)p * T + i) * nr);
}

// icos_crosslin_angle.f90 for every (view, template, operator).
__global__ void k_alpha_table(const float* __restrict__ views, int V, const float* __restrict__ tort,
                              int T, const float* __restrict__ ops, float d2r, float r2d,
                              float2* __restrict__ alpha) {
    long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long total = (long)V * T * 60;
    if (q >= total) return;
    int j = (int)(q % 60);
    int i = (int)((q / 60) % T);
    int v = (int)(q / (60L * T));
    float e1[9], e2[9];
    euler_mat(views[v * 2], views[v * 2 + 1], 0.0f, d2r, e1);
    euler_mat(tort[i * 3], tort[i * 3 + 1], tort[i * 3 + 2], d2r, e2);
    float a1, a2;
    crosslin_pair(e1, e2, ops + j * 9, r2d, &a1, &a2);
    alpha[q] = make_float2(a1, a2);
}

// ort_cent_11.f90:1-94 (state = theta, phi, omega, x, y, pr per image).
__global__ void k_refine_candidates(float* __restrict__ state, int B, float dang, float dtran,
                                    const float* __restrict__ ops, float d2r,
                                    float* __restrict__ cand) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= B) return;
    float* st = state + p * 6;
    float th0 = st[0], ph0 = st[1], om0 = st[2], x0 = st[3], y0 = st[4];
    asu_fold(&th0, &ph0, &om0, ops, d2r);
    st[0] = th0; st[1] = ph0; st[2] = om0;
    for (int jj = 0; jj <= 10; ++jj) {
        float th = th0, ph = ph0, om = om0, x = x0, y = y0;
        switch (jj) {
            case 1: th = th0 - dang; break;
            case 2: th = th0 + dang; break;
            case 3: ph = ph0 - dang; break;
            case 4: ph = ph0 + dang; break;
            case 5: om = om0 - dang; break;
            case 6: om = om0 + dang; break;
            case 7: x = x0 - dtran; break;
            case 8: x = x0 + dtran; break;
            case 9: y = y0 - dtran; break;
            case 10: y = y0 + dtran; break;
            default: break;
        }
        asu_fold(&th, &ph, &om, ops, d2r);
        float* o = cand + ((long)p * 11 + jj) * 5;
        o[0] = th; o[1] = ph; o[2] = om; o[3] = x; o[4] = y;
    }
}

// One block per candidate row: its Euler matrix and the T template matrices once in shared
// memory, then crosslin_pair for every (template, operator).
__global__ void k_refine_alpha(const float* __restrict__ cand, long ncand_rows,
                               const float* __restrict__ tort, int T, const float* __restrict__ ops,
                               float d2r, float r2d, float2* __restrict__ alpha) {
    extern __shared__ float em[];  // [9] candidate, then [T][9] templates
    const long pc = blockIdx.x;    // p * ncand + c
    if (pc >= ncand_rows) return;
    const float* c = cand + pc * 5;
    if (threadIdx.x == 0) euler_mat(c[0], c[1], c[2], d2r, em);
    for (int i = threadIdx.x; i < T; i += blockDim.x)
        euler_mat(tort[i * 3], tort[i * 3 + 1], tort[i * 3 + 2], d2r, em + 9 + 9 * i);
    __syncthreads();
    float2* out = alpha + pc * T * 60;
    for (int q = threadIdx.x; q < T * 60; q += blockDim.x) {
        const int i = q / 60, j = q - 60 * i;
        float a1, a2;
        crosslin_pair(em, em + 9 + 9 * i, ops + j * 9, r2d, &a1, &a2);
        out[q] = make_float2(a1, a2);
    }
}

// ort_refinement.f90:85-91: first minimum of the 11 scores.
__global__ void k_refine_select(const float* __restrict__ cand, const float* __restrict__ pr, int B,
                                float* __restrict__ state) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= B) return;
    const float* v = pr + p * 11;
    int mn = 0;
    for (int jj = 1; jj <= 10; ++jj)
        if (v[jj] < v[mn]) mn = jj;
    const float* c = cand + ((long)p * 11 + mn) * 5;
    float* st = state + p * 6;
    st[0] = c[0]; st[1] = c[1]; st[2] = c[2]; st[3] = c[3]; st[4] = c[4]; st[5] = v[mn];
}

// ---------------------------------------------------------------------------
// reconstruction finish: reconstruct.f90:151-241 (Friedel completion, divide by the
// CTF^2 weights in FP64, (-1)^(h+k+l) sign) into FFT3d = cmplx(fa, -fb).
// ---------------------------------------------------------------------------
__device__ __forceinline__ long acc_index(const Band& bd, int hx, int ky, int lz) {
    return acc_cell(bd, hx, ky, lz);
}
__device__ __forceinline__ long vol_index(int nx, int hx, int ky, int lz) {
    int h = nx / 2;
    return ((long)(lz + h) * nx + (ky + h)) * nx + (hx + h);
}
__device__ __forceinline__ float qdiv(float a, float w) { return (float)((double)a / (double)w); }

// reconstruct.f90:156-157 keeps |h| <= maxR with a real radius; merge_reconstruct.f90:10,
// 42 stores the radius in an integer, which keeps int(|h|) <= maxR.
__device__ __forceinline__ bool in_fold(int d2, int R, int int_shell) {
    const float dr = sqrtf((float)d2);
    return int_shell ? (int)dr <= R : dr <= (float)R;
}

__global__ void k_rec_fold_plane0(const float4* __restrict__ acc, Band bd, int int_shell,
                                  float2* __restrict__ vol) {
    const int R = bd.max_r, span = 2 * R + 1;
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    int n_a = R * span, n_b = R;
    if (q > n_a + n_b) return;
    if (q == n_a + n_b) {  // origin: reconstruct.f90:205-208
        float4 v = acc[acc_index(bd, 0, 0, 0)];
        vol[vol_index(bd.nx, 0, 0, 0)] = make_float2(qdiv(v.x, v.z), -0.0f);
        return;
    }
    int hx, ky;
    if (q < n_a) { ky = 1 + q / span; hx = q % span - R; }
    else { ky = 0; hx = 1 + (q - n_a); }
    float4 v1 = acc[acc_index(bd, hx, ky, 0)];
    float4 v2 = acc[acc_index(bd, -hx, -ky, 0)];
    float fa1 = 0.f, fb1 = 0.f, fa2 = 0.f, fb2 = 0.f;
    if (in_fold(hx * hx + ky * ky, R, int_shell)) {
        float w = v1.z + v2.z;
        fa1 = qdiv(v1.x + v2.x, w);
        fb1 = qdiv(v1.y - v2.y, w);
        if (((hx + ky) & 1) == 0) { fa2 = fa1; fb2 = -fb1; }
        else { fa1 = -fa1; fb1 = -fb1; fa2 = fa1; fb2 = -fb1; }
    }
    vol[vol_index(bd.nx, hx, ky, 0)] = make_float2(fa1, -fb1);
    vol[vol_index(bd.nx, -hx, -ky, 0)] = make_float2(fa2, -fb2);
}

__global__ void k_rec_fold_upper(const float4* __restrict__ acc, Band bd, int int_shell,
                                 float2* __restrict__ vol) {
    const int R = bd.max_r, span = 2 * R + 1;
    long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long total = (long)R * span * span;
    if (q >= total) return;
    int hx = (int)(q % span) - R;
    int ky = (int)((q / span) % span) - R;
    int lz = 1 + (int)(q / ((long)span * span));
    float fa1 = 0.f, fb1 = 0.f;
    if (in_fold(hx * hx + ky * ky + lz * lz, R, int_shell)) {
        float4 v = acc[acc_index(bd, hx, ky, lz)];
        fa1 = qdiv(v.x, v.z);
        fb1 = qdiv(v.y, v.z);
        if ((hx + ky + lz) & 1) { fa1 = -fa1; fb1 = -fb1; }
    }
    vol[vol_index(bd.nx, hx, ky, lz)] = make_float2(fa1, -fb1);
    vol[vol_index(bd.nx, -hx, -ky, -lz)] = make_float2(fa1, fb1);
}

// shift3dComplex (FFTW.f90:304-321) and the real part (reconstruct.f90:246-247)
__global__ void k_rec_real(const float2* __restrict__ vol, int nx, float* __restrict__ map) {
    long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long n3 = (long)nx * nx * nx;
    if (q >= n3) return;
    int hx = (int)(q % nx), ky = (int)((q / nx) % nx), lz = (int)(q / ((long)nx * nx));
    float v = vol[q].x;
    map[q] = ((hx + ky + lz) & 1) ? -v : v;
}

// project_template2d.f90:33-73: one thread per output pixel, z summed in order.
__global__ void k_project(const float* __restrict__ map, int nx, const float* __restrict__ eul,
                          float d2r, float* __restrict__ out) {
    __shared__ float rot[9];
    const int o = blockIdx.y;
    if (threadIdx.x == 0) euler_mat(eul[o * 3], eul[o * 3 + 1], eul[o * 3 + 2], d2r, rot);
    __syncthreads();
    const long nn = (long)nx * nx;
    long i2 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i2 >= nn) return;
    const int h = nx / 2;
    const int ix = (int)(i2 % nx), iy = (int)(i2 / nx);
    float acc = 0.0f;
    for (int iz = 0; iz < nx; ++iz) {
        float xp[3] = {(float)ix - (float)h, (float)iy - (float)h, (float)iz - (float)h};
        if (sqrtf(xp[0] * xp[0] + xp[1] * xp[1] + xp[2] * xp[2]) >= (float)(h - 1)) continue;
        float x[3];
        mv3(rot, xp, x);
        x[0] = x[0] + (float)h; x[1] = x[1] + (float)h; x[2] = x[2] + (float)h;
        int jx = (int)x[0], jy = (int)x[1], jz = (int)x[2];
        float xb = x[0] - (float)jx, yb = x[1] - (float)jy, zb = x[2] - (float)jz;
        long n1 = (long)jz * nn + (long)jy * nx + jx;
        acc = acc + (1.f - xb) * (1.f - yb) * (1.f - zb) * map[n1];
        acc = acc + xb * (1.f - yb) * (1.f - zb) * map[n1 + 1];
        acc = acc + (1.f - xb) * yb * (1.f - zb) * map[n1 + nx];
        acc = acc + xb * yb * (1.f - zb) * map[n1 + nx + 1];
        acc = acc + (1.f - xb) * (1.f - yb) * zb * map[n1 + nn];
        acc = acc + xb * (1.f - yb) * zb * map[n1 + nn + 1];
        acc = acc + (1.f - xb) * yb * zb * map[n1 + nn + nx];
        acc = acc + xb * yb * zb * map[n1 + nn + nx + 1];
    }
    out[(long)o * nn + i2] = acc;
}

// project2d_FT3dTo2d.f90:27-84: trilinear central section of a centred 3D FT.
__global__ void k_sections(const float* __restrict__ fre, const float* __restrict__ fim, int nx,
                           const float* __restrict__ eul, float d2r, float* __restrict__ ore,
                           float* __restrict__ oim) {
    __shared__ float rot[9];
    const int o = blockIdx.y;
    if (threadIdx.x == 0) euler_mat(eul[o * 3], eul[o * 3 + 1], eul[o * 3 + 2], d2r, rot);
    __syncthreads();
    const long nn = (long)nx * nx;
    long n = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int h = nx / 2;
    const int ix = (int)(n % nx) - h, iy = (int)(n / nx) - h;
    float xp[3] = {(float)ix, (float)iy, 0.0f}, xx[3];
    mv3(rot, xp, xx);
    float vr = 0.f, vi = 0.f;
    if (!(sqrtf(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]) > (float)(h - 2))) {
        xx[0] = xx[0] + (float)h; xx[1] = xx[1] + (float)h; xx[2] = xx[2] + (float)h;
        int hx = (int)xx[0], ky = (int)xx[1], lz = (int)xx[2];
        float xb = xx[0] - (float)hx, yb = xx[1] - (float)ky, zb = xx[2] - (float)lz;
        long b0 = (long)lz * nn + (long)ky * nx + hx;
        const float w1 = (1.f - xb) * (1.f - yb) * (1.f - zb), w2 = xb * (1.f - yb) * (1.f - zb);
        const float w3 = (1.f - xb) * yb * (1.f - zb), w4 = xb * yb * (1.f - zb);
        const float w5 = (1.f - xb) * (1.f - yb) * zb, w6 = xb * (1.f - yb) * zb;
        const float w7 = (1.f - xb) * yb * zb, w8 = xb * yb * zb;
        vr = w1 * fre[b0] + w2 * fre[b0 + 1] + w3 * fre[b0 + nx] + w4 * fre[b0 + nx + 1] +
             w5 * fre[b0 + nn] + w6 * fre[b0 + nn + 1] + w7 * fre[b0 + nn + nx] +
             w8 * fre[b0 + nn + nx + 1];
        vi = w1 * fim[b0] + w2 * fim[b0 + 1] + w3 * fim[b0 + nx] + w4 * fim[b0 + nx + 1] +
             w5 * fim[b0 + nn] + w6 * fim[b0 + nn + 1] + w7 * fim[b0 + nn + nx] +
             w8 * fim[b0 + nn + nx + 1];
    }
    ore[(long)o * nn + n] = vr;
    oim[(long)o * nn + n] = vi;
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace

void launch_prep_images(const float* imgs, int B, int nx, const float* ox, const float* oy,
                        int use_mask, float mask_px, int normalize, float2* fft, int* flag,
                        cudaStream_t st) {
    k_prep_images<<<B, 1024, 0, st>>>(imgs, nx, ox, oy, use_mask, mask_px, normalize, angles().pi,
                                      fft, flag);
}

void launch_post_fft(const float2* fft, int B, Band bd, const float* sx, const float* sy,
                     float2* band, float* fcut, cudaStream_t st) {
    size_t sm = (size_t)bd.nr * (2 * sizeof(double) + sizeof(int)) + 16;
    k_post_fft<<<B, 1024, sm, st>>>(fft, bd, sx, sy, angles().pi, band, fcut);
}

void launch_ctf_band(int B, Band bd, const float* dfs, float apix, float vol, float cs,
                     float ampwg, float* ctf, cudaStream_t st) {
    dim3 g(cdiv((long)bd.W * bd.W, 256), B);
    k_ctf_band<<<g, 256, 0, st>>>(bd, dfs, apix, vol, cs, ampwg, angles().pi, ctf);
}

void launch_tmpl_fcut(const float2* tband, int T, const float* ctf, int B, Band bd, float* tfcut,
                      cudaStream_t st) {
    size_t sm = (size_t)bd.nr * (2 * sizeof(double) + sizeof(int)) + 16;
    dim3 g(T, B);
    k_tmpl_fcut<<<g, 256, sm, st>>>(tband, T, ctf, bd, tfcut);
}

void launch_alpha_table(const float* views, int V, const float* tort, int T, const float* ops,
                        float2* alpha, cudaStream_t st) {
    long total = (long)V * T * 60;
    HostAngles a = angles();
    k_alpha_table<<<cdiv(total, 128), 128, 0, st>>>(views, V, tort, T, ops, a.d2r, a.r2d, alpha);
}

void launch_refine_candidates(float* state, int B, float dang, float dtran, const float* ops,
                              float* cand, cudaStream_t st) {
    k_refine_candidates<<<cdiv(B, 64), 64, 0, st>>>(state, B, dang, dtran, ops, angles().d2r, cand);
}

void launch_refine_alpha(const float* cand, int B, const float* tort, int T, const float* ops,
                         float2* alpha, cudaStream_t st, int ncand) {
    const long rows = (long)B * ncand;
    const size_t sm = sizeof(float) * 9 * (T + 1);
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_refine_alpha, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    HostAngles a = angles();
    k_refine_alpha<<<(unsigned)rows, 256, sm, st>>>(cand, rows, tort, T, ops, a.d2r, a.r2d, alpha);
}

void launch_refine_select(const float* cand, const float* pr, int B, float* state,
                          cudaStream_t st) {
    k_refine_select<<<cdiv(B, 64), 64, 0, st>>>(cand, pr, B, state);
}

void launch_rec_fold(const float4* acc, Band bd, int int_shell, float2* vol, cudaStream_t st) {
    const int R = bd.max_r, span = 2 * R + 1;
    int n0 = R * span + R + 1;
    k_rec_fold_plane0<<<cdiv(n0, 256), 256, 0, st>>>(acc, bd, int_shell, vol);
    long n1 = (long)R * span * span;
    k_rec_fold_upper<<<cdiv(n1, 256), 256, 0, st>>>(acc, bd, int_shell, vol);
}

void launch_rec_real(const float2* vol, int nx, float* map, cudaStream_t st) {
    long n3 = (long)nx * nx * nx;
    k_rec_real<<<cdiv(n3, 256), 256, 0, st>>>(vol, nx, map);
}

void launch_project(const float* map, int nx, const float* eul, int n, float* out,
                    cudaStream_t st) {
    dim3 g(cdiv((long)nx * nx, 128), n);
    k_project<<<g, 128, 0, st>>>(map, nx, eul, angles().d2r, out);
}

void launch_sections(const float* fre, const float* fim, int nx, const float* eul, int n,
                     float* ore, float* oim, cudaStream_t st) {
    dim3 g(cdiv((long)nx * nx, 256), n);
    k_sections<<<g, 256, 0, st>>>(fre, fim, nx, eul, angles().d2r, ore, oim);
}

}  // namespace cryoim
