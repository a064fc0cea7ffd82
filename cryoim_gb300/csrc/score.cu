// score.cu — cross-common-line phase-residual scoring and symmetrised insertion.
//
// k_pr_omega is the hot kernel of the global search (cal_crosslin_PR_omega.f90 for
// every asymmetric-unit view of every particle).  One CTA owns one (particle, view):
//   * the particle's band-limited Fourier window (W x W float2) sits in shared memory
//     for the whole CTA, so every bilinear tap is a shared-memory load;
//   * thread (g, k) owns omega index k and accumulates PR1(k), PR2(k) in registers over
//     the lines j = g, g+G, ... of every template (no cross-thread reduction until the
//     end of the view), with per-line FP32 partial sums folded into Kahan-compensated
//     running sums;
//   * per template, the 60 x nR template line samples (template x CTF, bilinear) are
//     staged once into shared memory as (amplitude or -1 if below Fcut, phase);
//   * the per-view argmin over omega is folded into a per-particle 64-bit key
//     (PR bits << 32 | column-major index) with atomicMin, which reproduces Fortran
//     minloc's first-occurrence rule.
// The sampling positions x = FR*cos + nx/2 are rounded exactly as the reference
// rounds them (separate multiply and add), so the bilinear taps and weights match it.
#include <cstdio>

#include <type_traits>

#include "geom.cuh"
#include "kernels.h"

namespace cryoim {
namespace {

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}
// h + l += x with Knuth's TwoSum: the pair holds the running sum to ~2^-48 relative in
// FP32 arithmetic (GB300's FP64 pipe is far slower than its FP32 pipe)
__device__ __forceinline__ void two_sum_acc(float& h, float& l, float x) {
    const float s2 = h + x, bb = s2 - h;
    l += (h - (s2 - bb)) + (x - bb);
    h = s2;
}

__device__ __forceinline__ float bilerp(float ax, float ay, float v00, float v10, float v01,
                                        float v11) {
    float bx = 1.0f - ax, by = 1.0f - ay;
    return bx * by * v00 + ax * by * v10 + bx * ay * v01 + ax * ay * v11;
}

struct Consts {
    float d2r, r2d, pi, tpi;
};

// Template line sample (template x CTF, bilinear) at angle alpha2, radius fr.
__device__ __forceinline__ void tmpl_sample_cs(const float2* __restrict__ tb, const float* __restrict__ cb,
                                               int W, int offW, float nxh, float cs, float sn, float fr,
                                               float* re, float* im) {
    float x = __fadd_rn(__fmul_rn(fr, cs), nxh), y = __fadd_rn(__fmul_rn(fr, sn), nxh);
    int lx = (int)x, ly = (int)y;
    float ax = __fsub_rn(x, (float)lx), ay = __fsub_rn(y, (float)ly);
    int b0 = ly * W + lx - offW;
    float2 t00 = tb[b0], t10 = tb[b0 + 1], t01 = tb[b0 + W], t11 = tb[b0 + W + 1];
    if (cb) {
        float c00 = cb[b0], c10 = cb[b0 + 1], c01 = cb[b0 + W], c11 = cb[b0 + W + 1];
        t00.x = __fmul_rn(t00.x, c00); t00.y = __fmul_rn(t00.y, c00);
        t10.x = __fmul_rn(t10.x, c10); t10.y = __fmul_rn(t10.y, c10);
        t01.x = __fmul_rn(t01.x, c01); t01.y = __fmul_rn(t01.y, c01);
        t11.x = __fmul_rn(t11.x, c11); t11.y = __fmul_rn(t11.y, c11);
    }
    *re = bilerp(ax, ay, t00.x, t10.x, t01.x, t11.x);
    *im = bilerp(ax, ay, t00.y, t10.y, t01.y, t11.y);
}

// The same sample from a band stored as (pixel, right neighbour) pairs: two 16-byte loads
// carry the four taps, the values and the arithmetic are tmpl_sample_cs's.
__device__ __forceinline__ void tmpl_sample_pairs(const float4* __restrict__ tb, int W, int offW, float nxh, float cs,
                                                  float sn, float fr, float* re, float* im) {
    float x = __fadd_rn(__fmul_rn(fr, cs), nxh), y = __fadd_rn(__fmul_rn(fr, sn), nxh);
    int lx = (int)x, ly = (int)y;
    float ax = __fsub_rn(x, (float)lx), ay = __fsub_rn(y, (float)ly);
    int b0 = ly * W + lx - offW;
    const float4 r0 = tb[b0], r1 = tb[b0 + W];
    *re = bilerp(ax, ay, r0.x, r0.z, r1.x, r1.z);
    *im = bilerp(ax, ay, r0.y, r0.w, r1.y, r1.w);
}

__device__ __forceinline__ void tmpl_sample(const float2* __restrict__ tb, const float* __restrict__ cb,
                                            int W, int offW, float nxh, float alpha2, float fr,
                                            float d2r, float* re, float* im) {
    float ang = __fmul_rn(alpha2, d2r);
    tmpl_sample_cs(tb, cb, W, offW, nxh, cosf(ang), sinf(ang), fr, re, im);
}

// Angle between two complex numbers z1, z2 from their cross and dot products, in [0, pi]:
// |arg(z2 conj z1)| = the reference's |phase2 - phase1| folded into [0, pi]
// (cal_crosslin_PR_omega.f90:53-60).  atan on [0, 1] is a 6-term odd polynomial fitted
// to atan(t)/t by reweighted least squares on [0, 1] (max error 1.7e-6 rad in FP32).
__device__ __forceinline__ float angle_between(float cross, float dot, float pi) {
    const float a = fabsf(cross), b = fabsf(dot);
    const float mx = fmaxf(a, b), mn = fminf(a, b);
    const float t = mn * __frcp_rn(mx);
    const float s = t * t;
    float p = fmaf(s, -0.011719364672899246f, 0.05264794081449509f);
    p = fmaf(p, s, -0.11642702668905258f);
    p = fmaf(p, s, 0.19354058802127838f);
    p = fmaf(p, s, -0.33262285590171814f);
    p = fmaf(p, s, 0.9999772310256958f);
    float r = t * p;
    r = (a > b) ? 0.5f * pi - r : r;
    return (dot < 0.0f) ? pi - r : r;
}

// angle_between with the hardware reciprocal estimate (relative error ~2^-23, below the
// polynomial's 1.7e-6 rad) in place of the correctly rounded one.
__device__ __forceinline__ float angle_between_est(float cross, float dot, float pi) {
    const float a = fabsf(cross), b = fabsf(dot);
    const float mx = fmaxf(a, b), mn = fminf(a, b);
    float rc;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rc) : "f"(mx));
    const float t = mn * rc;
    const float s = t * t;
    float p = fmaf(s, -0.011719364672899246f, 0.05264794081449509f);
    p = fmaf(p, s, -0.11642702668905258f);
    p = fmaf(p, s, 0.19354058802127838f);
    p = fmaf(p, s, -0.33262285590171814f);
    p = fmaf(p, s, 0.9999772310256958f);
    float r = t * p;
    r = (a > b) ? 0.5f * pi - r : r;
    return (dot < 0.0f) ? pi - r : r;
}

__global__ void __launch_bounds__(768, 1) k_pr_omega(PrOmegaArgs a, int nomp, Consts K) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const Band bd = a.bd;
    const int W = bd.W, nr = bd.nr, minR = bd.min_r;
    float2* sband = reinterpret_cast<float2*>(smraw);
    // per (line, radius): template sample (a2, b2), half amplitude (-1 below its cut),
    // particle cut at that radius
    float4* sline = reinterpret_cast<float4*>(sband + W * W);
    float* sfc0 = reinterpret_cast<float*>(sline + 60 * nr);
    float* salpha = sfc0 + ((nr + 3) & ~3);
    float* sred = salpha + 64;
    unsigned long long* skey = reinterpret_cast<unsigned long long*>(sred + 2 * blockDim.x);

    const int p = blockIdx.y, t = threadIdx.x;
    const int G = blockDim.x / nomp, g = t / nomp, k = t - g * nomp;
    {
        const float4* gb = reinterpret_cast<const float4*>(a.band + (long)p * W * W);
        float4* sb4 = reinterpret_cast<float4*>(sband);
        for (int q = t; q < (W * W) / 2; q += blockDim.x) sb4[q] = gb[q];
        for (int q = t; q < nr; q += blockDim.x) sfc0[q] = a.fcut0[(long)p * nr + q];
    }
    const float nxh = (float)(bd.nx / 2);
    const int offW = bd.off * W + bd.off;
    const float* ctfp = a.ctf ? a.ctf + (long)p * W * W : nullptr;
    const float* tfc = a.tfcut + (long)p * a.tfcut_pstride;
    const float womega = __fmul_rn(a.step, (float)k);
    const int nwarps = blockDim.x >> 5;

    for (int v = blockIdx.x; v < a.V; v += gridDim.x) {
        float pr1 = 0.f, pr2 = 0.f, c1 = 0.f, c2 = 0.f;
        for (int i = 0; i < a.T; ++i) {
            __syncthreads();
            const float2* al = a.alpha + ((long)v * a.T + i) * 60;
            if (t < 60) {
                float2 aa = al[t];
                salpha[t] = (aa.x < 999.0f && aa.y < 999.0f) ? aa.x : 1000.0f;
            }
            const float2* tb = a.tband + (long)i * W * W;
            const float* fct = tfc + (long)i * nr;
            for (int q = t; q < 60 * nr; q += blockDim.x) {
                int j = q / nr, iq = q - j * nr;
                float2 aa = al[j];
                float4 e = make_float4(0.f, 0.f, -1.0f, sfc0[iq]);
                if (aa.x < 999.0f && aa.y < 999.0f) {
                    float re, im;
                    tmpl_sample(tb, ctfp, W, offW, nxh, aa.y, (float)(minR + iq), K.d2r, &re, &im);
                    float amp = sqrtf(re * re + im * im);
                    if (amp >= fct[iq]) { e.x = re; e.y = im; e.z = 0.5f * amp; }
                }
                sline[q] = e;
            }
            __syncthreads();
            if (k < a.nomega) {
                for (int j = g; j < 60; j += G) {
                    const float al1 = salpha[j];
                    if (!(al1 < 999.0f)) continue;
                    const float ang = __fmul_rn(__fsub_rn(al1, womega), K.d2r);
                    float sn, cs;
                    sincosf(ang, &sn, &cs);
                    const float2 csn = make_float2(cs, sn), half2c = make_float2(nxh, nxh);
                    const float4* sl = sline + j * nr;
                    float2 acc = make_float2(0.f, 0.f);  // (sum diff*w, sum w) of this line
#pragma unroll 8
                    for (int iq = 0; iq < nr; ++iq) {
                        const float4 e = sl[iq];
                        if (e.z < 0.0f) continue;
                        const float fr = (float)(minR + iq);
                        // sample position (x, y) = FR (cos, sin) + nx/2, then its cell
                        const float2 xy = __ffma2_rn(make_float2(fr, fr), csn, half2c);
                        const int lx = (int)xy.x, ly = (int)xy.y;
                        const float2 f = __fadd2_rn(xy, make_float2(-(float)lx, -(float)ly));
                        const int b0 = ly * W + lx - offW;
                        const float2 t00 = sband[b0], t10 = sband[b0 + 1];
                        const float2 t01 = sband[b0 + W], t11 = sband[b0 + W + 1];
                        // bilinear on (re, im) pairs: lerp in x on both rows, then in y
                        const float2 ax2 = make_float2(f.x, f.x), ay2 = make_float2(f.y, f.y);
                        const float2 m1 = make_float2(-1.f, -1.f);
                        const float2 v0 = __ffma2_rn(ax2, __ffma2_rn(t00, m1, t10), t00);
                        const float2 v1 = __ffma2_rn(ax2, __ffma2_rn(t01, m1, t11), t01);
                        const float2 z = __ffma2_rn(ay2, __ffma2_rn(v0, m1, v1), v0);
                        const float2 zz = __fmul2_rn(z, z);
                        const float sq = zz.x + zz.y;
                        const float amp1 = sq * rsqrtf(sq);  // NaN for 0: fails the cut
                        // the particle's cut as a select: ~70 % of the lanes pass it, so a
                        // branch would run both sides anyway
                        const float2 pd = __fmul2_rn(z, make_float2(e.x, e.y));
                        const float2 pc = __fmul2_rn(z, make_float2(e.y, -e.x));
                        const float d = angle_between_est(pc.x + pc.y, pd.x + pd.y, K.pi);
                        const float w = fmaf(0.5f, amp1, e.z);
                        const float2 na = __ffma2_rn(make_float2(d, 1.0f), make_float2(w, w), acc);
                        const bool ok = amp1 >= e.w;
                        acc.x = ok ? na.x : acc.x;
                        acc.y = ok ? na.y : acc.y;
                    }
                    kahan_add(pr1, c1, acc.x);
                    kahan_add(pr2, c2, acc.y);
                }
            }
        }
        sred[2 * t] = pr1;
        sred[2 * t + 1] = pr2;
        __syncthreads();
        unsigned long long key = ~0ull;
        if (g == 0 && k < a.nomega) {
            float s1 = 0.f, s2 = 0.f;
            for (int gg = 0; gg < G; ++gg) {
                s1 += sred[2 * (gg * nomp + k)];
                s2 += sred[2 * (gg * nomp + k) + 1];
            }
            const float pr = (s2 > 1.0e-10f) ? s1 / s2 * K.r2d : 999.0f;
            const int base = __float_as_int(a.views[(long)v * 4 + 2]);
            if (a.pr_array) a.pr_array[(long)p * a.per + base + k] = pr;
            key = ((unsigned long long)__float_as_uint(pr) << 32) | (unsigned)(base + k);
        }
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
            key = other < key ? other : key;
        }
        if ((t & 31) == 0) skey[t >> 5] = key;
        __syncthreads();
        if (t < 32) {
            key = (t < nwarps) ? skey[t] : ~0ull;
            for (int o = 16; o > 0; o >>= 1) {
                unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
                key = other < key ? other : key;
            }
            if (t == 0) atomicMin(a.best + p, key);
        }
    }
}

// cal_crosslin_PR.f90:2-71 for the 11 candidates of each particle; the candidate
// origin shift (img2d_FT_centshift.f90) is applied to each bilinear tap, which is the
// same per-pixel arithmetic as shifting the whole transform first.
__global__ void __launch_bounds__(512) k_pr_single(PrSingleArgs a, Consts K) {
    __shared__ double sh[2][32];
    __shared__ float sline[4][60];  // cos, sin of the particle line; cos, sin of the template line
    __shared__ int svalid[60];
    const Band bd = a.bd;
    const int W = bd.W, nr = bd.nr, minR = bd.min_r, nx = bd.nx;
    const int c = blockIdx.x, p = blockIdx.y;
    if (a.ncount && c >= a.ncount[p]) return;  // padding slot (whole block)
    const float* cd = a.cand + ((long)p * a.ncand + c) * 5;
    const float nxh = (float)(nx / 2);
    const float xs = __fadd_rn(cd[3], nxh), ys = __fadd_rn(cd[4], nxh);
    const int offW = bd.off * W + bd.off;
    const float2* pb = a.band + (long)p * W * W;
    const float* ctfp = a.ctf ? a.ctf + (long)p * W * W : nullptr;
    const float* fc0 = a.fcut0 + (long)p * nr;
    const float* tfc = a.tfcut + (long)p * a.tfcut_pstride;
    const float twopi = __fmul_rn(2.0f, K.pi);
    float h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f;  // per-thread sums as TwoSum pairs
    for (int i = 0; i < a.T; ++i) {
        const float2* al = a.alpha + (((long)p * a.ncand + c) * a.T + i) * 60;
        const float2* tb = a.tband + (long)i * W * W;
        const float* fct = tfc + (long)i * nr;
        // the two in-plane directions of each common line, once per line
        __syncthreads();
        if (threadIdx.x < 60) {
            const float2 aa = al[threadIdx.x];
            const bool ok = aa.x < 999.0f && aa.y < 999.0f;
            svalid[threadIdx.x] = ok;
            if (ok) {
                const float a1 = __fmul_rn(aa.x, K.d2r), a2 = __fmul_rn(aa.y, K.d2r);
                sline[0][threadIdx.x] = cosf(a1);
                sline[1][threadIdx.x] = sinf(a1);
                sline[2][threadIdx.x] = cosf(a2);
                sline[3][threadIdx.x] = sinf(a2);
            }
        }
        __syncthreads();
        for (int q = threadIdx.x; q < 60 * nr; q += blockDim.x) {
            int j = q / nr, iq = q - j * nr;
            if (!svalid[j]) continue;
            const float fr = (float)(minR + iq);
            // particle sample with the candidate origin shift on each tap
            float cs = sline[0][j], sn = sline[1][j];
            float x = __fadd_rn(__fmul_rn(fr, cs), nxh), y = __fadd_rn(__fmul_rn(fr, sn), nxh);
            int lx = (int)x, ly = (int)y;
            float ax = __fsub_rn(x, (float)lx), ay = __fsub_rn(y, (float)ly);
            float tr[4], ti[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                int tx = lx + (u & 1), ty = ly + (u >> 1);
                float2 vv = pb[ty * W + tx - offW];
                int hx = tx - nx / 2, ky = ty - nx / 2;
                float ph = __fdiv_rn(__fmul_rn(twopi, __fadd_rn(__fmul_rn(xs, (float)hx), __fmul_rn(ys, (float)ky))),
                                     (float)nx);
                float s, co;
                sincosf(ph, &s, &co);
                tr[u] = __fadd_rn(__fmul_rn(vv.x, co), __fmul_rn(vv.y, s));
                ti[u] = __fadd_rn(__fmul_rn(-vv.x, s), __fmul_rn(vv.y, co));
            }
            float re1 = bilerp(ax, ay, tr[0], tr[1], tr[2], tr[3]);
            float im1 = bilerp(ax, ay, ti[0], ti[1], ti[2], ti[3]);
            float re2, im2;
            tmpl_sample_cs(tb, ctfp, W, offW, nxh, sline[2][j], sline[3][j], fr, &re2, &im2);
            float amp1 = sqrtf(re1 * re1 + im1 * im1);
            float amp2 = sqrtf(re2 * re2 + im2 * im2);
            if (amp1 >= fc0[iq] && amp2 >= fct[iq]) {
                float ph1 = atan2f(im1, re1), ph2 = atan2f(im2, re2);
                float d = fabsf(ph2 - ph1);
                d = fminf(d, K.tpi - d);
                float w = 0.5f * (amp1 + amp2);
                two_sum_acc(h1, l1, d * w);
                two_sum_acc(h2, l2, w);
            }
        }
    }
    double p1 = (double)h1 + (double)l1, p2 = (double)h2 + (double)l2;
    for (int o = 16; o > 0; o >>= 1) {
        p1 += __shfl_xor_sync(0xffffffffu, p1, o);
        p2 += __shfl_xor_sync(0xffffffffu, p2, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) { sh[0][w] = p1; sh[1][w] = p2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s1 = 0, s2 = 0;
        for (int q = 0; q < nw; ++q) { s1 += sh[0][q]; s2 += sh[1][q]; }
        float f1 = (float)s1, f2 = (float)s2;
        a.pr[(long)p * a.ncand + c] = (f2 > 1.0e-10f) ? f1 / f2 * 180.0f / K.pi : 1000.0f;
    }
}

// Grouped rescoring: up to RG candidates of one particle that share a view (theta,
// phi) and differ in omega.  The template side of a term (line direction, taps, cut)
// does not depend on omega, so each (template, line, radius) sample of the templates
// is taken once and compared with the RG particle samples.  groups[g] = (particle,
// first candidate slot, count).  Every candidate sits at the particle's origin (band
// pre-shifted, templates pre-multiplied by the particle's CTF), and the per-term
// arithmetic is the exhaustive scorer's (angle_between, Kahan sums per thread), so its
// values match k_pr_omega's.
constexpr int RG = 4;
__global__ void __launch_bounds__(512) k_pr_rescore_g(PrSingleArgs a, const int4* __restrict__ groups, Consts K) {
    extern __shared__ float rsm[];
    __shared__ double sh[2][RG][16];
    const Band bd = a.bd;
    const int W = bd.W, nr = bd.nr, minR = bd.min_r, nx = bd.nx, T = a.T;
    const int4 gr = groups[blockIdx.x];
    const int p = gr.x, c0 = gr.y, m = gr.z;
    float* spl = rsm;                          // [RG][T][60][2]: cos, sin of the particle lines
    float* stl = spl + (long)RG * T * 120;     // [T][60][2]: cos, sin of the template lines
    float* sfc = stl + (long)T * 120;          // [T + 1][nr]: template cuts, then the particle's
    int* sval = reinterpret_cast<int*>(sfc + (long)(T + 1) * nr);  // [T][60]
    for (int q = threadIdx.x; q < T * 60; q += blockDim.x) {
        const float2 aa = a.alpha[((long)p * a.ncand + c0) * T * 60 + q];
        const bool ok = aa.x < 999.0f && aa.y < 999.0f;
        sval[q] = ok;
        if (ok) {
            const float a2 = __fmul_rn(aa.y, K.d2r);
            stl[2 * q] = cosf(a2);
            stl[2 * q + 1] = sinf(a2);
        }
    }
    for (int q = threadIdx.x; q < m * T * 60; q += blockDim.x) {
        const int g = q / (T * 60), r = q - g * T * 60;
        const float2 aa = a.alpha[((long)p * a.ncand + c0 + g) * T * 60 + r];
        const float a1 = __fmul_rn(aa.x, K.d2r);
        spl[2 * q] = cosf(a1);
        spl[2 * q + 1] = sinf(a1);
    }
    const float* tfc = a.tfcut + (long)p * a.tfcut_pstride;
    for (int q = threadIdx.x; q < T * nr; q += blockDim.x) sfc[q] = tfc[q];
    for (int q = threadIdx.x; q < nr; q += blockDim.x) sfc[T * nr + q] = a.fcut0[(long)p * nr + q];
    __syncthreads();
    const float nxh = (float)(nx / 2);
    const int offW = bd.off * W + bd.off;
    const float4* sb = a.sband + (long)p * W * W;
    const float4* tbc0 = a.tbandc ? a.tbandc + (long)p * T * W * W : nullptr;
    const float* ctfp = a.ctf ? a.ctf + (long)p * W * W : nullptr;
    const int per_t = 60 * nr;
    float f1[RG], f2[RG], k1[RG], k2[RG];
#pragma unroll
    for (int g = 0; g < RG; ++g) { f1[g] = 0.f; f2[g] = 0.f; k1[g] = 0.f; k2[g] = 0.f; }
    // (template i, line j, radius iq) of the flat index q = (i * 60 + j) * nr + iq, advanced
    // by blockDim.x per iteration without integer divisions
    const int step_j = (int)blockDim.x / nr, step_iq = (int)blockDim.x - step_j * nr;
    int i = (int)threadIdx.x / per_t, j = ((int)threadIdx.x - i * per_t) / nr;
    int iq = (int)threadIdx.x - i * per_t - j * nr;
    auto advance = [&]() {
        iq += step_iq;
        j += step_j;
        if (iq >= nr) { iq -= nr; ++j; }
        while (j >= 60) { j -= 60; ++i; }
    };
    for (int q = threadIdx.x; q < T * per_t; q += blockDim.x, advance()) {
        const int lj = i * 60 + j;
        if (!sval[lj]) continue;
        const float fr = (float)(minR + iq);
        float re2, im2;
        if (tbc0)
            tmpl_sample_pairs(tbc0 + (long)i * W * W, W, offW, nxh, stl[2 * lj], stl[2 * lj + 1], fr, &re2, &im2);
        else
            tmpl_sample_cs(a.tband + (long)i * W * W, ctfp, W, offW, nxh, stl[2 * lj], stl[2 * lj + 1], fr, &re2,
                           &im2);
        const float amp2 = sqrtf(re2 * re2 + im2 * im2);
        if (!(amp2 >= sfc[i * nr + iq])) continue;
        const float cut1 = sfc[T * nr + iq];
#pragma unroll
        for (int g = 0; g < RG; ++g) {
            if (g >= m) break;
            const float cs = spl[2 * ((long)g * T * 60 + lj)], sn = spl[2 * ((long)g * T * 60 + lj) + 1];
            const float x = __fadd_rn(__fmul_rn(fr, cs), nxh), y = __fadd_rn(__fmul_rn(fr, sn), nxh);
            const int lx = (int)x, ly = (int)y;
            const float ax = __fsub_rn(x, (float)lx), ay = __fsub_rn(y, (float)ly);
            const int b0 = ly * W + lx - offW;
            const float4 r0 = sb[b0], r1 = sb[b0 + W];  // (tap, right tap) of rows y, y + 1
            const float2 t00 = make_float2(r0.x, r0.y), t10 = make_float2(r0.z, r0.w);
            const float2 t01 = make_float2(r1.x, r1.y), t11 = make_float2(r1.z, r1.w);
            const float re1 = bilerp(ax, ay, t00.x, t10.x, t01.x, t11.x);
            const float im1 = bilerp(ax, ay, t00.y, t10.y, t01.y, t11.y);
            const float amp1 = sqrtf(re1 * re1 + im1 * im1);
            if (amp1 >= cut1) {
                const float d = angle_between(re1 * im2 - im1 * re2, re1 * re2 + im1 * im2, K.pi);
                const float w = 0.5f * (amp1 + amp2);
                kahan_add(f1[g], k1[g], d * w);
                kahan_add(f2[g], k2[g], w);
            }
        }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int g = 0; g < RG; ++g) {
        double p1 = (double)f1[g], p2 = (double)f2[g];
        for (int o = 16; o > 0; o >>= 1) {
            p1 += __shfl_xor_sync(0xffffffffu, p1, o);
            p2 += __shfl_xor_sync(0xffffffffu, p2, o);
        }
        if (l == 0) { sh[0][g][w] = p1; sh[1][g][w] = p2; }
    }
    __syncthreads();
    if (threadIdx.x < m) {
        const int g = threadIdx.x;
        double s1 = 0, s2 = 0;
        for (int q = 0; q < nw; ++q) { s1 += sh[0][g][q]; s2 += sh[1][g][q]; }
        const float g1 = (float)s1, g2 = (float)s2;
        a.pr[(long)p * a.ncand + c0 + g] = (g2 > 1.0e-10f) ? g1 / g2 * 180.0f / K.pi : 1000.0f;
    }
}

// Grouped rescoring with the particle's shifted band in shared memory.  The groups, the
// tables and the template side are k_pr_rescore_g's; the particle side reads its four
// taps from a [W][SP] float2 copy of the band in shared memory (SP = the smallest pitch
// >= W that is 3 mod 16: 8-byte taps of a line of radii fall on distinct bank pairs
// for vertical lines and spread over 4-8 for diagonal ones) instead of 16-byte
// pixel pairs from L1, and its per-term arithmetic is k_pr_omega's in packed FP32x2
// operations, so a term has the value the exhaustive search gives it.  One block of
// RS_THREADS threads per SM (the band is 136 KB at W = 130).
// A two-phase variant (per template: the template samples that pass their cut compacted
// into a shared-memory list by a block-wide scan, then the candidates over the list with
// full warps) was built and measured 1.7x slower (4.72 against 2.79 ms for the four
// launches of the profile case): its four barriers per template leave the template
// samples' L2 latency exposed with one block per SM, where the flat loop overlaps it.
// Measured alternatives of the flat loop on the same 256-particle workload (rescoring
// time, one lane): the candidate loop with a run-time count and branches on the cuts
// 1.12x, a per-warp queue of the samples that pass the template cut (full warps in the
// candidate loop, but a longer shared-memory dependency chain) 1.36x, the template taps
// fetched one iteration ahead 1.12x (no gain: not latency-bound), 768 threads 1.07x, 512
// threads 1.34x, branch-free items or two items per iteration 1.07x.
constexpr int RS_THREADS = 1024;
__host__ __device__ inline int rescore_pitch(int W) { return W + ((3 - W % 16) + 16) % 16; }
__global__ void __launch_bounds__(RS_THREADS, 1) k_pr_rescore_s(PrSingleArgs a, const int4* __restrict__ groups,
                                                                  Consts K) {
    extern __shared__ __align__(16) float rsm[];
    __shared__ double sh[2][RG][RS_THREADS / 32];
    const Band bd = a.bd;
    const int W = bd.W, nr = bd.nr, minR = bd.min_r, nx = bd.nx, T = a.T;
    const int SP = rescore_pitch(W);
    const int4 gr = groups[blockIdx.x];
    const int p = gr.x, c0 = gr.y, m = gr.z;
    float2* sbd = reinterpret_cast<float2*>(rsm);   // [W][SP] shifted particle band
    float* spl = rsm + 2L * W * SP;                 // [RG][T][60][2]: cos, sin of the particle lines
    float* stl = spl + (long)RG * T * 120;          // [T][60][2]: cos, sin of the template lines
    float* sfc = stl + (long)T * 120;               // [T + 1][nr]: template cuts, then the particle's
    int* sval = reinterpret_cast<int*>(sfc + (long)(T + 1) * nr);  // [T][60]
    const float4* sb = a.sband + (long)p * W * W;
    for (int row = threadIdx.x >> 5; row < W; row += RS_THREADS / 32)
        for (int col = threadIdx.x & 31; col < W; col += 32) {
            const float4 v = sb[(long)row * W + col];
            sbd[row * SP + col] = make_float2(v.x, v.y);
        }
    // line directions from the view table, as k_pr_omega computes them: the template's
    // cos/sin of alpha2, the particle's sincos of (alpha1 - omega) for each candidate
    const int* co = a.corient + (long)p * a.ncand + c0;
    const float2* va = a.valpha + (long)(co[0] / a.nom) * T * 60;
    for (int q = threadIdx.x; q < T * 60; q += RS_THREADS) {
        const float2 aa = va[q];
        const bool ok = aa.x < 999.0f && aa.y < 999.0f;
        sval[q] = ok;
        if (ok) {
            const float a2 = __fmul_rn(aa.y, K.d2r);
            stl[2 * q] = cosf(a2);
            stl[2 * q + 1] = sinf(a2);
        }
    }
    for (int q = threadIdx.x; q < m * T * 60; q += RS_THREADS) {
        const int g = q / (T * 60), r = q - g * T * 60;
        const float2 aa = va[r];
        const float womega = __fmul_rn(a.step, (float)(co[g] % a.nom));
        const float ang = __fmul_rn(__fsub_rn(aa.x, womega), K.d2r);
        float sn, cs;
        sincosf(ang, &sn, &cs);
        spl[2 * q] = cs;
        spl[2 * q + 1] = sn;
    }
    const float* tfc = a.tfcut + (long)p * a.tfcut_pstride;
    for (int q = threadIdx.x; q < T * nr; q += RS_THREADS) sfc[q] = tfc[q];
    for (int q = threadIdx.x; q < nr; q += RS_THREADS) sfc[T * nr + q] = a.fcut0[(long)p * nr + q];
    __syncthreads();
    const float nxh = (float)(nx / 2);
    const int offW = bd.off * W + bd.off, offS = bd.off * SP + bd.off;
    const float4* tbc0 = a.tbandc ? a.tbandc + (long)p * T * W * W : nullptr;
    const float* ctfp = a.ctf ? a.ctf + (long)p * W * W : nullptr;
    const int per_t = 60 * nr;
    const int step_j = RS_THREADS / nr, step_iq = RS_THREADS - step_j * nr;
    int i = (int)threadIdx.x / per_t, j = ((int)threadIdx.x - i * per_t) / nr;
    int iq = (int)threadIdx.x - i * per_t - j * nr;
    auto advance = [&]() {
        iq += step_iq;
        j += step_j;
        if (iq >= nr) { iq -= nr; ++j; }
        while (j >= 60) { j -= 60; ++i; }
    };
    const float2 nxh2 = make_float2(nxh, nxh);
    const int wi = threadIdx.x >> 5, l = threadIdx.x & 31;
    // The group's candidate count M is a compile-time constant of each instance of the
    // loop, so the M candidates' terms of one template sample are independent chains that
    // the compiler interleaves; the two amplitude cuts are selects, not branches (with
    // ~70 % of the samples passing each cut, a warp runs both sides of such a branch
    // anyway).  A term that fails a cut leaves the sums unchanged.
    auto run = [&](auto mc) {
        constexpr int M = decltype(mc)::value;
        // (PR numerator, weight) sums: per thread a plain FP32 pair over its ~40 terms of a
        // candidate (like k_pr_omega's per-line partials), then FP64 across the block
        float2 fs[M];
#pragma unroll
        for (int g = 0; g < M; ++g) fs[g] = make_float2(0.f, 0.f);
        for (int q = threadIdx.x; q < T * per_t; q += RS_THREADS, advance()) {
            const int lj = i * 60 + j;
            if (!sval[lj]) continue;
            const float fr = (float)(minR + iq);
            float re2, im2;
            if (tbc0)
                tmpl_sample_pairs(tbc0 + (long)i * W * W, W, offW, nxh, stl[2 * lj], stl[2 * lj + 1], fr, &re2,
                                  &im2);
            else
                tmpl_sample_cs(a.tband + (long)i * W * W, ctfp, W, offW, nxh, stl[2 * lj], stl[2 * lj + 1], fr,
                               &re2, &im2);
            const float amp2 = sqrtf(re2 * re2 + im2 * im2);
            const bool ok2 = amp2 >= sfc[i * nr + iq];
            const float cut1 = sfc[T * nr + iq];
            const float2 fr2 = make_float2(fr, fr), e2 = make_float2(re2, im2), e2c = make_float2(im2, -re2);
            const float half2 = 0.5f * amp2;
            const float2 m1 = make_float2(-1.f, -1.f);
#pragma unroll
            for (int g = 0; g < M; ++g) {
                // k_pr_omega's per-term arithmetic: position by FMA, bilinear as lerps on
                // (re, im) pairs, amplitude sq * rsqrt(sq), weight 0.5 amp1 + 0.5 amp2
                const float2 cs = *reinterpret_cast<const float2*>(&spl[2 * ((long)g * T * 60 + lj)]);
                const float2 xy = __ffma2_rn(fr2, cs, nxh2);
                const int lx = (int)xy.x, ly = (int)xy.y;
                const float2 f = __fadd2_rn(xy, make_float2(-(float)lx, -(float)ly));
                const float2* tp = sbd + (ly * SP + lx - offS);
                const float2 t00 = tp[0], t10 = tp[1], t01 = tp[SP], t11 = tp[SP + 1];
                const float2 ax2 = make_float2(f.x, f.x), ay2 = make_float2(f.y, f.y);
                const float2 v0 = __ffma2_rn(ax2, __ffma2_rn(t00, m1, t10), t00);
                const float2 v1 = __ffma2_rn(ax2, __ffma2_rn(t01, m1, t11), t01);
                const float2 z = __ffma2_rn(ay2, __ffma2_rn(v0, m1, v1), v0);
                const float2 zz = __fmul2_rn(z, z);
                const float sq = zz.x + zz.y;
                const float amp1 = sq * rsqrtf(sq);  // NaN for 0: fails the cut
                const float2 pd = __fmul2_rn(z, e2);
                const float2 pc = __fmul2_rn(z, e2c);
                const float d = angle_between_est(pc.x + pc.y, pd.x + pd.y, K.pi);
                const float w = fmaf(0.5f, amp1, half2);
                const float2 nf = __ffma2_rn(make_float2(d, 1.0f), make_float2(w, w), fs[g]);
                const bool ok = ok2 && amp1 >= cut1;
                fs[g].x = ok ? nf.x : fs[g].x;
                fs[g].y = ok ? nf.y : fs[g].y;
            }
        }
#pragma unroll
        for (int g = 0; g < M; ++g) {
            double p1 = (double)fs[g].x, p2 = (double)fs[g].y;
            for (int o = 16; o > 0; o >>= 1) {
                p1 += __shfl_xor_sync(0xffffffffu, p1, o);
                p2 += __shfl_xor_sync(0xffffffffu, p2, o);
            }
            if (l == 0) { sh[0][g][wi] = p1; sh[1][g][wi] = p2; }
        }
    };
    switch (m) {
        case 1: run(std::integral_constant<int, 1>()); break;
        case 2: run(std::integral_constant<int, 2>()); break;
        case 3: run(std::integral_constant<int, 3>()); break;
        default: run(std::integral_constant<int, RG>()); break;
    }
    __syncthreads();
    if (threadIdx.x < m) {
        const int g = threadIdx.x;
        double s1 = 0, s2 = 0;
        for (int q = 0; q < RS_THREADS / 32; ++q) { s1 += sh[0][g][q]; s2 += sh[1][g][q]; }
        const float g1 = (float)s1, g2 = (float)s2;
        a.pr[(long)p * a.ncand + c0 + g] = (g2 > 1.0e-10f) ? g1 / g2 * 180.0f / K.pi : 1000.0f;
    }
}

// The particle transform shifted to the origin its candidates share (cand[p][0][3..4]):
// per pixel the same phase rotation k_pr_single applies to each bilinear tap
// (img2d_FT_centshift.f90), computed once per pixel instead of once per tap.
// Stored as pairs: out[p][m] = (pixel m, its right neighbour m + 1; zero past the row's
// end), so a bilinear sample reads two aligned 16-byte pairs instead of four taps.
__device__ __forceinline__ float2 shifted_pixel(const float2* band, int m, int W, int off, int nx, float xs,
                                                float ys, float twopi) {
    const int by = m / W, bx = m - by * W;
    const int hx = bx + off - nx / 2, ky = by + off - nx / 2;
    const float2 vv = band[m];
    float ph = __fdiv_rn(__fmul_rn(twopi, __fadd_rn(__fmul_rn(xs, (float)hx), __fmul_rn(ys, (float)ky))),
                         (float)nx);
    float s, co;
    sincosf(ph, &s, &co);
    return make_float2(__fadd_rn(__fmul_rn(vv.x, co), __fmul_rn(vv.y, s)),
                       __fadd_rn(__fmul_rn(-vv.x, s), __fmul_rn(vv.y, co)));
}
__global__ void k_shift_band(const float2* __restrict__ band, const float* __restrict__ cand, int ncand, Band bd,
                             Consts K, float4* __restrict__ out) {
    const int W = bd.W, nx = bd.nx, p = blockIdx.y;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= W * W) return;
    const float* cd = cand + (long)p * ncand * 5;
    const float nxh = (float)(nx / 2);
    const float xs = __fadd_rn(cd[3], nxh), ys = __fadd_rn(cd[4], nxh);
    const float twopi = __fmul_rn(2.0f, K.pi);
    const float2* b = band + (long)p * W * W;
    const float2 v0 = shifted_pixel(b, m, W, bd.off, nx, xs, ys, twopi);
    const float2 v1 = (m % W) + 1 < W ? shifted_pixel(b, m + 1, W, bd.off, nx, xs, ys, twopi) : make_float2(0.f, 0.f);
    out[(long)p * W * W + m] = make_float4(v0.x, v0.y, v1.x, v1.y);
}

// reconstruct.f90:103-145: rotate each half-plane sample, apply the 60 operators,
// fold to z >= 0 and splat (a*ctf, b*ctf*signz, ctf^2) trilinearly.  One thread per
// (operator, sample), consecutive threads on consecutive samples of one operator: the
// samples run along hx, so a warp's splats land on neighbouring voxels and its float4
// vector reductions share L2 sectors (the three sums of a voxel are one reduction).
__device__ __forceinline__ void mv3_rn(const float* m, const float* v, float* o) {
    float t0 = __fmul_rn(m[0], v[0]); t0 = __fadd_rn(t0, __fmul_rn(m[1], v[1])); t0 = __fadd_rn(t0, __fmul_rn(m[2], v[2]));
    float t1 = __fmul_rn(m[3], v[0]); t1 = __fadd_rn(t1, __fmul_rn(m[4], v[1])); t1 = __fadd_rn(t1, __fmul_rn(m[5], v[2]));
    float t2 = __fmul_rn(m[6], v[0]); t2 = __fadd_rn(t2, __fmul_rn(m[7], v[1])); t2 = __fadd_rn(t2, __fmul_rn(m[8], v[2]));
    o[0] = t0; o[1] = t1; o[2] = t2;
}

__global__ void __launch_bounds__(256) k_insert(InsertArgs a) {
    const int p = blockIdx.y;
    if (!a.sel[p]) return;
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long)a.nsamples * a.nsym) return;
    const int k = (int)(q / a.nsamples), s = (int)(q - (long)k * a.nsamples);
    const Band bd = a.bd;
    const int W = bd.W, R = bd.max_r;
    const int2 hk = a.samples[s];
    const float* rot = a.rot + p * 9;
    float xv[3] = {(float)hk.x, (float)hk.y, 0.0f}, x00[3], x0[3];
    mv3_rn(rot, xv, x00);
    mv3_rn(a.ops + k * 9, x00, x0);
    float signz = 1.0f;
    if (x0[2] < 0.0f) { x0[0] = -x0[0]; x0[1] = -x0[1]; x0[2] = -x0[2]; signz = -1.0f; }
    x0[0] = __fadd_rn(x0[0], a.off_xy);
    x0[1] = __fadd_rn(x0[1], a.off_xy);
    x0[2] = __fadd_rn(x0[2], a.off_z);
    const int lx = (int)x0[0], ly = (int)x0[1], lz = (int)x0[2];
    const float ax = x0[0] - (float)lx, ay = x0[1] - (float)ly, az = x0[2] - (float)lz;
    const float bx = 1.0f - ax, by = 1.0f - ay, bz = 1.0f - az;
    float dx[8];
    dx[0] = __fmul_rn(__fmul_rn(bx, by), bz);
    dx[1] = __fmul_rn(__fmul_rn(ax, by), bz);
    dx[2] = __fmul_rn(__fmul_rn(bx, ay), bz);
    dx[3] = __fmul_rn(__fmul_rn(ax, ay), bz);
    dx[4] = __fmul_rn(__fmul_rn(bx, by), az);
    dx[5] = __fmul_rn(__fmul_rn(ax, by), az);
    dx[6] = __fmul_rn(__fmul_rn(bx, ay), az);
    dx[7] = __fmul_rn(__fmul_rn(ax, ay), az);
    const int bidx = (hk.y + R) * W + (hk.x + R);
    const float2 fv = a.band[(long)p * W * W + bidx];
    const float c = a.ctf ? a.ctf[(long)p * W * W + bidx] : 1.0f;
    const float c2 = __fmul_rn(c, c);
    const int AW = bd.AW;
    const int ix = lx - a.base_xy, iy = ly - a.base_xy, iz = lz - a.base_z;
    if (ix < 0 || iy < 0 || iz < 0 || ix > AW - 2 || iy > AW - 2 || iz > R) return;  // never taken
    const long base = ((long)iz * AW + iy) * AW + ix;
    const long offs[8] = {0, 1, AW, AW + 1, (long)AW * AW, (long)AW * AW + 1, (long)AW * AW + AW,
                          (long)AW * AW + AW + 1};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        float va = __fmul_rn(__fmul_rn(fv.x, dx[j]), c);
        float vb = __fmul_rn(__fmul_rn(__fmul_rn(fv.y, dx[j]), c), signz);
        float vw = __fmul_rn(dx[j], c2);
        atomicAdd(a.acc + base + offs[j], make_float4(va, vb, vw, 0.0f));
    }
}

Consts consts() {
    Angles an = host_angles();
    Consts K;
    K.d2r = an.deg2rad;
    K.pi = an.pi;
    K.tpi = an.tpi;
    K.r2d = 180.0f / an.pi;
    return K;
}

}  // namespace

int pr_omega_smem_bytes(const Band& bd, int nomega, int* threads) {
    int nomp = (nomega + 31) / 32 * 32;
    if (nomp > 768) return -1;
    int G = 768 / nomp;
    if (G < 1) G = 1;
    int nt = G * nomp;
    if (threads) *threads = nt;
    size_t b = (size_t)bd.W * bd.W * 8 + (size_t)60 * bd.nr * 16 + (size_t)((bd.nr + 3) & ~3) * 4 +
               64 * 4 + (size_t)2 * nt * 4 + 32 * 8;
    return (int)b;
}

cudaError_t launch_pr_omega(const PrOmegaArgs& a, int B, cudaStream_t st) {
    int nt = 0;
    int sm = pr_omega_smem_bytes(a.bd, a.nomega, &nt);
    if (sm < 0) return cudaErrorInvalidValue;
    int nomp = (a.nomega + 31) / 32 * 32;
    cudaError_t e = cudaFuncSetAttribute(k_pr_omega, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    dim3 grid(a.V, B);
    k_pr_omega<<<grid, nt, sm, st>>>(a, nomp, consts());
    return cudaGetLastError();
}

cudaError_t launch_shift_band(const float2* band, const float* cand, int ncand, const Band& bd, int B,
                              float4* out, cudaStream_t st) {
    const int n = bd.W * bd.W;
    dim3 grid((n + 255) / 256, B);
    k_shift_band<<<grid, 256, 0, st>>>(band, cand, ncand, bd, consts(), out);
    return cudaGetLastError();
}

// out[p][i] = tband[i] x ctf[p] per band pixel (the products tmpl_sample forms per tap)
__global__ void k_tband_ctf(const float2* __restrict__ tband, int T, const float* __restrict__ ctf, long w2, int W,
                            float4* __restrict__ out) {
    const int p = blockIdx.y;
    const long n = (long)T * w2;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const long m = q % w2;
        const float2 t = tband[q];
        const float c = ctf[(long)p * w2 + m];
        float2 u = make_float2(0.f, 0.f);
        if ((m % W) + 1 < W) {  // the right neighbour in the same row
            const float2 t1 = tband[q + 1];
            const float c1 = ctf[(long)p * w2 + m + 1];
            u = make_float2(__fmul_rn(t1.x, c1), __fmul_rn(t1.y, c1));
        }
        out[(long)p * n + q] = make_float4(__fmul_rn(t.x, c), __fmul_rn(t.y, c), u.x, u.y);
    }
}

cudaError_t launch_tband_ctf(const float2* tband, int T, const float* ctf, const Band& bd, int B, float4* out,
                             cudaStream_t st) {
    const long w2 = (long)bd.W * bd.W;
    dim3 grid((int)std::min<long>((T * w2 + 255) / 256, 4096), B);
    k_tband_ctf<<<grid, 256, 0, st>>>(tband, T, ctf, w2, bd.W, out);
    return cudaGetLastError();
}

cudaError_t launch_pr_single(const PrSingleArgs& a, int B, cudaStream_t st) {
    dim3 grid(a.ncand, B);
    k_pr_single<<<grid, 512, 0, st>>>(a, consts());
    return cudaGetLastError();
}

cudaError_t launch_pr_rescore_groups(const PrSingleArgs& a, const int4* groups, int ngroups, cudaStream_t st) {
    if (!a.sband || ngroups < 1) return cudaErrorInvalidValue;
    const size_t sm = sizeof(float) * ((size_t)RG * a.T * 120 + (size_t)a.T * 120 + (size_t)(a.T + 1) * a.bd.nr) +
                      sizeof(int) * a.T * 60;
    // the band in shared memory where it fits beside the tables (W <= ~140 at T = 20)
    const size_t sm_s = sm + sizeof(float2) * (size_t)a.bd.W * rescore_pitch(a.bd.W);
    if (pr_rescore_shared_band(a.bd, a.T)) {
        if (!a.valpha || !a.corient || a.nom < 1) return cudaErrorInvalidValue;
        cudaError_t e = cudaFuncSetAttribute(k_pr_rescore_s, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_s);
        if (e != cudaSuccess) return e;
        k_pr_rescore_s<<<ngroups, RS_THREADS, sm_s, st>>>(a, groups, consts());
        return cudaGetLastError();
    }
    if (sm > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_pr_rescore_g, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_pr_rescore_g<<<ngroups, 512, sm, st>>>(a, groups, consts());
    return cudaGetLastError();
}

int pr_rescore_group_size() { return RG; }

bool pr_rescore_shared_band(const Band& bd, int T) {
    const size_t sm = sizeof(float) * ((size_t)RG * T * 120 + (size_t)T * 120 + (size_t)(T + 1) * bd.nr) +
                      sizeof(int) * T * 60;
    const size_t sm_s = sm + sizeof(float2) * (size_t)bd.W * rescore_pitch(bd.W);
    return sm_s + sizeof(double) * 2 * RG * (RS_THREADS / 32) <= 227 * 1024;
}

cudaError_t launch_insert(const InsertArgs& a, int B, cudaStream_t st) {
    long total = (long)a.nsamples * a.nsym;
    dim3 grid((unsigned)((total + 255) / 256), B);
    k_insert<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace cryoim
