// local.cu — local_refine's refinement of sub-particles against a local map
// (local_refine/SRC/refine_PR.f90), compiled with -fmad=false so the FP32 arithmetic
// rounds where the Fortran reference rounds.
//
//   * k_softmask3d_*: img3d_softmask.f90 (cosine edge at imgmask, the edge-shell mean
//     outside);
//   * k_local_ft: the map's transform as refine_PR.f90:48-52 builds it (checkerboard,
//     forward FFT / n^3, checkerboard; real and imaginary parts, standard sign);
//   * k_local_box: img2d_norm of the whole image (stack files only) and the
//     img2d_local_box.f90 window around (local_hx0, local_ky0), wrapping at the edges;
//   * k_local_ctf: getCTF2d.f90 of local_refine (defocus already in Angstrom);
//   * k_wlp: the Gaussian weight exp(-r^2 / (2 maxRes^2)) of refine_PR.f90:42-46;
//   * k_local_pr: one CTA per (sub-particle, candidate): the candidate's central section
//     of the map transform (FFT3d_slice.f90), its origin phase (img2d_FTphase.f90),
//     checkerboard x CTF x weight, and the phase residual against the sub-particle's
//     weighted transform (cal_PR_FT.f90), FP32 terms in FP64 block sums.
#include <cuda_runtime.h>

#include "geom.cuh"
#include "kernels.h"

namespace cryoim {
namespace {

inline int cdiv(long a, int b) { return (int)((a + b - 1) / b); }

// h + l += x with Knuth's TwoSum: the pair holds the running sum to ~2^-48 relative
__device__ __forceinline__ void two_sum_acc(float& h, float& l, float x) {
    const float s2 = h + x, bb = s2 - h;
    l += (h - (s2 - bb)) + (x - bb);
    h = s2;
}

__device__ double bsum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
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

__device__ __forceinline__ float cube_radius(long q, int nx) {
    const int iz = (int)(q / ((long)nx * nx)) - nx / 2, iy = (int)((q / nx) % nx) - nx / 2,
              ix = (int)(q % nx) - nx / 2;
    return sqrtf((float)(ix * ix + iy * iy + iz * iz));
}

// img3d_softmask.f90:18-31: sum and count of the edge shell
__global__ void k_softmask3d_ring(const float* __restrict__ d, int nx, float inn, float out, double* __restrict__ acc) {
    __shared__ double sh[32];
    const long n3 = (long)nx * nx * nx;
    double s = 0, k = 0;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long)gridDim.x * blockDim.x) {
        const float r = cube_radius(q, nx);
        if (r > inn && r <= out) { s += (double)d[q]; k += 1.0; }
    }
    s = bsum(s, sh);
    k = bsum(k, sh);
    if (threadIdx.x == 0) { atomicAdd(acc, s); atomicAdd(acc + 1, k); }
}

// img3d_softmask.f90:35-46 (summ is a real there)
__global__ void k_softmask3d_apply(float* __restrict__ d, int nx, float inn, float out, float pi,
                                   const double* __restrict__ acc) {
    const long n3 = (long)nx * nx * nx;
    float summ = (float)acc[0];
    if (acc[1] != 0.0) summ = summ / (float)acc[1];
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long)gridDim.x * blockDim.x) {
        const float r = cube_radius(q, nx);
        if (r > inn && r <= out) {
            const float edge = (1.0f + cosf(pi * (r - inn) / 6.0f)) / 2.0f;
            d[q] = d[q] * edge + (1.0f - edge) * summ;
        }
        if (r > out) d[q] = summ;
    }
}

// refine_PR.f90:48-52 with img3d_FFT.f90: (Re, Im) / n^3 times (-1)^(x+y+z)
__global__ void k_local_ft(const float2* __restrict__ ft, int nx, float* __restrict__ fr, float* __restrict__ fi) {
    const long n3 = (long)nx * nx * nx;
    const float s = (float)nx * (float)nx * (float)nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(q / ((long)nx * nx)), iy = (int)((q / nx) % nx), ix = (int)(q % nx);
        float re = ft[q].x / s, im = ft[q].y / s;
        if ((ix + iy + iz) & 1) { re = -re; im = -im; }
        fr[q] = re;
        fi[q] = im;
    }
}

// One CTA per sub-particle: img2d_norm of the whole image when normalize (refine_PR.f90:
// 86-87), then the nx x nx window centred on (hx0, ky0) (img2d_local_box.f90:6-17).
__global__ void k_local_box(const float* __restrict__ imgs, int nx0, const int* __restrict__ hk, int nx,
                            int normalize, float* __restrict__ out) {
    __shared__ double sh[32];
    const long nn0 = (long)nx0 * nx0, nn = (long)nx * nx;
    const float* a = imgs + (long)blockIdx.x * nn0;
    float avg = 0.f, nd = 1.f;
    if (normalize) {
        // per thread an FP32 TwoSum pair (exact to ~2^-48), FP64 across the block: GB300's
        // FP64 pipe is far slower than its FP32 pipe
        float h = 0.f, l = 0.f;
        for (long i = threadIdx.x; i < nn0; i += blockDim.x) two_sum_acc(h, l, a[i]);
        const double s = bsum((double)h + (double)l, sh);
        avg = (float)s / (float)nn0;
        h = 0.f;
        l = 0.f;
        for (long i = threadIdx.x; i < nn0; i += blockDim.x) {
            const float d = a[i] - avg;
            two_sum_acc(h, l, d * d);
        }
        const double s2 = bsum((double)h + (double)l, sh);
        nd = sqrtf((float)s2 / (float)nn0);
    }
    const int ix = hk[2 * blockIdx.x], iy = hk[2 * blockIdx.x + 1];
    float* o = out + (long)blockIdx.x * nn;
    for (long i = threadIdx.x; i < nn; i += blockDim.x) {
        int hx = (int)(i % nx) + ix - nx / 2, ky = (int)(i / nx) + iy - nx / 2;
        if (hx < 0) hx += nx0;
        if (hx >= nx0) hx -= nx0;
        if (ky < 0) ky += nx0;
        if (ky >= nx0) ky -= nx0;
        const long i2 = (long)ky * nx0 + hx;
        float v = 0.0f;  // the reference leaves a window pixel unset when still outside
        if (i2 >= 0 && i2 < nn0) {
            v = a[i2];
            if (normalize) v = (v - avg) / nd;
        }
        o[i] = v;
    }
}

// getCTF2d.f90 of local_refine (defocus in Angstrom), one CTA row per sub-particle
__global__ void k_local_ctf(const float* __restrict__ dfs, int nx, float apix, float vol, float cs0, float ampwg,
                            float pi, float* __restrict__ ctf) {
    const int p = blockIdx.y;
    const long nn = (long)nx * nx;
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nn) return;
    const float d2r = pi / 180.0f;
    const float lam = 0.387818f / sqrtf(1.0f * vol * (1.0f + 0.978459E-3f * vol));
    const float cs = cs0 * 1.0e7f, df1 = dfs[3 * p], df2 = dfs[3 * p + 1], astig = dfs[3 * p + 2] * d2r;
    const int ky = (int)(q / nx) - nx / 2, hx = (int)(q % nx) - nx / 2;
    float phi = atan2f((float)ky, (float)hx);
    if (phi < 0.0f) phi = phi + 2.0f * pi;
    phi = phi - astig;
    const float c = cosf(phi), s = sinf(phi);
    const float df = df1 * (c * c) + df2 * (s * s);
    const float res = sqrtf((float)(hx * hx + ky * ky)) / (float)nx / apix;
    const float r2 = res * res, r4 = r2 * r2, lam3 = lam * lam * lam;
    const float phase = 2.0f * pi * (-(cs * lam3 * r4 / 4.0f) + df * lam * r2 / 2.0f);
    const float sq = sqrtf(1.0f - ampwg * ampwg);
    ctf[(long)p * nn + q] = -(sq * sinf(phase) + ampwg * cosf(phase));
}

__device__ __forceinline__ float wlp_of(int i, int nx, float max_r) {
    const int ky = i / nx, hx = i % nx;
    const float r2 = (float)((hx - nx / 2) * (hx - nx / 2) + (ky - nx / 2) * (ky - nx / 2)) / 2.0f / (max_r * max_r);
    return expf(-r2);
}

// refine_PR.f90:119-120: the sub-particle transform times the weight
__global__ void k_wlp(float2* __restrict__ b, int nx, long n, float max_r) {
    const long nn = (long)nx * nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const float w = wlp_of((int)(q % nn), nx, max_r);
        const float2 v = b[q];
        b[q] = make_float2(v.x * w, v.y * w);
    }
}

// FFT3d_slice.f90:19-78 at pixel (ix, iy) of the section, one component
__device__ __forceinline__ void slice_at(const float* __restrict__ fr, const float* __restrict__ fi, int nx,
                                         const float* rot, int ix, int iy, float* sa, float* sb) {
    *sa = 0.0f;
    *sb = 0.0f;
    float xx[3];
    for (int i = 0; i < 3; ++i) {
        float t = rot[3 * i] * (float)ix;
        t = t + rot[3 * i + 1] * (float)iy;
        t = t + rot[3 * i + 2] * 0.0f;
        xx[i] = t;
    }
    if (sqrtf(xx[0] * xx[0] + xx[1] * xx[1] + xx[2] * xx[2]) > (float)(nx / 2 - 2)) return;
    const float h = (float)(nx / 2);
    xx[0] = xx[0] + h; xx[1] = xx[1] + h; xx[2] = xx[2] + h;
    const int hx = (int)xx[0], ky = (int)xx[1], lz = (int)xx[2];
    const float xb = xx[0] - (float)hx, yb = xx[1] - (float)ky, zb = xx[2] - (float)lz;
    const long nn = (long)nx * nx;
    const long b0 = (long)lz * nn + (long)ky * nx + hx;
    const long o[8] = {b0, b0 + 1, b0 + nx, b0 + nx + 1, b0 + nn, b0 + nn + 1, b0 + nn + nx, b0 + nn + nx + 1};
    const float w[8] = {(1.f - xb) * (1.f - yb) * (1.f - zb), xb * (1.f - yb) * (1.f - zb),
                        (1.f - xb) * yb * (1.f - zb),        xb * yb * (1.f - zb),
                        (1.f - xb) * (1.f - yb) * zb,        xb * (1.f - yb) * zb,
                        (1.f - xb) * yb * zb,                xb * yb * zb};
    float a = w[0] * __ldg(fr + o[0]), b = w[0] * __ldg(fi + o[0]);
#pragma unroll
    for (int j = 1; j < 8; ++j) {
        a = a + w[j] * __ldg(fr + o[j]);
        b = b + w[j] * __ldg(fi + o[j]);
    }
    *sa = a;
    *sb = b;
}

// cand: (P x C) x 5 (theta, phi, omega, x, y); part: P x nx^2 weighted transforms;
// ctf: P x nx^2 or null; out: P x C phase residuals
__global__ void __launch_bounds__(256) k_local_pr(const float* __restrict__ cand, int C,
                                                  const float* __restrict__ fr, const float* __restrict__ fi, int nx,
                                                  const float2* __restrict__ part, const float* __restrict__ ctf,
                                                  float max_r, float d2r, float pi, float* __restrict__ out) {
    __shared__ float rot[9];
    __shared__ double sh[32];
    const int c = blockIdx.x, p = blockIdx.y;
    const float* cd = cand + ((long)p * C + c) * 5;
    if (threadIdx.x == 0) euler_mat(cd[0], cd[1], cd[2], d2r, rot);
    __syncthreads();
    const float x0 = cd[3], y0 = cd[4];
    const long nn = (long)nx * nx;
    const float2* pt = part + (long)p * nn;
    const float* ct = ctf ? ctf + (long)p * nn : nullptr;
    const float tpi = 2.0f * pi;
    float pr1 = 0.0f, pr2 = 0.0f;
    for (int i = threadIdx.x; i < (int)nn; i += blockDim.x) {
        const int ky = i / nx - nx / 2, hx = i % nx - nx / 2;
        const float dr = sqrtf((float)(hx * hx + ky * ky));
        if (!(dr >= -1.0f && dr <= max_r)) continue;
        float sa, sb;
        slice_at(fr, fi, nx, rot, hx, ky, &sa, &sb);
        // img2d_FTphase.f90:11-17
        const float ph = 2.0f * pi * (x0 * (float)hx + y0 * (float)ky) / (float)nx;
        const float cs = cosf(ph), sn = sinf(ph);
        float a1 = sa * cs + sb * sn, b1 = -sa * sn + sb * cs;
        // refine_PR.f90:135-136 (or 196-197): shift2d x CTF2d x w_lp
        const float s = ((i / nx + i % nx) & 1) ? -1.0f : 1.0f;
        const float cv = ct ? ct[i] : 1.0f, w = wlp_of(i, nx, max_r);
        a1 = a1 * s * cv * w;
        b1 = b1 * s * cv * w;
        const float2 q = pt[i];
        // cal_PR_FT.f90:16-27
        float amp1 = sqrtf(a1 * a1 + b1 * b1);
        const float amp2 = sqrtf(q.x * q.x + q.y * q.y);
        const float p1 = atan2f(b1, a1), p2 = atan2f(q.y, q.x);
        float diff = fabsf(p2 - p1);
        diff = fmodf(diff, tpi);
        if (diff > pi) diff = tpi - diff;
        amp1 = amp1 + amp2;
        pr1 = diff * amp1 + pr1;
        pr2 = amp1 + pr2;
    }
    const double s1 = bsum((double)pr1, sh), s2 = bsum((double)pr2, sh);
    if (threadIdx.x == 0) out[(long)p * C + c] = s2 > 1.0e-10 ? (float)(s1 / s2) * 180.0f / pi : 1000.0f;
}

// ---- local_box's sub-image stack mode (loc_box.f90:34-91) ----------------------
// The whole image with the checkerboard of img2d_centshift.f90, as a complex row.
__global__ void k_lb_checker(const float* __restrict__ imgs, int nx0, const int* __restrict__ src,
                             float2* __restrict__ work) {
    const long nn0 = (long)nx0 * nx0;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn0) return;
    const int ky = (int)(t / nx0), hx = (int)(t - (long)ky * nx0);
    const float v = imgs[(long)src[blockIdx.y] * nn0 + t];
    work[(long)blockIdx.y * nn0 + t] = make_float2(((hx + ky) & 1) ? -v : v, 0.0f);
}
// img2d_centshift.f90:21-32 on the forward transform: the 1/N^2 of the forward FFT
// (FFTW.f90:185), then F exp(-i phase), phase = 2 pi (x hx + y ky) / N at the shift
// (x, y) = (-particle x, -particle y).
__global__ void k_lb_phase(float2* __restrict__ work, int nx0, const float* __restrict__ xy, float pi) {
    const long nn0 = (long)nx0 * nx0;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn0) return;
    const int ky = (int)(t / nx0) - nx0 / 2, hx = (int)(t - (long)(t / nx0) * nx0) - nx0 / 2;
    const float x = xy[2 * blockIdx.y], y = xy[2 * blockIdx.y + 1];
    const float2 f = work[(long)blockIdx.y * nn0 + t];
    const float a = f.x / (float)nn0, b = f.y / (float)nn0;
    const float phase = 2.0f * pi * (x * (float)hx + y * (float)ky) / (float)nx0;
    const float c = cosf(phase), sn = sinf(phase);
    work[(long)blockIdx.y * nn0 + t] = make_float2(a * c + b * sn, -a * sn + b * c);
}
// loc_box.f90:60-79: one CTA per sub-image, the sub x sub box from pixel (hx0, ky0) of
// the centred image (the real part of the inverse transform times the checkerboard),
// wrapped at the edges, then img2d_norm.f90 of the box with FP32 TwoSum sums combined
// in FP64.  img2d_norm of the whole image before the cut (loc_box.f90:47) is an affine
// map with positive scale, which the box's own normalisation removes, so it is not
// applied.  hk[k] = (hx0, ky0, image slot).
__global__ void k_lb_cut(const float2* __restrict__ work, int nx0, const int* __restrict__ hk, int sub,
                         float* __restrict__ out) {
    __shared__ double sh[32];
    const long nn0 = (long)nx0 * nx0, ns = (long)sub * sub;
    const int hx0 = hk[3 * blockIdx.x], ky0 = hk[3 * blockIdx.x + 1], slot = hk[3 * blockIdx.x + 2];
    const float2* w = work + (long)slot * nn0;
    auto pix = [&](long t) {
        const int ty = (int)(t / sub);
        int hx = (int)(t - (long)ty * sub) + hx0, ky = ty + ky0;
        hx %= nx0;
        if (hx < 0) hx += nx0;
        ky %= nx0;
        if (ky < 0) ky += nx0;
        const float v = w[(long)ky * nx0 + hx].x;
        return ((hx + ky) & 1) ? -v : v;
    };
    float h = 0.f, l = 0.f;
    for (long t = threadIdx.x; t < ns; t += blockDim.x) two_sum_acc(h, l, pix(t));
    const float avg = (float)(bsum((double)h + (double)l, sh) / (double)ns);
    h = 0.f;
    l = 0.f;
    for (long t = threadIdx.x; t < ns; t += blockDim.x) {
        const float d = pix(t) - avg;
        two_sum_acc(h, l, d * d);
    }
    const float nd = (float)sqrt(bsum((double)h + (double)l, sh) / (double)ns);
    float* o = out + (long)blockIdx.x * ns;
    for (long t = threadIdx.x; t < ns; t += blockDim.x) o[t] = (pix(t) - avg) / nd;
}

}  // namespace

cudaError_t launch_local_softmask(float* map, int nx, float mask, double* acc2, cudaStream_t st) {
    float inn = mask - 3.0f;
    if (inn <= 0.0f) inn = 0.0f;
    float out = mask + 3.0f;
    if (out > (float)(nx / 2)) out = (float)(nx / 2);
    cudaError_t e = cudaMemsetAsync(acc2, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    const long n3 = (long)nx * nx * nx;
    const int grid = cdiv(n3, 256) < 4096 ? cdiv(n3, 256) : 4096;
    k_softmask3d_ring<<<grid, 256, 0, st>>>(map, nx, inn, out, acc2);
    k_softmask3d_apply<<<grid, 256, 0, st>>>(map, nx, inn, out, host_angles().pi, acc2);
    return cudaGetLastError();
}

cudaError_t launch_local_ft(const float2* ft, int nx, float* fr, float* fi, cudaStream_t st) {
    const long n3 = (long)nx * nx * nx;
    k_local_ft<<<cdiv(n3, 256) < 8192 ? cdiv(n3, 256) : 8192, 256, 0, st>>>(ft, nx, fr, fi);
    return cudaGetLastError();
}

void launch_local_box(const float* imgs, int nx0, const int* hk, int nx, int normalize, int B, float* out,
                      cudaStream_t st) {
    k_local_box<<<B, 1024, 0, st>>>(imgs, nx0, hk, nx, normalize, out);
}

void launch_local_ctf(const float* dfs, int nx, float apix, float vol, float cs, float ampwg, int B, float* ctf,
                      cudaStream_t st) {
    dim3 g(cdiv((long)nx * nx, 256), B);
    k_local_ctf<<<g, 256, 0, st>>>(dfs, nx, apix, vol, cs, ampwg, host_angles().pi, ctf);
}

void launch_wlp(float2* b, int nx, long n, float max_r, cudaStream_t st) {
    k_wlp<<<cdiv(n, 256) < 16384 ? cdiv(n, 256) : 16384, 256, 0, st>>>(b, nx, n, max_r);
}

void launch_local_pr(const float* cand, int C, const float* fr, const float* fi, int nx, const float2* part,
                     const float* ctf, float max_r, int B, float* out, cudaStream_t st) {
    dim3 g(C, B);
    const Angles an = host_angles();
    k_local_pr<<<g, 256, 0, st>>>(cand, C, fr, fi, nx, part, ctf, max_r, an.deg2rad, an.pi, out);
}

void launch_lb_checker(const float* imgs, int nx0, const int* src, int B, float2* work, cudaStream_t st) {
    dim3 g(cdiv((long)nx0 * nx0, 256), B);
    k_lb_checker<<<g, 256, 0, st>>>(imgs, nx0, src, work);
}

void launch_lb_phase(float2* work, int nx0, const float* xy, int B, cudaStream_t st) {
    dim3 g(cdiv((long)nx0 * nx0, 256), B);
    k_lb_phase<<<g, 256, 0, st>>>(work, nx0, xy, host_angles().pi);
}

void launch_lb_cut(const float2* work, int nx0, const int* hk, int n, int sub, float* out, cudaStream_t st) {
    if (n > 0) k_lb_cut<<<n, 512, 0, st>>>(work, nx0, hk, sub, out);
}

}  // namespace cryoim
