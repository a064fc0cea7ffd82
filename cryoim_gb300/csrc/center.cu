// center.cu — origin centring of icosprocess mode 3 (calc_center.f90 with a model,
// calc_center_selfrot180.f90 without), compiled with -fmad=false so the FP32 arithmetic
// rounds where the Fortran reference rounds.
//
// Every 2D transform of the reference goes through img2d_FFT.f90: z = a + i b, forward
// FFT / nx^2 or backward FFT, returned as (Re, -Im).  Here the buffers are float2 (a, b)
// in that convention: cuFFT runs on (a, b) as a complex number and k_ref_post rewrites
// its output (x, y) as (x / s, -y / s), s = nx^2 forward and 1 backward.  The elementwise
// steps between transforms (checkerboard, Gaussian low pass, CTF, cross-power) are the
// reference's own, in its order.
#include <cuda_runtime.h>

#include "geom.cuh"
#include "kernels.h"

namespace cryoim {
namespace {

inline int cdiv(long a, int b) { return (int)((a + b - 1) / b); }

__device__ double block_sum(double v, double* sh) {
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

// img3d_mask.f90:3-56 at the map centre, pass 1: FP64 sum and count of the edge shell.
__global__ void k_mask3d_ring(const float* __restrict__ d, int nx, float R1, float R2, double* __restrict__ acc) {
    __shared__ double sh[32];
    const long n3 = (long)nx * nx * nx;
    const float c = (float)(nx / 2);
    double s = 0, k = 0;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(q / ((long)nx * nx)), iy = (int)((q / nx) % nx), ix = (int)(q % nx);
        const float yy = (-c + (float)iy) * (-c + (float)iy), xx = (-c + (float)ix) * (-c + (float)ix),
                    zz = (-c + (float)iz) * (-c + (float)iz);
        const float ra = sqrtf(xx + yy + zz);
        if (ra > R1 && ra <= R2) { s += (double)d[q]; k += 1.0; }
    }
    s = block_sum(s, sh);
    k = block_sum(k, sh);
    if (threadIdx.x == 0) { atomicAdd(acc, s); atomicAdd(acc + 1, k); }
}

// pass 2: cosine edge, the shell mean outside.
__global__ void k_mask3d_apply(float* __restrict__ d, int nx, float R1, float R2, float pi,
                               const double* __restrict__ acc) {
    const long n3 = (long)nx * nx * nx;
    const float c = (float)(nx / 2);
    double summ = acc[0];
    if (acc[1] != 0.0) summ = summ / (double)(float)acc[1];
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(q / ((long)nx * nx)), iy = (int)((q / nx) % nx), ix = (int)(q % nx);
        const float yy = (-c + (float)iy) * (-c + (float)iy), xx = (-c + (float)ix) * (-c + (float)ix),
                    zz = (-c + (float)iz) * (-c + (float)iz);
        const float ra = sqrtf(xx + yy + zz);
        if (ra > R1 && ra <= R2) {
            const float edge = (1.0f + cosf(pi * (ra - R1) / 6.0f)) / 2.0f;
            d[q] = (float)((double)(d[q] * edge) + (double)(1.0f - edge) * summ);
        }
        if (ra > R2) d[q] = (float)summ;
    }
}

// calc_center.f90:29-38: shift3dComplex, forward FFT / nx^3, shift3dComplex; the real
// and -imaginary parts as the section source (ft3d_r, ft3d_i).
__global__ void k_center_ft(const float2* __restrict__ ft, int nx, float* __restrict__ fr, float* __restrict__ fi) {
    const long n3 = (long)nx * nx * nx;
    const float s = (float)nx * (float)nx * (float)nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(q / ((long)nx * nx)), iy = (int)((q / nx) % nx), ix = (int)(q % nx);
        float re = ft[q].x / s, im = ft[q].y / s;
        if ((ix + iy + iz) & 1) { re = -re; im = -im; }
        fr[q] = re;
        fi[q] = -im;
    }
}

// after a cuFFT of (a, b): (x, y) -> (x / s, -y / s), img2d_FFT.f90:15-17
__global__ void k_ref_post(float2* __restrict__ b, long n, float s) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const float2 v = b[q];
        b[q] = make_float2(v.x / s, -(v.y / s));
    }
}

// img2d_lowpass.f90:19-25: a, b <- a Huv / nx^2, Huv = exp(-r^2 / (2 lp^2)), r from nx/2
__global__ void k_lowpass(float2* __restrict__ b, int nx, long n, int lp) {
    const long nn = (long)nx * nx;
    const float lowpass = 2.0f * (float)(lp * lp);
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nn), ky = i / nx, hx = i % nx;
        const float r2 = (float)((hx - nx / 2) * (hx - nx / 2) + (ky - nx / 2) * (ky - nx / 2));
        const float huv = expf(-r2 / lowpass);
        const float2 v = b[q];
        b[q] = make_float2(v.x * huv / (float)nn, v.y * huv / (float)nn);
    }
}

// img2d_applyCTF.f90:20-21
__global__ void k_ctf_mul(float2* __restrict__ b, const float* __restrict__ ctf, long n) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const float2 v = b[q];
        b[q] = make_float2(v.x * ctf[q], v.y * ctf[q]);
    }
}

// real part times (-1)^(hx+ky) (the closing "a = a * shift2d" of a transform pair)
__global__ void k_real_shift(const float2* __restrict__ b, int nx, long n, float* __restrict__ out) {
    const long nn = (long)nx * nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nn);
        const float v = b[q].x;
        out[q] = ((i / nx + i % nx) & 1) ? -v : v;
    }
}

// (a, b) <- (re, im) times (-1)^(hx+ky): project2d_FT3dTo2d.f90:86-87; with im == nullptr,
// (a, 0): the opening "a = a * shift2d; b = 0" of a transform pair
__global__ void k_pack_shift(const float* __restrict__ re, const float* __restrict__ im, int nx, long n,
                             float2* __restrict__ b) {
    const long nn = (long)nx * nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nn);
        float a = re[q], c = im ? im[q] : 0.0f;
        if ((i / nx + i % nx) & 1) { a = -a; c = -c; }
        b[q] = make_float2(a, im ? c : 0.0f);
    }
}

// (a, 0) without a shift: cross_correlation.f90:10-13
__global__ void k_pack(const float* __restrict__ re, long n, float2* __restrict__ b) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        b[q] = make_float2(re[q], 0.0f);
}

// img2d_norm.f90 per image (sums in FP64)
__global__ void k_norm(float* __restrict__ img, int nx) {
    __shared__ double sh[32];
    const long nn = (long)nx * nx;
    float* a = img + (long)blockIdx.x * nn;
    double s = 0;
    for (long i = threadIdx.x; i < nn; i += blockDim.x) s += (double)a[i];
    s = block_sum(s, sh);
    const float avg = (float)s / (float)nn;
    double s2 = 0;
    for (long i = threadIdx.x; i < nn; i += blockDim.x) {
        const float d = a[i] - avg;
        s2 += (double)(d * d);
    }
    s2 = block_sum(s2, sh);
    const float nd = sqrtf((float)s2 / (float)nn);
    for (long i = threadIdx.x; i < nn; i += blockDim.x) a[i] = (a[i] - avg) / nd;
}

// cross_correlation.f90:16-23: x = a1 a2 + b1 b2, y = b1 a2 - a1 b2, times (-1)^(hx+ky)
__global__ void k_cross_power(float2* __restrict__ f1, const float2* __restrict__ f2, int nx, long n) {
    const long nn = (long)nx * nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nn);
        const float2 u = f1[q], v = f2[q];
        float x = u.x * v.x + u.y * v.y, y = u.y * v.x - u.x * v.y;
        if ((i / nx + i % nx) & 1) { x = -x; y = -y; }
        f1[q] = make_float2(x, y);
    }
}

// calc_center_selfrot180.f90:41-52: a2 = a1 rotated 180 degrees about (nx/2, nx/2); row 0
// and column 0 of a1 are zeroed (their partners fall outside the box).  (ky, hx) ->
// (nx-ky, nx-hx) maps rows and columns 1..nx-1 onto themselves, so the threads of row 0
// and column 0 are the ones that clear row 0 and column 0 of a2.
__global__ void k_rot180(float* __restrict__ a1, float* __restrict__ a2, int nx, long n) {
    const long nn = (long)nx * nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const long p = q / nn;
        const int i = (int)(q % nn), ky = i / nx, hx = i % nx;
        if (hx == 0 || ky == 0) {
            a1[q] = 0.0f;
            a2[p * nn + (long)(ky == 0 ? 0 : (nx - ky)) * nx + (hx == 0 ? 0 : (nx - hx))] = 0.0f;
        } else {
            a2[p * nn + (long)(nx - ky) * nx + (nx - hx)] = a1[q];
        }
    }
}

// guass_regression.f90: quadratic fit of log z over the 3 x 3 neighbourhood
__device__ void gauss_fit(const float z[3][3], float* dx, float* dy, float* cc) {
    float c10 = 0.f, c01 = 0.f, c11 = 0.f, c20 = 0.f, c02 = 0.f, c00 = 0.f;
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c10 = c10 + (float)i * logf(z[j + 1][i + 1]);
    c10 = c10 / 6.0f;
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c01 = c01 + (float)j * logf(z[j + 1][i + 1]);
    c01 = c01 / 6.0f;
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c11 = c11 + (float)(i * j) * logf(z[j + 1][i + 1]);
    c11 = c11 / 4.0f;
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c20 = c20 + (float)(3 * i * i - 2) * logf(z[j + 1][i + 1]);
    c20 = c20 / 6.0f;
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c02 = c02 + (float)(3 * j * j - 2) * logf(z[j + 1][i + 1]);
    c02 = c02 / 6.0f;
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) c00 = c00 + (float)(5 - 3 * i * i - 3 * j * j) * logf(z[j + 1][i + 1]);
    c00 = c00 / 9.0f;
    const float den = 4.0f * c20 * c02 - c11 * c11;
    *dx = (c11 * c01 - 2.0f * c10 * c02) / den;
    *dy = (c11 * c10 - 2.0f * c01 * c20) / den;
    *cc = expf(c00 - c20 * (*dx * *dx) - c11 * *dx * *dy - c02 * (*dy * *dy));
}

// calc_center.f90:65-80 / calc_center_selfrot180.f90:55-70: first maximum of the
// correlation map (the real parts), its 3 x 3 neighbourhood (linear index clamped to the
// image), the Gaussian fit; out = (centx, centy, cc) per particle, halved for the
// self-rotation form.
__global__ void k_peak(const float2* __restrict__ cc, int nx, int half, float* __restrict__ out) {
    __shared__ float sv[32];
    __shared__ int si[32];
    const long nn = (long)nx * nx;
    const float2* m = cc + (long)blockIdx.x * nn;
    float bv = -3.4e38f;
    int bi = 0x7fffffff;
    for (int i = threadIdx.x; i < (int)nn; i += blockDim.x) {
        const float v = m[i].x;
        if (v > bv) { bv = v; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if ((threadIdx.x & 31) == 0) { sv[threadIdx.x >> 5] = bv; si[threadIdx.x >> 5] = bi; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        if (sv[w] > sv[0] || (sv[w] == sv[0] && si[w] < si[0])) { sv[0] = sv[w]; si[0] = si[w]; }
    const int n0 = si[0], iy0 = n0 / nx, ix0 = n0 % nx;
    float z[3][3];
    for (int ky = -1; ky <= 1; ++ky)
        for (int hx = -1; hx <= 1; ++hx) {
            long j = (long)(iy0 + ky) * nx + (ix0 + hx);
            if (j < 0) j = 0;
            if (j >= nn) j = nn - 1;
            z[ky + 1][hx + 1] = m[j].x;
        }
    float dx, dy, c;
    gauss_fit(z, &dx, &dy, &c);
    float cx = (float)(ix0 - nx / 2) + dx, cy = (float)(iy0 - nx / 2) + dy;
    if (half) { cx = cx / 2.0f; cy = cy / 2.0f; }
    if (fabsf(cx) >= (float)nx / 16.0f) cx = 0.0f;
    if (fabsf(cy) >= (float)nx / 16.0f) cy = 0.0f;
    out[3 * blockIdx.x] = cx;
    out[3 * blockIdx.x + 1] = cy;
    out[3 * blockIdx.x + 2] = c;
}

}  // namespace

cudaError_t launch_mask3d(float* map, int nx, float mask, double* acc2, cudaStream_t st) {
    float R1 = mask - 3.0f;
    if (R1 <= 0.0f) R1 = 0.0f;
    float R2 = mask + 3.0f;
    if (R2 > (float)(nx / 2)) R2 = (float)(nx / 2);
    cudaError_t e = cudaMemsetAsync(acc2, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    const long n3 = (long)nx * nx * nx;
    const int grid = cdiv(n3, 256) < 4096 ? cdiv(n3, 256) : 4096;
    k_mask3d_ring<<<grid, 256, 0, st>>>(map, nx, R1, R2, acc2);
    k_mask3d_apply<<<grid, 256, 0, st>>>(map, nx, R1, R2, host_angles().pi, acc2);
    return cudaGetLastError();
}

cudaError_t launch_center_ft(const float2* ft, int nx, float* fr, float* fi, cudaStream_t st) {
    const long n3 = (long)nx * nx * nx;
    k_center_ft<<<cdiv(n3, 256) < 8192 ? cdiv(n3, 256) : 8192, 256, 0, st>>>(ft, nx, fr, fi);
    return cudaGetLastError();
}

static int grid_of(long n) { return cdiv(n, 256) < 16384 ? cdiv(n, 256) : 16384; }

void launch_ref_post(float2* b, long n, float s, cudaStream_t st) { k_ref_post<<<grid_of(n), 256, 0, st>>>(b, n, s); }
void launch_lowpass(float2* b, int nx, long n, int lp, cudaStream_t st) {
    k_lowpass<<<grid_of(n), 256, 0, st>>>(b, nx, n, lp);
}
void launch_ctf_mul(float2* b, const float* ctf, long n, cudaStream_t st) {
    k_ctf_mul<<<grid_of(n), 256, 0, st>>>(b, ctf, n);
}
void launch_real_shift(const float2* b, int nx, long n, float* out, cudaStream_t st) {
    k_real_shift<<<grid_of(n), 256, 0, st>>>(b, nx, n, out);
}
void launch_pack_shift(const float* re, const float* im, int nx, long n, float2* b, cudaStream_t st) {
    k_pack_shift<<<grid_of(n), 256, 0, st>>>(re, im, nx, n, b);
}
void launch_pack(const float* re, long n, float2* b, cudaStream_t st) { k_pack<<<grid_of(n), 256, 0, st>>>(re, n, b); }
void launch_norm(float* img, int nx, int B, cudaStream_t st) { k_norm<<<B, 1024, 0, st>>>(img, nx); }
void launch_cross_power(float2* f1, const float2* f2, int nx, long n, cudaStream_t st) {
    k_cross_power<<<grid_of(n), 256, 0, st>>>(f1, f2, nx, n);
}
void launch_rot180(float* a1, float* a2, int nx, long n, cudaStream_t st) {
    k_rot180<<<grid_of(n), 256, 0, st>>>(a1, a2, nx, n);
}
void launch_peak(const float2* cc, int nx, int B, int half, float* out, cudaStream_t st) {
    k_peak<<<B, 1024, 0, st>>>(cc, nx, half, out);
}

}  // namespace cryoim
