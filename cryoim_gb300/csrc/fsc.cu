// fsc.cu — half-map Fourier shell correlation and the FSC-weighted map
// (icosprocess/SRC/reconstruct_FSC.f90:25-178), compiled with -fmad=false so the FP32
// cell arithmetic keeps the reference's operation order.
//
// Inputs are the odd and even tnf partials: (fa, fb, wg) over the half box
// (maxR+1) x (2maxR+1) x (2maxR+1), cell (hx, ky, lz) at ((lz*t + ky+maxR)*t + hx+maxR),
// t = 2maxR+1.  Shells are ir = int(sqrt(hx^2+ky^2+lz^2)) <= maxR.  The shell sums are
// FP64 (the reference sums in FP32, in loop order); the cell algebra is FP32.
#include <cuda_runtime.h>

#include "kernels.h"

namespace cryoim {
namespace {

inline int cdiv(long a, int b) { return (int)((a + b - 1) / b); }

__device__ __forceinline__ int shell_of(int hx, int ky, int lz) {
    return (int)sqrtf((float)(hx * hx + ky * ky + lz * lz));
}

__device__ __forceinline__ long vol_at(int nx, int hx, int ky, int lz) {
    const int h = nx / 2;
    return ((long)(lz + h) * nx + (ky + h)) * nx + (hx + h);
}

// reconstruct_FSC.f90:30-47: wg += 1; a, b /= wg; per shell sum a1 a2 + b1 b2,
// a1^2 + b1^2, a2^2 + b2^2.  Block-local FP64 shell sums in shared memory, then one
// global atomic per shell and block.
__global__ void k_fsc_shells(FscArgs a, double* __restrict__ sums) {
    extern __shared__ double sh[];
    const int R = a.max_r, t = 2 * R + 1, ns = R + 1;
    for (int i = threadIdx.x; i < 3 * ns; i += blockDim.x) sh[i] = 0.0;
    __syncthreads();
    const long n = (long)ns * t * t;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int hx = (int)(q % t) - R, ky = (int)((q / t) % t) - R, lz = (int)(q / ((long)t * t));
        const int ir = shell_of(hx, ky, lz);
        if (ir > R) continue;
        const float w1 = a.wg1[q] + 1.0f, w2 = a.wg2[q] + 1.0f;
        const double a1 = a.fa1[q] / w1, b1 = a.fb1[q] / w1;
        const double a2 = a.fa2[q] / w2, b2 = a.fb2[q] / w2;
        atomicAdd(&sh[ir], a1 * a2 + b1 * b2);
        atomicAdd(&sh[ns + ir], a1 * a1 + b1 * b1);
        atomicAdd(&sh[2 * ns + ir], a2 * a2 + b2 * b2);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * ns; i += blockDim.x)
        if (sh[i] != 0.0) atomicAdd(&sums[i], sh[i]);
}

struct Cell {
    float a, b, w;
};

// reconstruct_FSC.f90:30-35, 64-90: the summed, FSC-weighted cell (a1, b1, wg1 after
// the second "wg1 = wg1 + 1").
__device__ __forceinline__ Cell combined(const FscArgs& a, const float* __restrict__ wt, int hx, int ky,
                                         int lz) {
    const int R = a.max_r, t = 2 * R + 1;
    const long q = ((long)lz * t + (ky + R)) * t + (hx + R);
    const float w1 = a.wg1[q] + 1.0f, w2 = a.wg2[q] + 1.0f;
    float a1 = a.fa1[q] / w1, b1 = a.fb1[q] / w1;
    float a2 = a.fa2[q] / w2, b2 = a.fb2[q] / w2;
    a1 = a1 * w1; b1 = b1 * w1;
    a2 = a2 * w2; b2 = b2 * w2;
    Cell c;
    c.a = a1 + a2;
    c.b = b1 + b2;
    c.w = w1 + w2 - 2.0f;
    const int ir = shell_of(hx, ky, lz);
    if (ir <= R) {
        c.a = c.a * wt[ir]; c.b = c.b * wt[ir]; c.w = c.w * wt[ir];
    } else {
        c.a = 0.0f; c.b = 0.0f;
    }
    c.w = c.w + 1.0f;
    return c;
}

// reconstruct_FSC.f90:96-147: the lz = 0 plane (pairs (hx, ky) / (-hx, -ky) with ky >= 1,
// or ky = 0 and hx >= 1) and the origin.  FFT3d = cmplx(fa, fb).
__global__ void k_fsc_fold_plane0(FscArgs a, const float* __restrict__ wt, float2* __restrict__ vol) {
    const int R = a.max_r, span = 2 * R + 1;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_a = R * span, n_b = R;
    if (q > n_a + n_b) return;
    if (q == n_a + n_b) {
        const Cell c = combined(a, wt, 0, 0, 0);
        vol[vol_at(a.nx, 0, 0, 0)] = make_float2(c.a / c.w, 0.0f);
        return;
    }
    int hx, ky;
    if (q < n_a) { ky = 1 + q / span; hx = q % span - R; }
    else { ky = 0; hx = 1 + (q - n_a); }
    if (shell_of(hx, ky, 0) > R) return;
    const Cell c1 = combined(a, wt, hx, ky, 0), c2 = combined(a, wt, -hx, -ky, 0);
    const float w = c1.w + c2.w;
    float fa1 = (c1.a + c2.a) / w, fb1 = (c1.b - c2.b) / w, fa2, fb2;
    if (((hx + ky) & 1) == 0) { fa2 = fa1; fb2 = -fb1; }
    else { fa1 = -fa1; fb1 = -fb1; fa2 = fa1; fb2 = -fb1; }
    vol[vol_at(a.nx, hx, ky, 0)] = make_float2(fa1, fb1);
    vol[vol_at(a.nx, -hx, -ky, 0)] = make_float2(fa2, fb2);
}

// reconstruct_FSC.f90:150-167: planes lz = 1 .. maxR and their Friedel mates.
__global__ void k_fsc_fold_upper(FscArgs a, const float* __restrict__ wt, float2* __restrict__ vol) {
    const int R = a.max_r, span = 2 * R + 1;
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long)R * span * span) return;
    const int hx = (int)(q % span) - R, ky = (int)((q / span) % span) - R;
    const int lz = 1 + (int)(q / ((long)span * span));
    if (shell_of(hx, ky, lz) > R) return;
    const Cell c = combined(a, wt, hx, ky, lz);
    float fa = c.a / c.w, fb = c.b / c.w;
    if ((hx + ky + lz) & 1) { fa = -fa; fb = -fb; }
    vol[vol_at(a.nx, hx, ky, lz)] = make_float2(fa, fb);
    vol[vol_at(a.nx, -hx, -ky, -lz)] = make_float2(fa, -fb);
}

}  // namespace

cudaError_t launch_fsc_shells(const FscArgs& a, double* sums, int sms, cudaStream_t st) {
    const int ns = a.max_r + 1, t = 2 * a.max_r + 1;
    const long n = (long)ns * t * t;
    int grid = cdiv(n, 256);
    if (grid > 4 * sms) grid = 4 * sms;
    cudaError_t e = cudaMemsetAsync(sums, 0, sizeof(double) * 3 * ns, st);
    if (e != cudaSuccess) return e;
    k_fsc_shells<<<grid, 256, sizeof(double) * 3 * ns, st>>>(a, sums);
    return cudaGetLastError();
}

cudaError_t launch_fsc_fold(const FscArgs& a, const float* wt, float2* vol, cudaStream_t st) {
    const int R = a.max_r, span = 2 * R + 1;
    const long n3 = (long)a.nx * a.nx * a.nx;
    cudaError_t e = cudaMemsetAsync(vol, 0, sizeof(float2) * n3, st);
    if (e != cudaSuccess) return e;
    k_fsc_fold_plane0<<<cdiv((long)R * span + R + 1, 256), 256, 0, st>>>(a, wt, vol);
    k_fsc_fold_upper<<<cdiv((long)R * span * span, 256), 256, 0, st>>>(a, wt, vol);
    return cudaGetLastError();
}

}  // namespace cryoim
