// mapops.cu — real-space operations on whole maps, compiled with -fmad=false so the FP32
// arithmetic rounds where the Fortran reference rounds:
//   * k_icosavg: real-space icosahedral average (icosprocess/SRC/img3d_icosavg.f90:45-123),
//     an nx^3 x 60 trilinear gather, one thread per voxel, the 60 operators in shared
//     memory, the sum taken operator by operator and term by term as the reference does;
//   * k_merge_real: the last step of merge_reconstruct_FSC.f90:190-198 (origin shift by
//     sign and a spherical cut at imgmask).
#include <cuda_runtime.h>

#include "kernels.h"

namespace cryoim {
namespace {

inline int cdiv(long a, int b) { return (int)((a + b - 1) / b); }

// img3d_icosavg.f90:45-123.  Voxels with r > r0 become 0; a voxel inside averages the
// trilinear samples of the map at S x + nx/2 over the 60 operators S.  A corner that
// falls outside the nx^3 array (only for r0 beyond nx/2 - 2, where the reference reads
// past its array) contributes 0.
__global__ void __launch_bounds__(256) k_icosavg(const float* __restrict__ in, int nx, float r0,
                                                 const float* __restrict__ ops, int nsym,
                                                 float* __restrict__ out) {
    __shared__ float s_ops[60 * 9];
    for (int i = threadIdx.x; i < nsym * 9; i += blockDim.x) s_ops[i] = ops[i];
    __syncthreads();
    const long n3 = (long)nx * nx * nx, nn = (long)nx * nx;
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n3) return;
    const int h = nx / 2;
    const int hx = (int)(q % nx) - h, ky = (int)((q / nx) % nx) - h, lz = (int)(q / nn) - h;
    const float r = sqrtf((float)(hx * hx + ky * ky + lz * lz));
    if (r > r0) { out[q] = 0.0f; return; }
    const float x0[3] = {(float)hx, (float)ky, (float)lz};
    const float fh = (float)h;
    float acc = 0.0f;
    for (int s = 0; s < nsym; ++s) {
        const float* m = s_ops + 9 * s;
        float x[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float t = m[3 * i] * x0[0];
            t = t + m[3 * i + 1] * x0[1];
            t = t + m[3 * i + 2] * x0[2];
            x[i] = t + fh;
        }
        const int ix = (int)x[0], iy = (int)x[1], iz = (int)x[2];
        const float ax = x[0] - (float)ix, ay = x[1] - (float)iy, az = x[2] - (float)iz;
        const float bx = 1.0f - ax, by = 1.0f - ay, bz = 1.0f - az;
        const long n1 = (long)iz * nn + (long)iy * nx + ix;
        const long nb[8] = {n1, n1 + 1, n1 + nx, n1 + nx + 1, n1 + nn, n1 + nn + 1, n1 + nn + nx, n1 + nn + nx + 1};
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (nb[j] >= 0 && nb[j] < n3) ? __ldg(in + nb[j]) : 0.0f;
        acc = acc + bx * by * bz * v[0];
        acc = acc + ax * by * bz * v[1];
        acc = acc + bx * ay * bz * v[2];
        acc = acc + ax * ay * bz * v[3];
        acc = acc + bx * by * az * v[4];
        acc = acc + ax * by * az * v[5];
        acc = acc + bx * ay * az * v[6];
        acc = acc + ax * ay * az * v[7];
    }
    out[q] = acc / (float)nsym;
}

// merge_reconstruct_FSC.f90:190-198: real part, (-1)^(x+y+z), zero beyond imgmask.
__global__ void k_merge_real(const float2* __restrict__ vol, int nx, float r0, float* __restrict__ map) {
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long nn = (long)nx * nx;
    if (q >= nn * nx) return;
    const int hx = (int)(q % nx), ky = (int)((q / nx) % nx), lz = (int)(q / nn), h = nx / 2;
    const float r = sqrtf((float)((hx - h) * (hx - h) + (ky - h) * (ky - h) + (lz - h) * (lz - h)));
    float v = 0.0f;
    if (r <= r0) {
        v = vol[q].x;
        if ((hx + ky + lz) & 1) v = -v;
    }
    map[q] = v;
}

}  // namespace

cudaError_t launch_icosavg(const float* in, int nx, float r0, const float* ops, int nsym, float* out,
                           cudaStream_t st) {
    const long n3 = (long)nx * nx * nx;
    k_icosavg<<<cdiv(n3, 256), 256, 0, st>>>(in, nx, r0, ops, nsym, out);
    return cudaGetLastError();
}

cudaError_t launch_merge_real(const float2* vol, int nx, float r0, float* map, cudaStream_t st) {
    const long n3 = (long)nx * nx * nx;
    k_merge_real<<<cdiv(n3, 256), 256, 0, st>>>(vol, nx, r0, map);
    return cudaGetLastError();
}

}  // namespace cryoim
