// contract.cu — the projection-matching contraction form of the global search.
//
// Score: for particle p, origin s and orientation R,
//     CC(p, s, R) = Re sum_h  A_ps(h) conj(B_R(h)) / (|A_p| |B_R|)
// over the half-plane band samples h (minR <= |h| <= maxR), with
//     A_ps(h) = CTF_p(h) P_p(h) exp(2 pi i h.(s + nx/2)/nx)     (the particle, its CTF and
//               the origin shift of img2d_FT_centshift.f90, so the reference's CTF
//               multiply and origin ramps sit on the particle side of the product)
//     B_R(h)  = M(R (hx, ky, 0))                                (trilinear central section
//               of the centred 3D Fourier map, project2d_FT3dTo2d.f90:30-83)
// Stacking (Re, Im) along K turns it into one real contraction
//     C[(p,s), R] = sum_k A[(p,s), k] B[R, k],   K = 2 x samples,
// which gemm_tc.cu runs on the tensor cores in BF16 with FP32 accumulation.  The
// normalisation sums are FP64; the best candidates are rescored in FP64 here and with
// the reference's phase residual (k_pr_single) by the driver.
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include "geom.cuh"
#include "kernels.h"

namespace cryoim {
namespace {

__device__ double block_sum_double(double v, double* sh) {
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

// map * (-1)^(x+y+z) as complex, so the forward FFT is centred at nx/2
__global__ void k_map_checker(const float* __restrict__ map, int nx, float2* __restrict__ out) {
    const long n3 = (long)nx * nx * nx;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long)gridDim.x * blockDim.x) {
        int x = (int)(q % nx), y = (int)((q / nx) % nx), z = (int)(q / ((long)nx * nx));
        float v = map[q];
        out[q] = make_float2(((x + y + z) & 1) ? -v : v, 0.0f);
    }
}

// Band cube of the transform: frequencies -(R+1) .. R+1 per axis, phase referenced to
// the map centre ((-1)^(kx+ky+kz)), standard complex convention, scaled by 1/nx^3.
__global__ void k_map_band(const float2* __restrict__ ft, int nx, int R, float2* __restrict__ cube) {
    const int C = 2 * R + 3, h = nx / 2;
    const long total = (long)C * C * C;
    const float s = 1.0f / ((float)nx * (float)nx * (float)nx);
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
        int x = (int)(q % C), y = (int)((q / C) % C), z = (int)(q / ((long)C * C));
        int kx = x - (R + 1), ky = y - (R + 1), kz = z - (R + 1);
        float2 v = ft[((long)(kz + h) * nx + (ky + h)) * nx + (kx + h)];
        float sg = ((kx + ky + kz) & 1) ? -s : s;
        cube[q] = make_float2(v.x * sg, v.y * sg);
    }
}

// Gaussian-kernel interpolation of the band cube (C^3 float2, frequency k at index
// k + off): the 3 x 3 x 3 voxels around the nearest one to (x, y, z), each weighted by
// exp(-d^2 / (2 sigma^2)) (gk = 1 / (2 sigma^2); the weight is separable in x, y, z),
// normalised by the weights' sum.  |(x, y, z)| <= maxR keeps every tap inside the cube.
__device__ __forceinline__ float2 gauss_sample(const float2* __restrict__ cube, int C, int off, float x, float y,
                                               float z, float gk) {
    const float rx = rintf(x), ry = rintf(y), rz = rintf(z);
    float wx[3], wy[3], wz[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float ex = x - (rx + (float)(d - 1)), ey = y - (ry + (float)(d - 1)), ez = z - (rz + (float)(d - 1));
        wx[d] = expf(-gk * ex * ex);
        wy[d] = expf(-gk * ey * ey);
        wz[d] = expf(-gk * ez * ez);
    }
    const float2* b = cube + ((long)((int)rz + off - 1) * C + ((int)ry + off - 1)) * C + ((int)rx + off - 1);
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int dz = 0; dz < 3; ++dz)
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            const float2* r = b + ((long)dz * C + dy) * C;
            const float w = wz[dz] * wy[dy];
            const float2 v0 = r[0], v1 = r[1], v2 = r[2];
            acc.x += w * (wx[0] * v0.x + wx[1] * v1.x + wx[2] * v2.x);
            acc.y += w * (wx[0] * v0.y + wx[1] * v1.y + wx[2] * v2.y);
        }
    const float inv = 1.0f / ((wx[0] + wx[1] + wx[2]) * (wy[0] + wy[1] + wy[2]) * (wz[0] + wz[1] + wz[2]));
    return make_float2(acc.x * inv, acc.y * inv);
}

// Section rows are stored pre-swizzled: within each 128-byte block of K, the 16-byte
// chunk c of row r sits at chunk c ^ (r & 7), the order in which a TMA load with the
// 128-byte swizzle would place it in shared memory.  A row copied verbatim into a tile
// row of the same residue mod 8 (a TMA box without swizzle) is then already in the
// layout the tensor cores read; a row copied by index into any tile row has its chunks
// re-ordered by the XOR of the two residues (gemm_tc.cu, B rows by index).  Index of
// (Re, Im) pair i of row r: BF16 rows hold 32 pairs per block (4 per chunk), FP8 rows 64
// (8 per chunk).
__device__ __forceinline__ long bf16_pair_at(long i, long r) {
    return (i & ~31L) | ((((i >> 2) & 7) ^ (r & 7)) << 2) | (i & 3);
}
__device__ __forceinline__ long fp8_pair_at(long i, long r) {
    return (i & ~63L) | ((((i >> 3) & 7) ^ (r & 7)) << 3) | (i & 7);
}

// One CTA per orientation n = view * nomega + iomega: section samples in shared
// memory, norm (FP32 per thread, FP64 across the block), then the unit-norm row in BF16
// (Re, Im interleaved, zero pad).  The trilinear interpolation runs on the texture
// units: the band cube is a float2 3D array with linear filtering (hardware weights in
// 1/256 steps, well inside the BF16 rounding of the row), texel centres at +0.5, zero
// outside the cube.
__global__ void __launch_bounds__(512) k_slice_bf16(cudaTextureObject_t cube, int R,
                                                    const int2* __restrict__ samples, int S, int Kpad,
                                                    const float* __restrict__ views, int nom, float step,
                                                    float d2r, long n0, __nv_bfloat162* __restrict__ B,
                                                    const float2* __restrict__ lin, float gk, float sc) {
    extern __shared__ float2 ssec[];
    __shared__ double sh[32];
    __shared__ float rot[9];
    const long n = n0 + blockIdx.x;
    const int v = (int)(n / nom), io = (int)(n % nom);
    if (threadIdx.x == 0) {
        euler_mat(views[2 * v], views[2 * v + 1], step * (float)io, d2r, rot);
        for (int i = 0; i < 9; ++i) rot[i] *= sc;  // cube voxels per frequency unit
    }
    __syncthreads();
    const float off = (float)(R + 1) + 0.5f;
    float part = 0.0f;
    // four samples per step: their fetches are independent and in flight together
#pragma unroll 4
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        const int2 hk = samples[i];
        const float hx = (float)hk.x, ky = (float)hk.y;
        const float x = rot[0] * hx + rot[1] * ky, y = rot[3] * hx + rot[4] * ky, z = rot[6] * hx + rot[7] * ky;
        const float2 val = gk > 0.0f ? gauss_sample(lin, 2 * R + 3, R + 1, x, y, z, gk)
                                     : tex3D<float2>(cube, x + off, y + off, z + off);
        ssec[i] = val;
        part += val.x * val.x + val.y * val.y;
    }
    const double nrm = block_sum_double((double)part, sh);
    const float inv = nrm > 0.0 ? (float)(1.0 / sqrt(nrm)) : 0.0f;
    __nv_bfloat162* row = B + (long)blockIdx.x * (Kpad / 2);
    for (int i = threadIdx.x; i < Kpad / 2; i += blockDim.x) {
        float2 val = i < S ? ssec[i] : make_float2(0.f, 0.f);
        row[bf16_pair_at(i, n)] = __floats2bfloat162_rn(val.x * inv, val.y * inv);
    }
}

// Local grids: one CTA per (particle p, grid point l) with l = (i * n + j) * n + k,
// n = 2 m + 1, orientation (theta_p + (i - m) s, phi_p + (j - m) s, omega_p + (k - m) s)
// from centre[3 p ..]; particle p's rows start at row p * lpitch (lpitch >= n^3); the
// row is built exactly as k_slice_bf16 builds it.
// With pctf (the CTF of each particle at each sample), a row is normalised by |CTF S|
// instead of |S|: the particle's own grid, so the contraction's score is the unbiased
// projection-matching correlation sum Re(P conj(CTF S)) / (|P| |CTF S|) (with A rows
// normalised by |P|), whose maximum lies at the particle's orientation.  Normalising by
// |S| (a section shared by every particle, as in the global bank) moves the maximum by
// a fraction of a degree on whole particles and by degrees on the local maps' sections.
__global__ void __launch_bounds__(512) k_slice_bf16_local(cudaTextureObject_t cube, int R,
                                                          const int2* __restrict__ samples, int S, int Kpad,
                                                          const float* __restrict__ centre, int m, float step,
                                                          float d2r, long n0, __nv_bfloat162* __restrict__ B,
                                                          const float2* __restrict__ lin, float gk, long lpitch,
                                                          const float* __restrict__ pctf, float sc) {
    extern __shared__ float2 ssec[];
    __shared__ double sh[32];
    __shared__ float rot[9];
    const int n = 2 * m + 1;
    const long nloc = (long)n * n * n;
    const long q = n0 + blockIdx.x;
    const int p = (int)(q / lpitch), l = (int)(q % lpitch);
    if (l >= nloc) return;  // padding row between particles' grids (never a valid column)
    const int i = l / (n * n), j = (l / n) % n, k = l % n;
    if (threadIdx.x == 0) {
        euler_mat(centre[3 * p] + step * (float)(i - m), centre[3 * p + 1] + step * (float)(j - m),
                  centre[3 * p + 2] + step * (float)(k - m), d2r, rot);
        for (int e = 0; e < 9; ++e) rot[e] *= sc;  // cube voxels per frequency unit
    }
    __syncthreads();
    const float off = (float)(R + 1) + 0.5f;
    float part = 0.0f;
#pragma unroll 4
    for (int t = threadIdx.x; t < S; t += blockDim.x) {
        const int2 hk = samples[t];
        const float hx = (float)hk.x, ky = (float)hk.y;
        const float x = rot[0] * hx + rot[1] * ky, y = rot[3] * hx + rot[4] * ky, z = rot[6] * hx + rot[7] * ky;
        const float2 val = gk > 0.0f ? gauss_sample(lin, 2 * R + 3, R + 1, x, y, z, gk)
                                     : tex3D<float2>(cube, x + off, y + off, z + off);
        ssec[t] = val;
        const float cw = pctf ? pctf[(long)p * S + t] : 1.0f;
        part += cw * cw * (val.x * val.x + val.y * val.y);
    }
    const double nrm = block_sum_double((double)part, sh);
    const float inv = nrm > 0.0 ? (float)(1.0 / sqrt(nrm)) : 0.0f;
    __nv_bfloat162* row = B + (long)blockIdx.x * (Kpad / 2);
    for (int t = threadIdx.x; t < Kpad / 2; t += blockDim.x) {
        float2 val = t < S ? ssec[t] : make_float2(0.f, 0.f);
        row[bf16_pair_at(t, q)] = __floats2bfloat162_rn(val.x * inv, val.y * inv);
    }
}

// The same rows, one CTA per (particle p, i, j) cutting the n rows k = 0 .. n - 1 (the
// omega steps) in turn: a thread holds its samples (h, k, CTF^2) in registers across the
// rows and a row's values in registers until its norm is known, so the CTA needs no
// shared-memory row and the SM's L1 stays large for the texture fetches, which
// neighbouring omegas share (0.25 degrees moves a sample by a fraction of a voxel).
// Each row's values, norm and BF16 row are k_slice_bf16_local's; the norm's FP32
// per-thread partials cover fewer samples (it agrees to FP32 rounding).
constexpr int LSR_THREADS = 256, LSR_SPT = 8;  // rows of up to 2,048 samples (pairs)
__global__ void __launch_bounds__(LSR_THREADS) k_slice_bf16_local_rows(
    cudaTextureObject_t cube, int R, const int2* __restrict__ samples, int S, int Kpad,
    const float* __restrict__ centre, int m, float step, float d2r, __nv_bfloat162* __restrict__ B,
    const float2* __restrict__ lin, float gk, long lpitch, const float* __restrict__ pctf, float sc) {
    extern __shared__ float rots[];  // [n][9]
    __shared__ double wsum[2][LSR_THREADS / 32];
    const int n = 2 * m + 1;
    const int p = blockIdx.y, ij = blockIdx.x;
    const int i = ij / n, j = ij % n;
    for (int k = threadIdx.x; k < n; k += LSR_THREADS) {
        float* rot = rots + 9 * k;
        euler_mat(centre[3 * p] + step * (float)(i - m), centre[3 * p + 1] + step * (float)(j - m),
                  centre[3 * p + 2] + step * (float)(k - m), d2r, rot);
        for (int e = 0; e < 9; ++e) rot[e] *= sc;  // cube voxels per frequency unit
    }
    float hx[LSR_SPT], ky[LSR_SPT], cw2[LSR_SPT];
#pragma unroll
    for (int s = 0; s < LSR_SPT; ++s) {
        const int t = threadIdx.x + s * LSR_THREADS;
        hx[s] = 0.0f;
        ky[s] = 0.0f;
        cw2[s] = 0.0f;
        if (t < S) {
            const int2 hk = samples[t];
            hx[s] = (float)hk.x;
            ky[s] = (float)hk.y;
            const float cw = pctf ? pctf[(long)p * S + t] : 1.0f;
            cw2[s] = cw * cw;
        }
    }
    __syncthreads();
    const float off = (float)(R + 1) + 0.5f;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = 0; k < n; ++k) {
        const float* rot = rots + 9 * k;
        const float r0 = rot[0], r1 = rot[1], r3 = rot[3], r4 = rot[4], r6 = rot[6], r7 = rot[7];
        float2 val[LSR_SPT];
        float part = 0.0f;
#pragma unroll
        for (int s = 0; s < LSR_SPT; ++s) {
            val[s] = make_float2(0.f, 0.f);
            if (threadIdx.x + s * LSR_THREADS < S) {
                const float x = r0 * hx[s] + r1 * ky[s], y = r3 * hx[s] + r4 * ky[s], z = r6 * hx[s] + r7 * ky[s];
                val[s] = gk > 0.0f ? gauss_sample(lin, 2 * R + 3, R + 1, x, y, z, gk)
                                   : tex3D<float2>(cube, x + off, y + off, z + off);
                part += cw2[s] * (val[s].x * val[s].x + val[s].y * val[s].y);
            }
        }
        // norm: FP64 across the block in a fixed order (warps, then the warps' sums)
        double d = (double)part;
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (lane == 0) wsum[k & 1][wid] = d;
        __syncthreads();  // also orders this row's reads of wsum[k & 1] before row k + 2 writes it
        double nrm = 0.0;
#pragma unroll
        for (int w = 0; w < LSR_THREADS / 32; ++w) nrm += wsum[k & 1][w];
        const float inv = nrm > 0.0 ? (float)(1.0 / sqrt(nrm)) : 0.0f;
        const long q = (long)p * lpitch + (long)ij * n + k;
        __nv_bfloat162* row = B + q * (Kpad / 2);
#pragma unroll
        for (int s = 0; s < LSR_SPT; ++s) {
            const int t = threadIdx.x + s * LSR_THREADS;
            if (t < Kpad / 2) row[bf16_pair_at(t, q)] = __floats2bfloat162_rn(val[s].x * inv, val[s].y * inv);
        }
    }
}

// FP64 sum over samples of |CTF * P|^2 per particle (the origin shift keeps it); with
// pc, also the samples CTF * (a, b) themselves in FP64, in sample order.
// With norm0, also the sum of |P|^2 without the CTF; with pctf, the CTF at each sample.
__global__ void k_particle_norm(const float2* __restrict__ band, const float* __restrict__ ctf, Band bd,
                                const int2* __restrict__ samples, int S, double* __restrict__ norm,
                                double2* __restrict__ pc, double* __restrict__ norm0, float* __restrict__ pctf) {
    __shared__ double sh[32];
    const int p = blockIdx.x, W = bd.W, R = bd.max_r;
    const float2* b = band + (long)p * W * W;
    const float* c = ctf ? ctf + (long)p * W * W : nullptr;
    double acc = 0.0, acc0 = 0.0;
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        const int2 hk = samples[i];
        const int q = (hk.y + R) * W + (hk.x + R);
        const double cv = c ? (double)c[q] : 1.0;
        const double re = b[q].x * cv, im = b[q].y * cv;
        acc += re * re + im * im;
        acc0 += (double)b[q].x * b[q].x + (double)b[q].y * b[q].y;
        if (pc) pc[(long)p * S + i] = make_double2(re, im);
        if (pctf) pctf[(long)p * S + i] = c ? c[q] : 1.0f;
    }
    acc = block_sum_double(acc, sh);
    if (threadIdx.x == 0) norm[p] = acc;
    if (norm0) {
        acc0 = block_sum_double(acc0, sh);
        if (threadIdx.x == 0) norm0[p] = acc0;
    }
}

// The origin phase exp(i 2pi/n (sx hx + sy ky)) of a row of A is separable: the block
// tabulates (cos, sin) of 2pi/n sx hx for hx in [0, R] and of 2pi/n sy ky for ky in
// [-R, R] (3R + 2 entries in shared memory) and multiplies the two per sample.
__device__ __forceinline__ void origin_phasors(float sx, float sy, int R, float two_pi_over_n, float2* tab) {
    for (int i = threadIdx.x; i < 3 * R + 2; i += blockDim.x) {
        const float a = i <= R ? two_pi_over_n * (sx * (float)i) : two_pi_over_n * (sy * (float)(i - 2 * R - 1));
        float sn, cs;
        sincosf(a, &sn, &cs);
        tab[i] = make_float2(cs, sn);
    }
    __syncthreads();
}
__device__ __forceinline__ void phasor_at(const float2* tab, int R, int2 hk, float* sn, float* cs) {
    const float2 ex = tab[hk.x], ey = tab[R + 1 + R + hk.y];
    *cs = ex.x * ey.x - ex.y * ey.y;
    *sn = ex.y * ey.x + ex.x * ey.y;
}

// Rows (p, o0 .. o0 + AO - 1) of A: CTF x particle x origin phase ramp, unit norm,
// BF16.  Each thread reads a sample's transform and CTF once and writes it for AO
// origins (phasor tables of all AO origins in shared memory).
constexpr int AO = 8;
__global__ void __launch_bounds__(256) k_build_a(const float2* __restrict__ band, const float* __restrict__ ctf,
                                                 Band bd, const int2* __restrict__ samples, int S, int Kpad,
                                                 const float* __restrict__ origins, int O,
                                                 const float* __restrict__ poff,
                                                 const double* __restrict__ norm, float two_pi_over_n,
                                                 __nv_bfloat162* __restrict__ A) {
    extern __shared__ float2 ptab[];  // [AO][3 R + 2]
    const int o0 = blockIdx.x * AO, p = blockIdx.y, W = bd.W, R = bd.max_r, nt = 3 * R + 2;
    const int no = min(AO, O - o0);
    const float2* b = band + (long)p * W * W;
    const float* c = ctf ? ctf + (long)p * W * W : nullptr;
    // origins relative to the particle's own (poff) or absolute
    const float hx = (float)(bd.nx / 2) + (poff ? poff[2 * p] : 0.0f);
    const float hy = (float)(bd.nx / 2) + (poff ? poff[2 * p + 1] : 0.0f);
    const float inv = norm[p] > 0.0 ? (float)(1.0 / sqrt(norm[p])) : 0.0f;
    for (int j = 0; j < no; ++j) {
        const float sx = origins[2 * (o0 + j)] + hx, sy = origins[2 * (o0 + j) + 1] + hy;
        for (int i = threadIdx.x; i < nt; i += blockDim.x) {
            const float a = i <= R ? two_pi_over_n * (sx * (float)i)
                                   : two_pi_over_n * (sy * (float)(i - 2 * R - 1));
            float sn, cs;
            sincosf(a, &sn, &cs);
            ptab[j * nt + i] = make_float2(cs, sn);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < Kpad / 2; i += blockDim.x) {
        if (i < S) {
            const int2 hk = samples[i];
            const int q = (hk.y + R) * W + (hk.x + R);
            const float2 ab = b[q];  // (a, b) = (Re F, -Im F) referenced to pixel 0
            const float cv = (c ? c[q] : 1.0f) * inv;
            for (int j = 0; j < no; ++j) {
                float sn, cs;
                phasor_at(ptab + j * nt, R, hk, &sn, &cs);
                // centshift: (a', b') = (a cos + b sin, -a sin + b cos); P = a' - i b'
                const float a2 = ab.x * cs + ab.y * sn, b2 = -ab.x * sn + ab.y * cs;
                A[((long)p * O + o0 + j) * (Kpad / 2) + i] = __floats2bfloat162_rn(a2 * cv, -b2 * cv);
            }
        } else {
            for (int j = 0; j < no; ++j)
                A[((long)p * O + o0 + j) * (Kpad / 2) + i] = __floats2bfloat162_rn(0.f, 0.f);
        }
    }
}

// Per (particle, column tile): the best of its O origin rows -> (cc, orientation,
// origin).  Distinct tiles hold distinct orientations.
__global__ void k_tile_best(const float* __restrict__ topv, const int* __restrict__ topi, int O,
                            int ntiles, float* __restrict__ bv_out, int* __restrict__ bo_out,
                            int* __restrict__ borig_out) {
    __shared__ float sv[32];
    __shared__ int si[32];
    const int t = blockIdx.x, p = blockIdx.y;
    float bv = -3.0e38f;
    int bi = -1;
    for (int o = threadIdx.x; o < O; o += blockDim.x) {
        const float v = topv[((long)p * O + o) * ntiles + t];
        if (v > bv) { bv = v; bi = o; }
    }
    for (int off = 16; off > 0; off >>= 1) {
        float ov = __shfl_xor_sync(0xffffffffu, bv, off);
        int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ov > bv || (ov == bv && oi >= 0 && oi < bi)) { bv = ov; bi = oi; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) { sv[w] = bv; si[w] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < nw; ++q)
            if (sv[q] > sv[0] || (sv[q] == sv[0] && si[q] >= 0 && si[q] < si[0])) { sv[0] = sv[q]; si[0] = si[q]; }
        const long o = (long)p * ntiles + t;
        bv_out[o] = sv[0];
        borig_out[o] = si[0] < 0 ? 0 : si[0];
        bo_out[o] = si[0] < 0 ? -1 : topi[((long)p * O + si[0]) * ntiles + t];
    }
}

// Per particle: the k best entries of cnt (value, orientation, origin) triples, by
// repeated block argmax (selected values are set to -inf in v, a scratch array).
__global__ void k_select_topk(float* __restrict__ v, const int* __restrict__ orient,
                              const int* __restrict__ origin, int cnt_per_particle, int k,
                              int* __restrict__ out_orient, int* __restrict__ out_origin,
                              float* __restrict__ out_cc) {
    __shared__ float sv[32];
    __shared__ long si[32];
    const int p = blockIdx.x;
    const long base = (long)p * cnt_per_particle, cnt = cnt_per_particle;
    float* topv = v;
    for (int r = 0; r < k; ++r) {
        float bv = -3.0e38f;
        long bi = -1;
        for (long q = threadIdx.x; q < cnt; q += blockDim.x) {
            float v = topv[base + q];
            if (v > bv) { bv = v; bi = q; }
        }
        for (int off = 16; off > 0; off >>= 1) {
            float ov = __shfl_xor_sync(0xffffffffu, bv, off);
            long oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ov > bv || (ov == bv && oi < bi && oi >= 0)) { bv = ov; bi = oi; }
        }
        const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
        if (l == 0) { sv[w] = bv; si[w] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            float v0 = sv[0];
            long i0 = si[0];
            for (int q = 1; q < nw; ++q)
                if (sv[q] > v0 || (sv[q] == v0 && si[q] < i0 && si[q] >= 0)) { v0 = sv[q]; i0 = si[q]; }
            if (i0 >= 0 && v0 > -3.0e38f) {
                out_orient[p * k + r] = orient[base + i0];
                out_origin[p * k + r] = origin[base + i0];
                out_cc[p * k + r] = v0;
                topv[base + i0] = -3.0e38f;
            } else {
                out_orient[p * k + r] = -1;
                out_origin[p * k + r] = 0;
                out_cc[p * k + r] = -3.0e38f;
            }
        }
        __syncthreads();
    }
}

// Proposal form, per particle: the k best (origin row, column tile) maxima with
// distinct orientations.  v[o * ntiles + t] is the best CC of tile t at origin o and
// col[...] its column in the gathered list; once a column is taken, every entry that
// names it is retired, so the candidates are k distinct orientations, each at its best
// origin.  Columns are remapped to orientations on the host.
// One block per particle of a group: seg[b] = (offset of its entries, its ntiles).
__global__ void k_select_distinct(float* __restrict__ v0, const int* __restrict__ col0, int O,
                                  const int2* __restrict__ seg, int k, int* __restrict__ out_col0,
                                  int* __restrict__ out_origin0, float* __restrict__ out_cc0) {
    __shared__ float sv[32];
    __shared__ int si[32];
    __shared__ int taken;
    const int2 sg = seg[blockIdx.x];
    const int ntiles = sg.y, cnt = O * ntiles;
    float* v = v0 + sg.x;
    const int* col = col0 + sg.x;
    int* out_col = out_col0 + (long)blockIdx.x * k;
    int* out_origin = out_origin0 + (long)blockIdx.x * k;
    float* out_cc = out_cc0 + (long)blockIdx.x * k;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = 0; r < k; ++r) {
        float bv = -3.0e38f;
        int bi = -1;
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const float x = v[q];
            if (col[q] >= 0 && x > bv) { bv = x; bi = q; }
        }
        for (int off = 16; off > 0; off >>= 1) {
            float ov = __shfl_xor_sync(0xffffffffu, bv, off);
            int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ov > bv || (ov == bv && oi >= 0 && (bi < 0 || oi < bi))) { bv = ov; bi = oi; }
        }
        if (l == 0) { sv[w] = bv; si[w] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            float v0 = sv[0];
            int i0 = si[0];
            for (int q = 1; q < nw; ++q)
                if (sv[q] > v0 || (sv[q] == v0 && si[q] >= 0 && (i0 < 0 || si[q] < i0))) { v0 = sv[q]; i0 = si[q]; }
            if (i0 >= 0 && v0 > -3.0e38f) {
                out_col[r] = col[i0];
                out_origin[r] = i0 / ntiles;
                out_cc[r] = v0;
                taken = col[i0];
            } else {
                out_col[r] = -1;
                out_origin[r] = 0;
                out_cc[r] = -3.0e38f;
                taken = -1;
            }
        }
        __syncthreads();
        const int t = taken;
        if (t >= 0)
            for (int q = threadIdx.x; q < cnt; q += blockDim.x)
                if (col[q] == t) v[q] = -3.0e38f;
        __syncthreads();
    }
}

// FP64 rescoring of one (particle, candidate): the same CC with every product,
// interpolation and sum in double precision.
// FP64 rescoring, one (candidate, particle, sample chunk) per block: the three sums of
// the CC (p.q, |p|^2, |q|^2) over samples [S*s/NS, S*(s+1)/NS).  The section sample
// is interpolated at FP64-rotated coordinates; its trilinear blend of the FP32 cube runs
// in FP32 (the data's own precision), every product and sum after it in FP64.  The
// origin shift exp(-i 2pi (sx hx + sy ky)/n) is separable, so each block tabulates the
// per-hx and per-ky phasors in double once and multiplies them per sample.
constexpr int CC_SPLIT = 4;

__global__ void k_cc_fp64(const float2* __restrict__ cube, const double2* __restrict__ pcband, Band bd,
                          const int2* __restrict__ samples, int S, const float* __restrict__ cand, int k,
                          double* __restrict__ part, double gk, const float* __restrict__ pctf, int Rq, double sc) {
    extern __shared__ double2 ctab[];  // [R + 1] per hx, then [2R + 1] per ky
    __shared__ double sh[32];
    __shared__ double rot[9];
    // R: the band; Rq: the cube's radius (its side C = 2 Rq + 3), sc cube voxels per frequency
    const int c = blockIdx.x, p = blockIdx.y, sp = blockIdx.z, R = bd.max_r, C = 2 * Rq + 3, off = Rq + 1;
    const float* cd = cand + ((long)p * k + c) * 5;
    if (threadIdx.x == 0) {
        const double d2r = 3.14159265358979323846 / 180.0;
        double t = cd[0] * d2r, ph = cd[1] * d2r, om = cd[2] * d2r;
        double c1 = cos(ph), c2 = cos(t), c3 = cos(om), s1 = sin(ph), s2 = sin(t), s3 = sin(om);
        rot[0] = c1 * c2 * c3 - s1 * s3; rot[1] = -c1 * c2 * s3 - c3 * s1; rot[2] = c1 * s2;
        rot[3] = c2 * c3 * s1 + c1 * s3; rot[4] = -c2 * s1 * s3 + c1 * c3; rot[5] = s1 * s2;
        rot[6] = -c3 * s2;               rot[7] = s2 * s3;                 rot[8] = c2;
        for (int i = 0; i < 9; ++i) rot[i] *= sc;
    }
    const double h = (double)(bd.nx / 2), sx = cd[3] + h, sy = cd[4] + h;
    const double tpn = 2.0 * 3.14159265358979323846 / (double)bd.nx;
    double2* tx = ctab;
    double2* ty = ctab + (R + 1);
    for (int i = threadIdx.x; i < 3 * R + 2; i += blockDim.x) {
        double th, sn, cs;
        if (i <= R) th = tpn * (sx * (double)i);
        else th = tpn * (sy * (double)(i - (R + 1) - R));
        sincos(th, &sn, &cs);
        ctab[i] = make_double2(cs, sn);
    }
    __syncthreads();
    const double2* pcb = pcband + (long)p * S;  // CTF x (a, b) per sample, FP64 (k_particle_norm)
    double dot = 0, nb = 0;  // the particle's norm is the same for every candidate: k_particle_norm
    const int i0 = (int)((long)S * sp / gridDim.z), i1 = (int)((long)S * (sp + 1) / gridDim.z);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int2 hk = samples[i];
        const double x = rot[0] * hk.x + rot[1] * hk.y, y = rot[3] * hk.x + rot[4] * hk.y,
                     z = rot[6] * hk.x + rot[7] * hk.y;
        double sr, si;
        if (gk > 0.0) {
            // Gaussian kernel in FP64 over the 27 voxels around the nearest one
            const double rx = rint(x), ry = rint(y), rz = rint(z);
            double wx[3], wy[3], wz[3];
            for (int d = 0; d < 3; ++d) {
                const double ex = x - (rx + (d - 1)), ey = y - (ry + (d - 1)), ez = z - (rz + (d - 1));
                wx[d] = exp(-gk * ex * ex);
                wy[d] = exp(-gk * ey * ey);
                wz[d] = exp(-gk * ez * ez);
            }
            const float2* b0 = cube + ((long)((int)rz + off - 1) * C + ((int)ry + off - 1)) * C + ((int)rx + off - 1);
            double ar = 0.0, ai = 0.0;
            for (int dz = 0; dz < 3; ++dz)
                for (int dy = 0; dy < 3; ++dy) {
                    const float2* rr = b0 + ((long)dz * C + dy) * C;
                    const double w = wz[dz] * wy[dy];
                    ar += w * (wx[0] * rr[0].x + wx[1] * rr[1].x + wx[2] * rr[2].x);
                    ai += w * (wx[0] * rr[0].y + wx[1] * rr[1].y + wx[2] * rr[2].y);
                }
            const double inv = 1.0 / ((wx[0] + wx[1] + wx[2]) * (wy[0] + wy[1] + wy[2]) * (wz[0] + wz[1] + wz[2]));
            sr = ar * inv;
            si = ai * inv;
        } else {
            // the cube holds FP32 values: its trilinear blend runs in FP32 at the FP64-rotated
            // coordinates rounded once to FP32 (|x| <= maxR + 1: within 2^-17 px), the products
            // and sums below in FP64
            const float xf = (float)x, yf = (float)y, zf = (float)z;
            const float fx = floorf(xf), fy = floorf(yf), fz = floorf(zf);
            const int ix = (int)fx + off, iy = (int)fy + off, iz = (int)fz + off;
            const float ax = xf - fx, ay = yf - fy, az = zf - fz;
            const float2* cb0 = cube + ((long)iz * C + iy) * C + ix;
            float2 r0, r1;
            {
                const float2 v000 = cb0[0], v001 = cb0[1], v010 = cb0[C], v011 = cb0[C + 1];
                const float2 v100 = cb0[C * C], v101 = cb0[C * C + 1], v110 = cb0[C * C + C], v111 = cb0[C * C + C + 1];
                const float2 a0 = make_float2(fmaf(ax, v001.x - v000.x, v000.x), fmaf(ax, v001.y - v000.y, v000.y));
                const float2 a1 = make_float2(fmaf(ax, v011.x - v010.x, v010.x), fmaf(ax, v011.y - v010.y, v010.y));
                const float2 a2 = make_float2(fmaf(ax, v101.x - v100.x, v100.x), fmaf(ax, v101.y - v100.y, v100.y));
                const float2 a3 = make_float2(fmaf(ax, v111.x - v110.x, v110.x), fmaf(ax, v111.y - v110.y, v110.y));
                r0 = make_float2(fmaf(ay, a1.x - a0.x, a0.x), fmaf(ay, a1.y - a0.y, a0.y));
                r1 = make_float2(fmaf(ay, a3.x - a2.x, a2.x), fmaf(ay, a3.y - a2.y, a2.y));
            }
            sr = (double)fmaf(az, r1.x - r0.x, r0.x);
            si = (double)fmaf(az, r1.y - r0.y, r0.y);
        }
        // cos/sin of tpn (sx hx + sy ky) from the two tabulated phasors
        const double2 ex = tx[hk.x], ey = ty[hk.y + R];
        const double cs = ex.x * ey.x - ex.y * ey.y, sn = ex.y * ey.x + ex.x * ey.y;
        // the origin-shifted particle sample (img2d_FT_centshift.f90, b = -Im convention)
        const double2 pc = pcb[i];
        const double pr = pc.x * cs + pc.y * sn, pi = pc.x * sn - pc.y * cs;
        dot += pr * sr + pi * si;
        const double cw = pctf ? (double)pctf[(long)p * S + i] : 1.0;
        nb += cw * cw * (sr * sr + si * si);
    }
    dot = block_sum_double(dot, sh);
    nb = block_sum_double(nb, sh);
    if (threadIdx.x == 0) {
        double* o = part + (((long)p * k + c) * gridDim.z + sp) * 3;
        o[0] = dot;
        o[1] = 0.0;
        o[2] = nb;
    }
}

// CC of each (particle, candidate) from its chunks' sums, in chunk order.
// CC = dot / sqrt(|P|^2 |S|^2): the chunks' dot and section norms, the particle's FP64 norm
// (sum over the samples of |CTF P|^2, k_particle_norm; the origin phase keeps it)
__global__ void k_cc_fp64_finish(const double* __restrict__ part, int n, int ns, const double* __restrict__ pnorm,
                                 int k, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double dot = 0, nb = 0;
    for (int s = 0; s < ns; ++s) {
        dot += part[((long)i * ns + s) * 3];
        nb += part[((long)i * ns + s) * 3 + 2];
    }
    const double na = pnorm[i / k];
    out[i] = (na > 0 && nb > 0) ? dot / sqrt(na * nb) : 0.0;
}

// ---- FP8-e4m3 operands ---------------------------------------------------------
// Both operands are unit-norm rows whose elements span a wide range: low-frequency
// samples carry most of the norm, high-frequency ones little.  Each radial band b =
// int(|h|) of the samples gets a power-of-two scale 2^e_b on the B side (the sections)
// and 2^-e_b on the A side (the particles), so every product, hence every score, is
// unchanged, while each band of B uses the top of the e4m3 range (max 448).  A whole A
// row is further scaled by 2^f_p per particle (its origins share it), which scales all
// of that particle's scores alike and is removed from the reported CC.

__device__ __forceinline__ int sample_band(int2 hk) {
    return (int)sqrtf((float)(hk.x * hk.x + hk.y * hk.y));
}

// Largest |Re| or |Im| of B per band over every stride-th row (float bits, non-negative,
// so unsigned order is float order).
__global__ void k_band_absmax(const __nv_bfloat162* __restrict__ B, long n, int Kpad, const int2* __restrict__ samples,
                              int S, int nband, int stride, unsigned* __restrict__ out) {
    extern __shared__ unsigned smax[];
    for (int b = threadIdx.x; b < nband; b += blockDim.x) smax[b] = 0u;
    __syncthreads();
    for (long r = (long)blockIdx.x * stride; r < n; r += (long)gridDim.x * stride) {
        const __nv_bfloat162* row = B + r * (Kpad / 2);
        for (int i = threadIdx.x; i < S; i += blockDim.x) {
            const float2 v = __bfloat1622float2(row[bf16_pair_at(i, r)]);
            const float m = fmaxf(fabsf(v.x), fabsf(v.y));
            atomicMax(&smax[sample_band(samples[i])], __float_as_uint(m));
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nband; b += blockDim.x)
        if (smax[b]) atomicMax(&out[b], smax[b]);
}

// One CTA per row: B8[r] = e4m3(B[r] * mulB[sample]), zero padded to Kpad8 bytes.
__global__ void k_b_to_e4m3(const __nv_bfloat162* __restrict__ B, int Kpad, int S, const float* __restrict__ mulB,
                            int Kpad8, unsigned short* __restrict__ B8) {
    const long r = blockIdx.x;
    const __nv_bfloat162* row = B + r * (Kpad / 2);
    unsigned short* out = B8 + r * (Kpad8 / 2);
    for (int i = threadIdx.x; i < Kpad8 / 2; i += blockDim.x) {
        float2 v = make_float2(0.f, 0.f);
        if (i < S) {
            v = __bfloat1622float2(row[bf16_pair_at(i, r)]);
            v.x *= mulB[i];
            v.y *= mulB[i];
        }
        out[fp8_pair_at(i, r)] = __nv_cvt_float2_to_fp8x2(v, __NV_SATFINITE, __NV_E4M3);
    }
}

// Per particle: f_p = floor(log2(224 / max_i |A_i| mulA_i)) with |A_i| = |CTF P| / |A|.
__global__ void k_particle_exp8(const float2* __restrict__ band, const float* __restrict__ ctf, Band bd,
                                const int2* __restrict__ samples, int S, const double* __restrict__ norm,
                                const float* __restrict__ mulA, int* __restrict__ fexp) {
    __shared__ float sm[32];
    const int p = blockIdx.x, W = bd.W, R = bd.max_r;
    const float2* b = band + (long)p * W * W;
    const float* c = ctf ? ctf + (long)p * W * W : nullptr;
    const float inv = norm[p] > 0.0 ? (float)(1.0 / sqrt(norm[p])) : 0.0f;
    float m = 0.0f;
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        const int2 hk = samples[i];
        const int q = (hk.y + R) * W + (hk.x + R);
        const float a = sqrtf(b[q].x * b[q].x + b[q].y * b[q].y) * fabsf(c ? c[q] : 1.0f);
        m = fmaxf(m, a * inv * mulA[i]);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, sm[w]);
        m = fmaxf(m, sm[0]);
        fexp[p] = m > 0.0f ? (int)floorf(log2f(224.0f / m)) : 0;
    }
}

// Row (p, o) of A in e4m3: k_build_a's value x mulA[sample] x 2^f_p.
__global__ void __launch_bounds__(256) k_build_a8(const float2* __restrict__ band, const float* __restrict__ ctf,
                                                  Band bd, const int2* __restrict__ samples, int S, int Kpad8,
                                                  const float* __restrict__ origins, int O,
                                                  const float* __restrict__ poff,
                                                  const double* __restrict__ norm, const float* __restrict__ mulA,
                                                  const int* __restrict__ fexp, float two_pi_over_n,
                                                  unsigned short* __restrict__ A8) {
    extern __shared__ float2 ptab[];
    const int o = blockIdx.x, p = blockIdx.y, W = bd.W, R = bd.max_r;
    const float2* b = band + (long)p * W * W;
    const float* c = ctf ? ctf + (long)p * W * W : nullptr;
    const float h = (float)(bd.nx / 2);
    const float sx = origins[2 * o] + h + (poff ? poff[2 * p] : 0.0f);
    const float sy = origins[2 * o + 1] + h + (poff ? poff[2 * p + 1] : 0.0f);
    const float inv = norm[p] > 0.0 ? (float)(1.0 / sqrt(norm[p])) : 0.0f;
    const float pscale = ldexpf(1.0f, fexp[p]);
    unsigned short* row = A8 + ((long)p * O + o) * (Kpad8 / 2);
    origin_phasors(sx, sy, R, two_pi_over_n, ptab);
    for (int i = threadIdx.x; i < Kpad8 / 2; i += blockDim.x) {
        float re = 0.f, im = 0.f;
        if (i < S) {
            const int2 hk = samples[i];
            const int q = (hk.y + R) * W + (hk.x + R);
            const float2 ab = b[q];
            float sn, cs;
            phasor_at(ptab, R, hk, &sn, &cs);
            const float a2 = ab.x * cs + ab.y * sn, b2 = -ab.x * sn + ab.y * cs;
            const float cv = (c ? c[q] : 1.0f) * inv * mulA[i] * pscale;
            re = a2 * cv;
            im = -b2 * cv;
        }
        row[i] = __nv_cvt_float2_to_fp8x2(make_float2(re, im), __NV_SATFINITE, __NV_E4M3);
    }
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace

cudaError_t launch_band_absmax(const void* B, long n, int Kpad, const int2* samples, int S, int nband, int stride,
                               unsigned* out, int sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned) * nband, st);
    if (e != cudaSuccess) return e;
    long rows = (n + stride - 1) / stride;
    int grid = (int)(rows < 4L * sms ? rows : 4L * sms);
    k_band_absmax<<<grid, 256, sizeof(unsigned) * nband, st>>>((const __nv_bfloat162*)B, n, Kpad, samples, S, nband,
                                                               stride, out);
    return cudaGetLastError();
}

cudaError_t launch_b_to_e4m3(const void* B, long n, int Kpad, int S, const float* mulB, int Kpad8, void* B8,
                             cudaStream_t st) {
    for (long r0 = 0; r0 < n; r0 += 1L << 30) {
        long nb = n - r0 < (1L << 30) ? n - r0 : (1L << 30);
        k_b_to_e4m3<<<(unsigned)nb, 256, 0, st>>>((const __nv_bfloat162*)B + r0 * (Kpad / 2), Kpad, S, mulB, Kpad8,
                                                  (unsigned short*)B8 + r0 * (Kpad8 / 2));
    }
    return cudaGetLastError();
}

void launch_build_a8(const float2* band, const float* ctf, Band bd, const int2* samples, int S, int Kpad8,
                     const float* origins, int O, const double* norm, const float* mulA, int* fexp, int B, void* A8,
                     cudaStream_t st, const float* poff) {
    k_particle_exp8<<<B, 256, 0, st>>>(band, ctf, bd, samples, S, norm, mulA, fexp);
    dim3 g(O, B);
    const float tpn = 2.0f * host_angles().pi / (float)bd.nx;
    k_build_a8<<<g, 256, sizeof(float2) * (3 * bd.max_r + 2), st>>>(band, ctf, bd, samples, S, Kpad8, origins, O,
                                                                     poff, norm, mulA, fexp, tpn,
                                  (unsigned short*)A8);
}

void launch_map_checker(const float* map, int nx, float2* work, cudaStream_t st) {
    const long n3 = (long)nx * nx * nx;
    k_map_checker<<<cdiv(n3, 256) < 65535 ? cdiv(n3, 256) : 65535, 256, 0, st>>>(map, nx, work);
}

void launch_map_band(const float2* ft, int nx, int R, float2* cube, cudaStream_t st) {
    const long c3 = (long)(2 * R + 3) * (2 * R + 3) * (2 * R + 3);
    k_map_band<<<cdiv(c3, 256) < 65535 ? cdiv(c3, 256) : 65535, 256, 0, st>>>(ft, nx, R, cube);
}

// The band cube ((2R+3)^3 float2, x fastest) as a 3D array behind a linear-filtering
// texture (unnormalised coordinates, zero border).  Release with free_cube_texture.
cudaError_t make_cube_texture(const float2* cube, int R, cudaStream_t st, cudaArray_t* arr,
                              cudaTextureObject_t* tex) {
    const int C = 2 * R + 3;
    cudaChannelFormatDesc fd = cudaCreateChannelDesc<float2>();
    cudaError_t e = cudaMalloc3DArray(arr, &fd, make_cudaExtent(C, C, C));
    if (e != cudaSuccess) return e;
    cudaMemcpy3DParms cp{};
    cp.srcPtr = make_cudaPitchedPtr(const_cast<float2*>(cube), (size_t)C * sizeof(float2), C, C);
    cp.dstArray = *arr;
    cp.extent = make_cudaExtent(C, C, C);
    cp.kind = cudaMemcpyDeviceToDevice;
    if ((e = cudaMemcpy3DAsync(&cp, st)) != cudaSuccess) return e;
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = *arr;
    cudaTextureDesc td{};
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    return cudaCreateTextureObject(tex, &rd, &td, nullptr);
}

void free_cube_texture(cudaArray_t arr, cudaTextureObject_t tex) {
    if (tex) cudaDestroyTextureObject(tex);
    if (arr) cudaFreeArray(arr);
}

constexpr int SLICE_THREADS = 256;  // threads per section row
cudaError_t launch_slice_bf16(cudaTextureObject_t cube, int R, const int2* samples, int S, int Kpad,
                              const float* views, int nom, float step, long n0, long count, void* B,
                              cudaStream_t st, const float2* lin, float sigma, float sc) {
    const float gk = (lin && sigma > 0.0f) ? 1.0f / (2.0f * sigma * sigma) : 0.0f;
    size_t sm = (size_t)S * sizeof(float2);
    cudaError_t e = cudaFuncSetAttribute(k_slice_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    for (long c0 = 0; c0 < count; c0 += 65535) {
        long nb = count - c0 < 65535 ? count - c0 : 65535;
        k_slice_bf16<<<(unsigned)nb, SLICE_THREADS, sm, st>>>(cube, R, samples, S, Kpad, views, nom, step,
                                                   host_angles().deg2rad, n0 + c0,
                                                   (__nv_bfloat162*)B + c0 * (Kpad / 2), lin, gk, sc);
    }
    return cudaGetLastError();
}

// a local grid's rows are short (a few thousand samples at sub-particle sizes): fewer
// threads per row keep the per-row norm reduction from dominating
constexpr int LOCAL_SLICE_THREADS = 64;
cudaError_t launch_slice_bf16_local(cudaTextureObject_t cube, int R, const int2* samples, int S, int Kpad,
                                    const float* centre, int m, float step, long count, void* B, cudaStream_t st,
                                    const float2* lin, float sigma, long lpitch, const float* pctf, float sc) {
    if (lpitch <= 0) lpitch = (long)(2 * m + 1) * (2 * m + 1) * (2 * m + 1);
    const float gk = (lin && sigma > 0.0f) ? 1.0f / (2.0f * sigma * sigma) : 0.0f;
    const long n = 2L * m + 1;
    if (Kpad / 2 <= LSR_THREADS * LSR_SPT && count % lpitch == 0 && n * n <= 65535 && count / lpitch <= 65535) {
        // the whole grid of each of count / lpitch particles: rows by (p, i, j) lines of omegas
        dim3 grid((unsigned)(n * n), (unsigned)(count / lpitch));
        k_slice_bf16_local_rows<<<grid, LSR_THREADS, sizeof(float) * 9 * (size_t)n, st>>>(
            cube, R, samples, S, Kpad, centre, m, step, host_angles().deg2rad, (__nv_bfloat162*)B, lin, gk, lpitch,
            pctf, sc);
        return cudaGetLastError();
    }
    size_t sm = (size_t)S * sizeof(float2);
    cudaError_t e =
        cudaFuncSetAttribute(k_slice_bf16_local, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    for (long c0 = 0; c0 < count; c0 += 65535) {
        long nb = count - c0 < 65535 ? count - c0 : 65535;
        k_slice_bf16_local<<<(unsigned)nb, LOCAL_SLICE_THREADS, sm, st>>>(cube, R, samples, S, Kpad, centre, m, step,
                                                         host_angles().deg2rad, c0,
                                                         (__nv_bfloat162*)B + c0 * (Kpad / 2), lin, gk, lpitch,
                                                         pctf, sc);
    }
    return cudaGetLastError();
}

void launch_particle_norm(const float2* band, const float* ctf, Band bd, const int2* samples, int S,
                          int B, double* norm, cudaStream_t st, double2* pc, double* norm0, float* pctf) {
    k_particle_norm<<<B, 256, 0, st>>>(band, ctf, bd, samples, S, norm, pc, norm0, pctf);
}

void launch_build_a(const float2* band, const float* ctf, Band bd, const int2* samples, int S, int Kpad,
                    const float* origins, int O, const double* norm, int B, void* A, cudaStream_t st,
                    const float* poff) {
    const float tpn = 2.0f * host_angles().pi / (float)bd.nx;
    dim3 ga((O + AO - 1) / AO, B);
    const int sm = (int)(sizeof(float2) * AO * (3 * bd.max_r + 2));
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_build_a, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    k_build_a<<<ga, 256, sm, st>>>(band, ctf, bd, samples, S, Kpad, origins, O, poff, norm, tpn,
                                   (__nv_bfloat162*)A);
}

void launch_select_topk(const float* topv, const int* topi, int O, int ntiles, int k, int B,
                        float* tile_v, int* tile_o, int* tile_orig, int* orient, int* origin, float* cc,
                        cudaStream_t st) {
    dim3 g(ntiles, B);
    k_tile_best<<<g, 256, 0, st>>>(topv, topi, O, ntiles, tile_v, tile_o, tile_orig);
    k_select_topk<<<B, 512, 0, st>>>(tile_v, tile_o, tile_orig, ntiles, k, orient, origin, cc);
}

void launch_select_distinct(float* topv, const int* topi, int O, const int2* seg, int B, int k, int* col,
                            int* origin, float* cc, cudaStream_t st) {
    k_select_distinct<<<B, 512, 0, st>>>(topv, topi, O, seg, k, col, origin, cc);
}

long cc_fp64_scratch(int k, int B) { return (long)k * B * CC_SPLIT * 3; }

void launch_cc_fp64(const float2* cube, const double2* pcband, Band bd, const int2* samples, int S,
                    const float* cand, int k, int B, const double* pnorm, double* scratch, double* out,
                    cudaStream_t st, float sigma, const float* pctf, int cube_r, float sc) {
    dim3 g(k, B, CC_SPLIT);
    const size_t sm = sizeof(double2) * (3 * bd.max_r + 2);
    const double gk = sigma > 0.0f ? 1.0 / (2.0 * (double)sigma * (double)sigma) : 0.0;
    k_cc_fp64<<<g, 256, sm, st>>>(cube, pcband, bd, samples, S, cand, k, scratch, gk, pctf,
                                  cube_r < 0 ? bd.max_r : cube_r, (double)sc);
    k_cc_fp64_finish<<<(k * B + 127) / 128, 128, 0, st>>>(scratch, k * B, CC_SPLIT, pnorm, k, out);
}

}  // namespace cryoim
