// learn.cu — the learned orientation proposer: a small rotation-equivariant CNN on each
// particle's polar power spectrum, trained on projections the library itself renders.
//
// Input: |F|^2 of the particle's band (the masked, unshifted transform the search uses)
// on a polar grid of LP_NR radii over [minR, maxR] x LP_NT angles over [0, 180 deg)
// (a power spectrum is point-symmetric, so half a turn holds all of it); log, then each
// radius normalised to zero mean and unit variance over angle, which removes the
// isotropic CTF envelope and the noise level.  An in-plane rotation of the particle is
// a circular shift along the angle axis, so every layer is circular in angle:
//   4 x conv 3x3 (circular in angle, zero-padded in radius) + ReLU, average pooling of
//   radius pairs after layers 2-4 (64 -> 8 radii);
//   a linear mix of (channel, radius) -> LP_CM channels per angle: g[b][c][t];
//   the head: one learned template T[v][c][t] per view v of a coarse view grid, scored
//   at every circular shift s, sc[b][v][s] = sum_{c,t} g[b][c][(t + s) % NT] T[v][c][t].
// A cell (v, s) names a view and an in-plane angle (and the angle + 180 deg).  Training
// minimises the cross entropy against a target spread over neighbouring views and
// shifts.  Everything is FP32 on the CUDA cores: the proposer costs a few ms per batch
// next to the contraction it feeds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "geom.cuh"
#include "kernels.h"

namespace cryoim {
namespace {

constexpr int NR = LP_NR, NT = LP_NT, CM = LP_CM;

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// block-wide sum / max (blockDim a multiple of 32, <= 1024); all threads get the result
__device__ float block_sum(float v, float* sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    float r = (l < nw) ? sh[l] : 0.0f;
    r = warp_sum(r);
    return r;
}
__device__ float block_max(float v, float* sh) {
    v = warp_max(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    float r = (l < nw) ? sh[l] : -3.0e38f;
    r = warp_max(r);
    return r;
}

// ---- training data: CTF, origin shift and noise on rendered projections ----------

// CTF (getCTF2d.f90 with defocus in um, Cs in mm, astigmatism angle in degrees) times
// exp(-2 pi i (hx ox + ky oy) / n) applied to v: the forward model of a particle at
// origin (ox, oy).  pp = (df1, df2, astig, ox, oy); volt <= 0: no CTF.
__device__ __forceinline__ float2 ctf_shift(float2 v, int hx, int ky, int nx, const float* pp, float apix,
                                            float volt, float cs, float ampwg) {
    const float pi = 3.14159265358979f;
    float ctf = 1.0f;
    if (volt > 0.0f) {
        const float lam = 0.387818f / sqrtf(volt * (1.0f + 0.978459e-3f * volt));
        float ph = atan2f((float)ky, (float)hx);
        if (ph < 0.0f) ph += 2.0f * pi;
        ph -= pp[2] * pi / 180.0f;
        const float c = cosf(ph), s = sinf(ph);
        const float df = (pp[0] * c * c + pp[1] * s * s) * 1.0e4f;
        const float res2 = (float)(hx * hx + ky * ky) / ((float)nx * apix * (float)nx * apix);
        const float chi = 2.0f * pi * (-cs * 1.0e7f * lam * lam * lam * res2 * res2 * 0.25f + df * lam * res2 * 0.5f);
        ctf = -(sqrtf(1.0f - ampwg * ampwg) * sinf(chi) + ampwg * cosf(chi));
    }
    float sn, cn;
    sincosf(-2.0f * pi * ((float)hx * pp[3] + (float)ky * pp[4]) / (float)nx, &sn, &cn);
    return make_float2(ctf * (v.x * cn - v.y * sn), ctf * (v.x * sn + v.y * cn));
}

// The map zero-padded to (2n)^3 (the map at [n/2, 3n/2) per axis) times (-1)^(x+y+z),
// as complex: its transform samples the map's at half-integer frequencies, so the
// trilinear slices below interpolate a twice-oversampled transform.
__global__ void k_pad_checker(const float* __restrict__ map, int n, float2* __restrict__ out) {
    const int m = 2 * n;
    const long total = (long)m * m * m;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
        const int x = (int)(q % m), y = (int)((q / m) % m), z = (int)(q / ((long)m * m));
        const int X = x - n / 2, Y = y - n / 2, Z = z - n / 2;
        float v = 0.0f;
        if (X >= 0 && X < n && Y >= 0 && Y < n && Z >= 0 && Z < n) v = map[((long)Z * n + Y) * n + X];
        out[q] = make_float2(((x + y + z) & 1) ? -v : v, 0.0f);
    }
}

// Transform of a rendered particle by the Fourier slice theorem: at centred frequency
// (hx, ky) with |h| <= R1, the band cube (texture, side 2 Rc + 3, phase at the map
// centre, scaled 1 / (scale n)^3) of the map padded scale times, sampled at
// scale R_euler (hx, ky, 0), times (scale n)^3 and (-1)^(hx + ky) (the phase moved to
// pixel 0, the convention of the forward transform of img * (-1)^(x+y)), then CTF and
// origin shift; zero outside.  Its inverse, times (-1)^(x+y) / n^2, is the real-space
// projection (k_project's geometry) low-passed at R1.
__global__ void k_render_section(cudaTextureObject_t cube, int Rc, int R1, int scale, int nx,
                                 const float* __restrict__ eul, const float* __restrict__ par, float apix, float volt,
                                 float cs, float ampwg, float d2r, float2* __restrict__ ft) {
    __shared__ float rot[9];
    const int b = blockIdx.y;
    if (threadIdx.x == 0) euler_mat(eul[3 * b], eul[3 * b + 1], eul[3 * b + 2], d2r, rot);
    __syncthreads();
    const long nn = (long)nx * nx;
    const float sn = (float)(scale * nx), n3 = sn * sn * sn, off = (float)(Rc + 1) + 0.5f, sc = (float)scale;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += (long)gridDim.x * blockDim.x) {
        const int hx = (int)(q % nx) - nx / 2, ky = (int)(q / nx) - nx / 2;
        float2 out = make_float2(0.f, 0.f);
        if (hx * hx + ky * ky <= R1 * R1) {
            const float fx = sc * (float)hx, fy = sc * (float)ky;
            const float x = rot[0] * fx + rot[1] * fy, y = rot[3] * fx + rot[4] * fy, z = rot[6] * fx + rot[7] * fy;
            float2 v = tex3D<float2>(cube, x + off, y + off, z + off);
            const float sg = ((hx + ky) & 1) ? -n3 : n3;
            v.x *= sg;
            v.y *= sg;
            out = ctf_shift(v, hx, ky, nx, par + 5 * b, apix, volt, cs, ampwg);
        }
        ft[(long)b * nn + q] = out;
    }
}

// Re(inverse) * (-1)^(x+y) / n^2 and its variance inside the disc r <= 0.4 n
__global__ void k_cplx_to_real(const float2* __restrict__ in, int nx, float* __restrict__ out,
                               float* __restrict__ var) {
    __shared__ float sh[32];
    const int b = blockIdx.x;
    const long nn = (long)nx * nx;
    const float inv = 1.0f / (float)nn, rr = 0.4f * (float)nx;
    float s1 = 0.f, s2 = 0.f, cnt = 0.f;
    for (long q = threadIdx.x; q < nn; q += blockDim.x) {
        const int x = (int)(q % nx), y = (int)(q / nx);
        float v = in[(long)b * nn + q].x * inv;
        if ((x + y) & 1) v = -v;
        out[(long)b * nn + q] = v;
        const float dx = (float)(x - nx / 2), dy = (float)(y - nx / 2);
        if (dx * dx + dy * dy <= rr * rr) { s1 += v; s2 += v * v; cnt += 1.0f; }
    }
    s1 = block_sum(s1, sh);
    s2 = block_sum(s2, sh);
    cnt = block_sum(cnt, sh);
    if (threadIdx.x == 0) {
        const float m = s1 / fmaxf(cnt, 1.0f);
        var[b] = fmaxf(s2 / fmaxf(cnt, 1.0f) - m * m, 0.0f);
    }
}

// counter-based normal deviates (splitmix64 -> two uniforms -> Box-Muller)
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__global__ void k_add_noise(float* __restrict__ img, int nx, const float* __restrict__ var, float snr,
                            unsigned long long seed) {
    const int b = blockIdx.y;
    const long nn = (long)nx * nx;
    const float sd = snr > 0.0f ? sqrtf(var[b] / snr) : 0.0f;
    if (sd == 0.0f) return;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += (long)gridDim.x * blockDim.x) {
        const uint64_t h = mix64(seed ^ mix64((uint64_t)b * (uint64_t)nn + (uint64_t)q));
        const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);
        const float u2 = (float)((h >> 16) & 0xFFFFFFull) * (1.0f / 16777216.0f);
        img[(long)b * nn + q] += sd * sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    }
}

// ---- features ------------------------------------------------------------------
// One block per particle: bilinear |F|^2 of the band at (n/2 + r cos a, n/2 + r sin a),
// log(P + 1e-6 mean P), then per radius (P - mean) / (std + 1e-6) over the angles.
__global__ void __launch_bounds__(256) k_features(const float2* __restrict__ band, Band bd,
                                                  float* __restrict__ feat) {
    __shared__ float s[NR * NT];
    __shared__ float sh[32];
    const int b = blockIdx.x, W = bd.W, nx = bd.nx;
    const float2* pb = band + (long)b * W * W;
    const float h = (float)(nx / 2);
    const float pi = 3.14159265358979f;
    float part = 0.f;
    for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) {
        const int ir = q / NT, it = q - ir * NT;
        const float r = (float)bd.min_r + (float)(bd.max_r - bd.min_r) * (float)ir / (float)(NR - 1);
        float sn, cn;
        sincosf(pi * (float)it / (float)NT, &sn, &cn);
        const float x = r * cn + h, y = r * sn + h;
        const int lx = (int)floorf(x), ly = (int)floorf(y);
        const float ax = x - (float)lx, ay = y - (float)ly;
        float p[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int tx = lx + (u & 1) - bd.off, ty = ly + (u >> 1) - bd.off;
            const float2 v = pb[(long)ty * W + tx];
            p[u] = v.x * v.x + v.y * v.y;
        }
        const float v = (1.f - ay) * ((1.f - ax) * p[0] + ax * p[1]) + ay * ((1.f - ax) * p[2] + ax * p[3]);
        s[q] = v;
        part += v;
    }
    const float mean = block_sum(part, sh) / (float)(NR * NT);
    __syncthreads();
    const float eps = 1.0e-6f * mean + 1.0e-30f;
    for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) s[q] = logf(s[q] + eps);
    __syncthreads();
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int ir = w; ir < NR; ir += nw) {
        float a = 0.f;
        for (int it = l; it < NT; it += 32) a += s[ir * NT + it];
        const float m = warp_sum(a) / (float)NT;
        float d = 0.f;
        for (int it = l; it < NT; it += 32) {
            const float e = s[ir * NT + it] - m;
            d += e * e;
        }
        const float inv = 1.0f / (sqrtf(warp_sum(d) / (float)NT) + 1.0e-6f);
        for (int it = l; it < NT; it += 32) feat[((long)b * NR + ir) * NT + it] = (s[ir * NT + it] - m) * inv;
    }
}

// ---- network layers --------------------------------------------------------------
// 3x3 convolution, circular in angle (NT = 128 = blockDim), zero-padded in radius:
// out[b][co][h][t] = bias[co] + sum_{ci,dh,dt} in[b][ci][h+dh-1][t+dt-1] W[co][ci][dh][dt],
// ReLU if relu.  Block (h tile of HT rows, co tile of CT, b).
template <int CT, int HT>
__global__ void __launch_bounds__(NT) k_conv3(const float* __restrict__ in, int Cin, int H,
                                             const float* __restrict__ Wt, const float* __restrict__ bias, int Cout,
                                             int relu, float* __restrict__ out) {
    __shared__ float sx[HT + 2][NT + 2];
    __shared__ float sw[CT * 9];
    const int t = threadIdx.x, h0 = blockIdx.x * HT, co0 = blockIdx.y * CT, b = blockIdx.z;
    float acc[CT][HT];
#pragma unroll
    for (int c = 0; c < CT; ++c)
#pragma unroll
        for (int r = 0; r < HT; ++r) acc[c][r] = 0.f;
    // the next input channel's rows (and halo) and weights are loaded into registers
    // while the current one is used from shared memory
    float px[HT + 2], ph[HT + 2], pw[2];
    auto fetch = [&](int ci) {
        const float* ip = in + ((long)b * Cin + ci) * H * NT;
#pragma unroll
        for (int r = 0; r < HT + 2; ++r) {
            const int hh = h0 + r - 1;
            const bool ok = hh >= 0 && hh < H;
            px[r] = ok ? ip[hh * NT + t] : 0.f;
            ph[r] = (ok && (t == 0 || t == NT - 1)) ? ip[hh * NT + (t == 0 ? NT - 1 : 0)] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int q = t + u * NT;
            pw[u] = q < CT * 9 ? Wt[((long)(co0 + q / 9) * Cin + ci) * 9 + q % 9] : 0.f;
        }
    };
    fetch(0);
    for (int ci = 0; ci < Cin; ++ci) {
        __syncthreads();
#pragma unroll
        for (int r = 0; r < HT + 2; ++r) {
            sx[r][t + 1] = px[r];
            if (t == 0) sx[r][0] = ph[r];
            if (t == NT - 1) sx[r][NT + 1] = ph[r];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
            if (t + u * NT < CT * 9) sw[t + u * NT] = pw[u];
        __syncthreads();
        if (ci + 1 < Cin) fetch(ci + 1);
        float x[HT + 2][3];
#pragma unroll
        for (int r = 0; r < HT + 2; ++r)
#pragma unroll
            for (int d = 0; d < 3; ++d) x[r][d] = sx[r][t + d];
#pragma unroll
        for (int c = 0; c < CT; ++c)
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float wv = sw[c * 9 + k];
#pragma unroll
                for (int r = 0; r < HT; ++r) acc[c][r] = fmaf(wv, x[r + k / 3][k % 3], acc[c][r]);
            }
    }
#pragma unroll
    for (int c = 0; c < CT; ++c) {
        const float bv = bias ? bias[co0 + c] : 0.f;
#pragma unroll
        for (int r = 0; r < HT; ++r) {
            float v = acc[c][r] + bv;
            if (relu) v = fmaxf(v, 0.f);
            out[(((long)b * Cout + co0 + c) * H + h0 + r) * NT + t] = v;
        }
    }
}

// Weight and bias gradients of k_conv3 from dpre (the gradient before the ReLU):
// dW[co][ci][dh][dt] += sum_{b,h,t} dpre[b][co][h][t] in[b][ci][h+dh-1][t+dt-1].
// Block (co tile, ci, b chunk); the 128 angle threads reduce, then one atomic each.
template <int CT>
__global__ void __launch_bounds__(NT) k_conv3_wgrad(const float* __restrict__ in, const float* __restrict__ dpre,
                                                   int B, int Cin, int H, int Cout, int bchunk,
                                                   float* __restrict__ dW, float* __restrict__ db) {
    __shared__ float red[4][CT * 10];
    const int t = threadIdx.x, co0 = blockIdx.x * CT, ci = blockIdx.y, b0 = blockIdx.z * bchunk;
    const int tm = (t + NT - 1) % NT, tp = (t + 1) % NT;
    float acc[CT][10];
#pragma unroll
    for (int c = 0; c < CT; ++c)
#pragma unroll
        for (int k = 0; k < 10; ++k) acc[c][k] = 0.f;
    for (int b = b0; b < min(B, b0 + bchunk); ++b) {
        const float* ip = in + ((long)b * Cin + ci) * H * NT;
        // rows h-1, h, h+1 at t-1, t, t+1, rolled down one row per step
        float x[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        x[2][0] = __ldg(ip + tm);
        x[2][1] = __ldg(ip + t);
        x[2][2] = __ldg(ip + tp);
        for (int h = 0; h < H; ++h) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                x[0][d] = x[1][d];
                x[1][d] = x[2][d];
            }
            const bool ok = h + 1 < H;
            x[2][0] = ok ? __ldg(ip + (h + 1) * NT + tm) : 0.f;
            x[2][1] = ok ? __ldg(ip + (h + 1) * NT + t) : 0.f;
            x[2][2] = ok ? __ldg(ip + (h + 1) * NT + tp) : 0.f;
#pragma unroll
            for (int c = 0; c < CT; ++c) {
                const float g = __ldg(dpre + (((long)b * Cout + co0 + c) * H + h) * NT + t);
#pragma unroll
                for (int k = 0; k < 9; ++k) acc[c][k] = fmaf(g, x[k / 3][k % 3], acc[c][k]);
                acc[c][9] += g;
            }
        }
    }
    const int w = t >> 5, l = t & 31;
#pragma unroll
    for (int c = 0; c < CT; ++c)
#pragma unroll
        for (int k = 0; k < 10; ++k) {
            const float v = warp_sum(acc[c][k]);
            if (l == 0) red[w][c * 10 + k] = v;
        }
    __syncthreads();
    for (int q = t; q < CT * 10; q += NT) {
        const float v = red[0][q] + red[1][q] + red[2][q] + red[3][q];
        const int c = q / 10, k = q % 10;
        if (k < 9) atomicAdd(dW + ((long)(co0 + c) * Cin + ci) * 9 + k, v);
        else if (ci == 0) atomicAdd(db + co0 + c, v);
    }
}

// dpre = dout where out > 0 (the ReLU gate), else 0, four elements per thread step
// (in place: dout and dpre may be the same buffer; n is a multiple of 4, the buffers 16-byte aligned)
__global__ void k_relu_grad(const float4* __restrict__ out, const float4* dout, long n4, float4* dpre) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long)gridDim.x * blockDim.x) {
        const float4 o = out[q], d = dout[q];
        dpre[q] = make_float4(o.x > 0.f ? d.x : 0.f, o.y > 0.f ? d.y : 0.f, o.z > 0.f ? d.z : 0.f,
                              o.w > 0.f ? d.w : 0.f);
    }
}

// Wf[ci][co][2-dh][2-dt] = W[co][ci][dh][dt]: the data gradient is a k_conv3 with Wf
__global__ void k_flip(const float* __restrict__ W, int Cout, int Cin, float* __restrict__ Wf) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= Cout * Cin * 9) return;
    const int k = q % 9, ci = (q / 9) % Cin, co = q / (9 * Cin);
    Wf[((long)ci * Cout + co) * 9 + (8 - k)] = W[q];
}

// average of radius pairs: p[b][c][h][t] = (a[..][2h][t] + a[..][2h+1][t]) / 2.  Output row
// (b, c, h) reads input rows 2(b, c, h) and 2(b, c, h) + 1, so no index is split; four
// angles per thread step (rows of NT floats, 16-byte aligned)
constexpr int NT4 = NT / 4;
__global__ void k_pool(const float4* __restrict__ a, long nout4, float4* __restrict__ p) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < nout4; q += (long)gridDim.x * blockDim.x) {
        const long row = q / NT4;
        const float4* src = a + row * (2 * NT4) + (q - row * NT4);
        const float4 u = src[0], v = src[NT4];
        p[q] = make_float4(0.5f * (u.x + v.x), 0.5f * (u.y + v.y), 0.5f * (u.z + v.z), 0.5f * (u.w + v.w));
    }
}
// gradient through the pooling and, given the pooled layer's ReLU output a (or none), its gate
__global__ void k_pool_grad(const float4* __restrict__ dp, long nout4, const float4* __restrict__ a,
                            float4* __restrict__ da) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < nout4; q += (long)gridDim.x * blockDim.x) {
        const long row = q / NT4;
        const long o = row * (2 * NT4) + (q - row * NT4);
        const float4 g = dp[q];
        const float4 v = make_float4(0.5f * g.x, 0.5f * g.y, 0.5f * g.z, 0.5f * g.w);
        if (!a) {
            da[o] = v;
            da[o + NT4] = v;
            continue;
        }
        const float4 u0 = a[o], u1 = a[o + NT4];
        da[o] = make_float4(u0.x > 0.f ? v.x : 0.f, u0.y > 0.f ? v.y : 0.f, u0.z > 0.f ? v.z : 0.f,
                            u0.w > 0.f ? v.w : 0.f);
        da[o + NT4] = make_float4(u1.x > 0.f ? v.x : 0.f, u1.y > 0.f ? v.y : 0.f, u1.z > 0.f ? v.z : 0.f,
                                  u1.w > 0.f ? v.w : 0.f);
    }
}

// g[b][o][t] = b5[o] + sum_k W5[o][k] x[b][k][t], K = LP_MIXK
__global__ void __launch_bounds__(NT) k_mix(const float* __restrict__ x, const float* __restrict__ W5,
                                           const float* __restrict__ b5, float* __restrict__ g) {
    __shared__ float sw[CM * LP_MIXK];
    const int b = blockIdx.x, t = threadIdx.x;
    for (int q = t; q < CM * LP_MIXK; q += NT) sw[q] = W5[q];
    __syncthreads();
    float acc[CM];
#pragma unroll
    for (int o = 0; o < CM; ++o) acc[o] = b5[o];
    for (int k = 0; k < LP_MIXK; ++k) {
        const float v = x[((long)b * LP_MIXK + k) * NT + t];
#pragma unroll
        for (int o = 0; o < CM; ++o) acc[o] = fmaf(sw[o * LP_MIXK + k], v, acc[o]);
    }
#pragma unroll
    for (int o = 0; o < CM; ++o) g[((long)b * CM + o) * NT + t] = acc[o];
}
// dx[b][k][t] = sum_o W5[o][k] dg[b][o][t]
__global__ void __launch_bounds__(NT) k_mix_dx(const float* __restrict__ dg, const float* __restrict__ W5,
                                              float* __restrict__ dx) {
    __shared__ float sw[CM * LP_MIXK];
    const int b = blockIdx.x, t = threadIdx.x;
    for (int q = t; q < CM * LP_MIXK; q += NT) sw[q] = W5[q];
    __syncthreads();
    float d[CM];
#pragma unroll
    for (int o = 0; o < CM; ++o) d[o] = dg[((long)b * CM + o) * NT + t];
    for (int k = 0; k < LP_MIXK; ++k) {
        float a = 0.f;
#pragma unroll
        for (int o = 0; o < CM; ++o) a = fmaf(sw[o * LP_MIXK + k], d[o], a);
        dx[((long)b * LP_MIXK + k) * NT + t] = a;
    }
}
// dW5[o][k] = sum_{b,t} dg[b][o][t] x[b][k][t]; db5[o] = sum dg (block k = 0 adds it)
__global__ void __launch_bounds__(256) k_mix_dw(const float* __restrict__ x, const float* __restrict__ dg, int B,
                                               float* __restrict__ dW5, float* __restrict__ db5) {
    __shared__ float sh[32];
    const int k = blockIdx.x;
    float acc[CM], accb[CM];
#pragma unroll
    for (int o = 0; o < CM; ++o) { acc[o] = 0.f; accb[o] = 0.f; }
    const int t = threadIdx.x % NT;  // blockDim is a multiple of NT
    for (long b = threadIdx.x / NT; b < B; b += blockDim.x / NT) {
        const float v = x[(b * LP_MIXK + k) * NT + t];
#pragma unroll
        for (int o = 0; o < CM; ++o) {
            const float d = dg[(b * CM + o) * NT + t];
            acc[o] = fmaf(d, v, acc[o]);
            accb[o] += d;
        }
    }
    for (int o = 0; o < CM; ++o) {
        const float s = block_sum(acc[o], sh);
        if (threadIdx.x == 0) dW5[o * LP_MIXK + k] = s;
        if (k == 0) {
            const float sb = block_sum(accb[o], sh);
            if (threadIdx.x == 0) db5[o] = sb;
        }
    }
}

// Head in the frequency domain.  With X^(f) = sum_t x(t) e^{-2 pi i f t / NT} (the real
// transform, f = 0 .. NT/2), the circular correlation sc(s) = sum_t g(t + s) T(t) has
// the transform G^(f) conj(T^(f)); its gradients are dT(t) <-> sum_b conj(D^(f)) G^(f)
// and dg(u) <-> sum_v D^(f) T^(f), D = the transform of dsc over s.  Transforms are
// 128-point sums against a twiddle table (NT^2 / 2 operations each, a few per particle
// and view), products over the NT / 2 + 1 frequencies.
constexpr int NF = NT / 2 + 1;
constexpr int DR = 8;  // rows per block step of the real transforms

__device__ __forceinline__ void twiddles(float2* tw) {
    for (int k = threadIdx.x; k < NT; k += blockDim.x) {
        float sn, cs;
        sincospif(2.0f * (float)k / (float)NT, &sn, &cs);
        tw[k] = make_float2(cs, sn);
    }
}

// X[r][f] = sum_t x[r][t] e^{-2 pi i f t / NT} for rows r < n; block of NT threads,
// rows in a grid-stride loop
__global__ void __launch_bounds__(NT) k_rdft(const float* __restrict__ x, long n, float2* __restrict__ X) {
    __shared__ float2 tw[NT];
    __shared__ float sx[DR][NT];
    twiddles(tw);
    for (long r0 = (long)blockIdx.x * DR; r0 < n; r0 += (long)gridDim.x * DR) {
        __syncthreads();
#pragma unroll
        for (int i = 0; i < DR; ++i) sx[i][threadIdx.x] = r0 + i < n ? x[(r0 + i) * NT + threadIdx.x] : 0.f;
        __syncthreads();
        const int f = threadIdx.x;
        if (f < NF) {
            float re[DR], im[DR];
#pragma unroll
            for (int i = 0; i < DR; ++i) re[i] = im[i] = 0.f;
            for (int t = 0; t < NT; ++t) {
                const float2 w = tw[(f * t) & (NT - 1)];
#pragma unroll
                for (int i = 0; i < DR; ++i) {
                    re[i] = fmaf(sx[i][t], w.x, re[i]);
                    im[i] = fmaf(-sx[i][t], w.y, im[i]);
                }
            }
#pragma unroll
            for (int i = 0; i < DR; ++i)
                if (r0 + i < n) X[(r0 + i) * NF + f] = make_float2(re[i], im[i]);
        }
    }
}

// x[r][t] = (1/NT) sum over all f of X e^{+2 pi i f t / NT} for Hermitian spectra given
// on f = 0 .. NT/2; beta: x = inverse + beta * x (0 or 1)
__global__ void __launch_bounds__(NT) k_irdft(const float2* __restrict__ X, long n, float* __restrict__ x) {
    __shared__ float2 tw[NT];
    __shared__ float2 sX[DR][NF];
    twiddles(tw);
    const float inv = 1.0f / (float)NT;
    for (long r0 = (long)blockIdx.x * DR; r0 < n; r0 += (long)gridDim.x * DR) {
        __syncthreads();
        if (threadIdx.x < NF) {
#pragma unroll
            for (int i = 0; i < DR; ++i)
                sX[i][threadIdx.x] = r0 + i < n ? X[(r0 + i) * NF + threadIdx.x] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        const int t = threadIdx.x;
        float acc[DR], a2[DR];
#pragma unroll
        for (int i = 0; i < DR; ++i) {
            acc[i] = sX[i][0].x + ((t & 1) ? -sX[i][NT / 2].x : sX[i][NT / 2].x);
            a2[i] = 0.f;
        }
        for (int f = 1; f < NT / 2; ++f) {
            const float2 w = tw[(f * t) & (NT - 1)];
#pragma unroll
            for (int i = 0; i < DR; ++i) {
                a2[i] = fmaf(sX[i][f].x, w.x, a2[i]);
                a2[i] = fmaf(-sX[i][f].y, w.y, a2[i]);
            }
        }
#pragma unroll
        for (int i = 0; i < DR; ++i)
            if (r0 + i < n) x[(r0 + i) * NT + t] = (acc[i] + 2.0f * a2[i]) * inv;
    }
}

// Xs[b][v][f] = sum_c G[b][c][f] conj(TT[v][c][f])
__global__ void k_head_prod(const float2* __restrict__ G, const float2* __restrict__ TT, int B, int V,
                            float2* __restrict__ Xs) {
    const long n = (long)B * V * NF;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int f = (int)(q % NF);
        const long bv = q / NF;
        const int v = (int)(bv % V), b = (int)(bv / V);
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int c = 0; c < CM; ++c) {
            const float2 g = G[((long)b * CM + c) * NF + f], t = TT[((long)v * CM + c) * NF + f];
            re = fmaf(g.x, t.x, fmaf(g.y, t.y, re));
            im = fmaf(g.y, t.x, fmaf(-g.x, t.y, im));
        }
        Xs[q] = make_float2(re, im);
    }
}

// dTT[v][c][f] = sum_b conj(D[b][v][f]) G[b][c][f]
__global__ void k_head_dTT(const float2* __restrict__ D, const float2* __restrict__ G, int B, int V,
                           float2* __restrict__ dTT) {
    const long n = (long)V * CM * NF;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int f = (int)(q % NF);
        const long vc = q / NF;
        const int c = (int)(vc % CM), v = (int)(vc / CM);
        float re = 0.f, im = 0.f;
        for (int b = 0; b < B; ++b) {
            const float2 d = D[((long)b * V + v) * NF + f], g = G[((long)b * CM + c) * NF + f];
            re = fmaf(d.x, g.x, fmaf(d.y, g.y, re));
            im = fmaf(d.x, g.y, fmaf(-d.y, g.x, im));
        }
        dTT[q] = make_float2(re, im);
    }
}

// dG[b][c][f] = sum_v D[b][v][f] TT[v][c][f]
__global__ void k_head_dG(const float2* __restrict__ D, const float2* __restrict__ TT, int B, int V,
                          float2* __restrict__ dG) {
    const long n = (long)B * CM * NF;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int f = (int)(q % NF);
        const long bc = q / NF;
        const int c = (int)(bc % CM), b = (int)(bc / CM);
        float re = 0.f, im = 0.f;
        for (int v = 0; v < V; ++v) {
            const float2 d = D[((long)b * V + v) * NF + f], t = TT[((long)v * CM + c) * NF + f];
            re = fmaf(d.x, t.x, fmaf(-d.y, t.y, re));
            im = fmaf(d.x, t.y, fmaf(d.y, t.x, im));
        }
        dG[q] = make_float2(re, im);
    }
}

// Soft-target cross entropy over the V x NT cells of each particle.  truth[b] = (view
// unit vector, shift); target(v, s) = exp(-(angle(v, v*) / sv)^2 - (d(s, s*) / ss)^2),
// normalised.  dsc = (softmax - target) / B; loss[b] = -sum target log softmax.
__global__ void __launch_bounds__(256) k_loss(const float* __restrict__ sc, int B, int V,
                                             const float* __restrict__ vview, const float* __restrict__ truth,
                                             float sv, float ss, float* __restrict__ dsc, float* __restrict__ loss) {
    __shared__ float sh[32];
    const int b = blockIdx.x;
    const long n = (long)V * NT;
    const float* x = sc + (long)b * n;
    const float* tr = truth + 4 * b;
    const float rad2deg = 57.29577951308232f;
    // the target's exponent -(av^2 + as^2) is taken relative to its largest value over the
    // cells (the normalised target is unchanged), so its sum is >= 1 even for a label far
    // from every view class (an orientation at an asymmetric-unit edge that no operator
    // folds inside in FP32)
    float mx = -3.0e38f, dmin = 3.0e38f;
    for (long q = threadIdx.x; q < n; q += blockDim.x) {
        mx = fmaxf(mx, x[q]);
        const int v = (int)(q / NT), s = (int)(q % NT);
        const float dot = vview[3 * v] * tr[0] + vview[3 * v + 1] * tr[1] + vview[3 * v + 2] * tr[2];
        const float av = acosf(fminf(fmaxf(dot, -1.f), 1.f)) * rad2deg / sv;
        int ds = abs(s - (int)tr[3]) % NT;
        ds = min(ds, NT - ds);
        const float as = (float)ds / ss;
        dmin = fminf(dmin, av * av + as * as);
    }
    mx = block_max(mx, sh);
    dmin = -block_max(-dmin, sh);
    float se = 0.f, st = 0.f, stx = 0.f;
    for (long q = threadIdx.x; q < n; q += blockDim.x) {
        const int v = (int)(q / NT), s = (int)(q % NT);
        se += expf(x[q] - mx);
        const float dot = vview[3 * v] * tr[0] + vview[3 * v + 1] * tr[1] + vview[3 * v + 2] * tr[2];
        const float av = acosf(fminf(fmaxf(dot, -1.f), 1.f)) * rad2deg / sv;
        int ds = abs(s - (int)tr[3]) % NT;
        ds = min(ds, NT - ds);
        const float as = (float)ds / ss;
        const float tg = expf(dmin - av * av - as * as);
        st += tg;
        stx += tg * (x[q] - mx);
    }
    se = block_sum(se, sh);
    st = block_sum(st, sh);
    stx = block_sum(stx, sh);
    const float lse = logf(se);
    if (threadIdx.x == 0) loss[b] = -(stx / st - lse);
    const float ist = 1.0f / st, ise = 1.0f / se, ib = 1.0f / (float)B;
    for (long q = threadIdx.x; q < n; q += blockDim.x) {
        const int v = (int)(q / NT), s = (int)(q % NT);
        const float dot = vview[3 * v] * tr[0] + vview[3 * v + 1] * tr[1] + vview[3 * v + 2] * tr[2];
        const float av = acosf(fminf(fmaxf(dot, -1.f), 1.f)) * rad2deg / sv;
        int ds = abs(s - (int)tr[3]) % NT;
        ds = min(ds, NT - ds);
        const float as = (float)ds / ss;
        const float tg = expf(dmin - av * av - as * as);
        dsc[(long)b * n + q] = (expf(x[q] - mx) * ise - tg * ist) * ib;
    }
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, long n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const float gq = g[q];
        const float mq = b1 * m[q] + (1.f - b1) * gq, vq = b2 * v[q] + (1.f - b2) * gq * gq;
        m[q] = mq;
        v[q] = vq;
        w[q] -= lr * (mq * c1) / (sqrtf(vq * c2) + eps);
    }
}

// The k best cells of each particle's V x NT scores (repeated block argmax; sc is
// scratch: taken cells are set to -inf).
__global__ void __launch_bounds__(512) k_topk_cells(float* __restrict__ sc, long n, int k, int* __restrict__ cell,
                                                   float* __restrict__ val) {
    __shared__ float sv[32];
    __shared__ long si[32];
    const int b = blockIdx.x;
    float* x = sc + (long)b * n;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = 0; r < k; ++r) {
        float bv = -3.0e38f;
        long bi = -1;
        for (long q = threadIdx.x; q < n; q += blockDim.x)
            if (x[q] > bv) { bv = x[q]; bi = q; }
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const long oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi >= 0 && (bi < 0 || oi < bi))) { bv = ov; bi = oi; }
        }
        if (l == 0) { sv[w] = bv; si[w] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            float v0 = sv[0];
            long i0 = si[0];
            for (int q = 1; q < nw; ++q)
                if (sv[q] > v0 || (sv[q] == v0 && si[q] >= 0 && (i0 < 0 || si[q] < i0))) { v0 = sv[q]; i0 = si[q]; }
            cell[b * k + r] = (int)i0;
            val[b * k + r] = v0;
            if (i0 >= 0) x[i0] = -3.0e38f;
        }
        __syncthreads();
    }
}

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }
inline int grid_for(long n, int tpb) {
    const long g = (n + tpb - 1) / tpb;
    return (int)(g < 65535L * 16 ? g : 65535L * 16);
}

}  // namespace

void launch_lp_pad_checker(const float* map, int n, float2* out, cudaStream_t st) {
    const long total = 8L * n * n * n;
    k_pad_checker<<<grid_for(total, 256), 256, 0, st>>>(map, n, out);
}
void launch_lp_render(cudaTextureObject_t cube, int Rc, int R1, int scale, int nx, const float* eul, const float* par,
                      int B, float apix, float volt, float cs, float ampwg, float d2r, float2* ft, cudaStream_t st) {
    dim3 g(cdiv((long)nx * nx, 256 * 4), B);
    k_render_section<<<g, 256, 0, st>>>(cube, Rc, R1, scale, nx, eul, par, apix, volt, cs, ampwg, d2r, ft);
}
void launch_lp_cplx_to_real(const float2* in, int nx, int B, float* out, float* var, cudaStream_t st) {
    k_cplx_to_real<<<B, 512, 0, st>>>(in, nx, out, var);
}
void launch_lp_add_noise(float* img, int nx, int B, const float* var, float snr, unsigned long long seed,
                         cudaStream_t st) {
    dim3 g(cdiv((long)nx * nx, 256 * 4), B);
    k_add_noise<<<g, 256, 0, st>>>(img, nx, var, snr, seed);
}
void launch_lp_features(const float2* band, const Band& bd, int B, float* feat, cudaStream_t st) {
    k_features<<<B, 256, 0, st>>>(band, bd, feat);
}
cudaError_t launch_lp_conv3(const float* in, int B, int Cin, int H, const float* W, const float* bias, int Cout,
                            bool relu, float* out, cudaStream_t st) {
    if (Cout % 16 || H % 4) return cudaErrorInvalidValue;
    dim3 g(H / 4, Cout / 16, B);
    k_conv3<16, 4><<<g, NT, 0, st>>>(in, Cin, H, W, bias, Cout, relu ? 1 : 0, out);
    return cudaGetLastError();
}
cudaError_t launch_lp_conv3_wgrad(const float* in, const float* dpre, int B, int Cin, int H, int Cout, float* dW,
                                  float* db, cudaStream_t st) {
    if (Cout % 8) return cudaErrorInvalidValue;
    const int bchunk = 8;
    dim3 g(Cout / 8, Cin, cdiv(B, bchunk));
    k_conv3_wgrad<8><<<g, NT, 0, st>>>(in, dpre, B, Cin, H, Cout, bchunk, dW, db);
    return cudaGetLastError();
}
void launch_lp_relu_grad(const float* out, const float* dout, long n, float* dpre, cudaStream_t st) {
    const long n4 = n / 4;  // n = B x C x NR x NT, a multiple of 4
    k_relu_grad<<<grid_for(n4, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(out),
                                                   reinterpret_cast<const float4*>(dout), n4,
                                                   reinterpret_cast<float4*>(dpre));
}
void launch_lp_flip(const float* W, int Cout, int Cin, float* Wf, cudaStream_t st) {
    k_flip<<<cdiv((long)Cout * Cin * 9, 256), 256, 0, st>>>(W, Cout, Cin, Wf);
}
void launch_lp_pool(const float* a, int B, int C, int Hout, float* p, cudaStream_t st) {
    const long n4 = (long)B * C * Hout * NT4;
    k_pool<<<grid_for(n4, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(a), n4, reinterpret_cast<float4*>(p));
}
void launch_lp_pool_grad(const float* dp, int B, int C, int Hout, const float* a, float* da, cudaStream_t st) {
    const long n4 = (long)B * C * Hout * NT4;
    k_pool_grad<<<grid_for(n4, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(dp), n4,
                                                   reinterpret_cast<const float4*>(a),
                                                   reinterpret_cast<float4*>(da));
}
void launch_lp_mix(const float* x, int B, const float* W5, const float* b5, float* g, cudaStream_t st) {
    k_mix<<<B, NT, 0, st>>>(x, W5, b5, g);
}
void launch_lp_mix_grad(const float* x, const float* dg, int B, const float* W5, float* dx, float* dW5, float* db5,
                        cudaStream_t st) {
    if (dx) k_mix_dx<<<B, NT, 0, st>>>(dg, W5, dx);
    k_mix_dw<<<LP_MIXK, 256, 0, st>>>(x, dg, B, dW5, db5);
}
long lp_head_scratch(int B, int V) { return (long)NF * (2L * B * CM + 2L * V * CM + 2L * B * V); }

// scratch (float2): G [B][CM][NF], TT [V][CM][NF], X [B][V][NF], then the backward's
// D [B][V][NF], dTT [V][CM][NF], dG [B][CM][NF] reuse the same layout
cudaError_t launch_lp_head(const float* g, const float* T, int B, int V, float* sc, float2* scratch, cudaStream_t st) {
    float2* G = scratch;
    float2* TT = G + (long)B * CM * NF;
    float2* X = TT + (long)V * CM * NF;
    const int gmax = 152 * 16;
    k_rdft<<<(int)std::min<long>(((long)B * CM + DR - 1) / DR, gmax), NT, 0, st>>>(g, (long)B * CM, G);
    k_rdft<<<(int)std::min<long>(((long)V * CM + DR - 1) / DR, gmax), NT, 0, st>>>(T, (long)V * CM, TT);
    k_head_prod<<<grid_for((long)B * V * NF, 256), 256, 0, st>>>(G, TT, B, V, X);
    k_irdft<<<(int)std::min<long>(((long)B * V + DR - 1) / DR, gmax), NT, 0, st>>>(X, (long)B * V, sc);
    return cudaGetLastError();
}
void launch_lp_head_grad(const float* g, const float* T, const float* dsc, int B, int V, float* dg, float* dT,
                         float2* scratch, cudaStream_t st) {
    // G and TT from the forward are still in the scratch
    float2* G = scratch;
    float2* TT = G + (long)B * CM * NF;
    float2* D = TT + (long)V * CM * NF;  // over X
    float2* dTT = D + (long)B * V * NF;
    float2* dG = dTT + (long)V * CM * NF;
    const int gmax = 152 * 16;
    k_rdft<<<(int)std::min<long>(((long)B * V + DR - 1) / DR, gmax), NT, 0, st>>>(dsc, (long)B * V, D);
    k_head_dTT<<<grid_for((long)V * CM * NF, 128), 128, 0, st>>>(D, G, B, V, dTT);
    k_head_dG<<<grid_for((long)B * CM * NF, 128), 128, 0, st>>>(D, TT, B, V, dG);
    k_irdft<<<(int)std::min<long>(((long)V * CM + DR - 1) / DR, gmax), NT, 0, st>>>(dTT, (long)V * CM, dT);
    k_irdft<<<(int)std::min<long>(((long)B * CM + DR - 1) / DR, gmax), NT, 0, st>>>(dG, (long)B * CM, dg);
}
void launch_lp_loss(const float* sc, int B, int V, const float* vview, const float* truth, float sv, float ss,
                    float* dsc, float* loss, cudaStream_t st) {
    k_loss<<<B, 256, 0, st>>>(sc, B, V, vview, truth, sv, ss, dsc, loss);
}
void launch_lp_adam(float* w, const float* g, float* m, float* v, long n, float lr, int step, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
    k_adam<<<grid_for(n, 256), 256, 0, st>>>(w, g, m, v, n, lr, b1, b2, 1.0e-8f, c1, c2);
}
void launch_lp_topk(float* sc, int B, int V, int k, int* cell, float* val, cudaStream_t st) {
    k_topk_cells<<<B, 512, 0, st>>>(sc, (long)V * NT, k, cell, val);
}

}  // namespace cryoim
