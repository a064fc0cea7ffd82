// conv_tc.cu — the learned proposer's 3x3 convolutions on the 5th-generation tensor
// cores: tcgen05.mma kind::tf32 (operands rounded to TF32, 10 mantissa bits, to nearest
// with ties away from zero, as they are staged in shared memory; FP32 accumulation in
// TMEM).  Activations keep the layout of learn.cu: [b][c][h][t] FP32, t = 128 angles
// (circular), h = radius (zero-padded).
//
// k_conv3_tc — forward, and data gradient with the flipped weights:
//   out[b][co][h][t] = bias[co] + sum_{ci,dh,dt} W[co][ci][dh][dt] in[b][ci][h+dh-1][t+dt-1].
//   Per output row (b, h) one product D[t][(dt, co)] = sum_{dh, ci} X_{h+dh-1}[t][ci] Wd[(dt, co)][ci]
//   (M = 128 angles, N = 3 Cout, K = 3 blocks of 32 channels, zero-padded), and the angle
//   offset of the kernel's three columns is applied to the product's rows afterwards:
//   out[t][co] = D[t-1][(0, co)] + D[t][(1, co)] + D[t+1][(2, co)] (lane shuffles across
//   the 128 TMEM lanes).  Each input row is therefore staged once, unshifted, and serves
//   three consecutive output rows from a ring of three.
// k_conv3_wgrad_tc — weight and bias gradients:
//   dW[co][ci][dh][dt] = sum_{b,h,s} dpre[b][co][h][s-dt+1] in[b][ci][h+dh-1][s].
//   Per (b, h): D[(dt, co)][(dh, ci)] += sum_s Pd[(dt, co)][s] X_{h+dh-1}[ci][s] (K = 128
//   angles), accumulated in TMEM over all rows of the block; the angle offset is applied
//   while dpre is staged.  One atomic add per weight per block at the end.
//
// 128 threads per block (the 128 TMEM lanes); thread t stages angle t.  Operands use the
// K-major 128-byte-swizzled layout (tc.cuh).  Waits are bounded (1 s); a timeout sets
// *err, every thread of the block leaves together, the outstanding MMAs are waited for
// (bounded) and TMEM is freed.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"
#include "tc.cuh"

namespace cryoim {
namespace {

constexpr int CT_NT = 128;               // angles = threads = product rows
constexpr int CT_TMEM_COLS = 128;
constexpr unsigned long long CT_WAIT_NS = 1000000000ull;
constexpr int CT_ROW_BYTES = CT_NT * 128;  // one staged input row: 128 angles x 32 channels x 4 B

__device__ __forceinline__ float tf32r(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// instruction descriptor of kind::tf32: D = F32 (bits 4-5 = 1), A and B = TF32 (2 at bits
// 7-9 and 10-12), both K-major, N >> 3 at bits 17-22, M = 128 (M >> 4 at bits 24-28)
__host__ __device__ constexpr uint32_t idesc_tf32(int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::su32(slot)),
                 "r"(CT_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t tmem) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(CT_TMEM_COLS)
                 : "memory");
}

struct ConvTcArgs {
    const float* in;    // [B][Cin][H][128]
    const float* W;     // [Cout][Cin][3][3]
    const float* bias;  // [Cout] or null
    float* out;         // [B][Cout][H][128]
    int B, Cin, H, relu, rows_per_cta;
    int* err;
};

template <int COUT>
constexpr int conv_fwd_smem() {
    return 1024 + 3 * CT_ROW_BYTES + 3 * (3 * COUT * 128) + 8 * COUT * 4 + 64;
}

// 256 threads: warps w and w + 4 share TMEM lanes 32 (w & 3) .. + 31 (angle t); the
// half h = w >> 2 stages channels 16 h .. 16 h + 15 of angle t and writes the output
// channels co of its half (COUT / 2 of them) in the epilogue.
constexpr int CT_FWD_THREADS = 256;

template <int COUT>
__global__ void __launch_bounds__(CT_FWD_THREADS, 2) k_conv3_tc(ConvTcArgs a) {
    constexpr int N = 3 * COUT;          // product columns (dt, co)
    constexpr int WB = N * 128;          // one dh block of the weight operand
    constexpr int CH = COUT / 2;         // output channels per half
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    unsigned char* sX = sm;                      // ring of 3 staged input rows
    unsigned char* sWt = sm + 3 * CT_ROW_BYTES;  // 3 dh blocks of N rows
    float* sEdge = (float*)(sWt + 3 * WB);       // [2][4 lane quarters][COUT]
    uint64_t* bar = (uint64_t*)(sEdge + 8 * COUT);
    uint32_t* tslot = (uint32_t*)(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, half = warp >> 2;
    const int t = 32 * quarter + lane;  // the angle (product row, TMEM lane) of this thread
    const int Cin = a.Cin, H = a.H;
    const long q0 = (long)blockIdx.x * a.rows_per_cta;
    const long q1 = min((long)a.B * H, q0 + a.rows_per_cta);
    if (q0 >= q1) return;  // uniform over the block

    if (tid == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot);
    // weights: block dh, row n = dt * COUT + co, element ci (zero beyond Cin)
    for (int i = tid; i < 3 * N * 32; i += CT_FWD_THREADS) {
        const int dh = i / (N * 32), rem = i - dh * N * 32, n = rem >> 5, ci = rem & 31;
        const int dt = n / COUT, co = n - dt * COUT;
        const float v = ci < Cin ? tf32r(__ldg(a.W + ((co * Cin + ci) * 3 + dh) * 3 + dt)) : 0.f;
        *(float*)(sWt + dh * WB + tc::swz128_off4(n, ci)) = v;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    constexpr uint32_t idesc = idesc_tf32(N);

    // input row hh of sample b: this thread loads channels 16 half .. + 15 of angle t into
    // registers (load), rounds them to TF32 and writes them to a ring slot (put)
    float pre[16];
    const long cs = (long)H * CT_NT;
    const int c0 = 16 * half;
    auto load = [&](int b, int hh) {
        const bool ok = hh >= 0 && hh < H;
        const float* src = a.in + ((long)b * Cin * H + (ok ? hh : 0)) * CT_NT + t;
#pragma unroll
        for (int c = 0; c < 16; ++c) pre[c] = (ok && c0 + c < Cin) ? __ldg(src + (c0 + c) * cs) : 0.f;
    };
    auto put = [&](int slot) {
        unsigned char* dst = sX + slot * CT_ROW_BYTES + t * 128;
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4) {
            const int c4 = 4 * half + k4;
            *(float4*)(dst + ((c4 ^ (t & 7)) << 4)) = make_float4(tf32r(pre[4 * k4]), tf32r(pre[4 * k4 + 1]),
                                                                   tf32r(pre[4 * k4 + 2]), tf32r(pre[4 * k4 + 3]));
        }
    };

    uint32_t phase = 0;
    int cur_b = -1, prev_h = -2;
    bool ok = true, have = false;  // have: pre already holds the row this step stages
    for (long q = q0; q < q1; ++q) {
        const int b = (int)(q / H), h = (int)(q - (long)b * H);
        // ring slot of input row h' is (h' + 1) % 3
        if (b != cur_b || h != prev_h + 1) {
            load(b, h - 1);
            put(h % 3);
            load(b, h);
            put((h + 1) % 3);
            cur_b = b;
            have = false;
        }
        prev_h = h;
        if (!have) load(b, h + 1);
        put((h + 2) % 3);
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
#pragma unroll
            for (int dh = 0; dh < 3; ++dh) {
                const uint32_t xa = tc::su32(sX + ((h + dh) % 3) * CT_ROW_BYTES);
                const uint32_t wb = tc::su32(sWt + dh * WB);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    mma_tf32(tmem, tc::sdesc(xa + kk * 32), tc::sdesc(wb + kk * 32), idesc, (dh | kk) != 0);
            }
            tc::commit(bar);
        }
        // the row the next step stages is loaded while the MMAs and the epilogue run
        have = false;
        if (q + 1 < q1 && h + 1 < H) {
            load(b, h + 2);
            have = true;
        }
        const bool got = tc::mbar_wait(bar, phase, a.err, false, CT_WAIT_NS);
        phase ^= 1u;
        if (!__syncthreads_and(got)) {
            ok = false;
            break;
        }
        tc::fence_after();
        // this half's output channels co = CH half .. + CH - 1, each at dt = 0, 1, 2
        float P0[CH], P1[CH], P2[CH];
        const uint32_t tlane = tmem + ((uint32_t)(32 * quarter) << 16);
        if constexpr (CH == 16) {  // columns dt * 32 + 16 half .. + 15
            tc::tmem_ld16(tlane + 16 * half, P0);
            tc::tmem_ld16(tlane + 32 + 16 * half, P1);
            tc::tmem_ld16(tlane + 64 + 16 * half, P2);
        } else {  // columns dt * 16 .. + 15, of which this half takes 8 half .. + 7
            float tmp[16];
            tc::tmem_ld16(tlane, tmp);
#pragma unroll
            for (int c = 0; c < CH; ++c) P0[c] = half ? tmp[CH + c] : tmp[c];
            tc::tmem_ld16(tlane + 16, tmp);
#pragma unroll
            for (int c = 0; c < CH; ++c) P1[c] = half ? tmp[CH + c] : tmp[c];
            tc::tmem_ld16(tlane + 32, tmp);
#pragma unroll
            for (int c = 0; c < CH; ++c) P2[c] = half ? tmp[CH + c] : tmp[c];
        }
        if (lane == 31) {
#pragma unroll
            for (int c = 0; c < CH; ++c) sEdge[quarter * COUT + CH * half + c] = P0[c];
        }
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < CH; ++c) sEdge[(4 + quarter) * COUT + CH * half + c] = P2[c];
        }
        tc::fence_before();
        __syncthreads();
        const int qp = (quarter + 3) & 3, qn = (quarter + 1) & 3;
        float* orow = a.out + ((long)b * COUT * H + h) * CT_NT + t;
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            const int co = CH * half + c;
            float lo = __shfl_up_sync(0xffffffffu, P0[c], 1);
            float hi = __shfl_down_sync(0xffffffffu, P2[c], 1);
            if (lane == 0) lo = sEdge[qp * COUT + co];
            if (lane == 31) hi = sEdge[(4 + qn) * COUT + co];
            float v = lo + P1[c] + hi;
            if (a.bias) v += __ldg(a.bias + co);
            if (a.relu) v = fmaxf(v, 0.f);
            orow[(long)co * H * CT_NT] = v;
        }
    }
    if (!ok && tid == 0) tc::mbar_wait(bar, phase ^ 1u, a.err, false, CT_WAIT_NS);  // MMAs still in flight
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tmem_free(tmem);
    }
}

struct ConvWgTcArgs {
    const float* in;    // [B][Cin][H][128]
    const float* dpre;  // [B][Cout][H][128]
    float* dW;          // [Cout][Cin][3][3], accumulated
    float* db;          // [Cout], accumulated
    int B, Cin, H, rows_per_cta;
    int* err;
};

// Staged-operand geometry of the weight gradient.  A (dpre, rows (dt, co)): 4 planes of
// 32 angles; plane p starts at p * PA with PA = 3 Cout rows of 128 B, so the MMA's rows
// beyond 3 Cout read the next plane (their products are never used).  B (input rows,
// rows ci): 4 planes of PB = max(8, Cin) rows; the MMA reads NB = max(16, Cin) rows.
struct WgGeom {
    int PA, A_BYTES, PB, NB, SLOT;
};
__host__ __device__ inline WgGeom wg_geom(int cout, int cin) {
    WgGeom g;
    const int M = 3 * cout;
    g.PA = M * 128;
    g.A_BYTES = 4 * g.PA + (128 - M) * 128;
    const int rowsB = cin < 8 ? 8 : cin;
    g.NB = cin < 16 ? 16 : cin;
    g.PB = rowsB * 128;
    g.SLOT = 4 * g.PB + (g.NB - rowsB) * 128;
    return g;
}
inline int conv_wgrad_smem(int cout, int cin) {
    const WgGeom g = wg_geom(cout, cin);
    return 1024 + g.A_BYTES + 3 * g.SLOT + 64;
}

// 256 threads: warps w and w + 4 share TMEM lanes 32 (w & 3) .. + 31 (angle t when
// staging, product row (dt, co) in the epilogue); the half h = w >> 2 stages the output
// channels co of its half (dpre) and the input channels 16 h .. 16 h + 15, and adds the
// columns ci of its half to dW at the end.
template <int COUT>
__global__ void __launch_bounds__(CT_FWD_THREADS, 2) k_conv3_wgrad_tc(ConvWgTcArgs a) {
    constexpr int M = 3 * COUT;
    constexpr int CH = COUT / 2;  // dpre channels per half
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    const int Cin = a.Cin, H = a.H;
    const WgGeom g = wg_geom(COUT, Cin);
    unsigned char* sA = sm;
    unsigned char* sB = sm + g.A_BYTES;
    uint64_t* bar = (uint64_t*)(sB + 3 * g.SLOT);
    uint32_t* tslot = (uint32_t*)(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, half = warp >> 2;
    const int t = 32 * quarter + lane;
    const long q0 = (long)blockIdx.x * a.rows_per_cta;
    const long q1 = min((long)a.B * H, q0 + a.rows_per_cta);
    if (q0 >= q1) return;  // uniform over the block

    if (tid == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot);
    // rows the MMAs read but whose products are unused start out as zeros
    for (int i = tid; i < (g.A_BYTES + 3 * g.SLOT) / 16; i += CT_FWD_THREADS)
        ((float4*)sm)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_tf32(g.NB);

    float dbacc[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) dbacc[c] = 0.f;
    // dpre row h (preA: this thread's angle, this half's co) and input row hh (preB: this
    // half's ci) are loaded into registers a step ahead, then rounded and written to
    // shared memory
    float preA[CH], preB[16];
    const long cs = (long)H * CT_NT;
    const int co0 = CH * half, ci0 = 16 * half;
    auto loadA = [&](int b, int h) {
        const float* src = a.dpre + ((long)b * COUT * H + h) * CT_NT + t;
#pragma unroll
        for (int c = 0; c < CH; ++c) preA[c] = __ldg(src + (co0 + c) * cs);
    };
    auto putA = [&]() {
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            dbacc[c] += preA[c];
            const float v = tf32r(preA[c]);
#pragma unroll
            for (int dt = 0; dt < 3; ++dt) {
                const int s = (t + dt - 1) & (CT_NT - 1), m = dt * COUT + co0 + c;
                *(float*)(sA + (s >> 5) * g.PA + tc::swz128_off4(m, s & 31)) = v;
            }
        }
    };
    auto loadB = [&](int b, int hh) {
        const bool ok = hh >= 0 && hh < H;
        const float* src = a.in + ((long)b * Cin * H + (ok ? hh : 0)) * CT_NT + t;
#pragma unroll
        for (int c = 0; c < 16; ++c) preB[c] = (ok && ci0 + c < Cin) ? __ldg(src + (ci0 + c) * cs) : 0.f;
    };
    auto putB = [&](int slot) {
        unsigned char* dst = sB + slot * g.SLOT + (t >> 5) * g.PB;
#pragma unroll
        for (int c = 0; c < 16; ++c)
            if (ci0 + c < Cin) *(float*)(dst + tc::swz128_off4(ci0 + c, t & 31)) = tf32r(preB[c]);
    };

    uint32_t phase = 0;
    int cur_b = -1, prev_h = -2;
    bool ok = true, have = false;  // have: preA / preB already hold this step's rows
    for (long q = q0; q < q1; ++q) {
        const int b = (int)(q / H), h = (int)(q - (long)b * H);
        if (b != cur_b || h != prev_h + 1) {
            loadB(b, h - 1);
            putB(h % 3);
            loadB(b, h);
            putB((h + 1) % 3);
            cur_b = b;
            have = false;
        }
        prev_h = h;
        if (!have) {
            loadB(b, h + 1);
            loadA(b, h);
        }
        putB((h + 2) % 3);
        putA();
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
            const uint32_t a0 = tc::su32(sA);
            for (int dh = 0; dh < 3; ++dh) {
                const uint32_t xb = tc::su32(sB + ((h + dh) % 3) * g.SLOT);
#pragma unroll
                for (int kk = 0; kk < 16; ++kk) {
                    const int p = kk >> 2, off = (kk & 3) * 32;
                    mma_tf32(tmem + (uint32_t)(dh * 32), tc::sdesc(a0 + p * g.PA + off),
                             tc::sdesc(xb + p * g.PB + off), idesc, (q > q0 || kk > 0) ? 1u : 0u);
                }
            }
            tc::commit(bar);
        }
        // the next step's rows are loaded while the MMAs run
        have = false;
        if (q + 1 < q1 && h + 1 < H) {
            loadB(b, h + 2);
            loadA(b, h + 1);
            have = true;
        }
        const bool got = tc::mbar_wait(bar, phase, a.err, false, CT_WAIT_NS);
        phase ^= 1u;
        if (!__syncthreads_and(got)) {
            ok = false;
            break;
        }
        tc::fence_after();
    }
    if (ok) {
        // product row t = (dt, co); this half's columns dh * 32 + 16 half .. + 15 (ci)
        float D[48];
        const uint32_t tlane = tmem + ((uint32_t)(32 * quarter) << 16);
#pragma unroll
        for (int dh = 0; dh < 3; ++dh) tc::tmem_ld16(tlane + (uint32_t)(dh * 32 + 16 * half), D + 16 * dh);
        if (t < M) {
            const int dt = t / COUT, co = t - dt * COUT;
            for (int dh = 0; dh < 3; ++dh)
                for (int c = 0; c < 16 && ci0 + c < Cin; ++c)
                    atomicAdd(a.dW + ((co * Cin + ci0 + c) * 3 + dh) * 3 + dt, D[16 * dh + c]);
        }
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            float v = dbacc[c];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(a.db + co0 + c, v);
        }
    } else if (tid == 0) {
        tc::mbar_wait(bar, phase ^ 1u, a.err, false, CT_WAIT_NS);  // MMAs still in flight
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tmem_free(tmem);
    }
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            n = v;
        else
            return 1;
    }
    return n;
}

// rows per block so that about two blocks per SM run the layer
int rows_per_block(long rows) {
    const long target = 2L * sm_count();
    return (int)((rows + target - 1) / target);
}

}  // namespace

cudaError_t launch_lp_conv3_tc(const float* in, int B, int Cin, int H, const float* W, const float* bias, int Cout,
                               bool relu, float* out, int* err, cudaStream_t st) {
    if (B < 1 || H < 1 || Cin < 1 || Cin > 32 || (Cout != 16 && Cout != 32) || !err) return cudaErrorInvalidValue;
    ConvTcArgs a{in, W, bias, out, B, Cin, H, relu ? 1 : 0, 0, err};
    const long rows = (long)B * H;
    a.rows_per_cta = rows_per_block(rows);
    const int grid = (int)((rows + a.rows_per_cta - 1) / a.rows_per_cta);
    cudaError_t e;
    if (Cout == 32) {
        constexpr int smem = conv_fwd_smem<32>();
        static bool set = false;
        if (!set) {
            if ((e = cudaFuncSetAttribute(k_conv3_tc<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
                return e;
            set = true;
        }
        k_conv3_tc<32><<<grid, CT_FWD_THREADS, smem, st>>>(a);
    } else {
        constexpr int smem = conv_fwd_smem<16>();
        static bool set = false;
        if (!set) {
            if ((e = cudaFuncSetAttribute(k_conv3_tc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
                return e;
            set = true;
        }
        k_conv3_tc<16><<<grid, CT_FWD_THREADS, smem, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_lp_conv3_wgrad_tc(const float* in, const float* dpre, int B, int Cin, int H, int Cout, float* dW,
                                     float* db, int* err, cudaStream_t st) {
    if (B < 1 || H < 1 || !(Cin == 1 || (Cin % 8 == 0 && Cin <= 32)) || (Cout != 16 && Cout != 32) || !err)
        return cudaErrorInvalidValue;
    ConvWgTcArgs a{in, dpre, dW, db, B, Cin, H, 0, err};
    const long rows = (long)B * H;
    a.rows_per_cta = rows_per_block(rows);
    const int grid = (int)((rows + a.rows_per_cta - 1) / a.rows_per_cta);
    const int smem = conv_wgrad_smem(Cout, Cin);
    const int smax = conv_wgrad_smem(32, 32);
    cudaError_t e;
    if (Cout == 32) {
        static bool set = false;
        if (!set) {
            if ((e = cudaFuncSetAttribute(k_conv3_wgrad_tc<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax)))
                return e;
            set = true;
        }
        k_conv3_wgrad_tc<32><<<grid, CT_FWD_THREADS, smem, st>>>(a);
    } else {
        static bool set = false;
        if (!set) {
            if ((e = cudaFuncSetAttribute(k_conv3_wgrad_tc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax)))
                return e;
            set = true;
        }
        k_conv3_wgrad_tc<16><<<grid, CT_FWD_THREADS, smem, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace cryoim
