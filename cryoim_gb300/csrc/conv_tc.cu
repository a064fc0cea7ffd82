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

template <int COUT>
__global__ void __launch_bounds__(CT_NT) k_conv3_tc(ConvTcArgs a) {
    constexpr int N = 3 * COUT;          // product columns (dt, co)
    constexpr int WB = N * 128;          // one dh block of the weight operand
    constexpr int NP = (N + 31) / 32 * 32;
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    unsigned char* sX = sm;                      // ring of 3 staged input rows
    unsigned char* sWt = sm + 3 * CT_ROW_BYTES;  // 3 dh blocks of N rows
    float* sEdge = (float*)(sWt + 3 * WB);       // [2][4 warps][COUT]
    uint64_t* bar = (uint64_t*)(sEdge + 8 * COUT);
    uint32_t* tslot = (uint32_t*)(bar + 1);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int Cin = a.Cin, H = a.H;
    const long q0 = (long)blockIdx.x * a.rows_per_cta;
    const long q1 = min((long)a.B * H, q0 + a.rows_per_cta);
    if (q0 >= q1) return;  // uniform over the block

    if (t == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot);
    // weights: block dh, row n = dt * COUT + co, element ci (zero beyond Cin)
    for (int i = t; i < 3 * N * 32; i += CT_NT) {
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

    // input row hh of sample b: thread t loads angle t's channels into registers (load),
    // rounds them to TF32 and writes them to a ring slot (put)
    float pre[32];
    const long cs = (long)H * CT_NT;
    auto load = [&](int b, int hh) {
        const bool ok = hh >= 0 && hh < H;
        const float* src = a.in + ((long)b * Cin * H + (ok ? hh : 0)) * CT_NT + t;
#pragma unroll
        for (int c = 0; c < 32; ++c) pre[c] = (ok && c < Cin) ? __ldg(src + c * cs) : 0.f;
    };
    auto put = [&](int slot) {
        unsigned char* dst = sX + slot * CT_ROW_BYTES + t * 128;
#pragma unroll
        for (int c4 = 0; c4 < 8; ++c4)
            *(float4*)(dst + ((c4 ^ (t & 7)) << 4)) = make_float4(tf32r(pre[4 * c4]), tf32r(pre[4 * c4 + 1]),
                                                                   tf32r(pre[4 * c4 + 2]), tf32r(pre[4 * c4 + 3]));
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
        if (t == 0) {
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
        float P[NP];
        const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll
        for (int c = 0; c < NP / 32; ++c) tc::tmem_ld32(trow + c * 32, P + c * 32);
        if (lane == 31) {
#pragma unroll
            for (int co = 0; co < COUT; ++co) sEdge[warp * COUT + co] = P[co];
        }
        if (lane == 0) {
#pragma unroll
            for (int co = 0; co < COUT; ++co) sEdge[(4 + warp) * COUT + co] = P[2 * COUT + co];
        }
        tc::fence_before();
        __syncthreads();
        const int wp = (warp + 3) & 3, wn = (warp + 1) & 3;
        float* orow = a.out + ((long)b * COUT * H + h) * CT_NT + t;
#pragma unroll
        for (int co = 0; co < COUT; ++co) {
            float lo = __shfl_up_sync(0xffffffffu, P[co], 1);
            float hi = __shfl_down_sync(0xffffffffu, P[2 * COUT + co], 1);
            if (lane == 0) lo = sEdge[wp * COUT + co];
            if (lane == 31) hi = sEdge[(4 + wn) * COUT + co];
            float v = lo + P[COUT + co] + hi;
            if (a.bias) v += __ldg(a.bias + co);
            if (a.relu) v = fmaxf(v, 0.f);
            orow[(long)co * H * CT_NT] = v;
        }
    }
    if (!ok && t == 0) tc::mbar_wait(bar, phase ^ 1u, a.err, false, CT_WAIT_NS);  // MMAs still in flight
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

template <int COUT>
__global__ void __launch_bounds__(CT_NT) k_conv3_wgrad_tc(ConvWgTcArgs a) {
    constexpr int M = 3 * COUT;
    extern __shared__ unsigned char smraw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    const int Cin = a.Cin, H = a.H;
    const WgGeom g = wg_geom(COUT, Cin);
    unsigned char* sA = sm;
    unsigned char* sB = sm + g.A_BYTES;
    uint64_t* bar = (uint64_t*)(sB + 3 * g.SLOT);
    uint32_t* tslot = (uint32_t*)(bar + 1);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const long q0 = (long)blockIdx.x * a.rows_per_cta;
    const long q1 = min((long)a.B * H, q0 + a.rows_per_cta);
    if (q0 >= q1) return;  // uniform over the block

    if (t == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot);
    // rows the MMAs read but whose products are unused start out as zeros
    for (int i = t; i < (g.A_BYTES + 3 * g.SLOT) / 16; i += CT_NT) ((float4*)sm)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_tf32(g.NB);

    float dbacc[COUT];
#pragma unroll
    for (int co = 0; co < COUT; ++co) dbacc[co] = 0.f;
    // dpre row h (preA: this thread's angle, every co) and input row hh (preB: every ci)
    // are loaded into registers a step ahead, then rounded and written to shared memory
    float preA[COUT], preB[32];
    const long cs = (long)H * CT_NT;
    auto loadA = [&](int b, int h) {
        const float* src = a.dpre + ((long)b * COUT * H + h) * CT_NT + t;
#pragma unroll
        for (int co = 0; co < COUT; ++co) preA[co] = __ldg(src + co * cs);
    };
    auto putA = [&]() {
#pragma unroll
        for (int co = 0; co < COUT; ++co) {
            dbacc[co] += preA[co];
            const float v = tf32r(preA[co]);
#pragma unroll
            for (int dt = 0; dt < 3; ++dt) {
                const int s = (t + dt - 1) & (CT_NT - 1), m = dt * COUT + co;
                *(float*)(sA + (s >> 5) * g.PA + tc::swz128_off4(m, s & 31)) = v;
            }
        }
    };
    auto loadB = [&](int b, int hh) {
        const bool ok = hh >= 0 && hh < H;
        const float* src = a.in + ((long)b * Cin * H + (ok ? hh : 0)) * CT_NT + t;
#pragma unroll
        for (int c = 0; c < 32; ++c) preB[c] = (ok && c < Cin) ? __ldg(src + c * cs) : 0.f;
    };
    auto putB = [&](int slot) {
        unsigned char* dst = sB + slot * g.SLOT + (t >> 5) * g.PB;
#pragma unroll
        for (int ci = 0; ci < 32; ++ci)
            if (ci < Cin) *(float*)(dst + tc::swz128_off4(ci, t & 31)) = tf32r(preB[ci]);
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
        if (t == 0) {
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
        float D[96];
        const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll
        for (int c = 0; c < 3; ++c) tc::tmem_ld32(trow + c * 32, D + c * 32);
        if (t < M) {
            const int dt = t / COUT, co = t - dt * COUT;
            for (int dh = 0; dh < 3; ++dh)
                for (int ci = 0; ci < Cin; ++ci)
                    atomicAdd(a.dW + ((co * Cin + ci) * 3 + dh) * 3 + dt, D[dh * 32 + ci]);
        }
#pragma unroll
        for (int co = 0; co < COUT; ++co) {
            float v = dbacc[co];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(a.db + co, v);
        }
    } else if (t == 0) {
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
        k_conv3_tc<32><<<grid, CT_NT, smem, st>>>(a);
    } else {
        constexpr int smem = conv_fwd_smem<16>();
        static bool set = false;
        if (!set) {
            if ((e = cudaFuncSetAttribute(k_conv3_tc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
                return e;
            set = true;
        }
        k_conv3_tc<16><<<grid, CT_NT, smem, st>>>(a);
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
        k_conv3_wgrad_tc<32><<<grid, CT_NT, smem, st>>>(a);
    } else {
        static bool set = false;
        if (!set) {
            if ((e = cudaFuncSetAttribute(k_conv3_wgrad_tc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax)))
                return e;
            set = true;
        }
        k_conv3_wgrad_tc<16><<<grid, CT_NT, smem, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace cryoim
