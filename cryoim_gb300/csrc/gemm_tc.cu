// gemm_tc.cu — BF16 x BF16 (or FP8-e4m3 x FP8-e4m3) -> FP32 contraction on the
// 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM, operands staged by
// TMA), with a fused per-tile argmax epilogue.  This is the dense cross-correlation of the
// projection-matching form: C[m, n] = sum_k A[m, k] B[n, k] with both operands K-major,
// where a row of A is one (particle, origin) and a row of B one orientation's central
// section.  The full C is never stored: each (row, 256-column tile) reduces to
// (max, argmax).
//
// Persistent kernel, one CTA per SM, 704 threads:
//   warp 0    : TMA producer (one lane) filling a 4-stage ring of 128-row A and 256-row
//               B tiles of 128 bytes per row (64 BF16 or 128 FP8 elements, 128-byte
//               swizzle), mbarrier full/empty handshakes (A only when B rows come by
//               index);
//   warp 1    : MMA issuer (one lane): 4 x tcgen05.mma (M128 N256, K16 BF16 / K32 FP8,
//               32 bytes of K each) per stage into one of two TMEM accumulators
//               (2 x 256 columns), tcgen05.commit frees the stage and, at the end of a
//               tile, signals the epilogue;
//   warps 2-5 : epilogue, one TMEM lane (= output row) per thread: tcgen05.ld 32
//               columns at a time, running max/argmax, then release the accumulator;
//   warps 6-21: with B rows by index (the proposal forms' rows, picked from the section
//               bank), 16 rows of each B tile each, copied with 16-byte cp.async.
// Tiles are visited m-fastest so consecutive CTAs share a B tile through L2.
// Every wait is bounded (2 s of %globaltimer); a timeout sets *err, the issuer drains
// its MMAs, the producer waits for its copies, and TMEM is freed before exit.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "../../include/cryoim.h"
#include "kernels.h"
#include "tc.cuh"

namespace cryoim {
namespace {

constexpr int GM = 128, GN = 256, GKB = 128, NSTAGE = 4;  // GKB: bytes of K per stage
constexpr int A_BYTES = GM * GKB, B_BYTES = GN * GKB;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int TMEM_COLS = 512;
constexpr int NWARP_CORE = 6, NWARP_B = 16;  // producer, issuer, 4 epilogue; B loaders (b_mode 2)
// B loaders: cp.async groups (stages) in flight before the oldest is waited for and
// signalled.  The signal of stage s follows the issue of stage s + B_LAG, which waits for
// the issuer to free that slot: NSTAGE - 2 leaves the issuer a stage of slack (NSTAGE - 1
// made it wait for every signal and ran the contraction at 0.19 of the peak, not 0.31)
constexpr int B_LAG = NSTAGE - 2;
constexpr int NTHREADS = 32 * (NWARP_CORE + NWARP_B);
constexpr unsigned long long WAIT_NS = 2000000000ull;
// ring, alignment slack, barriers (256 B), the current tile's B row table (b_mode 2)
constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + 1024 + 256 + GN * 8;

// instruction descriptors: D=F32 (bits 4-5), A and B formats at bits 7-9 and 10-12
// (kind::f16: BF16 = 1; kind::f8f6f4: E4M3 = 0), both K-major (bits 15, 16 = 0),
// N>>3 at bits 17-22, M>>4 at bits 24-28
constexpr uint32_t IDESC_BF16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(GN >> 3) << 17) |
                                ((uint32_t)(GM >> 4) << 24);
constexpr uint32_t IDESC_E4M3 = (1u << 4) | ((uint32_t)(GN >> 3) << 17) | ((uint32_t)(GM >> 4) << 24);

using tc::su32;
using tc::mbar_init;
using tc::mbar_expect_tx;
using tc::mbar_arrive;
using tc::sdesc;
using tc::tmem_ld32;
// Bounded wait with this kernel's limit (2 s, or the launch's own for the failure-path test).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t par, int* err, bool abort_on_err,
                                          unsigned long long wait_ns) {
    return tc::mbar_wait(b, par, err, abort_on_err, wait_ns ? wait_ns : WAIT_NS);
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int c0, int c1,
                                            uint64_t* b) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(su32(dst)),
        "l"((uint64_t)tm), "r"(c0), "r"(c1), "r"(su32(b))
        : "memory");
}
// 16-byte global -> shared copy through L2 (completes at this thread's next wait_group)
__device__ __forceinline__ void cp16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { tc::fence_before(); }
__device__ __forceinline__ void tc_fence_after() { tc::fence_after(); }
__device__ __forceinline__ void tc_commit(uint64_t* b) { tc::commit(b); }
template <bool F8>
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t bdesc, uint32_t acc) {
    if constexpr (F8) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(d),
            "l"(a), "l"(bdesc), "r"(IDESC_E4M3), "r"(acc)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
            "l"(a), "l"(bdesc), "r"(IDESC_BF16), "r"(acc)
            : "memory");
    }
}
// Tile t of the launch -> its product, tile coordinates and operand rows.
struct TileAt {
    int mt, nt, a_row, b_row, m_valid, n_valid, n_tiles, topv_off;
};
__device__ __forceinline__ TileAt tile_at(const GemmArgmaxArgs& g, int t) {
    TileAt r;
    if (!g.groups) {
        r.mt = t % g.m_tiles;
        r.nt = t / g.m_tiles;
        r.a_row = r.mt * GM;
        r.b_row = r.nt * GN;
        r.m_valid = g.m_valid;
        r.n_valid = g.n_valid;
        r.n_tiles = g.n_tiles;
        r.topv_off = 0;
        return r;
    }
    int q = 0;
    while (q + 1 < g.ngroups && __ldg(&g.groups[q + 1].tile_start) <= t) ++q;
    const GemmGroup* G = g.groups + q;
    const int local = t - __ldg(&G->tile_start), mtiles = __ldg(&G->m_tiles);
    r.mt = local % mtiles;
    r.nt = local / mtiles;
    r.a_row = __ldg(&G->a_row0) + r.mt * GM;
    r.b_row = __ldg(&G->b_row0) + r.nt * GN;
    r.m_valid = __ldg(&G->m_valid);
    r.n_valid = __ldg(&G->n_valid);
    r.n_tiles = __ldg(&G->n_tiles);
    r.topv_off = __ldg(&G->topv_off);
    return r;
}

// F8 = false: BF16 operands, 64 elements of K per stage; true: FP8-e4m3, 128 elements.
template <bool F8>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_gemm_argmax(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  GemmArgmaxArgs g) {
    constexpr int GK = F8 ? GKB : GKB / 2;  // K elements per stage
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = sm;
    unsigned char* sB = sm + NSTAGE * A_BYTES;
    uint64_t* bars = (uint64_t*)(sB + NSTAGE * B_BYTES);
    uint64_t* full = bars;
    uint64_t* empty = bars + NSTAGE;
    uint64_t* accf = bars + 2 * NSTAGE;
    uint64_t* acce = accf + 2;
    uint64_t* drain = acce + 2;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    // b_mode 2: per tile row, the byte offset of its bank row | the bank row's residue
    unsigned long long* srow = (unsigned long long*)((unsigned char*)bars + 256);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        // b_mode 2: a stage is full after the A copy's arrival (with its bytes) and each B
        // loader warp's arrival once its copies have landed
        for (int s = 0; s < NSTAGE; ++s) { mbar_init(full + s, g.b_mode == 2 ? 1 + NWARP_B : 1); mbar_init(empty + s, 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(accf + b, 1); mbar_init(acce + b, 128); }
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
        if (g.b_mode != 2) asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int total = g.groups ? g.total_tiles : g.m_tiles * g.n_tiles;

    if (warp >= NWARP_CORE) {
        // B rows by index (b_mode 2; idle otherwise): warp w of the NWARP_B loaders copies
        // tile rows 16 w .. 16 w + 15, lane: 16-byte chunk p = lane % 8 of rows
        // 16 w + 4 i + lane / 8 (a row's 128 bytes from 8 adjacent lanes), re-swizzled
        // from the bank row's residue to the tile row's.  A stage's copies are one
        // cp.async group; B_LAG groups stay in flight, then the oldest is waited for, made
        // visible to the tensor core (proxy fence) and its stage's full barrier receives
        // the warp's arrival.
        if (g.b_mode == 2) {
            const int wb = warp - NWARP_CORE, rq = lane >> 3, p = lane & 7;
            // this warp's rows of the current tile: byte offset of the bank row | its residue
            unsigned long long* soff = srow + (size_t)wb * (GN / NWARP_B);
            int s = 0, npend = 0;
            uint32_t ph = 0;
            auto signal_oldest = [&]() {
                tc::fence_proxy_async();
                __syncwarp();
                const int so = (s - npend + NSTAGE) % NSTAGE;
                if (lane == 0) mbar_arrive(full + so);
                --npend;
            };
            bool ok = true;
            for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
                const TileAt ta = tile_at(g, t);
                __syncwarp();  // the previous tile's copies are issued (they read soff)
                for (int j = lane; j < GN / NWARP_B; j += 32) {
                    const int jt = wb * (GN / NWARP_B) + j;
                    const int jj = ta.nt * GN + jt < ta.n_valid ? jt : -ta.nt * GN;  // padding: the group's first row
                    const long n = __ldg(g.b_index + ta.b_row + jj);
                    soff[j] = (unsigned long long)(n * g.b_row_bytes) | (unsigned long long)(n & 7);
                }
                __syncwarp();
                for (int kb = 0; kb < g.kblocks; ++kb) {
                    const bool okl = mbar_wait(empty + s, ph ^ 1u, g.err, true, g.wait_ns);
                    if (!__all_sync(0xffffffffu, okl)) { ok = false; break; }
                    const uint32_t sb = su32(sB + s * B_BYTES) + (uint32_t)(wb * (GN / NWARP_B) * 128);
                    const unsigned char* src0 = g.b_rows + (long)kb * GKB + p * 16;
#pragma unroll
                    for (int i = 0; i < GN / NWARP_B / 4; ++i) {
                        const int r = 4 * i + rq;  // row within this warp's 64 (same residue as in the tile)
                        const unsigned long long v = soff[r];
                        cp16(sb + r * 128 + ((p ^ (int)(v & 7) ^ (r & 7)) << 4), src0 + (v & ~15ull));
                    }
                    cp_commit();
                    if (++s == NSTAGE) { s = 0; ph ^= 1u; }
                    if (++npend > B_LAG) {
                        cp_wait<B_LAG>();
                        signal_oldest();
                    }
                }
            }
            // every copy lands (and every issued stage is signalled) before the CTA can exit
            cp_wait<0>();
            while (npend > 0) signal_oldest();
        }
    } else if (warp == 0) {
        if (lane == 0) {
            int s = 0;
            uint32_t ph = 0;
            uint32_t last_par[NSTAGE];
            bool used[NSTAGE];
            for (int i = 0; i < NSTAGE; ++i) { used[i] = false; last_par[i] = 0; }
            bool ok = true;
            for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
                const TileAt ta = tile_at(g, t);
                for (int kb = 0; kb < g.kblocks; ++kb) {
                    if (!mbar_wait(empty + s, ph ^ 1u, g.err, true, g.wait_ns)) { ok = false; break; }
                    if (g.withhold && blockIdx.x == 0 && t == 0 && kb == g.withhold - 1) {
                        // failure-path test: this stage is never loaded and its barrier never completes
                        if (++s == NSTAGE) { s = 0; ph ^= 1u; }
                        continue;
                    }
                    mbar_expect_tx(full + s, g.b_mode == 2 ? A_BYTES : STAGE_BYTES);
                    tma_load_2d(sA + s * A_BYTES, &tmA, kb * GK, ta.a_row, full + s);
                    if (g.b_mode != 2) tma_load_2d(sB + s * B_BYTES, &tmB, kb * GK, ta.b_row, full + s);
                    used[s] = true;
                    last_par[s] = ph;
                    if (++s == NSTAGE) { s = 0; ph ^= 1u; }
                }
            }
            // every issued copy lands before the CTA can exit
            for (int i = 0; i < NSTAGE; ++i)
                if (used[i]) mbar_wait(full + i, last_par[i], g.err, false, g.wait_ns);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int s = 0, lt = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < total && ok; t += gridDim.x, ++lt) {
                const int b = lt & 1;
                const uint32_t aph = (uint32_t)(lt >> 1) & 1u;
                if (!mbar_wait(acce + b, aph ^ 1u, g.err, true, g.wait_ns)) break;
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(b * GN);
                for (int kb = 0; kb < g.kblocks; ++kb) {
                    if (!mbar_wait(full + s, ph, g.err, true, g.wait_ns)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = su32(sA + s * A_BYTES), b0 = su32(sB + s * B_BYTES);
#pragma unroll
                    for (int kk = 0; kk < GKB / 32; ++kk)
                        tc_mma<F8>(d, sdesc(a0 + kk * 32), sdesc(b0 + kk * 32), (kb | kk) != 0);
                    tc_commit(empty + s);
                    if (++s == NSTAGE) { s = 0; ph ^= 1u; }
                }
                if (ok) tc_commit(accf + b);
            }
            // all issued MMAs complete before TMEM is released
            tc_commit(drain);
            mbar_wait(drain, 0, g.err, false, g.wait_ns);
        }
    } else if (warp >= 2) {
        const int q = warp & 3;
        const int row_in_tile = 32 * q + lane;
        int lt = 0;
        for (int t = blockIdx.x; t < total; t += gridDim.x, ++lt) {
            const int b = lt & 1;
            const uint32_t aph = (uint32_t)(lt >> 1) & 1u;
            if (!mbar_wait(accf + b, aph, g.err, true, g.wait_ns)) break;
            tc_fence_after();
            const TileAt ta = tile_at(g, t);
            const long row = (long)ta.mt * GM + row_in_tile;
            float best = -3.0e38f;
            int bi = -1;
            for (int c = 0; c < GN / 32; ++c) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * GN + c * 32), v);
                const int col0 = ta.nt * GN + c * 32;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int col = col0 + j;
                    if (col < ta.n_valid && v[j] > best) { best = v[j]; bi = col; }
                }
                if (g.cfull && row < ta.m_valid) {
                    for (int j = 0; j < 32; ++j)
                        if (col0 + j < ta.n_valid) g.cfull[row * g.ldc + col0 + j] = v[j];
                }
            }
            tc_fence_before();
            mbar_arrive(acce + b);
            if (row < ta.m_valid) {
                g.topv[ta.topv_off + row * ta.n_tiles + ta.nt] = best;
                g.topi[ta.topv_off + row * ta.n_tiles + ta.nt] = bi;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// rows x k elements (BF16, or FP8 as bytes), row-major (k contiguous), box = 128 bytes
// of k x box_rows, 128-byte swizzle
bool make_map(CUtensorMap* m, const void* base, long rows, int k, int box_rows, bool f8, bool swizzle = true) {
    auto fn = encode_fn();
    if (!fn) return false;
    const int esz = f8 ? 1 : 2;
    cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)k * esz};
    cuuint32_t box[2] = {(cuuint32_t)(GKB / esz), (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, f8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                    const_cast<void*>(base), dims, strides, box,
                    es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

int gemm_tile_n() { return GN; }
int gemm_tile_m() { return GM; }

cudaError_t launch_gemm_argmax(const void* a, const void* b, int M, int N, int K, bool f8,
                               const GemmArgmaxArgs& in, int num_sms, cudaStream_t st) {
    const int gk = f8 ? GKB : GKB / 2;
    if (K % gk != 0 || M < 1 || N < 1) return cudaErrorInvalidValue;
    if (((uintptr_t)a & 15) || ((uintptr_t)b & 15)) return cudaErrorInvalidValue;
    CUtensorMap ta, tb;
    if (!make_map(&ta, a, M, K, GM, f8) || !make_map(&tb, b, N, K, GN, f8, in.b_mode == 0))
        return cudaErrorInvalidValue;
    GemmArgmaxArgs g = in;
    g.m_tiles = (M + GM - 1) / GM;
    g.n_tiles = (N + GN - 1) / GN;
    g.kblocks = K / gk;
    g.m_valid = M;
    g.n_valid = N;
    auto kern = f8 ? k_gemm_argmax<true> : k_gemm_argmax<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    int total = g.m_tiles * g.n_tiles;
    int grid = total < num_sms ? total : num_sms;
    kern<<<grid, NTHREADS, SMEM_BYTES, st>>>(ta, tb, g);
    return cudaGetLastError();
}

cudaError_t launch_gemm_argmax_grouped(const void* a, long Mtot, const void* b, long Ntot, int K, bool f8,
                                       GemmGroup* hg, int ngroups, GemmGroup* dg, const GemmArgmaxArgs& in,
                                       int num_sms, cudaStream_t st) {
    const int gk = f8 ? GKB : GKB / 2;
    if (K % gk != 0 || Mtot < 1 || Ntot < 1 || ngroups < 1 || in.cfull) return cudaErrorInvalidValue;
    if (((uintptr_t)a & 15) || ((uintptr_t)b & 15)) return cudaErrorInvalidValue;
    long total = 0;
    for (int i = 0; i < ngroups; ++i) {
        GemmGroup& q = hg[i];
        if (q.m_valid < 1 || q.n_valid < 1 || q.a_row0 < 0 || q.b_row0 < 0 ||
            (long)q.a_row0 + q.m_valid > Mtot || (long)q.b_row0 + q.n_valid > Ntot)
            return cudaErrorInvalidValue;
        q.m_tiles = (q.m_valid + GM - 1) / GM;
        q.n_tiles = (q.n_valid + GN - 1) / GN;
        q.tile_start = (int)total;
        total += (long)q.m_tiles * q.n_tiles;
    }
    if (total > (1L << 30)) return cudaErrorInvalidValue;
    if (in.b_mode == 1)  // pre-swizzled rows: every group's tiles start at a multiple of 8 rows
        for (int i = 0; i < ngroups; ++i)
            if (hg[i].b_row0 % 8) return cudaErrorInvalidValue;
    // b_mode 2: b is the bank (in.b_rows), Ntot the length of the index list in.b_index
    if (in.b_mode == 2 && (!in.b_index || in.b_rows != b || ((uintptr_t)in.b_rows & 15) ||
                           in.b_row_bytes % 16 || in.b_row_bytes < (long)K * (f8 ? 1 : 2)))
        return cudaErrorInvalidValue;
    CUtensorMap ta, tb;
    if (!make_map(&ta, a, Mtot, K, GM, f8)) return cudaErrorInvalidValue;
    if (in.b_mode == 2)
        tb = ta;  // not read
    else if (!make_map(&tb, b, Ntot, K, GN, f8, in.b_mode == 0))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyAsync(dg, hg, sizeof(GemmGroup) * ngroups, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    GemmArgmaxArgs g = in;
    g.groups = dg;
    g.ngroups = ngroups;
    g.total_tiles = (int)total;
    g.kblocks = K / gk;
    auto kern = f8 ? k_gemm_argmax<true> : k_gemm_argmax<false>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    const int grid = total < num_sms ? (int)total : num_sms;
    kern<<<grid, NTHREADS, SMEM_BYTES, st>>>(ta, tb, g);
    return cudaGetLastError();
}

cudaError_t launch_gemm_bf16_argmax(const void* a, const void* b, int M, int N, int K,
                                    const GemmArgmaxArgs& in, int num_sms, cudaStream_t st) {
    return launch_gemm_argmax(a, b, M, N, K, false, in, num_sms, st);
}

}  // namespace cryoim

// Kernel-level test hook (device pointers): C = A B^T with per-(row, 256-column tile)
// max/argmax, optional full C.  d_err receives 1 if a pipeline wait timed out.
static int gemm_hook(const void* d_a, const void* d_b, int32_t M, int32_t N, int32_t K, float* d_topv,
                     int32_t* d_topi, float* d_c, int32_t* d_err, void* stream, bool f8, int withhold = 0,
                     unsigned long long wait_ns = 0) {
    const int kq = f8 ? 128 : 64;
    if (!d_a || !d_b || !d_topv || !d_topi || !d_err) return CRYOIM_ERR_ARG;
    if (M < 1 || N < 1 || K < kq || K % kq) return CRYOIM_ERR_SIZE;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return CRYOIM_ERR_CUDA;
    cryoim::GemmArgmaxArgs g{};
    g.topv = d_topv;
    g.topi = d_topi;
    g.cfull = d_c;
    g.ldc = N;
    g.err = d_err;
    g.withhold = withhold;
    g.wait_ns = wait_ns;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(d_err, 0, sizeof(int), st) != cudaSuccess) return CRYOIM_ERR_CUDA;
    cudaError_t e = cryoim::launch_gemm_argmax(d_a, d_b, M, N, K, f8, g, sms, st);
    return e == cudaSuccess ? CRYOIM_OK : CRYOIM_ERR_CUDA;
}

extern "C" int cryoim_gemm_bf16_argmax(const void* d_a, const void* d_b, int32_t M, int32_t N,
                                       int32_t K, float* d_topv, int32_t* d_topi, float* d_c,
                                       int32_t* d_err, void* stream) {
    return gemm_hook(d_a, d_b, M, N, K, d_topv, d_topi, d_c, d_err, stream, false);
}

extern "C" int cryoim_gemm_e4m3_argmax(const void* d_a, const void* d_b, int32_t M, int32_t N,
                                       int32_t K, float* d_topv, int32_t* d_topi, float* d_c,
                                       int32_t* d_err, void* stream) {
    return gemm_hook(d_a, d_b, M, N, K, d_topv, d_topi, d_c, d_err, stream, true);
}

// The failure path of the pipeline: CTA 0 leaves k-stage `stage` of its first tile
// unloaded and every wait gives up after wait_us microseconds; *d_err comes back 1, the
// kernel returns, its TMEM is released, and the next launch runs normally.
extern "C" int cryoim_gemm_bf16_argmax_withhold(const void* d_a, const void* d_b, int32_t M, int32_t N,
                                                int32_t K, float* d_topv, int32_t* d_topi, int32_t* d_err,
                                                int32_t stage, int32_t wait_us, void* stream) {
    if (stage < 0 || stage >= K / 64 || wait_us < 100 || wait_us > 2000000) return CRYOIM_ERR_ARG;
    return gemm_hook(d_a, d_b, M, N, K, d_topv, d_topi, nullptr, d_err, stream, false, stage + 1,
                     (unsigned long long)wait_us * 1000ull);
}
