// noalloc.cu — phase-residual scoring of refinement candidates with no device
// allocation (cryoim_prscore_noalloc).
//
// Some callers cannot allocate device memory at the moment they score: code running
// under a fixed memory budget owned by another allocator, or a host loop that must
// not touch the CUDA allocator between steps.  This entry point takes only caller-
// owned device buffers and keeps its intermediate results (candidate list, common-
// line angle table, template amplitude cuts, the 11 scores) in one file-scope
// __device__ array of fixed size, so it never calls cudaMalloc/cudaFree or an
// allocating library routine.
//
// The array lives for the lifetime of the process on every GPU that loads the
// library.  In host code its name is only a host-side stand-in, so the device address
// is looked up once per device with cudaGetSymbolAddress (first call on that device,
// which also copies the 60 symmetry operators into it) and passed to the kernels.  That
// address and table are kept for the life of the process, so the entry point must not
// be used across a cudaDeviceReset of the device.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/cryoim.h"
#include "kernels.h"

using namespace cryoim;

namespace {

constexpr int kMaxT = CRYOIM_NOALLOC_MAX_TEMPLATES;
constexpr int kMaxR = CRYOIM_NOALLOC_MAX_RADII;
// layout (floats): candidates 11x5 | scores 11 | operators 540 | template cuts T x nR |
//                  angle pairs 11 x T x 60 float2
constexpr long kCandOff = 0, kPrOff = 64, kOpsOff = 128, kCutOff = 128 + 544;
constexpr long kAlphaOff = kCutOff + (long)kMaxT * kMaxR;
constexpr long kScratchFloats = kAlphaOff + 2L * 11 * kMaxT * 60;

static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

std::mutex g_mu;
float* g_dev_ptr[64] = {nullptr};

// Status codes only: this entry point reports through its return value.
int set_error(int code, const char*) { return code; }

// Candidate list of 11 entries from the caller's K (pad with the last one).
__global__ void k_pad_candidates(const float* __restrict__ cand, int K, float* __restrict__ out) {
    int t = threadIdx.x;
    if (t < 55) {
        int c = t / 5, e = t % 5;
        int src = c < K ? c : K - 1;
        out[t] = cand[src * 5 + e];
    }
}

// Set-up on the current device: look up the array's device address and store the
// symmetry operators in it.  Returns the device address or nullptr.
float* scratch_for_current_device(int* err) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        *err = set_error(CRYOIM_ERR_CUDA, "no current CUDA device");
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_dev_ptr[dev]) return g_dev_ptr[dev];
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        *err = set_error(CRYOIM_ERR_CUDA, cudaGetErrorString(e));
        return nullptr;
    }
    float ops[540];
    cryoim_icos_ops(ops);
    e = cudaMemcpy((float*)p + kOpsOff, ops, sizeof(ops), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        *err = set_error(CRYOIM_ERR_CUDA, cudaGetErrorString(e));
        return nullptr;
    }
    g_dev_ptr[dev] = (float*)p;
    return g_dev_ptr[dev];
}

}  // namespace

extern "C" int cryoim_prscore_noalloc(int32_t nx, int32_t min_r, int32_t max_r,
                                      const float* d_band, const float* d_fcut0,
                                      const float* d_ctf_band, const float* d_tmpl_band,
                                      const float* d_tmpl_fcut, const float* d_tmpl_ort,
                                      int32_t T, const float* d_cand, int32_t K, float* d_pr,
                                      void* stream) {
    if (!d_band || !d_fcut0 || !d_tmpl_band || !d_tmpl_ort || !d_cand || !d_pr ||
        (!d_ctf_band && !d_tmpl_fcut))
        return set_error(CRYOIM_ERR_ARG, "cryoim_prscore_noalloc: null device pointer");
    if (nx < 8 || (nx & 1) || min_r < 0 || max_r < min_r || max_r > nx / 2 - 2)
        return set_error(CRYOIM_ERR_ARG, "cryoim_prscore_noalloc: bad nx/min_r/max_r");
    if (T < 1 || T > kMaxT)
        return set_error(CRYOIM_ERR_SIZE, "cryoim_prscore_noalloc: T must be 1..CRYOIM_NOALLOC_MAX_TEMPLATES");
    if (K < 1 || K > CRYOIM_NOALLOC_MAX_CANDIDATES)
        return set_error(CRYOIM_ERR_SIZE, "cryoim_prscore_noalloc: K must be 1..CRYOIM_NOALLOC_MAX_CANDIDATES");
    if (max_r - min_r + 1 > kMaxR)
        return set_error(CRYOIM_ERR_SIZE, "cryoim_prscore_noalloc: max_r-min_r+1 exceeds CRYOIM_NOALLOC_MAX_RADII");
    // errors left pending on this thread by earlier work are not this call's
    (void)cudaGetLastError();
    int err = CRYOIM_OK;
    float* s = scratch_for_current_device(&err);
    if (!s) return err;
    cudaStream_t st = (cudaStream_t)stream;
    const Band bd = make_band(nx, min_r, max_r);
    float* cand = s + kCandOff;
    float* pr = s + kPrOff;
    float* ops = s + kOpsOff;
    float* cuts = s + kCutOff;
    float2* alpha = reinterpret_cast<float2*>(s + kAlphaOff);
    // every scratch region below is fully rewritten by this call before it is read
    k_pad_candidates<<<1, 64, 0, st>>>(d_cand, K, cand);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        launch_refine_alpha(cand, 1, d_tmpl_ort, T, ops, alpha, st);
        e = cudaGetLastError();
    }
    const float* tfc = d_tmpl_fcut;
    if (e == cudaSuccess && d_ctf_band) {
        launch_tmpl_fcut(reinterpret_cast<const float2*>(d_tmpl_band), T, d_ctf_band, 1, bd, cuts, st);
        e = cudaGetLastError();
        tfc = cuts;
    }
    if (e != cudaSuccess) return set_error(CRYOIM_ERR_CUDA, cudaGetErrorString(e));
    PrSingleArgs a{};
    a.band = reinterpret_cast<const float2*>(d_band);
    a.fcut0 = d_fcut0;
    a.tband = reinterpret_cast<const float2*>(d_tmpl_band);
    a.tfcut = tfc;
    a.tfcut_pstride = 0;
    a.ctf = d_ctf_band;
    a.cand = cand;
    a.alpha = alpha;
    a.T = T;
    a.bd = bd;
    a.pr = pr;
    e = launch_pr_single(a, 1, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_pr, pr, sizeof(float) * K, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CRYOIM_ERR_CUDA, cudaGetErrorString(e));
    return CRYOIM_OK;
}
