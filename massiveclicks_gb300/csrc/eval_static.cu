// mc_evaluate_static: test-set log-likelihood and perplexity sums computed
// without allocating any memory.
//
// Some callers cannot call cudaMalloc at the moment they need an evaluation:
// a serving process that has handed all device memory to its own pool, code
// running under a memory budget that forbids new allocations, or a host
// thread that must not touch the allocator (and its implicit synchronisation)
// while other streams are busy.  This entry point takes the caller's device
// buffers as inputs, writes the results to the caller's host memory, and keeps
// its intermediate sums in a fixed file-scope device array instead of an
// allocation.
//
// Scratch: g_eval_scratch holds one partial row of 12 doubles per block
// (log-likelihood sum, one log2 sum per rank, the count of out-of-range
// indices) plus one final row.  Each block covers
// EVAL_STATIC_SESSIONS_PER_BLOCK sessions, so a call needs ceil(n / 2048)
// rows; with EVAL_STATIC_MAX_BLOCKS rows the array is 768 KB and the largest
// accepted n is 16,777,216 sessions.  Every GPU on which this library's
// device code is loaded holds the array until the process exits.  CUDA loads
// device code lazily by default, so the array is reserved on a device by the
// first call of this entry point there (a call with n_sessions = 0 does only
// that set-up): a caller whose own pool takes the device memory makes that
// call first.
//
// Every call shares the array and it keeps the last call's contents; a call
// writes every row it reads before reading it, so nothing needs clearing, but
// calls that overlap on the GPU (different streams, or several host threads)
// race on it and must be serialised by the caller.  The reduction order is
// fixed, so a call's result does not depend on timing.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda.h>
#include <cuda_runtime.h>

#include "mclicks.h"
#include "host_internal.h"
#include "common.cuh"

namespace {

constexpr int EVAL_STATIC_THREADS = 256;
constexpr int EVAL_STATIC_SESSIONS_PER_THREAD = 8;
constexpr int EVAL_STATIC_SESSIONS_PER_BLOCK = EVAL_STATIC_THREADS * EVAL_STATIC_SESSIONS_PER_THREAD;  // 2048
constexpr int EVAL_STATIC_MAX_BLOCKS = 8192;
constexpr int EVAL_ROW = MC_R + 2;  // ll, log2 per rank, out-of-range indices
constexpr int EVAL_SUMS = MC_R + 1;
constexpr int64_t EVAL_STATIC_MAX_SESSIONS = (int64_t)EVAL_STATIC_SESSIONS_PER_BLOCK * EVAL_STATIC_MAX_BLOCKS;

// Partial rows [0, EVAL_STATIC_MAX_BLOCKS) and the final row after them.
static __device__ __align__(256) double g_eval_scratch[(EVAL_STATIC_MAX_BLOCKS + 1) * EVAL_ROW];

// Per-session terms: (sum_r log p_r) / 10 with p_r the conditional click
// probability, and log2 q_r with q_r the full click probability
// (click_models/*.cu get_log_conditional_click_probs / get_full_click_probs).
__device__ void session_terms(int model, unsigned m, const float (&a)[MC_R], const float (&sv)[MC_R], const float* pub,
                              double& ll, double (&l2)[MC_R]) {
    float lc[MC_R], fp[MC_R];
    if (model == MC_PBM || model == MC_UBM) {
        int prev[MC_R];
        int last = MC_R - 1;
        for (int r = 0; r < MC_R; r++) { prev[r] = last; if ((m >> r) & 1u) last = r; }
        for (int r = 0; r < MC_R; r++) {
            float e = model == MC_PBM ? pub[r] : pub[r * (r + 1) / 2 + prev[r]];
            float ae = a[r] * e;
            lc[r] = ((m >> r) & 1u) ? logf(ae) : logf(1.f - ae);
        }
        if (model == MC_PBM) {
            for (int r = 0; r < MC_R; r++) {
                float ae = a[r] * pub[r];
                fp[r] = ((m >> r) & 1u) ? ae : 1.f - ae;
            }
        } else {
            float marg[MC_R];
            for (int r = 0; r < MC_R; r++) {
                float cp = 0.f;
                for (int pc = -1; pc < r; pc++) {
                    int pcc = pc < 0 ? 9 : pc;
                    float none = 1.f;
                    for (int b = pc + 1; b < r; b++) none *= 1.f - a[b] * pub[b * (b + 1) / 2 + pcc];
                    float tmp = none * (a[r] * pub[r * (r + 1) / 2 + pcc]);
                    cp += pc >= 0 ? marg[pc] * tmp : tmp;
                }
                marg[r] = cp;
                fp[r] = ((m >> r) & 1u) ? cp : 1.f - cp;
            }
        }
    } else {
        const bool dbn = model == MC_DBN;
        float g = pub[0], t1 = pub[0], t2 = pub[1], t3 = pub[2];
        float ex = 1.f;
        for (int r = 0; r < MC_R; r++) {
            float cp;
            if ((m >> r) & 1u) {
                cp = a[r] * ex;
                ex = dbn ? g * (1.f - sv[r]) : t2 * (1.f - a[r]) + t3 * a[r];
            } else {
                cp = 1.f - a[r] * ex;
                ex *= (dbn ? g : t1) * (1.f - a[r]) / cp;
            }
            lc[r] = logf(cp);
        }
        ex = 1.f;
        for (int r = 0; r < MC_R; r++) {
            float ae = a[r] * ex;
            fp[r] = ((m >> r) & 1u) ? ae : 1.f - ae;
            ex *= dbn ? g * (1.f - a[r]) + g * a[r] * (1.f - sv[r]) : (1.f - a[r]) * t1 + a[r] * ((1.f - a[r]) * t2 + a[r] * t3);
        }
    }
    double s = 0.0;
    for (int r = 0; r < MC_R; r++) {
        s += (double)lc[r];
        l2[r] = (double)log2f(fp[r]);
    }
    ll = s / 10.0;
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block b covers sessions [b * 2048, (b + 1) * 2048) and writes row b.
__global__ void __launch_bounds__(EVAL_STATIC_THREADS) eval_static_kernel(
    int model, int64_t n, int64_t n_qd, const int32_t* __restrict__ pidx, const uint16_t* __restrict__ click,
    const float* __restrict__ atr, const float* __restrict__ sat, const float* __restrict__ pub, double* scratch) {
    __shared__ double red[EVAL_ROW][EVAL_STATIC_THREADS / 32];
    __shared__ float pub_s[MC_UBM_SLOTS];
    const int n_pub = model == MC_PBM ? MC_R : model == MC_UBM ? MC_UBM_SLOTS : model == MC_DBN ? 1 : 3;
    for (int k = threadIdx.x; k < n_pub; k += blockDim.x) pub_s[k] = pub[k];
    __syncthreads();
    double acc[EVAL_ROW];
    for (int k = 0; k < EVAL_ROW; k++) acc[k] = 0.0;
    const int64_t base = (int64_t)blockIdx.x * EVAL_STATIC_SESSIONS_PER_BLOCK;
    for (int j = 0; j < EVAL_STATIC_SESSIONS_PER_THREAD; j++) {
        int64_t s = base + (int64_t)j * EVAL_STATIC_THREADS + threadIdx.x;
        if (s >= n) break;
        unsigned m = click[s];
        float a[MC_R], sv[MC_R];
        for (int r = 0; r < MC_R; r++) {
            int p = pidx[s * MC_R + r];
            bool seen = p >= 0 && (int64_t)p < n_qd;
            if (!seen && p != -1) acc[EVAL_SUMS] += 1.0;  // neither a pair index nor the unseen marker
            a[r] = seen ? atr[p] : 0.5f;
            sv[r] = (model == MC_DBN && seen) ? sat[p] : 0.5f;
        }
        double ll, l2[MC_R];
        session_terms(model, m, a, sv, pub_s, ll, l2);
        acc[0] += ll;
        for (int r = 0; r < MC_R; r++) acc[1 + r] += l2[r];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < EVAL_ROW; k++) {
        double v = warp_sum_d(acc[k]);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < EVAL_ROW) {
        double v = 0.0;
        for (int w = 0; w < EVAL_STATIC_THREADS / 32; w++) v += red[threadIdx.x][w];
        scratch[(int64_t)blockIdx.x * EVAL_ROW + threadIdx.x] = v;
    }
}

// One block: sums the partial rows in a fixed order into the final row.
__global__ void eval_static_reduce_kernel(int blocks, double* scratch) {
    __shared__ double red[EVAL_ROW][32];
    int k = threadIdx.x / 32, lane = threadIdx.x & 31;
    if (k < EVAL_ROW) {
        double v = 0.0;
        for (int b = lane; b < blocks; b += 32) v += scratch[(int64_t)b * EVAL_ROW + k];
        red[k][lane] = v;
    }
    __syncthreads();
    if (threadIdx.x < EVAL_ROW) {
        double v = 0.0;
        for (int l = 0; l < 32; l++) v += red[threadIdx.x][l];
        scratch[(int64_t)EVAL_STATIC_MAX_BLOCKS * EVAL_ROW + threadIdx.x] = v;
    }
}

// Device address of g_eval_scratch, looked up with cudaGetSymbolAddress once
// per device context (with that device current) and cached beside the
// context's unique id: after cudaDeviceReset the device gets a new primary
// context with another id, and the address is looked up again.
constexpr int MAX_DEVICES = 64;
std::mutex g_addr_mutex;
struct ScratchAddr {
    double* ptr = nullptr;
    unsigned long long ctx_id = 0;
};
ScratchAddr g_addr[MAX_DEVICES];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int cuda_fail(const char* what, cudaError_t e) {
    cudaGetLastError();
    return mch::set_error(MC_ERR_CUDA, std::string("evaluate_static: ") + what + ": " + cudaGetErrorString(e));
}

// Id of the context current on this thread (the device's primary context
// once cudaSetDevice has made it current).
int current_context_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return cuda_fail("driver entry points", e);
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return mch::set_error(MC_ERR_CUDA, "evaluate_static: cuCtxGetCurrent / cuCtxGetId unavailable");
        g_ctx_get_current = (CtxGetCurrentFn)f1;
        g_ctx_get_id = (CtxGetIdFn)f2;
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_get_id(ctx, id) != CUDA_SUCCESS)
        return mch::set_error(MC_ERR_CUDA, "evaluate_static: no current CUDA context");
    return MC_OK;
}

// Makes `device` current (initialising its primary context) and returns the
// array's address in that context.
int scratch_address(int device, double** out) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail("cudaSetDevice", e);
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc) return rc;
    ScratchAddr& a = g_addr[device];
    if (!a.ptr || a.ctx_id != id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_eval_scratch);
        if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress", e);
        a.ptr = static_cast<double*>(p);
        a.ctx_id = id;
    }
    *out = a.ptr;
    return MC_OK;
}

}  // namespace

extern "C" int mc_evaluate_static(int model_type, int64_t n_sessions, const int32_t* pidx, const uint16_t* click_mask,
                                  int64_t n_qd, const float* atr, const float* sat, const float* pub, double* ll_sum,
                                  double* log2_sums, void* stream) {
    using mch::set_error;
    if (model_type < 0 || model_type > 3)
        return set_error(MC_ERR_INVALID, "evaluate_static: model type must be MC_PBM, MC_CCM, MC_DBN or MC_UBM");
    if (n_sessions < 0 || n_qd < 0) return set_error(MC_ERR_INVALID, "evaluate_static: negative size");
    if (n_sessions > EVAL_STATIC_MAX_SESSIONS)
        return set_error(MC_ERR_INVALID, "evaluate_static: " + std::to_string(n_sessions) + " sessions exceed the maximum of " +
                                             std::to_string(EVAL_STATIC_MAX_SESSIONS) + " (fixed scratch of " +
                                             std::to_string(EVAL_STATIC_MAX_BLOCKS) + " partial rows)");
    if (!ll_sum || !log2_sums) return set_error(MC_ERR_INVALID, "evaluate_static: null output");
    if (n_sessions > 0 && (!pidx || !click_mask || !atr || !pub || (model_type == MC_DBN && !sat)))
        return set_error(MC_ERR_INVALID, "evaluate_static: null input");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_fail("cudaGetDevice", e);
    if (device < 0 || device >= MAX_DEVICES) return set_error(MC_ERR_INVALID, "evaluate_static: device ordinal too large");
    double* scratch = nullptr;
    int rc = scratch_address(device, &scratch);
    if (rc) return rc;
    if (n_sessions == 0) {  // the set-up alone
        *ll_sum = 0.0;
        for (int r = 0; r < MC_R; r++) log2_sums[r] = 0.0;
        return MC_OK;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int blocks = (int)((n_sessions + EVAL_STATIC_SESSIONS_PER_BLOCK - 1) / EVAL_STATIC_SESSIONS_PER_BLOCK);
    eval_static_kernel<<<blocks, EVAL_STATIC_THREADS, 0, st>>>(model_type, n_sessions, n_qd, pidx, click_mask, atr,
                                                               model_type == MC_DBN ? sat : nullptr, pub, scratch);
    eval_static_reduce_kernel<<<1, EVAL_ROW * 32, 0, st>>>(blocks, scratch);
    double out[EVAL_ROW];
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, scratch + (int64_t)EVAL_STATIC_MAX_BLOCKS * EVAL_ROW, sizeof(out), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail("evaluation", e);
    if (out[EVAL_SUMS] != 0.0)
        return set_error(MC_ERR_INVALID, "evaluate_static: " + std::to_string((int64_t)out[EVAL_SUMS]) +
                                             " indices are neither -1 nor in [0, n_qd)");
    *ll_sum = out[0];
    for (int r = 0; r < MC_R; r++) log2_sums[r] = out[1 + r];
    return MC_OK;
}
