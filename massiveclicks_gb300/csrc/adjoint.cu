// DBN session log-likelihood and its gradient with respect to logit
// parameters: alpha (attractiveness), beta (satisfaction) per query-document
// pair and gamma (continuation), a = sigmoid(alpha), s = sigmoid(beta),
// g = sigmoid(gamma).
//
// The log-likelihood is the reference's conditional click model
// (dbn.cu:611-639): with ex_0 = 1, at each rank r
//   clicked:    p_r = a ex_r,      ex_{r+1} = g (1 - s)
//   unclicked:  p_r = 1 - a ex_r,  ex_{r+1} = ex_r g (1 - a) / p_r
// and LL = sum_r log p_r.  One thread per session runs this recursion forward,
// keeps the ten examination messages in registers, and walks it back
// (reverse mode) to the adjoints of a, s and g; the messages are recomputed
// by every call instead of being stored.  Sessions grouped by query go
// through the model's tiles, with the gradient summed per tile in shared
// memory; other session orders through FP64 global atomics per session.
#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace mcd {

template <typename T>
__device__ __forceinline__ T sigm(float x) {
    return T(1) / (T(1) + exp(-(T)x));
}

template <typename T>
__device__ __forceinline__ T tlog(T x) { return log(x); }

// 1 / x, correctly rounded in both precisions (the FP32 reciprocal
// instruction with round-to-nearest costs a fraction of a full division).
__device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }

__device__ __forceinline__ double warp_sum_dd(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One session: log-likelihood and, if grad is set, adjoints scaled by scale
// added to the FP64 gradient arrays.
template <typename T>
__device__ double session_adjoint(const AdjointArgs& A, int64_t s, bool grad) {
    int p[MC_R];
    T a[MC_R], sv[MC_R], ex[MC_R + 1], pr[MC_R];
    const unsigned m = A.click[s];
    const T g = sigm<T>(A.gamma[0]);
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        p[r] = A.pidx[(int64_t)r * A.stride + s];
        a[r] = sigm<T>(A.alpha[p[r]]);
        sv[r] = sigm<T>(A.beta[p[r]]);
    }
    ex[0] = T(1);
    double ll = 0.0;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        if ((m >> r) & 1u) {
            pr[r] = a[r] * ex[r];
            ex[r + 1] = g * (T(1) - sv[r]);
        } else {
            pr[r] = T(1) - a[r] * ex[r];
            ex[r + 1] = ex[r] * g * (T(1) - a[r]) / pr[r];
        }
        ll += (double)tlog(pr[r]);
    }
    if (!grad) return ll;
    // Reverse pass: e_bar is the adjoint of ex_{r+1}.
    T e_bar = T(0), g_bar = T(0);
    const T w = (T)A.scale;
#pragma unroll
    for (int r = MC_R - 1; r >= 0; r--) {
        T a_bar, ex_bar;
        if ((m >> r) & 1u) {
            // p = a ex, ex' = g (1 - s)
            a_bar = T(1) / a[r];
            ex_bar = T(1) / ex[r];
            g_bar += e_bar * (T(1) - sv[r]);
            T s_bar = -e_bar * g;
            atomicAdd(A.g_beta + p[r], (double)(w * s_bar * sv[r] * (T(1) - sv[r])));
        } else {
            // p = 1 - a ex, ex' = ex g (1 - a) / p
            T ip = T(1) / pr[r];
            a_bar = -ex[r] * ip + e_bar * ex[r] * g * (ex[r] - T(1)) * ip * ip;
            ex_bar = -a[r] * ip + e_bar * g * (T(1) - a[r]) * ip * ip;
            g_bar += e_bar * ex[r] * (T(1) - a[r]) * ip;
        }
        atomicAdd(A.g_alpha + p[r], (double)(w * a_bar * a[r] * (T(1) - a[r])));
        e_bar = ex_bar;
    }
    atomicAdd(A.g_gamma, (double)(w * g_bar * g * (T(1) - g)));
    return ll;
}

template <typename T>
__global__ void __launch_bounds__(256) adjoint_kernel(AdjointArgs A, bool grad) {
    __shared__ double red[8];
    double ll = 0.0;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.count; i += step)
        ll += session_adjoint<T>(A, A.begin + i, grad);
    ll = warp_sum_dd(ll);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ll;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) v += red[k];
        atomicAdd(A.ll_out, v);
    }
}

// Tile path (sessions grouped by query, as the model's tiles describe them):
// a block takes whole tiles; a tile whose query-document window fits in
// shared memory gets its window's values sigmoid(alpha), sigmoid(beta)
// staged once and its gradient summed in shared memory, then written out in
// one pass per window entry: a plain store for a tile that owns its window
// (whole queries: no other tile touches those pairs), FP64 atomics for a
// chunk of a split query.  A wider window takes the per-session kernel's
// global atomics.  The continuation gradient and the log-likelihood go
// through registers and one FP64 atomic per block.
// A window of at most kSmallWin pairs (a head query's chunk: a few dozen
// documents shown to thousands of sessions) sums into kSmallCopies copies of
// its bins, one per (warp, lane % 4), so that only lanes of one warp with the
// same lane % 4 meet on an address; the copies are added at the flush.
constexpr int kSmallWin = 64;
constexpr int kSmallCopies = 32;

template <typename T>
__host__ __device__ constexpr int adjoint_smem_elems(int window_max) {
    return 4 * window_max > 2 * kSmallWin + 2 * kSmallWin * kSmallCopies ? 4 * window_max
                                                                        : 2 * kSmallWin + 2 * kSmallWin * kSmallCopies;
}

// Three 256-thread blocks per SM in FP32 (at most 85 registers; a few spill),
// which measured faster than two without spills; FP64 is the checking path.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) adjoint_tiles_kernel(AdjointArgs A, const TileDev* __restrict__ tiles, int t0,
                                                           int t1, int window_max, bool grad) {
    extern __shared__ __align__(16) unsigned char sm[];
    // Wide window: va, vs, ga, gb of window_max entries each.  Small window
    // (<= kSmallWin): va, vs of kSmallWin entries, then the copies
    // [kSmallCopies][2][kSmallWin] (alpha, beta).
    T* const base = reinterpret_cast<T*>(sm);
    __shared__ double red[2][8];
    const T g = sigm<T>(A.gamma[0]);
    const T w = (T)A.scale;
    double ll = 0.0;
    T g_bar_acc = T(0);
    const int64_t r0 = A.begin, r1 = A.begin + A.count;
    for (int t = t0 + blockIdx.x; t < t1; t += gridDim.x) {
        const TileDev tile = tiles[t];
        const int64_t s0 = tile.s_begin > r0 ? tile.s_begin : r0;
        const int64_t s1 = tile.s_begin + tile.s_count < r1 ? tile.s_begin + tile.s_count : r1;
        if (s0 >= s1) continue;  // uniform over the block
        const bool staged = tile.qd_count <= window_max;
        const bool small = staged && tile.qd_count <= kSmallWin;
        const int wcap = small ? kSmallWin : window_max;
        T* const va = base;
        T* const vs = base + wcap;
        T* const ga = base + 2 * wcap;             // wide window only
        T* const gb = base + 3 * wcap;
        T* const cp = base + 2 * kSmallWin;        // small window: the copies
        T* const my = cp + ((threadIdx.x >> 5) * 4 + (threadIdx.x & 3)) * 2 * kSmallWin;
        if (staged) {
            for (int i = threadIdx.x; i < tile.qd_count; i += blockDim.x) {
                va[i] = sigm<T>(A.alpha[tile.qd_begin + i]);
                vs[i] = sigm<T>(A.beta[tile.qd_begin + i]);
                if (!small) { ga[i] = T(0); gb[i] = T(0); }
            }
            if (small)
                for (int i = threadIdx.x; i < 2 * kSmallWin * kSmallCopies; i += blockDim.x) cp[i] = T(0);
            __syncthreads();
        }
        // Each thread loads its next session's indices and clicks while it
        // works on the current one (global loads are the longest wait here).
        int pn[MC_R];
        unsigned mn = 0;
        if (s0 + threadIdx.x < s1) {
            mn = A.click[s0 + threadIdx.x];
#pragma unroll
            for (int r = 0; r < MC_R; r++) pn[r] = A.pidx[(int64_t)r * A.stride + s0 + threadIdx.x];
        }
        for (int64_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
            int rl[MC_R];
            T a[MC_R], sv[MC_R], ex[MC_R + 1], ip[MC_R];  // ip: 1 / p of unclicked ranks
            const unsigned m = mn;
            int pc[MC_R];
#pragma unroll
            for (int r = 0; r < MC_R; r++) pc[r] = pn[r];
            if (s + blockDim.x < s1) {
                mn = A.click[s + blockDim.x];
#pragma unroll
                for (int r = 0; r < MC_R; r++) pn[r] = A.pidx[(int64_t)r * A.stride + s + blockDim.x];
            }
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                const int p = pc[r];
                // A tile's sessions show only its window's pairs (the tiles
                // are built so); the clamp keeps shared-memory accesses in
                // bounds regardless.
                rl[r] = staged ? min(max(p - (int)tile.qd_begin, 0), tile.qd_count - 1) : p;
                a[r] = staged ? va[rl[r]] : sigm<T>(A.alpha[p]);
                sv[r] = staged ? vs[rl[r]] : sigm<T>(A.beta[p]);
            }
            ex[0] = T(1);
            T lls = T(0);
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                T pr;
                if ((m >> r) & 1u) {
                    pr = a[r] * ex[r];
                    ex[r + 1] = g * (T(1) - sv[r]);
                    ip[r] = T(0);
                } else {
                    pr = T(1) - a[r] * ex[r];
                    ip[r] = rcp(pr);
                    ex[r + 1] = ex[r] * g * (T(1) - a[r]) * ip[r];
                }
                lls += tlog(pr);
            }
            ll += (double)lls;
            if (!grad) continue;
            T e_bar = T(0);
#pragma unroll
            for (int r = MC_R - 1; r >= 0; r--) {
                T a_bar, ex_bar;
                if ((m >> r) & 1u) {
                    a_bar = rcp(a[r]);
                    ex_bar = rcp(ex[r]);
                    g_bar_acc += e_bar * (T(1) - sv[r]);
                    const T db = w * (-e_bar * g) * sv[r] * (T(1) - sv[r]);
                    if (small) atomicAdd(my + kSmallWin + rl[r], db);
                    else if (staged) atomicAdd(gb + rl[r], db);
                    else atomicAdd(A.g_beta + rl[r], (double)db);
                } else {
                    const T q = ip[r];
                    a_bar = -ex[r] * q + e_bar * ex[r] * g * (ex[r] - T(1)) * q * q;
                    ex_bar = -a[r] * q + e_bar * g * (T(1) - a[r]) * q * q;
                    g_bar_acc += e_bar * ex[r] * (T(1) - a[r]) * q;
                }
                const T da = w * a_bar * a[r] * (T(1) - a[r]);
                if (small) atomicAdd(my + rl[r], da);
                else if (staged) atomicAdd(ga + rl[r], da);
                else atomicAdd(A.g_alpha + rl[r], (double)da);
                e_bar = ex_bar;
            }
        }
        if (staged) {
            __syncthreads();
            if (grad) {
                const bool owned = tile.split < 0;
                for (int i = threadIdx.x; i < tile.qd_count; i += blockDim.x) {
                    const int64_t q = tile.qd_begin + i;
                    double sa, sb;
                    if (small) {
                        sa = 0.0;
                        sb = 0.0;
                        for (int c = 0; c < kSmallCopies; c++) {
                            sa += (double)cp[c * 2 * kSmallWin + i];
                            sb += (double)cp[c * 2 * kSmallWin + kSmallWin + i];
                        }
                    } else {
                        sa = (double)ga[i];
                        sb = (double)gb[i];
                    }
                    if (owned) {
                        A.g_alpha[q] = sa;
                        A.g_beta[q] = sb;
                    } else {
                        if (sa != 0.0) atomicAdd(A.g_alpha + q, sa);
                        if (sb != 0.0) atomicAdd(A.g_beta + q, sb);
                    }
                }
            }
            __syncthreads();  // the window arrays are reused by the next tile
        }
    }
    double gg = grad ? (double)(w * g_bar_acc * g * (T(1) - g)) : 0.0;
    ll = warp_sum_dd(ll);
    gg = warp_sum_dd(gg);
    if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = ll; red[1][threadIdx.x >> 5] = gg; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0, u = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { v += red[0][k]; u += red[1][k]; }
        atomicAdd(A.ll_out, v);
        if (grad && u != 0.0) atomicAdd(A.g_gamma, u);
    }
}

__global__ void grad_to_float_kernel(const double* src, float* dst, int64_t n) {
    int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) dst[i] = (float)src[i];
}

cudaError_t launch_adjoint(const AdjointArgs& A, bool grad, bool fp64, int n_sm, cudaStream_t st) {
    if (A.count <= 0) return cudaSuccess;
    int64_t blocks = (A.count + 255) / 256;
    int g = (int)(blocks < 8 * n_sm ? blocks : 8 * n_sm);
    if (fp64) adjoint_kernel<double><<<g, 256, 0, st>>>(A, grad);
    else adjoint_kernel<float><<<g, 256, 0, st>>>(A, grad);
    return cudaGetLastError();
}

size_t adjoint_tiles_smem(int window_max, bool fp64) {
    return (size_t)adjoint_smem_elems<float>(window_max) * (fp64 ? 8 : 4);
}

// Resident blocks per SM of the tile kernel for a shared-memory size, per
// device and precision, found once: the attribute and occupancy queries cost
// more host time than a minibatch's kernel.  The kernel's dynamic
// shared-memory limit only ever grows, so no call shrinks it under another.
static int adjoint_blocks_per_sm(bool fp64, size_t smem, cudaError_t* err) {
    static std::mutex mu;
    static std::map<std::tuple<int, bool, size_t>, int> cache;
    static std::map<std::pair<int, bool>, size_t> limit;
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return 0;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({dev, fp64, smem});
    if (it != cache.end()) return it->second;
    size_t& lim = limit[{dev, fp64}];
    if (smem > lim) {
        *err = fp64 ? cudaFuncSetAttribute(adjoint_tiles_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                    : cudaFuncSetAttribute(adjoint_tiles_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (*err != cudaSuccess) return 0;
        lim = smem;
    }
    int per_sm = 0;
    *err = fp64 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_tiles_kernel<double>, 256, smem)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_tiles_kernel<float>, 256, smem);
    if (*err != cudaSuccess) return 0;
    cache[{dev, fp64, smem}] = per_sm;
    return per_sm;
}

cudaError_t launch_adjoint_tiles(const AdjointArgs& A, const TileDev* tiles, int t0, int t1, int window_max, bool grad,
                                 bool fp64, int n_sm, cudaStream_t st) {
    if (A.count <= 0 || t1 <= t0) return cudaSuccess;
    const size_t smem = adjoint_tiles_smem(window_max, fp64);
    cudaError_t e = cudaSuccess;
    const int per_sm = adjoint_blocks_per_sm(fp64, smem, &e);
    if (e != cudaSuccess) return e;
    const int n = t1 - t0;
    const int cap = (per_sm > 0 ? per_sm : 1) * n_sm;
    const int g = n < cap ? n : cap;
    if (fp64) adjoint_tiles_kernel<double><<<g, 256, smem, st>>>(A, tiles, t0, t1, window_max, grad);
    else adjoint_tiles_kernel<float><<<g, 256, smem, st>>>(A, tiles, t0, t1, window_max, grad);
    return cudaGetLastError();
}

cudaError_t launch_grad_to_float(const double* src, float* dst, int64_t n, int n_sm, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    int g = (int)(blocks < 8 * n_sm ? blocks : 8 * n_sm);
    grad_to_float_kernel<<<g, 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

}  // namespace mcd
