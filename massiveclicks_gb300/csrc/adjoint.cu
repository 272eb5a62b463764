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
// memory (FP32: fixed-point bins, constant terms counted, whole tiles read a
// packed copy of their sessions in click-mask order); other session orders
// through FP64 global atomics per session.
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
// FP32: the correctly rounded reciprocal equals the correctly rounded 1 / y.
template <>
__device__ __forceinline__ float sigm<float>(float x) {
    return __frcp_rn(1.0f + expf(-x));
}

template <typename T>
__device__ __forceinline__ T tlog(T x) { return log(x); }

// 1 / x: in FP32 the approximate reciprocal (within 2 ulp), which measured
// 6% faster over a pass than the correctly rounded one at the same gradient
// error against FP64; exact division in FP64.
__device__ __forceinline__ float rcp(float x) { return __fdividef(1.0f, x); }
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
//
// FP32 bins are 32-bit fixed point added with integer shared-memory atomics
// (a float add in shared memory costs several times an integer one here).
// The derivative of LL with respect to a logit, per occurrence and before the
// caller's scale, is E[A_r | clicks] - a_r for alpha and E[S_r | clicks] - s_r
// for beta (the score of a Bernoulli latent's logit).  Three kinds of term are
// constants and are counted instead of added (a fixed-point rounding repeated
// over many equal values would not average out):
//   * a clicked rank: A_r = 1, the alpha term is 1 - a;
//   * an unclicked rank before the last click: it was examined (a later rank
//     was), A_r = 0, the alpha term is -a;
//   * a clicked rank before the last click: the later click shows that the
//     user went on (S_r = 0), the beta term is -s.
// With n_before the occurrences at or before the session's last click, the
// flush adds n_click - a n_before to alpha and -(n_click - n_last) s to beta.
// What is summed in fixed point:
//   * alpha of an unclicked rank, in [-a, 0], scaled by 2^(sh_q + b) with
//     b = 126 - e(a) (e the binary exponent of a, at least 66), so that
//     |v 2^b| < 1 keeps a small a's relative precision;
//   * beta of the last clicked rank, in [-1, 1], scaled by 2^sh_q.
// sh = 29 - ceil(log2 n), n a bound on the adds the bin can receive in the
// tile; values are clamped to twice their bound (which only removes rounding
// garbage), so no bin can pass 2^30.  A tile whose sessions all lie in the
// called range takes its counts, and its bounds (the occurrences after the
// last click for alpha, the last clicks for beta), from the per-tile counts
// built once per tile layout (AdjointArgs::tcnt); a tile cut by the range
// ends counts with integer atomics, with n = min(occurrences of the pair in
// the training set, 10 * the tile's sessions in range) for both bins.  The flush computes in FP32
// with exact power-of-two factors (FP64 arithmetic is slow here, and the
// gradient is returned in FP32).  The FP64 instantiation keeps FP64 bins and
// adds every term (the checking path).
constexpr int kSmallWin = 64;
constexpr int kSmallCopies = 32;

// Per-entry value arrays: sigmoid(alpha), sigmoid(beta) and, in FP32, the
// fixed-point scales 2^sh of the alpha and beta bins.
template <typename T>
__host__ __device__ constexpr int adjoint_value_arrays() { return sizeof(T) == 4 ? 4 : 2; }
// Per-entry bins: FP32 alpha, beta (fixed point), then the counts of clicks,
// last clicks and occurrences at or before the last click; FP64 alpha, beta.
template <typename T>
__host__ __device__ constexpr int adjoint_bins() { return sizeof(T) == 4 ? 5 : 2; }

template <typename T>
__host__ __device__ constexpr int adjoint_smem_elems(int window_max) {
    return (adjoint_value_arrays<T>() + adjoint_bins<T>()) * window_max >
                   adjoint_value_arrays<T>() * kSmallWin + adjoint_bins<T>() * kSmallWin * kSmallCopies
               ? (adjoint_value_arrays<T>() + adjoint_bins<T>()) * window_max
               : adjoint_value_arrays<T>() * kSmallWin + adjoint_bins<T>() * kSmallWin * kSmallCopies;
}

// 2^sh for an entry that can receive at most n adds.
__device__ __forceinline__ float adjoint_fx_scale(uint32_t n) {
    const int need = n > 1u ? 32 - __clz(n - 1u) : 0;
    return __int_as_float((127 + 29 - need) << 23);
}

// (126 - e(a)) << 23 for the boost 2^b of an alpha term, e(a) the exponent
// field of a clamped below at 66 (b <= 60).
__device__ __forceinline__ int adjoint_boost_bits(float a) {
    return (126 << 23) - max(__float_as_int(a) & 0x7F800000, 66 << 23);
}

template <typename T>
struct AdjointBin { using type = T; };
template <>
struct AdjointBin<float> { using type = int; };

// Where a tile's gradient goes: a small window's (warp, lane % 4) copy of its
// bins, a wide window's shared bins, or (a window too wide to stage) the FP64
// global arrays.
enum AdjointTileKind { kAdjSmall = 0, kAdjWide = 1, kAdjGlobal = 2 };

// A tile's view for its sessions: window values and scales, this thread's
// bins (array k at bins + k * wcap), the tile's first window pair, and its
// packed sessions in click-mask order (prel [10][spad], pclk [spad]).
template <typename T>
struct AdjointTile {
    const T* va;
    const T* vs;
    const float* scl_a;
    const float* scl_b;
    typename AdjointBin<T>::type* bins;
    int wcap;
    int qd_begin, qd_count;
    const uint16_t* prel;
    const uint16_t* pclk;
    int spad;
};

// The sessions [s0, s1) of one tile, one thread per session: the forward
// recursion (log-likelihood) and, if grad, the reverse pass into the tile's
// bins.  KIND, COUNT (FP32 counted terms by atomics: a tile cut by the called
// range) and PACKED (the tile's sessions read from its packed copy, in
// click-mask order, so that the lanes of a warp take the same branches) are
// template parameters, so that the unrolled loop of each kind carries no
// branch on the kind and stays small in the instruction cache.
template <typename T, int KIND, bool COUNT, bool PACKED>
__device__ __forceinline__ void adjoint_sessions(const AdjointArgs& A, const AdjointTile<T>& W, int64_t s0,
                                                 int64_t s1, T g, T w, bool grad, T& lls_tile, T& g_bar_acc) {
    constexpr bool FX = sizeof(T) == 4 && KIND != kAdjGlobal;  // counted terms and fixed-point bins
    using Bin = typename AdjointBin<T>::type;
    auto a_of = [&](int rl) -> T { return KIND == kAdjGlobal ? sigm<T>(A.alpha[rl]) : W.va[rl]; };
    auto s_of = [&](int rl) -> T { return KIND == kAdjGlobal ? sigm<T>(A.beta[rl]) : W.vs[rl]; };
    // Session k of the tile's range: its indices (window entries when packed)
    // and clicks.
    auto load = [&](int64_t k, int (&p)[MC_R], unsigned& m) {
        if constexpr (PACKED) {
            m = W.pclk[k];
#pragma unroll
            for (int r = 0; r < MC_R; r++) p[r] = W.prel[r * W.spad + k];
        } else {
            m = A.click[s0 + k];
#pragma unroll
            for (int r = 0; r < MC_R; r++) p[r] = A.pidx[(int64_t)r * A.stride + s0 + k];
        }
    };
    // Each thread loads its next session's indices and clicks while it works
    // on the current one (global loads are the longest wait here).
    const int64_t n = s1 - s0;
    int pn[MC_R];
    unsigned mn = 0;
    if (threadIdx.x < n) load(threadIdx.x, pn, mn);
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
        int rl[MC_R];
        T ex[MC_R + 1], ip[MC_R];  // ip: 1 / p of unclicked ranks
        const unsigned m = mn;
        // A tile's sessions show only its window's pairs (the tiles are built
        // so, and the packing checked it); the clamp keeps shared-memory
        // accesses in bounds regardless.  rl is the window entry, or the pair
        // for a window too wide to stage.
#pragma unroll
        for (int r = 0; r < MC_R; r++)
            rl[r] = KIND == kAdjGlobal || PACKED ? pn[r] : min(max(pn[r] - W.qd_begin, 0), W.qd_count - 1);
        if (k + blockDim.x < n) load(k + blockDim.x, pn, mn);
        T a[MC_R], sv[MC_R];
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            a[r] = a_of(rl[r]);
            sv[r] = s_of(rl[r]);
        }
        ex[0] = T(1);
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
            lls_tile += tlog(pr);
        }
        if (!grad) continue;
        // Reverse pass, e_bar the adjoint of ex_{r+1}; a and s are read again
        // (fewer registers live across the passes).
        const int last = m ? 31 - __clz(m) : -1;
        T e_bar = T(0);
#pragma unroll
        for (int r = MC_R - 1; r >= 0; r--) {
            const T ar = a_of(rl[r]);
            T ex_bar;
            if (COUNT && r <= last) atomicAdd(W.bins + 4 * W.wcap + rl[r], Bin(1));
            if ((m >> r) & 1u) {
                // p = a ex, ex' = g (1 - s): alpha term 1 - a
                const T sr = s_of(rl[r]);
                ex_bar = rcp(ex[r]);
                g_bar_acc += e_bar * (T(1) - sr);
                const T db = (-e_bar * g) * sr * (T(1) - sr);
                if constexpr (FX) {
                    if (COUNT) atomicAdd(W.bins + 2 * W.wcap + rl[r], Bin(1));
                    if (r == last) {
                        if (COUNT) atomicAdd(W.bins + 3 * W.wcap + rl[r], Bin(1));
                        atomicAdd(W.bins + W.wcap + rl[r],
                                  __float2int_rn(fminf(fmaxf(db, -2.0f), 2.0f) * W.scl_b[rl[r]]));
                    }
                } else if constexpr (KIND != kAdjGlobal) {
                    atomicAdd(W.bins + rl[r], (Bin)(w * (T(1) - ar)));
                    atomicAdd(W.bins + W.wcap + rl[r], (Bin)(w * db));
                } else if (sizeof(T) == 4 && A.f_alpha) {
                    atomicAdd(A.f_alpha + rl[r], (float)(w * (T(1) - ar)));
                    atomicAdd(A.f_beta + rl[r], (float)(w * db));
                } else {
                    atomicAdd(A.g_alpha + rl[r], (double)(w * (T(1) - ar)));
                    atomicAdd(A.g_beta + rl[r], (double)(w * db));
                }
            } else {
                // p = 1 - a ex, ex' = ex g (1 - a) / p
                const T q = ip[r];
                const T a_bar = -ex[r] * q + e_bar * ex[r] * g * (ex[r] - T(1)) * q * q;
                ex_bar = -ar * q + e_bar * g * (T(1) - ar) * q * q;
                g_bar_acc += e_bar * ex[r] * (T(1) - ar) * q;
                const T da = a_bar * ar * (T(1) - ar);
                if constexpr (FX) {
                    if (r > last) {
                        const float sc = W.scl_a[rl[r]];
                        const float scb = __int_as_float(__float_as_int(sc) + adjoint_boost_bits(ar));
                        const float x = fminf(fmaxf(da * scb, -2.0f * sc), 2.0f * sc);
                        atomicAdd(W.bins + rl[r], __float2int_rn(x));
                    }
                } else if constexpr (KIND != kAdjGlobal) {
                    atomicAdd(W.bins + rl[r], (Bin)(w * da));
                } else if (sizeof(T) == 4 && A.f_alpha) {
                    atomicAdd(A.f_alpha + rl[r], (float)(w * da));
                } else {
                    atomicAdd(A.g_alpha + rl[r], (double)(w * da));
                }
            }
            e_bar = ex_bar;
        }
    }
}

// The rare kinds out of line: a window too wide to stage, the tiles a called
// range cuts (at most two per call; they count with atomics), forward-only
// calls and the FP64 instantiation (session order).  Only the two hot loops,
// whole staged tiles from their packed copies, are inlined into the kernel;
// with every kind inlined, the loop fell out of the instruction cache and the
// kernel spilled.
template <typename T, int KIND, bool COUNT>
__device__ __noinline__ void adjoint_sessions_cold(const AdjointArgs& A, const AdjointTile<T>& W, int64_t s0,
                                                   int64_t s1, T g, T w, bool grad, T& lls_tile, T& g_bar_acc) {
    adjoint_sessions<T, KIND, COUNT, false>(A, W, s0, s1, g, w, grad, lls_tile, g_bar_acc);
}

// Four 256-thread blocks per SM in FP32 (at most 64 registers; the out-of-line
// kinds spill around their calls), which measured faster than three (80
// registers) and two; FP64 is the checking path.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) adjoint_tiles_kernel(AdjointArgs A, const TileDev* __restrict__ tiles, int t0,
                                                           int t1, int window_max, bool grad) {
    constexpr bool FX = sizeof(T) == 4;
    using Bin = typename AdjointBin<T>::type;
    constexpr int NV = adjoint_value_arrays<T>();
    constexpr int NB = adjoint_bins<T>();
    extern __shared__ __align__(16) unsigned char sm[];
    // Wide window: va, vs (, scl_a, scl_b) of window_max entries each, then
    // NB bin arrays.  Small window (<= kSmallWin): va, vs (, scl_a, scl_b) of
    // kSmallWin entries, then the copies [kSmallCopies][NB][kSmallWin].
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
        float* const scl_a = reinterpret_cast<float*>(base + 2 * wcap);  // FP32 only
        float* const scl_b = reinterpret_cast<float*>(base + 3 * wcap);
        // counts from the per-tile table (all the tile's sessions in range)
        const int64_t toff = (FX && A.tcnt) ? A.tcnt_off[t] : -1;
        const bool full = toff >= 0 && s0 == tile.s_begin && s1 == tile.s_begin + tile.s_count;
        // Bin array k of this thread at bins + k * wcap: a wide window's
        // shared array, or its (warp, lane % 4) copy of a small window's.
        Bin* const bins = small ? reinterpret_cast<Bin*>(base + NV * kSmallWin) +
                                      ((threadIdx.x >> 5) * 4 + (threadIdx.x & 3)) * NB * kSmallWin
                                : reinterpret_cast<Bin*>(base + NV * wcap);
        if (staged) {
            const int64_t nb = 10 * (s1 - s0);
            const uint32_t n_bound = nb < (int64_t)UINT32_MAX ? (uint32_t)nb : UINT32_MAX;
            for (int i = threadIdx.x; i < tile.qd_count; i += blockDim.x) {
                va[i] = sigm<T>(A.alpha[tile.qd_begin + i]);
                vs[i] = sigm<T>(A.beta[tile.qd_begin + i]);
                if (!small) { bins[i] = Bin(0); bins[wcap + i] = Bin(0); }
                if constexpr (FX) {
                    if (full) {
                        // the counted terms from the per-tile counts, in the
                        // count bins (no count atomics for this tile)
                        const uint4 c = A.tcnt[toff + i];
                        scl_a[i] = adjoint_fx_scale(c.x - c.y);
                        scl_b[i] = adjoint_fx_scale(c.w);
                        if (!small) { bins[2 * wcap + i] = (Bin)c.z; bins[3 * wcap + i] = (Bin)c.w; bins[4 * wcap + i] = (Bin)c.y; }
                    } else {
                        scl_a[i] = scl_b[i] = adjoint_fx_scale(min(A.cnt[tile.qd_begin + i].x, n_bound));
                        if (!small) { bins[2 * wcap + i] = Bin(0); bins[3 * wcap + i] = Bin(0); bins[4 * wcap + i] = Bin(0); }
                    }
                }
            }
            if (small) {
                // copy 0 of a whole tile holds its counts (written once the
                // zeroing is done), the other copies' count bins stay 0
                Bin* const cp = reinterpret_cast<Bin*>(base + NV * kSmallWin);
                for (int i = threadIdx.x; i < NB * kSmallWin * kSmallCopies; i += blockDim.x) cp[i] = Bin(0);
                if constexpr (FX) {
                    if (full) {
                        __syncthreads();
                        for (int i = threadIdx.x; i < tile.qd_count; i += blockDim.x) {
                            const uint4 c = A.tcnt[toff + i];
                            cp[2 * kSmallWin + i] = (Bin)c.z;
                            cp[3 * kSmallWin + i] = (Bin)c.w;
                            cp[4 * kSmallWin + i] = (Bin)c.y;
                        }
                    }
                }
            }
            __syncthreads();
        }
        // The tile's log-likelihood in T, folded into FP64 once per tile.
        AdjointTile<T> W;
        W.va = va;
        W.vs = vs;
        W.scl_a = scl_a;
        W.scl_b = scl_b;
        W.bins = bins;
        W.wcap = wcap;
        W.qd_begin = (int)tile.qd_begin;
        W.qd_count = tile.qd_count;
        W.prel = nullptr;
        W.pclk = nullptr;
        W.spad = 0;
        T lls = T(0);
        const bool count = FX && staged && !full && grad;
        const bool packed = FX && staged && full && A.pblk;
        if (packed) {
            const TileDev pt = A.ptiles[t];
            W.prel = reinterpret_cast<const uint16_t*>(A.pblk + pt.blk_off);
            W.spad = (tile.s_count + 7) & ~7;
            W.pclk = W.prel + 10 * W.spad;
        }
        if (small) {
            if (packed) adjoint_sessions<T, kAdjSmall, false, true>(A, W, s0, s1, g, w, grad, lls, g_bar_acc);
            else if (count) adjoint_sessions_cold<T, kAdjSmall, true>(A, W, s0, s1, g, w, grad, lls, g_bar_acc);
            else adjoint_sessions_cold<T, kAdjSmall, false>(A, W, s0, s1, g, w, grad, lls, g_bar_acc);
        } else if (staged) {
            if (packed) adjoint_sessions<T, kAdjWide, false, true>(A, W, s0, s1, g, w, grad, lls, g_bar_acc);
            else if (count) adjoint_sessions_cold<T, kAdjWide, true>(A, W, s0, s1, g, w, grad, lls, g_bar_acc);
            else adjoint_sessions_cold<T, kAdjWide, false>(A, W, s0, s1, g, w, grad, lls, g_bar_acc);
        } else {
            adjoint_sessions_cold<T, kAdjGlobal, false>(A, W, s0, s1, g, w, grad, lls, g_bar_acc);
        }
        ll += (double)lls;
        if (staged) {
            __syncthreads();
            if (grad) {
                const bool owned = tile.split < 0;
                for (int i = threadIdx.x; i < tile.qd_count; i += blockDim.x) {
                    const int64_t q = tile.qd_begin + i;
                    // the entry's bins, summed over the copies of a small window
                    // (32-bit: the bound on an entry's adds covers all copies)
                    int sum[NB];
                    double dsum[NB];
                    for (int k = 0; k < NB; k++) { sum[k] = 0; dsum[k] = 0.0; }
                    if (small) {
                        const Bin* cp = reinterpret_cast<const Bin*>(base + NV * kSmallWin);
                        for (int c = 0; c < kSmallCopies; c++)
                            for (int k = 0; k < NB; k++) {
                                if constexpr (FX) sum[k] += cp[(c * NB + k) * kSmallWin + i];
                                else dsum[k] += cp[(c * NB + k) * kSmallWin + i];
                            }
                    } else {
                        const Bin* b = reinterpret_cast<const Bin*>(base + NV * wcap);
                        for (int k = 0; k < NB; k++) {
                            if constexpr (FX) sum[k] = b[k * wcap + i];
                            else dsum[k] = b[k * wcap + i];
                        }
                    }
                    double sa = dsum[0], sb = dsum[1];
                    float fa_out = 0.0f, fb_out = 0.0f;
                    if constexpr (FX) {
                        // 2^-sh and 2^-(sh + b) (exact), the counted terms, the caller's scale
                        const float a = va[i], sv = vs[i];
                        const float inv_a = __int_as_float(__float_as_int(__frcp_rn(scl_a[i])) - adjoint_boost_bits(a));
                        const float inv_b = __frcp_rn(scl_b[i]);
                        const float nc = (float)sum[2], nl = (float)sum[3], nb = (float)sum[4];
                        const float fa = (float)sum[0] * inv_a + (nc - a * nb);
                        const float fb = (float)sum[1] * inv_b - (nc - nl) * sv;
                        fa_out = w * fa;
                        fb_out = w * fb;
                        sa = (double)fa_out;
                        sb = (double)fb_out;
                    }
                    if (FX && A.f_alpha) {
                        if (owned) {
                            A.f_alpha[q] = fa_out;
                            A.f_beta[q] = fb_out;
                        } else {
                            if (fa_out != 0.0f) atomicAdd(A.f_alpha + q, fa_out);
                            if (fb_out != 0.0f) atomicAdd(A.f_beta + q, fb_out);
                        }
                    } else if (owned) {
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
    return fp64 ? (size_t)adjoint_smem_elems<double>(window_max) * 8 : (size_t)adjoint_smem_elems<float>(window_max) * 4;
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

// One block per staged tile: the tile's counts in shared memory
// ([4][qd_count]: occurrences, at or before the last click, clicks, last
// clicks), then written out.  Parameter-independent, built once per tile
// layout.
__global__ void __launch_bounds__(256) adjoint_counts_kernel(const TileDev* __restrict__ tiles, int n_tiles,
                                                             const int32_t* __restrict__ pidx,
                                                             const uint16_t* __restrict__ click, int64_t stride,
                                                             const int64_t* __restrict__ off, uint4* out) {
    extern __shared__ unsigned cnt_sm[];
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const int64_t o = off[t];
        if (o < 0) continue;  // uniform over the block
        const TileDev tile = tiles[t];
        const int n = tile.qd_count;
        for (int i = threadIdx.x; i < 4 * n; i += blockDim.x) cnt_sm[i] = 0u;
        __syncthreads();
        for (int64_t s = tile.s_begin + threadIdx.x; s < tile.s_begin + tile.s_count; s += blockDim.x) {
            const unsigned m = click[s];
            const int last = m ? 31 - __clz(m) : -1;
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                const int rl = min(max(pidx[(int64_t)r * stride + s] - (int)tile.qd_begin, 0), n - 1);
                atomicAdd(cnt_sm + rl, 1u);
                if (r <= last) atomicAdd(cnt_sm + n + rl, 1u);
                if ((m >> r) & 1u) atomicAdd(cnt_sm + 2 * n + rl, 1u);
                if (r == last) atomicAdd(cnt_sm + 3 * n + rl, 1u);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            out[o + i] = make_uint4(cnt_sm[i], cnt_sm[n + i], cnt_sm[2 * n + i], cnt_sm[3 * n + i]);
        __syncthreads();  // the counts are reused by the next tile
    }
}

cudaError_t launch_adjoint_counts(const TileDev* tiles, int n_tiles, int window_max, const int32_t* pidx,
                                  const uint16_t* click, int64_t stride, const int64_t* off, uint4* out, int n_sm,
                                  cudaStream_t st) {
    if (n_tiles <= 0) return cudaSuccess;
    const size_t smem = (size_t)16 * (size_t)window_max;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(adjoint_counts_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const int g = n_tiles < 4 * n_sm ? n_tiles : 4 * n_sm;
    adjoint_counts_kernel<<<g, 256, smem, st>>>(tiles, n_tiles, pidx, click, stride, off, out);
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
