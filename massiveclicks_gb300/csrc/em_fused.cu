// Fused EM iteration: E-step, statistics reduction and M-step in one
// persistent kernel launch per iteration.
//
// Work: a queue of session tiles (host-built, see model.cu).  Each tile is a
// run of whole queries (or a chunk of one large query) whose qd indices form
// one contiguous window.  Persistent CTAs (two per SM), every warp a worker:
//   * thread 0 keeps a ring of shared-memory stages filled: for the next tile
//     from the global queue it issues bulk async copies (cp.async.bulk,
//     completion on an mbarrier) of the tile's packed sessions (uint16
//     window-relative indices, rank-major, and click masks) and of the
//     window's parameter values; a stage is refilled right after the tile
//     that used it is done, with a tile index fetched one iteration ahead;
//   * the warps wait on the stage's mbarrier; then, as one pool of warp-sized
//     items taken from a shared counter, they run the E-step of that tile
//     (one thread per session, entirely from shared memory, each private
//     statistic added into a shared-memory bin per qd, each public one into
//     registers) and the M-step of the tile before it, whose bins are in the
//     other of two bin buffers:
//       - owned tile (whole queries): M-step for the window straight from the
//         bins and the click counts (copied into shared memory one tile
//         ahead), written in place to global memory (no other tile reads
//         those parameters);
//       - split tile (part of a large query): one warp folds the bins into the
//         query's FP64 global bins, and the warp that completes the query's
//         last tile runs its M-step;
//     one barrier ends the item pool and frees the tile's stage.
//   * public statistics: warp shuffles -> shared FP32 partial per tile -> FP64
//     per-CTA accumulator -> one FP64 global atomic per bin per CTA; the CTA
//     that completes the fit's last tile runs the public M-step into the other
//     half of a double buffer.
// No CTA waits on another CTA: every hand-off is "last to arrive finishes".
// Waits inside a CTA (mbarriers) are bounded; on expiry the kernel records
// ST_TIMEOUT in the fit's status word and stops.
//
// A tile whose window does not fit in shared memory (a query with more qd than
// the window capacity) is processed "direct": sessions and parameters read
// from global memory, statistics added with FP64 global atomics.
//
// E-step forms.  The reference evaluates PBM/UBM in closed form
// (pbm.cu:191-253, ubm.cu:185-247) and DBN/CCM through a 10x10 table of tail
// click probabilities and 80 log-space factors per session (dbn.cu:207-467,
// ccm.cu:185-478, factor.cu:73-274).  Here the same quantities are computed
// without logarithms:
//   * a rank r before the last click l has a zero z=0 factor, so its gamma/tau
//     update is a ratio independent of the tail: exactly (1, 1) for DBN and for
//     an unclicked CCM rank, (u, u) / (1-u, 1-u) with u = (1-a)t2 / ((1-a)t2 + a t3)
//     for a clicked CCM rank;
//   * for r >= l every tail that starts after r is all-unclicked and, as in the
//     reference, reads the documents at ranks 0, 1, ...; its click-probability
//     product is the r-th prefix of one forward recursion P' = P - a E,
//     E' = E g (1 - a) (E = P * examination), computed once per session;
//   * the conditional examination at ranks >= l comes from the same unnormalised
//     recursion started at the last click (nothing before it feeds it), with a
//     power-of-two rescale when P gets small (per-rank scaling), so no division
//     is needed until the final ratio.
#include <cstdint>
#include <cuda_runtime.h>
#include <cub/block/block_radix_sort.cuh>

#include "common.cuh"
#include "count_step.cuh"
#include "kernels.h"

namespace mcd {

#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------------------
// mbarrier and bulk-copy primitives (PTX ISA: mbarrier, cp.async.bulk)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// try_wait that may suspend the thread until the phase completes or about
// `ns` nanoseconds pass (the suspend-time hint), instead of polling.
__device__ __forceinline__ bool mbar_try_wait_for(uint64_t* bar, uint32_t parity, uint32_t ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Limit of one mbarrier wait, and a tile index whose stage fill declares 16
// bytes more than it copies (-1: none), so that the wait for that stage runs
// out with every copy landed: both set by set_wait_hooks for the tests of the
// timeout path.
__device__ unsigned long long g_wait_limit_ns = 4000000000ull;
__device__ int g_stall_tile = -1;

// Bounded wait: gives up after g_wait_limit_ns of wall-clock time (4 s unless
// a test shortened it; should the timer not advance, after 2^24 rounds of at
// least 256 ns each).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    const uint64_t limit = g_wait_limit_ns;
    for (uint32_t i = 0; i < (1u << 24); i++) {
        if (mbar_try_wait_for(bar, parity, 200000u)) return true;
        if (global_ns() - t0 > limit) break;
        __nanosleep(256);
    }
    atomicOr(status, ST_TIMEOUT);
    return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void workers_sync(int n_threads) {
    asm volatile("bar.sync 1, %0;" ::"r"(n_threads) : "memory");
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }

// ---------------------------------------------------------------------------
// Session / parameter sources and private-statistic sinks
// ---------------------------------------------------------------------------
// Staged tile in shared memory: window-relative indices, rank-major.
struct SmemSrc {
    const uint16_t* rel;   // [10][spad]
    const uint16_t* clk;   // [spad]
    const float* atr;      // window values, index woff + rel
    const float* sat;
    int spad, woff;
    __device__ __forceinline__ bool load(int sl, int (&rl)[MC_R], unsigned& m) const {
#pragma unroll
        for (int r = 0; r < MC_R; r++) rl[r] = rel[r * spad + sl];
        m = clk[sl];
        return true;
    }
    __device__ __forceinline__ bool head(int sl, unsigned& m) const { m = clk[sl]; return true; }
    __device__ __forceinline__ int rel_at(int r, int sl) const { return rel[r * spad + sl]; }
    __device__ __forceinline__ float a(int rl) const { return atr[woff + rl]; }
    __device__ __forceinline__ float s(int rl) const { return sat[woff + rl]; }
};

// Direct tile: sessions and values from global memory (window too large).
struct GlobSrc {
    const int32_t* pidx;
    const uint16_t* clk;
    const float* atr;
    const float* sat;
    int64_t stride, s_begin, qd_begin;
    int qd_count;
    int* status;
    __device__ __forceinline__ bool load(int sl, int (&rl)[MC_R], unsigned& m) const {
        bool ok = true;
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            int64_t p = (int64_t)__ldg(pidx + (int64_t)r * stride + s_begin + sl) - qd_begin;
            rl[r] = (int)p;
            ok = ok && p >= 0 && p < qd_count;
        }
        m = __ldg(clk + s_begin + sl);
        if (!ok) atomicOr(status, ST_BAD_INDEX);
        return ok;
    }
    // Click mask, after checking that all ten indices fall inside the window.
    __device__ __forceinline__ bool head(int sl, unsigned& m) const {
        int rl[MC_R];
        return load(sl, rl, m);
    }
    __device__ __forceinline__ int rel_at(int r, int sl) const {
        return (int)((int64_t)__ldg(pidx + (int64_t)r * stride + s_begin + sl) - qd_begin);
    }
    __device__ __forceinline__ float a(int rl) const { return atr[qd_begin + rl]; }
    __device__ __forceinline__ float s(int rl) const { return sat[qd_begin + rl]; }
};

// Statistic k of window entry rl at bins[k * stride + rl]: each statistic is
// a contiguous array, so the lanes' random entries spread over all 32 banks.
//
// A tile's bins hold 32-bit unsigned fixed point, v * 2^shift added with
// integer atomics, when the tile's shift (fx_scale) allows at least
// FX_MIN_SHIFT fraction bits; otherwise FP32 added with float atomics.
// Shared-memory float atomics are several times the cost of integer ones
// here, and at about nine adds per session they were a third of the launch.
// The fixed-point sum of a bin is exact (integer addition, any order); each
// added value carries one rounding of at most 2^-(shift+1).
//
// Attractiveness values are proportional to the pair's own attractiveness a,
// which ranges over several decades (2e-4 for a pair that is rarely clicked),
// so one absolute step per tile would cost a small-a pair most of its
// relative precision.  Each attractiveness add is therefore scaled by a
// further 2^b, b = 126 - e(a), where e(a) is the biased exponent of a clamped
// below at 126 - kMaxBoost: for a < 1, a 2^b lies in [1/2, 1) (or below 1/2
// when clamped).  Every add of one pair in one tile sees the same a (the
// values of the iteration before), so the bin is one fixed-point sum with
// step 2^-(shift + b).  Each add stores the pair's e(a) in the tile's boost
// slot (the same byte from every add); the M-step takes 2^-(shift + b) in
// place of 2^-shift.  Boost bytes start at 126 (b = 0).  With e in [66, 255]
// and shift in [FX_MIN_SHIFT, 30], the scale's biased exponent
// 127 + shift + 126 - e lies in [18, 217] and the M-step factor's
// 127 - shift + e - 126 in [37, 236]: both normal, built by exponent
// arithmetic, exact.
constexpr int kMaxBoost = 60;

// e(a) << 23: the exponent field of a, at least (126 - kMaxBoost) << 23.
__device__ __forceinline__ int boost_exponent_bits(float a) {
    return max(__float_as_int(a) & 0x7F800000, (126 - kMaxBoost) << 23);
}

// 2^-(shift + b) from x = 2^-shift and a stored e(a) byte.
__device__ __forceinline__ float unboost(float x, int e) { return __int_as_float(__float_as_int(x) + ((e - 126) << 23)); }

struct SmemSink {
    float* bins;
    int stride;
    float scale;     // 2^shift for fixed point, 0 for FP32
    uint8_t* boost;  // e(a) of each window entry of this tile (fixed point)
    __device__ __forceinline__ void add(int rl, int k, float v) const {
        if (scale != 0.0f) atomicAdd(reinterpret_cast<unsigned*>(bins) + k * stride + rl, __float2uint_rn(v * scale));
        else atomicAdd(bins + k * stride + rl, v);
    }
    // Attractiveness statistic (k = 0) of an entry whose attractiveness is a.
    __device__ __forceinline__ void add_a(int rl, float v, float a) const {
        if (scale != 0.0f) {
            const int e = boost_exponent_bits(a);
            boost[rl] = (uint8_t)(e >> 23);
            const float sc = __int_as_float(__float_as_int(scale) + (126 << 23) - e);
            atomicAdd(reinterpret_cast<unsigned*>(bins) + rl, __float2uint_rn(v * sc));
        } else {
            atomicAdd(bins + rl, v);
        }
    }
};

// Fixed point needs sum <= 2^31 for every bin: a bin takes at most one value
// per packed (session, rank) showing its pair, so at most max_occ values (the
// tile's largest packed occurrence count, found when the tile is packed),
// each below 2^ev (fx_value_exponent).  shift = 31 - ceil(log2 max_occ) - ev.
// A boosted attractiveness value is v 2^b = (v / a)(a 2^b) < v / a for a < 1,
// and fx_value_exponent bounds v / a as well as v.
constexpr int FX_MIN_SHIFT = 20;

__device__ __forceinline__ float fx_scale(int max_occ, int ev) {
    if (max_occ <= 0) return 0.0f;
    const int need = (max_occ > 1 ? 32 - __clz(max_occ - 1) : 0) + ev;
    const int shift = 31 - need;
    return shift >= FX_MIN_SHIFT ? __int_as_float((127 + shift) << 23) : 0.0f;
}

// ev with every private statistic value below 2^ev, with a factor 2 of margin
// for rounding.  DBN attractiveness a(1 - eps)/(1 - eps car) and satisfaction
// s/(1 - (1 - s) g car), the CCM unclicked attractiveness term and the PBM /
// UBM terms (a - ae)/(1 - ae) are at most 1 (car <= 1, eps <= 1, e <= 1), and
// so are their attractiveness terms divided by a.  The CCM term of a clicked
// last rank, a / (1 - (t2 (1 - a) + t3 a) car), and that term divided by a,
// are at most 1 / (1 - max(t2, t3)).
__device__ __forceinline__ int fx_value_exponent(int model, const float* pub) {
    if (model != CCM) return 1;
    const float tm = fmaxf(pub[1], pub[2]);
    const float vb = 2.0f * fmaxf(1.0f, __frcp_ru(1.0f - tm));
    const unsigned c = (unsigned)fminf(ceilf(vb), 2147483648.0f);
    return 32 - __clz(c - 1);
}
struct GlobSink {
    double* bins;
    int ns;
    __device__ __forceinline__ void add(int rl, int k, float v) const { atomicAdd(bins + (int64_t)rl * ns + k, (double)v); }
    __device__ __forceinline__ void add_a(int rl, float v, float) const { add(rl, 0, v); }
};

// ---------------------------------------------------------------------------
// PBM (pbm.cu:191-253): unclicked rank -> atr += (a - ae)/(1 - ae),
// exm[r] += (e - ae)/(1 - ae); clicked contributions are constant counts.
// ---------------------------------------------------------------------------
template <class Src, class Sink>
__device__ __forceinline__ void estep_pbm(const Src& src, const Sink& sink, int sl, const float* pub, float (&acc)[MC_R]) {
    int rl[MC_R];
    unsigned m;
    if (!src.load(sl, rl, m)) return;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        if (!((m >> r) & 1u)) {
            float a = src.a(rl[r]);
            float e = pub[r];
            float ae = a * e;
            float inv = __fdividef(1.0f, 1.0f - ae);
            sink.add_a(rl[r], (a - ae) * inv, a);
            acc[r] += (e - ae) * inv;
        }
    }
}

// ---------------------------------------------------------------------------
// UBM (ubm.cu:185-247): examination slot r(r+1)/2 + prev_r (prev = 9 when no
// earlier click).  A slot written by two ranks of one session keeps the later
// rank's value; the counts of written / clicked-written slots are constants.
// ---------------------------------------------------------------------------
template <class Src, class Sink>
__device__ __forceinline__ void estep_ubm(const Src& src, const Sink& sink, int sl, bool valid, const float* pub,
                                          int (&key)[MC_R], float (&var)[MC_R]) {
#pragma unroll
    for (int r = 0; r < MC_R; r++) { key[r] = -1; var[r] = 0.0f; }
    if (!valid) return;
    int rl[MC_R];
    unsigned m;
    if (!src.load(sl, rl, m)) return;
    int slot[MC_R];
    int last = 9;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        slot[r] = r * (r + 1) / 2 + last;
        if ((m >> r) & 1u) last = r;
    }
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        bool alive = true;
#pragma unroll
        for (int r2 = r + 1; r2 < MC_R; r2++) alive = alive && (slot[r2] != slot[r]);
        if (!((m >> r) & 1u)) {
            float a = src.a(rl[r]);
            float e = pub[slot[r]];
            float ae = a * e;
            float inv = __fdividef(1.0f, 1.0f - ae);
            sink.add_a(rl[r], (a - ae) * inv, a);
            if (alive) { key[r] = slot[r]; var[r] = (e - ae) * inv; }
        }
    }
}

// Warp-level reduction of the UBM public statistics: for each rank, each of its
// r + 1 possible slots is summed over the lanes that chose it.
__device__ __forceinline__ void reduce_ubm_public(const int (&key)[MC_R], const float (&var)[MC_R], float* pub_tile) {
    int lane = threadIdx.x & 31;
    // Sessions of a tile are sorted by click mask and the slots depend only on
    // the mask, so most warps hold one key per rank in every lane: one sum
    // and one atomic per rank.
    // Every lane executes every shuffle (no short-circuit around it).
    bool same = true;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        const int k0 = __shfl_sync(FULL_MASK, key[r], 0);
        same &= key[r] == k0;
    }
    if (__all_sync(FULL_MASK, same)) {
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            if (key[r] >= 0) {  // uniform over the warp
                float v = warp_sum(var[r]);
                if (lane == 0) atomicAdd(pub_tile + 2 * key[r], v);
            }
        }
        return;
    }
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
#pragma unroll
        for (int p = 0; p <= r; p++) {
            int cand = r * (r + 1) / 2 + (p == r ? 9 : p);
            unsigned hit = __ballot_sync(FULL_MASK, key[r] == cand);
            if (hit) {
                float v = warp_sum(key[r] == cand ? var[r] : 0.0f);
                if (lane == 0) atomicAdd(pub_tile + 2 * cand, v);
            }
        }
    }
}

// Rescale an unnormalised (P, E) pair by 2^64 when P gets small.
__device__ __forceinline__ void rescale(float& P, float& E) {
    if (P < 5.421010862e-20f) { P *= 1.8446744e19f; E *= 1.8446744e19f; }
}

// ---------------------------------------------------------------------------
// DBN (dbn.cu:207-467)
// ---------------------------------------------------------------------------
template <class Src, class Sink>
__device__ __forceinline__ void estep_dbn(const Src& src, const Sink& sink, int sl, float g, float& gnum, float& gden) {
    unsigned m;
    if (!src.head(sl, m)) return;
    const int l = m ? 31 - __clz(m) : MC_R;
    // Ranks before the last click contribute exactly (1, 1) each, a session
    // without clicks (10, 10) and nothing else: constants of the fit, added to
    // the public M-step at upload (model.cu), so they are skipped here.
    if (l == MC_R) return;
    // Only a, car and the all-unclicked prefix products stay in registers;
    // satisfaction values and window indices are re-read from shared memory.
    float a[MC_R];
    int rls[MC_R];
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        rls[r] = src.rel_at(r, sl);
        a[r] = src.a(rls[r]);
    }
    // car_r = a_r + g (1 - a_r) car_{r+1}, car_10 = 0 (compute_exm_car).
    float car[MC_R + 1];
    car[MC_R] = 0.0f;
#pragma unroll
    for (int r = MC_R - 1; r >= 0; r--) car[r] = a[r] + g * (1.0f - a[r]) * car[r + 1];
    // Prefix products of the all-unclicked tail over documents 0, 1, ...
    float Pu[MC_R];
    Pu[0] = 1.0f;
    {
        float Eu = 1.0f;
#pragma unroll
        for (int j = 0; j < MC_R - 1; j++) {
            Pu[j + 1] = Pu[j] - a[j] * Eu;
            Eu *= g * (1.0f - a[j]);
        }
    }
    // One forward pass: the unconditional examination eps_r at every rank;
    // from the last click on, the conditional examination (P, E), which the
    // click at l restarts (so nothing before l feeds it), and the statistics.
    // Ranks before l depend on the session only through l, so warps of
    // sessions sorted by l take one branch per rank.
    float eps = 1.0f, P = 1.0f, E = 1.0f;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        const int rl = rls[r];
        const float s_r = src.s(rl);
        const float R = (r < MC_R - 1) ? Pu[MC_R - 1 - r] : 1.0f;
        if (r < l) {
        } else if (r == l) {
            // Clicked last rank: satisfaction and gamma.
            float cs = 1.0f - s_r;
            float w = cs * g;
            float B = __fdividef(1.0f, 1.0f - w * (1.0f - R));
            gnum += w * R * B;
            gden += cs * (1.0f - g + g * R) * B;
            sink.add(rl, 1, __fdividef(s_r, 1.0f - cs * g * car[r + 1]));
            E = g * cs;
            P = 1.0f;
        } else {
            // Unclicked rank after the last click (t = g E, u = t (1 - R)).
            const float t = g * E;
            const float u = t * (1.0f - R);
            const float D = __fdividef(1.0f, P - u);
            gnum += t * R * D;
            gden += (E - u) * D;
            sink.add_a(rl, __fdividef(a[r] * (1.0f - eps), 1.0f - eps * car[r]), a[r]);
            P = P - a[r] * E;
            E = t * (1.0f - a[r]);
            rescale(P, E);
        }
        eps *= g * (1.0f - a[r] * s_r);  // g (1 - a) + g a (1 - s)
    }
}

// ---------------------------------------------------------------------------
// CCM (ccm.cu:185-478); tau statistics t[0..5] = (t1 num, t1 den, t2 num,
// t2 den, t3 num, t3 den).
// ---------------------------------------------------------------------------
template <class Src, class Sink>
__device__ __forceinline__ void estep_ccm(const Src& src, const Sink& sink, int sl, float t1, float t2, float t3,
                                          float (&t)[6]) {
    unsigned m;
    if (!src.head(sl, m)) return;
    const int l = m ? 31 - __clz(m) : MC_R;
    if (l == MC_R) return;  // constant contributions only (added at upload)
    float a[MC_R];
    int rls[MC_R];
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        rls[r] = src.rel_at(r, sl);
        a[r] = src.a(rls[r]);
    }
    float car[MC_R + 1];
    car[MC_R] = 0.0f;
#pragma unroll
    for (int r = MC_R - 1; r >= 0; r--) car[r] = a[r] + (1.0f - a[r]) * t1 * car[r + 1];
    float Pu[MC_R];
    Pu[0] = 1.0f;
    {
        float Eu = 1.0f;
#pragma unroll
        for (int j = 0; j < MC_R - 1; j++) {
            Pu[j + 1] = Pu[j] - a[j] * Eu;
            Eu *= t1 * (1.0f - a[j]);
        }
    }
    float eps = 1.0f, P = 1.0f, E = 1.0f;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        const float R = (r < MC_R - 1) ? Pu[MC_R - 1 - r] : 1.0f;
        const float ia = 1.0f - a[r];
        if (r < l) {
            // Before the last click (P, E) is not needed: the click at l
            // restarts it.  A clicked rank: only the tau_2 / tau_3 split
            // depends on the parameters.  An unclicked rank adds exactly
            // (1, 1) to tau_1: a constant of the fit, added at upload.
            if ((m >> r) & 1u) {
                // u = x / (x + y) and 1 - u = y / (x + y), each from its own
                // numerator: 1 - u formed by subtraction loses the small
                // tau_3 share to cancellation when tau_3 is near 0.
                float x = ia * t2, y = a[r] * t3;
                float inv = __fdividef(1.0f, x + y);
                float u = x * inv, v = y * inv;
                t[2] += u; t[3] += u;
                t[4] += v; t[5] += v;
            }
        } else if (r == l) {
            float k2 = 1.0f - t2 * (1.0f - R), k3 = 1.0f - t3 * (1.0f - R);
            float B = __fdividef(1.0f, ia * k2 + a[r] * k3);
            t[2] += ia * t2 * R * B; t[3] += ia * k2 * B;
            t[4] += a[r] * t3 * R * B; t[5] += a[r] * k3 * B;
            float cont = t2 * ia + t3 * a[r];
            sink.add_a(rls[r], __fdividef(a[r], 1.0f - cont * car[r + 1]), a[r]);
            E = cont;
            P = 1.0f;
        } else {
            // Unclicked rank after the last click (te = t1 E, u = te (1 - R)).
            const float te = t1 * E;
            const float u = te * (1.0f - R);
            const float D = __fdividef(1.0f, P - u);
            t[0] += te * R * D;
            t[1] += (E - u) * D;
            sink.add_a(rls[r], __fdividef((1.0f - eps) * a[r], 1.0f - eps * car[r]), a[r]);
            P = P - a[r] * E;
            E = te * ia;
            rescale(P, E);
        }
        eps *= ia * t1 + a[r] * (ia * t2 + a[r] * t3);
    }
}

// ---------------------------------------------------------------------------
// M-step of one qd from its counts and variable statistics.
//   PBM / UBM / DBN attractiveness: (1 + clicks + v0) / (2 + occurrences)
//   CCM attractiveness:             (1 + clicks + v0) / (2 + occurrences + clicks)
//   DBN satisfaction, parity:       (1 + unclicked + v1) / (2 + clicks + 2 unclicked)
//   DBN satisfaction, clean:        (1 + v1) / (2 + clicks)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float clamp_f(float v) { return v < MC_TOP ? v : MC_TOP; }

__device__ __forceinline__ void mstep_qd_f(int model, int mode, uint2 cnt, float v0, float v1, float* atr, float* sat) {
    float occ = (float)cnt.x, clk = (float)cnt.y;
    float den = model == CCM ? 2.0f + occ + clk : 2.0f + occ;
    *atr = clamp_f(__fdividef(1.0f + clk + v0, den));
    if (model == DBN) {
        float un = occ - clk;
        float sn = mode == PARITY ? 1.0f + un + v1 : 1.0f + v1;
        float sd = mode == PARITY ? 2.0f + clk + 2.0f * un : 2.0f + clk;
        *sat = clamp_f(__fdividef(sn, sd));
    }
}

__device__ __forceinline__ void mstep_qd_d(int model, int mode, uint2 cnt, double v0, double v1, float* atr, float* sat) {
    double occ = (double)cnt.x, clk = (double)cnt.y;
    double den = model == CCM ? 2.0 + occ + clk : 2.0 + occ;
    double v = (1.0 + clk + v0) / den;
    *atr = (float)(v < (double)MC_TOP ? v : (double)MC_TOP);
    if (model == DBN) {
        double un = occ - clk;
        double sn = mode == PARITY ? 1.0 + un + v1 : 1.0 + v1;
        double sd = mode == PARITY ? 2.0 + clk + 2.0 * un : 2.0 + clk;
        double w = sn / sd;
        *sat = (float)(w < (double)MC_TOP ? w : (double)MC_TOP);
    }
}

// Public M-step of a fit whose last tile has finished (all threads of one CTA).
__device__ void finalize_public(const FitDev& f, int ctid, int nc, int* s_it) {
    if (ctid == 0) *s_it = *(volatile int*)f.iter;
    workers_sync(nc);
    int nb = (*s_it + 1) & 1;
    for (int k = ctid; k < f.n_pub; k += nc) {
        double num = f.pub_const[2 * k] + ld_cg(f.pub_bins + 2 * k);
        double den = f.pub_const[2 * k + 1] + ld_cg(f.pub_bins + 2 * k + 1);
        double v = num / den;
        f.pub_theta[nb * MC_MAX_PUB + k] = (float)(v < (double)MC_TOP ? v : (double)MC_TOP);
        f.pub_bins[2 * k] = 0.0;
        f.pub_bins[2 * k + 1] = 0.0;
    }
    workers_sync(nc);
    if (ctid == 0) {
        *f.tiles_done = 0;
        __threadfence();
        *(volatile int*)f.iter = *s_it + 1;
    }
}

// Shared-memory layout of one CTA (dynamic part), all 16-byte aligned:
//   bins     float [2 buffers][nb statistics][window_max]; the k-th tile a
//            CTA takes accumulates into buffer k & 1 (nb = 2 when satisfaction
//            is a private statistic, else 1)
//   counts   uint32 [2 slots][window_max + 8]: the window's 16-bit click-count
//            pairs of the k-th tile in slot k & 1, read by its M-step
//   boost    uint8 [2 slots][window_max + 8]: e(a) of the k-th tile's window
//            entries (fixed-point attractiveness bins) in slot k & 1
//   stage s  { uint16 rel[10][spt_pad], uint16 clk[spt_pad],
//              float atr[window_max + 8], float sat[window_max + 8] (DBN) }
//            for s < n_stages
// A slot index k & 1 is an element offset of (window_max + 8) in both the
// count and the boost slots.
struct Layout {
    uint32_t bins_stride, bins_buf, cnt_off, cnt_slot, boost_off, stage_off, stage_bytes, sess_bytes, atr_off, sat_off;
};

__host__ __device__ inline int layout_stats(int model) { return (model == DBN || model < 0) ? 2 : 1; }

__host__ __device__ inline Layout make_layout(int model, int spt, int window_max) {
    Layout L;
    const uint32_t spad = (uint32_t)((spt + 7) & ~7);
    const uint32_t w = (uint32_t)window_max + 8;
    const uint32_t nb = (uint32_t)layout_stats(model);
    L.bins_stride = (uint32_t)window_max;
    L.bins_buf = nb * (uint32_t)window_max;
    L.cnt_off = (2u * L.bins_buf * 4u + 15u) & ~15u;
    L.cnt_slot = w;
    L.boost_off = L.cnt_off + ((2u * w * 4u + 15u) & ~15u);
    L.stage_off = L.boost_off + ((2u * w + 15u) & ~15u);
    L.sess_bytes = 11u * spad * 2u;
    L.atr_off = (L.sess_bytes + 15u) & ~15u;
    L.sat_off = L.atr_off + w * 4u;
    L.stage_bytes = (L.sat_off + (nb > 1 ? w * 4u : 0u) + 15u) & ~15u;
    return L;
}

template <int MODEL>
__device__ __forceinline__ int model_of(const FitDev& f) { return MODEL >= 0 ? MODEL : f.model; }

// qd per lane in one owned-tile M-step item (an item covers 32 * kMQ qd).
constexpr int kMQ = 4;

template <int MODEL>
__global__ void __launch_bounds__(FUSED_THREADS, FUSED_MIN_CTAS)
em_fused_kernel(const FitDev* __restrict__ fits, const TileDev* __restrict__ tiles, int n_tiles,
                const SplitDev* __restrict__ splits, WorkState* ws, int window_max, int spt, int n_stages,
                const CountFitDev* __restrict__ cfits, int n_cfits, int count_blocks) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ double pub_acc[MC_MAX_PUB];
    __shared__ float pub_tile[2][MC_MAX_PUB];
    __shared__ float pub_th[MC_MAX_PUB];
    __shared__ __align__(8) uint64_t full_bar[FUSED_MAX_STAGES], cnt_bar[2];
    __shared__ int stage_tile[FUSED_MAX_STAGES];
    __shared__ TileDev stage_desc[FUSED_MAX_STAGES];   // the staged tile's descriptor
    __shared__ TileDev s_desc[2];                      // the k-th tile's descriptor in slot k & 1
    __shared__ __align__(16) FitDev s_fit[2];          // current fit and the one before
    __shared__ int s_last, s_it, s_abort, s_chunk;

    const Layout L = make_layout(MODEL, spt, window_max);
    float* bins = reinterpret_cast<float*>(smem);
    uint32_t* cnt_slots = reinterpret_cast<uint32_t*>(smem + L.cnt_off);
    const int tid = threadIdx.x;
    const int nc = blockDim.x;  // every warp takes work items
    int* const status = fits[0].status;
    static_assert(sizeof(FitDev) % 8 == 0, "FitDev is copied as 8-byte words");

    if (tid == 0) {
        for (int s = 0; s < n_stages; s++) mbar_init(&full_bar[s], 1);
        mbar_init(&cnt_bar[0], 1);
        mbar_init(&cnt_bar[1], 1);
        s_abort = 0;
    }
    for (int k = tid; k < MC_MAX_PUB; k += blockDim.x) { pub_acc[k] = 0.0; pub_tile[0][k] = 0.0f; pub_tile[1][k] = 0.0f; }
    for (int k = tid; k < (int)(2 * L.bins_buf); k += blockDim.x) bins[k] = 0.0f;
    // Boost bytes start at 126 (b = 0): an entry without attractiveness adds
    // keeps a byte in [66, 255], so its M-step factor stays finite (its bin is 0).
    for (int k = tid; k < (int)(2 * L.cnt_slot); k += blockDim.x) smem[L.boost_off + k] = 126;
    fence_async_shared();
    __syncthreads();

    // Stage filling, by thread 0 only.  The j-th tile this CTA takes goes to
    // stage j % n_stages: bulk copies of its packed sessions and of its
    // window's values, completion on full_bar.  A stage is refilled at the
    // start of the iteration after the one that used it (the barrier ending
    // that iteration is the release), with a tile index fetched one
    // iteration earlier, so the atomic's latency is off the critical path.
    auto fill_stage = [&](int st, int t) {
        fence_async_shared();  // generic reads of the old contents before the async writes
        if (t >= n_tiles) {
            stage_tile[st] = -1;
            mbar_arrive(&full_bar[st]);
            return;
        }
        const TileDev tile = tiles[t];
        stage_tile[st] = t;
        stage_desc[st] = tile;
        if (tile.qd_count > window_max) {  // direct tile: nothing to stage
            mbar_arrive(&full_bar[st]);
            return;
        }
        const FitDev& f = fits[tile.fit];
        const float* f_sat = layout_stats(MODEL) > 1 ? f.sat : nullptr;
        unsigned char* sb = smem + L.stage_off + (size_t)st * L.stage_bytes;
        const int64_t a0 = tile.qd_begin & ~(int64_t)3;
        const int64_t a1 = (tile.qd_begin + tile.qd_count + 3) & ~(int64_t)3;
        const uint32_t wn = (uint32_t)(a1 - a0);
        const uint32_t sess = 11u * (uint32_t)((tile.s_packed + 7) & ~7) * 2u;
        mbar_arrive_expect_tx(&full_bar[st], sess + wn * 4 + (f_sat ? wn * 4 : 0) + (t == g_stall_tile ? 16u : 0u));
        if (sess) bulk_g2s(sb, reinterpret_cast<const unsigned char*>(f.tblk) + tile.blk_off, sess, &full_bar[st]);
        bulk_g2s(sb + L.atr_off, f.atr + a0, wn * 4, &full_bar[st]);
        if (f_sat) bulk_g2s(sb + L.sat_off, f_sat + a0, wn * 4, &full_bar[st]);
    };
    // Tile indices come in runs of consecutive tiles (guided self-scheduling:
    // a run is about 1/4 of the queue left per CTA, at most 16 and at least 1,
    // estimated from the position this CTA last took), so a CTA's tiles are
    // mostly neighbours: one fit, adjacent qd ranges.
    int run_next = 0, run_end = 0;  // thread 0: the current run [run_next, run_end)
    auto take_tile = [&]() -> int {
        if (run_next >= run_end) {
            int r = (n_tiles - run_end) / (4 * (int)gridDim.x);
            r = r < 1 ? 1 : (r > 16 ? 16 : r);
            run_next = (int)atomicAdd(&ws->next_tile, (unsigned)r);
            run_end = run_next + r;
        }
        return run_next++;
    };
    int t_pre = 0;   // thread 0: the next tile index, fetched an iteration ahead
    int filled = 0;  // thread 0: stage fills issued so far
    if (tid == 0) {
        for (int s = 0; s < n_stages; s++) fill_stage(s, take_tile());
        filled = n_stages;
        t_pre = take_tile();
    }

    {
        // ---------------- the tile loop ----------------------------------------
        // Iteration k runs, as one pool of warp-sized items taken from a shared
        // counter, the E-step of the k-th tile (bins buffer k & 1) and the
        // M-step of the (k-1)-th tile (buffer (k-1) & 1, complete since the
        // barrier that ended iteration k-1).  An M-step needs only its bins and
        // the click counts in global memory, so the k-th tile's stage is
        // released at the barrier that ends iteration k.  Tile and fit
        // descriptors are read from shared memory (stage_desc -> s_desc,
        // s_fit), never from global memory inside the loop.
        const int ctid = tid;
        const int lane = tid & 31;
        const int warp = tid >> 5;
        int cur_fit = -1;
        int cur_ev = 1;        // fx_value_exponent of the current fit
        float sc_prev = 0.0f;  // bins scale of the previous tile (0: FP32)
        unsigned cur_count = 0;
        int prev_t = -1;
        int fs = 0, pfs = 0;  // s_fit slots of the current fit and of the previous tile's fit

        auto fold_pub = [&](int buf, const FitDev& f) {  // warp 0: a tile's FP32 partial into FP64
            for (int q = lane; q < 2 * f.n_pub; q += 32) {
                pub_acc[q] += (double)pub_tile[buf][q];
                pub_tile[buf][q] = 0.0f;
            }
        };
        auto flush_fit = [&](const FitDev& f, unsigned count) {
            workers_sync(nc);
            for (int k = ctid; k < 2 * f.n_pub; k += nc) {
                double v = pub_acc[k];
                if (v != 0.0) atomicAdd(f.pub_bins + k, v);
                pub_acc[k] = 0.0;
            }
            __threadfence();
            workers_sync(nc);
            if (ctid == 0) {
                unsigned old = atomicAdd(f.tiles_done, count);
                s_last = (old + count == (unsigned)f.n_tiles);
            }
            workers_sync(nc);
            if (s_last) {
                __threadfence();
                finalize_public(f, ctid, nc, &s_it);
            }
            workers_sync(nc);
        };
        auto next_chunk = [&]() {
            int c = 0;
            if (lane == 0) c = atomicAdd(&s_chunk, 1);
            return __shfl_sync(FULL_MASK, c, 0);
        };

        for (int k = 0;; k++) {
            const int st = k % n_stages;
            const uint32_t round = (uint32_t)(k / n_stages);
            // Every thread observes the completed phase itself.
            if (!mbar_wait(&full_bar[st], round & 1u, status)) s_abort = 1;
            if (ctid == 0) {
                s_chunk = 0;
                s_desc[k & 1] = stage_desc[st];  // slot k & 1 last held tile k - 2, done
            }
            workers_sync(nc);
            if (*(volatile int*)&s_abort) {
                // Copies this CTA issued may still be in flight: the previous
                // tile's counts and the stages filled but not yet consumed.
                if (ctid == 0) {
                    if (prev_t >= 0) mbar_wait(&cnt_bar[(k - 1) & 1], ((uint32_t)(k - 1) >> 1) & 1u, status);
                    for (int j = k; j < filled; j++)
                        mbar_wait(&full_bar[j % n_stages], (uint32_t)(j / n_stages) & 1u, status);
                }
                break;
            }
            const int t = stage_tile[st];
            if (ctid == 0 && k > 0) {
                fill_stage((k - 1) % n_stages, t_pre);  // the (k - 1 + n_stages)-th tile
                filled++;
                t_pre = take_tile();
            }
            TileDev tile{};
            if (t >= 0) tile = s_desc[k & 1];
            TileDev ptile{};
            if (prev_t >= 0) ptile = s_desc[(k - 1) & 1];

            // ---- public partial of the previous tile; fit changes -------------
            bool folded = prev_t < 0;
            if (t >= 0 && tile.fit != cur_fit) {
                if (cur_fit >= 0) {
                    if (warp == 0 && !folded) fold_pub((k - 1) & 1, s_fit[fs]);
                    folded = true;
                    flush_fit(s_fit[fs], cur_count);
                    fs ^= 1;  // the other slot's fit has no tile left in flight
                }
                cur_fit = tile.fit;
                cur_count = 0;
                if (ctid < (int)(sizeof(FitDev) / 8))
                    reinterpret_cast<uint64_t*>(&s_fit[fs])[ctid] = reinterpret_cast<const uint64_t*>(fits + cur_fit)[ctid];
                // Public values are fixed for the whole launch of a fit.
                const FitDev& fg = fits[cur_fit];
                int it = *(volatile int*)fg.iter;
                for (int q = ctid; q < fg.n_pub; q += nc) pub_th[q] = fg.pub_theta[(it & 1) * MC_MAX_PUB + q];
                workers_sync(nc);
                cur_ev = fx_value_exponent(model_of<MODEL>(s_fit[fs]), pub_th);
            }
            if (warp == 0 && !folded) fold_pub((k - 1) & 1, s_fit[pfs]);
            // Click counts of this tile's window for its M-step (next
            // iteration) into count slot k & 1, free since the M-step of tile
            // k - 2 ended with the last barrier.  Every tile advances the
            // slot's barrier by one phase, with or without a copy.
            if (ctid == 0 && t >= 0) {
                if (tile.split < 0) {
                    const int64_t c0 = tile.qd_begin & ~(int64_t)3;
                    const uint32_t cwn = (uint32_t)(((tile.qd_begin + tile.qd_count + 3) & ~(int64_t)3) - c0);
                    fence_async_shared();
                    mbar_arrive_expect_tx(&cnt_bar[k & 1], cwn * 4);
                    bulk_g2s(cnt_slots + (k & 1) * L.cnt_slot, s_fit[fs].cnt16 + c0, cwn * 4, &cnt_bar[k & 1]);
                } else {
                    mbar_arrive(&cnt_bar[k & 1]);
                }
            }

            // ---- the pool: E-step chunks of tile t, then M-step items of prev_t -
            const bool direct = t >= 0 && tile.qd_count > window_max;
            const float sc = (t >= 0 && !direct) ? fx_scale(tile.max_occ, cur_ev) : 0.0f;
            // 2^-shift of the previous tile's bins (exact), 0 for FP32 bins.
            const float inv_prev = sc_prev != 0.0f ? __frcp_rn(sc_prev) : 0.0f;
            const unsigned* ubins_m = reinterpret_cast<const unsigned*>(bins) + ((k - 1) & 1) * L.bins_buf;
            const uint8_t* boost_m = smem + L.boost_off + ((k - 1) & 1) * L.cnt_slot;
            const int n_sess = t < 0 ? 0 : (direct ? tile.s_count : tile.s_packed);
            const int nE = (n_sess + 31) >> 5;
            const int nM = prev_t < 0 ? 0 : (ptile.split >= 0 ? 1 : (ptile.qd_count + 32 * kMQ - 1) / (32 * kMQ));
            if (prev_t >= 0 && ptile.split < 0 &&
                !mbar_wait(&cnt_bar[(k - 1) & 1], ((uint32_t)(k - 1) >> 1) & 1u, status))
                s_abort = 1;  // counts unreliable; the status word already says so
            const uint32_t* cnt_m = cnt_slots + ((k - 1) & 1) * L.cnt_slot + (ptile.qd_begin & 3);
            const int total = nE + nM;
            float* bins_e = bins + (k & 1) * L.bins_buf;
            float* bins_m = bins + ((k - 1) & 1) * L.bins_buf;
            float* pub_k = pub_tile[k & 1];

            // M-step items of the previous tile.  Owned tile: 32 * kMQ qd per item,
            // straight from the bins and the counts, written in place.  Split
            // tile: one item, the warp folds the bins into the query's FP64
            // bins and, if its tile is the query's last, runs the query's M-step.
            auto mstep_item = [&](int mi) {
                const FitDev& pf = s_fit[pfs];
                const int pmodel = model_of<MODEL>(pf);
                const int pns = private_stats(pmodel);
                if (ptile.split < 0) {
                    // kMQ qd per lane; the counts are loaded first, then each qd's update.
                    uint32_t pc[kMQ];
#pragma unroll
                    for (int j = 0; j < kMQ; j++) {
                        const int i = mi * (32 * kMQ) + j * 32 + lane;
                        pc[j] = i < ptile.qd_count ? cnt_m[i] : 0u;
                    }
#pragma unroll
                    for (int j = 0; j < kMQ; j++) {
                        const int i = mi * (32 * kMQ) + j * 32 + lane;
                        if (i < ptile.qd_count) {
                            float v0, v1 = 0.0f;
                            if (inv_prev != 0.0f) {
                                v0 = __uint2float_rn(ubins_m[i]) * unboost(inv_prev, boost_m[i]);
                                if (pns > 1) v1 = __uint2float_rn(ubins_m[L.bins_stride + i]) * inv_prev;
                            } else {
                                v0 = bins_m[i];
                                if (pns > 1) v1 = bins_m[L.bins_stride + i];
                            }
                            bins_m[i] = 0.0f;
                            if (pns > 1) bins_m[L.bins_stride + i] = 0.0f;
                            const int64_t q = ptile.qd_begin + i;
                            mstep_qd_f(pmodel, pf.mode, make_uint2(pc[j] & 0xFFFFu, pc[j] >> 16), v0, v1, pf.atr + q,
                                       pns > 1 ? pf.sat + q : nullptr);
                        }
                    }
                    return;
                }
                const SplitDev sp = splits[ptile.split];
                double* gb = pf.split_bins + sp.bin_offset;
                if (ptile.qd_count <= window_max) {
                    for (int i = lane; i < ptile.qd_count; i += 32)
                        for (int kk = 0; kk < pns; kk++) {
                            const int j = kk * L.bins_stride + i;
                            const float inv = kk == 0 ? unboost(inv_prev, boost_m[i]) : inv_prev;
                            const double v = inv_prev != 0.0f ? (double)ubins_m[j] * (double)inv : (double)bins_m[j];
                            if (v != 0.0) { atomicAdd(gb + (int64_t)i * pns + kk, v); bins_m[j] = 0.0f; }
                        }
                }
                __threadfence();
                __syncwarp();
                unsigned last = 0;
                if (lane == 0) last = atomicAdd(pf.split_count + sp.local, 1u) + 1 == (unsigned)sp.n_tiles;
                last = __shfl_sync(FULL_MASK, last, 0);
                if (last) {
                    __threadfence();
                    for (int i = lane; i < sp.qd_count; i += 32) {
                        int64_t q = sp.qd_begin + i;
                        uint2 cn = __ldg(pf.cnt + q);
                        double v0 = ld_cg(gb + (int64_t)i * pns);
                        double v1 = pns > 1 ? ld_cg(gb + (int64_t)i * pns + 1) : 0.0;
                        mstep_qd_d(pmodel, pf.mode, cn, v0, v1, pf.atr + q, pns > 1 ? pf.sat + q : nullptr);
                        gb[(int64_t)i * pns] = 0.0;
                        if (pns > 1) gb[(int64_t)i * pns + 1] = 0.0;
                    }
                    if (lane == 0) pf.split_count[sp.local] = 0;
                }
            };

            const FitDev& f = s_fit[fs];
            const int model = t >= 0 ? model_of<MODEL>(f) : -1;
            const unsigned char* sb = smem + L.stage_off + (size_t)st * L.stage_bytes;
            const int64_t a0 = tile.qd_begin & ~(int64_t)3;
            SmemSrc ssrc;
            ssrc.spad = (tile.s_packed + 7) & ~7;
            ssrc.rel = reinterpret_cast<const uint16_t*>(sb);
            ssrc.clk = ssrc.rel + 10 * ssrc.spad;
            ssrc.atr = reinterpret_cast<const float*>(sb + L.atr_off);
            ssrc.sat = reinterpret_cast<const float*>(sb + L.sat_off);
            ssrc.woff = (int)(tile.qd_begin - a0);
            GlobSrc gsrc;
            gsrc.pidx = f.pidx; gsrc.clk = f.click; gsrc.atr = f.atr; gsrc.sat = f.sat;
            gsrc.stride = f.stride; gsrc.s_begin = tile.s_begin; gsrc.qd_begin = tile.qd_begin;
            gsrc.qd_count = tile.qd_count; gsrc.status = f.status;
            SmemSink ssink{bins_e, (int)L.bins_stride, sc, smem + L.boost_off + (k & 1) * L.cnt_slot};
            GlobSink gsink{direct ? f.split_bins + splits[tile.split].bin_offset : nullptr,
                           t >= 0 ? private_stats(model) : 1};

            // E-step chunks first (the long dependency chains start early);
            // M-step items fill in behind them.
            auto run_pool = [&](auto&& echunk) {
                for (int c = next_chunk(); c < total; c = next_chunk()) {
                    if (c < nE) echunk((c << 5) + lane);
                    else mstep_item(c - nE);
                }
            };
            if (model == PBM) {
                float acc[MC_R];
#pragma unroll
                for (int r = 0; r < MC_R; r++) acc[r] = 0.0f;
                run_pool([&](int sl) {
                    if (sl < n_sess) {
                        if (direct) estep_pbm(gsrc, gsink, sl, pub_th, acc);
                        else estep_pbm(ssrc, ssink, sl, pub_th, acc);
                    }
                });
#pragma unroll
                for (int r = 0; r < MC_R; r++) {
                    float v = warp_sum(acc[r]);
                    if (lane == 0 && v != 0.0f) atomicAdd(pub_k + 2 * r, v);
                }
            } else if (model == UBM) {
                run_pool([&](int sl) {
                    int key[MC_R];
                    float var[MC_R];
                    if (direct) estep_ubm(gsrc, gsink, sl, sl < n_sess, pub_th, key, var);
                    else estep_ubm(ssrc, ssink, sl, sl < n_sess, pub_th, key, var);
                    reduce_ubm_public(key, var, pub_k);
                });
            } else if (model == DBN) {
                float gn = 0.0f, gd = 0.0f;
                const float g = pub_th[0];
                run_pool([&](int sl) {
                    if (sl < n_sess) {
                        if (direct) estep_dbn(gsrc, gsink, sl, g, gn, gd);
                        else estep_dbn(ssrc, ssink, sl, g, gn, gd);
                    }
                });
                gn = warp_sum(gn);
                gd = warp_sum(gd);
                if (lane == 0) { atomicAdd(pub_k + 0, gn); atomicAdd(pub_k + 1, gd); }
            } else if (model == CCM) {
                float tt[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                const float t1 = pub_th[0], t2 = pub_th[1], t3 = pub_th[2];
                run_pool([&](int sl) {
                    if (sl < n_sess) {
                        if (direct) estep_ccm(gsrc, gsink, sl, t1, t2, t3, tt);
                        else estep_ccm(ssrc, ssink, sl, t1, t2, t3, tt);
                    }
                });
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    float v = warp_sum(tt[q]);
                    if (lane == 0) atomicAdd(pub_k + q, v);
                }
            } else {
                run_pool([&](int) {});
            }
            // A direct tile's statistics went to global memory: order them
            // before the barrier, after which the split counter is raised.
            if (direct) __threadfence();
            workers_sync(nc);
            if (t < 0) break;
            prev_t = t;
            pfs = fs;
            sc_prev = sc;
            cur_count++;
        }
        if (cur_fit >= 0 && !*(volatile int*)&s_abort) flush_fit(s_fit[fs], cur_count);
    }

    // ---------------- count chunks of batched PBM / UBM fits ---------------
    // With the tile queue empty, the CTA takes chunks of kCountChunk pairs of
    // the batch's count-path fits from a second queue (count_step), in the
    // shared memory the stage ring and bins used: no copy is in flight once
    // the tile loop has ended (every stage filled after the last tile holds
    // no tile), and the last M-step ended with the loop's final barrier.
    if (n_cfits > 0) {
        __shared__ int s_cchunk, s_cfit, s_cint[2];
        float* csm = reinterpret_cast<float*>(smem);
        for (;;) {
            __syncthreads();
            if (tid == 0) {
                const int c = *(volatile int*)&s_abort ? count_blocks : (int)atomicAdd(&ws->next_count, 1u);
                s_cchunk = c;
                if (c < count_blocks) {  // the fit owning chunk c: last with blk_begin <= c
                    int lo = 0, hi = n_cfits - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) / 2;
                        if (cfits[mid].blk_begin <= c) lo = mid; else hi = mid - 1;
                    }
                    s_cfit = lo;
                }
            }
            __syncthreads();
            const int c = s_cchunk;
            if (c >= count_blocks) break;
            const CountFitDev cf = cfits[s_cfit];
            const int64_t q0 = (int64_t)(c - cf.blk_begin) * kCountChunk;
            const int64_t q1 = q0 + kCountChunk < cf.n_qd ? q0 + kCountChunk : cf.n_qd;
            count_step<16>(*cf.fit, cf.off, cf.ent, q0 + tid, q1, blockDim.x, (unsigned)cf.n_blocks, csm, s_cint);
        }
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        unsigned e = atomicAdd(&ws->ctas_exited, 1u);
        if (e == gridDim.x - 1) {
            ws->next_tile = 0;
            ws->next_count = 0;
            ws->ctas_exited = 0;
        }
    }
}

cudaError_t set_wait_hooks(unsigned long long wait_limit_ns, int stall_tile) {
    cudaError_t e = cudaMemcpyToSymbol(g_wait_limit_ns, &wait_limit_ns, sizeof wait_limit_ns);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_stall_tile, &stall_tile, sizeof stall_tile);
    return e;
}

size_t fused_smem_bytes(int model, int window_max, int spt, int n_stages, bool with_counts) {
    Layout L = make_layout(model, spt, window_max);
    const size_t tiles = (size_t)L.stage_off + (size_t)n_stages * L.stage_bytes;
    return with_counts && tiles < count_step_smem<16>() ? count_step_smem<16>() : tiles;
}

cudaError_t launch_em_fused(int model, const FitDev* fits, const TileDev* tiles, int n_tiles, const SplitDev* splits,
                            WorkState* ws, int window_max, int spt, int n_stages, int grid, int block,
                            const CountFitDev* cfits, int n_cfits, int count_blocks, cudaStream_t stream) {
    size_t smem = fused_smem_bytes(model, window_max, spt, n_stages, n_cfits > 0);
    switch (model) {
        case PBM: em_fused_kernel<PBM><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max, spt, n_stages, cfits, n_cfits, count_blocks); break;
        case CCM: em_fused_kernel<CCM><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max, spt, n_stages, cfits, n_cfits, count_blocks); break;
        case DBN: em_fused_kernel<DBN><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max, spt, n_stages, cfits, n_cfits, count_blocks); break;
        case UBM: em_fused_kernel<UBM><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max, spt, n_stages, cfits, n_cfits, count_blocks); break;
        default: em_fused_kernel<-1><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max, spt, n_stages, cfits, n_cfits, count_blocks); break;
    }
    return cudaGetLastError();
}

cudaError_t fused_set_smem_limits(size_t bytes) {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(em_fused_kernel<PBM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes))) return e;
    if ((e = cudaFuncSetAttribute(em_fused_kernel<CCM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes))) return e;
    if ((e = cudaFuncSetAttribute(em_fused_kernel<UBM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes))) return e;
    if ((e = cudaFuncSetAttribute(em_fused_kernel<DBN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes))) return e;
    return cudaFuncSetAttribute(em_fused_kernel<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t fused_occupancy(int model, int block, size_t smem, int* blocks_per_sm) {
    switch (model) {
        case PBM: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<PBM>, block, smem);
        case CCM: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<CCM>, block, smem);
        case DBN: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<DBN>, block, smem);
        case UBM: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<UBM>, block, smem);
        default: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<-1>, block, smem);
    }
}

// Packs the tiles' sessions into the staged layout: per tile, rank-major
// uint16 window-relative indices [10][spad] followed by the click masks
// [spad] (padding zeroed), spad = s_packed rounded up to 8.  Sessions are
// ordered by click pattern (DBN: last-click rank; CCM: last-click rank, then
// mask; PBM/UBM: click mask) so the lanes of a warp take the same branches: a
// block radix sort of (pattern << 16 | position) on the pattern bits the
// model's E-step branches on, stable, so equal patterns keep their session
// order.  DBN and CCM sessions without clicks
// carry no variable statistic (their constant contributions are folded in at
// upload) and are left out; s_packed records how many sessions remain.
// Direct tiles keep no packed block.
constexpr int kPackThreads = 256;
constexpr int kPackMinKeys = 4 * kPackThreads;  // keys[] holds at least this many

template <int ITEMS>
using PackSort = cub::BlockRadixSort<uint32_t, kPackThreads, ITEMS, cub::NullType, 5>;

union PackSortStorage {
    typename PackSort<4>::TempStorage s4;
    typename PackSort<8>::TempStorage s8;
    typename PackSort<16>::TempStorage s16;
};

// Sort keys of one tile's sessions, in blocked order (thread t holds
// positions t * ITEMS ...): pattern in the high half, position in the low;
// positions past the tile get the largest key.  Sorted keys go to keys[].
template <int ITEMS>
__device__ __forceinline__ void pack_sort(PackSortStorage& tmp, uint32_t* keys, const uint16_t* click, int64_t s_begin,
                                          int s_count, bool drop_clickless, int begin_bit) {
    uint32_t k[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
        const int i = threadIdx.x * ITEMS + j;
        uint32_t key = 0xFFFFFFFFu;
        if (i < s_count) {
            const unsigned m = click[s_begin + i];
            const uint32_t k16 = drop_clickless ? (m ? (((uint32_t)(31 - __clz(m)) << 10) | m) : 0xFFFFu) : m;
            key = (k16 << 16) | (uint32_t)i;
        }
        k[j] = key;
    }
    // Patterns are below 0x2800; clickless sessions and padding (0xFFFF) read
    // 0x3FFF on bits [16, 30) and sort after them, padding last (stability).
    PackSort<ITEMS>(reinterpret_cast<typename PackSort<ITEMS>::TempStorage&>(tmp)).Sort(k, begin_bit, 30);
#pragma unroll
    for (int j = 0; j < ITEMS; j++) keys[threadIdx.x * ITEMS + j] = k[j];
}

// Three blocks per SM (80 registers): 0.2 ms less per upload of 16M sessions
// than two blocks at the 116 registers the 16-item sort would take.
__global__ void __launch_bounds__(kPackThreads, 3) pack_tiles_kernel(int model, TileDev* tiles, int n_tiles, int window_max,
                                                                 int n_keys, const int32_t* planes, int64_t stride,
                                                                 const uint16_t* click, unsigned char* tblk, int* status) {
    extern __shared__ uint32_t keys[];   // [n_keys] sort keys, then [window_max] occurrence counts
    __shared__ PackSortStorage sort_tmp;
    __shared__ int s_kept, s_max_occ;
    unsigned* occ = keys + n_keys;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const TileDev tile = tiles[t];
        if (tile.qd_count > window_max) continue;
        for (int i = threadIdx.x; i < tile.qd_count; i += blockDim.x) occ[i] = 0;
        const bool drop_clickless = model == DBN || model == CCM;
        // The DBN E-step branches on the last-click rank only: one radix pass
        // over its 4 bits; CCM also on the clicks before it, PBM / UBM on the
        // mask: the 14 pattern bits.
        const int begin_bit = model == DBN ? 26 : 16;
        if (tile.s_count <= 4 * kPackThreads)
            pack_sort<4>(sort_tmp, keys, click, tile.s_begin, tile.s_count, drop_clickless, begin_bit);
        else if (tile.s_count <= 8 * kPackThreads)
            pack_sort<8>(sort_tmp, keys, click, tile.s_begin, tile.s_count, drop_clickless, begin_bit);
        else
            pack_sort<16>(sort_tmp, keys, click, tile.s_begin, tile.s_count, drop_clickless, begin_bit);
        __syncthreads();
        int kept = 0;
        for (int i = threadIdx.x; i < tile.s_count; i += blockDim.x) kept += (keys[i] >> 16) != 0xFFFFu;
        if (threadIdx.x == 0) s_kept = 0;
        __syncthreads();
        atomicAdd(&s_kept, kept);
        __syncthreads();
        // The host sized the tile's block for tile.s_packed sessions.
        int n_kept = s_kept;
        if (n_kept > tile.s_packed) {
            if (threadIdx.x == 0) atomicOr(status, ST_BAD_INDEX);
            n_kept = tile.s_packed;
        }
        const int spad = (n_kept + 7) & ~7;
        uint16_t* rel = reinterpret_cast<uint16_t*>(tblk + tile.blk_off);
        uint16_t* clk = rel + 10 * spad;
        if (threadIdx.x == 0) s_max_occ = 0;
        for (int i = threadIdx.x; i < spad; i += blockDim.x) {
            bool in = i < n_kept;
            int64_t s = tile.s_begin + (in ? (int64_t)(keys[i] & 0xFFFFu) : 0);
            for (int r = 0; r < MC_R; r++) {
                int64_t p = in ? (int64_t)planes[(int64_t)r * stride + s] - tile.qd_begin : 0;
                if (p < 0 || p >= tile.qd_count) { atomicOr(status, ST_BAD_INDEX); p = 0; }
                rel[r * spad + i] = (uint16_t)p;
                if (in) atomicAdd(occ + p, 1u);
            }
            clk[i] = in ? click[s] : (uint16_t)0;
        }
        __syncthreads();
        unsigned mx = 0;
        for (int i = threadIdx.x; i < tile.qd_count; i += blockDim.x) mx = occ[i] > mx ? occ[i] : mx;
        if (mx) atomicMax(&s_max_occ, (int)mx);
        __syncthreads();
        if (threadIdx.x == 0) {
            tiles[t].s_packed = n_kept;
            tiles[t].max_occ = s_max_occ;
        }
        __syncthreads();
    }
}

cudaError_t launch_pack_tiles(int model, TileDev* tiles, int n_tiles, int window_max, int max_tile_sessions, const int32_t* planes,
                              int64_t stride, const uint16_t* click, unsigned char* tblk, int* status, int n_sm,
                              cudaStream_t st) {
    if (n_tiles == 0) return cudaSuccess;
    // keys[] holds 256 x ITEMS keys of the largest class a tile may take.
    int P = kPackMinKeys;
    while (P < max_tile_sessions) P <<= 1;
    int g = n_tiles < 8 * n_sm ? n_tiles : 8 * n_sm;
    const size_t smem = ((size_t)P + (size_t)window_max) * 4;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(pack_tiles_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    pack_tiles_kernel<<<g, kPackThreads, smem, st>>>(model, tiles, n_tiles, window_max, P, planes, stride, click, tblk,
                                                     status);
    return cudaGetLastError();
}

}  // namespace mcd
