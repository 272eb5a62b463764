// Fused EM iteration: E-step, statistics reduction and M-step in one
// persistent kernel launch per iteration.
//
// Work: a queue of session tiles (host-built, see model.cu).  A CTA takes the
// next tile, zeroes a shared-memory bin per qd of the tile's window, runs the
// E-step with one thread per session, adds each private statistic into its bin
// (shared-memory atomics) and each public statistic into registers, then:
//   * owned tile (whole queries): M-step for the window straight from the bins,
//     written in place (no other tile reads those parameters);
//   * split tile (part of a large query): bins are folded into FP64 global bins
//     and the last tile of that query runs its M-step;
//   * public statistics: warp shuffles -> one shared FP32 partial per tile ->
//     an FP64 per-CTA accumulator -> one FP64 global atomic per bin per CTA;
//     the CTA that completes the fit's last tile runs the public M-step into
//     the other half of a double buffer.
// Nothing waits on anything: every hand-off is "last to arrive finishes".
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
//     recursion restarted at each click, with a power-of-two rescale when P gets
//     small (per-rank scaling), so no division is needed until the final ratio.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace mcd {

#define FULL_MASK 0xffffffffu

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }

struct TileCtx {
    const FitDev* f;
    int64_t qd_begin;
    int qd_count;
    bool wide;          // window too large for shared memory: FP64 global bins directly
    float* sbins;       // shared bins, [qd_count * ns]
    double* gbins;      // global FP64 bins of a wide tile
    int ns;             // private statistics per qd
    const float* pub;   // current public values
};

__device__ __forceinline__ void add_private(const TileCtx& c, int rel, int k, float v) {
    if (c.wide) atomicAdd(c.gbins + (int64_t)rel * c.ns + k, (double)v);
    else atomicAdd(c.sbins + rel * c.ns + k, v);
}

// Loads the ten parameter indices of session s relative to the window;
// returns false (and flags the fit) if one falls outside it.
__device__ __forceinline__ bool load_rel(const TileCtx& c, int64_t s, int (&rel)[MC_R]) {
    const FitDev& f = *c.f;
    bool ok = true;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        int64_t p = (int64_t)__ldg(f.pidx + (int64_t)r * f.stride + s) - c.qd_begin;
        rel[r] = (int)p;
        ok = ok && (p >= 0) && (p < c.qd_count);
    }
    if (!ok) atomicOr(f.status, ST_BAD_INDEX);
    return ok;
}

// ---------------------------------------------------------------------------
// PBM (pbm.cu:191-253): unclicked rank -> atr += (a - ae)/(1 - ae),
// exm[r] += (e - ae)/(1 - ae); clicked contributions are constant counts.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void estep_pbm(const TileCtx& c, int64_t s, float (&pub)[MC_R]) {
    int rel[MC_R];
    if (!load_rel(c, s, rel)) return;
    const FitDev& f = *c.f;
    unsigned m = __ldg(f.click + s);
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        if (!((m >> r) & 1u)) {
            float a = f.atr[c.qd_begin + rel[r]];
            float e = c.pub[r];
            float ae = a * e;
            float inv = __fdividef(1.0f, 1.0f - ae);
            add_private(c, rel[r], 0, (a - ae) * inv);
            pub[r] += (e - ae) * inv;
        }
    }
}

// ---------------------------------------------------------------------------
// UBM (ubm.cu:185-247): examination slot r(r+1)/2 + prev_r (prev = 9 when no
// earlier click).  A slot written by two ranks of one session keeps the later
// rank's value; the counts of written / clicked-written slots are constants.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void estep_ubm(const TileCtx& c, int64_t s, bool valid, int (&key)[MC_R], float (&var)[MC_R]) {
#pragma unroll
    for (int r = 0; r < MC_R; r++) { key[r] = -1; var[r] = 0.0f; }
    if (!valid) return;
    int rel[MC_R];
    if (!load_rel(c, s, rel)) return;
    const FitDev& f = *c.f;
    unsigned m = __ldg(f.click + s);
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
            float a = f.atr[c.qd_begin + rel[r]];
            float e = c.pub[slot[r]];
            float ae = a * e;
            float inv = __fdividef(1.0f, 1.0f - ae);
            add_private(c, rel[r], 0, (a - ae) * inv);
            if (alive) { key[r] = slot[r]; var[r] = (e - ae) * inv; }
        }
    }
}

// Warp-level reduction of the UBM public statistics: for each rank, each of its
// r + 1 possible slots is summed over the lanes that chose it.
__device__ __forceinline__ void reduce_ubm_public(const int (&key)[MC_R], const float (&var)[MC_R], float* pub_tile) {
    int lane = threadIdx.x & 31;
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
__device__ __forceinline__ void estep_dbn(const TileCtx& c, int64_t s, float& gnum, float& gden) {
    int rel[MC_R];
    if (!load_rel(c, s, rel)) return;
    const FitDev& f = *c.f;
    unsigned m = __ldg(f.click + s);
    int l = m ? 31 - __clz(m) : MC_R;
    float a[MC_R], sv[MC_R];
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        a[r] = f.atr[c.qd_begin + rel[r]];
        sv[r] = f.sat[c.qd_begin + rel[r]];
    }
    float g = c.pub[0];
    // Ranks before the last click: (1, 1) each (all ten for a click-less session).
    gnum += (float)l;
    gden += (float)l;
    if (l == MC_R) return;  // no clicks: no attractiveness / satisfaction terms either

    // Unconditional examination (compute_exm_car) and car, backwards.
    float eps[MC_R], car[MC_R + 1];
    eps[0] = 1.0f;
#pragma unroll
    for (int r = 0; r < MC_R - 1; r++) eps[r + 1] = eps[r] * (g * (1.0f - a[r]) + g * a[r] * (1.0f - sv[r]));
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

    // Conditional examination up to rank l (restarting at every click).
    float P = 1.0f, E = 1.0f;
#pragma unroll
    for (int j = 0; j < MC_R; j++) {
        if (j < l) {
            if ((m >> j) & 1u) { E = g * (1.0f - sv[j]); P = 1.0f; }
            else { P = P - a[j] * E; E = E * g * (1.0f - a[j]); rescale(P, E); }
        }
    }
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        float R = (r < MC_R - 1) ? Pu[MC_R - 1 - r] : 1.0f;
        if (r == l) {
            // Clicked last rank: satisfaction and gamma.
            float cs = 1.0f - sv[r];
            float w = cs * g;
            float B = __fdividef(1.0f, 1.0f - w * (1.0f - R));
            gnum += w * R * B;
            gden += cs * (1.0f - g + g * R) * B;
            add_private(c, rel[r], 1, __fdividef(sv[r], 1.0f - cs * g * car[r + 1]));
            E = g * cs;
            P = 1.0f;
        } else if (r > l) {
            // Unclicked rank after the last click.
            float D = __fdividef(1.0f, P - g * E * (1.0f - R));
            gnum += g * R * E * D;
            gden += E * (1.0f - g * (1.0f - R)) * D;
            add_private(c, rel[r], 0, __fdividef(a[r] * (1.0f - eps[r]), 1.0f - eps[r] * car[r]));
            P = P - a[r] * E;
            E = E * g * (1.0f - a[r]);
            rescale(P, E);
        }
    }
}

// ---------------------------------------------------------------------------
// CCM (ccm.cu:185-478); tau statistics t[0..5] = (t1 num, t1 den, t2 num,
// t2 den, t3 num, t3 den).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void estep_ccm(const TileCtx& c, int64_t s, float (&t)[6]) {
    int rel[MC_R];
    if (!load_rel(c, s, rel)) return;
    const FitDev& f = *c.f;
    unsigned m = __ldg(f.click + s);
    int l = m ? 31 - __clz(m) : MC_R;
    float a[MC_R];
#pragma unroll
    for (int r = 0; r < MC_R; r++) a[r] = f.atr[c.qd_begin + rel[r]];
    float t1 = c.pub[0], t2 = c.pub[1], t3 = c.pub[2];

    // Ranks before the last click.
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        if (r < l) {
            if ((m >> r) & 1u) {
                float x = (1.0f - a[r]) * t2, y = a[r] * t3;
                float u = __fdividef(x, x + y);
                t[2] += u; t[3] += u;
                t[4] += 1.0f - u; t[5] += 1.0f - u;
            } else {
                t[0] += 1.0f; t[1] += 1.0f;
            }
        }
    }
    if (l == MC_R) return;

    float eps[MC_R], car[MC_R + 1];
    eps[0] = 1.0f;
#pragma unroll
    for (int r = 0; r < MC_R - 1; r++)
        eps[r + 1] = eps[r] * ((1.0f - a[r]) * t1 + a[r] * ((1.0f - a[r]) * t2 + a[r] * t3));
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
    float P = 1.0f, E = 1.0f;
#pragma unroll
    for (int j = 0; j < MC_R; j++) {
        if (j < l) {
            if ((m >> j) & 1u) { E = t2 * (1.0f - a[j]) + t3 * a[j]; P = 1.0f; }
            else { P = P - a[j] * E; E = E * t1 * (1.0f - a[j]); rescale(P, E); }
        }
    }
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        float R = (r < MC_R - 1) ? Pu[MC_R - 1 - r] : 1.0f;
        if (r == l) {
            float ia = 1.0f - a[r];
            float k2 = 1.0f - t2 * (1.0f - R), k3 = 1.0f - t3 * (1.0f - R);
            float B = __fdividef(1.0f, ia * k2 + a[r] * k3);
            t[2] += ia * t2 * R * B; t[3] += ia * k2 * B;
            t[4] += a[r] * t3 * R * B; t[5] += a[r] * k3 * B;
            float cont = t2 * ia + t3 * a[r];
            add_private(c, rel[r], 0, __fdividef(a[r], 1.0f - cont * car[r + 1]));
            E = cont;
            P = 1.0f;
        } else if (r > l) {
            float D = __fdividef(1.0f, P - t1 * E * (1.0f - R));
            t[0] += t1 * R * E * D;
            t[1] += E * (1.0f - t1 * (1.0f - R)) * D;
            add_private(c, rel[r], 0, __fdividef((1.0f - eps[r]) * a[r], 1.0f - eps[r] * car[r]));
            P = P - a[r] * E;
            E = E * t1 * (1.0f - a[r]);
            rescale(P, E);
        }
    }
}

// ---------------------------------------------------------------------------
// M-step of one qd from its counts and variable statistics.
//   PBM / UBM / DBN attractiveness: (1 + clicks + v0) / (2 + occurrences)
//   CCM attractiveness:             (1 + clicks + v0) / (2 + occurrences + clicks)
//   DBN satisfaction, parity:       (1 + unclicked + v1) / (2 + clicks + 2 unclicked)
//   DBN satisfaction, clean:        (1 + v1) / (2 + clicks)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void mstep_qd(int model, int mode, uint2 cnt, T v0, T v1, float* atr, float* sat) {
    T occ = (T)cnt.x, clk = (T)cnt.y;
    T den = model == CCM ? T(2) + occ + clk : T(2) + occ;
    T v = (T(1) + clk + v0) / den;
    *atr = (float)(v < (T)MC_TOP ? v : (T)MC_TOP);
    if (model == DBN) {
        T un = occ - clk;
        T sn = mode == PARITY ? T(1) + un + v1 : T(1) + v1;
        T sd = mode == PARITY ? T(2) + clk + T(2) * un : T(2) + clk;
        T w = sn / sd;
        *sat = (float)(w < (T)MC_TOP ? w : (T)MC_TOP);
    }
}

// Public M-step of a fit whose last tile has finished (run by one CTA).
__device__ void finalize_public(const FitDev& f) {
    __shared__ int s_it;
    if (threadIdx.x == 0) s_it = *(volatile int*)f.iter;
    __syncthreads();
    int nb = (s_it + 1) & 1;
    for (int k = threadIdx.x; k < f.n_pub; k += blockDim.x) {
        double num = f.pub_const[2 * k] + ld_cg(f.pub_bins + 2 * k);
        double den = f.pub_const[2 * k + 1] + ld_cg(f.pub_bins + 2 * k + 1);
        double v = num / den;
        f.pub_theta[nb * MC_MAX_PUB + k] = (float)(v < (double)MC_TOP ? v : (double)MC_TOP);
        f.pub_bins[2 * k] = 0.0;
        f.pub_bins[2 * k + 1] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *f.tiles_done = 0;
        __threadfence();
        *(volatile int*)f.iter = s_it + 1;
    }
}

template <int MODEL>
__device__ __forceinline__ int model_of(const FitDev& f) { return MODEL >= 0 ? MODEL : f.model; }

template <int MODEL>
__global__ void __launch_bounds__(512) em_fused_kernel(const FitDev* __restrict__ fits, const TileDev* __restrict__ tiles,
                                                       int n_tiles, const SplitDev* __restrict__ splits,
                                                       WorkState* ws, int window_max) {
    extern __shared__ __align__(16) float sbins[];
    __shared__ double pub_acc[MC_MAX_PUB];
    __shared__ float pub_tile[MC_MAX_PUB];
    __shared__ float pub_th[MC_MAX_PUB];
    __shared__ int s_tile;
    __shared__ int s_last;

    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    const int lane = tid & 31;
    for (int k = tid; k < MC_MAX_PUB; k += nthr) { pub_acc[k] = 0.0; pub_tile[k] = 0.0f; }
    int cur_fit = -1;
    unsigned cur_count = 0;

    auto flush_fit = [&](int fit_id, unsigned count) {
        const FitDev& f = fits[fit_id];
        __syncthreads();
        for (int k = tid; k < 2 * f.n_pub; k += nthr) {
            double v = pub_acc[k];
            if (v != 0.0) atomicAdd(f.pub_bins + k, v);
            pub_acc[k] = 0.0;
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            unsigned old = atomicAdd(f.tiles_done, count);
            s_last = (old + count == (unsigned)f.n_tiles);
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            finalize_public(f);
        }
        __syncthreads();
    };

    for (;;) {
        if (tid == 0) s_tile = (int)atomicAdd(&ws->next_tile, 1u);
        __syncthreads();
        const int t = s_tile;
        __syncthreads();
        if (t >= n_tiles) break;
        const TileDev tile = tiles[t];
        if (tile.fit != cur_fit) {
            if (cur_fit >= 0) flush_fit(cur_fit, cur_count);
            cur_fit = tile.fit;
            cur_count = 0;
        }
        const FitDev& f = fits[tile.fit];
        const int model = model_of<MODEL>(f);
        const int ns = private_stats(model);
        const int n_pub = f.n_pub;

        TileCtx c;
        c.f = &f;
        c.qd_begin = tile.qd_begin;
        c.qd_count = tile.qd_count;
        c.wide = tile.qd_count > window_max;
        c.sbins = sbins;
        c.ns = ns;
        c.gbins = tile.split >= 0 ? f.split_bins + splits[tile.split].bin_offset : nullptr;
        c.pub = pub_th;
        if (!c.wide)
            for (int i = tid; i < tile.qd_count * ns; i += nthr) sbins[i] = 0.0f;
        {
            int it = *(volatile int*)f.iter;
            for (int k = tid; k < n_pub; k += nthr) pub_th[k] = f.pub_theta[(it & 1) * MC_MAX_PUB + k];
        }
        __syncthreads();

        // ---- E-step over the tile's sessions -------------------------------
        const int rounds = (tile.s_count + nthr - 1) / nthr;
        if (model == PBM) {
            float pub[MC_R];
#pragma unroll
            for (int r = 0; r < MC_R; r++) pub[r] = 0.0f;
            for (int rd = 0; rd < rounds; rd++) {
                int sl = rd * nthr + tid;
                if (sl < tile.s_count) estep_pbm(c, tile.s_begin + sl, pub);
            }
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                float v = warp_sum(pub[r]);
                if (lane == 0 && v != 0.0f) atomicAdd(pub_tile + 2 * r, v);
            }
        } else if (model == UBM) {
            for (int rd = 0; rd < rounds; rd++) {
                int sl = rd * nthr + tid;
                int key[MC_R];
                float var[MC_R];
                estep_ubm(c, tile.s_begin + sl, sl < tile.s_count, key, var);
                reduce_ubm_public(key, var, pub_tile);
            }
        } else if (model == DBN) {
            float gn = 0.0f, gd = 0.0f;
            for (int rd = 0; rd < rounds; rd++) {
                int sl = rd * nthr + tid;
                if (sl < tile.s_count) estep_dbn(c, tile.s_begin + sl, gn, gd);
            }
            gn = warp_sum(gn);
            gd = warp_sum(gd);
            if (lane == 0) { atomicAdd(pub_tile + 0, gn); atomicAdd(pub_tile + 1, gd); }
        } else {
            float tt[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int rd = 0; rd < rounds; rd++) {
                int sl = rd * nthr + tid;
                if (sl < tile.s_count) estep_ccm(c, tile.s_begin + sl, tt);
            }
#pragma unroll
            for (int k = 0; k < 6; k++) {
                float v = warp_sum(tt[k]);
                if (lane == 0) atomicAdd(pub_tile + k, v);
            }
        }
        __syncthreads();

        // ---- M-step of the window ------------------------------------------
        if (tile.split < 0) {
            for (int i = tid; i < tile.qd_count; i += nthr) {
                int64_t q = tile.qd_begin + i;
                uint2 cn = __ldg(f.cnt + q);
                float v0 = sbins[i * ns];
                float v1 = ns > 1 ? sbins[i * ns + 1] : 0.0f;
                mstep_qd<float>(model, f.mode, cn, v0, v1, f.atr + q, ns > 1 ? f.sat + q : nullptr);
            }
        } else {
            const SplitDev sp = splits[tile.split];
            double* gb = f.split_bins + sp.bin_offset;
            if (!c.wide) {
                for (int i = tid; i < tile.qd_count * ns; i += nthr) {
                    float v = sbins[i];
                    if (v != 0.0f) atomicAdd(gb + i, (double)v);
                }
            }
            __threadfence();
            __syncthreads();
            if (tid == 0) {
                unsigned old = atomicAdd(f.split_count + tile.split, 1u);
                s_last = (old + 1 == (unsigned)sp.n_tiles);
            }
            __syncthreads();
            if (s_last) {
                __threadfence();
                for (int i = tid; i < sp.qd_count; i += nthr) {
                    int64_t q = sp.qd_begin + i;
                    uint2 cn = __ldg(f.cnt + q);
                    double v0 = ld_cg(gb + (int64_t)i * ns);
                    double v1 = ns > 1 ? ld_cg(gb + (int64_t)i * ns + 1) : 0.0;
                    mstep_qd<double>(model, f.mode, cn, v0, v1, f.atr + q, ns > 1 ? f.sat + q : nullptr);
                    gb[(int64_t)i * ns] = 0.0;
                    if (ns > 1) gb[(int64_t)i * ns + 1] = 0.0;
                }
                if (tid == 0) f.split_count[tile.split] = 0;
            }
        }

        // ---- fold the tile's public partial into the CTA's FP64 accumulator
        for (int k = tid; k < 2 * n_pub; k += nthr) {
            pub_acc[k] += (double)pub_tile[k];
            pub_tile[k] = 0.0f;
        }
        cur_count++;
        __syncthreads();
    }
    if (cur_fit >= 0) flush_fit(cur_fit, cur_count);
    if (tid == 0) {
        __threadfence();
        unsigned e = atomicAdd(&ws->ctas_exited, 1u);
        if (e == gridDim.x - 1) {
            ws->next_tile = 0;
            ws->ctas_exited = 0;
        }
    }
}

size_t fused_smem_bytes(int model, int window_max) {
    int ns = model < 0 ? 2 : private_stats(model);
    return (size_t)window_max * ns * sizeof(float);
}

cudaError_t launch_em_fused(int model, const FitDev* fits, const TileDev* tiles, int n_tiles, const SplitDev* splits,
                            WorkState* ws, int window_max, int grid, int block, cudaStream_t stream) {
    size_t smem = fused_smem_bytes(model, window_max);
    switch (model) {
        case PBM: em_fused_kernel<PBM><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max); break;
        case CCM: em_fused_kernel<CCM><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max); break;
        case DBN: em_fused_kernel<DBN><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max); break;
        case UBM: em_fused_kernel<UBM><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max); break;
        default: em_fused_kernel<-1><<<grid, block, smem, stream>>>(fits, tiles, n_tiles, splits, ws, window_max); break;
    }
    return cudaGetLastError();
}

cudaError_t fused_set_smem_limits(int window_max) {
    cudaError_t e = cudaSuccess;
    size_t b2 = fused_smem_bytes(-1, window_max), b1 = fused_smem_bytes(PBM, window_max);
    e = cudaFuncSetAttribute(em_fused_kernel<PBM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b1);
    if (e) return e;
    e = cudaFuncSetAttribute(em_fused_kernel<CCM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b1);
    if (e) return e;
    e = cudaFuncSetAttribute(em_fused_kernel<UBM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b1);
    if (e) return e;
    e = cudaFuncSetAttribute(em_fused_kernel<DBN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b2);
    if (e) return e;
    return cudaFuncSetAttribute(em_fused_kernel<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b2);
}

cudaError_t fused_occupancy(int model, int block, int window_max, int* blocks_per_sm) {
    size_t smem = fused_smem_bytes(model, window_max);
    switch (model) {
        case PBM: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<PBM>, block, smem);
        case CCM: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<CCM>, block, smem);
        case DBN: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<DBN>, block, smem);
        case UBM: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<UBM>, block, smem);
        default: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, em_fused_kernel<-1>, block, smem);
    }
}

}  // namespace mcd
