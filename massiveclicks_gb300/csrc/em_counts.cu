// PBM and UBM EM iterations from counts per (qd, statistic key).
//
// In the PBM and UBM E-steps (pbm.cu:191-253, ubm.cu:185-247) an unclicked
// occurrence of pair qd under examination parameter e_k adds
// (a - a e_k) / (1 - a e_k) to the qd's attractiveness numerator and, unless
// a later rank of the same session writes the same UBM slot (last write wins),
// (e_k - a e_k) / (1 - a e_k) to parameter k's numerator; a clicked occurrence
// adds constants (folded into the fit's constants at upload).  The key k is
// the rank (PBM) or the examination slot r(r+1)/2 + previous click (UBM), so
// the terms depend on the session only through (qd, k, alive) and
//   numerator of qd = clicks + sum over entries count * f(a_qd, e_k)
//   numerator of k  = constants + sum over alive entries count * h(a_qd, e_k).
// At upload every unclicked occurrence becomes a 64-bit key (qd, k, alive);
// sorting and run-length encoding them gives the entries of each qd (CSR).
// An iteration is one pass over the qd pairs: a thread takes a qd, evaluates
// its entries and runs its M-step in place.  The public terms go into
// per-warp shared bins, then FP64 block sums, then one FP64 global atomic per
// parameter per block; the block that finishes last runs the public M-step
// into the other half of the double buffer, as the tile kernel does, so the
// fit's state (pub_theta, iter) is the same for both paths.
#include <cstdint>
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>

#include "common.cuh"
#include "kernels.h"

namespace mcd {

constexpr unsigned long long kNoKey = ~0ull;  // clicked occurrence: sorts after every key
constexpr uint32_t kMaxCount = 1u << 25;      // count field of an entry

// Keys ((qd << 7) | (k << 1) | alive) of the unclicked occurrences of sessions
// [0, n); position s * 10 + r.
__global__ void count_keys_kernel(int64_t n, int64_t stride, const int32_t* __restrict__ planes,
                                  const uint16_t* __restrict__ click, int model, unsigned long long* __restrict__ keys) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += step) {
        const unsigned m = click[s];
        int slot[MC_R];
        int last = 9;
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            slot[r] = model == PBM ? r : r * (r + 1) / 2 + last;
            if ((m >> r) & 1u) last = r;
        }
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            unsigned long long key = kNoKey;
            if (!((m >> r) & 1u)) {
                bool alive = true;
#pragma unroll
                for (int r2 = r + 1; r2 < MC_R; r2++) alive = alive && slot[r2] != slot[r];
                const int64_t p = planes[(int64_t)r * stride + s];
                key = ((unsigned long long)p << 7) | ((unsigned long long)slot[r] << 1) | (alive ? 1ull : 0ull);
            }
            keys[s * MC_R + r] = key;
        }
    }
}

// Entry i = (count << 7) | (k << 1) | alive of run i; flags a count too large.
__global__ void count_entries_kernel(int64_t runs, const unsigned long long* __restrict__ uniq,
                                     const uint32_t* __restrict__ counts, uint32_t* __restrict__ ent, int* overflow) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < runs; i += step) {
        const uint32_t c = counts[i];
        if (c >= kMaxCount) atomicOr(overflow, 1);
        ent[i] = (c << 7) | (uint32_t)(uniq[i] & 0x7Full);
    }
}

// off[q] = first run whose qd is >= q, q in [0, n_qd].
__global__ void count_offsets_kernel(int64_t n_qd, int64_t runs, const unsigned long long* __restrict__ uniq,
                                     uint32_t* __restrict__ off) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q <= n_qd; q += step) {
        int64_t lo = 0, hi = runs;
        while (lo < hi) {
            const int64_t mid = (lo + hi) / 2;
            if ((int64_t)(uniq[mid] >> 7) < q) lo = mid + 1; else hi = mid;
        }
        off[q] = (uint32_t)lo;
    }
}

static int grid_for(int64_t n, int n_sm) {
    int64_t b = (n + 255) / 256;
    int g = (int)(b < 16 * n_sm ? b : 16 * n_sm);
    return g < 1 ? 1 : g;
}

template <class T>
static cudaError_t tmp_alloc(T** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T) > 0 ? count * sizeof(T) : 1);
}

cudaError_t build_counts(int model, int64_t n, int64_t stride, int64_t n_qd, const int32_t* planes, const uint16_t* click,
                         int n_sm, cudaStream_t st, uint32_t** off_out, uint32_t** ent_out, int64_t* n_entries,
                         int* usable) {
    *off_out = nullptr;
    *ent_out = nullptr;
    *n_entries = 0;
    *usable = 0;
    const int64_t nk = n * MC_R;
    if (nk >= ((int64_t)1 << 32) || n_qd >= ((int64_t)1 << 56)) return cudaSuccess;  // keep the tile path
    unsigned long long *keys = nullptr, *sorted = nullptr, *uniq = nullptr;
    uint32_t* counts = nullptr;
    int* d_small = nullptr;  // [0] overflow flag, [1..2] run count (int64)
    void* temp = nullptr;
    uint32_t *off = nullptr, *ent = nullptr;
    cudaError_t e = cudaSuccess;
    auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    auto release = [&]() {
        cudaFree(keys); cudaFree(sorted); cudaFree(uniq); cudaFree(counts); cudaFree(d_small); cudaFree(temp);
    };
    // Real keys are below 2^end_bit - 1 once 2^(end_bit - 7) - 1 >= n_qd, so
    // the sentinel (all ones) still sorts last on the low end_bit bits.
    int end_bit = 8;
    while (end_bit < 64 && (((int64_t)1 << (end_bit - 7)) - 1) < n_qd) end_bit++;
    ck(tmp_alloc(&keys, (size_t)nk));
    ck(tmp_alloc(&sorted, (size_t)nk));
    ck(tmp_alloc(&uniq, (size_t)nk));
    ck(tmp_alloc(&counts, (size_t)nk));
    ck(tmp_alloc(&d_small, 4));
    size_t sort_bytes = 0, rle_bytes = 0;
    if (e == cudaSuccess) {
        ck(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, keys, sorted, (int64_t)nk, 0, end_bit, st));
        ck(cub::DeviceRunLengthEncode::Encode(nullptr, rle_bytes, sorted, uniq, counts,
                                              reinterpret_cast<int64_t*>(d_small + 2), (int64_t)nk, st));
        ck(cudaMalloc(&temp, sort_bytes > rle_bytes ? sort_bytes : rle_bytes));
    }
    if (e != cudaSuccess) { release(); return e; }
    ck(cudaMemsetAsync(d_small, 0, 16, st));
    count_keys_kernel<<<grid_for(n, n_sm), 256, 0, st>>>(n, stride, planes, click, model, keys);
    ck(cudaGetLastError());
    ck(cub::DeviceRadixSort::SortKeys(temp, sort_bytes, keys, sorted, (int64_t)nk, 0, end_bit, st));
    ck(cub::DeviceRunLengthEncode::Encode(temp, rle_bytes, sorted, uniq, counts,
                                          reinterpret_cast<int64_t*>(d_small + 2), (int64_t)nk, st));
    int64_t runs = 0;
    ck(cudaMemcpyAsync(&runs, d_small + 2, 8, cudaMemcpyDeviceToHost, st));
    ck(cudaStreamSynchronize(st));
    if (e != cudaSuccess) { release(); return e; }
    // The clicked occurrences form the last run (the sentinel), if any.
    unsigned long long last_key = 0;
    if (runs > 0) {
        ck(cudaMemcpy(&last_key, uniq + runs - 1, 8, cudaMemcpyDeviceToHost));
        if (last_key == kNoKey) runs--;
    }
    ck(tmp_alloc(&off, (size_t)n_qd + 1));
    ck(tmp_alloc(&ent, (size_t)(runs > 0 ? runs : 1)));
    if (e == cudaSuccess) {
        count_entries_kernel<<<grid_for(runs, n_sm), 256, 0, st>>>(runs, uniq, counts, ent, d_small);
        ck(cudaGetLastError());
        count_offsets_kernel<<<grid_for(n_qd + 1, n_sm), 256, 0, st>>>(n_qd, runs, uniq, off);
        ck(cudaGetLastError());
    }
    int overflow = 0;
    ck(cudaMemcpyAsync(&overflow, d_small, 4, cudaMemcpyDeviceToHost, st));
    ck(cudaStreamSynchronize(st));
    release();
    if (e != cudaSuccess || overflow) {
        cudaFree(off);
        cudaFree(ent);
        return e;  // on overflow: success without the count path
    }
    *off_out = off;
    *ent_out = ent;
    *n_entries = runs;
    *usable = 1;
    return cudaSuccess;
}

// One thread per qd: its entries, its M-step in place; the public terms of the
// alive entries go into per-warp shared bins.  (A warp per 32 qd with
// coalesced entry reads, a next-qd prefetch and register bins for PBM were
// all slower at 22.6M qd: the kernel is bound by the shared-memory pipe and
// lane divergence, not by DRAM latency.)
__global__ void __launch_bounds__(256, 8) em_counts_kernel(const FitDev* __restrict__ fp, const uint32_t* __restrict__ off,
                                                           const uint32_t* __restrict__ ent) {
    __shared__ float e[64];
    __shared__ float wbin[8][64];
    __shared__ int s_last, s_it;
    const FitDev& f = *fp;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int n_pub = f.n_pub;
    if (tid == 0) s_it = *(volatile int*)f.iter;
    for (int k = tid; k < 8 * 64; k += blockDim.x) (&wbin[0][0])[k] = 0.0f;
    __syncthreads();
    if (tid < 64) e[tid] = tid < n_pub ? f.pub_theta[(s_it & 1) * MC_MAX_PUB + tid] : 0.0f;
    __syncthreads();
    float* mybin = wbin[warp];
    const int64_t n_qd = f.n_qd;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + tid; q < n_qd; q += step) {
        const float a = f.atr[q];
        const uint2 c = f.cnt[q];
        const uint32_t i1 = __ldg(off + q + 1);
        float v0 = 0.0f;
        for (uint32_t i = __ldg(off + q); i < i1; i++) {
            const uint32_t x = __ldg(ent + i);
            const int k = (int)((x >> 1) & 63u);
            const float ek = e[k];
            const float ae = a * ek;
            const float w = (float)(x >> 7) * __fdividef(1.0f, 1.0f - ae);
            v0 += w * (a - ae);
            if (x & 1u) atomicAdd(mybin + k, w * (ek - ae));
        }
        // M-step, PBM and UBM in both modes: (1 + clicks + v0) / (2 + occurrences).
        const float v = __fdividef(1.0f + (float)c.y + v0, 2.0f + (float)c.x);
        f.atr[q] = v < MC_TOP ? v : MC_TOP;
    }
    __syncthreads();
    if (tid < n_pub) {
        double s = 0.0;
        for (int w = 0; w < 8; w++) s += (double)wbin[w][tid];
        if (s != 0.0) atomicAdd(f.pub_bins + 2 * tid, s);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(f.tiles_done, 1u) + 1 == gridDim.x;
    __syncthreads();
    if (!s_last) return;
    // Last block: public M-step.
    __threadfence();
    const int nb = (s_it + 1) & 1;
    if (tid < n_pub) {
        const double num = f.pub_const[2 * tid] + __ldcg(f.pub_bins + 2 * tid);
        const double den = f.pub_const[2 * tid + 1] + __ldcg(f.pub_bins + 2 * tid + 1);
        const double v = num / den;
        f.pub_theta[nb * MC_MAX_PUB + tid] = (float)(v < (double)MC_TOP ? v : (double)MC_TOP);
        f.pub_bins[2 * tid] = 0.0;
        f.pub_bins[2 * tid + 1] = 0.0;
    }
    __syncthreads();
    if (tid == 0) {
        *f.tiles_done = 0;
        __threadfence();
        *(volatile int*)f.iter = s_it + 1;
    }
}

cudaError_t launch_em_counts(const FitDev* fit, const uint32_t* off, const uint32_t* ent, int64_t n_qd, int n_sm,
                             cudaStream_t st) {
    const int64_t blocks = (n_qd + 255) / 256;
    int g = (int)(blocks < 8 * n_sm ? blocks : 8 * n_sm);
    if (g < 1) g = 1;
    em_counts_kernel<<<g, 256, 0, st>>>(fit, off, ent);
    return cudaGetLastError();
}

}  // namespace mcd
