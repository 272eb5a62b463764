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
#include <cub/device/device_scan.cuh>
#include <thrust/iterator/reverse_iterator.h>

#include "common.cuh"
#include "count_step.cuh"
#include "devmem.h"
#include "kernels.h"

namespace mcd {

constexpr uint32_t kMaxCount = 1u << 25;  // count field of an entry

// Keys ((qd << 7) | (k << 1) | alive) of the unclicked occurrences; a clicked
// occurrence gets the all-ones key, which sorts after every real key.  The key
// of (session s, rank r) sits at r * n + s: the sort does not care where a key
// starts, and rank-major positions make the stores coalesced.
template <class K>
__global__ void count_keys_kernel(int64_t n, int64_t stride, const int32_t* __restrict__ planes,
                                  const uint16_t* __restrict__ click, int model, K* __restrict__ keys) {
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
            K key = ~K(0);
            if (!((m >> r) & 1u)) {
                bool alive = true;
#pragma unroll
                for (int r2 = r + 1; r2 < MC_R; r2++) alive = alive && slot[r2] != slot[r];
                const K p = (K)planes[(int64_t)r * stride + s];
                key = (p << 7) | ((K)slot[r] << 1) | (alive ? K(1) : K(0));
            }
            keys[(int64_t)r * n + s] = key;
        }
    }
}

// Entry i = (count << 7) | (k << 1) | alive of run i; flags a count too large.
template <class K>
__global__ void count_entries_kernel(int64_t runs, const K* __restrict__ uniq, const uint32_t* __restrict__ counts,
                                     uint32_t* __restrict__ ent, int* overflow) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < runs; i += step) {
        const uint32_t c = counts[i];
        if (c >= kMaxCount) atomicOr(overflow, 1);
        ent[i] = (c << 7) | (uint32_t)(uniq[i] & K(0x7F));
    }
}

// off[q] = first run whose qd is >= q, for q in [0, n_qd], in two parallel
// steps: the first run of each qd writes its index at off[qd] (the others
// hold ~0, off[n_qd] = runs), then a suffix minimum fills each gap with the
// next qd's value.
template <class K>
__global__ void count_first_run_kernel(int64_t runs, const K* __restrict__ uniq, uint32_t* __restrict__ off) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < runs; i += step) {
        const int64_t q = (int64_t)(uniq[i] >> 7);
        if (i == 0 || (int64_t)(uniq[i - 1] >> 7) != q) off[q] = (uint32_t)i;
    }
}

struct MinU32 {
    __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a < b ? a : b; }
};

// PBM: dense[qd * 10 + rank] = count of run i (every PBM key is alive and
// unique per (qd, rank)); flags a count above 65535.
template <class K>
__global__ void count_dense_kernel(int64_t runs, const K* __restrict__ uniq, const uint32_t* __restrict__ counts,
                                   uint16_t* __restrict__ dense, int* overflow) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < runs; i += step) {
        const uint32_t c = counts[i];
        if (c > 0xFFFFu) { atomicOr(overflow, 1); continue; }
        const int64_t q = (int64_t)(uniq[i] >> 7);
        const int r = (int)((uniq[i] >> 1) & K(63));
        dense[q * MC_R + r] = (uint16_t)c;
    }
}

static int grid_for(int64_t n, int n_sm) {
    int64_t b = (n + 255) / 256;
    int g = (int)(b < 16 * n_sm ? b : 16 * n_sm);
    return g < 1 ? 1 : g;
}

template <class T>
static cudaError_t tmp_alloc(T** p, size_t count) {
    return mch::dev_alloc(reinterpret_cast<void**>(p), count * sizeof(T) > 0 ? count * sizeof(T) : 1);
}

// K = uint32_t while qd < 2^25 - 1 (the all-ones key stays above every real
// key), else uint64_t.  The sort runs over the low end_bit bits, the fewest
// that hold every real key below 2^end_bit - 1.
template <class K>
static cudaError_t build_counts_t(int model, int64_t n, int64_t stride, int64_t n_qd, const int32_t* planes,
                                  const uint16_t* click, int n_sm, cudaStream_t st, uint32_t** off_out,
                                  uint32_t** ent_out, int64_t* n_entries, uint16_t** dense_out, int* usable) {
    const int64_t nk = n * MC_R;
    K *keys = nullptr, *alt = nullptr;
    uint32_t* counts = nullptr;
    int64_t* d_small = nullptr;  // [0] run count, [1] overflow flags: CSR (low word), dense (high word)
    void* temp = nullptr;
    uint32_t *off = nullptr, *ent = nullptr;
    uint16_t* dense = nullptr;
    cudaError_t e = cudaSuccess;
    auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    auto release = [&]() {  // after the stream has drained
        cudaStreamSynchronize(st);
        mch::dev_free(keys); mch::dev_free(alt); mch::dev_free(counts); mch::dev_free(d_small); mch::dev_free(temp);
    };
    int end_bit = 8;
    while (end_bit < (int)(8 * sizeof(K)) && (((int64_t)1 << (end_bit - 7)) - 1) < n_qd) end_bit++;
    ck(tmp_alloc(&keys, (size_t)nk));
    ck(tmp_alloc(&alt, (size_t)nk));
    ck(tmp_alloc(&counts, (size_t)nk));
    ck(tmp_alloc(&d_small, 2));
    size_t sort_bytes = 0, rle_bytes = 0;
    cub::DoubleBuffer<K> db(keys, alt);
    if (e == cudaSuccess) {
        ck(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, db, (int64_t)nk, 0, end_bit, st));
        ck(cub::DeviceRunLengthEncode::Encode(nullptr, rle_bytes, keys, alt, counts, d_small, (int64_t)nk, st));
        ck(mch::dev_alloc(&temp, sort_bytes > rle_bytes ? sort_bytes : rle_bytes));
    }
    if (e != cudaSuccess) { release(); return e; }
    ck(cudaMemsetAsync(d_small, 0, 16, st));
    count_keys_kernel<K><<<grid_for(n, n_sm), 256, 0, st>>>(n, stride, planes, click, model, keys);
    ck(cudaGetLastError());
    ck(cub::DeviceRadixSort::SortKeys(temp, sort_bytes, db, (int64_t)nk, 0, end_bit, st));
    K* sorted = db.Current();
    K* uniq = db.Alternate();
    ck(cub::DeviceRunLengthEncode::Encode(temp, rle_bytes, sorted, uniq, counts, d_small, (int64_t)nk, st));
    int64_t runs = 0;
    ck(cudaMemcpyAsync(&runs, d_small, 8, cudaMemcpyDeviceToHost, st));
    ck(cudaStreamSynchronize(st));
    if (e != cudaSuccess) { release(); return e; }
    // The clicked occurrences form the last run (the all-ones key), if any.
    if (runs > 0) {
        K last_key = 0;
        ck(cudaMemcpy(&last_key, uniq + runs - 1, sizeof(K), cudaMemcpyDeviceToHost));
        if (last_key == ~K(0)) runs--;
    }
    const uint32_t runs32 = (uint32_t)runs;  // < 2^32: n * 10 < 2^32 entries at most
    ck(tmp_alloc(&off, (size_t)n_qd + 1));
    ck(tmp_alloc(&ent, (size_t)(runs > 0 ? runs : 1)));
    if (model == PBM && dense_out) ck(tmp_alloc(&dense, (size_t)n_qd * MC_R));
    int* overflow = reinterpret_cast<int*>(d_small + 1);
    if (e == cudaSuccess) {
        ck(cudaMemsetAsync(off, 0xFF, (size_t)n_qd * sizeof(uint32_t), st));
        ck(cudaMemcpyAsync(off + n_qd, &runs32, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        count_entries_kernel<K><<<grid_for(runs, n_sm), 256, 0, st>>>(runs, uniq, counts, ent, overflow);
        ck(cudaGetLastError());
        count_first_run_kernel<K><<<grid_for(runs, n_sm), 256, 0, st>>>(runs, uniq, off);
        ck(cudaGetLastError());
        {
            auto rev = thrust::make_reverse_iterator(off + n_qd + 1);
            size_t scan_bytes = 0;
            ck(cub::DeviceScan::InclusiveScan(nullptr, scan_bytes, rev, rev, MinU32(), (int64_t)n_qd + 1, st));
            void* scan_tmp = nullptr;
            ck(mch::dev_alloc(&scan_tmp, scan_bytes ? scan_bytes : 1));
            if (e == cudaSuccess)
                ck(cub::DeviceScan::InclusiveScan(scan_tmp, scan_bytes, rev, rev, MinU32(), (int64_t)n_qd + 1, st));
            if (scan_tmp) {
                cudaStreamSynchronize(st);
                mch::dev_free(scan_tmp);
            }
        }
        if (dense) {
            ck(cudaMemsetAsync(dense, 0, (size_t)n_qd * MC_R * sizeof(uint16_t), st));
            count_dense_kernel<K><<<grid_for(runs, n_sm), 256, 0, st>>>(runs, uniq, counts, dense, overflow + 1);
            ck(cudaGetLastError());
        }
    }
    int flags[2] = {0, 0};
    ck(cudaMemcpyAsync(flags, overflow, 8, cudaMemcpyDeviceToHost, st));
    ck(cudaStreamSynchronize(st));
    release();
    if (e != cudaSuccess || flags[0]) {
        mch::dev_free(off);
        mch::dev_free(ent);
        mch::dev_free(dense);
        return e;  // on overflow: success without the count path
    }
    if (flags[1]) {  // a count above 16 bits: the entries only
        mch::dev_free(dense);
        dense = nullptr;
    }
    *off_out = off;
    *ent_out = ent;
    *n_entries = runs;
    if (dense_out) *dense_out = dense;
    *usable = 1;
    return cudaSuccess;
}

cudaError_t build_counts(int model, int64_t n, int64_t stride, int64_t n_qd, const int32_t* planes, const uint16_t* click,
                         int n_sm, cudaStream_t st, uint32_t** off_out, uint32_t** ent_out, int64_t* n_entries,
                         uint16_t** dense_out, int* usable) {
    *off_out = nullptr;
    *ent_out = nullptr;
    *n_entries = 0;
    if (dense_out) *dense_out = nullptr;
    *usable = 0;
    if (n * MC_R >= ((int64_t)1 << 32) || n_qd >= ((int64_t)1 << 56)) return cudaSuccess;  // keep the tile path
    if (n_qd <= ((int64_t)1 << 25) - 2)
        return build_counts_t<uint32_t>(model, n, stride, n_qd, planes, click, n_sm, st, off_out, ent_out, n_entries,
                                        dense_out, usable);
    return build_counts_t<unsigned long long>(model, n, stride, n_qd, planes, click, n_sm, st, off_out, ent_out, n_entries,
                                              dense_out, usable);
}

// One thread per qd: its entries, its M-step in place; the public terms of the
// alive entries go into per-warp shared bins.  (A warp per 32 qd with
// coalesced entry reads, a next-qd prefetch and register bins for PBM were
// all slower at 22.6M qd: the kernel is bound by the shared-memory pipe and
// lane divergence, not by DRAM latency.)
//
// One block's share of an iteration: count_step (count_step.cuh) over static
// shared memory.
template <int COPIES>
__device__ __forceinline__ void count_iteration(const FitDev& f, const uint32_t* __restrict__ off,
                                                const uint32_t* __restrict__ ent, int64_t q_first, int64_t q_end,
                                                int64_t q_step, unsigned n_blocks) {
    __shared__ __align__(16) float sm[count_step_smem<COPIES>() / sizeof(float)];
    __shared__ int s_int[2];
    count_step<COPIES>(f, off, ent, q_first, q_end, q_step, n_blocks, sm, s_int);
}

// One fit: blocks stride over its qd.
template <int COPIES>
__global__ void __launch_bounds__(256) em_counts_kernel(const FitDev* __restrict__ fp, const uint32_t* __restrict__ off,
                                                        const uint32_t* __restrict__ ent) {
    const FitDev& f = *fp;
    count_iteration<COPIES>(f, off, ent, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, f.n_qd,
                            (int64_t)gridDim.x * blockDim.x, gridDim.x);
}

// Grid of a grid-stride count launch: enough blocks for one qd per thread, at
// most blocks_per_sm per SM.
static int count_grid(int64_t n_qd, int block, int blocks_per_sm, int n_sm) {
    const int64_t blocks = (n_qd + block - 1) / block;
    const int64_t cap = (int64_t)blocks_per_sm * n_sm;
    const int g = (int)(blocks < cap ? blocks : cap);
    return g < 1 ? 1 : g;
}

bool count_shape_valid(const CountShape& c, bool dense) {
    if (c.block < 64 || c.block > 256 || c.block % 32 || c.blocks_per_sm < 1 || c.blocks_per_sm > 32) return false;
    return dense || c.copies == 4 || c.copies == 8 || c.copies == 16;
}

cudaError_t launch_em_counts(const FitDev* fit, const uint32_t* off, const uint32_t* ent, int64_t n_qd, int n_sm,
                             const CountShape& c, cudaStream_t st) {
    const int g = count_grid(n_qd, c.block, c.blocks_per_sm, n_sm);
    switch (c.copies) {
        case 4: em_counts_kernel<4><<<g, c.block, 0, st>>>(fit, off, ent); break;
        case 16: em_counts_kernel<16><<<g, c.block, 0, st>>>(fit, off, ent); break;
        default: em_counts_kernel<8><<<g, c.block, 0, st>>>(fit, off, ent); break;
    }
    return cudaGetLastError();
}

// PBM from dense counts: row q holds the unclicked occurrences of qd q at
// ranks 0..9 (uint16), so every thread runs the same ten-rank loop and the
// rank sums stay in registers (no shared atomics); warp sums, then FP64 block
// sums, then one global atomic per rank per block.
__global__ void __launch_bounds__(256) em_counts_pbm_dense_kernel(const FitDev* __restrict__ fp,
                                                                    const uint16_t* __restrict__ dense) {
    __shared__ float wsum[8][MC_R];
    __shared__ float e[MC_R];  // read with one address per warp (broadcast)
    __shared__ int s_it;
    const FitDev& f = *fp;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_it = *(volatile int*)f.iter;
    __syncthreads();
    if (tid < MC_R) e[tid] = f.pub_theta[(s_it & 1) * MC_MAX_PUB + tid];
    __syncthreads();
    float acc[MC_R];
#pragma unroll
    for (int r = 0; r < MC_R; r++) acc[r] = 0.0f;
    const int64_t n_qd = f.n_qd;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + tid; q < n_qd; q += step) {
        const float a = f.atr[q];
        const uint2 c = f.cnt[q];
        const uint32_t* row = reinterpret_cast<const uint32_t*>(dense + q * MC_R);  // 20 B, 4-byte aligned
        uint32_t w2[MC_R / 2];
#pragma unroll
        for (int j = 0; j < MC_R / 2; j++) w2[j] = __ldg(row + j);
        float v0 = 0.0f;
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            const uint32_t k = (r & 1) ? (w2[r >> 1] >> 16) : (w2[r >> 1] & 0xFFFFu);
            if (k) {
                const float ae = a * e[r];
                const float w = (float)k * __fdividef(1.0f, 1.0f - ae);
                v0 += w * (a - ae);
                acc[r] += w * (e[r] - ae);
            }
        }
        const float v = __fdividef(1.0f + (float)c.y + v0, 2.0f + (float)c.x);
        f.atr[q] = v < MC_TOP ? v : MC_TOP;
    }
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        float v = acc[r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) wsum[warp][r] = v;
    }
    __syncthreads();
    if (tid < MC_R) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += (double)wsum[w][tid];
        if (s != 0.0) atomicAdd(f.pub_bins + 2 * tid, s);
    }
    __shared__ int s_last;
    count_public_finish(f, s_it, gridDim.x, &s_last);
}

cudaError_t launch_em_counts_pbm_dense(const FitDev* fit, const uint16_t* dense, int64_t n_qd, int n_sm,
                                       const CountShape& c, cudaStream_t st) {
    em_counts_pbm_dense_kernel<<<count_grid(n_qd, c.block, c.blocks_per_sm, n_sm), c.block, 0, st>>>(fit, dense);
    return cudaGetLastError();
}

// Many fits in one launch: fit i owns blocks [blk_begin, blk_begin + n_blocks),
// each a contiguous chunk of kCountChunk of its qd, so a block serves one fit
// and the fit's last block runs its public M-step.  (16 bin copies here, 8 in
// the one-fit kernel: the batch's short-lived blocks gained from more copies,
// the one-fit kernel's long grid-stride blocks lost occupancy to them.)
__global__ void __launch_bounds__(256, 6) em_counts_batch_kernel(const CountFitDev* __restrict__ fits, int n_fits) {
    __shared__ int s_fit;
    if (threadIdx.x == 0) {
        int lo = 0, hi = n_fits - 1;  // last fit with blk_begin <= blockIdx.x
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (fits[mid].blk_begin <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
        }
        s_fit = lo;
    }
    __syncthreads();
    const CountFitDev cf = fits[s_fit];
    const int64_t q0 = (int64_t)((int)blockIdx.x - cf.blk_begin) * kCountChunk;
    const int64_t q1 = q0 + kCountChunk < cf.n_qd ? q0 + kCountChunk : cf.n_qd;
    count_iteration<16>(*cf.fit, cf.off, cf.ent, q0 + threadIdx.x, q1, blockDim.x, (unsigned)cf.n_blocks);
}

cudaError_t launch_em_counts_batch(const CountFitDev* fits, int n_fits, int total_blocks, cudaStream_t st) {
    if (n_fits == 0 || total_blocks == 0) return cudaSuccess;
    em_counts_batch_kernel<<<total_blocks, 256, 0, st>>>(fits, n_fits);
    return cudaGetLastError();
}

}  // namespace mcd
