// One block's share of a PBM / UBM iteration from counts per (qd, key):
// shared by the count kernels (em_counts.cu) and the persistent tile kernel,
// which takes count chunks of batched fits as a second kind of work item
// (em_fused.cu).  See em_counts.cu for the count format.
#ifndef MCLICKS_COUNT_STEP_CUH
#define MCLICKS_COUNT_STEP_CUH

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace mcd {

// Shared memory a count step needs: 64 public values and COPIES copies of 8
// warps' public bins.
template <int COPIES>
__host__ __device__ constexpr size_t count_step_smem() {
    return (64 + (size_t)8 * MC_UBM_SLOTS * COPIES) * sizeof(float);
}

// After a block has added its public partial sums: the last of the fit's
// n_blocks blocks to finish runs the public M-step into the other half of the
// double buffer, clears the bins and the block counter and advances iter.
__device__ __forceinline__ void count_public_finish(const FitDev& f, int s_it, unsigned n_blocks, int* s_last) {
    const int tid = threadIdx.x;
    const int n_pub = f.n_pub;
    __threadfence();
    __syncthreads();
    if (tid == 0) *s_last = atomicAdd(f.tiles_done, 1u) + 1 == n_blocks;
    __syncthreads();
    if (!*s_last) return;
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

// The block takes qd q_first, q_first + q_step, ... below q_end; the fit's
// iteration is done by n_blocks blocks, and the last of them to finish runs
// the public M-step.  COPIES copies of each warp's public bins: lane l adds
// to copy l % COPIES, so only lanes that share a copy and a key meet on one
// shared-memory address.  sm: count_step_smem<COPIES>() bytes of shared
// memory, 16-byte aligned; s_int: two shared ints.  Blocks of 64 to 256
// threads.
template <int COPIES>
__device__ __forceinline__ void count_step(const FitDev& f, const uint32_t* __restrict__ off,
                                           const uint32_t* __restrict__ ent, int64_t q_first, int64_t q_end,
                                           int64_t q_step, unsigned n_blocks, float* sm, int* s_int) {
    float* e = sm;                        // [64]
    float* wbin = sm + 64;                // [8][MC_UBM_SLOTS][COPIES]
    const int tid = threadIdx.x, warp = tid >> 5;
    const int n_pub = f.n_pub;
    if (tid == 0) s_int[0] = *(volatile int*)f.iter;
    for (int k = tid; k < 8 * MC_UBM_SLOTS * COPIES; k += blockDim.x) wbin[k] = 0.0f;
    __syncthreads();
    const int s_it = s_int[0];
    if (tid < 64) e[tid] = tid < n_pub ? f.pub_theta[(s_it & 1) * MC_MAX_PUB + tid] : 0.0f;
    __syncthreads();
    float* mybin = wbin + (warp * MC_UBM_SLOTS) * COPIES + (tid & (COPIES - 1));
    for (int64_t q = q_first; q < q_end; q += q_step) {
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
            if (x & 1u) atomicAdd(mybin + k * COPIES, w * (ek - ae));
        }
        // M-step, PBM and UBM in both modes: (1 + clicks + v0) / (2 + occurrences).
        const float v = __fdividef(1.0f + (float)c.y + v0, 2.0f + (float)c.x);
        f.atr[q] = v < MC_TOP ? v : MC_TOP;
    }
    __syncthreads();
    if (tid < n_pub) {
        double s = 0.0;
        for (int w = 0; w < 8; w++)
            for (int c = 0; c < COPIES; c++) s += (double)wbin[(w * MC_UBM_SLOTS + tid) * COPIES + c];
        if (s != 0.0) atomicAdd(f.pub_bins + 2 * tid, s);
    }
    count_public_finish(f, s_it, n_blocks, s_int + 1);
    __syncthreads();  // the caller may reuse sm
}

}  // namespace mcd

#endif  // MCLICKS_COUNT_STEP_CUH
