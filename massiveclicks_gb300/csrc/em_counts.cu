// PBM EM iteration from per-(qd, rank) counts.
//
// In the PBM E-step (pbm.cu:191-253) an unclicked occurrence of pair qd at
// rank r adds (a - a e_r) / (1 - a e_r) to the qd's attractiveness numerator
// and (e_r - a e_r) / (1 - a e_r) to rank r's examination numerator; a clicked
// occurrence adds constants (folded into the fit's constants at upload).  The
// terms depend on the session only through (qd, r), so per iteration
//   attractiveness numerator of qd = clicks + sum_r n[qd][r] f(a_qd, e_r)
//   examination numerator of r     = clicks at r + sum_qd n[qd][r] h(a_qd, e_r)
// with n[qd][r] = unclicked occurrences of qd at rank r, counted at upload.
// One pass over the qd pairs replaces the pass over sessions: a thread takes a
// qd, evaluates its (at most ten) nonzero terms, and runs its M-step in place.
// Rank partials go through warp sums and an FP64 shared sum per block to one
// FP64 global atomic per rank per block; the block that finishes last runs the
// public M-step into the other half of the double buffer, as the tile kernel
// does, so the fit's state (pub_theta, iter) is the same for both paths.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace mcd {

__global__ void __launch_bounds__(256) pbm_counts_kernel(const FitDev* __restrict__ fp,
                                                         const uint32_t* __restrict__ ucnt) {
    __shared__ float e[MC_R];
    __shared__ double blk[MC_R];
    __shared__ int s_last, s_it;
    const FitDev& f = *fp;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) s_it = *(volatile int*)f.iter;
    __syncthreads();
    if (tid < MC_R) {
        e[tid] = f.pub_theta[(s_it & 1) * MC_MAX_PUB + tid];
        blk[tid] = 0.0;
    }
    __syncthreads();
    float acc[MC_R];
#pragma unroll
    for (int r = 0; r < MC_R; r++) acc[r] = 0.0f;
    const int64_t n_qd = f.n_qd;
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + tid; q < n_qd; q += step) {
        const float a = f.atr[q];
        const uint2 c = f.cnt[q];
        const uint2* row = reinterpret_cast<const uint2*>(ucnt + q * MC_R);  // 40 B per qd, 8-byte aligned
        uint32_t n[MC_R];
#pragma unroll
        for (int j = 0; j < MC_R / 2; j++) {
            const uint2 v = __ldg(row + j);
            n[2 * j] = v.x;
            n[2 * j + 1] = v.y;
        }
        float v0 = 0.0f;
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            if (n[r]) {
                const float ae = a * e[r];
                const float inv = __fdividef(1.0f, 1.0f - ae);
                const float w = (float)n[r] * inv;
                v0 += w * (a - ae);
                acc[r] += w * (e[r] - ae);
            }
        }
        // M-step (parity and clean agree for PBM): (1 + clicks + v0) / (2 + occurrences).
        const float v = __fdividef(1.0f + (float)c.y + v0, 2.0f + (float)c.x);
        f.atr[q] = v < MC_TOP ? v : MC_TOP;
    }
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        float s = acc[r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s != 0.0f) atomicAdd(&blk[r], (double)s);
    }
    __syncthreads();
    if (tid < MC_R && blk[tid] != 0.0) atomicAdd(f.pub_bins + 2 * tid, blk[tid]);
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(f.tiles_done, 1u) + 1 == gridDim.x;
    __syncthreads();
    if (!s_last) return;
    // Last block: public M-step of the examination parameters.
    __threadfence();
    const int nb = (s_it + 1) & 1;
    if (tid < f.n_pub) {
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

cudaError_t launch_pbm_counts(const FitDev* fit, const uint32_t* ucnt, int64_t n_qd, int n_sm, cudaStream_t st) {
    int64_t blocks = (n_qd + 255) / 256;
    int g = (int)(blocks < 8 * n_sm ? blocks : 8 * n_sm);
    if (g < 1) g = 1;
    pbm_counts_kernel<<<g, 256, 0, st>>>(fit, ucnt);
    return cudaGetLastError();
}

}  // namespace mcd
