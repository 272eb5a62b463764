// Log-likelihood and perplexity of a session set on the GPU: the reference's
// LogLikelihood::evaluate / Perplexity::evaluate (click_models/evaluation.cpp:25-66)
// with the per-model probabilities of get_log_conditional_click_probs and
// get_full_click_probs (pbm.cu:376-439, ubm.cu:376-468, dbn.cu:611-683,
// ccm.cu:600-660).  A doc unseen in training (index -1) takes attractiveness and
// satisfaction 1/2.  Per-rank probabilities are FP32; the per-session and
// global sums are FP64.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace mcd {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) eval_kernel(EvalArgs A) {
    __shared__ double red[MC_R + 1][8];
    double acc[MC_R + 1];
#pragma unroll
    for (int k = 0; k <= MC_R; k++) acc[k] = 0.0;
    const float* pub = A.iter ? A.pub + (*A.iter & 1) * MC_MAX_PUB : A.pub;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < A.n; s += stride) {
        unsigned m = A.click[s];
        float a[MC_R], sv[MC_R];
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            int p = A.pidx[(int64_t)r * A.stride + s];
            bool seen = p >= 0 && p < A.n_qd;
            a[r] = seen ? A.atr[p] : 0.5f;
            sv[r] = (A.model == DBN) ? (seen ? A.sat[p] : 0.5f) : 0.f;
        }
        float lc[MC_R], fp[MC_R];
        if (A.model == PBM || A.model == UBM) {
            int prev[MC_R];
            int last = MC_R - 1;
#pragma unroll
            for (int r = 0; r < MC_R; r++) { prev[r] = last; if ((m >> r) & 1u) last = r; }
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                float e = A.model == PBM ? pub[r] : pub[r * (r + 1) / 2 + prev[r]];
                float ae = a[r] * e;
                lc[r] = ((m >> r) & 1u) ? logf(ae) : logf(1.f - ae);
            }
            if (A.model == PBM) {
#pragma unroll
                for (int r = 0; r < MC_R; r++) {
                    float ae = a[r] * pub[r];
                    fp[r] = ((m >> r) & 1u) ? ae : 1.f - ae;
                }
            } else {
                // Marginal over the rank of the previous click (ubm.cu:412-468).
                float marg[MC_R];
#pragma unroll
                for (int r = 0; r < MC_R; r++) {
                    float cp = 0.f;
#pragma unroll
                    for (int pc = -1; pc < r; pc++) {
                        int pcc = pc < 0 ? 9 : pc;
                        float none = 1.f;
#pragma unroll
                        for (int b = pc + 1; b < r; b++) none *= 1.f - a[b] * pub[b * (b + 1) / 2 + pcc];
                        float tmp = none * (a[r] * pub[r * (r + 1) / 2 + pcc]);
                        cp += pc >= 0 ? marg[pc] * tmp : tmp;
                    }
                    marg[r] = cp;
                    fp[r] = ((m >> r) & 1u) ? cp : 1.f - cp;
                }
            }
        } else {
            float g = pub[0], t1 = pub[0], t2 = pub[1], t3 = pub[2];
            float ex = 1.f;
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                float cp;
                if ((m >> r) & 1u) {
                    cp = a[r] * ex;
                    ex = A.model == DBN ? g * (1.f - sv[r]) : t2 * (1.f - a[r]) + t3 * a[r];
                } else {
                    cp = 1.f - a[r] * ex;
                    ex *= (A.model == DBN ? g : t1) * (1.f - a[r]) / cp;
                }
                lc[r] = logf(cp);
            }
            ex = 1.f;
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                float ae = a[r] * ex;
                fp[r] = ((m >> r) & 1u) ? ae : 1.f - ae;
                ex *= A.model == DBN ? g * (1.f - a[r]) + g * a[r] * (1.f - sv[r])
                                     : (1.f - a[r]) * t1 + a[r] * ((1.f - a[r]) * t2 + a[r] * t3);
            }
        }
        double ls = 0.0;
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            ls += (double)lc[r];
            acc[1 + r] += (double)log2f(fp[r]);
        }
        acc[0] += ls / 10.0;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k <= MC_R; k++) {
        double v = warp_sum_d(acc[k]);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x <= MC_R) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[threadIdx.x][w];
        atomicAdd(A.out + threadIdx.x, v);
    }
}

cudaError_t launch_eval(const EvalArgs& A, int n_sm, cudaStream_t st) {
    if (A.n == 0) return cudaSuccess;
    int64_t blocks = (A.n + 255) / 256;
    int cap = 4 * n_sm;
    int g = (int)(blocks < cap ? blocks : cap);
    eval_kernel<<<g, 256, 0, st>>>(A);
    return cudaGetLastError();
}

}  // namespace mcd
