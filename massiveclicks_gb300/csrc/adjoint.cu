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
// by every call instead of being stored.  Gradients are accumulated in FP64.
#include <cstdint>
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

cudaError_t launch_grad_to_float(const double* src, float* dst, int64_t n, int n_sm, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    int g = (int)(blocks < 8 * n_sm ? blocks : 8 * n_sm);
    grad_to_float_kernel<<<g, 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

}  // namespace mcd
