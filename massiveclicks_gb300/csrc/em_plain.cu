// Plain GPU EM: the reference's GPU structure (parallel_em/kernel.cu:42-89,
// parallel_em.cu:462-609), restated for sm_103a as the baseline the fused
// kernel is measured against.  Per iteration:
//   1. E-step, one thread per session, over rank-major 8-byte records
//      {click, parameter index} (search.cuh:63-73, search.cu:342-356); each
//      session writes its statistics to per-session temporaries; DBN/CCM use
//      the reference's 10x10 tail table and log-space factors
//      (factor.cu:41-71, 176-205, device branch);
//   2. reset of every parameter to the prior (1, 2) (common.cu:71-82);
//   3. update: one float atomic pair per session and rank for private
//      parameters (common.cu:271-280), a block reduction plus one atomic pair
//      per block for each public parameter (common.cu:203-261).
// Unlike the reference's GPU path, temporaries that the E-step never writes are
// initialised once (to (1, 2) in parity mode, (0, 0) in clean mode), so the
// plain and fused paths compute the same statistics.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace mcd {

__device__ __forceinline__ float pvalue(float2 p) {
    float v = p.x / p.y;
    return v < MC_TOP ? v : MC_TOP;
}

__device__ __forceinline__ void set2(float2* dst, float a, float b) { *dst = make_float2(a, b); }

// Device factor of the reference (factor.cu:41-71 CCM, 176-205 DBN).
__device__ float plain_dbn_factor(const float (&cp)[MC_R][MC_R], const float (&ep)[MC_R + 1], int click, int last,
                                  int rank, float a, float s, float g, int x, int y, int z) {
    float la = __logf(a), lia = __logf(1.f - a), lg = __logf(g), lig = __logf(1.f - g), ls = __logf(s), lis = __logf(1.f - s);
    float lp = (click == 0) * lia + (click != 0) * la;
    lp += (x == 1) * ((z == 1) * (click == 0) * lg + (z != 1) * (click == 0) * lig);
    lp += (y == 0) * (click != 0) * (lis + (z == 1) * lg + (z != 1) * lig);
    lp += (y != 0) * (click != 0) * (z != 1) * ls;
    if ((z == 0 && last >= rank + 1) || (click == 0 && y == 1) || (x == 0 && click != 0) ||
        (x != 1 && z == 1 && click == 0) || (y != 0 && z == 1 && click != 0))
        return 0.f;
    if (z != 0 && rank + 1 < MC_R)
        for (int j = 0; j < MC_R - rank - 1; j++) lp += __logf(cp[rank + 1][j]);
    float e = ep[rank];
    lp += __logf((x == 1) * e + (x != 1) * (1.f - e));
    return __expf(lp);
}

__device__ float plain_ccm_factor(const float (&cp)[MC_R][MC_R], const float (&ep)[MC_R + 1], int click, int last,
                                  int rank, float a, float t1, float t2, float t3, int x, int y, int z) {
    float la = __logf(a), lia = __logf(1.f - a);
    float l1 = __logf(t1), li1 = __logf(1.f - t1), l2 = __logf(t2), li2 = __logf(1.f - t2), l3 = __logf(t3), li3 = __logf(1.f - t3);
    float lp = (click == 0) * lia + (click != 0) * la;
    lp += (x == 1) * ((z == 1) * (click == 0) * l1 + (z != 1) * (click == 0) * li1);
    lp += (y == 0) * (click != 0) * (lia + (z == 1) * l2 + (z != 1) * li2);
    lp += (y != 0) * (click != 0) * (la + (z == 1) * l3 + (z != 1) * li3);
    if ((z == 0 && last >= rank + 1) || (click == 0 && y == 1) || (x == 0 && click != 0) || (x != 1 && z == 1 && click == 0))
        return 0.f;
    if (z != 0 && rank + 1 < MC_R)
        for (int j = 0; j < MC_R - rank - 1; j++) lp += __logf(cp[rank + 1][j]);
    lp += __logf((x == 1) * ep[rank] + (x != 1) * (1.f - ep[rank]));
    return __expf(lp);
}

template <int MODEL>
__global__ void __launch_bounds__(128) plain_estep_kernel(PlainArgs A) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= A.n) return;
    const int64_t n = A.n;
    int click[MC_R], p[MC_R];
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        PlainRec rec = A.recs[(int64_t)r * n + s];
        click[r] = rec.click;
        p[r] = rec.pidx;
    }
    if (MODEL == PBM || MODEL == UBM) {
        int prev[MC_R];
        int last = MC_R - 1;
#pragma unroll
        for (int r = 0; r < MC_R; r++) { prev[r] = last; if (click[r] == 1) last = r; }
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            int slot = MODEL == PBM ? r : r * (r + 1) / 2 + prev[r];
            float a = pvalue(A.atr2[p[r]]);
            float e = pvalue(A.pub2[slot]);
            float na = 1.f, ne = 1.f;
            if (click[r] == 0) {
                float ae = a * e;
                na = (a - ae) / (1.f - ae);
                ne = (e - ae) / (1.f - ae);
            }
            set2(A.tmp_atr + (int64_t)r * n + s, na, 1.f);
            set2(A.tmp_pub + (int64_t)slot * n + s, ne, 1.f);
        }
        return;
    }
    int lastc = MC_R;
#pragma unroll
    for (int r = MC_R - 1; r >= 0; r--) if (click[r] == 1 && lastc == MC_R) lastc = r;
    float a[MC_R], sv[MC_R];
    float g = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
    if (MODEL == DBN) g = pvalue(A.pub2[0]);
    else { t1 = pvalue(A.pub2[0]); t2 = pvalue(A.pub2[1]); t3 = pvalue(A.pub2[2]); }
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        a[r] = pvalue(A.atr2[p[r]]);
        sv[r] = MODEL == DBN ? pvalue(A.sat2[p[r]]) : 0.f;
    }
    // compute_exm_car
    float exam[MC_R + 1], car[MC_R + 1], ht[MC_R];
    exam[0] = 1.f;
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        float tmp = MODEL == DBN ? g * (1.f - a[r]) : (1.f - a[r]) * t1;
        float step = MODEL == DBN ? tmp + g * a[r] * (1.f - sv[r]) : tmp + a[r] * ((1.f - a[r]) * t2 + a[r] * t3);
        exam[r + 1] = exam[r] * step;
        ht[r] = tmp;
    }
    car[MC_R] = 0.f;
#pragma unroll
    for (int r = MC_R - 1; r >= 0; r--) car[r] = a[r] + ht[r] * car[r + 1];
    // attractiveness (and satisfaction)
#pragma unroll
    for (int r = 0; r < MC_R; r++) {
        float num = 0.f, den = 1.f;
        if (click[r] == 1) {
            num += 1.f;
            if (MODEL == CCM) den += 1.f;
        } else if (r >= lastc) {
            num += MODEL == DBN ? (a[r] * (1.f - exam[r])) / (1.f - exam[r] * car[r])
                                : ((1.f - exam[r]) * a[r]) / (1.f - exam[r] * car[r]);
        }
        if (MODEL == CCM && click[r] == 1 && r == lastc)
            num += a[r] / (1.f - (t2 * (1.f - a[r]) + t3 * a[r]) * car[r + 1]);
        set2(A.tmp_atr + (int64_t)r * n + s, num, den);
        if (MODEL == DBN && click[r] == 1) {
            float sn = 0.f;
            if (r == lastc) {
                float cv = r < MC_R - 1 ? car[r + 1] : 0.f;
                sn += sv[r] / (1.f - (1.f - sv[r]) * g * cv);
            }
            set2(A.tmp_sat + (int64_t)r * n + s, sn, 1.f);
        }
    }
    // tail click probabilities (get_tail_clicks)
    float cp[MC_R][MC_R], ep[MC_R + 1];
    for (int i = 0; i < MC_R; i++)
        for (int j = 0; j < MC_R; j++) cp[i][j] = 0.f;
    ep[0] = 1.f;
    for (int st = 0; st < MC_R; st++) {
        float ex = 1.f;
        int j = 0;
        for (int res = st; res < MC_R; res++) {
            float aj = a[j], c;
            if (click[res] == 1) {
                c = aj * ex;
                ex = MODEL == DBN ? g * (1.f - sv[j]) : t2 * (1.f - aj) + t3 * aj;
            } else {
                c = 1.f - aj * ex;
                ex *= (MODEL == DBN ? g : t1) * (1.f - aj) / c;
            }
            cp[st][j] = c;
            if (st == 0) ep[j + 1] = ex;
            j++;
        }
    }
    // gamma / tau
    float pn[3] = {0.f, 0.f, 0.f}, pd[3] = {0.f, 0.f, 0.f};
    for (int r = 0; r < MC_R; r++) {
        float f[8], sum = 0.f;
        for (int k = 0; k < 8; k++) {
            int x = k >> 2, y = (k >> 1) & 1, z = k & 1;
            f[k] = MODEL == DBN ? plain_dbn_factor(cp, ep, click[r], lastc, r, a[r], sv[r], g, x, y, z)
                                : plain_ccm_factor(cp, ep, click[r], lastc, r, a[r], t1, t2, t3, x, y, z);
            sum += f[k];
        }
        if (MODEL == DBN) {
            pn[0] += f[5] / sum;
            pd[0] += (f[4] + f[5]) / sum;
        } else if (click[r] == 0) {
            float nu = (f[5] + f[7]) / sum;
            pn[0] += nu;
            pd[0] += nu + (f[4] + f[6]) / sum;
        } else {
            float n2 = f[5] / sum, n3 = f[7] / sum;
            pn[1] += n2; pd[1] += n2 + f[4] / sum;
            pn[2] += n3; pd[2] += n3 + f[6] / sum;
        }
    }
    int npub = MODEL == DBN ? 1 : 3;
    for (int k = 0; k < npub; k++) set2(A.tmp_pub + (int64_t)k * n + s, pn[k], pd[k]);
}

__global__ void plain_reset_kernel(float2* atr2, float2* sat2, int64_t n_qd, float2* pub2, int n_pub) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = i; k < n_qd; k += stride) {
        atr2[k] = make_float2(1.f, 2.f);
        if (sat2) sat2[k] = make_float2(1.f, 2.f);
    }
    if (i < n_pub) pub2[i] = make_float2(1.f, 2.f);
}

template <int MODEL>
__global__ void __launch_bounds__(128) plain_update_kernel(PlainArgs A) {
    __shared__ float red[2][4];
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = A.n;
    if (s < n) {
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            int p = A.recs[(int64_t)r * n + s].pidx;
            float2 u = __ldg(A.tmp_atr + (int64_t)r * n + s);
            atomicAdd(&A.atr2[p].x, u.x);
            atomicAdd(&A.atr2[p].y, u.y);
            if (MODEL == DBN) {
                float2 v = __ldg(A.tmp_sat + (int64_t)r * n + s);
                atomicAdd(&A.sat2[p].x, v.x);
                atomicAdd(&A.sat2[p].y, v.y);
            }
        }
    }
    const int npub = public_params(MODEL);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < npub; k++) {
        float2 u = s < n ? __ldg(A.tmp_pub + (int64_t)k * n + s) : make_float2(0.f, 0.f);
        for (int o = 16; o > 0; o >>= 1) {
            u.x += __shfl_xor_sync(0xffffffffu, u.x, o);
            u.y += __shfl_xor_sync(0xffffffffu, u.y, o);
        }
        if (lane == 0) { red[0][warp] = u.x; red[1][warp] = u.y; }
        __syncthreads();
        if (threadIdx.x == 0) {
            float x = 0.f, y = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) { x += red[0][w]; y += red[1][w]; }
            atomicAdd(&A.pub2[k].x, x);
            atomicAdd(&A.pub2[k].y, y);
        }
        __syncthreads();
    }
}

// Canonical value arrays <-> (num, den) pairs.
__global__ void values_to_pairs_kernel(const float* v, float2* pairs, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) pairs[i] = make_float2(v[i], 1.f);
}

__global__ void pairs_to_values_kernel(const float2* pairs, float* v, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) v[i] = pvalue(pairs[i]);
}

__global__ void fill2_kernel(float2* p, int64_t n, float a, float b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) p[i] = make_float2(a, b);
}

static int grid_for(int64_t n, int block, int cap = 65535 * 16) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

cudaError_t launch_plain_estep(int model, const PlainArgs& A, cudaStream_t st) {
    int g = grid_for(A.n, 128, 1 << 30);
    if (A.n == 0) return cudaSuccess;
    switch (model) {
        case PBM: plain_estep_kernel<PBM><<<g, 128, 0, st>>>(A); break;
        case CCM: plain_estep_kernel<CCM><<<g, 128, 0, st>>>(A); break;
        case DBN: plain_estep_kernel<DBN><<<g, 128, 0, st>>>(A); break;
        default: plain_estep_kernel<UBM><<<g, 128, 0, st>>>(A); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_plain_reset(const PlainArgs& A, int n_pub, cudaStream_t st) {
    int64_t m = A.n_qd > n_pub ? A.n_qd : n_pub;
    plain_reset_kernel<<<grid_for(m, 256), 256, 0, st>>>(A.atr2, A.sat2, A.n_qd, A.pub2, n_pub);
    return cudaGetLastError();
}

cudaError_t launch_plain_update(int model, const PlainArgs& A, cudaStream_t st) {
    int g = grid_for(A.n, 128, 1 << 30);
    if (A.n == 0) return cudaSuccess;
    switch (model) {
        case PBM: plain_update_kernel<PBM><<<g, 128, 0, st>>>(A); break;
        case CCM: plain_update_kernel<CCM><<<g, 128, 0, st>>>(A); break;
        case DBN: plain_update_kernel<DBN><<<g, 128, 0, st>>>(A); break;
        default: plain_update_kernel<UBM><<<g, 128, 0, st>>>(A); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_values_to_pairs(const float* v, float2* pairs, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    values_to_pairs_kernel<<<grid_for(n, 256, 8192), 256, 0, st>>>(v, pairs, n);
    return cudaGetLastError();
}

cudaError_t launch_pairs_to_values(const float2* pairs, float* v, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    pairs_to_values_kernel<<<grid_for(n, 256, 8192), 256, 0, st>>>(pairs, v, n);
    return cudaGetLastError();
}

__global__ void fill_value_kernel(float* p, int64_t n, float v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) p[i] = v;
}

cudaError_t launch_fill_value(float* p, int64_t n, float v, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    fill_value_kernel<<<grid_for(n, 256, 8192), 256, 0, st>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_fill2(float2* p, int64_t n, float a, float b, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    fill2_kernel<<<grid_for(n, 256, 8192), 256, 0, st>>>(p, n, a, b);
    return cudaGetLastError();
}

}  // namespace mcd
