// mc_model_*: one click-model fit on one GPU.  Host orchestration of the
// fused, plain and evaluation kernels behind the C-ABI (include/mclicks.h).
//
// Device layout of a fit (all resident in HBM):
//   pidx      int32 [10][stride]   rank-major planes of parameter indices
//   click     uint16 [n]           click bit masks
//   cnt       uint2 [n_qd]         {occurrences, clicked occurrences} per qd
//   atr, sat  float [n_qd]         current parameter values
//   pub_theta float [2][128]       public values, double-buffered by iteration
//   pub_bins  double [2 n_pub]     FP64 public statistic bins
//   tiles     TileDev [n_tiles]    work queue (whole queries or query chunks)
//   split_*   FP64 bins and counters of queries split over several tiles
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "mclicks.h"
#include "host_internal.h"
#include "devmem.h"
#include "pool.h"
#include "common.cuh"
#include "kernels.h"

using namespace mcd;
using mch::set_error;

namespace {

int cuda_fail(const char* what, cudaError_t e) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? MC_ERR_NOMEM : MC_ERR_CUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                             \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(#call, e_);  \
    } while (0)

template <typename T>
int dalloc(T** p, size_t count, int64_t* bytes) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = mch::dev_alloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_fail("cudaMalloc", e);
    *bytes += (int64_t)(count * sizeof(T));
    return MC_OK;
}

// Back to the device cache: no work may be pending on p (see settle()).
template <typename T>
void dfree(T*& p) {
    mch::dev_free((void*)p);
    p = nullptr;
}

// Waits for the device before buffers that kernels may still use are freed
// (what cudaFree itself would wait for).
template <typename... T>
void settle(T*... ps) {
    if (((ps != nullptr) || ...)) cudaDeviceSynchronize();
}

__global__ void pub_to_pairs_kernel(const float* theta, const int* iter, float2* pub2, int n_pub) {
    int k = threadIdx.x;
    if (k < n_pub) pub2[k] = make_float2(theta[(*iter & 1) * MC_MAX_PUB + k], 1.f);
}

__global__ void pairs_to_pub_kernel(const float2* pub2, float* theta, const int* iter, int n_pub) {
    int k = threadIdx.x;
    if (k < n_pub) {
        float v = pub2[k].x / pub2[k].y;
        theta[(*iter & 1) * MC_MAX_PUB + k] = v < MC_TOP ? v : MC_TOP;
    }
}

// flag = 1 when some query segment's qd range starts below the previous one's end.
__global__ void seg_order_kernel(int64_t n_seg, const int* __restrict__ lo, const int* __restrict__ hi, int* flag) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + 1; g < n_seg; g += (int64_t)gridDim.x * blockDim.x)
        if (lo[g] < hi[g - 1]) *flag = 1;
}

__global__ void fill_i32_kernel(int* __restrict__ p, int64_t n, int v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// One pass over the uploaded sessions (session-major pidx): range check,
// transposition into rank-major planes, per-qd occurrence / click counts, the
// qd range of each query segment, and the click counts behind the public
// constants (PBM: clicks per rank; UBM: written and clicked-written slots).
//
// One launch covers the sessions [s_first, s_end) (s_first a multiple of 32);
// block b takes the contiguous sessions from s_first + b * chunk (chunk a
// multiple of 32, so a warp's packbits word belongs to one block).  It first
// finds the qd range of its sessions; when that range has at most kPrepHist
// pairs -- always so inside a head query, whose sessions share one qd window --
// the occurrence and click counts go into a shared histogram that is flushed
// with one 64-bit atomic per pair.  Otherwise lanes with the same qd at a rank
// add their counts with one global atomic.  (Global atomics alone put a head
// query's few hot pairs on one L2 slice: 3.6 ms for 16M sessions.)
constexpr int kPrepHist = 6144;  // uint2 entries: 48 KB of dynamic shared memory
constexpr int kPrepThreads = 256;

__global__ void __launch_bounds__(kPrepThreads) prep_kernel(
    int64_t s_first, int64_t s_end, int64_t chunk, int64_t stride, int64_t n_qd, const int32_t* __restrict__ pidx_sm,
    const uint16_t* __restrict__ click, const int32_t* __restrict__ seg_id, int model, int32_t* planes, uint2* cnt,
    int* seg_lo, int* seg_hi, unsigned long long* pub_counts, uint32_t* packbits, int* flag) {
    extern __shared__ uint2 hist[];
    __shared__ unsigned int sc[MC_PUB_COUNTS];
    __shared__ int s_lo, s_hi;
    const int tid = threadIdx.x, lane = tid & 31;
    for (int k = tid; k < MC_PUB_COUNTS; k += blockDim.x) sc[k] = 0;
    if (tid == 0) { s_lo = INT_MAX; s_hi = INT_MIN; }
    __syncthreads();
    const int64_t b0 = s_first + (int64_t)blockIdx.x * chunk;
    const int64_t b1 = min(s_end, b0 + chunk);
    {
        int lo = INT_MAX, hi = INT_MIN;
        for (int64_t s = b0 + tid; s < b1; s += blockDim.x) {
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                const int p = pidx_sm[s * MC_R + r];
                if (p >= 0 && (int64_t)p < n_qd) { lo = min(lo, p); hi = max(hi, p + 1); }
            }
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (lane == 0) { atomicMin(&s_lo, lo); atomicMax(&s_hi, hi); }
    }
    __syncthreads();
    const int h_lo = s_lo;
    const int h_n = s_hi > s_lo ? s_hi - s_lo : 0;
    const bool local = h_n <= kPrepHist;  // uniform over the block
    if (local)
        for (int k = tid; k < h_n; k += blockDim.x) hist[k] = make_uint2(0u, 0u);
    __syncthreads();
    for (int64_t s0 = b0; s0 < b1; s0 += blockDim.x) {
        const int64_t s = s0 + tid;
        const bool valid = s < b1;
        int lo = INT_MAX, hi = INT_MIN;
        int64_t seg = -1;
        const unsigned m = valid ? click[s] : 0u;
        // Bit s of packbits: session s has a click (32 consecutive sessions per warp).
        const unsigned word = __ballot_sync(0xffffffffu, m != 0u);
        const int64_t w0 = s0 + (tid & ~31);  // first session of this warp, a multiple of 32
        if (lane == 0 && w0 < b1) packbits[w0 >> 5] = word;
        if (valid) seg = seg_id[s];
        int last = 9, slot[MC_R];
#pragma unroll
        for (int r = 0; r < MC_R; r++) {
            int p = -1;
            if (valid) {
                p = pidx_sm[s * MC_R + r];
                if (p < 0 || (int64_t)p >= n_qd) { atomicOr(flag, 1); p = 0; }
                planes[(int64_t)r * stride + s] = p;
                lo = min(lo, p);
                hi = max(hi, p + 1);
            }
            const bool c = valid && ((m >> r) & 1u);
            if (local) {
                const unsigned hp = (unsigned)(p - h_lo);
                if (valid && hp < (unsigned)h_n) {
                    atomicAdd(&hist[hp].x, 1u);
                    if (c) atomicAdd(&hist[hp].y, 1u);
                }
            } else {
                // every lane takes part in the match and the ballot (invalid lanes hold p = -1)
                const unsigned peers = __match_any_sync(0xffffffffu, p);
                const unsigned clicked = __ballot_sync(0xffffffffu, c) & peers;
                if (valid && lane == __ffs(peers) - 1)
                    atomicAdd(reinterpret_cast<unsigned long long*>(cnt + p),
                              (unsigned long long)__popc(peers) | ((unsigned long long)__popc(clicked) << 32));
            }
            slot[r] = r * (r + 1) / 2 + last;
            if (c) last = r;
            if (model == 0) {  // clicks per rank, summed over the warp
                const unsigned nc = __popc(__ballot_sync(0xffffffffu, c));
                if (lane == 0 && nc) atomicAdd(&sc[r], nc);
            }
        }
        {  // per-session counts of the public constants, summed over the warp
            const int lc = m ? 31 - __clz(m) : MC_R;
            unsigned v = 0;
            if (valid && model == 2) v = (unsigned)lc;
            if (valid && model == 1) v = (unsigned)(lc - __popc(m & ((1u << lc) - 1u)));
            v = __reduce_add_sync(0xffffffffu, v);
            if (lane == 0 && v)
                atomicAdd(&sc[model == 2 ? MC_CNT_DBN_BEFORE_LAST : MC_CNT_CCM_UNCLICKED_BEFORE_LAST], v);
        }
        if (valid && model == 3) {
#pragma unroll
            for (int r = 0; r < MC_R; r++) {
                bool alive = true;
#pragma unroll
                for (int r2 = r + 1; r2 < MC_R; r2++) alive = alive && slot[r2] != slot[r];
                if (alive) {
                    atomicAdd(&sc[slot[r]], 1u);
                    if ((m >> r) & 1u) atomicAdd(&sc[MC_UBM_SLOTS + slot[r]], 1u);
                }
            }
        }
        // Segment ranges, aggregated over the lanes of a warp that share a segment.
        const unsigned peers = __match_any_sync(0xffffffffu, (unsigned long long)seg);
        const int wlo = __reduce_min_sync(peers, lo);
        const int whi = __reduce_max_sync(peers, hi);
        if (valid && lane == __ffs(peers) - 1) {
            atomicMin(&seg_lo[seg], wlo);
            atomicMax(&seg_hi[seg], whi);
        }
    }
    __syncthreads();
    if (local)
        for (int k = tid; k < h_n; k += blockDim.x) {
            const uint2 h = hist[k];
            if (h.x) atomicAdd(reinterpret_cast<unsigned long long*>(cnt + h_lo + k),
                               (unsigned long long)h.x | ((unsigned long long)h.y << 32));
        }
    for (int k = tid; k < MC_PUB_COUNTS; k += blockDim.x)
        if (sc[k]) atomicAdd(&pub_counts[k], (unsigned long long)sc[k]);
}

// The plain path's 8-byte rank-major records, built from the planes.
// Query segments on the device.  Block b covers sessions [b * 2048, (b + 1) * 2048),
// eight consecutive sessions per thread; a session starts a segment when its
// query differs from the previous session's.
constexpr int kSegBlock = 2048;

__global__ void seg_count_kernel(int64_t n, const int32_t* __restrict__ query, int* __restrict__ blk_count) {
    __shared__ int warp_sum[8];
    const int64_t base = (int64_t)blockIdx.x * kSegBlock + (int64_t)threadIdx.x * 8;
    int c = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int64_t s = base + k;
        if (s < n) c += (s == 0 || query[s] != query[s - 1]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < 8; w++) t += warp_sum[w];
        blk_count[blockIdx.x] = t;
    }
}

// Writes seg_begin[] (the first session of every segment, in order) and the
// segment index of every session; blk_off[b] is the number of segments that
// start before block b.
__global__ void seg_write_kernel(int64_t n, const int32_t* __restrict__ query, const int64_t* __restrict__ blk_off,
                                 int64_t* __restrict__ seg_begin, int32_t* __restrict__ seg_id) {
    __shared__ int warp_sum[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kSegBlock + (int64_t)threadIdx.x * 8;
    unsigned flags = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int64_t s = base + k;
        if (s < n && (s == 0 || query[s] != query[s - 1])) flags |= 1u << k;
    }
    const int c = __popc(flags);
    int incl = c;  // inclusive scan over the lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; w++) before += warp_sum[w];
    int64_t idx = blk_off[blockIdx.x] + before + incl - c;  // segments starting before this thread's first session
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int64_t s = base + k;
        if (s >= n) break;
        if ((flags >> k) & 1u) seg_begin[idx++] = s;
        seg_id[s] = (int32_t)(idx - 1);
    }
}

// Click counts as 16-bit pairs for the fused M-step of whole-query tiles.
__global__ void pack_counts_kernel(const uint2* __restrict__ cnt, uint32_t* __restrict__ cnt16, int64_t n) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
        const uint2 c = cnt[i];
        cnt16[i] = (c.x < 65535u ? c.x : 65535u) | ((c.y < 65535u ? c.y : 65535u) << 16);
    }
}

__global__ void build_recs_kernel(int64_t n, int64_t stride, const int32_t* planes, const uint16_t* click, PlainRec* recs) {
    int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += step) {
        unsigned m = click[s];
        for (int r = 0; r < MC_R; r++) {
            PlainRec pr;
            pr.click = (signed char)((m >> r) & 1u);
            pr.pidx = planes[(int64_t)r * stride + s];
            recs[(int64_t)r * n + s] = pr;
        }
    }
}

constexpr int kGraphChunk = 64;

struct ParamDesc {
    const char* name;
    int kind;  // 0 = public, 1 = attractiveness, 2 = satisfaction
};

}  // namespace

// Chunks of the upload's host-to-device copy of the session indices; the
// upload pass runs on each chunk as soon as it has landed.
static const int kUploadChunks = 8;

// A host array in page-locked memory from the library's pool (mch::host_alloc):
// upload readbacks land in it directly.  resize keeps no contents.
template <class T>
struct PinnedArray {
    T* p = nullptr;
    size_t n = 0, cap = 0;
    PinnedArray() = default;
    PinnedArray(const PinnedArray&) = delete;
    PinnedArray& operator=(const PinnedArray&) = delete;
    ~PinnedArray() { mch::host_free(p); }
    cudaError_t resize(size_t m) {
        if (m > cap) {
            mch::host_free(p);
            p = nullptr;
            n = cap = 0;
            void* q = nullptr;
            cudaError_t e = mch::host_alloc(&q, std::max<size_t>(m, 1) * sizeof(T));
            if (e != cudaSuccess) return e;
            p = static_cast<T*>(q);
            cap = m;
        }
        n = m;
        return cudaSuccess;
    }
    size_t size() const { return n; }
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
    T* data() { return p; }
};

struct mc_model {
    int model = 0, mode = 0, device = 0, n_pub = 0, n_sm = 0;
    int64_t n = 0, stride = 0, n_qd = 0, bytes = 0;
    bool uploaded = false, fused_ok = false;
    std::string fused_reason;
    // query segments of the training set: sessions and qd range
    PinnedArray<int64_t> seg_begin;
    PinnedArray<int32_t> seg_lo, seg_hi;  // qd range [lo, hi) of each segment, as the upload pass finds it
    PinnedArray<uint32_t> packbits;  // bit s: training session s has a click
    int spt = 1024, wqd = 1536, block = 256, stages = 2, ctas_per_sm = 1;
    // fused state
    int32_t* d_pidx = nullptr;
    uint16_t* d_click = nullptr;
    uint2* d_cnt = nullptr;
    uint32_t* d_cnt16 = nullptr;
    uint32_t* d_coff = nullptr;  // PBM/UBM: per-qd entry offsets [n_qd + 1] of the count path
    uint32_t* d_cent = nullptr;  // PBM/UBM: entries (count << 7 | key << 1 | alive)
    uint16_t* d_cdense = nullptr;  // PBM: uint16 [n_qd][10] counts by rank (when all fit 16 bits)
    int64_t n_cent = 0;
    float *d_atr = nullptr, *d_sat = nullptr, *d_pub_theta = nullptr;
    double *d_pub_bins = nullptr, *d_pub_const = nullptr, *d_split_bins = nullptr;
    unsigned *d_split_count = nullptr, *d_tiles_done = nullptr;
    int *d_iter = nullptr, *d_status = nullptr;
    FitDev* d_fit = nullptr;
    TileDev* d_tiles = nullptr;
    SplitDev* d_splits = nullptr;
    WorkState* d_ws = nullptr;
    int n_tiles = 0, n_splits = 0, grid = 0;
    bool tiles_ready = false;  // tiles built for the current shape (PBM/UBM build them only for batches)
    std::vector<int64_t> h_tile_begin;  // first session of each tile, ascending (adjoint range lookups)
    // Adjoint per-tile counts (adjoint_counts_kernel): entry offset of each
    // staged tile (-1 otherwise), built with the tiles; the counts themselves
    // on the first FP32 adjoint call over the tiles.
    std::vector<int64_t> h_adj_off;
    int64_t adj_entries = 0;
    int64_t* d_adj_off = nullptr;
    uint4* d_adj_cnt = nullptr;
    // Every session of each staged tile packed in click-mask order (the
    // packing kernel's PBM layout, no session dropped), for the adjoint's
    // whole tiles; built with the counts.
    TileDev* d_adj_tiles = nullptr;
    unsigned char* d_adj_blk = nullptr;
    int64_t adj_bytes = 0;
    // Launch shapes of the count kernels (entry kernel; dense PBM kernel).
    CountShape count_shape{8, 256, 8};
    CountShape dense_shape{0, 256, 6};
    unsigned char* d_tblk = nullptr;
    int64_t split_bins_count = 0;
    int64_t tile_bytes = 0;
    // plain state (allocated on first use)
    PlainRec* d_recs = nullptr;
    float2 *d_atr2 = nullptr, *d_sat2 = nullptr, *d_pub2 = nullptr, *d_tmp_atr = nullptr, *d_tmp_sat = nullptr,
           *d_tmp_pub = nullptr;
    int64_t plain_bytes = 0;
    // FP64 gradient accumulators of the adjoint (allocated on first use):
    // [alpha: qd_alloc][beta: qd_alloc][gamma][log-likelihood]
    double* d_grad = nullptr;
    // evaluation set
    int64_t n_test = 0, test_stride = 0;
    int32_t* d_test_pidx = nullptr;
    uint16_t* d_test_click = nullptr;
    double* d_eval = nullptr;
    int64_t test_bytes = 0;
    // graphs of the fused loop: a full chunk and a remainder
    struct GraphSlot { cudaGraphExec_t exec = nullptr; int iters = -1; };  // also used by mc_batch
    GraphSlot graphs[2];
    cudaStream_t own_stream = nullptr;
    // Side stream of the upload's host-to-device copies and one event per chunk.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ev[kUploadChunks + 1] = {};

    int ensure_copy_stream() {
        if (!copy_stream) CK(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t& ev : copy_ev)
            if (!ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        return MC_OK;
    }

    std::vector<ParamDesc> params() const {
        switch (model) {
            case MC_PBM: return {{"examination", 0}, {"attractiveness", 1}};
            case MC_UBM: return {{"examination", 0}, {"attractiveness", 1}};
            case MC_DBN: return {{"attractiveness", 1}, {"satisfaction", 2}, {"continuation", 0}};
            default: return {{"attractiveness", 1}, {"continuation", 0}};
        }
    }

    void drop_graph() {
        for (GraphSlot& g : graphs) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
            g.iters = -1;
        }
    }

    void free_tiles() {
        settle(d_tiles, d_splits, d_split_bins, d_split_count, d_tblk);
        dfree(d_tiles);
        dfree(d_splits);
        dfree(d_split_bins);
        dfree(d_split_count);
        dfree(d_tblk);
        bytes -= tile_bytes;
        tile_bytes = 0;
        tiles_ready = false;
        h_tile_begin.clear();
        settle(d_adj_off, d_adj_cnt, d_adj_tiles, d_adj_blk);
        dfree(d_adj_off);
        dfree(d_adj_cnt);
        dfree(d_adj_tiles);
        dfree(d_adj_blk);
        bytes -= adj_bytes;
        adj_bytes = 0;
        h_adj_off.clear();
        adj_entries = 0;
    }

    void free_plain() {
        settle(d_recs, d_atr2, d_sat2, d_pub2, d_tmp_atr, d_tmp_sat, d_tmp_pub);
        dfree(d_recs); dfree(d_atr2); dfree(d_sat2); dfree(d_pub2); dfree(d_tmp_atr); dfree(d_tmp_sat); dfree(d_tmp_pub);
        bytes -= plain_bytes;
        plain_bytes = 0;
    }

    void free_train() {
        drop_graph();
        free_tiles();
        free_plain();
        settle(d_pidx, d_click, d_atr, d_fit, d_grad);
        dfree(d_pidx); dfree(d_click); dfree(d_cnt); dfree(d_cnt16); dfree(d_coff); dfree(d_cent); dfree(d_cdense); dfree(d_atr); dfree(d_sat); dfree(d_pub_theta);
        dfree(d_pub_bins); dfree(d_pub_const); dfree(d_tiles_done); dfree(d_iter); dfree(d_status);
        dfree(d_fit); dfree(d_ws); dfree(d_grad);
        bytes = test_bytes;
        n_cent = 0;
        uploaded = false;
    }

    void free_test() {
        settle(d_test_pidx, d_test_click, d_eval);
        dfree(d_test_pidx); dfree(d_test_click); dfree(d_eval);
        bytes -= test_bytes;
        test_bytes = 0;
        n_test = 0;
    }

    cudaStream_t pick(void* s) {
        if (s) return (cudaStream_t)s;
        if (!own_stream) cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking);
        return own_stream;
    }

    int64_t qd_alloc() const { return ((std::max<int64_t>(n_qd, 1) + 3) & ~(int64_t)3) + 4; }
    int build_tiles();
    // Tiles for the tile kernel (batched launches, autotuning): built at upload
    // for DBN/CCM, on first use for the count-path models.
    int ensure_tiles() {
        if (!fused_ok) return set_error(MC_ERR_INVALID, "tile path unavailable: " + fused_reason);
        return tiles_ready ? MC_OK : build_tiles();
    }
    FitDev make_desc() const;
    int write_fit_desc();
    // Every parameter at its prior value 1/2 (the default Param (1, 2), param.cuh:18-39)
    // and the iteration counter at 0, queued on st.
    int prior_values(cudaStream_t st) {
        const std::vector<float> half(2 * MC_MAX_PUB, 0.5f);
        CK(launch_fill_value(d_atr, qd_alloc(), 0.5f, st));
        if (d_sat) CK(launch_fill_value(d_sat, qd_alloc(), 0.5f, st));
        CK(cudaMemcpyAsync(d_pub_theta, half.data(), 2 * MC_MAX_PUB * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(d_iter, 0, 4, st));
        return MC_OK;
    }
    int ensure_plain(cudaStream_t st);
};

// Bound on the sessions of one staged tile (its packing sort holds them all
// in shared memory).
static const int kTileSessions = 4096;

// Splits the query segments into tiles.  A staged tile holds at most `spt`
// packed sessions (those its E-step reads: for DBN and CCM the sessions with
// a click, otherwise all), at most kTileSessions sessions in all, and a window
// of at most `wqd` qd.  A query above a bound becomes a split query:
// consecutive chunks that share FP64 bins, cut so that the chunks carry equal
// numbers of packed sessions; a query whose window exceeds `wqd` is read
// directly from global memory in chunks of at most `spt` sessions.
int mc_model::build_tiles() {
    drop_graph();
    free_tiles();
    const int ns = private_stats(model);
    const bool drop = (model == MC_DBN || model == MC_CCM) && packbits.size() == (size_t)((n + 31) / 32);
    auto packed_at = [&](int64_t s) -> int { return drop ? (int)((packbits[(size_t)(s >> 5)] >> (s & 31)) & 1u) : 1; };
    // Packed sessions in [b, e): popcounts of the covered words, the two end
    // words masked.
    auto packed_in = [&](int64_t b, int64_t e) -> int64_t {
        if (!drop) return e - b;
        if (b >= e) return 0;
        const int64_t wb = b >> 5, we = (e - 1) >> 5;
        const uint32_t head = 0xFFFFFFFFu << (b & 31);
        const uint32_t tail = (e & 31) ? (0xFFFFFFFFu >> (32 - (e & 31))) : 0xFFFFFFFFu;
        if (wb == we) return __builtin_popcount(packbits[(size_t)wb] & head & tail);
        int64_t c = __builtin_popcount(packbits[(size_t)wb] & head) + __builtin_popcount(packbits[(size_t)we] & tail);
        for (int64_t w = wb + 1; w < we; w++) c += __builtin_popcount(packbits[(size_t)w]);
        return c;
    };
    const int64_t max_sess = std::max<int64_t>(spt, kTileSessions);
    const size_t n_seg = seg_lo.size();
    // Segments are tiled in chunks on several host threads (a chunk boundary
    // also ends a tile, wherever the threads run); the chunks' tile and split
    // lists are then joined in order.  A chunk's work grows with its segments
    // and with its sessions (popcounts over their click words), and a head
    // query holds millions of sessions, so chunks are cut at equal shares of
    // segments + sessions / 32.
    auto build_range = [&](size_t g0, size_t g1, std::vector<TileDev>& tiles, std::vector<SplitDev>& splits,
                           int64_t& bin_off) {
        TileDev cur{};
        bool open = false;
        auto close = [&]() {
            if (open) tiles.push_back(cur);
            open = false;
        };
        auto new_split = [&](int64_t lo, int64_t hi) {
            SplitDev sp;
            sp.qd_begin = lo;
            sp.qd_count = (int)(hi - lo);
            sp.n_tiles = 0;
            sp.bin_offset = bin_off;
            sp.local = (int)splits.size();
            sp.pad_ = 0;
            bin_off += (hi - lo) * ns;
            splits.push_back(sp);
            return (int)splits.size() - 1;
        };
        auto split_tile = [&](int sid, int64_t b, int64_t e, int pk) {
            TileDev t{};
            t.fit = 0;
            t.split = sid;
            t.s_begin = b;
            t.s_count = (int)(e - b);
            t.qd_begin = splits[(size_t)sid].qd_begin;
            t.qd_count = splits[(size_t)sid].qd_count;
            t.blk_off = 0;
            t.s_packed = pk;
            tiles.push_back(t);
            splits[(size_t)sid].n_tiles++;
        };
        for (size_t g = g0; g < g1; g++) {
            const int64_t sb = seg_begin[g], sc = seg_begin[g + 1] - sb;
            const int64_t lo = seg_lo[g], hi = seg_hi[g];
            if (hi - lo > wqd) {  // direct: every session read from global memory
                close();
                const int sid = new_split(lo, hi);
                const int64_t nt = (sc + spt - 1) / spt;
                for (int64_t k = 0; k < nt; k++) {
                    const int64_t b = sb + sc * k / nt, e = sb + sc * (k + 1) / nt;
                    split_tile(sid, b, e, (int)(e - b));
                }
                continue;
            }
            const int64_t pk = packed_in(sb, sb + sc);
            if (pk > spt || sc > max_sess) {  // staged split query
                close();
                const int sid = new_split(lo, hi);
                const int64_t nt0 = std::max<int64_t>(1, (pk + spt - 1) / spt);
                const int64_t target = std::max<int64_t>(1, (pk + nt0 - 1) / nt0);
                const int64_t e = sb + sc;
                int64_t b = sb;
                int tpk = 0;
                for (int64_t s = sb; s < e;) {
                    // A whole aligned word that reaches neither bound is taken at once.
                    if ((s & 31) == 0 && s + 32 <= e) {
                        const int w = drop ? __builtin_popcount(packbits[(size_t)(s >> 5)]) : 32;
                        if (tpk + w < target && s + 32 - b < max_sess) {
                            tpk += w;
                            s += 32;
                            continue;
                        }
                    }
                    tpk += packed_at(s);
                    if ((tpk == target || s + 1 - b == max_sess) && s + 1 < e) {
                        split_tile(sid, b, s + 1, tpk);
                        b = s + 1;
                        tpk = 0;
                    }
                    s++;
                }
                split_tile(sid, b, e, tpk);
                continue;
            }
            if (open && (cur.s_packed + pk > spt || cur.s_count + sc > max_sess || hi - cur.qd_begin > wqd)) close();
            if (!open) {
                cur = TileDev{};
                cur.fit = 0;
                cur.split = -1;
                cur.s_begin = sb;
                cur.s_count = 0;
                cur.s_packed = 0;
                cur.qd_begin = lo;
                open = true;
            }
            cur.s_count += (int)sc;
            cur.s_packed += (int)pk;
            cur.qd_count = (int)(hi - cur.qd_begin);
        }
        close();
    };
    const size_t n_threads = mch::pool_threads();
    // Work before segment g, g + seg_begin[g] / 32, grows with g: each cut is
    // a binary search for the next share.
    std::vector<size_t> cut{0};
    {
        auto work = [&](size_t g) { return (int64_t)g + seg_begin[g] / 32; };
        const int64_t per = std::max<int64_t>(4096, work(n_seg) / (int64_t)(4 * n_threads) + 1);
        while (cut.back() < n_seg) {
            const int64_t target = work(cut.back()) + per;
            size_t lo = cut.back() + 1, hi = n_seg;  // first g in [lo, hi] with work(g) >= target, else n_seg
            while (lo < hi) {
                const size_t mid = lo + (hi - lo) / 2;
                if (work(mid) >= target) hi = mid; else lo = mid + 1;
            }
            cut.push_back(lo);
        }
    }
    const size_t n_chunks = n_seg ? cut.size() - 1 : 0;
    std::vector<std::vector<TileDev>> chunk_tiles(n_chunks);
    std::vector<std::vector<SplitDev>> chunk_splits(n_chunks);
    std::vector<int64_t> chunk_bins(n_chunks, 0);
    mch::parallel_for(n_chunks, [&](size_t c) {
        build_range(cut[c], cut[c + 1], chunk_tiles[c], chunk_splits[c], chunk_bins[c]);
    });
    // The chunks' tiles and splits in chunk order, each chunk copied into its
    // place by the pool (one append after another took a third of the host
    // tiling time).
    std::vector<size_t> t_at(n_chunks + 1, 0), s_at(n_chunks + 1, 0);
    std::vector<int64_t> b_at(n_chunks + 1, 0);
    for (size_t c = 0; c < n_chunks; c++) {
        t_at[c + 1] = t_at[c] + chunk_tiles[c].size();
        s_at[c + 1] = s_at[c] + chunk_splits[c].size();
        b_at[c + 1] = b_at[c] + chunk_bins[c];
    }
    std::vector<TileDev> tiles(t_at[n_chunks]);
    std::vector<SplitDev> splits(s_at[n_chunks]);
    const int64_t bin_off = b_at[n_chunks];
    mch::parallel_for(n_chunks, [&](size_t c) {
        const int soff = (int)s_at[c];
        TileDev* td = tiles.data() + t_at[c];
        for (TileDev t : chunk_tiles[c]) {
            if (t.split >= 0) t.split += soff;
            *td++ = t;
        }
        SplitDev* sd = splits.data() + s_at[c];
        for (SplitDev sp : chunk_splits[c]) {
            sp.local += soff;
            sp.bin_offset += b_at[c];
            *sd++ = sp;
        }
    });
    // Packed session blocks of the staged (non-direct) tiles, 16-byte aligned.
    // Sized by the packed counts, which the packing kernel checks.
    int64_t blk = 0;
    int max_tile_sessions = 1;
    for (TileDev& t : tiles) {
        t.blk_off = blk;
        if (t.qd_count <= wqd) {
            blk += 22 * (int64_t)((t.s_packed + 7) & ~7);
            max_tile_sessions = std::max(max_tile_sessions, t.s_count);
        }
    }
    n_tiles = (int)tiles.size();
    h_tile_begin.resize(tiles.size());
    for (size_t i = 0; i < tiles.size(); i++) h_tile_begin[i] = tiles[i].s_begin;
    if (!std::is_sorted(h_tile_begin.begin(), h_tile_begin.end())) h_tile_begin.clear();  // no range lookups
    h_adj_off.assign(tiles.size(), -1);
    adj_entries = 0;
    for (size_t i = 0; i < tiles.size(); i++)
        if (tiles[i].qd_count <= wqd) { h_adj_off[i] = adj_entries; adj_entries += tiles[i].qd_count; }
    n_splits = (int)splits.size();
    split_bins_count = bin_off;
    int64_t before = bytes;
    int rc;
    if ((rc = dalloc(&d_tiles, tiles.size(), &bytes))) return rc;
    if ((rc = dalloc(&d_splits, splits.size(), &bytes))) return rc;
    if ((rc = dalloc(&d_split_bins, (size_t)bin_off, &bytes))) return rc;
    if ((rc = dalloc(&d_split_count, splits.size(), &bytes))) return rc;
    if ((rc = dalloc(&d_tblk, (size_t)std::max<int64_t>(blk, 16), &bytes))) return rc;
    tile_bytes = bytes - before;
    if (!tiles.empty()) CK(cudaMemcpy(d_tiles, tiles.data(), tiles.size() * sizeof(TileDev), cudaMemcpyHostToDevice));
    if (!splits.empty()) CK(cudaMemcpy(d_splits, splits.data(), splits.size() * sizeof(SplitDev), cudaMemcpyHostToDevice));
    CK(cudaMemset(d_split_bins, 0, (size_t)std::max<int64_t>(bin_off, 1) * sizeof(double)));
    CK(cudaMemset(d_split_count, 0, std::max<size_t>(splits.size(), 1) * sizeof(unsigned)));
    // Shared memory: bins plus a ring of 2..4 copy stages.  Prefer the stage
    // count that keeps the most CTAs resident per SM, then the deepest ring.
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    const size_t static_smem = 4096;
    int best_score = -1;
    size_t best_smem = 0;
    for (int ns_ = 2; ns_ <= FUSED_MAX_STAGES; ns_++) {
        size_t sm_ = fused_smem_bytes(model, wqd, spt, ns_);
        if (sm_ + static_smem > (size_t)optin) break;
        CK(fused_set_smem_limits(sm_));
        int per_sm = 0;
        CK(fused_occupancy(model, block, sm_, &per_sm));
        int score = per_sm * 16 + ns_;
        if (per_sm >= 1 && score > best_score) { best_score = score; stages = ns_; best_smem = sm_; ctas_per_sm = per_sm; }
    }
    if (best_score < 0) return set_error(MC_ERR_INVALID, "tile shape does not fit in shared memory (reduce sessions per tile or window)");
    // The attribute is per kernel, shared by every model and batch: keep it at
    // the device maximum so no configuration can shrink it under another one.
    (void)best_smem;
    CK(fused_set_smem_limits((size_t)optin - static_smem));
    grid = std::max(1, std::min(n_tiles, ctas_per_sm * n_sm));
    int rc2 = write_fit_desc();
    if (rc2) return rc2;
    CK(launch_pack_tiles(model, d_tiles, n_tiles, wqd, max_tile_sessions, d_pidx, stride, d_click, d_tblk, d_status, n_sm, 0));
    CK(cudaDeviceSynchronize());
    int status = 0;
    CK(cudaMemcpy(&status, d_status, 4, cudaMemcpyDeviceToHost));
    if (status) return set_error(MC_ERR_INVALID, "tile packing found a parameter index outside its query's window");
    tiles_ready = true;
    return MC_OK;
}

FitDev mc_model::make_desc() const {
    FitDev f{};
    f.model = model;
    f.mode = mode;
    f.n = n;
    f.stride = stride;
    f.n_qd = n_qd;
    f.n_tiles = n_tiles;
    f.n_pub = n_pub;
    f.pidx = d_pidx;
    f.click = d_click;
    f.cnt = d_cnt;
    f.cnt16 = d_cnt16;
    f.tblk = d_tblk;
    f.atr = d_atr;
    f.sat = d_sat;
    f.pub_theta = d_pub_theta;
    f.pub_bins = d_pub_bins;
    f.pub_const = d_pub_const;
    f.split_bins = d_split_bins;
    f.split_count = d_split_count;
    f.tiles_done = d_tiles_done;
    f.iter = d_iter;
    f.status = d_status;
    return f;
}

int mc_model::write_fit_desc() {
    FitDev f = make_desc();
    CK(cudaMemcpy(d_fit, &f, sizeof(f), cudaMemcpyHostToDevice));
    return MC_OK;
}

int mc_model::ensure_plain(cudaStream_t st) {
    if (d_recs) return MC_OK;
    int64_t before = bytes;
    int rc;
    if ((rc = dalloc(&d_recs, (size_t)(n * MC_R), &bytes))) return rc;
    if ((rc = dalloc(&d_atr2, (size_t)n_qd, &bytes))) return rc;
    if (model == MC_DBN && (rc = dalloc(&d_sat2, (size_t)n_qd, &bytes))) return rc;
    if ((rc = dalloc(&d_pub2, (size_t)n_pub, &bytes))) return rc;
    if ((rc = dalloc(&d_tmp_atr, (size_t)(n * MC_R), &bytes))) return rc;
    if (model == MC_DBN && (rc = dalloc(&d_tmp_sat, (size_t)(n * MC_R), &bytes))) return rc;
    if ((rc = dalloc(&d_tmp_pub, (size_t)(n * n_pub), &bytes))) return rc;
    plain_bytes = bytes - before;
    if (n) {
        build_recs_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 8 * n_sm), 256, 0, st>>>(n, stride, d_pidx, d_click, d_recs);
        CK(cudaGetLastError());
    }
    // Temporaries the E-step never writes keep their initial value: the default
    // Param (1, 2) in parity mode (common.cu:57), nothing in clean mode.
    float a = mode == MC_MODE_PARITY ? 1.f : 0.f, b = mode == MC_MODE_PARITY ? 2.f : 0.f;
    CK(launch_fill2(d_tmp_atr, n * MC_R, a, b, st));
    if (d_tmp_sat) CK(launch_fill2(d_tmp_sat, n * MC_R, a, b, st));
    CK(launch_fill2(d_tmp_pub, n * n_pub, a, b, st));
    CK(cudaStreamSynchronize(st));
    return MC_OK;
}

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
extern "C" int mc_model_create(int model_type, int mode, int device, mc_model** out) {
    if (!out) return set_error(MC_ERR_INVALID, "model_create: null output");
    *out = nullptr;
    if (model_type < 0 || model_type > 3) return set_error(MC_ERR_INVALID, "model_create: model type must be 0..3");
    if (mode != MC_MODE_PARITY && mode != MC_MODE_CLEAN) return set_error(MC_ERR_INVALID, "model_create: bad mode");
    int count = 0;
    CK(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return set_error(MC_ERR_INVALID, "model_create: no such device");
    CK(cudaSetDevice(device));
    mc_model* m = new (std::nothrow) mc_model();
    if (!m) return set_error(MC_ERR_NOMEM, "model_create: out of host memory");
    m->model = model_type;
    m->mode = mode;
    m->device = device;
    m->n_pub = public_params(model_type);
    cudaDeviceGetAttribute(&m->n_sm, cudaDevAttrMultiProcessorCount, device);
    *out = m;
    return MC_OK;
}

extern "C" int mc_model_upload(mc_model* m, int64_t n, const int32_t* query, const int32_t* pidx,
                               const uint16_t* click, int64_t n_qd, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "model_upload: null model");
    if (n < 0 || n_qd < 0 || n > ((int64_t)1 << 31) - 64 || n_qd >= ((int64_t)1 << 31))
        return set_error(MC_ERR_INVALID, "model_upload: bad sizes");
    if (n > 0 && (!query || !pidx || !click)) return set_error(MC_ERR_INVALID, "model_upload: null input");
    CK(cudaSetDevice(m->device));
    m->free_train();
    cudaStream_t st = m->pick(stream);
    m->n = n;
    m->n_qd = n_qd;
    m->stride = std::max<int64_t>(32, (n + 31) / 32 * 32);

    // The query ids go up first, on st, so that the query segments are found
    // while the session indices and clicks follow on a side stream, in
    // chunks; the upload pass then runs on each chunk as its copy lands.  (With
    // the query copy queued behind the chunks, it landed last and every chunk's
    // upload pass waited for the end of the copies.)  The side stream first
    // waits for the work already queued on st (which may still be writing the
    // host buffers) and for the query copy.
    int rc;
    int32_t* d_src = nullptr;
    int32_t* d_q = nullptr;
    int64_t scratch = 0;
    if ((rc = dalloc(&d_src, (size_t)std::max<int64_t>(n * MC_R, 1), &scratch))) return rc;
    if ((rc = dalloc(&m->d_click, (size_t)std::max<int64_t>(n, 1), &m->bytes))) { dfree(d_src); return rc; }
    if ((rc = dalloc(&d_q, (size_t)std::max<int64_t>(n, 1), &scratch))) { dfree(d_src); return rc; }
    if (n) {
        cudaError_t eq = cudaMemcpyAsync(d_q, query, (size_t)n * 4, cudaMemcpyHostToDevice, st);
        if (eq != cudaSuccess) { dfree(d_src); dfree(d_q); m->free_train(); return cuda_fail("model_upload", eq); }
    }
    int n_chunks = 0;
    int64_t chunk_at[kUploadChunks + 1] = {0};
    if (n) {
        cudaError_t ec = cudaSuccess;
        if ((rc = m->ensure_copy_stream())) { dfree(d_src); return rc; }
        cudaStream_t cs = m->copy_stream;
        n_chunks = (int)std::min<int64_t>(kUploadChunks, std::max<int64_t>(1, n / 65536));
        for (int k = 0; k < n_chunks; k++) chunk_at[k] = std::min<int64_t>(n, (n * k / n_chunks + 31) / 32 * 32);
        chunk_at[n_chunks] = n;
        if (ec == cudaSuccess) ec = cudaEventRecord(m->copy_ev[kUploadChunks], st);
        if (ec == cudaSuccess) ec = cudaStreamWaitEvent(cs, m->copy_ev[kUploadChunks], 0);
        if (ec == cudaSuccess) ec = cudaMemcpyAsync(m->d_click, click, (size_t)n * 2, cudaMemcpyHostToDevice, cs);
        for (int k = 0; k < n_chunks && ec == cudaSuccess; k++) {
            const int64_t c0 = chunk_at[k], c1 = chunk_at[k + 1];
            if (c1 > c0)
                ec = cudaMemcpyAsync(d_src + c0 * MC_R, pidx + c0 * MC_R, (size_t)(c1 - c0) * MC_R * 4, cudaMemcpyHostToDevice, cs);
            if (ec == cudaSuccess) ec = cudaEventRecord(m->copy_ev[k], cs);
        }
        if (ec != cudaSuccess) {
            cudaStreamSynchronize(cs);
            cudaStreamSynchronize(st);
            dfree(d_src);
            dfree(d_q);
            m->free_train();
            return cuda_fail("model_upload", ec);
        }
    }
    // Frees the scratch after the copies and st have drained.
    auto drain = [&]() {
        if (m->copy_stream) cudaStreamSynchronize(m->copy_stream);
        cudaStreamSynchronize(st);
    };

    // Query segments (runs of equal query id), found on the device: block
    // counts, their prefix on the host, then seg_begin and each session's
    // segment index.
    int32_t* d_seg_id = nullptr;
    int64_t* d_seg_begin = nullptr;
    int64_t n_seg = 0;
    {
        int64_t scratch0 = 0;
        const int64_t nb = (n + kSegBlock - 1) / kSegBlock;
        int* d_blk = nullptr;
        int64_t* d_off = nullptr;
        int rc0;
        auto free0 = [&]() { dfree(d_blk); dfree(d_off); };
        if ((rc0 = dalloc(&d_seg_id, (size_t)std::max<int64_t>(n, 1), &scratch0)) ||
            (rc0 = dalloc(&d_blk, (size_t)std::max<int64_t>(nb, 1), &scratch0)) ||
            (rc0 = dalloc(&d_off, (size_t)std::max<int64_t>(nb, 1), &scratch0))) {
            drain();
            free0(); dfree(d_q); dfree(d_seg_id); dfree(d_src);
            return rc0;
        }
        std::vector<int> blk((size_t)nb);
        std::vector<int64_t> off((size_t)nb);
        cudaError_t e0 = cudaSuccess;
        auto ck0 = [&](cudaError_t x) { if (e0 == cudaSuccess) e0 = x; };
        if (n) {
            seg_count_kernel<<<(unsigned)nb, kSegBlock / 8, 0, st>>>(n, d_q, d_blk);
            ck0(cudaGetLastError());
            ck0(cudaMemcpyAsync(blk.data(), d_blk, (size_t)nb * 4, cudaMemcpyDeviceToHost, st));
            ck0(cudaStreamSynchronize(st));
            for (int64_t b = 0; b < nb; b++) { off[(size_t)b] = n_seg; n_seg += blk[(size_t)b]; }
            if (e0 == cudaSuccess && (rc0 = dalloc(&d_seg_begin, (size_t)std::max<int64_t>(n_seg, 1), &scratch0))) {
                drain();
                free0(); dfree(d_q); dfree(d_seg_id); dfree(d_src);
                return rc0;
            }
            ck0(cudaMemcpyAsync(d_off, off.data(), (size_t)nb * 8, cudaMemcpyHostToDevice, st));
            seg_write_kernel<<<(unsigned)nb, kSegBlock / 8, 0, st>>>(n, d_q, d_off, d_seg_begin, d_seg_id);
            ck0(cudaGetLastError());
        }
        ck0(m->seg_begin.resize((size_t)n_seg + 1));
        if (e0 == cudaSuccess) m->seg_begin[(size_t)n_seg] = n;
        if (n_seg && e0 == cudaSuccess)
            ck0(cudaMemcpyAsync(m->seg_begin.data(), d_seg_begin, (size_t)n_seg * 8, cudaMemcpyDeviceToHost, st));
        ck0(cudaStreamSynchronize(st));
        free0();
        dfree(d_q);
        if (e0 != cudaSuccess) {
            drain();
            dfree(d_seg_id); dfree(d_seg_begin); dfree(d_src);
            return cuda_fail("model_upload", e0);
        }
    }

    int64_t& B = m->bytes;
    auto fail_seg = [&](int code) {
        drain();
        dfree(d_seg_id); dfree(d_seg_begin); dfree(d_src);
        return code;
    };
    if ((rc = dalloc(&m->d_pidx, (size_t)(m->stride * MC_R), &B))) return fail_seg(rc);
    // Parameter arrays padded to a multiple of 4 entries plus 4, so 16-byte
    // aligned bulk copies of any window stay inside the allocation.
    const int64_t qd_alloc = m->qd_alloc();
    if ((rc = dalloc(&m->d_cnt, (size_t)qd_alloc, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_cnt16, (size_t)qd_alloc, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_atr, (size_t)qd_alloc, &B))) return fail_seg(rc);
    if (m->model == MC_DBN && (rc = dalloc(&m->d_sat, (size_t)qd_alloc, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_pub_theta, 2 * MC_MAX_PUB, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_pub_bins, (size_t)(2 * m->n_pub), &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_pub_const, (size_t)(2 * m->n_pub), &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_tiles_done, 1, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_iter, 1, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_status, 1, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_fit, 1, &B))) return fail_seg(rc);
    if ((rc = dalloc(&m->d_ws, 1, &B))) return fail_seg(rc);

    // Scratch for the preparation pass.
    int *d_seg_lo = nullptr, *d_seg_hi = nullptr, *d_flag = nullptr;
    unsigned long long* d_pub_counts = nullptr;
    uint32_t* d_packbits = nullptr;
    const int64_t n_words = (n + 31) / 32;
    auto free_scratch = [&]() { drain(); dfree(d_src); dfree(d_seg_begin); dfree(d_seg_id); dfree(d_seg_lo); dfree(d_seg_hi); dfree(d_flag); dfree(d_pub_counts); dfree(d_packbits); };
    if ((rc = dalloc(&d_seg_lo, (size_t)std::max<int64_t>(n_seg, 1), &scratch)) ||
        (rc = dalloc(&d_seg_hi, (size_t)std::max<int64_t>(n_seg, 1), &scratch)) ||
        (rc = dalloc(&d_flag, 2, &scratch)) || (rc = dalloc(&d_pub_counts, MC_PUB_COUNTS, &scratch)) ||
        (rc = dalloc(&d_packbits, (size_t)std::max<int64_t>(n_words, 1), &scratch))) {
        free_scratch();
        return rc;
    }
    cudaError_t e = cudaSuccess;
    auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    {
        const int64_t ns = std::max<int64_t>(n_seg, 1);
        const int g = (int)std::min<int64_t>((ns + 255) / 256, (int64_t)4 * m->n_sm);
        fill_i32_kernel<<<g, 256, 0, st>>>(d_seg_lo, ns, INT_MAX);
        fill_i32_kernel<<<g, 256, 0, st>>>(d_seg_hi, ns, INT_MIN);
        ck(cudaGetLastError());
    }
    ck(cudaMemsetAsync(d_flag, 0, 8, st));
    ck(cudaMemsetAsync(d_pub_counts, 0, MC_PUB_COUNTS * 8, st));
    // Planes: the upload pass writes sessions [0, n); only the padding up to
    // the stride needs clearing.
    if (m->stride > n)
        ck(cudaMemset2DAsync(m->d_pidx + n, (size_t)m->stride * 4, 0, (size_t)(m->stride - n) * 4, MC_R, st));
    ck(cudaMemsetAsync(m->d_cnt, 0, (size_t)qd_alloc * sizeof(uint2), st));
    if (n && e == cudaSuccess) {
        const int hist_bytes = kPrepHist * (int)sizeof(uint2);
        ck(cudaFuncSetAttribute(prep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, hist_bytes));
        for (int k = 0; k < n_chunks && e == cudaSuccess; k++) {
            const int64_t c0 = chunk_at[k], c1 = chunk_at[k + 1], len = c1 - c0;
            ck(cudaStreamWaitEvent(st, m->copy_ev[k], 0));
            if (len <= 0) continue;
            const int64_t grid = std::min<int64_t>((len + kPrepThreads - 1) / kPrepThreads, (int64_t)4 * m->n_sm);
            const int64_t chunk = ((len + grid - 1) / grid + 31) / 32 * 32;
            const int blocks = (int)((len + chunk - 1) / chunk);
            prep_kernel<<<blocks, kPrepThreads, hist_bytes, st>>>(c0, c1, chunk, m->stride, n_qd, d_src, m->d_click,
                                                                  d_seg_id, m->model, m->d_pidx, m->d_cnt, d_seg_lo,
                                                                  d_seg_hi, d_pub_counts, d_packbits, d_flag);
            ck(cudaGetLastError());
        }
    }
    {
        int grid = (int)std::min<int64_t>((qd_alloc + 255) / 256, (int64_t)8 * m->n_sm);
        pack_counts_kernel<<<grid, 256, 0, st>>>(m->d_cnt, m->d_cnt16, qd_alloc);
        ck(cudaGetLastError());
    }
    if (n_seg > 1) {
        const int g = (int)std::min<int64_t>((n_seg + 255) / 256, (int64_t)4 * m->n_sm);
        seg_order_kernel<<<g, 256, 0, st>>>(n_seg, d_seg_lo, d_seg_hi, d_flag + 1);
        ck(cudaGetLastError());
    }
    int flags[2] = {0, 0};  // [0] an index outside [0, n_qd), [1] segments out of order
    std::vector<unsigned long long> pub_counts(MC_PUB_COUNTS, 0);
    ck(cudaMemcpyAsync(flags, d_flag, 8, cudaMemcpyDeviceToHost, st));
    ck(cudaMemcpyAsync(pub_counts.data(), d_pub_counts, pub_counts.size() * 8, cudaMemcpyDeviceToHost, st));
    ck(m->packbits.resize((size_t)n_words));
    if (n_words && e == cudaSuccess)
        ck(cudaMemcpyAsync(m->packbits.data(), d_packbits, (size_t)n_words * 4, cudaMemcpyDeviceToHost, st));
    ck(m->seg_lo.resize((size_t)n_seg));
    ck(m->seg_hi.resize((size_t)n_seg));
    if (n_seg && e == cudaSuccess) {
        ck(cudaMemcpyAsync(m->seg_lo.data(), d_seg_lo, (size_t)n_seg * 4, cudaMemcpyDeviceToHost, st));
        ck(cudaMemcpyAsync(m->seg_hi.data(), d_seg_hi, (size_t)n_seg * 4, cudaMemcpyDeviceToHost, st));
    }
    ck(cudaStreamSynchronize(st));
    free_scratch();
    if (e != cudaSuccess) return cuda_fail("model_upload", e);
    if (flags[0]) {
        m->free_train();
        return set_error(MC_ERR_INVALID, "model_upload: a parameter index is outside [0, n_qd)");
    }
    if ((m->model == MC_PBM || m->model == MC_UBM) && n) {
        int usable = 0;
        int64_t n_ent = 0;
        e = build_counts(m->model, n, m->stride, n_qd, m->d_pidx, m->d_click, m->n_sm, st, &m->d_coff, &m->d_cent,
                         &n_ent, &m->d_cdense, &usable);
        if (e != cudaSuccess) {
            m->free_train();
            return cuda_fail("model_upload", e);
        }
        if (usable) {
            m->n_cent = n_ent;
            m->bytes += (int64_t)sizeof(uint32_t) * ((n_qd + 1) + std::max<int64_t>(n_ent, 1));
            if (m->d_cdense) m->bytes += (int64_t)sizeof(uint16_t) * n_qd * MC_R;
        }
    }

    // Fused path precondition: per-query qd ranges disjoint and increasing.
    m->fused_ok = !flags[1];
    if (!m->fused_ok)
        m->fused_reason = "sessions are not grouped by query with per-query contiguous parameter indices "
                          "(as Dataset::parse_dataset leaves them)";

    // Public constants: prior plus the parts fixed by the click pattern.
    std::vector<double> pconst((size_t)(2 * m->n_pub), 0.0);
    for (int k = 0; k < m->n_pub; k++) {
        double num = 1.0, den = 2.0;
        if (m->model == MC_PBM) { num += (double)pub_counts[(size_t)k]; den += (double)n; }
        // Ranks before a session's last click contribute exactly (1, 1) to the
        // DBN gamma and, when unclicked, to the CCM tau_1 (the z = 0 factor of
        // such a rank is zero); sessions without clicks contribute (10, 10).
        if (m->model == MC_DBN) {
            num += (double)pub_counts[MC_CNT_DBN_BEFORE_LAST];
            den += (double)pub_counts[MC_CNT_DBN_BEFORE_LAST];
        }
        if (m->model == MC_CCM && k == 0) {
            num += (double)pub_counts[MC_CNT_CCM_UNCLICKED_BEFORE_LAST];
            den += (double)pub_counts[MC_CNT_CCM_UNCLICKED_BEFORE_LAST];
        }
        if (m->model == MC_UBM) {
            double w = (double)pub_counts[(size_t)k], wc = (double)pub_counts[(size_t)(MC_UBM_SLOTS + k)];
            num += wc;
            den += w;
            if (m->mode == MC_MODE_PARITY) { num += (double)n - w; den += 2.0 * ((double)n - w); }
        }
        pconst[(size_t)(2 * k)] = num;
        pconst[(size_t)(2 * k + 1)] = den;
    }
    if ((rc = m->prior_values(st))) return rc;
    CK(cudaMemsetAsync(m->d_pub_bins, 0, (size_t)(2 * m->n_pub) * 8, st));
    CK(cudaMemcpyAsync(m->d_pub_const, pconst.data(), pconst.size() * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(m->d_tiles_done, 0, 4, st));
    CK(cudaMemsetAsync(m->d_status, 0, 4, st));
    CK(cudaMemsetAsync(m->d_ws, 0, sizeof(WorkState), st));
    CK(cudaStreamSynchronize(st));
    m->uploaded = true;
    // The count path (PBM/UBM) reads the fit descriptor whether or not the
    // sessions admit tiles; build_tiles rewrites it with the tile fields.
    if ((rc = m->write_fit_desc())) return rc;
    if (m->fused_ok && !m->d_coff && (rc = m->build_tiles())) return rc;
    return MC_OK;
}

extern "C" int mc_model_upload_test(mc_model* m, int64_t n, const int32_t* pidx, const uint16_t* click, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "model_upload_test: null model");
    if (n < 0) return set_error(MC_ERR_INVALID, "model_upload_test: negative size");
    if (n > 0 && (!pidx || !click)) return set_error(MC_ERR_INVALID, "model_upload_test: null input");
    CK(cudaSetDevice(m->device));
    m->free_test();
    cudaStream_t st = m->pick(stream);
    m->n_test = n;
    m->test_stride = std::max<int64_t>(32, (n + 31) / 32 * 32);
    std::vector<int32_t> planes((size_t)(m->test_stride * MC_R), -1);
    for (int64_t s = 0; s < n; s++)
        for (int r = 0; r < MC_R; r++) planes[(size_t)(r * m->test_stride + s)] = pidx[s * MC_R + r];
    int64_t before = m->bytes;
    int rc;
    if ((rc = dalloc(&m->d_test_pidx, planes.size(), &m->bytes))) return rc;
    if ((rc = dalloc(&m->d_test_click, (size_t)std::max<int64_t>(n, 1), &m->bytes))) return rc;
    if ((rc = dalloc(&m->d_eval, MC_R + 1, &m->bytes))) return rc;
    m->test_bytes = m->bytes - before;
    CK(cudaMemcpyAsync(m->d_test_pidx, planes.data(), planes.size() * 4, cudaMemcpyHostToDevice, st));
    if (n) CK(cudaMemcpyAsync(m->d_test_click, click, (size_t)n * 2, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    return MC_OK;
}

extern "C" int mc_model_configure(mc_model* m, int32_t spt, int32_t wqd, int32_t block) {
    if (!m) return set_error(MC_ERR_INVALID, "model_configure: null model");
    if (spt < 0 || wqd < 0 || block < 0) return set_error(MC_ERR_INVALID, "model_configure: negative value");
    if (block && (block % 32 || block < 64 || block > FUSED_THREADS))
        return set_error(MC_ERR_INVALID, "model_configure: block must be a multiple of 32 in [64, " + std::to_string(FUSED_THREADS) + "]");
    if (wqd && wqd > 16384) return set_error(MC_ERR_INVALID, "model_configure: window above 16384 qd");
    if (spt && spt > 4096) return set_error(MC_ERR_INVALID, "model_configure: sessions per tile above 4096");
    wqd = (wqd + 7) & ~7;
    CK(cudaSetDevice(m->device));
    const int spt0 = m->spt, wqd0 = m->wqd, block0 = m->block;
    if (spt) m->spt = spt;
    if (wqd) m->wqd = wqd;
    if (block) m->block = block;
    // Unchanged shape: the tiles, occupancy and graphs stay valid.
    if (m->spt == spt0 && m->wqd == wqd0 && m->block == block0) return MC_OK;
    // Count-path models rebuild tiles only if a batch already made them.
    if (m->uploaded && m->fused_ok && (!m->d_coff || m->tiles_ready)) return m->build_tiles();
    return MC_OK;
}

extern "C" int mc_model_get_config(const mc_model* m, int32_t* spt, int32_t* wqd, int32_t* block) {
    if (!m) return set_error(MC_ERR_INVALID, "model_get_config: null model");
    if (spt) *spt = m->spt;
    if (wqd) *wqd = m->wqd;
    if (block) *block = m->block;
    return MC_OK;
}

// One fused iteration: PBM and UBM from their per-(qd, key) counts, the
// other models (or sizes beyond the count format) through the tile kernel.
static cudaError_t launch_fused_once(mc_model* m, cudaStream_t st) {
    if (m->d_cdense) return launch_em_counts_pbm_dense(m->d_fit, m->d_cdense, m->n_qd, m->n_sm, m->dense_shape, st);
    if (m->d_coff) return launch_em_counts(m->d_fit, m->d_coff, m->d_cent, m->n_qd, m->n_sm, m->count_shape, st);
    return launch_em_fused(m->model, m->d_fit, m->d_tiles, m->n_tiles, m->d_splits, m->d_ws, m->wqd, m->spt, m->stages,
                           m->grid, m->block, nullptr, 0, 0, st);
}

static int launch_fused_loop(mc_model* m, int iters, cudaStream_t st) {
    for (int i = 0; i < iters; i++) CK(launch_fused_once(m, st));
    return MC_OK;
}

extern "C" int mc_model_em(mc_model* m, int32_t iters, int impl, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "model_em: null model");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "model_em: no training sessions uploaded");
    if (iters < 0) return set_error(MC_ERR_INVALID, "model_em: negative iteration count");
    if (impl != MC_IMPL_FUSED && impl != MC_IMPL_PLAIN) return set_error(MC_ERR_INVALID, "model_em: bad impl");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    if (iters == 0 || m->n == 0) return MC_OK;
    if (impl == MC_IMPL_FUSED) {
        // The count path (PBM/UBM) does not depend on the session order.
        if (!m->fused_ok && !m->d_coff)
            return set_error(MC_ERR_INVALID, "model_em: fused path unavailable: " + m->fused_reason);
        // The loop is captured as graphs of at most kGraphChunk iterations
        // (one full chunk, one remainder), each replayed as often as needed.
        const int full = iters / kGraphChunk, rem = iters % kGraphChunk;
        for (int pass = 0; pass < 2; pass++) {
            int len = pass == 0 ? kGraphChunk : rem;
            int reps = pass == 0 ? full : (rem ? 1 : 0);
            if (!reps) continue;
            auto& slot = m->graphs[pass];
            if (!slot.exec || slot.iters != len) {
                if (slot.exec) cudaGraphExecDestroy(slot.exec);
                slot.exec = nullptr;
                cudaGraph_t g = nullptr;
                CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                int rc = launch_fused_loop(m, len, st);
                cudaError_t e = cudaStreamEndCapture(st, &g);
                if (rc) { if (g) cudaGraphDestroy(g); return rc; }
                if (e != cudaSuccess) return cuda_fail("cudaStreamEndCapture", e);
                e = cudaGraphInstantiate(&slot.exec, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) { slot.exec = nullptr; return cuda_fail("cudaGraphInstantiate", e); }
                slot.iters = len;
            }
            for (int k = 0; k < reps; k++) CK(cudaGraphLaunch(slot.exec, st));
        }
    } else {
        int rc = m->ensure_plain(st);
        if (rc) return rc;
        PlainArgs A{m->n, m->n_qd, m->d_recs, m->d_atr2, m->d_sat2, m->d_pub2, m->d_tmp_atr, m->d_tmp_sat, m->d_tmp_pub};
        CK(launch_values_to_pairs(m->d_atr, m->d_atr2, m->n_qd, st));
        if (m->d_sat) CK(launch_values_to_pairs(m->d_sat, m->d_sat2, m->n_qd, st));
        pub_to_pairs_kernel<<<1, 64, 0, st>>>(m->d_pub_theta, m->d_iter, m->d_pub2, m->n_pub);
        CK(cudaGetLastError());
        for (int i = 0; i < iters; i++) {
            CK(launch_plain_estep(m->model, A, st));
            CK(launch_plain_reset(A, m->n_pub, st));
            CK(launch_plain_update(m->model, A, st));
        }
        CK(launch_pairs_to_values(m->d_atr2, m->d_atr, m->n_qd, st));
        if (m->d_sat) CK(launch_pairs_to_values(m->d_sat2, m->d_sat, m->n_qd, st));
        pairs_to_pub_kernel<<<1, 64, 0, st>>>(m->d_pub2, m->d_pub_theta, m->d_iter, m->n_pub);
        CK(cudaGetLastError());
    }
    if (!stream) CK(cudaStreamSynchronize(st));
    return MC_OK;
}

extern "C" int mc_model_process_sessions(mc_model* m, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "process_sessions: null model");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "process_sessions: no training sessions uploaded");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    int rc = m->ensure_plain(st);
    if (rc) return rc;
    PlainArgs A{m->n, m->n_qd, m->d_recs, m->d_atr2, m->d_sat2, m->d_pub2, m->d_tmp_atr, m->d_tmp_sat, m->d_tmp_pub};
    CK(launch_values_to_pairs(m->d_atr, m->d_atr2, m->n_qd, st));
    if (m->d_sat) CK(launch_values_to_pairs(m->d_sat, m->d_sat2, m->n_qd, st));
    pub_to_pairs_kernel<<<1, 64, 0, st>>>(m->d_pub_theta, m->d_iter, m->d_pub2, m->n_pub);
    CK(cudaGetLastError());
    CK(launch_plain_estep(m->model, A, st));
    if (!stream) CK(cudaStreamSynchronize(st));
    return MC_OK;
}

extern "C" int mc_model_update_parameters(mc_model* m, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "update_parameters: null model");
    if (!m->uploaded || !m->d_recs) return set_error(MC_ERR_STATE, "update_parameters: call process_sessions first");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    PlainArgs A{m->n, m->n_qd, m->d_recs, m->d_atr2, m->d_sat2, m->d_pub2, m->d_tmp_atr, m->d_tmp_sat, m->d_tmp_pub};
    CK(launch_plain_reset(A, m->n_pub, st));
    CK(launch_plain_update(m->model, A, st));
    CK(launch_pairs_to_values(m->d_atr2, m->d_atr, m->n_qd, st));
    if (m->d_sat) CK(launch_pairs_to_values(m->d_sat2, m->d_sat, m->n_qd, st));
    pairs_to_pub_kernel<<<1, 64, 0, st>>>(m->d_pub2, m->d_pub_theta, m->d_iter, m->n_pub);
    CK(cudaGetLastError());
    if (!stream) CK(cudaStreamSynchronize(st));
    return MC_OK;
}

extern "C" int mc_model_param_count(const mc_model* m) { return m ? (int)m->params().size() : 0; }

extern "C" int mc_model_param_info(const mc_model* m, int index, char* name, size_t name_len, int64_t* size, int* is_public) {
    if (!m) return set_error(MC_ERR_INVALID, "param_info: null model");
    auto ps = m->params();
    if (index < 0 || index >= (int)ps.size()) return set_error(MC_ERR_INVALID, "param_info: index out of range");
    if (name && name_len) {
        std::strncpy(name, ps[(size_t)index].name, name_len - 1);
        name[name_len - 1] = 0;
    }
    if (size) *size = ps[(size_t)index].kind == 0 ? m->n_pub : m->n_qd;
    if (is_public) *is_public = ps[(size_t)index].kind == 0;
    return MC_OK;
}

static int check_status(mc_model* m, cudaStream_t st) {
    CK(cudaStreamSynchronize(st));
    int status = 0;
    CK(cudaMemcpy(&status, m->d_status, 4, cudaMemcpyDeviceToHost));
    if (status & ST_TIMEOUT)
        return set_error(MC_ERR_DEVICE, "a kernel's wait for a tile's data timed out; the fit's results are incomplete (status " +
                                            std::to_string(status) + ")");
    if (status) return set_error(MC_ERR_DEVICE, "kernel reported a parameter index outside its query's window (status " + std::to_string(status) + ")");
    return MC_OK;
}

extern "C" int mc_test_wait_hooks(int device, int64_t wait_limit_ns, int32_t stall_tile) {
    if (wait_limit_ns < 0 || stall_tile < -1) return set_error(MC_ERR_INVALID, "test_wait_hooks: bad argument");
    int cur = 0;
    CK(cudaGetDevice(&cur));
    CK(cudaSetDevice(device));
    cudaError_t e = mcd::set_wait_hooks(wait_limit_ns ? (unsigned long long)wait_limit_ns : 4000000000ull, stall_tile);
    cudaSetDevice(cur);
    CK(e);
    return MC_OK;
}

static int current_iter(mc_model* m, int* it) {
    CK(cudaMemcpy(it, m->d_iter, 4, cudaMemcpyDeviceToHost));
    return MC_OK;
}

extern "C" int mc_model_get_param(mc_model* m, int index, float* values, void* stream) {
    if (!m || !values) return set_error(MC_ERR_INVALID, "get_param: null argument");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "get_param: no training sessions uploaded");
    auto ps = m->params();
    if (index < 0 || index >= (int)ps.size()) return set_error(MC_ERR_INVALID, "get_param: index out of range");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    int rc = check_status(m, st);
    if (rc) return rc;
    int kind = ps[(size_t)index].kind;
    if (kind == 0) {
        int it = 0;
        if ((rc = current_iter(m, &it))) return rc;
        CK(cudaMemcpy(values, m->d_pub_theta + (it & 1) * MC_MAX_PUB, (size_t)m->n_pub * 4, cudaMemcpyDeviceToHost));
    } else if (m->n_qd) {
        CK(cudaMemcpy(values, kind == 1 ? m->d_atr : m->d_sat, (size_t)m->n_qd * 4, cudaMemcpyDeviceToHost));
    }
    return MC_OK;
}

extern "C" int mc_model_set_param(mc_model* m, int index, const float* values, void* stream) {
    if (!m || !values) return set_error(MC_ERR_INVALID, "set_param: null argument");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "set_param: no training sessions uploaded");
    auto ps = m->params();
    if (index < 0 || index >= (int)ps.size()) return set_error(MC_ERR_INVALID, "set_param: index out of range");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    CK(cudaStreamSynchronize(st));
    int kind = ps[(size_t)index].kind;
    if (kind == 0) {
        int it = 0, rc;
        if ((rc = current_iter(m, &it))) return rc;
        CK(cudaMemcpy(m->d_pub_theta + (it & 1) * MC_MAX_PUB, values, (size_t)m->n_pub * 4, cudaMemcpyHostToDevice));
    } else if (m->n_qd) {
        CK(cudaMemcpy(kind == 1 ? m->d_atr : m->d_sat, values, (size_t)m->n_qd * 4, cudaMemcpyHostToDevice));
    }
    return MC_OK;
}

extern "C" int mc_model_evaluate(mc_model* m, int which, double* ll_sum, double* log2_sums, int64_t* n_sessions, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "evaluate: null model");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "evaluate: no training sessions uploaded");
    if (which != 0 && which != 1) return set_error(MC_ERR_INVALID, "evaluate: which must be 0 (train) or 1 (test)");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    int rc = check_status(m, st);
    if (rc) return rc;
    int it = 0;
    if ((rc = current_iter(m, &it))) return rc;
    double out[MC_R + 1] = {0};
    int64_t nn = which == 0 ? m->n : m->n_test;
    if (nn > 0) {
        if (!m->d_eval) {
            int64_t before = m->bytes;
            if ((rc = dalloc(&m->d_eval, MC_R + 1, &m->bytes))) return rc;
            m->test_bytes += m->bytes - before;
        }
        EvalArgs A;
        A.model = m->model;
        A.n = nn;
        A.stride = which == 0 ? m->stride : m->test_stride;
        A.n_qd = m->n_qd;
        A.pidx = which == 0 ? m->d_pidx : m->d_test_pidx;
        A.click = which == 0 ? m->d_click : m->d_test_click;
        A.atr = m->d_atr;
        A.sat = m->d_sat;
        A.pub = m->d_pub_theta + (it & 1) * MC_MAX_PUB;
        A.out = m->d_eval;
        CK(cudaMemsetAsync(m->d_eval, 0, (MC_R + 1) * 8, st));
        CK(launch_eval(A, m->n_sm, st));
        CK(cudaMemcpyAsync(out, m->d_eval, (MC_R + 1) * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    if (ll_sum) *ll_sum = out[0];
    if (log2_sums) for (int r = 0; r < MC_R; r++) log2_sums[r] = out[1 + r];
    if (n_sessions) *n_sessions = nn;
    return MC_OK;
}

extern "C" int mc_model_em_trace(mc_model* m, int32_t iters, double* train_ll, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "em_trace: null model");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "em_trace: no training sessions uploaded");
    if (iters < 0) return set_error(MC_ERR_INVALID, "em_trace: negative iteration count");
    if (iters > 0 && !train_ll) return set_error(MC_ERR_INVALID, "em_trace: null output");
    if (!m->fused_ok && !m->d_coff)
        return set_error(MC_ERR_INVALID, "em_trace: fused path unavailable: " + m->fused_reason);
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    if (iters == 0) return MC_OK;
    if (m->n == 0) {
        for (int i = 0; i < iters; i++) train_ll[i] = 0.0;
        return MC_OK;
    }
    double* d_trace = nullptr;
    int64_t scratch = 0;
    int rc = dalloc(&d_trace, (size_t)iters * (MC_R + 1), &scratch);
    if (rc) return rc;
    std::vector<double> host((size_t)iters * (MC_R + 1));
    cudaError_t e = cudaSuccess;
    auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    ck(cudaMemsetAsync(d_trace, 0, host.size() * 8, st));
    EvalArgs A;
    A.model = m->model;
    A.n = m->n;
    A.stride = m->stride;
    A.n_qd = m->n_qd;
    A.pidx = m->d_pidx;
    A.click = m->d_click;
    A.atr = m->d_atr;
    A.sat = m->d_sat;
    A.pub = m->d_pub_theta;
    A.iter = m->d_iter;  // the public half written by the iteration just run
    for (int i = 0; i < iters && e == cudaSuccess; i++) {
        ck(launch_fused_once(m, st));
        A.out = d_trace + (int64_t)i * (MC_R + 1);
        ck(launch_eval(A, m->n_sm, st));
    }
    ck(cudaMemcpyAsync(host.data(), d_trace, host.size() * 8, cudaMemcpyDeviceToHost, st));
    ck(cudaStreamSynchronize(st));
    dfree(d_trace);
    if (e != cudaSuccess) return cuda_fail("em_trace", e);
    if ((rc = check_status(m, st))) return rc;
    for (int i = 0; i < iters; i++) train_ll[i] = host[(size_t)i * (MC_R + 1)];
    return MC_OK;
}

// Times 3 fused iterations (after one warm-up) of the model's current shape.
static int time_fused(mc_model* m, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
    if (launch_fused_loop(m, 1, st) != MC_OK) return MC_ERR_INVALID;
    CK(cudaEventRecord(e0, st));
    if (launch_fused_loop(m, 3, st) != MC_OK) return MC_ERR_INVALID;
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(ms, e0, e1));
    return MC_OK;
}

// Count path: bin copies, block size and blocks per SM of the count kernel.
static int autotune_counts(mc_model* m, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1) {
    const bool dense = m->d_cdense != nullptr;
    const CountShape entry_cands[] = {{8, 256, 8}, {16, 256, 6}, {4, 256, 8}, {8, 128, 16}, {16, 128, 12}, {8, 192, 10}};
    const CountShape dense_cands[] = {{0, 256, 6}, {0, 256, 8}, {0, 128, 12}, {0, 128, 16}, {0, 192, 8}, {0, 256, 4}};
    CountShape& shape = dense ? m->dense_shape : m->count_shape;
    CountShape pick = shape;
    float best = 1e30f;
    for (const CountShape& c : dense ? dense_cands : entry_cands) {
        shape = c;
        float ms = 0.f;
        if (time_fused(m, st, e0, e1, &ms) != MC_OK) continue;
        if (ms < best) { best = ms; pick = c; }
    }
    shape = pick;
    return MC_OK;
}

extern "C" int mc_model_configure_counts(mc_model* m, int32_t copies, int32_t block, int32_t blocks_per_sm) {
    if (!m) return set_error(MC_ERR_INVALID, "model_configure_counts: null model");
    const bool dense = m->d_cdense != nullptr;
    CountShape c{dense ? 0 : copies, block, blocks_per_sm};
    if (!count_shape_valid(c, dense))
        return set_error(MC_ERR_INVALID, "model_configure_counts: copies 4, 8 or 16; block a multiple of 32 in [64, 256]; "
                                         "blocks per SM in [1, 32]");
    (dense ? m->dense_shape : m->count_shape) = c;
    return MC_OK;
}

extern "C" int mc_model_get_count_config(const mc_model* m, int32_t* copies, int32_t* block, int32_t* blocks_per_sm) {
    if (!m) return set_error(MC_ERR_INVALID, "model_get_count_config: null model");
    const CountShape& c = m->d_cdense ? m->dense_shape : m->count_shape;
    if (copies) *copies = c.copies;
    if (block) *block = c.block;
    if (blocks_per_sm) *blocks_per_sm = c.blocks_per_sm;
    return MC_OK;
}

extern "C" int mc_model_autotune(mc_model* m, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "autotune: null model");
    if (!m->uploaded || (!m->fused_ok && !m->d_coff))
        return set_error(MC_ERR_STATE, "autotune: needs uploaded sessions and the fused path");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    CK(cudaStreamSynchronize(st));
    // Snapshot of the state the trial iterations change.
    std::vector<float> atr((size_t)m->qd_alloc()), sat, th(2 * MC_MAX_PUB);
    int it0 = 0;
    CK(cudaMemcpy(atr.data(), m->d_atr, atr.size() * 4, cudaMemcpyDeviceToHost));
    if (m->d_sat) { sat.resize(atr.size()); CK(cudaMemcpy(sat.data(), m->d_sat, sat.size() * 4, cudaMemcpyDeviceToHost)); }
    CK(cudaMemcpy(th.data(), m->d_pub_theta, th.size() * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&it0, m->d_iter, 4, cudaMemcpyDeviceToHost));
    auto restore = [&]() -> int {
        CK(cudaMemcpy(m->d_atr, atr.data(), atr.size() * 4, cudaMemcpyHostToDevice));
        if (m->d_sat) CK(cudaMemcpy(m->d_sat, sat.data(), sat.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(m->d_pub_theta, th.data(), th.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(m->d_iter, &it0, 4, cudaMemcpyHostToDevice));
        return check_status(m, st);
    };
    if (m->d_coff) {
        cudaEvent_t c0, c1;
        CK(cudaEventCreate(&c0));
        CK(cudaEventCreate(&c1));
        int rc = autotune_counts(m, st, c0, c1);
        cudaEventDestroy(c0);
        cudaEventDestroy(c1);
        if (rc) return rc;
        return restore();
    }
    struct Cand { int spt, wqd, block; };
    const Cand cands[] = {{1024, 1536, 256}, {512, 1024, 256}, {1024, 1024, 256}, {2048, 1536, 256},
                          {512, 1024, 160}, {1024, 1536, 192}, {512, 768, 160}, {256, 512, 128}};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    Cand pick = {m->spt, m->wqd, m->block};
    for (const Cand& c : cands) {
        m->spt = c.spt; m->wqd = c.wqd; m->block = c.block;
        if (m->build_tiles() != MC_OK) continue;
        float ms = 0.f;
        if (time_fused(m, st, e0, e1, &ms) != MC_OK) continue;
        if (ms < best) { best = ms; pick = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    m->spt = pick.spt; m->wqd = pick.wqd; m->block = pick.block;
    int rc = m->build_tiles();
    if (rc) return rc;
    return restore();
}

extern "C" int mc_model_fused_path(const mc_model* m, int32_t* path, int64_t* n_entries) {
    if (!m || !path || !n_entries) return set_error(MC_ERR_INVALID, "model_fused_path: null argument");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "model_fused_path: no training sessions uploaded");
    *path = m->d_cdense ? 2 : m->d_coff ? 1 : 0;
    *n_entries = m->d_coff ? m->n_cent : 0;
    return MC_OK;
}

extern "C" int mc_model_memory(const mc_model* m, int64_t* bytes) {
    if (!m || !bytes) return set_error(MC_ERR_INVALID, "model_memory: null argument");
    *bytes = m->bytes;
    return MC_OK;
}

extern "C" void mc_model_destroy(mc_model* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    m->free_test();
    m->free_train();
    if (m->own_stream) cudaStreamDestroy(m->own_stream);
    if (m->copy_stream) cudaStreamDestroy(m->copy_stream);
    for (cudaEvent_t ev : m->copy_ev)
        if (ev) cudaEventDestroy(ev);
    delete m;
}

extern "C" int mc_model_init_parameters(mc_model* m, void* stream) {
    if (!m) return set_error(MC_ERR_INVALID, "init_parameters: null model");
    if (!m->uploaded) return set_error(MC_ERR_STATE, "init_parameters: no training sessions uploaded");
    CK(cudaSetDevice(m->device));
    cudaStream_t st = m->pick(stream);
    if (int rc = m->prior_values(st)) return rc;
    CK(cudaStreamSynchronize(st));
    return MC_OK;
}

// ---------------------------------------------------------------------------
// Batches: several fits in one persistent launch per iteration
// ---------------------------------------------------------------------------
struct mc_batch {
    std::vector<mc_model*> models;
    int device = 0, n_sm = 0, kernel_model = -1;
    int spt = 0, wqd = 0, block = 0, stages = 2, grid = 1, n_tiles = 0;
    FitDev* d_fits = nullptr;
    TileDev* d_tiles = nullptr;
    SplitDev* d_splits = nullptr;
    WorkState* d_ws = nullptr;
    // Fits on the count path (PBM/UBM) run in one batched count launch.
    CountFitDev* d_cfits = nullptr;
    int n_cfits = 0, count_blocks = 0;
    // Count chunks taken by the tile launch itself (one launch per iteration)
    // or by a count launch after it (the default: measured faster, since the
    // count kernel runs more warps per SM than the tile kernel's two CTAs).
    bool single_launch = false;
    int grid_cap = 1;  // resident tile-kernel CTAs on the device
    mc_model::GraphSlot graphs[2];
    cudaStream_t own_stream = nullptr;
    int64_t bytes = 0;

    void release() {
        for (auto& g : graphs) { if (g.exec) cudaGraphExecDestroy(g.exec); g.exec = nullptr; g.iters = -1; }
        settle(d_fits, d_tiles, d_splits, d_ws, d_cfits);
        dfree(d_fits); dfree(d_tiles); dfree(d_splits); dfree(d_ws); dfree(d_cfits);
        if (own_stream) cudaStreamDestroy(own_stream);
        own_stream = nullptr;
    }
};

// One iteration of every fit: the tile kernel over the tile fits, then the
// batched count kernel over the count-path fits.
static int batch_launch_loop(mc_batch* b, int iters, cudaStream_t st) {
    for (int i = 0; i < iters; i++) {
        // single_launch: the tile kernel takes the count chunks of the
        // count-path fits after its tiles; otherwise a count launch follows
        // the tile launch.  A batch without tile fits runs the count kernel.
        const bool merged = b->single_launch && b->n_tiles && b->n_cfits;
        if (b->n_tiles) {
            const int grid = std::max(1, std::min(b->n_tiles + (merged ? b->count_blocks : 0), b->grid_cap));
            CK(launch_em_fused(b->kernel_model, b->d_fits, b->d_tiles, b->n_tiles, b->d_splits, b->d_ws, b->wqd, b->spt,
                               b->stages, grid, b->block, merged ? b->d_cfits : nullptr, merged ? b->n_cfits : 0,
                               merged ? b->count_blocks : 0, st));
        }
        if (b->n_cfits && !merged) CK(launch_em_counts_batch(b->d_cfits, b->n_cfits, b->count_blocks, st));
    }
    return MC_OK;
}

extern "C" int mc_batch_create(int n_models, mc_model* const* models, mc_batch** out) {
    if (!out || !models || n_models < 1) return set_error(MC_ERR_INVALID, "batch_create: need at least one model");
    *out = nullptr;
    for (int i = 0; i < n_models; i++) {
        mc_model* m = models[i];
        if (!m || !m->uploaded) return set_error(MC_ERR_STATE, "batch_create: every model must have uploaded sessions");
        if (!m->fused_ok) return set_error(MC_ERR_INVALID, "batch_create: model " + std::to_string(i) + ": " + m->fused_reason);
        if (m->device != models[0]->device) return set_error(MC_ERR_INVALID, "batch_create: models on different devices");
    }
    CK(cudaSetDevice(models[0]->device));
    // Count-path fits (PBM/UBM with their counts) need no tiles; the others
    // share one tile shape: the first tile fit's.
    auto on_counts = [](const mc_model* m) { return m->d_coff != nullptr; };
    mc_model* m0 = models[0];
    for (int i = 0; i < n_models; i++)
        if (!on_counts(models[i])) { m0 = models[i]; break; }
    for (int i = 0; i < n_models; i++) {
        mc_model* m = models[i];
        if (on_counts(m) || m == m0) continue;
        if (m->spt != m0->spt || m->wqd != m0->wqd || m->block != m0->block) {
            int rc = mc_model_configure(m, m0->spt, m0->wqd, m0->block);
            if (rc) return rc;
        }
    }
    mc_batch* b = new (std::nothrow) mc_batch();
    if (!b) return set_error(MC_ERR_NOMEM, "batch_create: out of host memory");
    b->models.assign(models, models + n_models);
    b->device = m0->device;
    b->n_sm = m0->n_sm;
    b->spt = m0->spt;
    b->wqd = m0->wqd;
    b->block = m0->block;
    b->kernel_model = m0->model;
    std::vector<FitDev> fits;
    std::vector<TileDev> tiles;
    std::vector<SplitDev> splits;
    std::vector<CountFitDev> cfits;
    for (int i = 0; i < n_models; i++) {
        mc_model* m = models[i];
        // fits[] keeps one entry per model, so a tile's fit index is the model's.
        fits.push_back(m->make_desc());
        if (on_counts(m)) {
            CountFitDev c{};
            c.fit = m->d_fit;
            c.off = m->d_coff;
            c.ent = m->d_cent;
            c.n_qd = m->n_qd;
            c.blk_begin = b->count_blocks;
            c.n_blocks = (int)((m->n_qd + kCountChunk - 1) / kCountChunk);
            if (c.n_blocks == 0) continue;
            b->count_blocks += c.n_blocks;
            cfits.push_back(c);
            continue;
        }
        if (m->model != b->kernel_model) b->kernel_model = -1;
        if (int rc = m->ensure_tiles()) { delete b; return rc; }
        fits.back() = m->make_desc();
        std::vector<TileDev> t((size_t)m->n_tiles);
        std::vector<SplitDev> sp((size_t)m->n_splits);
        cudaError_t e = cudaSuccess;
        if (!t.empty()) e = cudaMemcpy(t.data(), m->d_tiles, t.size() * sizeof(TileDev), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && !sp.empty()) e = cudaMemcpy(sp.data(), m->d_splits, sp.size() * sizeof(SplitDev), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { delete b; return cuda_fail("batch_create", e); }
        int split_off = (int)splits.size();
        for (TileDev& x : t) {
            x.fit = i;
            if (x.split >= 0) x.split += split_off;
            tiles.push_back(x);
        }
        splits.insert(splits.end(), sp.begin(), sp.end());
    }
    b->n_tiles = (int)tiles.size();
    b->n_cfits = (int)cfits.size();
    int rc;
    if ((rc = dalloc(&b->d_fits, fits.size(), &b->bytes)) || (rc = dalloc(&b->d_tiles, tiles.size(), &b->bytes)) ||
        (rc = dalloc(&b->d_splits, splits.size(), &b->bytes)) || (rc = dalloc(&b->d_ws, 1, &b->bytes)) ||
        (rc = dalloc(&b->d_cfits, cfits.size(), &b->bytes))) {
        b->release();
        delete b;
        return rc;
    }
    cudaError_t e = cudaMemcpy(b->d_fits, fits.data(), fits.size() * sizeof(FitDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !cfits.empty())
        e = cudaMemcpy(b->d_cfits, cfits.data(), cfits.size() * sizeof(CountFitDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !tiles.empty()) e = cudaMemcpy(b->d_tiles, tiles.data(), tiles.size() * sizeof(TileDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !splits.empty()) e = cudaMemcpy(b->d_splits, splits.data(), splits.size() * sizeof(SplitDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->d_ws, 0, sizeof(WorkState));
    if (e != cudaSuccess) { b->release(); delete b; return cuda_fail("batch_create", e); }
    if (b->n_tiles == 0) {  // count-path fits only
        *out = b;
        return MC_OK;
    }
    // Shared memory and occupancy of the common launch.
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
    int best = -1;
    size_t best_smem = 0;
    for (int ns_ = 2; ns_ <= FUSED_MAX_STAGES && e == cudaSuccess; ns_++) {
        size_t sm_ = fused_smem_bytes(b->kernel_model, b->wqd, b->spt, ns_, b->n_cfits > 0);
        if (sm_ + 4096 > (size_t)optin) break;
        if ((e = fused_set_smem_limits(sm_)) != cudaSuccess) break;
        int per_sm = 0;
        if ((e = fused_occupancy(b->kernel_model, b->block, sm_, &per_sm)) != cudaSuccess) break;
        int score = per_sm * 16 + ns_;
        if (per_sm >= 1 && score > best) { best = score; b->stages = ns_; best_smem = sm_; b->grid = per_sm; }
    }
    if (e == cudaSuccess && best >= 0) e = fused_set_smem_limits((size_t)optin - 4096);
    (void)best_smem;
    if (e != cudaSuccess || best < 0) {
        b->release();
        delete b;
        return e != cudaSuccess ? cuda_fail("batch_create", e) : set_error(MC_ERR_INVALID, "batch_create: tile shape does not fit");
    }
    b->grid_cap = b->grid * b->n_sm;
    *out = b;
    return MC_OK;
}

extern "C" int mc_batch_em(mc_batch* b, int32_t iters, void* stream) {
    if (!b) return set_error(MC_ERR_INVALID, "batch_em: null batch");
    if (iters < 0) return set_error(MC_ERR_INVALID, "batch_em: negative iteration count");
    CK(cudaSetDevice(b->device));
    cudaStream_t st = (cudaStream_t)stream;
    if (!st) {
        if (!b->own_stream) CK(cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking));
        st = b->own_stream;
    }
    if (iters == 0 || (b->n_tiles == 0 && b->n_cfits == 0)) return MC_OK;
    const int full = iters / kGraphChunk, rem = iters % kGraphChunk;
    for (int pass = 0; pass < 2; pass++) {
        int len = pass == 0 ? kGraphChunk : rem;
        int reps = pass == 0 ? full : (rem ? 1 : 0);
        if (!reps) continue;
        auto& slot = b->graphs[pass];
        if (!slot.exec || slot.iters != len) {
            if (slot.exec) cudaGraphExecDestroy(slot.exec);
            slot.exec = nullptr;
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int rc = batch_launch_loop(b, len, st);
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (rc) { if (g) cudaGraphDestroy(g); return rc; }
            if (e != cudaSuccess) return cuda_fail("cudaStreamEndCapture", e);
            e = cudaGraphInstantiate(&slot.exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { slot.exec = nullptr; return cuda_fail("cudaGraphInstantiate", e); }
            slot.iters = len;
        }
        for (int k = 0; k < reps; k++) CK(cudaGraphLaunch(slot.exec, st));
    }
    if (!stream) CK(cudaStreamSynchronize(st));
    return MC_OK;
}

extern "C" int mc_batch_info(const mc_batch* b, int32_t* n_models, int32_t* n_tiles, int32_t* mixed_models) {
    if (!b) return set_error(MC_ERR_INVALID, "batch_info: null batch");
    if (n_models) *n_models = (int32_t)b->models.size();
    if (n_tiles) *n_tiles = b->n_tiles;
    if (mixed_models) *mixed_models = b->kernel_model < 0;
    return MC_OK;
}

extern "C" int mc_batch_configure(mc_batch* b, int single_launch) {
    if (!b) return set_error(MC_ERR_INVALID, "batch_configure: null batch");
    if (b->single_launch != (single_launch != 0)) {
        b->single_launch = single_launch != 0;
        for (auto& g : b->graphs) {  // recaptured on the next mc_batch_em
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
            g.iters = -1;
        }
    }
    return MC_OK;
}

extern "C" int mc_batch_launches(const mc_batch* b, int32_t* launches_per_iteration) {
    if (!b || !launches_per_iteration) return set_error(MC_ERR_INVALID, "batch_launches: null argument");
    *launches_per_iteration = (b->n_tiles ? 1 : 0) + (b->n_cfits && !(b->single_launch && b->n_tiles) ? 1 : 0);
    return MC_OK;
}

extern "C" void mc_batch_destroy(mc_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    b->release();
    delete b;
}

// ---------------------------------------------------------------------------
// DBN log-likelihood and its adjoint (adjoint.cu)
// ---------------------------------------------------------------------------
static int adjoint_common(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha, const float* beta,
                          const float* gamma, const char* who) {
    if (!m) return set_error(MC_ERR_INVALID, std::string(who) + ": null model");
    if (!m->uploaded) return set_error(MC_ERR_STATE, std::string(who) + ": no training sessions uploaded");
    if (s_begin < 0 || s_count < 0 || s_begin + s_count > m->n)
        return set_error(MC_ERR_INVALID, std::string(who) + ": session range outside the training set");
    if (s_count > 0 && (!alpha || !beta || !gamma)) return set_error(MC_ERR_INVALID, std::string(who) + ": null parameter");
    CK(cudaSetDevice(m->device));
    if (!m->d_grad) {
        int64_t before = m->bytes;
        int rc = dalloc(&m->d_grad, (size_t)(2 * m->qd_alloc() + 2), &m->bytes);
        if (rc) return rc;
        (void)before;
    }
    return MC_OK;
}

static AdjointArgs adjoint_args(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha, const float* beta,
                                const float* gamma, double scale) {
    AdjointArgs A;
    A.begin = s_begin;
    A.count = s_count;
    A.stride = m->stride;
    A.pidx = m->d_pidx;
    A.click = m->d_click;
    A.alpha = alpha;
    A.beta = beta;
    A.gamma = gamma;
    A.cnt = m->d_cnt;
    A.tcnt = nullptr;
    A.tcnt_off = nullptr;
    A.f_alpha = nullptr;
    A.f_beta = nullptr;
    A.ptiles = nullptr;
    A.pblk = nullptr;
    A.scale = scale;
    A.g_alpha = m->d_grad;
    A.g_beta = m->d_grad + m->qd_alloc();
    A.g_gamma = m->d_grad + 2 * m->qd_alloc();
    A.ll_out = m->d_grad + 2 * m->qd_alloc() + 1;
    return A;
}

// Sessions grouped by query with tiles built: the adjoint's tile path.
static bool adjoint_tile_path(const mc_model* m) {
    return m->fused_ok && m->tiles_ready && !m->h_tile_begin.empty();
}

// The FP32 gradient's per-tile counts (adjoint_counts_kernel), built once per
// tile layout on the first call that takes the tile path.
static int ensure_adjoint_counts(mc_model* m, cudaStream_t st) {
    if (!adjoint_tile_path(m) || m->adj_entries == 0 || m->d_adj_cnt) return MC_OK;
    // The packed copy: the model's tile descriptors with every session of a
    // staged tile kept (s_packed = s_count) and their own block offsets.
    std::vector<TileDev> at((size_t)m->n_tiles);
    CK(cudaMemcpy(at.data(), m->d_tiles, at.size() * sizeof(TileDev), cudaMemcpyDeviceToHost));
    int64_t blk = 0;
    int max_sessions = 1;
    for (TileDev& t : at) {
        t.blk_off = blk;
        if (t.qd_count <= m->wqd) {
            t.s_packed = t.s_count;
            blk += 22 * (int64_t)((t.s_count + 7) & ~7);
            max_sessions = std::max(max_sessions, t.s_count);
        }
    }
    const int64_t before = m->bytes;
    int rc = dalloc(&m->d_adj_off, m->h_adj_off.size(), &m->bytes);
    if (!rc) rc = dalloc(&m->d_adj_cnt, (size_t)m->adj_entries, &m->bytes);
    if (!rc) rc = dalloc(&m->d_adj_tiles, at.size(), &m->bytes);
    if (!rc) rc = dalloc(&m->d_adj_blk, (size_t)std::max<int64_t>(blk, 16), &m->bytes);
    if (rc) {
        dfree(m->d_adj_off);
        dfree(m->d_adj_cnt);
        dfree(m->d_adj_tiles);
        dfree(m->d_adj_blk);
        m->bytes = before;
        return rc;
    }
    m->adj_bytes = m->bytes - before;
    CK(cudaMemcpyAsync(m->d_adj_off, m->h_adj_off.data(), m->h_adj_off.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                       st));
    CK(cudaMemcpyAsync(m->d_adj_tiles, at.data(), at.size() * sizeof(TileDev), cudaMemcpyHostToDevice, st));
    CK(launch_adjoint_counts(m->d_tiles, m->n_tiles, m->wqd, m->d_pidx, m->d_click, m->stride, m->d_adj_off,
                             m->d_adj_cnt, m->n_sm, st));
    CK(launch_pack_tiles(MC_PBM, m->d_adj_tiles, m->n_tiles, m->wqd, max_sessions, m->d_pidx, m->stride, m->d_click,
                         m->d_adj_blk, m->d_status, m->n_sm, st));
    CK(cudaStreamSynchronize(st));  // the host arrays stay alive meanwhile
    return check_status(m, st);
}

// Gradient outputs.  The FP32 tile path writes the alpha and beta gradients
// straight into the caller's FP32 arrays (cleared here); the FP64 and
// per-session paths accumulate in the model's FP64 arrays, converted after.
// The gamma gradient and the log-likelihood are FP64 in both.
static int adjoint_outputs(mc_model* m, AdjointArgs& A, bool fp64, float* d_alpha, float* d_beta, cudaStream_t st) {
    if (!fp64 && adjoint_tile_path(m)) {
        int rc = ensure_adjoint_counts(m, st);
        if (rc) return rc;
        CK(cudaMemsetAsync(d_alpha, 0, (size_t)m->n_qd * 4, st));
        CK(cudaMemsetAsync(d_beta, 0, (size_t)m->n_qd * 4, st));
        CK(cudaMemsetAsync(A.g_gamma, 0, 2 * 8, st));  // g_gamma, ll_out
        A.f_alpha = d_alpha;
        A.f_beta = d_beta;
        return MC_OK;
    }
    CK(cudaMemsetAsync(m->d_grad, 0, (size_t)(2 * m->qd_alloc() + 2) * 8, st));
    return MC_OK;
}

static cudaError_t adjoint_finish(mc_model* m, const AdjointArgs& A, float* d_alpha, float* d_beta, float* d_gamma,
                                  cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    if (!A.f_alpha) {
        e = launch_grad_to_float(A.g_alpha, d_alpha, m->n_qd, m->n_sm, st);
        if (e == cudaSuccess) e = launch_grad_to_float(A.g_beta, d_beta, m->n_qd, m->n_sm, st);
    }
    if (e == cudaSuccess) e = launch_grad_to_float(A.g_gamma, d_gamma, 1, m->n_sm, st);
    return e;
}

// Through the tiles when the sessions are grouped by query (tiles built),
// else one thread per session with global atomics.
static cudaError_t run_adjoint(mc_model* m, const AdjointArgs& A0, bool grad, bool fp64, cudaStream_t st) {
    AdjointArgs A = A0;
    if (adjoint_tile_path(m)) {
        if (grad && !fp64 && m->d_adj_cnt) {
            A.tcnt = m->d_adj_cnt;
            A.tcnt_off = m->d_adj_off;
            A.ptiles = m->d_adj_tiles;
            A.pblk = m->d_adj_blk;
        }
        const auto& tb = m->h_tile_begin;
        // tiles [t0, t1) intersect [begin, begin + count): tile starts ascend
        int t0 = (int)(std::upper_bound(tb.begin(), tb.end(), A.begin) - tb.begin()) - 1;
        if (t0 < 0) t0 = 0;
        const int t1 = (int)(std::lower_bound(tb.begin(), tb.end(), A.begin + A.count) - tb.begin());
        return launch_adjoint_tiles(A, m->d_tiles, t0, t1, m->wqd, grad, fp64, m->n_sm, st);
    }
    return launch_adjoint(A, grad, fp64, m->n_sm, st);
}

extern "C" int mc_dbn_loglik_forward(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha,
                                     const float* beta, const float* gamma, int fp64, double* loglik, void* stream) {
    int rc = adjoint_common(m, s_begin, s_count, alpha, beta, gamma, "dbn_loglik_forward");
    if (rc) return rc;
    if (!loglik) return set_error(MC_ERR_INVALID, "dbn_loglik_forward: null output");
    cudaStream_t st = m->pick(stream);
    AdjointArgs A = adjoint_args(m, s_begin, s_count, alpha, beta, gamma, 0.0);
    CK(cudaMemsetAsync(A.ll_out, 0, 8, st));
    CK(run_adjoint(m, A, false, fp64 != 0, st));
    CK(cudaMemcpyAsync(loglik, A.ll_out, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return MC_OK;
}

extern "C" int mc_dbn_loglik_backward(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha,
                                      const float* beta, const float* gamma, int fp64, double grad_output,
                                      float* d_alpha, float* d_beta, float* d_gamma, double* loglik, void* stream) {
    int rc = adjoint_common(m, s_begin, s_count, alpha, beta, gamma, "dbn_loglik_backward");
    if (rc) return rc;
    if (!d_alpha || !d_beta || !d_gamma) return set_error(MC_ERR_INVALID, "dbn_loglik_backward: null gradient output");
    cudaStream_t st = m->pick(stream);
    AdjointArgs A = adjoint_args(m, s_begin, s_count, alpha, beta, gamma, grad_output);
    if ((rc = adjoint_outputs(m, A, fp64 != 0, d_alpha, d_beta, st))) return rc;
    CK(run_adjoint(m, A, true, fp64 != 0, st));
    CK(adjoint_finish(m, A, d_alpha, d_beta, d_gamma, st));
    if (loglik) {
        CK(cudaMemcpyAsync(loglik, A.ll_out, 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    } else if (!stream) {
        CK(cudaStreamSynchronize(st));
    }
    return MC_OK;
}

extern "C" int mc_dbn_loglik_grad(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha, const float* beta,
                                  const float* gamma, int fp64, float* d_alpha, float* d_beta, float* d_gamma,
                                  double* d_loglik, void* stream) {
    int rc = adjoint_common(m, s_begin, s_count, alpha, beta, gamma, "dbn_loglik_grad");
    if (rc) return rc;
    if (!d_alpha || !d_beta || !d_gamma || !d_loglik) return set_error(MC_ERR_INVALID, "dbn_loglik_grad: null output");
    cudaStream_t st = m->pick(stream);
    AdjointArgs A = adjoint_args(m, s_begin, s_count, alpha, beta, gamma, 1.0);
    if ((rc = adjoint_outputs(m, A, fp64 != 0, d_alpha, d_beta, st))) return rc;
    CK(run_adjoint(m, A, true, fp64 != 0, st));
    CK(adjoint_finish(m, A, d_alpha, d_beta, d_gamma, st));
    CK(cudaMemcpyAsync(d_loglik, A.ll_out, 8, cudaMemcpyDeviceToDevice, st));
    if (!stream) CK(cudaStreamSynchronize(st));
    return MC_OK;
}
