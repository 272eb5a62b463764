// Launch entry points of the kernels, used by the host orchestration in model.cu.
#ifndef MCLICKS_KERNELS_H
#define MCLICKS_KERNELS_H

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace mcd {

// ---- fused EM (em_fused.cu) -------------------------------------------------
struct CountFitDev;
// Dynamic shared memory of the tile kernel; with_counts: enough for the count
// chunks of batched count-path fits as well.
size_t fused_smem_bytes(int model, int window_max, int spt, int n_stages, bool with_counts = false);
cudaError_t fused_set_smem_limits(size_t bytes);
cudaError_t fused_occupancy(int model, int block, size_t smem, int* blocks_per_sm);
// Wait limit of the fused kernel's mbarrier waits and a tile whose stage is
// made to stall (-1: none), on the current device; for the timeout tests.
cudaError_t set_wait_hooks(unsigned long long wait_limit_ns, int stall_tile);
// cfits / n_cfits / count_blocks: count-path fits of a batch whose chunks the
// same launch takes after the tiles (nullptr, 0, 0 for none).
cudaError_t launch_em_fused(int model, const FitDev* fits, const TileDev* tiles, int n_tiles, const SplitDev* splits,
                            WorkState* ws, int window_max, int spt, int n_stages, int grid, int block,
                            const CountFitDev* cfits, int n_cfits, int count_blocks, cudaStream_t stream);
// PBM/UBM iterations from counts per (qd, statistic key) (em_counts.cu).
// build_counts sorts the unclicked occurrences of the uploaded sessions into
// per-qd entries (CSR: off[n_qd + 1], ent[n_entries]); *usable = 0 keeps the
// tile path (sizes beyond the entry format).
// For PBM, *dense (if dense is not null) also receives uint16 [n_qd][10]
// counts by rank, or nullptr when a count exceeds 16 bits.
cudaError_t build_counts(int model, int64_t n, int64_t stride, int64_t n_qd, const int32_t* planes, const uint16_t* click,
                         int n_sm, cudaStream_t st, uint32_t** off, uint32_t** ent, int64_t* n_entries,
                         uint16_t** dense, int* usable);
// Launch shape of the one-fit count kernels: copies of each warp's public
// bins (4, 8 or 16; the entry kernel), threads per block (64..256, a multiple
// of 32) and the most blocks per SM of the grid-stride grid.
struct CountShape {
    int copies, block, blocks_per_sm;
};
bool count_shape_valid(const CountShape& c, bool dense);
cudaError_t launch_em_counts_pbm_dense(const FitDev* fit, const uint16_t* dense, int64_t n_qd, int n_sm,
                                       const CountShape& c, cudaStream_t st);
cudaError_t launch_em_counts(const FitDev* fit, const uint32_t* off, const uint32_t* ent, int64_t n_qd, int n_sm,
                             const CountShape& c, cudaStream_t st);
// Batched count path: fit i takes blocks [blk_begin, blk_begin + n_blocks),
// one chunk of kCountChunk qd each (n_blocks = ceil(n_qd / kCountChunk)).
constexpr int kCountChunk = 2048;
struct CountFitDev {
    const FitDev* fit;
    const uint32_t* off;
    const uint32_t* ent;
    int64_t n_qd;
    int blk_begin, n_blocks;
};
cudaError_t launch_em_counts_batch(const CountFitDev* fits, int n_fits, int total_blocks, cudaStream_t st);
cudaError_t launch_pack_tiles(int model, TileDev* tiles, int n_tiles, int window_max, int max_tile_sessions, const int32_t* planes,
                              int64_t stride, const uint16_t* click, unsigned char* tblk, int* status, int n_sm,
                              cudaStream_t st);

// ---- plain EM (em_plain.cu) -------------------------------------------------
// The reference's 8-byte device record (data/search.cuh:63-73).
struct PlainRec {
    signed char click;
    int pidx;
};

struct PlainArgs {
    int64_t n, n_qd;
    const PlainRec* recs;  // [10][n]
    float2* atr2;          // [n_qd] (num, den)
    float2* sat2;          // [n_qd] (DBN)
    float2* pub2;          // [n_pub]
    float2* tmp_atr;       // [10][n]
    float2* tmp_sat;       // [10][n] (DBN)
    float2* tmp_pub;       // [n_pub][n]
};

cudaError_t launch_plain_estep(int model, const PlainArgs& A, cudaStream_t st);
cudaError_t launch_plain_reset(const PlainArgs& A, int n_pub, cudaStream_t st);
cudaError_t launch_plain_update(int model, const PlainArgs& A, cudaStream_t st);
cudaError_t launch_values_to_pairs(const float* v, float2* pairs, int64_t n, cudaStream_t st);
cudaError_t launch_pairs_to_values(const float2* pairs, float* v, int64_t n, cudaStream_t st);
cudaError_t launch_fill2(float2* p, int64_t n, float a, float b, cudaStream_t st);
cudaError_t launch_fill_value(float* p, int64_t n, float v, cudaStream_t st);

// ---- evaluation (eval.cu) ---------------------------------------------------
struct EvalArgs {
    int model;
    int64_t n, stride, n_qd;
    const int32_t* pidx;    // [10][stride]
    const uint16_t* click;  // [n]
    const float* atr;
    const float* sat;
    const float* pub;       // current public values
    double* out;            // [11]: log-likelihood sum, then log2 sums per rank
    // Optional: with iter set, pub is the [2][MC_MAX_PUB] double buffer and
    // the half (*iter & 1) read on the device is the current one.
    const int* iter = nullptr;
};

cudaError_t launch_eval(const EvalArgs& A, int n_sm, cudaStream_t st);

// ---- DBN log-likelihood adjoint (adjoint.cu) ---------------------------------
struct AdjointArgs {
    int64_t begin, count, stride;
    const int32_t* pidx;     // [10][stride]
    const uint16_t* click;
    const float* alpha;      // logits [n_qd]
    const float* beta;       // logits [n_qd]
    const float* gamma;      // logit [1]
    const uint2* cnt;        // [n_qd] occurrences (x) of each pair in the training set
    // Per staged tile t (tcnt_off[t] >= 0), per window entry i, at
    // tcnt[tcnt_off[t] + i]: the counts over all of the tile's sessions of
    // occurrences, occurrences at or before the session's last click, clicks
    // and last clicks (adjoint_counts_kernel); null when not built.
    const uint4* tcnt;
    const int64_t* tcnt_off;
    // Every session of each staged tile packed in click-mask order (the
    // packing kernel's layout: uint16 [10][spad] window indices, uint16
    // [spad] clicks at ptiles[t].blk_off), read for whole tiles; null when
    // not built.
    const TileDev* ptiles;
    const unsigned char* pblk;
    double scale;            // gradient scale (the caller's grad_output)
    double* g_alpha;         // FP64 gradient accumulators
    double* g_beta;
    // FP32 tile path: the alpha and beta gradients written straight into these
    // (cleared by the caller) instead of g_alpha, g_beta; null otherwise.
    float* f_alpha;
    float* f_beta;
    double* g_gamma;
    double* ll_out;          // log-likelihood sum
};

cudaError_t launch_adjoint(const AdjointArgs& A, bool grad, bool fp64, int n_sm, cudaStream_t st);
// Tiles [t0, t1) of a model whose sessions are grouped by query; sessions
// outside [A.begin, A.begin + A.count) are skipped.
cudaError_t launch_adjoint_tiles(const AdjointArgs& A, const TileDev* tiles, int t0, int t1, int window_max, bool grad,
                                 bool fp64, int n_sm, cudaStream_t st);
cudaError_t launch_grad_to_float(const double* src, float* dst, int64_t n, int n_sm, cudaStream_t st);
// The parameter-independent per-tile counts of AdjointArgs::tcnt for tiles
// [0, n_tiles) (tiles with off[t] < 0 are skipped).
cudaError_t launch_adjoint_counts(const TileDev* tiles, int n_tiles, int window_max, const int32_t* pidx,
                                  const uint16_t* click, int64_t stride, const int64_t* off, uint4* out, int n_sm,
                                  cudaStream_t st);

}  // namespace mcd

#endif  // MCLICKS_KERNELS_H
