// Device-side data layout shared by the fused kernel, the plain kernels and
// the evaluation kernels.
//
// Training sessions are sorted by query (as ingest leaves them).  Because
// query-document (qd) indices are assigned in order of first appearance over
// that order (data/dataset.cpp:314-339), the qd indices of one query form a
// contiguous range, and consecutive queries own consecutive ranges.  A tile of
// whole queries therefore owns a contiguous qd window that no other tile reads:
// the fused kernel privatises that window's statistics in shared memory and
// runs the M-step for it in place, with no global reduction.  A query too large
// for one tile is split into several tiles whose statistics meet in FP64 global
// bins; the last of them to finish runs that query's M-step.
#ifndef MCLICKS_COMMON_CUH
#define MCLICKS_COMMON_CUH

#include <cstdint>

#define MC_R 10
#define MC_UBM_SLOTS 55
#define MC_MAX_PUB 128         // >= 2 * public parameters of any model (UBM: 55 slots)

// Fused kernel: at most this many threads per CTA (every warp takes work
// items; thread 0 also fills the copy ring), CTAs per SM it is compiled for,
// and at most this many shared-memory stages in its copy ring.
#define FUSED_THREADS 256
#define FUSED_MIN_CTAS 2
#define FUSED_MAX_STAGES 4

// Param::value() clamp (click_models/param.cu:116-128).
#define MC_TOP (1.0f - 0.000001f)

namespace mcd {

enum { PBM = 0, CCM = 1, DBN = 2, UBM = 3 };
enum { PARITY = 0, CLEAN = 1 };

// Private statistics privatised per qd: DBN keeps attractiveness and
// satisfaction, the others attractiveness only.
__host__ __device__ inline int private_stats(int model) { return model == DBN ? 2 : 1; }
// Public parameters of each model (parameter arrays of click_models/*.cuh).
__host__ __device__ inline int public_params(int model) {
    return model == PBM ? MC_R : model == UBM ? MC_UBM_SLOTS : model == DBN ? 1 : 3;
}

struct FitDev {
    int model, mode;
    int64_t n;             // training sessions
    int64_t stride;        // plane stride of pidx (>= n, multiple of 32)
    int64_t n_qd;
    int n_tiles;
    int n_pub;
    const int32_t* pidx;   // [10][stride], rank-major planes
    const uint16_t* click; // [n] bit masks
    const uint2* cnt;      // [n_qd] {occurrences, clicked occurrences}
    const uint32_t* cnt16; // [n_qd] occurrences | clicked << 16, each saturated at
                           // 65535 (exact for qd of whole-query tiles: <= 10 * 4096)
    const unsigned char* tblk;  // packed tile blocks (uint16 window-relative indices + clicks)
    float* atr;            // [n_qd] current values
    float* sat;            // [n_qd] current values (DBN)
    float* pub_theta;      // [2][MC_MAX_PUB], buffer (iter & 1) is current
    double* pub_bins;      // [2 * n_pub] FP64 statistic bins (num, den interleaved)
    const double* pub_const;  // [2 * n_pub] constant (prior + click-count) parts
    double* split_bins;    // FP64 bins of split queries
    unsigned* split_count; // tiles finished per split query
    unsigned* tiles_done;  // tiles finished this iteration
    int* iter;             // iterations completed
    int* status;           // error word (0 = ok)
};

struct TileDev {
    int fit;
    int split;          // -1, or index into the split table
    int64_t s_begin;    // first session
    int s_count;        // sessions
    int qd_count;       // window size
    int64_t qd_begin;   // window start
    int64_t blk_off;    // byte offset of the tile's packed block in FitDev::tblk
    int s_packed;       // sessions in the packed block (see pack_tiles_kernel)
    int max_occ;        // largest number of packed (session, rank) entries showing one
                        // window pair; sets the fixed-point scale of the tile's bins
};

struct SplitDev {
    int64_t qd_begin;
    int qd_count;
    int n_tiles;
    int64_t bin_offset; // into the fit's split_bins, in doubles
    int local;          // index of this split query's counter in the fit's split_count
    int pad_;
};

struct WorkState {
    unsigned next_tile;
    unsigned ctas_exited;
    unsigned next_count;   // count chunks of batched count-path fits taken so far
    unsigned pad_;
};

// Counters of the upload pass beyond the UBM slot counts.
#define MC_PUB_COUNTS 128
#define MC_CNT_DBN_BEFORE_LAST 120   // DBN: sum over sessions of the last-click rank (10 if none)
#define MC_CNT_CCM_UNCLICKED_BEFORE_LAST 121  // CCM: unclicked ranks before the last click (10 if none)

// Status bits.
enum { ST_BAD_INDEX = 1, ST_TIMEOUT = 2 };

__device__ __forceinline__ float clamp_top(float v) { return v < MC_TOP ? v : MC_TOP; }

}  // namespace mcd

#endif  // MCLICKS_COMMON_CUH
