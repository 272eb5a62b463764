/* mclicks.h — C-ABI of the GB300 EM trainer for click models.
 *
 * This is the boundary below the reference's host C++ API (ClickModel_Hst,
 * em_parallel, the mclicks CLI).  Every entry point takes plain pointers and
 * sizes, returns an int status (MC_OK = 0) and leaves a message for
 * mc_last_error() on failure; the reference instead printed and aborted
 * (utils/utils.cuh:27-42, parallel_em/communicator.cpp:119-133).
 *
 * Each declaration names the reference interface it replaces (file:line
 * within the reference project).  Streams are passed as `void*` holding a
 * cudaStream_t (NULL = the legacy default stream); no call is re-entrant on
 * one handle.
 */
#ifndef MCLICKS_H
#define MCLICKS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MC_MAX_SERP 10           /* utils/definitions.h:50 */

/* Model ids of --model-type (main.cpp:178-183). */
enum { MC_PBM = 0, MC_CCM = 1, MC_DBN = 2, MC_UBM = 3 };

/* Statistics mode.  PARITY reproduces the reference's CPU path, where a
 * per-session statistic slot the E-step never writes keeps the default
 * Param (1,2) (click_models/param.cuh:23-24, common.cu:57) and is summed
 * every iteration (UBM examination slots, ubm.cu:222 with common.cu:161-163;
 * DBN satisfaction of unclicked ranks, dbn.cu:358-376).  CLEAN sums only the
 * slots that were written. */
enum { MC_MODE_PARITY = 0, MC_MODE_CLEAN = 1 };

/* EM implementation: one fused persistent kernel per iteration, or the plain
 * two-kernel E-step + scatter of the reference's GPU path
 * (parallel_em/kernel.cu:42-89) with the same statistics semantics. */
enum { MC_IMPL_FUSED = 0, MC_IMPL_PLAIN = 1 };

/* Status codes. */
enum {
    MC_OK = 0,
    MC_ERR_INVALID = 1,   /* bad argument */
    MC_ERR_IO = 2,        /* file could not be read or written */
    MC_ERR_CUDA = 3,      /* a CUDA call failed */
    MC_ERR_NOMEM = 4,     /* host or device allocation failed */
    MC_ERR_STATE = 5,     /* call out of order (e.g. EM before upload) */
    MC_ERR_DEVICE = 6     /* a kernel reported an error through its status word */
};

/* Copies the last error message of the calling thread into buf (always
 * NUL-terminated); returns the last status code. */
int mc_last_error(char* buf, size_t len);

/* Library version string. */
const char* mc_version(void);

/* ---------------------------------------------------------------------------
 * Synthetic click logs (test and benchmark inputs).
 * ------------------------------------------------------------------------- */
typedef struct mc_synth_config {
    int64_t n_sessions;      /* sessions to generate */
    int32_t n_queries;       /* query ids are Zipf(zipf_s) over [0, n_queries) */
    int32_t pool;            /* candidate docs per query (10..256) */
    double zipf_s;
    int32_t click_model;     /* ground truth: 0 PBM, 1 CCM, 2 DBN */
    int32_t reserved;
    double atr_beta_b;       /* attractiveness / relevance ~ Beta(1, b) */
    double sat_beta_b;       /* DBN satisfaction ~ Beta(1, b) */
    double gamma;            /* DBN continuation */
    double tau1, tau2, tau3; /* CCM continuation */
    double pbm_exam_scale;   /* PBM examination gamma_r = scale / sqrt(r + 1) */
    uint64_t seed;
} mc_synth_config;

/* Fills c with one of three presets: 0 = 40k sessions / 1k queries Zipf 1.1 /
 * 20-doc pools / PBM clicks; 1 = 2M / 100k / Zipf 1.0 / 30 / DBN clicks;
 * 2 = 20M / 1M / Zipf 1.0 / 50 / CCM clicks. */
void mc_synth_config_default(mc_synth_config* c, int preset);

/* Sessions [first, first + count) in arrival order: query[count],
 * docs[count * 10] (session-major), click_mask[count] (bit r = rank r). */
int mc_synth_generate(const mc_synth_config* cfg, int64_t first, int64_t count,
                      int32_t* query, int32_t* docs, uint16_t* click_mask);

/* Writes n_sessions + 1 sessions in the reference's text log format
 * (README.md:39-52); the reader keeps n_sessions of them (dataset.cpp:240-242). */
int mc_synth_write_log(const mc_synth_config* cfg, const char* path);

/* ---------------------------------------------------------------------------
 * Dataset ingest (host).  Replaces Dataset::parse_dataset
 * (data/dataset.cpp:421-455) for one worker: parse (dataset.cpp:224-305),
 * tail test split (dataset.cpp:385-397), unstable std::sort of the training
 * sessions by query (dataset.cpp:17-43), query-document indices in order of
 * first appearance (dataset.cpp:314-339), test filtering
 * (dataset.cpp:349-374).  Bit-exact with the reference.
 * ------------------------------------------------------------------------- */
typedef struct mc_dataset mc_dataset;

int mc_dataset_parse(const char* path, int32_t max_sessions, float test_share, mc_dataset** out);

/* How mc_dataset_parse reads a log (process-wide; no counterpart in the
 * reference, which reads line by line with std::getline, dataset.cpp:224-305):
 * block_bytes per read (default 64 MB) and the number of runs of lines each
 * block is cut into and parsed in parallel (default one per hardware thread).
 * 0 restores a default.  The output does not depend on either: small values
 * make short logs cross many block and run boundaries, as a large log does. */
int mc_ingest_configure(int64_t block_bytes, int32_t runs);

/* Same split/sort/index steps on sessions already in memory, in arrival
 * order (as the parser would have produced them). */
int mc_dataset_from_sessions(int64_t n, const int32_t* query, const int32_t* docs,
                             const uint16_t* click_mask, float test_share, mc_dataset** out);

int mc_dataset_info(const mc_dataset* d, int64_t* n_train, int64_t* n_test, int64_t* n_qd);

/* Copies one set out (which = 0 train, 1 test).  docs and pidx are
 * session-major [n * 10]; pidx is -1 for a test doc unseen in training.
 * Any output pointer may be NULL. */
int mc_dataset_copy(const mc_dataset* d, int which, int32_t* query, int32_t* docs,
                    int32_t* pidx, uint16_t* click_mask);

void mc_dataset_free(mc_dataset* d);

/* ---------------------------------------------------------------------------
 * Click model on the GPU.
 * ------------------------------------------------------------------------- */
typedef struct mc_model mc_model;

/* Replaces create_cm_host / create_cm_dev (click_models/base.cu:19-88) and
 * Kernel::initialize (parallel_em/kernel.cu:24-33). */
int mc_model_create(int model_type, int mode, int device, mc_model** out);

/* Replaces convert_to_device (data/search.cu:342-356),
 * allocate_memory_on_device (parallel_em/parallel_em.cu:281-309) and
 * init_parameters (click_models/common.cu:31-61): uploads the training
 * sessions (sorted by query, as ingest leaves them; pidx session-major
 * [n * 10] in [0, n_qd)), builds the tile work queue and sets every
 * parameter to the prior value 1/2. */
int mc_model_upload(mc_model* m, int64_t n_train, const int32_t* query, const int32_t* pidx,
                    const uint16_t* click_mask, int64_t n_qd, void* stream);

/* Uploads the evaluation set (pidx may hold -1 for unseen docs). */
int mc_model_upload_test(mc_model* m, int64_t n_test, const int32_t* pidx,
                         const uint16_t* click_mask, void* stream);

/* Replaces the value initialisation of init_parameters
 * (click_models/common.cu:31-61): every parameter back to the prior 1/2 and
 * the iteration counter to 0, keeping the uploaded sessions. */
int mc_model_init_parameters(mc_model* m, void* stream);

/* Tile shape of the fused kernel: sessions per tile, query-document window
 * per tile (shared-memory privatisation width) and threads per block.
 * 0 keeps the current value.  Rebuilds the work queue. */
int mc_model_configure(mc_model* m, int32_t sessions_per_tile, int32_t window_qd, int32_t block_size);
int mc_model_get_config(const mc_model* m, int32_t* sessions_per_tile, int32_t* window_qd, int32_t* block_size);

/* Times a few fused iterations for each candidate shape and keeps the
 * fastest: the tile shape (sessions per tile, window, block) on the tile
 * path; on the count path (mc_model_fused_path: PBM, UBM) the count kernel's
 * bin copies, block size and blocks per SM.  Parameters are restored
 * afterwards.  (No counterpart in the reference, whose launches are fixed at
 * BLOCK_SIZE threads, utils/definitions.h.) */
int mc_model_autotune(mc_model* m, void* stream);

/* Launch shape of the count-path kernels (no counterpart in the reference):
 * copies of each warp's public bins (4, 8 or 16; ignored by the dense PBM
 * kernel), threads per block (a multiple of 32 in [64, 256]) and blocks per
 * SM of the grid.  Results do not depend on the shape. */
int mc_model_configure_counts(mc_model* m, int32_t copies, int32_t block, int32_t blocks_per_sm);
int mc_model_get_count_config(const mc_model* m, int32_t* copies, int32_t* block, int32_t* blocks_per_sm);

/* Runs n_iterations EM iterations: replaces the loop of em_parallel
 * (parallel_em/parallel_em.cu:462-609): Kernel::em_training, reset_parameters,
 * Kernel::update and the public-parameter sync.  The fused loop is captured
 * once as a CUDA graph and replayed.  Asynchronous on `stream`. */
int mc_model_em(mc_model* m, int32_t n_iterations, int impl, void* stream);

/* The two halves of one plain iteration, for callers that drive the
 * reference's process_session / update_parameters split
 * (click_models/base.cuh:41-42). */
int mc_model_process_sessions(mc_model* m, void* stream);
int mc_model_update_parameters(mc_model* m, void* stream);

/* Parameter arrays, in the order of ClickModel_Hst::get_parameters(ALL)
 * (pbm.cu:305-321, ccm.cu:531-533, dbn.cu:535-538, ubm.cu:299-315):
 *   PBM: examination[10], attractiveness[n_qd]
 *   UBM: examination[55], attractiveness[n_qd]
 *   DBN: attractiveness[n_qd], satisfaction[n_qd], continuation[1]
 *   CCM: attractiveness[n_qd], continuation[3]
 * is_public follows get_parameter_information (pbm.cu:120-132 etc.). */
int mc_model_param_count(const mc_model* m);
int mc_model_param_info(const mc_model* m, int index, char* name, size_t name_len,
                        int64_t* size, int* is_public);

/* Replaces transfer_parameters(D2H) + get_parameters (common.cu:93-102):
 * copies the current parameter values (FP32, = Param::value(), param.cu:116-128)
 * of array `index` to host memory.  Synchronous. */
int mc_model_get_param(mc_model* m, int index, float* values, void* stream);

/* Replaces set_parameters + transfer_parameters(H2D). */
int mc_model_set_param(mc_model* m, int index, const float* values, void* stream);

/* Replaces LogLikelihood::evaluate / Perplexity::evaluate
 * (click_models/evaluation.cpp:25-66) on the GPU for the training (which = 0)
 * or uploaded test (which = 1) set.  Outputs FP64 sums:
 *   *ll_sum = sum over sessions of (sum_r log p_r) / 10      (p_r conditional)
 *   log2_sums[r] = sum over sessions of log2 q_r             (q_r full)
 *   *n_sessions = sessions evaluated.
 * LL = ll_sum / n; perplexity at rank r = 2^(-log2_sums[r] / n)
 * (parallel_em/parallel_em.cu:697-723).  Synchronous. */
int mc_model_evaluate(mc_model* m, int which, double* ll_sum, double* log2_sums, int64_t* n_sessions,
                      void* stream);

/* Training log-likelihood per iteration: n_iterations fused iterations, each
 * followed on the device by the evaluation of the training sessions under the
 * parameters that iteration produced; train_ll[i] (host, n_iterations values)
 * receives ll_sum of mc_model_evaluate(which = 0) after iteration i + 1.  The
 * reference logs only the final test-set values (parallel_em.cu:634-723);
 * this traces convergence without a host round trip between iterations.
 * Allocates a device array of 88 * n_iterations bytes for the call.
 * Synchronous. */
int mc_model_em_trace(mc_model* m, int32_t n_iterations, double* train_ll, void* stream);

/* Which kernel one fused iteration of the uploaded model launches: *path = 0
 * the tile kernel over the sessions, 1 the count kernel over the per-(qd, key)
 * occurrence counts built at upload (UBM, and PBM when a count exceeds 16
 * bits), 2 the PBM kernel over dense uint16 [n_qd][10] counts by rank;
 * *n_entries = the number of (qd, key) count entries (0 on the tile path).  The reference has one E-step kernel per
 * model (pbm.cu:191-253, ubm.cu:185-247); this reports which equivalent runs. */
int mc_model_fused_path(const mc_model* m, int32_t* path, int64_t* n_entries);

/* Testing hook for the timeout path of the fused kernel (the reference stops
 * the job on an error, communicator.cpp:119-133; here every wait inside a
 * kernel is bounded and an expired wait surfaces as MC_ERR_DEVICE).  On
 * `device`, sets the limit of one mbarrier wait to wait_limit_ns (0 restores
 * the default of 4 s) and makes the stage fill of tile index stall_tile
 * declare 16 bytes more than it copies, so that the wait for that stage runs
 * out while every copy has landed (-1: no tile).  Affects every model on the
 * device until reset; calls that read results then return MC_ERR_DEVICE. */
int mc_test_wait_hooks(int device, int64_t wait_limit_ns, int32_t stall_tile);

/* Device memory held by the model, in bytes. */
int mc_model_memory(const mc_model* m, int64_t* bytes);

/* Device blocks the library freed are kept in a per-device cache and handed
 * out again (models created and destroyed with the same sizes then skip
 * cudaMalloc / cudaFree).  mc_empty_cache frees the cached blocks of one device
 * (-1: all, and also the page-locked host buffers kept for upload readbacks)
 * back to the driver; mc_cache_bytes reports how much device memory is
 * cached. */
int mc_empty_cache(int device, int64_t* bytes_released);
int mc_cache_bytes(int device, int64_t* bytes);

/* Replaces destroy_parameters (pbm.cu:445-460 etc.). */
void mc_model_destroy(mc_model* m);

/* ---------------------------------------------------------------------------
 * Batched fits: several independent fits (any mix of model types, e.g. one per
 * query partition) advanced together, one persistent launch per iteration over
 * the union of their tiles.  The reference runs one model per process
 * (parallel_em/parallel_em.cu:364-372); this replaces many such runs.
 * ------------------------------------------------------------------------- */
typedef struct mc_batch mc_batch;

/* The models must be uploaded and on one device.  Models on the tile path
 * (mc_model_fused_path = 0) share one persistent tile launch and are given the
 * first such model's tile shape; models on the count path (PBM, UBM) share
 * one batched count launch.  Models keep their own parameters and may still
 * be used alone; they must not be re-uploaded or reconfigured while the batch
 * exists. */
int mc_batch_create(int n_models, mc_model* const* models, mc_batch** out);

/* n_iterations fused iterations of every model, captured as CUDA graphs and
 * replayed.  NULL stream = internal stream, synchronous. */
int mc_batch_em(mc_batch* b, int32_t n_iterations, void* stream);

/* n_tiles: tiles of the tile launch; mixed_models: its tile fits are of more
 * than one model type (the model-generic kernel runs). */
int mc_batch_info(const mc_batch* b, int32_t* n_models, int32_t* n_tiles, int32_t* mixed_models);

/* How a batch with both kinds of fit runs an iteration (no counterpart in the
 * reference, which runs one model per process, parallel_em.cu:364-372):
 * single_launch = 1 makes the persistent tile launch take the count chunks of
 * the count-path fits (PBM, UBM) after its tiles, one launch per iteration;
 * 0 (the default) follows the tile launch with a count launch.  The default
 * is the faster on the 256-fit benchmark (0.34 against 0.40 ms per
 * iteration): the count kernel runs three times the warps per SM that the
 * tile kernel's two CTAs hold.  Results are the same either way. */
int mc_batch_configure(mc_batch* b, int single_launch);

/* Kernel launches one iteration of the batch makes (0, 1 or 2). */
int mc_batch_launches(const mc_batch* b, int32_t* launches_per_iteration);

void mc_batch_destroy(mc_batch* b);

/* ---------------------------------------------------------------------------
 * DBN log-likelihood as a function of logit parameters, and its gradient: a
 * forward/backward pair shaped like an autograd function.  The likelihood is
 * the reference's conditional DBN click probability (click_models/dbn.cu:611-639)
 * summed over training sessions [s_begin, s_begin + s_count) of the model's
 * uploaded set, with attractiveness a = sigmoid(alpha[qd]), satisfaction
 * s = sigmoid(beta[qd]) and continuation g = sigmoid(gamma[0]).  alpha and beta
 * ([n_qd]) and gamma ([1]) are device arrays.  fp64 = 1 evaluates in double
 * precision (for verification), 0 in single; sums are FP64 either way.
 * ------------------------------------------------------------------------- */
int mc_dbn_loglik_forward(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha, const float* beta,
                          const float* gamma, int fp64, double* loglik, void* stream);

/* Writes grad_output * d(log-likelihood)/d(alpha, beta, gamma) to the device
 * arrays d_alpha, d_beta ([n_qd]) and d_gamma ([1]), overwriting them; the
 * forward messages are recomputed, not stored.  *loglik (optional) receives
 * the log-likelihood. */
int mc_dbn_loglik_backward(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha, const float* beta,
                           const float* gamma, int fp64, double grad_output, float* d_alpha, float* d_beta,
                           float* d_gamma, double* loglik, void* stream);

/* The log-likelihood and its gradient in one pass, without a host round trip
 * (for a trainer that steps on the device): *d_loglik (a device double)
 * receives the log-likelihood, d_alpha, d_beta ([n_qd]) and d_gamma ([1])
 * (device arrays, overwritten) its gradient.  Asynchronous on `stream`.  No
 * counterpart in the reference (its EM has no gradient); the pair above
 * computes the same quantities in two calls. */
int mc_dbn_loglik_grad(mc_model* m, int64_t s_begin, int64_t s_count, const float* alpha, const float* beta,
                       const float* gamma, int fp64, float* d_alpha, float* d_beta, float* d_gamma, double* d_loglik,
                       void* stream);

/* ---------------------------------------------------------------------------
 * Allocation-free evaluation.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory at the moment they evaluate:
 * a serving process whose device memory is already handed to its own pool, a
 * job under a memory budget that forbids new allocations, a host thread that
 * must not enter the allocator (and its implicit synchronisation) while other
 * streams run.  Computes the same sums as mc_model_evaluate from the caller's
 * own device buffers into the caller's host memory, keeping its intermediate
 * sums in a fixed file-scope device array (768 KB on every GPU where the
 * library's device code is loaded, held until the process exits) instead of an
 * allocation; it calls no allocating CUDA or library routine.
 *
 * model_type: MC_PBM (0), MC_CCM (1), MC_DBN (2) or MC_UBM (3).
 * Limit: n_sessions <= 16,777,216; a larger call fails with MC_ERR_INVALID.
 * Inputs (device memory): pidx session-major [n * 10], each -1 (doc unseen in
 * training) or in [0, n_qd), any other value failing the call with
 * MC_ERR_INVALID; click_mask [n]; atr [n_qd]; sat [n_qd] (MC_DBN; NULL
 * otherwise); pub = the model's public values, by model code: MC_PBM 10
 * examination, MC_CCM 3 continuation, MC_DBN 1 continuation, MC_UBM 55
 * examination.
 * Outputs (host memory): *ll_sum and log2_sums[10], as mc_model_evaluate.
 * Set-up: the first call on a device makes it current, loads the library's
 * device code there if CUDA has not yet (which reserves the array) and looks
 * up the array's device address; a call with n_sessions = 0 does only that.
 * Make that first call before any stream capture on the device, and before a
 * pool of the caller's takes the device's free memory.  The address is kept
 * per device context, and looked up again after cudaDeviceReset.
 * All calls share the array: calls that overlap on the GPU race, so serialise
 * them.  Synchronous on `stream`. */
int mc_evaluate_static(int model_type, int64_t n_sessions, const int32_t* pidx, const uint16_t* click_mask,
                       int64_t n_qd, const float* atr, const float* sat, const float* pub, double* ll_sum,
                       double* log2_sums, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MCLICKS_H */
