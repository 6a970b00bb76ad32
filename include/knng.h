/* knng.h -- C ABI of the GB300 kNN-graph builder (libknng.so).
 *
 * Drop-in for the compute core of Aftab5550/SISAP-2026-task1 src/main.cpp.
 * The reference has no library or FFI: its only interface is the process
 * (`main --task T --dataset F`, src/main.cpp:114-141) that reads /train
 * (src/main.cpp:149-177), builds the graph (src/main.cpp:179-457) and writes
 * knns/dists (src/main.cpp:459-480).  These entry points replace the code
 * between reading /train and writing the result file; the knng_main CLI keeps
 * the reference's argv, messages and output file on top of them.
 *
 * Conventions: every call returns 0 (KNNG_OK) or a negative knng_status; no
 * C++ exception crosses this boundary.  The caller owns every input and
 * output buffer; a knng_ctx owns its device memory and CUDA stream.  A ctx is
 * used by one host thread at a time.  Pointers marked _dev are device
 * pointers; `stream` arguments are cudaStream_t passed as void* (NULL = the
 * legacy default stream).
 */
#ifndef KNNG_H_
#define KNNG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes.  The reference returns -1 on every failure
 * (src/main.cpp:140, 197, 200, 484, 487); these refine that -1. */
typedef enum knng_status {
  KNNG_OK = 0,
  KNNG_E_ARGS = -1,    /* bad argument (null pointer, n < 2, bad parameter) */
  KNNG_E_DIM = -2,     /* d must be a multiple of 128 in [128, 1024] */
  KNNG_E_OOM = -3,     /* device allocation failed */
  KNNG_E_ADMIT = -4,   /* job refused by the memory-footprint admission */
  KNNG_E_TIMEOUT = -5, /* a bounded device wait gave up */
  KNNG_E_CUDA = -6,    /* CUDA runtime error (message: knng_last_error) */
  KNNG_E_REPLAY = -7,  /* replay pivot table does not match the forest */
  KNNG_E_BUSY = -8,    /* ticket not finished yet (knng_poll) */
  KNNG_E_NOTFOUND = -9, /* unknown ticket */
  KNNG_E_SCRATCH = -10, /* input too large for knng_init_graph_noalloc's fixed scratch */
  KNNG_E_BOUNDS = -11   /* a device bounds check failed: an id, permutation entry or leaf position
                           outside its array (bounds-checked build libknng_checked.so only) */
} knng_status;

enum { KNNG_QUANT_TRUNC = 0, KNNG_QUANT_ROUND = 1 };
enum { KNNG_JOIN_JACOBI = 0, KNNG_JOIN_INPLACE = 1 };
enum { KNNG_ORDER_NATURAL = 0, KNNG_ORDER_LEAF = 1 };
enum { KNNG_GRAM_DP4A = 0, KNNG_GRAM_TCGEN05 = 1 };
enum { KNNG_INIT_FOREST = 0, KNNG_INIT_RANDOM = 1, KNNG_INIT_BLOCK = 2 };
enum { KNNG_SKETCH_SIGN = 0, KNNG_SKETCH_HYPERPLANE = 1 };

/* Build parameters.  Defaults (knng_default_params) are the reference's
 * compile-time constants, src/main.cpp:19-29. */
typedef struct knng_params {
  int k_build;           /* K_BUILD = 50           src/main.cpp:22 */
  int k_eval;            /* K_EVAL = 15            src/main.cpp:21 */
  int num_trees;         /* NUM_TREES = 16         src/main.cpp:23 */
  int rerank_mult;       /* RERANK_MULTIPLIER = 8  src/main.cpp:24 */
  int leaf_size;         /* LEAF_SIZE = 64         src/main.cpp:25 */
  int max_iterations;    /* MAX_ITERATIONS = 30    src/main.cpp:27 */
  float early_stop_rate; /* EARLY_STOP_RATE = 0.04 src/main.cpp:28 */
  float rate_diff_tol;   /* RATE_DIFF_TOLERANCE = 0.01 src/main.cpp:29 */
  int quant_mode;        /* KNNG_QUANT_TRUNC: src/main.cpp:184-186 */
  int join_mode;         /* KNNG_JOIN_JACOBI (deterministic) or _INPLACE */
  int row_order;         /* KNNG_ORDER_LEAF: process rows in tree-0 leaf order */
  uint32_t seed;         /* 1337: src/main.cpp:210 (trees), :271 (fills) */
  int device;            /* CUDA device ordinal */
  int autotune;          /* 1: time the join configurations once per (d, size) */
  int use_graph;         /* 1: replay the NN-Descent phase as a CUDA graph */
  int gram_mode;         /* leaf Gram: KNNG_GRAM_DP4A or KNNG_GRAM_TCGEN05 (f16 tensor cores) */
  int init_mode;         /* KNNG_INIT_FOREST (src/main.cpp); KNNG_INIT_RANDOM, the archived
                            variant archive/nndescent_optimized.cpp:97-118 (needs n > k_build);
                            KNNG_INIT_BLOCK, the archived block-partitioned hybrid
                            archive/nndescent_hybrid.cpp:98-144 (see block_size, bridges) */
  int join_cache;        /* 1: each row keeps its previous iteration's distinct candidates with
                            their Hamming scores and known rejections (n * 6 KB of device
                            memory), so later iterations skip most sketch and row gathers;
                            results are identical either way.  0: no cache. */
  int block_size;        /* KNNG_INIT_BLOCK: rows per block; each job is split into
                            max(1, round(n / block_size)) equal consecutive blocks (10000:
                            the archive's 200000 rows / 20 blocks, nndescent_hybrid.cpp:20-21) */
  int bridges;           /* KNNG_INIT_BLOCK: last entries of each row replaced by random rows
                            (2, nndescent_hybrid.cpp:22); drawn with xorshift32 from seed + row */
  int wait_limit;        /* polls before a bounded device wait gives up with KNNG_E_TIMEOUT:
                            0 = the default (2^26); a negative value makes those waits give up
                            at once (only used to test the timeout path).  The tensor-core leaf
                            Gram's waits for its tensor-core work; its final drain always keeps
                            the full limit. */
  int join_ctas_per_sm;  /* 0: the autotuner picks the NN-Descent kernel variant; 3 or 4 with
                            join_cblock 2, 4 or 8 forces that variant (resident CTAs per SM x
                            Hamming candidates in flight) for every iteration and for
                            knng_join_iter.  Results are identical for every variant. */
  int join_cblock;
  int sketch_mode;       /* KNNG_SKETCH_SIGN: one sign bit per coordinate, d bits per row, as
                            src/main.cpp:182-190 (default).  KNNG_SKETCH_HYPERPLANE: 128 bits per
                            row, the signs of the int8 codes projected on 128 integer
                            hyperplanes drawn from `seed` (the README's random-hyperplane
                            sketch, README.md:33-34; no output of the reference to match) */
  int forest_fuse;       /* 1 (default): with native pivots, forest nodes of >= 512 members
                            are split three levels per pass over their code rows, the
                            descendants' pivots drawn from a seeded, evaluated sample of the
                            node's members; 0: one level per pass.  A replay table
                            (knng_forest) always splits one level per pass. */
} knng_params;

/* Per-build timings and convergence record (seconds, device-timed). */
typedef struct knng_stats {
  double quantize_s;  /* H2D copy + quantise/sketch (outside build_s, as :203) */
  double forest_s;    /* RP forest                 src/main.cpp:205-218 */
  double init_s;      /* leaf Gram + top-K init    src/main.cpp:220-316 */
  double join_s;      /* NN-Descent iterations     src/main.cpp:318-440 */
  double export_s;    /* top-k_eval export + D2H   src/main.cpp:445-457 */
  double build_s;     /* forest + init + join, the reference's buildtime */
  double total_s;     /* whole knng_build call */
  int iterations;     /* NN-Descent iterations run */
  int64_t updates[64];/* per-iteration update counts (src/main.cpp:433) */
  int64_t forest_levels;
  int64_t leaves;
  double device_s;        /* first to last device event of the call */
  double join_ms[64];     /* device time of each NN-Descent launch */
  int64_t join_candidates[64]; /* sketches scored per iteration (distinct candidates without a
                                  cached score) */
  int64_t join_dots[64];  /* int8 rows reranked per iteration */
  int64_t kernel_launches;/* libknng kernels launched by the call */
  int join_ctas_per_sm;   /* autotuned join configuration used */
  int join_cblock;
  int graph_used;         /* NN-Descent phase ran as a CUDA graph */
  int64_t join_distinct[64]; /* distinct two-hop candidates per iteration (all rows) */
  int64_t join_skipped[64];  /* rows copied through per iteration because neither their list nor
                                any neighbour's list changed in the previous one (double-buffered
                                iterations: their result is provably their current list) */
} knng_stats;

/* One job of a batch (knng_build_batch).  Inputs as for knng_build; status
 * and iterations are written back. */
typedef struct knng_job {
  const void* rows;
  int64_t n;
  int d;
  int rows_on_device;
  int32_t* knns;
  float* dists;
  int out_on_device;
  int status;      /* out: KNNG_OK or the error of the job's group */
  int iterations;  /* out: NN-Descent iterations the job ran */
} knng_job;

typedef struct knng_ctx knng_ctx;

/* Fill *p with the reference defaults (src/main.cpp:19-29). */
void knng_default_params(knng_params* p);

/* Create a context on p->device.  Replaces the reference's process start-up
 * and array allocation, src/main.cpp:143-163. */
int knng_create(knng_ctx** out, const knng_params* p);

/* Release the context and all its device memory. */
void knng_destroy(knng_ctx* ctx);

/* Build the all-points kNN graph of n rows of d float32 (row-major).
 * Replaces src/main.cpp:179-457 (quantise, forest, init, NN-Descent, export).
 * rows      : host or device pointer (rows_on_device selects).  Host rows in
 *             memory the device maps (pinned, registered or managed) are read
 *             in place by the quantise kernel over the host link; pageable
 *             rows (malloc, std::vector, numpy) are copied by host threads
 *             through pinned buffers of the context, and the device never
 *             touches the pageable memory itself.  Host knns/dists in
 *             pageable memory are written the same way.
 * knns      : n * k_eval int32, 1-based ids, each row worst -> best
 *             (src/main.cpp:452, 455).
 * dists     : n * k_eval float32 int8 inner products, same order (:453, 456).
 * out_on_device selects whether knns/dists are device pointers.
 * stats may be NULL.  The call works on the context's own non-blocking
 * stream and returns after the results are complete; device input must be
 * fully written before the call (it does not wait for other streams). */
int knng_build(knng_ctx* ctx, const void* rows, int64_t n, int d, int rows_on_device,
               int32_t* knns, float* dists, int out_on_device, knng_stats* stats);

/* Batched builds (no counterpart in the reference, which builds one graph per
 * process): independent jobs of any n and d are built together, jobs of equal
 * d as one problem laid out back to back -- one forest pass, one leaf Gram and
 * merge, one persistent join launch per iteration over every job's rows, the
 * NN-Descent phase replayed as a CUDA graph.  Each job keeps its own pivots,
 * random fills and early stop (src/main.cpp:432-439), so its knns/dists are
 * bit-identical to knng_build of that job alone.  Groups of different d run
 * concurrently, each on its own internal context and stream.  stats (may be
 * NULL): stage times summed over groups, device_s = the batch's span. */
int knng_build_batch(knng_ctx* ctx, knng_job* jobs, int count, knng_stats* stats);

/* ---- serving loop (no counterpart in the reference) ----
 * A server accepts build jobs as they arrive, admits them by device-memory
 * footprint against mem_budget_gb, and runs whatever fits as a batch on each of
 * `slots` worker streams, so jobs that arrive while others are on the GPU start
 * as soon as a slot and memory free up and overlap on the device.  The job's
 * rows and output buffers must stay valid until its ticket is done.  Each
 * result is bit-identical to knng_build of the job alone. */
typedef struct knng_server knng_server;

typedef struct knng_server_params {
  knng_params build;     /* build parameters of every job */
  int slots;             /* concurrent batches (worker streams), default 3 */
  double mem_budget_gb;  /* device memory the running batches may use, default 180 */
  int max_batch_jobs;    /* jobs per batch, default 64 */
} knng_server_params;

typedef struct knng_result {
  int status;            /* KNNG_OK, KNNG_E_ADMIT (larger than the budget), or a build error */
  int iterations;        /* NN-Descent iterations of the job */
  int batch_jobs;        /* size of the batch it ran in */
  double queued_s;       /* submit -> batch start */
  double run_s;          /* batch start -> done */
  double latency_s;      /* submit -> done */
} knng_result;

void knng_server_default_params(knng_server_params* p);
int knng_server_create(knng_server** out, const knng_server_params* p);
/* Queue one job (the descriptor is copied); *ticket identifies it. */
int knng_submit(knng_server* sv, const knng_job* job, uint64_t* ticket);
/* KNNG_OK with *r filled when done, KNNG_E_BUSY while queued or running. */
int knng_poll(knng_server* sv, uint64_t ticket, knng_result* r);
/* Block until done or timeout_s elapsed (KNNG_E_TIMEOUT). */
int knng_wait(knng_server* sv, uint64_t ticket, double timeout_s, knng_result* r);
/* Forget a finished ticket. */
int knng_release(knng_server* sv, uint64_t ticket);
/* Stop the workers after their running batches; queued jobs are dropped. */
void knng_server_destroy(knng_server* sv);

/* Device bytes a build of n rows of dimension d needs with parameters p
 * (NULL = defaults): the admission estimate of the serving loop.  Host rows
 * need no device staging (rows_on_device does not change the figure). */
int64_t knng_footprint_bytes(const knng_params* p, int64_t n, int d, int rows_on_device);

/* Return all of the context's device buffers to the stream-ordered pool
 * and free its pinned host staging buffers (kept for reuse otherwise). */
int knng_trim(knng_ctx* ctx);

/* Text for a status code, and the last detailed error message of ctx. */
const char* knng_status_string(int status);
const char* knng_last_error(const knng_ctx* ctx);

/* ---- stage entry points (device pointers; used by the parity tests) ---- */

/* a1, src/main.cpp:179-192: int8 codes [n][d] and sign sketches [n][d/64]
 * (bit k%64 of word k/64 set iff the clamped value is > 0). */
int knng_quantize(const float* x_dev, int64_t n, int d, int quant_mode, int8_t* codes_dev,
                  uint64_t* sketch_dev, void* stream);

/* Optional sketch (no counterpart in src/main.cpp, whose sketch is the sign
 * of each coordinate; its README.md:33-34 describes random hyperplanes):
 * sketch_dev[n][2] receives 128 bits per row, bit k set iff the exact int32
 * projection of the row's int8 codes on seeded integer hyperplane k is > 0.
 * Plane k, coordinate j: h = SplitMix64((seed << 32) ^ (k << 10 | j)),
 * value = sum over the 4 low bytes b of h of (b >> 2) - 32.  codes_dev must be
 * 16-byte aligned; d a multiple of 128 in [128, 1024]. */
int knng_sketch_hyperplane(const int8_t* codes_dev, int64_t n, int d, uint32_t seed, uint64_t* sketch_dev,
                           void* stream);

/* a2/a3, src/main.cpp:47-99, 205-232: RP forest.  perm_dev[t*n + p] is the id
 * at position p of tree t's leaf order; leaf_flag_dev[t*n + p] = 1 where a
 * leaf starts.  replay (host, may be NULL) holds n_replay internal nodes as
 * int32 sextuples (tree, level, start, size, p1_id, p2_id), e.g. the pivots
 * the reference's std::mt19937 draws; NULL draws pivots from a counter-based
 * hash of (seed, tree, start, size). */
int knng_forest(knng_ctx* ctx, const int8_t* codes_dev, int64_t n, int d,
                const int32_t* replay, int64_t n_replay, int32_t* perm_dev,
                uint8_t* leaf_flag_dev);

/* a4, src/main.cpp:220-314: initial graph ids/scores [n][k_build] from the
 * forest, ordered by (score desc, pool position asc). */
int knng_init_graph(knng_ctx* ctx, const int8_t* codes_dev, int64_t n, int d,
                    const int32_t* perm_dev, const uint8_t* leaf_flag_dev, int32_t* ids_dev,
                    int32_t* scores_dev);

/* a5, src/main.cpp:324-430: one NN-Descent iteration reading ids_in/scores_in
 * and writing ids_out/scores_out (the same pointers = in place).  sketch_dev
 * holds the context's sketch_mode's sketches: [n][d/64] sign sketches, or
 * [n][2] hyperplane sketches.  The rerank
 * set is the best k_build*rerank_mult candidates by (hamming desc, sequence
 * position asc), visited in that order.  *updates receives the number of
 * positions whose id changed. */
int knng_join_iter(knng_ctx* ctx, const int8_t* codes_dev, const uint64_t* sketch_dev, int64_t n,
                   int d, const int32_t* ids_in_dev, const int32_t* scores_in_dev,
                   int32_t* ids_out_dev, int32_t* scores_out_dev, int64_t* updates);

/* a6, src/main.cpp:446-457: knns = id + 1, dists = float(score) of the first
 * k_eval of k_build entries, each row reversed.  id_map (may be NULL) maps
 * internal ids to caller ids before the + 1. */
int knng_export(const int32_t* ids_dev, const int32_t* scores_dev, int64_t n, int k_build,
                int k_eval, const int32_t* id_map_dev, int32_t* knns_dev, float* dists_dev,
                void* stream);

/* No counterpart in the reference (it allocates with std::vector on the host
 * and has no device code).  The initial-graph stage of knng_init_graph for
 * callers that may not allocate device memory: processes whose GPU memory is
 * owned by another allocator (a framework's caching pool, a database's device
 * memory manager, a plugin host), where a raw cudaMalloc would escape or
 * fragment that pool and cudaFree would synchronise the whole device.  The
 * caller passes inputs and outputs as in knng_init_graph, plus the parameters
 * a context would hold; the stage's scratch is one fixed 64 MiB device array
 * inside libknng.so (held by every GPU that loads the library until exit), so
 * num_trees * n is limited to about 240,000 (about 15,000 rows with 16 trees);
 * larger inputs return KNNG_E_SCRATCH before any device work.  It calls no
 * cudaMalloc, cudaFree or allocating library routine.  The first call on each
 * device (with that device current) resolves the array's device address; make
 * it before any stream capture.  Calls share the array: calls that overlap on
 * the GPU race and must be serialised.  Returns after `stream` has finished
 * the stage (NULL = the legacy default stream). */
int knng_init_graph_noalloc(const int8_t* codes_dev, int64_t n, int d, int num_trees, int leaf_size,
                            int k_build, uint32_t seed, const int32_t* perm_dev,
                            const uint8_t* leaf_flag_dev, int32_t* ids_dev, int32_t* scores_dev,
                            void* stream);

/* PCA preprocessing, the reference's scripts/data_prep/apply_pca.py:25-33:
 * rows (n x d float32, host or device memory) are centred, projected onto the
 * `dims` principal components of their covariance (largest first, each
 * component's largest-magnitude entry positive, as sklearn's svd_flip), every
 * projected row is L2-normalised and rounded to float16 (IEEE half bits) into
 * out_f16 (n x dims, host or device).  variance_kept (may be NULL) receives the
 * fraction of the variance the components keep.  Uses cuBLAS and cuSOLVER on
 * `device`; values agree with sklearn's PCA to float32 precision.  Needs
 * about 4 n (d + dims) bytes of device memory.  Not part of the build path
 * (src/main.cpp never uses it). */
int knng_pca(const float* rows, int64_t n, int d, int dims, int device, uint16_t* out_f16,
             double* variance_kept);

#ifdef __cplusplus
}
#endif
#endif /* KNNG_H_ */
