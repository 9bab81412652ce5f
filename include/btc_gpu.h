/*
 * btc_gpu.h -- C ABI of the GB300-native BTC-GPU sparse CP-SGD path.
 *
 * The reference reaches its GPU code through three C++ seams with config in
 * mutable globals:
 *   tensor_SGD(train, test)                       tensor_SGD.h:101, tensor_SGD.cu:55-90
 *   block_problem(train, n, test, m, a, b, c, rate)   block.h:24-31,  block.cu:1233-1287
 *   sgd_train(train, n, test, m, a, b, c, num_parallel, max_parallel, ..., num_bs, bs, nbs)
 *                                                 sgd_Kernel.h:24-38, sgd_Kernel.cu:968-1361
 * This header replaces them with plain C entry points: a config struct in
 * place of the globals, a host-side schedule object in place of block_problem's
 * BS_node/b_node arrays, and a device context in place of sgd_train's body.
 * All pointers are caller-owned host memory unless stated; nothing here
 * exits the process: every call returns a btc_status.
 *
 * Layout conventions:
 *   coordinates  int32 triples (x, y, z), 0-based, row-major n x 3
 *   values       double (the reference's T_node::rate, tensor_SGD.h:52-55)
 *   factors      row-major [rows][rank] double on the host side; the device
 *                copy is stored in the context's dtype
 */
#ifndef BTC_GPU_H
#define BTC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BTC_ABI_VERSION 1

typedef enum btc_status {
    BTC_OK = 0,
    BTC_ERR_ARG = 1,         /* invalid argument or configuration */
    BTC_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    BTC_ERR_ALLOC = 3,       /* host or device allocation failed */
    BTC_ERR_STATE = 4,       /* call out of order / object in a failed state */
    BTC_ERR_IO = 5,          /* file could not be opened, read or written */
    BTC_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
    BTC_ERR_UNSUPPORTED = 7, /* valid request this library does not implement */
    BTC_ERR_RANGE = 8,       /* index or level outside the representable range */
    BTC_ERR_NO_DEVICE = 9,   /* no CUDA device visible */
    BTC_ERR_DEVICE = 10      /* a kernel reported an error status */
} btc_status;

typedef enum btc_dtype {
    BTC_DTYPE_F32 = 0,  /* FP32 factors, FP32 math (the plain path) */
    BTC_DTYPE_F64 = 1,  /* FP64 factors and math (the reference's precision) */
    BTC_DTYPE_BF16 = 2  /* BF16 factors, FP32 math, stochastic rounding */
} btc_dtype;

typedef enum btc_mode {
    /* Every slot of the schedule is cut into chunks that all SMs sweep in
     * schedule order; rows are read from L2 and updated with atomic adds,
     * as the reference's GPUs kernel does inside a slot. Not bit-reproducible. */
    BTC_MODE_HOGWILD = 0,
    /* Slots run one warp each, entries strictly in block order, and slots that
     * share a factor row run in schedule order.  Bit-identical to a serial
     * replay of the schedule (the FP64 instantiation matches the serial FP64
     * rule bit for bit). */
    BTC_MODE_DETERMINISTIC = 1,
    /* One CTA per slot: the slot's reused rows are staged in shared memory,
     * updated there, and each row is written back once as a delta. */
    BTC_MODE_STAGED = 2,
    /* The reference's lock-free variant (tensor_LF, sgd_Kernel.cu:401-451,
     * ToMatrix_LF, block.cu:1192-1217): the conflict-free strata before
     * padding, every block once, no coe weights, and the in-place rule
     * a += lr(e b c - reg a), then b with the new a, then c with the new a
     * and b, element by element.  Blocks run one warp each, entries in block
     * order, blocks sharing a row in strata order (F32 / F64; the FP64
     * instantiation equals the serial replay of the rule bit for bit).  The
     * reference runs it on one CTA whose threads race on shared rows. */
    BTC_MODE_LOCKFREE = 3
} btc_mode;

typedef enum btc_split { BTC_SPLIT_TRAIN = 0, BTC_SPLIT_TEST = 1 } btc_split;

/* Configuration: the reference's globals (tensor_SGD.h:25-42, defaults in
 * tensor_SGD.cu:24-41) plus the options this library adds. */
typedef struct btc_config {
    int32_t I, J, K;                /* mode sizes */
    int32_t epochs;                 /* default 1000 */
    int32_t rank;                   /* r, default 16 */
    double lr;                      /* default 0.005 */
    double reg;                     /* default 0.0005 */
    int32_t block_s;                /* block capacity, default 2048 */
    int32_t thread_size;            /* accepted for compatibility, default 512 */
    int32_t parallel_sequence_size; /* blocks per stratum on the GPU; 0 = auto; default 8 */
    int32_t requested_gpu_count;    /* accepted; the library always uses one GPU */
    int32_t dtype;                  /* btc_dtype, default BTC_DTYPE_F32 */
    int32_t mode;                   /* btc_mode, default BTC_MODE_HOGWILD */
    int32_t device;                 /* CUDA device ordinal, default 0 */
    /* SMs x max resident blocks per SM used by the auto stratum width
     * (block.cu:577-606); 0 = ask the device, -1 = no device (width =
     * widest conflict-free stratum) */
    int32_t resident_blocks;
    int32_t chunk;                  /* entries per Hogwild work item, 0 = auto */
    int32_t host_threads;           /* builder threads, 0 = hardware concurrency */
    int32_t ctas_per_sm;            /* staged kernel: CTAs sharing one SM's shared memory, 0 = auto */
    int32_t row_repeat;             /* staged kernel: most entries of one row in a tile; 0 = the
                                       power of two at or below 0.16 / lr, in [16, 512] */
    int32_t reserved[5];
} btc_config;

typedef struct btc_schedule_summary {
    int32_t num_blocks;          /* blocks created, including empty ones */
    int32_t nonempty_blocks;
    int32_t num_strata;          /* conflict-free strata before balancing */
    int32_t max_parallel_cf;     /* widest conflict-free stratum */
    int32_t target_gpu_blocks;   /* stratum width after balancing */
    int32_t num_groups;          /* strata after balancing (num_parallel - 1) */
    int32_t num_slots;           /* scheduled (block, stratum) pairs */
    int32_t max_parallel;        /* widest balanced stratum (the reference's grid size) */
    int64_t scheduled_updates;   /* entries executed per epoch (sum of slot nnz) */
    int64_t train_nnz;
    int32_t global_levels[3];    /* final global split level per axis */
    int32_t reserved;
    double build_seconds[3];     /* blocking, strata, balancing wall time */
} btc_schedule_summary;

typedef struct btc_metrics {
    double rmse, mae, er;        /* compute_metrics_gpu's outputs (sgd_Kernel.cu:136-201) */
    double sse, sae, ref2;       /* FP64 sums they are derived from */
    int64_t count;
} btc_metrics;

typedef struct btc_epoch_stats {
    double kernel_ms;            /* device time of the epoch's SGD launches (CUDA events) */
    int64_t updates;             /* entries executed */
    int32_t launches;            /* kernels launched for the epoch */
    int32_t device_status;       /* error word the kernels wrote (0 = none) */
} btc_epoch_stats;

typedef struct btc_schedule btc_schedule;
typedef struct btc_ctx btc_ctx;

const char *btc_status_string(btc_status s);
int32_t btc_abi_version(void);

/* Reference defaults (tensor_SGD.cu:24-41). */
btc_status btc_config_default(btc_config *cfg);
/* Validation as main.cpp:169-203 (rank in [1,100] lifted to [1,128]). */
btc_status btc_config_validate(const btc_config *cfg);

/* ---- text I/O (main.cpp:24-99) ------------------------------------------
 * Reads "x y z value" lines; skips empty lines, lines starting with '#' or
 * '%', and lines that do not start with three integers and a number;
 * subtracts coord_base; rejects out-of-range coordinates with BTC_ERR_RANGE
 * (the reference exits).  The arrays are allocated by the library and freed
 * with btc_free; *line_no receives the offending line on BTC_ERR_RANGE. */
btc_status btc_read_entries(const char *path, int32_t coord_base, int32_t I, int32_t J,
                            int32_t K, int32_t **xyz, double **val, int64_t *n,
                            int64_t *line_no);
void btc_free(void *p);
/* btc_read_entries through a binary cache (no reference counterpart): when
 * the file at `cache` was written for this source file (same size and
 * modification time) and the same coord_base, I, J, K, its entries are read
 * as they are; otherwise `path` is parsed with btc_read_entries and, on
 * success, the cache is written (atomically; an unwritable location is no
 * error).  The cache holds a 48-byte header, then n x 3 int32 coordinates
 * (base subtracted) and n doubles in host byte order.  *from_cache is 1 when
 * the entries came from the cache. */
btc_status btc_read_entries_cached(const char *path, const char *cache, int32_t coord_base,
                                   int32_t I, int32_t J, int32_t K, int32_t **xyz, double **val,
                                   int64_t *n, int64_t *line_no, int32_t *from_cache);
/* std::shuffle with std::mt19937(seed) over n entries, as main.cpp:303-306
 * does with seed 42; permutes xyz and val together. */
btc_status btc_shuffle_entries(int32_t *xyz, double *val, int64_t n, uint32_t seed);

/* ---- host schedule (replaces block_problem up to Preproccess_list,
 *      block.cu:1233-1278) ------------------------------------------------ */
btc_status btc_schedule_build(const btc_config *cfg, const int32_t *xyz, int64_t n,
                              btc_schedule **out);
btc_status btc_schedule_summarize(const btc_schedule *s, btc_schedule_summary *out);
/* per block: meta[4*b..] = nnz, level_x, level_y, level_z; codes[3*b+a] =
 * id bits 1..level-1 of axis a, MSB first (position 0 is always 0) */
btc_status btc_schedule_blocks(const btc_schedule *s, int32_t *meta, uint64_t *codes);
/* entry indices (into the array given to btc_schedule_build) of block b, in
 * block order; *n in: capacity, out: count */
btc_status btc_schedule_block_entries(const btc_schedule *s, int32_t b, int32_t *out,
                                      int32_t *n);
/* conflict-free strata before balancing: off[num_strata+1], ids[] */
btc_status btc_schedule_strata(const btc_schedule *s, int32_t *off, int32_t *ids);
/* balanced groups: off[num_groups+1], slot block ids, coe[3*slot] */
btc_status btc_schedule_groups(const btc_schedule *s, int32_t *off, int32_t *slot_block,
                               double *slot_coe);
/* block_parallel.txt, byte-compatible with block.cu:822-925 */
btc_status btc_schedule_write_report(const btc_schedule *s, const btc_config *cfg,
                                     const char *path);
void btc_schedule_free(btc_schedule *s);

/* ---- device context (replaces sgd_train's state, sgd_Kernel.cu:1042-1266)
 * Every train and test coordinate must lie in [0,I) x [0,J) x [0,K):
 * otherwise BTC_ERR_RANGE, before anything reaches the device. */
btc_status btc_ctx_create(const btc_config *cfg, const btc_schedule *s, const int32_t *train_xyz,
                          const double *train_val, int64_t ntrain, const int32_t *test_xyz,
                          const double *test_val, int64_t ntest, btc_ctx **out);
/* mode 0 = A (I rows), 1 = B (J rows), 2 = C (K rows); host is [rows][rank] */
btc_status btc_ctx_set_factors(btc_ctx *ctx, int32_t mode, const double *host);
btc_status btc_ctx_get_factors(btc_ctx *ctx, int32_t mode, double *host);
/* New learning rate and regularisation for the following epochs (no
 * counterpart in the reference, whose lr and reg are fixed per run).  The
 * rows that decay from their value at write time stay the ones chosen at
 * creation. */
btc_status btc_ctx_set_rates(btc_ctx *ctx, double lr, double reg);
/* (In staged contexts the tiles' row_repeat bound was chosen for the
 * creation lr: a much larger lr wants a context built with it.) */
/* U(lo, hi) init from a counter-based generator (seed, mode, row, col) */
btc_status btc_ctx_init_factors(btc_ctx *ctx, uint64_t seed, double lo, double hi);
/* One epoch: the reference's GPUs<<<max_parallel, thread_size>>> launch
 * (sgd_Kernel.cu:1283-1285). */
btc_status btc_train_epoch(btc_ctx *ctx, btc_epoch_stats *stats);
/* n epochs back to back on the context's stream, bracketed by CUDA events on
 * that stream; stats->kernel_ms is the device time of all n epochs. */
btc_status btc_train_epochs(btc_ctx *ctx, int32_t n, btc_epoch_stats *stats);
/* compute_metrics_gpu (sgd_Kernel.cu:136-201) on the train or test split;
 * FP64 sums on the GPU.  count 0 gives NaN metrics like the reference. */
btc_status btc_eval(btc_ctx *ctx, int32_t split, btc_metrics *out);
/* ---- per-tile timing and features (staged contexts) -----------------------
 * No counterpart in the reference: the data the learned cost model trains
 * on.  A tile is a run of one scheduled block's entries whose rows fit in
 * shared memory; BTC_TILE_FEATURES floats describe each (entries, staged rows,
 * row mix per mode, owner segments, longest segment, reuse, position in its
 * block).  btc_train_epoch_profiled is a normal training epoch that also
 * returns the nanoseconds each tile took on the GPU (%globaltimer). */
#define BTC_TILE_FEATURES 10
btc_status btc_ctx_tile_count(btc_ctx *ctx, int64_t *n);
btc_status btc_ctx_tile_features(btc_ctx *ctx, float *features);
btc_status btc_train_epoch_profiled(btc_ctx *ctx, uint32_t *tile_ns, btc_epoch_stats *stats);
/* The tiles of each scheduled slot: tile0[slot], ntiles[slot] (num_slots each;
   a slot whose block has no entries has tile0 -1 and ntiles 0). */
btc_status btc_ctx_slot_tiles(btc_ctx *ctx, int32_t *tile0, int32_t *ntiles);
/* Work units of the staged kernel: a CTA takes slots [unit_off[u],
 * unit_off[u+1]) at once (schedule order is kept).  unit_off[0] = 0,
 * unit_off[nunits] = num_slots, strictly increasing.  The default is one slot
 * per unit. */
btc_status btc_ctx_set_work_units(btc_ctx *ctx, const int32_t *unit_off, int32_t nunits);

/* ---- learned cost model ---------------------------------------------------
 * No counterpart in the reference.  A small MLP (n_in -> 32 -> 32 -> 1, tanh)
 * whose forward, backward and Adam kernels are this library's own CUDA code.
 * It learns the time of a tile from BTC_TILE_FEATURES features (trained on
 * log microseconds recorded by btc_train_epoch_profiled) and proposes the
 * work units of the staged kernel: runs of consecutive slots of balanced
 * predicted cost, so that CTAs take work less often without straggling.  The
 * plain heuristic (one slot per unit) is the fallback and measured epoch time
 * decides. */
typedef struct btc_mlp btc_mlp;
btc_status btc_mlp_create(int32_t n_in, int32_t n_hidden, uint64_t seed, int32_t device, btc_mlp **out);
btc_status btc_mlp_destroy(btc_mlp *m);
btc_status btc_mlp_param_count(const btc_mlp *m, int64_t *n);
btc_status btc_mlp_get_params(btc_mlp *m, float *host);
btc_status btc_mlp_set_params(btc_mlp *m, const float *host);
/* full-batch mean-squared-error gradient (n samples, n_in features each) */
btc_status btc_mlp_gradient(btc_mlp *m, const float *x, const float *y, int64_t n, float *grad, double *loss);
/* `steps` full-batch Adam steps; *final_loss is the loss after the last one */
btc_status btc_mlp_train(btc_mlp *m, const float *x, const float *y, int64_t n, int32_t steps, float lr,
                         double *final_loss);
btc_status btc_mlp_predict(btc_mlp *m, const float *x, int64_t n, float *y);
/* number of input features the model was created with */
int32_t btc_mlp_inputs(const btc_mlp *m);

/* ---- learned blocking -------------------------------------------------------
 * No counterpart in the reference (which splits at code-range midpoints,
 * block.cu:154-401, and pads strata with repeated blocks, block.cu:660-697).
 * A binary tree over the (i, j, k) space whose leaves hold <= block_s
 * entries, each node split at the median coordinate of its entries on the
 * axis the cost model predicts cheapest (model: BTC_BLOCK_FEATURES inputs,
 * log microseconds per block; NULL = the axes in turn); every block is
 * scheduled once per epoch, in conflict-free groups of at most
 * parallel_sequence_size blocks (8 when 0), heaviest predicted first; every
 * coe weight is 1.  Not bit-exact with the reference by design: measured
 * epoch time or time to a test RMSE decides between it and
 * btc_schedule_build.  The schedule works with every context mode. */
#define BTC_BLOCK_FEATURES 10
btc_status btc_schedule_build_learned(const btc_config *cfg, const int32_t *xyz, int64_t n, btc_mlp *model,
                                      btc_schedule **out);
/* boxes[6*b ..] = lo_x, hi_x, lo_y, hi_y, lo_z, hi_z of block b (learned
 * schedules only; BTC_ERR_STATE otherwise) */
btc_status btc_schedule_block_boxes(const btc_schedule *s, int32_t *boxes);
/* Training samples for the block cost model (staged contexts): one profiled
 * training epoch, then for every scheduled block with a measured time its
 * BTC_BLOCK_FEATURES features (entries, distinct rows and largest row share
 * per mode, ...) and the log of its microseconds.  *n in: capacity (samples),
 * out: samples written (or, with too small a capacity, the count needed). */
btc_status btc_ctx_block_profile(btc_ctx *ctx, float *features, float *log_us, int64_t *n);

typedef struct btc_learn_report {
    double plain_ms;      /* mean measured epoch time, one slot per unit */
    double learned_ms;    /* mean measured epoch time with the proposed units */
    double model_loss;    /* training loss (mean squared error of log microseconds) */
    double model_r2;      /* fraction of tile-time variance the model explains */
    int64_t samples;      /* tiles the model was trained on */
    int32_t units;        /* work units proposed */
    int32_t kept;         /* 1: the proposed units were kept; 0: the heuristic stayed */
} btc_learn_report;
/* profile one epoch, train `model`, propose units, time trial_epochs epochs of
 * each (they are training epochs) and keep the faster */
btc_status btc_ctx_learn_work_units(btc_ctx *ctx, btc_mlp *model, int32_t train_steps, int32_t trial_epochs,
                                    btc_learn_report *report);

/* ---- autotuner -------------------------------------------------------------
 * No counterpart in the reference.  Times the staged kernel on the context's
 * own tiles for every lane-group shape (lanes per entry x 16-byte vectors per
 * lane, same row coverage) and every CTAs-per-SM count the shared memory
 * allows, epochs_per_candidate training epochs each, and keeps the fastest.
 * The tile capacity (rows per tile for the rank) is fixed when the context
 * is created (cfg.ctas_per_sm). */
typedef struct btc_autotune_report {
    int32_t lanes_per_entry;
    int32_t vectors_per_lane;
    int32_t ctas_per_sm;
    int32_t candidates;
    double best_ms;       /* mean epoch time of the choice */
    double default_ms;    /* mean epoch time of the default shape and grid */
} btc_autotune_report;
btc_status btc_ctx_autotune(btc_ctx *ctx, int32_t epochs_per_candidate, btc_autotune_report *report);

/* ---- many tensors in one launch ------------------------------------------
 * No counterpart in the reference (its binary trains one tensor per run).
 * A batch runs the epochs of several staged contexts (same device, FP32 or
 * BF16 each the same) as ONE persistent kernel launch: the contexts' work
 * units are interleaved in proportion to their sizes into one list that all
 * CTAs drain from a single counter, every tensor with its own rank, tiles and
 * factors.  With use_graph the epoch (counter reset, the launch, BF16 master
 * refreshes, rounding-seed step) is captured once as a CUDA graph and
 * replayed.  The contexts must outlive the batch; btc_eval on each context
 * still works between batch epochs. */
typedef struct btc_batch btc_batch;
btc_status btc_batch_create(btc_ctx *const *ctxs, int32_t n, btc_batch **out);
btc_status btc_batch_train_epochs(btc_batch *b, int32_t epochs, int32_t use_graph, btc_epoch_stats *stats);
btc_status btc_batch_destroy(btc_batch *b);

/* Device stream the context launches on (a cudaStream_t). */
void *btc_ctx_stream(btc_ctx *ctx);
btc_status btc_ctx_destroy(btc_ctx *ctx);

/* One end-to-end step from host buffers: upload the factors, run one epoch,
 * evaluate the test split and read the factors back (the timed unit of the
 * end-to-end measurement). */
btc_status btc_train_epoch_host(btc_ctx *ctx, double *A, double *B, double *C,
                                btc_epoch_stats *stats, btc_metrics *test);

/* Visible CUDA devices (main.cpp:274-284 and the inventory of
 * sgd_Kernel.cu:492-503); name must hold 256 bytes. */
btc_status btc_device_count(int32_t *count);
btc_status btc_device_info(int32_t device, char *name, int32_t *sm_count, int64_t *memory_bytes);

/* ---- error sums without allocation ----------------------------------------
 * No counterpart in the reference: an added entry point for callers that
 * cannot call cudaMalloc -- hosts whose framework owns every device
 * allocation (a caching allocator that has reserved the memory, an engine
 * that forbids allocation after start-up), allocation-free real-time loops.
 * It computes the FP64 sums (SSE, SAE, sum ref^2) of compute_metrics_gpu
 * over n entries and writes them to sums[0..2].
 * Every pointer is DEVICE memory supplied by the caller: xyz is n x 3 int32,
 * val n doubles, A/B/C row-major factors of `dtype` (F32 or F64) with
 * `row_stride` elements per row (>= rank), sums 3 doubles.  Every entry's
 * x, y and z must name an existing row of A, B and C respectively: the
 * call is given no row counts and checks none.  The launch goes
 * on `stream` (a cudaStream_t, NULL for the default stream) and is not
 * waited for.
 * Its only scratch is a file-scope device array of BTC_NOALLOC_MAX_ENTRIES /
 * 1024 partial triples (1.5 MiB per GPU, held until exit); n above
 * BTC_NOALLOC_MAX_ENTRIES returns BTC_ERR_RANGE without launching.  The
 * first call on a device looks up that array's address (call it once before
 * any stream capture).  All calls on a device share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
#define BTC_NOALLOC_MAX_ENTRIES 67108864LL
btc_status btc_eval_sums_noalloc(const int32_t *xyz, const double *val, int64_t n, const void *A,
                                 const void *B, const void *C, int32_t dtype, int32_t rank,
                                 int64_t row_stride, double *sums, void *stream);

/* Page-locked host memory for the end-to-end transfers (cudaHostAlloc). */
btc_status btc_host_alloc(void **p, int64_t bytes);
void btc_host_free(void *p);

/* ---- synthetic tensors ---------------------------------------------------- */
typedef struct btc_gen_spec {
    int32_t I, J, K;
    int64_t nnz;               /* unique entries to produce */
    double zipf_s[3];          /* per mode; 0 = uniform */
    int32_t gt_rank;           /* ground-truth CP rank (values), 0 = log-normal values */
    double gt_std;             /* ground-truth factor std */
    double noise_std;
    double train_frac;         /* Bernoulli train probability */
    uint64_t seed;
    int32_t threads;           /* 0 = hardware concurrency */
    int32_t reserved[3];
} btc_gen_spec;

/* Library-allocated arrays (free with btc_free). */
btc_status btc_gen_tensor(const btc_gen_spec *spec, int32_t **train_xyz, double **train_val,
                          int64_t *ntrain, int32_t **test_xyz, double **test_val,
                          int64_t *ntest);

#ifdef __cplusplus
}
#endif
#endif /* BTC_GPU_H */
