/*
 * tilespgemm.h -- C ABI of the GB300-native tiled FP64 SpGEMM library
 * (libtilespgemm.so).  Plain C types only: no C++ or torch types cross it.
 *
 * It replaces the SpGEMM call of YuyaoNiu/TileSpGEMM.  In the reference that
 * call is the CLI driver main_spgemm-col.cu:4821-5577, which loads a Matrix
 * Market file (mmio_allinone, mmio_highlevel.h:593-759), converts CSR to
 * 16x16 tiles on the host (main_spgemm-col.cu:4968-5360) and runs the timed
 * device pipeline stepall_cuda_new (main_spgemm-col.cu:4431-4819), which
 * discards C.  Here the whole path -- CSR in, tile conversion, tile symbolic,
 * per-tile masks, numeric, CSR out -- runs on the GPU behind one call.
 *
 * Conventions
 *   - Every entry point returns tsg_status (0 = success).  Nothing exits or
 *     traps.  tsg_last_error() gives a one-line description of the last
 *     failure on the calling thread.
 *   - A context (tsg_ctx) owns one CUDA stream and one stream-ordered memory
 *     pool on one device.  Calls on one context are not re-entrant; use one
 *     context per host thread.
 *   - Values are FP64, column indices int32, row pointers int32 or int64
 *     (tsg_csr.rowptr_bits).  C's row pointer is int64 whenever its nnz does
 *     not fit int32, or when the caller asks for 64 bits.
 */
#ifndef TILESPGEMM_H
#define TILESPGEMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TSG_OK = 0,
    TSG_ERR_INVALID_ARG = 1,     /* NULL pointer, bad enum, negative size */
    TSG_ERR_CUDA = 2,            /* a CUDA runtime call failed */
    TSG_ERR_OOM = 3,             /* device or pinned host allocation failed */
    TSG_ERR_INT32_OVERFLOW = 4,  /* result needs int64 row pointers but the caller asked for int32 */
    TSG_ERR_BAD_MTX = 5,         /* Matrix Market file could not be opened or parsed */
    TSG_ERR_DEVICE_TIMEOUT = 6,  /* a bounded device-side wait gave up */
    TSG_ERR_SHAPE = 7,           /* A.n != B.m, or A*A on a non-square A */
    TSG_ERR_BAD_INPUT = 8,       /* row pointer not monotone / out of range, or column out of range */
    TSG_ERR_NOT_SUPPORTED = 9,   /* input larger than the supported index ranges */
    TSG_ERR_BUDGET = 10          /* request does not fit the memory budget it was admitted under */
} tsg_status;

typedef enum {
    TSG_OP_AB = 0,   /* C = A * B */
    TSG_OP_AA = 1,   /* C = A * A   (A square; the reference's default, AAT == 0) */
    TSG_OP_AAT = 2   /* C = A * A^T (the reference's AAT == 1 build) */
} tsg_op;

typedef enum {
    TSG_MEM_HOST = 0,    /* pointers are host memory (pageable or pinned) */
    TSG_MEM_DEVICE = 1   /* pointers are device memory on the context's device */
} tsg_mem;

/*
 * A CSR matrix.  The reference's SMatrix (main_spgemm-col.cu:34-39) plus the
 * shape and the location of the arrays.
 *   row_ptr: m+1 entries, int32 or int64 per rowptr_bits (32 or 64)
 *   col:     nnz int32 column indices (any order inside a row; duplicates are
 *            summed like the reference's CPU path does)
 *   val:     nnz doubles
 * For outputs, set all pointers to NULL: the library allocates them (device
 * pool or pinned host memory, per `where`) and tsg_csr_free releases them.
 */
typedef struct {
    int32_t m, n;
    int64_t nnz;
    int32_t rowptr_bits;   /* 32 or 64 */
    int32_t where;         /* tsg_mem */
    void *row_ptr;
    int32_t *col;
    double *val;
    void *owner;           /* library bookkeeping for outputs; NULL for caller-owned input */
} tsg_csr;

/* Options; tsg_opts_default fills the defaults. */
typedef struct {
    int32_t validate;        /* check row pointers and column ranges (default 1) */
    int32_t phase_times;     /* record per-phase CUDA-event times into tsg_stats (default 0) */
    int32_t out_rowptr_bits; /* 32, 64, or 0 = 32 when it fits, else 64 (default 0) */
    int32_t dense_tile_min;  /* C tile-rows whose mean tile nnz is >= this use the dense
                                16x16 accumulator (default 160; 257 = never) */
    int32_t smem_acc_max;    /* largest C tile-row (in entries) accumulated in shared memory (default 24576) */
    int32_t threads_numeric; /* threads per CTA of the numeric kernels: 128, 256 or 512 (default 256) */
    int32_t row_acc_max;     /* tile-rows too large for one CTA: rows of up to this many entries accumulate in
                                shared memory (one CTA per row); longer rows -- and rows of 1,536+ entries with
                                96+ per entry of A's row -- accumulate in C's value array, eight warps per row
                                (default 65535) */
    int32_t numeric_walk;    /* 0 = auto; 1 = lanes over one B row per A entry; 2 = packed (lanes over the row's
                                flattened (A entry, B entry) pairs); 3 = as 1 with the next B row's loads issued
                                one A entry ahead in the tile-row kernels.  Auto packs only when a B row repeats
                                a column, and loads ahead when the mean row lengths put fewer than 3 products on
                                an entry of C. */
    int32_t rows_global;     /* 1: rows of tile-rows too large for one CTA that would accumulate in shared memory
                                (one warp each) accumulate in C's value array instead, one warp each (default 0) */
    int32_t row_warps;       /* warps per row for those shared-memory rows: 1, 2 or 4, each warp a column range
                                (default 4, measured fastest) */
    int32_t count_products;  /* 1: calls given a tsg_stats count the intermediate products (nnz_cub, one extra
                                pass over A); 0: nnz_cub is reported as 0 (default 1) */
    int32_t small_path;      /* 1: tsg_spgemm runs A*B and A*A whose every row of A meets at most 128 entries of B
                                (A and B of at most 4 M entries) row by row, one warp per row of C, instead of
                                the tiled pipeline -- the same C, values included; a repeated shape waits on the
                                device once per call; 0: always the tiled pipeline (default 1) */
} tsg_opts;

/* Per-call statistics.  Sizes are always filled; times only with phase_times. */
typedef struct {
    int64_t nnz_a, nnz_b, nnz_c;
    int64_t nnz_cub;           /* intermediate products, sum over A(i,k) of nnz(B row k) */
    int64_t tiles_a, tiles_b, tiles_c;
    double ms_total;           /* host wall time of the call */
    double ms_convert;         /* CSR -> tiles for A and B (and B = A^T for AAT) */
    double ms_step1;           /* tile-level symbolic: C tile structure */
    double ms_step2;           /* C tile masks, row counts, row pointer scan */
    double ms_step3;           /* numeric + CSR write */
    double ms_h2d, ms_d2h;     /* host <-> device copies (host operands only) */
    int32_t n_syncs;           /* host waits on the device inside the call */
    int32_t bins[4];           /* C tile-rows per numeric bin: empty, shared sparse, shared dense, per-row or global */
    int32_t small_path;        /* 1: the small-product path ran (tiles_*, bins and phase times are 0) */
} tsg_stats;

typedef struct tsg_ctx tsg_ctx;

/* ---- context ----------------------------------------------------------- */

/* Fill *o with the defaults listed in tsg_opts. */
void tsg_opts_default(tsg_opts *o);

/* Create a context on `device`; opts may be NULL (defaults).  Replaces the
 * reference's cudaSetDevice + per-run stream and cudaMalloc setup
 * (main_spgemm-col.cu:4856-4862, :4509-4512, spgemm_nsparse_kernel.h:45-90). */
tsg_status tsg_create(tsg_ctx **ctx, int device, const tsg_opts *opts);
tsg_status tsg_destroy(tsg_ctx *ctx);

/* Description of the last failure on this thread ("" if none). */
const char *tsg_last_error(void);

/* Library version string. */
const char *tsg_version(void);

/* Diagnostics (no counterpart in the reference).  tsg_launch_count: kernel
 * launches this library has issued in this process.  tsg_get_stream: the
 * context's cudaStream_t, for ordering caller work or recording CUDA events
 * around the library's kernels.  tsg_measure_fp64_peak: the device's FP64
 * FMA throughput in GFLOP/s (2 FLOP per FMA), measured by a short kernel. */
int64_t tsg_launch_count(void);
void *tsg_get_stream(tsg_ctx *ctx);

/* Order the context's stream after the work already queued on `stream` (a
 * cudaStream_t of the caller's, e.g. the one that wrote a device operand;
 * NULL = the legacy default stream), without blocking the host: the next
 * call's kernels start once that work is done.  No counterpart in the
 * reference (its operands are copied synchronously). */
tsg_status tsg_stream_wait(tsg_ctx *ctx, void *stream);

/* Bytes of pinned host memory the process-wide cache of host output buffers
 * keeps for reuse (no counterpart in the reference): min(96 GB, 3/8 of the
 * host's memory), or the environment variable TSG_PINNED_CACHE_BYTES read at
 * the first use (a decimal byte count, at most half the host's memory; 0
 * keeps nothing, so every host result is pinned afresh). */
int64_t tsg_pinned_cache_cap(void);
tsg_status tsg_measure_fp64_peak(tsg_ctx *ctx, double *gflops);

/* Failure detection, tested without a GPU fault (no counterpart in the
 * reference, which checks no CUDA return code, spins without bound in its
 * look-back scan, utils_cuda_scan.h:167-170, and exits on an unknown bin,
 * spgemm_nsparse_kernel.h:1299).
 *
 * tsg_inject_alloc_failure: the `countdown`-th allocation from now of the
 *   given kind fails as if memory were exhausted -- kind 0: device memory
 *   from a context's pool, kind 1: pinned host memory (host results and
 *   staging).  Process-wide; countdown 0 disarms it.  The call that meets the
 *   failure returns TSG_ERR_OOM, releases what it holds, and its context
 *   stays usable.  tsg_alloc_failure_pending: allocations still to go before
 *   the armed failure (0: none armed, or it has fired).
 * tsg_check_bounded_wait: runs the library's single-pass device scan over n
 *   ones with its look-back waits limited to spin_limit polls, set up so
 *   that the first tile's sum is never published (no CTA takes tile 0).  The waits for it give up, the kernel finishes, and the
 *   call returns TSG_ERR_DEVICE_TIMEOUT -- what every call returns when a
 *   bounded device wait gives up -- with the context still usable.  TSG_OK
 *   would mean a wait did not give up. */
tsg_status tsg_inject_alloc_failure(int32_t kind, int64_t countdown);
int64_t tsg_alloc_failure_pending(int32_t kind);
tsg_status tsg_check_bounded_wait(tsg_ctx *ctx, int64_t n, int32_t spin_limit);

/* ---- matrix market load path ------------------------------------------- */

/*
 * Load a Matrix Market coordinate file into a host CSR with the semantics of
 * the reference's mmio_allinone (mmio_highlevel.h:593-759): 1-based indices
 * become 0-based; symmetric and hermitian files are mirrored with the same
 * value (the diagonal once); skew-symmetric files are not mirrored; pattern
 * entries are 1.0; integer values are converted to double; complex files
 * keep the real part; entries are neither sorted nor merged (file order per
 * row).  *is_symmetric (may be NULL) is 1 for symmetric/hermitian files.
 * The arrays are malloc'd host memory with int32 row pointers (the
 * reference's int); release them with tsg_csr_free(NULL, out).
 * The reference returns -1 (open), -2 (banner) or -4 (size line); all three
 * map to TSG_ERR_BAD_MTX here, as do truncated data lines and 'array' files.
 */
tsg_status tsg_load_mtx(const char *path, tsg_csr *out, int32_t *is_symmetric);

/* The same load with the data lines parsed on the device (no counterpart in
 * the reference, whose mmio_allinone reads with fscanf): the file's bytes
 * go up, one thread per line parses it, and the entries (mirrored for
 * symmetric/hermitian files) are ordered into CSR on the device.  *A is a
 * device CSR (int32 row pointers) equal to tsg_load_mtx's result, entry
 * for entry; release it with tsg_csr_free(ctx, A).  Values the device does
 * not convert exactly (more than 19 significant digits or beyond 2^53,
 * decimal exponents outside [-22, 22], hex, inf, nan) and malformed lines
 * are read by the host's line reader; files whose entries do not sit one
 * per line are read by tsg_load_mtx and uploaded.  Errors as tsg_load_mtx. */
tsg_status tsg_load_mtx_device(tsg_ctx *ctx, const char *path, tsg_csr *A, int32_t *is_symmetric);

/* Write a host CSR (for example C) as a Matrix Market coordinate real
 * general file in the format of the reference's mm_write_mtx_crd
 * (mmio.h:780-850): 1-based "i j value" lines in CSR order, values as
 * "%20.16g"; exact != 0 writes 17 significant digits instead, so the file
 * loads back bit for bit. */
tsg_status tsg_write_mtx(const char *path, const tsg_csr *M, int32_t exact);

/* Release arrays that the library allocated into *m (C outputs or a loaded
 * matrix); a matrix whose owner is NULL belongs to the caller and is left
 * alone.  ctx may be NULL for host matrices from tsg_load_mtx.  Outputs of
 * one batched call share memory that is released with the last of them. */
tsg_status tsg_csr_free(tsg_ctx *ctx, tsg_csr *m);

/* ---- SpGEMM -------------------------------------------------------------- */

/*
 * C = op(A, B) on the context's device.  Replaces stepall_cuda_new
 * (main_spgemm-col.cu:4431-4819) together with the host tile conversion in
 * main (main_spgemm-col.cu:4968-5360) and adds the tile -> CSR output the
 * reference lacks.
 *   op == TSG_OP_AB : B must be given, A.n == B.m
 *   op == TSG_OP_AA : B ignored (may be NULL), A.m == A.n
 *   op == TSG_OP_AAT: B ignored (may be NULL)
 * A and B may live on host or device (independently).  C is allocated by the
 * library where C->where says (host: pinned memory; device: the context's
 * pool) and released with tsg_csr_free.  C's rows list columns in ascending
 * order, one entry per structural nonzero (an entry whose products cancel to
 * 0.0 is kept, as in the reference).  stats may be NULL.
 */
tsg_status tsg_spgemm(tsg_ctx *ctx, tsg_op op, const tsg_csr *A, const tsg_csr *B,
                      tsg_csr *C, tsg_stats *stats);

/* ---- batched products ------------------------------------------------------ */

/*
 * C[i] = op(A[i], B[i]) for i < count (B used for TSG_OP_AB only), computed
 * as ONE SpGEMM over the block-diagonal stacking of the instances: each
 * instance's rows and columns start on a multiple of 16, so no tile
 * straddles two instances and the tile-rows of the stack form an
 * (instance, tile-row) work list that one symbolic pass and one numeric
 * launch per bin cover.  Operands must be all host or all device memory;
 * C[0].where chooses where all outputs go.  C[i] are views into one
 * allocation; release each with tsg_csr_free (the memory goes with the last).
 * No counterpart in the reference, which runs one product per process.
 */
tsg_status tsg_spgemm_batched(tsg_ctx *ctx, tsg_op op, int32_t count, const tsg_csr *A, const tsg_csr *B,
                              tsg_csr *C, tsg_stats *stats);

/* ---- plans: symbolic once, numeric many times ----------------------------- */

/*
 * The reference recomputes everything for every product (stepall_cuda_new
 * runs its four steps per call, main_spgemm-col.cu:4529-4747).  A plan keeps
 * the result of the symbolic phase -- A's and B's structure, C's tile
 * structure, row masks, row pointer and numeric bins -- resident on the
 * device, so products that repeat a pattern with new values run only the
 * numeric step.
 *
 * tsg_plan_create: symbolic phase of op(A, B) (A's and B's values are not
 *   needed; device operands are copied, so the caller may free them).
 * tsg_plan_execute: C = op(A, B) with new values: valA holds A's nnz values
 *   in A's CSR order, valB B's (used for TSG_OP_AB only; for A*A and A*A^T
 *   B's values come from valA).  `where` says whether the value arrays are
 *   host or device memory.  C is returned like tsg_spgemm's.
 * tsg_plan_nnz: nnz of C.  tsg_plan_device_bytes: device memory the plan holds.
 */
typedef struct tsg_plan tsg_plan;
tsg_status tsg_plan_create(tsg_ctx *ctx, tsg_op op, const tsg_csr *A, const tsg_csr *B, tsg_plan **plan,
                           tsg_stats *stats);
tsg_status tsg_plan_execute(tsg_ctx *ctx, tsg_plan *plan, const double *valA, const double *valB, int32_t where,
                            tsg_csr *C, tsg_stats *stats);
int64_t tsg_plan_nnz(const tsg_plan *plan);
int64_t tsg_plan_device_bytes(const tsg_plan *plan);
tsg_status tsg_plan_destroy(tsg_ctx *ctx, tsg_plan *plan);

/*
 * Device-resident numeric step (no counterpart in the reference).
 *
 * tsg_plan_create_batched: the symbolic phase of `count` independent
 *   products op(A[i], B[i]), packed as in tsg_spgemm_batched; such a plan
 *   runs only through the calls below.  tsg_plan_count: its instance count
 *   (1 for a plain plan).
 * tsg_plan_set_values: new operand values into the plan's resident
 *   buffers: valA holds every instance's A values one after the other
 *   (instance i from a_offsets[i], tsg_plan_value_offsets), valB likewise
 *   for A*B.  Host arrays are copied before the call returns; device
 *   arrays are copied in stream order on the context's stream.
 * tsg_plan_replay: the numeric step on the resident values into the plan's
 *   resident C, launched as one CUDA graph (captured at the first replay;
 *   the first call must not itself be inside a stream capture).
 *   Asynchronous on the context's stream.
 * tsg_plan_result: waits for the stream and returns a device view of
 *   instance `instance` of the resident C (int64 row pointer; owner NULL:
 *   the memory stays the plan's until the next replay or its destruction).
 * tsg_plan_tune: the autotuner (no counterpart in the reference, whose bin
 *   thresholds are constants: main_spgemm-col.cu:26-29 and
 *   spgemm_nsparse_kernel.h:4-14).  On the resident values it times the
 *   numeric step's variants -- threads per tile-row CTA and row walk, then,
 *   with the best of those, the bin thresholds that choose each tile-row's
 *   accumulator (dense_tile_min, smem_acc_max, row_acc_max of tsg_opts; the
 *   plan's tile-rows are binned again for each candidate) -- and keeps the
 *   fastest for later replays; every variant gives the same bits.
 * tsg_plan_settings: the numeric settings and bin thresholds the plan runs
 *   with (the context's until tsg_plan_tune picks others); any pointer may
 *   be NULL.
 */
tsg_status tsg_plan_create_batched(tsg_ctx *ctx, tsg_op op, int32_t count, const tsg_csr *A, const tsg_csr *B,
                                   tsg_plan **plan, tsg_stats *stats);
int32_t tsg_plan_count(const tsg_plan *plan);
tsg_status tsg_plan_value_offsets(const tsg_plan *plan, int64_t *a_offsets, int64_t *b_offsets);
tsg_status tsg_plan_set_values(tsg_ctx *ctx, tsg_plan *plan, const double *valA, const double *valB, int32_t where);
tsg_status tsg_plan_replay(tsg_ctx *ctx, tsg_plan *plan);
tsg_status tsg_plan_result(tsg_ctx *ctx, tsg_plan *plan, int32_t instance, tsg_csr *C);
tsg_status tsg_plan_tune(tsg_ctx *ctx, tsg_plan *plan, double *best_ms);
tsg_status tsg_plan_settings(const tsg_plan *plan, int32_t *threads, int32_t *walk, int32_t *dense_tile_min,
                             int32_t *smem_acc_max, int32_t *row_acc_max);

/* ---- serving: continuous batching of requests ------------------------------ */

/*
 * A request loop on one GPU (no counterpart in the reference).  Requests are
 * admitted while the device memory they may need fits budget_bytes (operands
 * plus an upper bound of C from the intermediate-product count); `workers`
 * slots, each with its own CUDA stream and memory pool, run admitted
 * requests concurrently, taking up to max_batch at a time.  A request with a
 * nonzero pattern_key keeps its symbolic result (a plan) in its worker's
 * cache (plan_cache_bytes, least recently used first out): a later request
 * with the same key and new values runs only the numeric step (a request
 * whose op, shapes, row pointers or sampled column indices differ from the
 * key's plan rebuilds it, so a reused key never runs another pattern's
 * numeric step on these checks).  Keyless requests of one op taken together
 * run as one batched product.
 * Operands are host memory and must stay valid until tsg_server_wait returns
 * the request.  Results are host CSRs (pinned); release them with
 * tsg_csr_free before destroying the server.
 */
typedef struct {
    int32_t device;
    int32_t workers;           /* concurrent slots (default 4) */
    int32_t max_batch;         /* requests a slot takes at once (default 32) */
    int64_t budget_bytes;      /* device memory admission budget (default 64 GiB) */
    int64_t plan_cache_bytes;  /* per-slot plan cache for numeric-only repeats (default 8 GiB) */
} tsg_server_opts;

typedef struct {
    double latency_ms;         /* submit -> result */
    double queue_ms;           /* submit -> taken by a slot */
    double run_ms;             /* taken -> result (the slot's whole group) */
    int32_t numeric_only;      /* 1 when a cached plan skipped the symbolic steps */
    int32_t batched_with;      /* requests computed in the same batched product */
    int32_t worker;            /* slot that ran it */
} tsg_server_result;

typedef struct tsg_server tsg_server;
void tsg_server_opts_default(tsg_server_opts *o);
tsg_status tsg_server_create(const tsg_server_opts *opts, tsg_server **server);
/* TSG_ERR_BUDGET: the request alone exceeds the budget. */
tsg_status tsg_server_submit(tsg_server *server, tsg_op op, const tsg_csr *A, const tsg_csr *B, uint64_t pattern_key,
                             int64_t *request_id);
/* Blocks until the request is done; C receives the result.  Submit and the
 * waits may be called from several threads; each request is returned once:
 * waiting for a request another thread is already waiting for returns
 * TSG_ERR_INVALID_ARG. */
tsg_status tsg_server_wait(tsg_server *server, int64_t request_id, tsg_csr *C, tsg_server_result *info);
/* Any completed request, in completion order (its id in *request_id): a
 * collector that frees results as they finish holds at most the requests in
 * flight.  Requests a tsg_server_wait is waiting for are left to it.
 * TSG_ERR_INVALID_ARG when no request is outstanding. */
tsg_status tsg_server_wait_any(tsg_server *server, int64_t *request_id, tsg_csr *C, tsg_server_result *info);
tsg_status tsg_server_destroy(tsg_server *server);

/* ---- tile form (the reference's device format) --------------------------- */

/*
 * C in the reference's 16x16 tile format, as stepall_cuda_new leaves it on the
 * device (main_spgemm-col.cu:4567-4658): tile-row pointer, sorted tile
 * columns, per-tile nnz prefix, 16 uint8 row starts per tile, uint8 local
 * columns, FP64 values and 16 uint16 row masks (bit 15-c for local column c).
 * The tile list includes tiles whose element-level product is empty (nnz 0,
 * mask 0, row starts 0), as the reference's does.  Arrays are device memory
 * from the context's pool; free with tsg_tiles_free.
 */
typedef struct {
    int32_t m, n;            /* shape of the matrix */
    int32_t blkm, blkn;      /* ceil(m/16), ceil(n/16) */
    int64_t numblk;          /* number of tiles */
    int64_t nnz;
    int64_t *blkrowptr;      /* blkm+1 */
    int32_t *blkcolidx;      /* numblk */
    int64_t *nnzb;           /* numblk+1, exclusive prefix of per-tile nnz */
    uint8_t *ptr;            /* 16*numblk */
    uint8_t *col;            /* nnz, local column */
    double *val;             /* nnz */
    uint16_t *mask;          /* 16*numblk */
    void *owner;
} tsg_tiles;

/* A CSR matrix (any location) -> tile form on the device, in the layout of
 * the reference's host conversion for A (main_spgemm-col.cu:4968-5240). */
tsg_status tsg_csr_to_tiles(tsg_ctx *ctx, const tsg_csr *A, tsg_tiles *T);

/* C = op(A, B) returned in tile form (the reference's stepall_cuda_new output). */
tsg_status tsg_spgemm_tiles(tsg_ctx *ctx, tsg_op op, const tsg_csr *A, const tsg_csr *B,
                            tsg_tiles *C, tsg_stats *stats);

/* Tile form -> CSR (device), the tile -> CSR output step. */
tsg_status tsg_tiles_to_csr(tsg_ctx *ctx, const tsg_tiles *T, tsg_csr *C);

/* Largest row count tsg_tiles_to_csr_noalloc accepts (its static scratch is
 * about 4 MiB per device). */
#define TSG_NOALLOC_MAX_ROWS 1048576

/* tsg_tiles_to_csr for callers that cannot allocate: no counterpart in the
 * reference.  T is device tile form (from tsg_csr_to_tiles or
 * tsg_spgemm_tiles); row_ptr (m+1 int64), col and val (T->nnz each) are
 * caller-provided device memory of ctx's device (device memory of another
 * GPU is refused with TSG_ERR_INVALID_ARG), and the result is the one
 * tsg_tiles_to_csr gives.  The call allocates no device or pinned memory: its
 * scratch (row counts, scan look-back state, error flags) is one static
 * device array, cleared at the start of every call.  T->m above
 * TSG_NOALLOC_MAX_ROWS is refused with TSG_ERR_NOT_SUPPORTED.  The first call
 * on a device after a context is created there looks up the array's address
 * (cudaGetSymbolAddress; a device reset can move the array, and contexts do
 * not survive one); make that call before any stream capture.  All contexts
 * of a device share the array, so
 * calls that overlap in time (other threads or streams) race: serialize them.
 * Returns after the result is complete (it waits on ctx's stream). */
tsg_status tsg_tiles_to_csr_noalloc(tsg_ctx *ctx, const tsg_tiles *T, int64_t *row_ptr, int32_t *col,
                                    double *val);

tsg_status tsg_tiles_free(tsg_ctx *ctx, tsg_tiles *T);

/* y = T x on the tile form, without going back to CSR (the reference's
 * tile-format consumer, the CCSB SpMV of ccsb_spmv.h:11-252).  x (T->n) and
 * y (T->m) are device memory; waits for the result. */
tsg_status tsg_tiles_spmv(tsg_ctx *ctx, const tsg_tiles *T, const double *x, double *y);

/* Copy a tile matrix's arrays to caller-provided host buffers (sizes from T). */
tsg_status tsg_tiles_download(tsg_ctx *ctx, const tsg_tiles *T, int64_t *blkrowptr, int32_t *blkcolidx,
                              int64_t *nnzb, uint8_t *ptr, uint8_t *col, double *val, uint16_t *mask);

/* Copy a CSR's arrays (any location) to caller-provided host buffers.
 * row_ptr receives int64 values whatever the source width. */
tsg_status tsg_csr_download(tsg_ctx *ctx, const tsg_csr *M, int64_t *row_ptr, int32_t *col, double *val);

/* Copy a CSR (host or device, either row-pointer width) into device memory
 * of the context's device that the library owns (tsg_csr_free releases
 * it), so that one operand can be multiplied many times without the
 * upload.  The reference's driver does the same: its 20 timed runs start
 * from tile arrays already on the device (main_spgemm-col.cu:4448-4503). */
tsg_status tsg_csr_to_device(tsg_ctx *ctx, const tsg_csr *H, tsg_csr *D);

/* Rows [r0, r1) of a CSR (any location) into caller-provided host buffers,
 * for checking or exporting part of a result too large to bring back whole
 * (no counterpart in the reference, which discards C).  row_ptr receives the
 * r1 - r0 + 1 row pointers of those rows as int64, as they are in M
 * (offsets into M's entries); col and val (either may be NULL: then only
 * the row pointers are copied) receive the entries
 * [row_ptr[0], row_ptr[r1 - r0]) of M. */
tsg_status tsg_csr_download_rows(tsg_ctx *ctx, const tsg_csr *M, int32_t r0, int32_t r1, int64_t *row_ptr,
                                 int32_t *col, double *val);

#ifdef __cplusplus
}
#endif

#endif /* TILESPGEMM_H */
