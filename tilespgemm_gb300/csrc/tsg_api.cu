// tsg_api.cu -- the C ABI (include/tilespgemm.h): contexts, memory, and the
// device pipeline CSR -> tiles -> step 1 -> step 2 -> step 3 -> CSR.
//
// The reference's timed pipeline (stepall_cuda_new, main_spgemm-col.cu:4431-4819)
// does about 20 cudaMalloc/cudaFree calls, creates streams and makes about 8
// blocking device->host copies per SpGEMM.  Here a call makes two host waits
// (after step 1 for C's tile count, after step 2 for C's nnz; both copies
// also carry the bin sizes and the device error flags), allocates from a
// stream-ordered pool that keeps its memory cached, and runs everything on
// one stream.
#include "tilespgemm.h"
#include "tsg_internal.cuh"
#include "tsg_mtx.h"
#include "tsg_numeric.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>
#include <mutex>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

namespace tsg {
cudaError_t tiles_init_attributes();
cudaError_t prepare_csr(Pool &pool, const void *rp, int rp_bits, const int *col, int m, int n, long long nnz,
                        long long *rp_out, int *flags, bool check_cols);
cudaError_t csr_to_tile_structure(Pool &pool, const long long *rp, const int *col, TileCSR &T, bool masks,
                                  int *flags, int *stat_max);
cudaError_t tile_symbolic(Pool &pool, const TileCSR &A, const TileCSR &B, long long *crp, int *ccol, int *cnt,
                          int *wide, int *flags, int *stat, bool count_pass, int *defer, unsigned *wbm, long long wpr);
cudaError_t csr_transpose(Pool &pool, const long long *rp, const int *col, const double *val, int m, int n,
                          long long nnz, long long *tp, int *tcol, double *tval, int *perm, int *flags);
cudaError_t aux_gather(Pool &pool, const int *perm, const double *src, double *dst, long long n);
cudaError_t aux_nnzcub(Pool &pool, const long long *rpA, const int *colA, int m, const long long *rpB, int kB,
                       unsigned long long *out);
cudaError_t aux_mask_popc(Pool &pool, const int *trp, int blkm, const uint16_t *mask, unsigned long long *out);
cudaError_t aux_rows_increasing(Pool &pool, const long long *rp, const int *col, int m, long long nnz,
                                unsigned long long *out);
cudaError_t aux_copy_scalars(Pool &pool, const long long *a, long long *da, const int *b, long long *db,
                             const int *c, long long *dc);
cudaError_t aux_rowptr_narrow(Pool &pool, const long long *in, int *out, long long n);
// the device Matrix Market reader (tsg_mtx_dev.cu)
cudaError_t mtx_lines(Pool &pool, const char *text, long long n, long long *&ends, long long &lines, int *flags);
cudaError_t mtx_parse(Pool &pool, const char *text, const long long *ends, long long lines, int kind, long long M,
                      long long N, unsigned char *st, int *lri, int *lci, double *lvv);
cudaError_t mtx_number_entries(Pool &pool, const unsigned char *st, long long lines, long long *tpos, int *flags);
cudaError_t mtx_take(Pool &pool, const unsigned char *st, const long long *tpos, long long lines, long long NZ,
                     long long M, bool symm, const int *lri, const int *lci, const double *lvv, int *ri, int *ci,
                     double *vv, unsigned long long *hn, long long *ht, long long *hl, int *bad);
cudaError_t mtx_patch(Pool &pool, long long n, const long long *ht, const int *hi, const int *hj, const double *hv,
                      int *ri, int *ci, double *vv);
cudaError_t mtx_emit(Pool &pool, const int *ri, const int *ci, long long NZ, bool symm, int *cnt, long long *eoff,
                     int *flags);
cudaError_t mtx_emit_fill(Pool &pool, const int *ri, const int *ci, const double *vv, long long NZ, bool symm,
                          const long long *eoff, int *key, int *col, double *val);
cudaError_t gather_i32(Pool &pool, const int *perm, const int *src, int *dst, long long n);
cudaError_t mtx_host_spans(Pool &pool, long long n, const long long *hl, const long long *ends, long long *span);
cudaError_t tiles_from_csr_c(Pool &pool, int m, int blkm, long long numblk, const long long *crp, const int *ccol,
                             const uint16_t *cmask, const long long *rowptr, const int *col, const double *val,
                             long long *nnzb, uint8_t *ptr, uint8_t *lcol, double *tval, int *flags);
cudaError_t tiles_payload_a(Pool &pool, int m, int n, const long long *rp, const int *col, const double *val,
                            const TileCSR &T, long long numblk, long long *nnzb, uint8_t *ptr, uint8_t *lcol,
                            double *tval, int *flags);
cudaError_t fp64_peak(cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, double *gflops);
cudaError_t csr_from_tiles(Pool &pool, int m, const long long *brp, const int *bcol, const long long *nnzb,
                           const uint8_t *ptr, const uint8_t *lcol, const double *tval, long long *rowptr, int *col,
                           double *val, int *flags, bool fill);
cudaError_t csr_rowcnt_from_tiles(cudaStream_t s, int m, const long long *brp, const long long *nnzb,
                                  const uint8_t *ptr, int *rowcnt);
cudaError_t csr_fill_from_tiles(cudaStream_t s, int m, const long long *brp, const int *bcol, const long long *nnzb,
                                const uint8_t *ptr, const uint8_t *lcol, const double *tval, const long long *rowptr,
                                int *col, double *val);
long long scan_status_words(long long n);
cudaError_t scan_unpublished_tile(Pool &pool, long long n, int spin_limit, int *flags);
cudaError_t tiles_spmv(cudaStream_t s, int m, int blkm, const long long *brp, const int *bcol, const long long *nnzb,
                       const uint8_t *ptr, const uint8_t *lcol, const double *tval, const double *x, int n, double *y);
cudaError_t scan_i32_to_i64_in(cudaStream_t s, const int *in, long long *out, long long n, int *flags,
                               unsigned *ticket, unsigned long long *status);
}  // namespace tsg

using namespace tsg;

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};

void tsg::count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// armed allocation failures per kind: the allocation that takes the count
// from 1 to 0 fails; 0 (or below) = disarmed
static std::atomic<long long> g_fail_alloc[2];

bool tsg::alloc_should_fail(int kind)
{
    std::atomic<long long> &c = g_fail_alloc[kind & 1];
    if (c.load(std::memory_order_relaxed) <= 0) return false;
    return c.fetch_sub(1, std::memory_order_relaxed) == 1;
}

namespace tsg {
void set_last_error(const char *msg) { g_err = msg; }
void noalloc_forget(int device);
void *make_malloc_owner(void *a, void *b, void *c);
}

static tsg_status fail(tsg_status st, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
static tsg_status fail(tsg_status st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

// status of a failed CUDA call: out of memory is TSG_ERR_OOM, the rest TSG_ERR_CUDA
static inline tsg_status cuda_status(cudaError_t e) { return e == cudaErrorMemoryAllocation ? TSG_ERR_OOM : TSG_ERR_CUDA; }

#define CUDA_OK(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            return fail(e_ == cudaErrorMemoryAllocation ? TSG_ERR_OOM : TSG_ERR_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                            \
        }                                                                                              \
    } while (0)

// A product shape the small-product path has seen on a context: the next
// call of that shape sizes C's buffers from nnzc and waits on the device
// only at the end; small = false: its rows exceed the path's limit (the
// tiled path takes it without trying).
struct SmallShape {
    int op = 0, m = 0, k = 0, n = 0;
    long long nnz_a = 0, nnz_b = 0, nnzc = 0;
    bool small = true;
    bool one_round = false;        // every row of the last call fit one warp round (32 products)
    long long *rowptr = nullptr;   // C's row pointer of the last call (device, m+1; the context's pool)
};

struct tsg_ctx {
    int device = 0;
    tsg_opts opts{};
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    int *dflags = nullptr;           // FLAG_COUNT ints, inside dstat (slots ST_HFLAGS on)
    long long *dstat = nullptr;      // 64 slots
    long long *hstat = nullptr;      // pinned mirror: 64 stat slots + FLAG_COUNT flags (as long long)
    std::mutex mu;
    cudaEvent_t ev[8] = {};
    bool counted = false;            // entered in the pinned cache's count of live contexts
    cudaStream_t side = nullptr;     // second stream for kernels that overlap the main one's (fork/join by events)
    cudaEvent_t fork = nullptr, join = nullptr;
    // host-link copies beside the kernels: operand values up during the
    // symbolic phase, C's row pointers and column indices down during the
    // numeric step
    cudaStream_t copy = nullptr;
    cudaEvent_t cfork = nullptr, vals_ev = nullptr, cols_ev = nullptr, copy_done = nullptr;
    cudaEvent_t ext_ev = nullptr;            // tsg_stream_wait: the caller's stream's point to wait for
    std::vector<SmallShape> small_shapes;   // the last SMALL_SHAPES shapes, newest last
};

namespace {

enum StatSlot {
    ST_NUMBLKC = 0, ST_MAXS = 1, ST_TILESA = 2, ST_TILESB = 3, ST_NNZCUB = 4, ST_POPCB = 5, ST_NNZC = 6,
    ST_NDEFER = 7,               // tile-rows left to the CTA step-2 kernel
    ST_BINS = 8,                 // step 2's bin statistics, BS_SLOTS slots (tsg_numeric.cuh)
    ST_BUNSORTED = 36,           // B rows whose columns are not strictly increasing
    ST_SMALL = 37,               // small-product path: rows over its limit, products, a row past one round (3 slots)
    ST_HFLAGS = 40,              // device: the flags (FLAG_COUNT ints); host: their mirror as int64
    ST_SLOTS = 64
};

// Owner of library-allocated arrays handed to a caller (tsg_csr.owner).
// Batched outputs share one owner; it is released when its last view is.
struct OutOwner {
    int where = TSG_MEM_DEVICE;   // TSG_MEM_DEVICE: pool memory; TSG_MEM_HOST: pinned; OWN_MALLOC: malloc
    tsg_ctx *ctx = nullptr;
    // views still alive; batched results are freed from several threads, so
    // the last decrement (and only it) releases the blocks
    std::atomic<int> refs{1};
    std::vector<std::pair<void *, size_t>> blocks;
};
constexpr int OWN_MALLOC = 2;

// Pinned host buffers (host outputs, staging) kept for reuse by all
// contexts of the process: pinning fresh pages runs at about 13 GB/s on the
// Grace host against ~190 GB/s for the copy itself, so a served stream of
// large outputs is bound by pinning unless buffers come back.  At most
// pinned_cap() bytes are kept (the largest are freed beyond it); the cache
// is emptied when the last context is destroyed.
struct PinnedCache {
    std::mutex mu;
    std::multimap<size_t, void *> bufs;           // kept buffers by their allocated size
    std::unordered_map<void *, size_t> size_of;   // allocated size of every buffer handed out or kept
    size_t bytes = 0;
    int live_contexts = 0;
};

PinnedCache &pinned_cache()
{
    static PinnedCache c;
    return c;
}

// min(96 GB, 3/8 of the host's memory), or the environment's
// TSG_PINNED_CACHE_BYTES (a decimal byte count, at most half the host's
// memory; 0 keeps nothing).  On the served stream (4 workers, outputs up to
// ~15 GB) a quarter of a 199 GB host gave 28-33 requests/s, 3/8 of it 37-39.
size_t pinned_cap()
{
    static const size_t cap = [] {
        const long pages = sysconf(_SC_PHYS_PAGES), psz = sysconf(_SC_PAGE_SIZE);
        const size_t ram = (pages > 0 && psz > 0) ? (size_t)pages * (size_t)psz : (size_t)16 << 30;
        if (const char *env = getenv("TSG_PINNED_CACHE_BYTES")) {
            char *end = nullptr;
            const long long v = strtoll(env, &end, 10);
            if (end != env && *end == '\0' && v >= 0) return std::min<size_t>((size_t)v, ram / 2);
        }
        return std::min<size_t>((size_t)96 << 30, ram / 8 * 3);
    }();
    return cap;
}

void *pinned_get(tsg_ctx *ctx, size_t bytes)
{
    (void)ctx;
    if (bytes == 0) bytes = 16;
    if (alloc_should_fail(1)) return nullptr;
    PinnedCache &pc = pinned_cache();
    {
        std::lock_guard<std::mutex> lk(pc.mu);
        // the smallest kept buffer that holds the request, up to twice its
        // size (on the served stream a 1.25x bound gave 22 requests/s, 2x 27)
        auto it = pc.bufs.lower_bound(bytes);
        if (it != pc.bufs.end() && it->first <= 2 * bytes + (16 << 20)) {
            void *p = it->second;
            pc.bytes -= it->first;
            pc.bufs.erase(it);
            return p;
        }
    }
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    std::lock_guard<std::mutex> lk(pc.mu);
    pc.size_of[p] = bytes;
    return p;
}

void pinned_put(tsg_ctx *ctx, void *p, size_t bytes)
{
    (void)ctx;
    if (bytes == 0) bytes = 16;
    PinnedCache &pc = pinned_cache();
    std::vector<void *> drop;
    {
        std::lock_guard<std::mutex> lk(pc.mu);
        auto sz = pc.size_of.find(p);
        if (sz != pc.size_of.end()) bytes = sz->second;   // the allocated size (a reused buffer may be larger)
        if (pc.live_contexts <= 0) {   // freed after the last context: nothing left to reuse it
            drop.push_back(p);
            p = nullptr;
        } else {
            pc.bufs.emplace(bytes, p);
            pc.bytes += bytes;
        }
        while (pc.bytes > pinned_cap() && !pc.bufs.empty()) {
            auto last = std::prev(pc.bufs.end());
            pc.bytes -= last->first;
            drop.push_back(last->second);
            pc.bufs.erase(last);
        }
        for (void *q : drop) pc.size_of.erase(q);
    }
    for (void *q : drop) cudaFreeHost(q);
}

void pinned_context_enter()
{
    PinnedCache &pc = pinned_cache();
    std::lock_guard<std::mutex> lk(pc.mu);
    ++pc.live_contexts;
}

void pinned_context_leave()
{
    PinnedCache &pc = pinned_cache();
    std::vector<void *> drop;
    {
        std::lock_guard<std::mutex> lk(pc.mu);
        if (--pc.live_contexts > 0) return;
        for (auto &kv : pc.bufs) { drop.push_back(kv.second); pc.size_of.erase(kv.second); }
        pc.bufs.clear();
        pc.bytes = 0;
    }
    for (void *q : drop) cudaFreeHost(q);
}

// device-side view of a CSR operand (after upload and preparation)
struct DevCSR {
    int m = 0, n = 0;
    long long nnz = 0;
    long long *rp = nullptr;   // int64, clamped
    const int *col = nullptr;
    const double *val = nullptr;
};

// Everything one call allocates from the pool; released together.
struct Scratch {
    Pool &pool;
    std::vector<void *> ptrs;
    explicit Scratch(Pool &p) : pool(p) {}
    template <class T> T *get(long long n) {
        T *p = pool.alloc_n<T>(n);
        if (p) ptrs.push_back(p);
        return p;
    }
    ~Scratch() { for (void *p : ptrs) pool.free(p); }
};

tsg_status check_csr(const tsg_csr *M, const char *name)
{
    if (!M) return fail(TSG_ERR_INVALID_ARG, "%s is NULL", name);
    if (M->m < 0 || M->n < 0 || M->nnz < 0) return fail(TSG_ERR_INVALID_ARG, "%s has a negative size", name);
    if (M->rowptr_bits != 32 && M->rowptr_bits != 64) return fail(TSG_ERR_INVALID_ARG, "%s.rowptr_bits must be 32 or 64", name);
    if (M->where != TSG_MEM_HOST && M->where != TSG_MEM_DEVICE) return fail(TSG_ERR_INVALID_ARG, "%s.where is not a tsg_mem", name);
    if (!M->row_ptr) return fail(TSG_ERR_INVALID_ARG, "%s.row_ptr is NULL", name);
    if (M->nnz > 0 && (!M->col || !M->val)) return fail(TSG_ERR_INVALID_ARG, "%s.col/val is NULL", name);
    if (M->nnz >= (1ll << 31)) return fail(TSG_ERR_NOT_SUPPORTED, "%s has %lld entries; operands are limited to 2^31-1", name, (long long)M->nnz);
    if (M->m > (1 << 30) || M->n > (1 << 30)) return fail(TSG_ERR_NOT_SUPPORTED, "%s is larger than 2^30 rows or columns", name);
    return TSG_OK;
}

// Upload (if on the host) and prepare one operand.
tsg_status stage_operand(tsg_ctx *ctx, Pool &pool, Scratch &sc, const tsg_csr *M, bool validate, DevCSR &D)
{
    D.m = M->m; D.n = M->n; D.nnz = M->nnz;
    const void *rp = M->row_ptr;
    const int *col = M->col;
    const double *val = M->val;
    const size_t rpb = (size_t)(M->m + 1) * (M->rowptr_bits == 64 ? 8 : 4);
    if (M->where == TSG_MEM_HOST) {
        void *drp = sc.get<char>((long long)rpb);
        int *dcol = sc.get<int>(M->nnz);
        double *dval = sc.get<double>(M->nnz);
        if (!drp || !dcol || !dval) return fail(TSG_ERR_OOM, "device pool allocation failed for an operand");
        CUDA_OK(cudaMemcpyAsync(drp, rp, rpb, cudaMemcpyHostToDevice, ctx->stream));
        if (M->nnz > 0) {
            CUDA_OK(cudaMemcpyAsync(dcol, col, sizeof(int) * (size_t)M->nnz, cudaMemcpyHostToDevice, ctx->stream));
            CUDA_OK(cudaMemcpyAsync(dval, val, sizeof(double) * (size_t)M->nnz, cudaMemcpyHostToDevice, ctx->stream));
        }
        rp = drp; col = dcol; val = dval;
    }
    D.rp = sc.get<long long>(M->m + 1);
    if (!D.rp) return fail(TSG_ERR_OOM, "device pool allocation failed");
    CUDA_OK(prepare_csr(pool, rp, M->rowptr_bits, col, M->m, M->n, M->nnz, D.rp, ctx->dflags, validate));
    D.col = col; D.val = val;
    return TSG_OK;
}

tsg_status build_tiles(Pool &pool, Scratch &sc, const DevCSR &D, TileCSR &T, tsg_ctx *ctx)
{
    T.m = D.m; T.n = D.n;
    T.blkm = ceil_div_i(D.m, TILE);
    T.blkn = ceil_div_i(D.n, TILE);
    long long cap = D.nnz;
    if ((long long)T.blkm * T.blkn < cap) cap = (long long)T.blkm * T.blkn;
    T.cap = cap;
    T.trp = sc.get<int>(T.blkm + 1);
    T.tcol = sc.get<int>(cap);
    T.mask = sc.get<uint16_t>(cap * TILE + 2);
    if (!T.trp || !T.tcol || !T.mask) return fail(TSG_ERR_OOM, "device pool allocation failed for tiles");
    CUDA_OK(csr_to_tile_structure(pool, D.rp, D.col, T, true, ctx->dflags, nullptr));
    return TSG_OK;
}

tsg_status read_flags(tsg_ctx *ctx)
{
    long long *hf = ctx->hstat + ST_HFLAGS;
    if (hf[FLAG_BAD_INPUT]) return fail(TSG_ERR_BAD_INPUT, "row pointer not monotone/in range or column index out of range");
    if (hf[FLAG_TIMEOUT]) return fail(TSG_ERR_DEVICE_TIMEOUT, "a bounded device wait gave up");
    if (hf[FLAG_OVERFLOW]) return fail(TSG_ERR_NOT_SUPPORTED, "an index count overflowed its type");
    if (hf[FLAG_INTERNAL]) return fail(TSG_ERR_CUDA, "internal bound check failed on the device");
    return TSG_OK;
}

// device -> pinned mirror of stats and flags, then wait
tsg_status host_wait(tsg_ctx *ctx, int *nsync)
{
    // the statistics and, behind them, the flags: one copy
    CUDA_OK(cudaMemcpyAsync(ctx->hstat, ctx->dstat, sizeof(long long) * ST_HFLAGS + sizeof(int) * FLAG_COUNT,
                            cudaMemcpyDeviceToHost, ctx->stream));
    static_assert(FLAG_COUNT <= ST_SLOTS - ST_HFLAGS, "flag mirror");
    static_assert(ST_BINS + BS_SLOTS <= ST_BUNSORTED && ST_BUNSORTED < ST_SMALL && ST_SMALL + 3 <= ST_HFLAGS,
                  "statistics slots");
    int hflags[FLAG_COUNT];
    CUDA_OK(cudaStreamSynchronize(ctx->stream));
    memcpy(hflags, ctx->hstat + ST_HFLAGS, sizeof(hflags));
    for (int f = 0; f < FLAG_COUNT; ++f) ctx->hstat[ST_HFLAGS + f] = hflags[f];
    if (nsync) ++*nsync;
    return read_flags(ctx);
}

double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

struct PhaseTimer {
    tsg_ctx *ctx;
    bool on;
    int n = 0;
    PhaseTimer(tsg_ctx *c, bool enable) : ctx(c), on(enable) {}
    void mark() { if (on && n < 8) cudaEventRecord(ctx->ev[n++], ctx->stream); }
};

// Everything the numeric step needs for one op(A, B), produced by the
// symbolic phase (conversion + steps 1-2).  A plan (tsg_plan) keeps one alive;
// tsg_spgemm builds one, runs the numeric step once and drops it.
struct PlanData {
    tsg_op op = TSG_OP_AA;
    int m = 0, k = 0, n = 0, blkm = 0;
    long long nnzA = 0, nnzB = 0, numblkC = 0, nnzC = 0, nnzcub = 0, tilesA = 0, tilesB = 0;
    long long *rpA = nullptr, *rpB = nullptr;      // int64 row pointers
    const int *colA = nullptr, *colB = nullptr;
    const double *valA = nullptr, *valB = nullptr; // values of the operands as staged
    double *valA_buf = nullptr, *valB_buf = nullptr; // plan-owned value buffers for later executions
    int *perm = nullptr;                           // A*A^T: B's entry q is A's entry perm[q]
    long long *crp = nullptr;
    int *ccol = nullptr;
    uint16_t *cmask = nullptr;
    long long *rowptrC = nullptr;
    unsigned char *bin = nullptr;
    int *binlist = nullptr;                        // tile-rows of each bin, NBIN * blkm
    long long bstat[BS_SLOTS] = {};                // step 2's bin statistics (counts, shared-memory sizes)
    int *rowlist = nullptr;                        // rows of each row class, NROWCLS * m
    bool dupsafe = false;
    bool b_increasing = true;                      // every B row's columns strictly increase
    int nsync = 0;
    cudaEvent_t vals_ev = nullptr;                 // set while operand values are still on their way up (copy stream)
    std::vector<void *> owned;
    // the main stream waits for the values' upload (before their first use,
    // and before any buffer of the plan is freed)
    void wait_values(cudaStream_t s) {
        if (vals_ev) { cudaStreamWaitEvent(s, vals_ev, 0); vals_ev = nullptr; }
    }
    template <class T> T *own(Pool &pool, long long n) {
        T *p = pool.alloc_n<T>(n);
        if (p) owned.push_back(p);
        return p;
    }
    void disown(void *p) {
        for (auto &q : owned) if (q == p) q = nullptr;
    }
    void release(Pool &pool) {
        wait_values(pool.stream);
        for (void *p : owned) pool.free(p);
        owned.clear();
    }
    long long device_bytes() const {
        return 8ll * (m + 1) * 2 + 4ll * (nnzA + nnzB) + 8ll * (nnzA + nnzB) + 8ll * (blkm + 1) +
               36ll * numblkC + 8ll * (m + 1) + 4ll * NBIN * blkm + 4ll * NROWCLS * m;
    }
};

tsg_status check_op(tsg_op op, const tsg_csr *A, const tsg_csr *B)
{
    tsg_status r = check_csr(A, "A");
    if (r) return r;
    if (op == TSG_OP_AB) {
        r = check_csr(B, "B");
        if (r) return r;
        if (A->n != B->m) return fail(TSG_ERR_SHAPE, "A is %d x %d but B is %d x %d", A->m, A->n, B->m, B->n);
    } else if (op == TSG_OP_AA) {
        if (A->m != A->n) return fail(TSG_ERR_SHAPE, "A*A needs a square A (got %d x %d)", A->m, A->n);
    } else if (op != TSG_OP_AAT) {
        return fail(TSG_ERR_INVALID_ARG, "unknown op %d", (int)op);
    }
    return TSG_OK;
}

// Stage one operand into the plan: row pointer (int64, validated), columns
// and values on the device.  Device operands are used in place unless
// `copy` (a plan must not keep the caller's device buffers).
tsg_status stage_into_plan(tsg_ctx *ctx, Pool &pool, PlanData &P, const tsg_csr *M, bool validate, bool copy,
                           long long *&rp64, const int *&col, const double *&val, double *&valbuf)
{
    const size_t rpb = (size_t)(M->m + 1) * (M->rowptr_bits == 64 ? 8 : 4);
    const void *rp = M->row_ptr;
    const int *c = M->col;
    const double *v = M->val;
    valbuf = nullptr;
    if (M->where == TSG_MEM_HOST || copy) {
        const cudaMemcpyKind kind = M->where == TSG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
        void *drp = P.own<char>(pool, (long long)rpb);
        int *dcol = P.own<int>(pool, M->nnz);
        double *dval = P.own<double>(pool, M->nnz);
        if (!drp || !dcol || !dval) return fail(TSG_ERR_OOM, "device pool allocation failed for an operand");
        CUDA_OK(cudaMemcpyAsync(drp, rp, rpb, kind, ctx->stream));
        if (M->nnz > 0) {
            CUDA_OK(cudaMemcpyAsync(dcol, c, sizeof(int) * (size_t)M->nnz, kind, ctx->stream));
            if (v && M->where == TSG_MEM_HOST && !copy) {
                // host values of a single call go up on the copy stream while
                // the symbolic phase runs (PlanData::wait_values joins them)
                CUDA_OK(cudaEventRecord(ctx->cfork, ctx->stream));
                CUDA_OK(cudaStreamWaitEvent(ctx->copy, ctx->cfork, 0));
                CUDA_OK(cudaMemcpyAsync(dval, v, sizeof(double) * (size_t)M->nnz, kind, ctx->copy));
                CUDA_OK(cudaEventRecord(ctx->vals_ev, ctx->copy));
                P.vals_ev = ctx->vals_ev;
            } else if (v) {
                CUDA_OK(cudaMemcpyAsync(dval, v, sizeof(double) * (size_t)M->nnz, kind, ctx->stream));
            }
        }
        rp = drp; c = dcol; v = dval;
        valbuf = dval;
    }
    rp64 = P.own<long long>(pool, M->m + 1);
    if (!rp64) return fail(TSG_ERR_OOM, "device pool allocation failed");
    CUDA_OK(prepare_csr(pool, rp, M->rowptr_bits, c, M->m, M->n, M->nnz, rp64, ctx->dflags, validate));
    col = c;
    val = v;
    return TSG_OK;
}

// Symbolic phase: staging, A^T for A*A^T, tiles, step 1, step 2 (two host waits).
// `keep` = the plan outlives the call (device operands are copied).
tsg_status plan_symbolic(tsg_ctx *ctx, Pool &pool, Scratch &sc, tsg_op op, const tsg_csr *A, const tsg_csr *B,
                         PlanData &P, bool keep, bool want_cub, PhaseTimer &tm, bool reset_flags = true)
{
    const bool validate = ctx->opts.validate != 0;
    tsg_status r = check_op(op, A, B);
    if (r) return r;
    if (reset_flags) CUDA_OK(cudaMemsetAsync(ctx->dflags, 0, sizeof(int) * FLAG_COUNT, ctx->stream));
    CUDA_OK(cudaMemsetAsync(ctx->dstat, 0, sizeof(long long) * ST_HFLAGS, ctx->stream));   // the flags stay
    tm.mark();  // 0
    P.op = op;
    P.m = A->m;
    P.k = A->n;
    P.nnzA = A->nnz;
    r = stage_into_plan(ctx, pool, P, A, validate, keep, P.rpA, P.colA, P.valA, P.valA_buf);
    if (r) return r;
    if (op == TSG_OP_AB) {
        P.n = B->n;
        P.nnzB = B->nnz;
        r = stage_into_plan(ctx, pool, P, B, validate, keep, P.rpB, P.colB, P.valB, P.valB_buf);
        if (r) return r;
    } else if (op == TSG_OP_AA) {
        P.n = A->n;
        P.nnzB = A->nnz;
        P.rpB = P.rpA; P.colB = P.colA; P.valB = P.valA;
    } else {
        P.n = A->m;
        P.nnzB = A->nnz;
        long long *tp = P.own<long long>(pool, P.k + 1);
        int *tc = P.own<int>(pool, P.nnzA);
        double *tv = P.own<double>(pool, P.nnzA);
        P.perm = P.own<int>(pool, P.nnzA);
        if (!tp || !tc || !tv || !P.perm) return fail(TSG_ERR_OOM, "device pool allocation failed for A^T");
        P.wait_values(ctx->stream);
        CUDA_OK(csr_transpose(pool, P.rpA, P.colA, P.valA, P.m, P.k, P.nnzA, tp, tc, tv, P.perm, ctx->dflags));
        P.rpB = tp; P.colB = tc; P.valB = tv; P.valB_buf = tv;
    }
    if (keep && !P.valA_buf) {   // AA/AAT plans built from device operands still need a value buffer
        P.valA_buf = P.own<double>(pool, P.nnzA);
        if (!P.valA_buf) return fail(TSG_ERR_OOM, "device pool allocation failed");
    }
    DevCSR dA, dB;
    dA.m = P.m; dA.n = P.k; dA.nnz = P.nnzA; dA.rp = P.rpA; dA.col = P.colA;
    dB.m = P.k; dB.n = P.n; dB.nnz = P.nnzB; dB.rp = P.rpB; dB.col = P.colB;

    TileCSR TA, TB;
    r = build_tiles(pool, sc, dA, TA, ctx);
    if (r) return r;
    if (op == TSG_OP_AA) TB = TA;
    else {
        r = build_tiles(pool, sc, dB, TB, ctx);
        if (r) return r;
    }
    {   // bitmaps of B's tile-rows for step 1's bitmap path
        TB.bmoff = sc.get<long long>(TB.blkm + 1);
        TB.bmw = sc.get<unsigned>(tile_bitmap_words_bound(TB));
        long long *wcount = sc.get<long long>(TB.blkm + 1);
        if (!TB.bmoff || !TB.bmw || !wcount) return fail(TSG_ERR_OOM, "device pool allocation failed (tile bitmaps)");
        CUDA_OK(tile_bitmaps(pool, TB, wcount, ctx->dflags));
    }
    tm.mark();  // 1

    // step 1, count: C's tile-row pointer
    P.blkm = TA.blkm;
    P.crp = P.own<long long>(pool, P.blkm + 1);
    int *cnt = sc.get<int>(P.blkm + 1);
    int *wide = sc.get<int>(P.blkm + 2);
    int *defer = sc.get<int>(P.blkm + 1);
    if (!P.crp || !cnt || !wide || !defer) return fail(TSG_ERR_OOM, "device pool allocation failed (step 1)");
    CUDA_OK(cudaMemsetAsync(defer + P.blkm, 0, sizeof(int), ctx->stream));
    // the wide tile-rows' window bitmaps, kept from step 1's count pass for
    // its fill pass, when they take at most 2 GB and an eighth of the free
    // device memory (else the fill takes the union again)
    unsigned *wbm = nullptr;
    const long long wpr = (long long)ceil_div_i(TB.n, TILE) / 32 + 2;
    {
        size_t free_b = 0, total_b = 0;
        const long long bytes = 4ll * wpr * P.blkm;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && bytes <= (2ll << 30) && bytes <= (long long)(free_b / 8))
            wbm = sc.get<unsigned>(wpr * P.blkm);
        cudaGetLastError();
    }
    CUDA_OK(tile_symbolic(pool, TA, TB, P.crp, nullptr, cnt, wide, ctx->dflags, (int *)(ctx->dstat + ST_MAXS), true,
                          defer, wbm, wpr));
    CUDA_OK(cudaMemcpyAsync(ctx->dstat + ST_NDEFER, defer + P.blkm, sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
    CUDA_OK(aux_copy_scalars(pool, P.crp + P.blkm, ctx->dstat + ST_NUMBLKC, TA.trp + TA.blkm, ctx->dstat + ST_TILESA,
                             TB.trp + TB.blkm, ctx->dstat + ST_TILESB));
    CUDA_OK(aux_mask_popc(pool, TB.trp, TB.blkm, TB.mask, (unsigned long long *)(ctx->dstat + ST_POPCB)));
    CUDA_OK(aux_rows_increasing(pool, P.rpB, P.colB, P.k, P.nnzB, (unsigned long long *)(ctx->dstat + ST_BUNSORTED)));
    if (want_cub)
        CUDA_OK(aux_nnzcub(pool, P.rpA, P.colA, P.m, P.rpB, P.k, (unsigned long long *)(ctx->dstat + ST_NNZCUB)));
    r = host_wait(ctx, &P.nsync);
    if (r) return r;
    P.numblkC = ctx->hstat[ST_NUMBLKC];
    const int maxS = (int)(ctx->hstat[ST_MAXS] & 0xffffffff);        // stat[0]: max C tiles per tile-row
    const int maxSpan = (int)(ctx->hstat[ST_MAXS] >> 32);              // stat[1]: max tile-column window
    const int ndefer = (int)(ctx->hstat[ST_NDEFER] & 0xffffffff);
    P.tilesA = ctx->hstat[ST_TILESA];
    P.tilesB = ctx->hstat[ST_TILESB];
    P.dupsafe = ctx->hstat[ST_POPCB] != P.nnzB;
    P.b_increasing = ctx->hstat[ST_BUNSORTED] == 0;
    P.nnzcub = ctx->hstat[ST_NNZCUB];
    if (P.numblkC >= (1ll << 31)) return fail(TSG_ERR_NOT_SUPPORTED, "C has %lld tiles; the limit is 2^31-1", P.numblkC);

    // step 1 fill + step 2: C's sorted tile columns, row masks, row counts,
    // numeric bins (one warp per tile-row where it fits, CTA kernels for the rest)
    P.ccol = P.own<int>(pool, P.numblkC);
    P.cmask = P.own<uint16_t>(pool, P.numblkC * TILE + 2);
    int *rowcnt = sc.get<int>(P.m + 1);
    P.bin = P.own<unsigned char>(pool, P.blkm + 1);
    P.binlist = P.own<int>(pool, (long long)NBIN * P.blkm);
    P.rowlist = P.own<int>(pool, (long long)NROWCLS * P.m);
    P.rowptrC = P.own<long long>(pool, P.m + 1);
    if (!P.ccol || !P.cmask || !rowcnt || !P.bin || !P.binlist || !P.rowlist || !P.rowptrC)
        return fail(TSG_ERR_OOM, "device pool allocation failed for C tiles");
    NumericBinParams bp{ctx->opts.dense_tile_min, ctx->opts.smem_acc_max, ctx->opts.row_acc_max, P.rpA,
                        ctx->opts.rows_global};
    CUDA_OK(symbolic_fill_fused(pool, TA, TB, P.m, P.crp, P.ccol, P.cmask, rowcnt, cnt, wide, ctx->dflags, P.rpB,
                                P.colB, P.rpA, P.colA, wbm, wpr));
    tm.mark();  // 2
    CUDA_OK(step2_masks(pool, TA, TB, P.m, P.blkm, P.crp, P.ccol, P.cmask, rowcnt, maxS, maxSpan, ctx->dflags, defer,
                        ndefer, P.rpB, P.colB, P.rpA, P.colA, P.b_increasing, ctx->side, ctx->fork, ctx->join));
    CUDA_OK(scan_i32_to_i64(pool, rowcnt, P.rowptrC, P.m, ctx->dflags));
    CUDA_OK(bin_tilerows(pool, P.blkm, P.m, P.crp, P.ccol, P.rowptrC, bp, P.bin, ctx->dstat + ST_BINS, P.binlist,
                         P.rowlist));
    CUDA_OK(cudaMemcpyAsync(ctx->dstat + ST_NNZC, P.rowptrC + P.m, sizeof(long long), cudaMemcpyDeviceToDevice,
                            ctx->stream));
    r = host_wait(ctx, &P.nsync);
    if (r) return r;
    P.nnzC = ctx->hstat[ST_NNZC];
    for (int b = 0; b < BS_SLOTS; ++b) {
        P.bstat[b] = ctx->hstat[ST_BINS + b];
    }
    tm.mark();  // 3
    return TSG_OK;
}

// Numeric phase into caller-provided col/val (nnzC each).
NumericArgs numeric_args(tsg_ctx *ctx, const PlanData &P, const double *valA, const double *valB, int *col,
                         double *val, const int *tr_coloff)
{
    NumericArgs na{};
    na.m = P.m; na.blkm = P.blkm;
    na.rpA = P.rpA; na.colA = P.colA; na.valA = valA;
    na.rpB = P.rpB; na.colB = P.colB; na.valB = valB;
    na.crp = P.crp; na.ccol = P.ccol; na.cmask = P.cmask;
    na.rowptrC = P.rowptrC; na.colC = col; na.valC = val;
    na.bin = P.bin; na.binlist = P.binlist; na.rowlist = P.rowlist; na.b_sorted = P.b_increasing; na.tr_coloff = tr_coloff; na.flags = ctx->dflags;
    na.nnzA = P.nnzA; na.n = P.n;
    return na;
}

// cols_done: C's column indices were written before (numeric_cols)
tsg_status plan_numeric(tsg_ctx *ctx, Pool &pool, PlanData &P, const double *valA, const double *valB, int *col,
                        double *val, const int *tr_coloff = nullptr, int threads = 0, int walk = -1,
                        bool cols_done = false)
{
    NumericArgs na = numeric_args(ctx, P, valA, valB, col, val, tr_coloff);
    na.cols_done = cols_done;
    P.wait_values(ctx->stream);
    if (walk < 0) walk = ctx->opts.numeric_walk;
    if (threads <= 0) threads = ctx->opts.threads_numeric;
    // repeated B columns need the packed walk.  Auto otherwise loads B one
    // step ahead when few products meet in one output (estimated from the
    // mean row lengths: under 3 per entry of C), where the walk is bound by
    // the latency of B's loads, and walks plainly (twice the warps per SM)
    // when many do.
    int kw = 0;
    if (P.dupsafe || walk == 2) kw = 1;
    else if (walk == 3) kw = 2;
    else if (walk == 0 && P.nnzC > 0 && P.k > 0 &&
             (double)P.nnzA * ((double)P.nnzB / P.k) < 3.0 * (double)P.nnzC) kw = 2;
    CUDA_OK(numeric_run(pool, na, P.bstat, kw, threads, ctx->opts.row_warps, ctx->side, ctx->fork, ctx->join));
    return TSG_OK;
}

void fill_stats(const PlanData &P, tsg_stats *st)
{
    if (!st) return;
    st->nnz_a = P.nnzA; st->nnz_b = P.nnzB; st->nnz_c = P.nnzC;
    st->nnz_cub = P.nnzcub;
    st->tiles_a = P.tilesA; st->tiles_b = P.tilesB; st->tiles_c = P.numblkC;
    st->n_syncs = P.nsync;
    st->bins[0] = (int)P.bstat[BIN_EMPTY];
    st->bins[1] = (int)(P.bstat[BIN_SPARSE_S] + P.bstat[BIN_SPARSE_M] + P.bstat[BIN_SPARSE_L]);
    st->bins[2] = (int)(P.bstat[BIN_DENSE_S] + P.bstat[BIN_DENSE_M] + P.bstat[BIN_DENSE_L]);
    st->bins[3] = (int)P.bstat[BIN_ROWS];
}

// C's row pointers for the caller (int64 copied, or narrowed to int32), on
// the main stream
cudaError_t output_rowptr(tsg_ctx *ctx, Pool &pool, int m, int bits, const long long *rowptr, void *&rp_dev)
{
    if (bits == 32) {
        int *rp32 = pool.alloc_n<int>(m + 1);
        rp_dev = rp32;
        return rp32 ? aux_rowptr_narrow(pool, rowptr, rp32, m + 1) : cudaErrorMemoryAllocation;
    }
    long long *rp64 = pool.alloc_n<long long>(m + 1);
    rp_dev = rp64;
    return rp64 ? cudaMemcpyAsync(rp64, rowptr, sizeof(long long) * (size_t)(m + 1), cudaMemcpyDeviceToDevice, ctx->stream)
                : cudaErrorMemoryAllocation;
}

int output_bits(const tsg_ctx *ctx, long long nnzC)
{
    const int bits = ctx->opts.out_rowptr_bits;
    return bits ? bits : (nnzC < (1ll << 31) ? 32 : 64);
}

// Host output started before the numeric step: C's row pointers and its
// column indices (numeric_cols, from the masks) go down on the copy stream
// while the numeric kernels run; the values follow in emit_output.
struct EarlyOut {
    bool on = false;
    int bits = 0;
    void *rp_dev = nullptr;
    void *hrp = nullptr, *hcol = nullptr, *hval = nullptr;
    size_t rpb = 0, cb = 0, vb = 0;
    double ms = 0;               // host time spent here (part of the d2h phase)
};

// Host output with C tiles of 8 entries or more on average: there the
// numeric kernels are bound by FP64 issue and the copy beside them is
// nearly free; with sparser tiles they wait on B's rows in L2, which the
// concurrent copy slows by about as much as it hides.
bool early_out_pays(const PlanData &P, const tsg_csr *C)
{
    return C->where == TSG_MEM_HOST && P.nnzC > 0 && P.nnzC >= 8 * P.numblkC;
}

tsg_status early_out_begin(tsg_ctx *ctx, Pool &pool, PlanData &P, int *col, double *val, EarlyOut &eo)
{
    auto t0 = std::chrono::steady_clock::now();
    eo.bits = output_bits(ctx, P.nnzC);
    if (eo.bits == 32 && P.nnzC >= (1ll << 31)) return TSG_OK;   // emit_output reports it
    eo.rpb = (size_t)(P.m + 1) * (eo.bits == 64 ? 8 : 4);
    eo.cb = sizeof(int) * (size_t)P.nnzC;
    eo.vb = sizeof(double) * (size_t)P.nnzC;
    eo.hrp = pinned_get(ctx, eo.rpb);
    eo.hcol = pinned_get(ctx, eo.cb);
    eo.hval = pinned_get(ctx, eo.vb);
    if (!eo.hrp || !eo.hcol || !eo.hval) return fail(TSG_ERR_OOM, "pinned host memory for C");
    eo.on = true;
    CUDA_OK(output_rowptr(ctx, pool, P.m, eo.bits, P.rowptrC, eo.rp_dev));
    NumericArgs na = numeric_args(ctx, P, P.valA, P.valB, col, val, nullptr);
    CUDA_OK(numeric_cols(pool, na));
    CUDA_OK(cudaEventRecord(ctx->cols_ev, ctx->stream));
    CUDA_OK(cudaStreamWaitEvent(ctx->copy, ctx->cols_ev, 0));
    CUDA_OK(cudaMemcpyAsync(eo.hrp, eo.rp_dev, eo.rpb, cudaMemcpyDeviceToHost, ctx->copy));
    CUDA_OK(cudaMemcpyAsync(eo.hcol, col, eo.cb, cudaMemcpyDeviceToHost, ctx->copy));
    CUDA_OK(cudaEventRecord(ctx->copy_done, ctx->copy));
    eo.ms = ms_since(t0);
    return TSG_OK;
}

// Undo early_out_begin after a failure: the copy stream is drained before
// anything is freed; the pinned buffers go back to the cache.
void early_out_abort(tsg_ctx *ctx, Pool &pool, EarlyOut &eo)
{
    cudaStreamSynchronize(ctx->copy);
    pool.free(eo.rp_dev);
    cudaStreamSynchronize(ctx->stream);
    if (eo.hrp) pinned_put(ctx, eo.hrp, eo.rpb);
    if (eo.hcol) pinned_put(ctx, eo.hcol, eo.cb);
    if (eo.hval) pinned_put(ctx, eo.hval, eo.vb);
    eo = EarlyOut{};
}

// Hand C (rowptr copied/narrowed from `rowptr`, col/val adopted) to the
// caller per C->where; frees col/val on failure.  With `eo` (host output
// begun by early_out_begin) only the values remain to be copied.
tsg_status emit_output(tsg_ctx *ctx, Pool &pool, int m, int n, long long nnzC, const long long *rowptr, int *col,
                       double *val, tsg_csr *C, tsg_stats *st, EarlyOut *eo = nullptr)
{
    if (eo && eo->on) {
        auto t_d2h = std::chrono::steady_clock::now();
        OutOwner *o = new OutOwner();
        o->ctx = ctx;
        o->where = C->where;
        C->m = m; C->n = n; C->nnz = nnzC; C->rowptr_bits = eo->bits;
        cudaError_t e = cudaMemcpyAsync(eo->hval, val, eo->vb, cudaMemcpyDeviceToHost, ctx->stream);
        cudaStreamWaitEvent(ctx->stream, ctx->copy_done, 0);
        pool.free(eo->rp_dev); pool.free(col); pool.free(val);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        o->blocks.push_back({eo->hrp, eo->rpb});
        o->blocks.push_back({eo->hcol, eo->cb});
        o->blocks.push_back({eo->hval, eo->vb});
        C->row_ptr = eo->hrp; C->col = (int *)eo->hcol; C->val = (double *)eo->hval;
        C->owner = o;
        if (st) st->ms_d2h = eo->ms + ms_since(t_d2h);
        *eo = EarlyOut{};
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            tsg_csr_free(ctx, C);
            cudaGetLastError();
            return fail(cuda_status(e), "output: %s", cudaGetErrorString(e));
        }
        return TSG_OK;
    }
    const int bits = output_bits(ctx, nnzC);
    if (bits == 32 && nnzC >= (1ll << 31)) {
        pool.free(col); pool.free(val);
        cudaStreamSynchronize(ctx->stream);
        return fail(TSG_ERR_INT32_OVERFLOW, "C has %lld entries; int32 row pointers cannot hold them", nnzC);
    }
    OutOwner *o = new OutOwner();
    o->ctx = ctx;
    o->where = C->where;
    C->m = m; C->n = n; C->nnz = nnzC; C->rowptr_bits = bits;
    void *rp_dev = nullptr;
    cudaError_t e = output_rowptr(ctx, pool, m, bits, rowptr, rp_dev);
    if (C->where == TSG_MEM_DEVICE) {
        o->blocks.push_back({rp_dev, 0});
        o->blocks.push_back({col, 0});
        o->blocks.push_back({val, 0});
        C->row_ptr = rp_dev; C->col = col; C->val = val;
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    } else {
        auto t_d2h = std::chrono::steady_clock::now();
        const size_t rpb = (size_t)(m + 1) * (bits == 64 ? 8 : 4);
        const size_t cb = sizeof(int) * (size_t)nnzC, vb = sizeof(double) * (size_t)nnzC;
        void *hrp = pinned_get(ctx, rpb), *hcol = pinned_get(ctx, cb), *hval = pinned_get(ctx, vb);
        if (!hrp || !hcol || !hval) e = cudaErrorMemoryAllocation;
        if (e == cudaSuccess) e = cudaMemcpyAsync(hrp, rp_dev, rpb, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess && nnzC > 0) e = cudaMemcpyAsync(hcol, col, cb, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess && nnzC > 0) e = cudaMemcpyAsync(hval, val, vb, cudaMemcpyDeviceToHost, ctx->stream);
        pool.free(rp_dev); pool.free(col); pool.free(val);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (hrp) o->blocks.push_back({hrp, rpb});
        if (hcol) o->blocks.push_back({hcol, cb});
        if (hval) o->blocks.push_back({hval, vb});
        C->row_ptr = hrp; C->col = (int *)hcol; C->val = (double *)hval;
        if (st) st->ms_d2h = ms_since(t_d2h);
    }
    C->owner = o;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        tsg_csr_free(ctx, C);
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? TSG_ERR_OOM : TSG_ERR_CUDA, "output: %s", cudaGetErrorString(e));
    }
    return TSG_OK;
}

void phase_times(tsg_ctx *ctx, tsg_stats *st, const PhaseTimer &tm)
{
    if (!st || !tm.on || tm.n < 5) return;
    float a = 0, b = 0, c1 = 0, d = 0;
    cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&c1, ctx->ev[2], ctx->ev[3]);
    cudaEventElapsedTime(&d, ctx->ev[3], ctx->ev[4]);
    st->ms_convert = a; st->ms_step1 = b; st->ms_step2 = c1; st->ms_step3 = d;
}


// ---- the small-product path ---------------------------------------------------

constexpr long long SMALL_NNZ_MAX = 1ll << 22;   // entries of A and of B at most
constexpr size_t SMALL_SHAPES = 32;
constexpr int SMALL_KEEP_ROWS = 1 << 22;   // C's row pointer is kept for shapes of up to this many rows (32 MB each)

SmallShape *small_shape_find(tsg_ctx *ctx, const SmallShape &k)
{
    for (auto &s : ctx->small_shapes)
        if (s.op == k.op && s.m == k.m && s.k == k.k && s.n == k.n && s.nnz_a == k.nnz_a && s.nnz_b == k.nnz_b)
            return &s;
    return nullptr;
}

// the shape's entry, updated or added (the oldest dropped past SMALL_SHAPES)
SmallShape *small_shape_record(tsg_ctx *ctx, const SmallShape &k)
{
    SmallShape *s = small_shape_find(ctx, k);
    if (!s) {
        if (ctx->small_shapes.size() >= SMALL_SHAPES) {
            if (ctx->small_shapes.front().rowptr) cudaFreeAsync(ctx->small_shapes.front().rowptr, ctx->stream);
            ctx->small_shapes.erase(ctx->small_shapes.begin());
        }
        ctx->small_shapes.push_back(k);
        s = &ctx->small_shapes.back();
        s->rowptr = nullptr;
    }
    s->nnzc = k.nnzc;
    s->small = k.small;
    s->one_round = k.one_round;
    if (!s->small && s->rowptr) { cudaFreeAsync(s->rowptr, ctx->stream); s->rowptr = nullptr; }
    return s;
}

// The small path's operands as the caller gave them: device arrays in
// place, host arrays uploaded as they are (row pointers in their own type)
// into buffers P owns.  Nothing is validated here.
tsg_status small_raw_operands(tsg_ctx *ctx, Pool &pool, PlanData &P, bool aa, const tsg_csr *A, const tsg_csr *B,
                              SmallOperands &o)
{
    auto view = [&](const tsg_csr *M, RowPtr &rp, const int *&col, const double *&val) -> tsg_status {
        const void *r = M->row_ptr;
        col = M->col;
        val = M->val;
        if (M->where == TSG_MEM_HOST) {
            const size_t rpb = (size_t)(M->m + 1) * (M->rowptr_bits == 64 ? 8 : 4);
            void *dr = P.own<char>(pool, (long long)rpb);
            int *dc = P.own<int>(pool, M->nnz);
            double *dv = P.own<double>(pool, M->nnz);
            if (!dr || !dc || !dv) return fail(TSG_ERR_OOM, "device pool allocation failed for an operand");
            CUDA_OK(cudaMemcpyAsync(dr, r, rpb, cudaMemcpyHostToDevice, ctx->stream));
            if (M->nnz > 0) {
                CUDA_OK(cudaMemcpyAsync(dc, col, sizeof(int) * (size_t)M->nnz, cudaMemcpyHostToDevice, ctx->stream));
                CUDA_OK(cudaMemcpyAsync(dv, val, sizeof(double) * (size_t)M->nnz, cudaMemcpyHostToDevice, ctx->stream));
            }
            r = dr; col = dc; val = dv;
        }
        if (M->rowptr_bits == 64) rp.p64 = static_cast<const long long *>(r);
        else rp.p32 = static_cast<const int *>(r);
        return TSG_OK;
    };
    tsg_status st = view(A, o.rpA, o.colA, o.valA);
    if (st) return st;
    if (aa) { o.rpB = o.rpA; o.colB = o.colA; o.valB = o.valA; }
    else if ((st = view(B, o.rpB, o.colB, o.valB))) return st;
    o.m = A->m; o.ka = A->n; o.kb = B->m; o.nb = B->n; o.nnzA = A->nnz; o.nnzB = B->nnz;
    o.b_is_a = aa;
    return TSG_OK;
}

// tsg_spgemm for products whose every row of A meets at most
// SMALL_MAX_PRODUCTS entries of B (A*B and A*A, operands of at most
// SMALL_NNZ_MAX entries): one warp per row of C (tsg_small.cu).  A shape's
// first call runs the count pass and scan, reads C's size back and fills
// (two host waits).  Later calls of the shape run the fill alone at the row
// pointer kept from the last call, counting every row again: when all counts
// agree that row pointer is C's and the call waits once; otherwise the count
// pass and scan run and the fill follows into buffers sized from the last
// call (a larger C is found at the wait and the fill repeated).
// taken = false: nothing was returned to the caller -- the product is not
// small, or turned out not to be -- and the tiled path runs instead.
tsg_status small_spgemm(tsg_ctx *ctx, tsg_op op, const tsg_csr *A, const tsg_csr *B, tsg_csr *C, tsg_stats *st,
                        bool &taken)
{
    taken = false;
    if (!ctx->opts.small_path || op == TSG_OP_AAT) return TSG_OK;
    if (check_op(op, A, B) != TSG_OK) { g_err.clear(); return TSG_OK; }   // the tiled path reports it
    const tsg_csr *Bm = op == TSG_OP_AB ? B : A;
    if (A->nnz > SMALL_NNZ_MAX || Bm->nnz > SMALL_NNZ_MAX) return TSG_OK;
    SmallShape key;
    key.op = (int)op; key.m = A->m; key.k = A->n; key.n = Bm->n; key.nnz_a = A->nnz; key.nnz_b = Bm->nnz;
    SmallShape *seen = small_shape_find(ctx, key);
    if (seen && !seen->small) return TSG_OK;
    taken = true;
    auto t0 = std::chrono::steady_clock::now();
    Pool pool{ctx->pool, ctx->stream};
    PlanData P;
    int *col = nullptr;
    double *val = nullptr;
    void *rp_dev = nullptr;
    void *cblock = nullptr;   // device output: C's columns, values and row pointer in one allocation
    auto drop_cv = [&]() {
        if (cblock) pool.free(cblock);
        else { pool.free(col); pool.free(val); }
        cblock = nullptr; col = nullptr; val = nullptr; rp_dev = nullptr;
    };
    // undo everything before a return (values' upload joined, the stream drained)
    auto release = [&]() {
        P.wait_values(ctx->stream);
        drop_cv();
        P.release(pool);
        cudaStreamSynchronize(ctx->stream);
    };
    auto give_up = [&](tsg_status r) { release(); cudaGetLastError(); return r; };
    auto cuda_fail = [&](cudaError_t e) { return give_up(fail(cuda_status(e), "small path: %s", cudaGetErrorString(e))); };
    // rows over the limit: the tiled path, now and for later calls of the shape
    auto not_small = [&]() {
        release();
        cudaGetLastError();
        key.small = false;
        small_shape_record(ctx, key);
        taken = false;
        return TSG_OK;
    };
    const bool validate = ctx->opts.validate != 0;
    unsigned long long *sstat = reinterpret_cast<unsigned long long *>(ctx->dstat + ST_SMALL);
    cudaError_t e = cudaMemsetAsync(ctx->dstat, 0, sizeof(long long) * ST_SLOTS, ctx->stream);   // flags too
    if (e != cudaSuccess) return cuda_fail(e);
    P.op = op; P.m = A->m; P.k = A->n; P.nnzA = A->nnz;
    P.n = Bm->n; P.nnzB = Bm->nnz;
    tsg_status r = TSG_OK;
    const bool dev_out = C->where == TSG_MEM_DEVICE;
    // C's row pointer type: 32-bit unless asked otherwise (C stays far below
    // 2^31 entries on this path: at most SMALL_MAX_PRODUCTS per entry of A)
    const int bits = ctx->opts.out_rowptr_bits ? ctx->opts.out_rowptr_bits : 32;
    // buffers of `cap` entries, the fill at `rowptr` (kept: rows counted
    // against it), the caller's row pointer for device output, the wait
    auto fill = [&](const SmallOperands &so, const long long *rowptr, long long cap, bool kept,
                    bool one_round) -> tsg_status {
        if (dev_out) {
            auto a256 = [](long long x) { return (size_t)((x + 255) & ~255ll); };
            const size_t oc = a256(4 * std::max(cap, 1ll)), ov = a256(8 * std::max(cap, 1ll));
            cblock = pool.alloc(oc + ov + (size_t)(P.m + 1) * (bits == 64 ? 8 : 4));
            if (cblock) {
                col = static_cast<int *>(cblock);
                val = reinterpret_cast<double *>(static_cast<char *>(cblock) + oc);
                rp_dev = static_cast<char *>(cblock) + oc + ov;
            }
        } else {
            col = pool.alloc_n<int>(cap);
            val = pool.alloc_n<double>(cap);
        }
        if (!col || !val) return fail(TSG_ERR_OOM, "device pool allocation failed for C (%lld entries)", cap);
        P.wait_values(ctx->stream);
        // the fill writes the caller's row pointer too (device output)
        cudaError_t fe = small_fill(pool, so, rowptr, cap, col, val, ctx->dflags, kept ? sstat : nullptr,
                                    dev_out ? rp_dev : nullptr, bits, one_round);
        if (fe != cudaSuccess) return fail(cuda_status(fe), "small path: %s", cudaGetErrorString(fe));
        return host_wait(ctx, &P.nsync);
    };
    const long long *rowptr = nullptr;   // C's row pointer: the kept one, or this call's scan
    long long nnzC = 0;
    if (seen && seen->rowptr && P.m > 0) {
        // the fill alone at the kept row pointer, on the operands as they
        // are (device) or as uploaded (host), which it validates itself
        SmallOperands ro;
        r = small_raw_operands(ctx, pool, P, op == TSG_OP_AA, A, Bm, ro);
        if (r) return give_up(r);
        ro.check = validate;
        r = fill(ro, seen->rowptr, seen->nnzc, true, seen->one_round);
        if (r) return give_up(r);
        if (ctx->hstat[ST_SMALL] == 0) {
            rowptr = seen->rowptr;
            nnzC = seen->nnzc;
        } else {   // a row differs from the kept pointer: the count pass decides
            drop_cv();
            P.release(pool);
            e = cudaMemsetAsync(ctx->dstat + ST_SMALL, 0, 3 * sizeof(long long), ctx->stream);
            if (e != cudaSuccess) return cuda_fail(e);
        }
    }
    SmallOperands so;   // staged and validated operands (count pass)
    if (!rowptr) {
        r = stage_into_plan(ctx, pool, P, A, validate, false, P.rpA, P.colA, P.valA, P.valA_buf);
        if (r) return give_up(r);
        if (op == TSG_OP_AB) {
            r = stage_into_plan(ctx, pool, P, B, validate, false, P.rpB, P.colB, P.valB, P.valB_buf);
            if (r) return give_up(r);
        } else {
            P.rpB = P.rpA; P.colB = P.colA; P.valB = P.valA;
        }
        so.rpA.p64 = P.rpA; so.rpB.p64 = P.rpB;
        so.colA = P.colA; so.colB = P.colB; so.valA = P.valA; so.valB = P.valB;
        so.m = P.m; so.ka = P.k; so.kb = Bm->m; so.nb = P.n; so.nnzA = P.nnzA; so.nnzB = P.nnzB;
        so.b_is_a = op == TSG_OP_AA;
    }
    if (!rowptr) {
        int *rowcnt = P.own<int>(pool, (long long)P.m + 1);
        P.rowptrC = P.own<long long>(pool, (long long)P.m + 1);
        if (!rowcnt || !P.rowptrC) return give_up(fail(TSG_ERR_OOM, "device pool allocation failed (small path)"));
        e = small_count(pool, so, rowcnt, sstat);
        if (e == cudaSuccess) e = scan_i32_to_i64(pool, rowcnt, P.rowptrC, P.m, ctx->dflags);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->dstat + ST_NNZC, P.rowptrC + P.m, sizeof(long long), cudaMemcpyDeviceToDevice,
                                ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e);
        long long cap = seen ? seen->nnzc + seen->nnzc / 8 + 64 : -1;
        if (cap < 0) {   // a new shape: C's size first
            r = host_wait(ctx, &P.nsync);
            if (r) return give_up(r);
            if (ctx->hstat[ST_SMALL] > 0) return not_small();
            cap = ctx->hstat[ST_NNZC];
        }
        for (int pass = 0;; ++pass) {
            r = fill(so, P.rowptrC, cap, false, false);
            if (r) return give_up(r);
            if (ctx->hstat[ST_SMALL] > 0) return not_small();
            if (ctx->hstat[ST_NNZC] <= cap || pass > 0) break;
            drop_cv();   // C outgrew the buffers sized from the shape's last call
            cap = ctx->hstat[ST_NNZC];
        }
        rowptr = P.rowptrC;
        nnzC = ctx->hstat[ST_NNZC];
    }
    const long long products = ctx->hstat[ST_SMALL + 1];
    key.nnzc = nnzC;
    // this call's rows all fit one round (from the count pass; a kept shape keeps its flag)
    key.one_round = rowptr == P.rowptrC ? ctx->hstat[ST_SMALL + 2] == 0 : seen->one_round;
    seen = small_shape_record(ctx, key);
    if (rowptr == P.rowptrC && P.m <= SMALL_KEEP_ROWS) {   // kept for the shape's next call (when memory allows)
        if (!seen->rowptr) seen->rowptr = pool.alloc_n<long long>((long long)P.m + 1);
        if (seen->rowptr)
            cudaMemcpyAsync(seen->rowptr, P.rowptrC, sizeof(long long) * ((size_t)P.m + 1), cudaMemcpyDeviceToDevice,
                            ctx->stream);
        cudaGetLastError();
    }
    if (st) {
        st->nnz_a = P.nnzA; st->nnz_b = P.nnzB; st->nnz_c = nnzC;
        st->nnz_cub = ctx->opts.count_products ? products : 0;
        st->small_path = 1;
    }
    if (dev_out) {
        OutOwner *o = new OutOwner();
        o->ctx = ctx;
        o->where = C->where;
        o->blocks.push_back({cblock, 0});   // the three arrays
        C->m = P.m; C->n = P.n; C->nnz = nnzC; C->rowptr_bits = bits;
        C->row_ptr = rp_dev; C->col = col; C->val = val;
        C->owner = o;
        P.release(pool);
    } else {
        r = emit_output(ctx, pool, P.m, P.n, nnzC, rowptr, col, val, C, st);   // frees col and val
        P.release(pool);
        if (r) { cudaStreamSynchronize(ctx->stream); return r; }
        if (st) st->n_syncs = 1;
    }
    if (st) {
        st->n_syncs += P.nsync;
        st->ms_total = ms_since(t0);
    }
    return TSG_OK;
}

}  // namespace

void *tsg::make_malloc_owner(void *a, void *b, void *c)
{
    OutOwner *o = new OutOwner();
    o->where = OWN_MALLOC;
    for (void *p : {a, b, c}) if (p) o->blocks.push_back({p, 0});
    return o;
}

// ============================================================================
// C ABI
// ============================================================================

extern "C" {

void tsg_opts_default(tsg_opts *o)
{
    if (!o) return;
    o->validate = 1;
    o->phase_times = 0;
    o->out_rowptr_bits = 0;
    o->dense_tile_min = 160;
    o->smem_acc_max = 24576;
    o->threads_numeric = 256;
    o->row_acc_max = 65535;
    o->numeric_walk = 0;
    o->rows_global = 0;
    o->row_warps = 4;
    o->count_products = 1;
    o->small_path = 1;
}

const char *tsg_last_error(void) { return g_err.c_str(); }

const char *tsg_version(void) { return "tilespgemm-gb300 0.1 (sm_103a)"; }

int64_t tsg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int64_t tsg_pinned_cache_cap(void) { return (int64_t)pinned_cap(); }

void *tsg_get_stream(tsg_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

tsg_status tsg_stream_wait(tsg_ctx *ctx, void *stream)
{
    if (!ctx) return fail(TSG_ERR_INVALID_ARG, "ctx is NULL");
    CUDA_OK(cudaSetDevice(ctx->device));
    CUDA_OK(cudaEventRecord(ctx->ext_ev, static_cast<cudaStream_t>(stream)));
    CUDA_OK(cudaStreamWaitEvent(ctx->stream, ctx->ext_ev, 0));
    return TSG_OK;
}

tsg_status tsg_inject_alloc_failure(int32_t kind, int64_t countdown)
{
    if (kind != 0 && kind != 1) return fail(TSG_ERR_INVALID_ARG, "kind must be 0 (device pool) or 1 (pinned host)");
    if (countdown < 0) return fail(TSG_ERR_INVALID_ARG, "countdown must be >= 0");
    g_fail_alloc[kind].store(countdown, std::memory_order_relaxed);
    return TSG_OK;
}

int64_t tsg_alloc_failure_pending(int32_t kind)
{
    if (kind != 0 && kind != 1) return -1;
    const long long c = g_fail_alloc[kind].load(std::memory_order_relaxed);
    return c > 0 ? c : 0;
}

tsg_status tsg_check_bounded_wait(tsg_ctx *ctx, int64_t n, int32_t spin_limit)
{
    if (!ctx) return fail(TSG_ERR_INVALID_ARG, "ctx is NULL");
    if (n < 1 || n > (1ll << 30) || spin_limit < 1)
        return fail(TSG_ERR_INVALID_ARG, "n must be in [1, 2^30] and spin_limit >= 1");
    CUDA_OK(cudaSetDevice(ctx->device));
    CUDA_OK(cudaMemsetAsync(ctx->dflags, 0, sizeof(int) * FLAG_COUNT, ctx->stream));
    Pool pool{ctx->pool, ctx->stream};
    const cudaError_t e = scan_unpublished_tile(pool, n, spin_limit, ctx->dflags);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? TSG_ERR_OOM : TSG_ERR_CUDA, "bounded-wait check: %s",
                    cudaGetErrorString(e));
    }
    const tsg_status r = host_wait(ctx, nullptr);
    // the flags of this check are not carried into the context's next call
    cudaMemsetAsync(ctx->dflags, 0, sizeof(int) * FLAG_COUNT, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return r;
}

tsg_status tsg_measure_fp64_peak(tsg_ctx *ctx, double *gflops)
{
    if (!ctx || !gflops) return fail(TSG_ERR_INVALID_ARG, "ctx/gflops is NULL");
    CUDA_OK(cudaSetDevice(ctx->device));
    double best = 0.0;
    CUDA_OK(tsg::fp64_peak(ctx->stream, ctx->ev[6], ctx->ev[7], &best));
    *gflops = best;
    return TSG_OK;
}

tsg_status tsg_create(tsg_ctx **out, int device, const tsg_opts *opts)
{
    if (!out) return fail(TSG_ERR_INVALID_ARG, "ctx out-pointer is NULL");
    *out = nullptr;
    int ndev = 0;
    CUDA_OK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(TSG_ERR_INVALID_ARG, "device %d out of range (%d devices)", device, ndev);
    CUDA_OK(cudaSetDevice(device));
    int major = 0, minor = 0;
    CUDA_OK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
    CUDA_OK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device));
    if (major * 10 + minor != 103)
        return fail(TSG_ERR_NOT_SUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a (GB300) only", device, major, minor);
    tsg_ctx *c = new tsg_ctx();
    c->device = device;
    pinned_context_enter();
    c->counted = true;
    tsg_opts_default(&c->opts);
    if (opts) c->opts = *opts;
    if (c->opts.threads_numeric != 128 && c->opts.threads_numeric != 256 && c->opts.threads_numeric != 512)
        c->opts.threads_numeric = 256;
    auto cleanup = [&](tsg_status st) { tsg_destroy(c); return st; };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking) != cudaSuccess)
        return cleanup(fail(TSG_ERR_CUDA, "cudaStreamCreate failed"));
    if (cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->cfork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->vals_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->cols_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->copy_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ext_ev, cudaEventDisableTiming) != cudaSuccess)
        return cleanup(fail(TSG_ERR_CUDA, "cudaEventCreate failed"));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&c->pool, &props) != cudaSuccess)
        return cleanup(fail(TSG_ERR_CUDA, "cudaMemPoolCreate failed"));
    unsigned long long thr = ~0ull;
    cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    if (cudaMalloc(&c->dstat, sizeof(long long) * ST_SLOTS) != cudaSuccess ||
        cudaMallocHost(&c->hstat, sizeof(long long) * ST_SLOTS) != cudaSuccess)
        return cleanup(fail(TSG_ERR_OOM, "context buffers"));
    c->dflags = reinterpret_cast<int *>(c->dstat + ST_HFLAGS);   // the flags sit behind the statistics
    if (cudaMemset(c->dstat, 0, sizeof(long long) * ST_SLOTS) != cudaSuccess)
        return cleanup(fail(TSG_ERR_CUDA, "context buffers"));
    for (auto &e : c->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return cleanup(fail(TSG_ERR_CUDA, "cudaEventCreate failed"));
    cudaError_t e = tiles_init_attributes();
    if (e == cudaSuccess) e = symbolic_init_attributes();
    if (e == cudaSuccess) e = numeric_init_attributes();
    if (e != cudaSuccess) return cleanup(fail(TSG_ERR_CUDA, "kernel attributes: %s", cudaGetErrorString(e)));
    noalloc_forget(device);   // tsg_tiles_to_csr_noalloc resolves its scratch address again
    *out = c;
    return TSG_OK;
}

tsg_status tsg_destroy(tsg_ctx *c)
{
    if (!c) return TSG_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->counted) pinned_context_leave();
    for (auto &e : c->ev) if (e) cudaEventDestroy(e);
    if (c->fork) cudaEventDestroy(c->fork);
    if (c->join) cudaEventDestroy(c->join);
    if (c->side) { cudaStreamSynchronize(c->side); cudaStreamDestroy(c->side); }
    if (c->copy) { cudaStreamSynchronize(c->copy); cudaStreamDestroy(c->copy); }
    for (cudaEvent_t e : {c->cfork, c->vals_ev, c->cols_ev, c->copy_done, c->ext_ev}) if (e) cudaEventDestroy(e);
    for (auto &sh : c->small_shapes) if (sh.rowptr) cudaFreeAsync(sh.rowptr, c->stream);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->dstat) cudaFree(c->dstat);
    if (c->hstat) cudaFreeHost(c->hstat);
    if (c->pool) cudaMemPoolDestroy(c->pool);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TSG_OK;
}

tsg_status tsg_csr_free(tsg_ctx *ctx, tsg_csr *M)
{
    if (!M) return TSG_OK;
    OutOwner *o = static_cast<OutOwner *>(M->owner);
    if (o && o->refs.fetch_sub(1, std::memory_order_acq_rel) == 1) {
        tsg_ctx *c = o->ctx ? o->ctx : ctx;
        if (o->where == TSG_MEM_DEVICE) {
            if (c) {
                cudaSetDevice(c->device);
                for (auto &b : o->blocks) cudaFreeAsync(b.first, c->stream);
                cudaStreamSynchronize(c->stream);
            }
        } else if (o->where == TSG_MEM_HOST) {
            for (auto &b : o->blocks) pinned_put(c, b.first, b.second);   // kept, or freed past the cap
        } else {
            for (auto &b : o->blocks) free(b.first);
        }
        delete o;
    }
    // caller-owned arrays (owner NULL) are left alone
    if (o) {
        M->row_ptr = nullptr; M->col = nullptr; M->val = nullptr; M->owner = nullptr;
        M->nnz = 0;
    }
    return TSG_OK;
}

tsg_status tsg_spgemm(tsg_ctx *ctx, tsg_op op, const tsg_csr *A, const tsg_csr *B, tsg_csr *C, tsg_stats *st)
{
    if (!ctx) return fail(TSG_ERR_INVALID_ARG, "ctx is NULL");
    if (!C) return fail(TSG_ERR_INVALID_ARG, "C is NULL");
    if (C->where != TSG_MEM_HOST && C->where != TSG_MEM_DEVICE) return fail(TSG_ERR_INVALID_ARG, "C->where is not a tsg_mem");
    auto t0 = std::chrono::steady_clock::now();
    CUDA_OK(cudaSetDevice(ctx->device));
    if (st) memset(st, 0, sizeof(*st));
    {
        bool taken = false;
        const tsg_status rs = small_spgemm(ctx, op, A, B, C, st, taken);
        if (taken) return rs;
    }
    Pool pool{ctx->pool, ctx->stream};
    PlanData P;
    PhaseTimer tm(ctx, st && ctx->opts.phase_times);
    int *col = nullptr;
    double *val = nullptr;
    EarlyOut eo;
    tsg_status r;
    {
        Scratch sc(pool);
        r = plan_symbolic(ctx, pool, sc, op, A, B, P, false, st != nullptr && ctx->opts.count_products, tm);
        if (!r && output_bits(ctx, P.nnzC) == 32 && P.nnzC >= (1ll << 31))   // before any work on C
            r = fail(TSG_ERR_INT32_OVERFLOW, "C has %lld entries; int32 row pointers cannot hold them", P.nnzC);
        if (!r) {
            col = pool.alloc_n<int>(P.nnzC);
            val = pool.alloc_n<double>(P.nnzC);
            if (!col || !val) r = fail(TSG_ERR_OOM, "device pool allocation failed for C (%lld entries)", P.nnzC);
        }
        if (!r && early_out_pays(P, C)) r = early_out_begin(ctx, pool, P, col, val, eo);
        if (!r) r = plan_numeric(ctx, pool, P, P.valA, P.valB, col, val, nullptr, 0, -1, eo.on);
        tm.mark();  // 4
    }
    if (r) {
        early_out_abort(ctx, pool, eo);
        pool.free(col); pool.free(val);
        P.release(pool);
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
        return r;
    }
    fill_stats(P, st);
    r = emit_output(ctx, pool, P.m, P.n, P.nnzC, P.rowptrC, col, val, C, st, &eo);
    P.release(pool);
    if (r) return r;
    if (st) {
        st->ms_total = ms_since(t0);
        phase_times(ctx, st, tm);
        st->n_syncs = P.nsync + 1;
    }
    return TSG_OK;
}

// ---- plans: symbolic once, numeric many times ------------------------------

}  // extern "C"

struct tsg_plan {
    tsg_ctx *ctx = nullptr;
    PlanData P;
    // batched plans (count > 0): layout of the packed instances
    int count = 0;
    std::vector<int> mi, ni;
    std::vector<long long> aoff, boff;   // first packed value of each instance (A, and B for A*B), count+1
    std::vector<long long> ebase, rpoff; // first C entry, first row-pointer entry of each instance
    int *d_trc = nullptr;                // per tile-row C column offset
    UnpackDesc *d_ud = nullptr;
    long long *rp_out = nullptr;         // instances' row pointers, rebased
    long long *d_ebase = nullptr;
    // resident result of tsg_plan_replay and its CUDA graph
    int *rcol = nullptr;
    double *rval = nullptr;
    cudaGraphExec_t gexec = nullptr;
    long long glaunches = 0;             // kernel launches in the graph
    int threads = 0, walk = -1;          // numeric settings picked by tsg_plan_tune (0 / -1: the context's)
    // bin thresholds the plan's bins were chosen with (the context's, or
    // tsg_plan_tune's pick)
    int dense_tile_min = 0, smem_acc_max = 0, row_acc_max = 0;
};

extern "C" {

tsg_status tsg_plan_create(tsg_ctx *ctx, tsg_op op, const tsg_csr *A, const tsg_csr *B, tsg_plan **plan,
                           tsg_stats *st)
{
    if (!ctx || !plan) return fail(TSG_ERR_INVALID_ARG, "ctx/plan is NULL");
    *plan = nullptr;
    CUDA_OK(cudaSetDevice(ctx->device));
    if (st) memset(st, 0, sizeof(*st));
    auto t0 = std::chrono::steady_clock::now();
    Pool pool{ctx->pool, ctx->stream};
    tsg_plan *pl = new tsg_plan();
    pl->ctx = ctx;
    PhaseTimer tm(ctx, false);
    tsg_status r;
    {
        Scratch sc(pool);
        r = plan_symbolic(ctx, pool, sc, op, A, B, pl->P, true, true, tm);
    }
    if (r == TSG_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess) r = fail(TSG_ERR_CUDA, "plan build failed");
    if (r) {
        pl->P.release(pool);
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
        delete pl;
        return r;
    }
    fill_stats(pl->P, st);
    if (st) st->ms_total = ms_since(t0);
    *plan = pl;
    return TSG_OK;
}

tsg_status tsg_plan_execute(tsg_ctx *ctx, tsg_plan *plan, const double *valA, const double *valB, int32_t where,
                            tsg_csr *C, tsg_stats *st)
{
    if (!ctx || !plan || !C) return fail(TSG_ERR_INVALID_ARG, "ctx/plan/C is NULL");
    if (plan->ctx != ctx) return fail(TSG_ERR_INVALID_ARG, "plan belongs to another context");
    if (where != TSG_MEM_HOST && where != TSG_MEM_DEVICE) return fail(TSG_ERR_INVALID_ARG, "where is not a tsg_mem");
    if (C->where != TSG_MEM_HOST && C->where != TSG_MEM_DEVICE) return fail(TSG_ERR_INVALID_ARG, "C->where is not a tsg_mem");
    if (plan->count > 0) return fail(TSG_ERR_NOT_SUPPORTED, "a batched plan runs with tsg_plan_set_values + tsg_plan_replay");
    PlanData &P = plan->P;
    if (P.nnzA > 0 && !valA) return fail(TSG_ERR_INVALID_ARG, "valA is NULL");
    if (P.op == TSG_OP_AB && P.nnzB > 0 && !valB) return fail(TSG_ERR_INVALID_ARG, "valB is NULL for A*B");
    auto t0 = std::chrono::steady_clock::now();
    CUDA_OK(cudaSetDevice(ctx->device));
    if (st) memset(st, 0, sizeof(*st));
    Pool pool{ctx->pool, ctx->stream};
    CUDA_OK(cudaMemsetAsync(ctx->dflags, 0, sizeof(int) * FLAG_COUNT, ctx->stream));
    const double *va = valA, *vb = valB;
    if (where == TSG_MEM_HOST && P.nnzA > 0) {
        CUDA_OK(cudaMemcpyAsync(P.valA_buf, valA, sizeof(double) * (size_t)P.nnzA, cudaMemcpyHostToDevice, ctx->stream));
        va = P.valA_buf;
    }
    if (P.op == TSG_OP_AB) {
        if (where == TSG_MEM_HOST && P.nnzB > 0) {
            CUDA_OK(cudaMemcpyAsync(P.valB_buf, valB, sizeof(double) * (size_t)P.nnzB, cudaMemcpyHostToDevice, ctx->stream));
            vb = P.valB_buf;
        }
    } else if (P.op == TSG_OP_AA) {
        vb = va;
    } else {
        CUDA_OK(aux_gather(pool, P.perm, va, P.valB_buf, P.nnzA));
        vb = P.valB_buf;
    }
    int *col = pool.alloc_n<int>(P.nnzC);
    double *val = pool.alloc_n<double>(P.nnzC);
    if (!col || !val) {
        pool.free(col); pool.free(val);
        return fail(TSG_ERR_OOM, "device pool allocation failed for C (%lld entries)", P.nnzC);
    }
    // host output of dense enough C tiles: column indices down during the
    // numeric step (as in tsg_spgemm)
    EarlyOut eo;
    tsg_status r = TSG_OK;
    if (early_out_pays(P, C)) r = early_out_begin(ctx, pool, P, col, val, eo);
    if (!r) r = plan_numeric(ctx, pool, P, va, vb, col, val, nullptr, 0, -1, eo.on);
    if (r) {
        early_out_abort(ctx, pool, eo);
        pool.free(col); pool.free(val);
        cudaStreamSynchronize(ctx->stream);
        return r;
    }
    fill_stats(P, st);
    r = emit_output(ctx, pool, P.m, P.n, P.nnzC, P.rowptrC, col, val, C, st, &eo);
    if (r) return r;
    // numeric kernels report an internal bound failure through the flags
    int hflags[FLAG_COUNT];
    CUDA_OK(cudaMemcpy(hflags, ctx->dflags, sizeof(hflags), cudaMemcpyDeviceToHost));
    if (hflags[FLAG_INTERNAL]) { tsg_csr_free(ctx, C); return fail(TSG_ERR_CUDA, "internal bound check failed on the device"); }
    if (st) { st->ms_total = ms_since(t0); st->n_syncs = 1; }
    return TSG_OK;
}

int64_t tsg_plan_nnz(const tsg_plan *plan) { return plan ? plan->P.nnzC : -1; }

int64_t tsg_plan_device_bytes(const tsg_plan *plan) { return plan ? plan->P.device_bytes() : -1; }

tsg_status tsg_plan_destroy(tsg_ctx *ctx, tsg_plan *plan)
{
    if (!plan) return TSG_OK;
    tsg_ctx *c = plan->ctx ? plan->ctx : ctx;
    if (c) {
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->stream);
        if (plan->gexec) cudaGraphExecDestroy(plan->gexec);
        Pool pool{c->pool, c->stream};
        plan->P.release(pool);
        cudaStreamSynchronize(c->stream);
    }
    delete plan;
    return TSG_OK;
}

tsg_status tsg_csr_download(tsg_ctx *ctx, const tsg_csr *M, int64_t *row_ptr, int32_t *col, double *val)
{
    if (!M) return fail(TSG_ERR_INVALID_ARG, "M is NULL");
    const int kind = M->where == TSG_MEM_DEVICE ? 1 : 0;
    if (kind && !ctx) return fail(TSG_ERR_INVALID_ARG, "device matrix needs a context");
    if (ctx) CUDA_OK(cudaSetDevice(ctx->device));
    const size_t rpb = (size_t)(M->m + 1) * (M->rowptr_bits == 64 ? 8 : 4);
    std::vector<char> tmp;
    const void *rp_src = M->row_ptr;
    if (row_ptr) {
        if (M->rowptr_bits == 64) {
            if (kind) CUDA_OK(cudaMemcpy(row_ptr, rp_src, rpb, cudaMemcpyDeviceToHost));
            else memcpy(row_ptr, rp_src, rpb);
        } else {
            tmp.resize(rpb);
            if (kind) CUDA_OK(cudaMemcpy(tmp.data(), rp_src, rpb, cudaMemcpyDeviceToHost));
            else memcpy(tmp.data(), rp_src, rpb);
            const int *p32 = reinterpret_cast<const int *>(tmp.data());
            for (int i = 0; i <= M->m; ++i) row_ptr[i] = p32[i];
        }
    }
    if (M->nnz > 0) {
        if (col) {
            if (kind) CUDA_OK(cudaMemcpy(col, M->col, sizeof(int) * (size_t)M->nnz, cudaMemcpyDeviceToHost));
            else memcpy(col, M->col, sizeof(int) * (size_t)M->nnz);
        }
        if (val) {
            if (kind) CUDA_OK(cudaMemcpy(val, M->val, sizeof(double) * (size_t)M->nnz, cudaMemcpyDeviceToHost));
            else memcpy(val, M->val, sizeof(double) * (size_t)M->nnz);
        }
    }
    return TSG_OK;
}


tsg_status tsg_csr_to_device(tsg_ctx *ctx, const tsg_csr *H, tsg_csr *D)
{
    if (!ctx || !D) return fail(TSG_ERR_INVALID_ARG, "ctx/D is NULL");
    tsg_status r = check_csr(H, "H");
    if (r) return r;
    CUDA_OK(cudaSetDevice(ctx->device));
    const cudaMemcpyKind kind = H->where == TSG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    const size_t rpb = (size_t)(H->m + 1) * (H->rowptr_bits == 64 ? 8 : 4);
    const size_t cb = sizeof(int) * (size_t)H->nnz, vb = sizeof(double) * (size_t)H->nnz;
    Pool pool{ctx->pool, ctx->stream};
    void *rp = pool.alloc(rpb);
    int *col = static_cast<int *>(pool.alloc(cb));
    double *val = static_cast<double *>(pool.alloc(vb));
    cudaError_t e = (rp && col && val) ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = cudaMemcpyAsync(rp, H->row_ptr, rpb, kind, ctx->stream);
    if (e == cudaSuccess && H->nnz > 0) e = cudaMemcpyAsync(col, H->col, cb, kind, ctx->stream);
    if (e == cudaSuccess && H->nnz > 0) e = cudaMemcpyAsync(val, H->val, vb, kind, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        pool.free(rp); pool.free(col); pool.free(val);
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
        return fail(cuda_status(e), "tsg_csr_to_device: %s", cudaGetErrorString(e));
    }
    OutOwner *o = new OutOwner();
    o->ctx = ctx;
    o->where = TSG_MEM_DEVICE;
    o->blocks = {{rp, 0}, {col, 0}, {val, 0}};
    D->m = H->m; D->n = H->n; D->nnz = H->nnz; D->rowptr_bits = H->rowptr_bits; D->where = TSG_MEM_DEVICE;
    D->row_ptr = rp; D->col = col; D->val = val; D->owner = o;
    return TSG_OK;
}

// Matrix Market file -> CSR on the device, the data lines parsed there
// (tsg_mtx_dev.cu); the result equals tsg_load_mtx's, uploaded.
tsg_status tsg_load_mtx_device(tsg_ctx *ctx, const char *path, tsg_csr *A, int32_t *is_symmetric)
{
    if (!ctx || !path || !A) return fail(TSG_ERR_INVALID_ARG, "ctx/path/A is NULL");
    memset(A, 0, sizeof(*A));
    CUDA_OK(cudaSetDevice(ctx->device));
    std::string text;
    if (!mtx_read_file(path, text)) return fail(TSG_ERR_BAD_MTX, "could not open the Matrix Market file");
    MtxHeader h;
    tsg_status r = mtx_header(text, h);
    if (r) return r;
    // files whose entries do not sit one per line: the host loader, uploaded
    auto host_path = [&]() -> tsg_status {
        tsg_csr H;
        tsg_status rh = tsg_load_mtx(path, &H, is_symmetric);
        if (rh) return rh;
        rh = tsg_csr_to_device(ctx, &H, A);
        tsg_csr_free(nullptr, &H);
        return rh;
    };
    if (!h.lines) return host_path();
    Pool pool{ctx->pool, ctx->stream};
    std::vector<void *> tmp;   // device scratch, freed on every return
    auto dalloc = [&](size_t bytes) -> void * {
        void *p = pool.alloc(bytes);
        if (p) tmp.push_back(p);
        return p;
    };
    auto release = [&]() {
        for (void *p : tmp) pool.free(p);
        tmp.clear();
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
    };
    auto cuda_fail = [&](cudaError_t e) {
        release();
        return fail(e == cudaErrorMemoryAllocation ? TSG_ERR_OOM : cuda_status(e), "device Matrix Market load: %s",
                    cudaGetErrorString(e));
    };
    auto mtx_fail = [&](const char *msg) { release(); return fail(TSG_ERR_BAD_MTX, "%s", msg); };
    const long long M = h.M, N = h.N, NZ = h.NZ;
    const char *data = text.data() + h.data;
    const long long nb = (long long)(text.size() - h.data);
    cudaError_t e = cudaMemsetAsync(ctx->dstat, 0, sizeof(long long) * ST_SLOTS, ctx->stream);   // flags too
    char *dtext = static_cast<char *>(dalloc((size_t)((nb + 15) & ~15ll)));
    if (!dtext) return cuda_fail(cudaErrorMemoryAllocation);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtext, data, (size_t)nb, cudaMemcpyHostToDevice, ctx->stream);
    long long *ends = nullptr, lines = 0;
    if (e == cudaSuccess) e = mtx_lines(pool, dtext, nb, ends, lines, ctx->dflags);
    if (ends) tmp.push_back(ends);
    if (e != cudaSuccess) return cuda_fail(e);
    // per line: what it holds; the entries' numbers in file order
    const long long L1 = std::max(lines, 1ll);
    unsigned char *st = static_cast<unsigned char *>(dalloc((size_t)L1));
    int *lri = static_cast<int *>(dalloc(sizeof(int) * (size_t)L1));
    int *lci = static_cast<int *>(dalloc(sizeof(int) * (size_t)L1));
    double *lvv = static_cast<double *>(dalloc(sizeof(double) * (size_t)L1));
    long long *tpos = static_cast<long long *>(dalloc(sizeof(long long) * (size_t)(lines + 1)));
    const long long NZ1 = std::max(NZ, 1ll);
    int *ri = static_cast<int *>(dalloc(sizeof(int) * (size_t)NZ1));
    int *ci = static_cast<int *>(dalloc(sizeof(int) * (size_t)NZ1));
    double *vv = static_cast<double *>(dalloc(sizeof(double) * (size_t)NZ1));
    unsigned long long *hn = static_cast<unsigned long long *>(dalloc(sizeof(unsigned long long) + 2 * sizeof(int)));
    long long *ht = static_cast<long long *>(dalloc(sizeof(long long) * (size_t)L1));
    long long *hl = static_cast<long long *>(dalloc(sizeof(long long) * (size_t)L1));
    if (!st || !lri || !lci || !lvv || !tpos || !ri || !ci || !vv || !hn || !ht || !hl)
        return cuda_fail(cudaErrorMemoryAllocation);
    int *bad = reinterpret_cast<int *>(hn + 1);
    long long total = 0;
    e = cudaMemsetAsync(hn, 0, sizeof(unsigned long long) + 2 * sizeof(int), ctx->stream);
    if (e == cudaSuccess && lines > 0) e = mtx_parse(pool, dtext, ends, lines, h.kind, M, N, st, lri, lci, lvv);
    if (e == cudaSuccess && lines > 0) e = mtx_number_entries(pool, st, lines, tpos, ctx->dflags);
    if (e == cudaSuccess && lines > 0)
        e = mtx_take(pool, st, tpos, lines, NZ, M, h.symm, lri, lci, lvv, ri, ci, vv, hn, ht, hl, bad);
    unsigned long long hcount = 0;
    int hbad[2] = {0, 0};
    if (e == cudaSuccess && lines > 0) e = cudaMemcpyAsync(&total, tpos + lines, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hcount, hn, sizeof(hcount), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e);
    // lines the device left: the host loader's line reader, several threads
    if (hcount > 0) {
        // their entry numbers and byte spans (gathered on the device)
        std::vector<long long> hts(hcount), spans(2 * hcount);
        long long *dspan = static_cast<long long *>(dalloc(2 * sizeof(long long) * hcount));
        if (!dspan) return cuda_fail(cudaErrorMemoryAllocation);
        e = mtx_host_spans(pool, (long long)hcount, hl, ends, dspan);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hts.data(), ht, sizeof(long long) * hcount, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(spans.data(), dspan, 2 * sizeof(long long) * hcount, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e);
        std::vector<int> hi(hcount), hj(hcount);
        std::vector<double> hv(hcount);
        std::atomic<int> malformed{0}, outside{0}, mirror{0};
        auto work = [&](size_t a, size_t b) {
            for (size_t k = a; k < b; ++k) {
                const char *q = data + spans[2 * k], *qe = data + spans[2 * k + 1];
                while (q < qe && (*q == ' ' || *q == '\t' || *q == '\r' || *q == '\v' || *q == '\f')) ++q;
                long long i = 0, j = 0;
                double v = 1.0;
                if (!mtx_line(q, qe, h.kind, i, j, v)) { malformed = 1; continue; }
                if (i < 1 || i > M || j < 1 || j > N) { outside = 1; continue; }
                if (h.symm && i != j && j - 1 >= M) mirror = 1;
                hi[k] = (int)(i - 1);
                hj[k] = (int)(j - 1);
                hv[k] = v;
            }
        };
        const size_t nt = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()),
                                           std::max<size_t>(1, hcount / 65536));
        std::vector<std::thread> th;
        for (size_t k = 1; k < nt; ++k) th.emplace_back(work, hcount * k / nt, hcount * (k + 1) / nt);
        work(0, hcount / nt);
        for (auto &t : th) t.join();
        if (malformed) { release(); return host_path(); }
        if (outside) hbad[0] = 1;
        if (mirror) hbad[1] = 1;
        long long *dht = static_cast<long long *>(dalloc(sizeof(long long) * hcount));
        int *dhi = static_cast<int *>(dalloc(sizeof(int) * hcount));
        int *dhj = static_cast<int *>(dalloc(sizeof(int) * hcount));
        double *dhv = static_cast<double *>(dalloc(sizeof(double) * hcount));
        if (!dht || !dhi || !dhj || !dhv) return cuda_fail(cudaErrorMemoryAllocation);
        e = cudaMemcpyAsync(dht, hts.data(), sizeof(long long) * hcount, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dhi, hi.data(), sizeof(int) * hcount, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dhj, hj.data(), sizeof(int) * hcount, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dhv, hv.data(), sizeof(double) * hcount, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = mtx_patch(pool, (long long)hcount, dht, dhi, dhj, dhv, ri, ci, vv);
        if (e != cudaSuccess) return cuda_fail(e);
    }
    // the host loader's checks, in its order
    if (hbad[0]) return mtx_fail("entry index outside the matrix");
    if (total < NZ) return mtx_fail("truncated data line");
    if (hbad[1]) return mtx_fail("symmetric entry mirrored outside the matrix");
    // the entries and their mirrors in file order -> stable sort by row
    int *cnt = static_cast<int *>(dalloc(sizeof(int) * (size_t)NZ1));
    long long *eoff = static_cast<long long *>(dalloc(sizeof(long long) * (size_t)(NZ + 1)));
    if (!cnt || !eoff) return cuda_fail(cudaErrorMemoryAllocation);
    long long E = 0;
    e = mtx_emit(pool, ri, ci, NZ, h.symm, cnt, eoff, ctx->dflags);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&E, eoff + NZ, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e);
    if (E > INT32_MAX) { release(); return fail(TSG_ERR_NOT_SUPPORTED, "more than 2^31-1 entries after mirroring"); }
    const long long E1 = std::max(E, 1ll);
    int *key = static_cast<int *>(dalloc(sizeof(int) * (size_t)E1));
    int *ecol = static_cast<int *>(dalloc(sizeof(int) * (size_t)E1));
    double *eval = static_cast<double *>(dalloc(sizeof(double) * (size_t)E1));
    long long *rp1 = static_cast<long long *>(dalloc(2 * sizeof(long long)));
    long long *tp = static_cast<long long *>(dalloc(sizeof(long long) * (size_t)(M + 1)));
    int *tcol = static_cast<int *>(dalloc(sizeof(int) * (size_t)E1));
    int *perm = static_cast<int *>(dalloc(sizeof(int) * (size_t)E1));
    int *rp32 = static_cast<int *>(pool.alloc(sizeof(int) * (size_t)(M + 1)));
    int *col = static_cast<int *>(pool.alloc(sizeof(int) * (size_t)E1));
    double *val = static_cast<double *>(pool.alloc(sizeof(double) * (size_t)E1));
    auto drop_out = [&]() { pool.free(rp32); pool.free(col); pool.free(val); };
    if (!key || !ecol || !eval || !rp1 || !tp || !tcol || !perm || !rp32 || !col || !val) {
        drop_out();
        return cuda_fail(cudaErrorMemoryAllocation);
    }
    const long long rp1h[2] = {0, E};
    e = mtx_emit_fill(pool, ri, ci, vv, NZ, h.symm, eoff, key, ecol, eval);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rp1, rp1h, sizeof(rp1h), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = csr_transpose(pool, rp1, key, eval, 1, (int)M, E, tp, tcol, val, perm, ctx->dflags);
    if (e == cudaSuccess) e = gather_i32(pool, perm, ecol, col, E);
    if (e == cudaSuccess) e = aux_rowptr_narrow(pool, tp, rp32, M + 1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { drop_out(); return cuda_fail(e); }
    r = host_wait(ctx, nullptr);   // the scans' bounded waits
    if (r) { drop_out(); release(); return r; }
    release();
    OutOwner *o = new OutOwner();
    o->ctx = ctx;
    o->where = TSG_MEM_DEVICE;
    o->blocks = {{rp32, 0}, {col, 0}, {val, 0}};
    A->m = (int32_t)M; A->n = (int32_t)N; A->nnz = E; A->rowptr_bits = 32; A->where = TSG_MEM_DEVICE;
    A->row_ptr = rp32; A->col = col; A->val = val; A->owner = o;
    if (is_symmetric) *is_symmetric = h.symm ? 1 : 0;
    return TSG_OK;
}

tsg_status tsg_csr_download_rows(tsg_ctx *ctx, const tsg_csr *M, int32_t r0, int32_t r1, int64_t *row_ptr,
                                 int32_t *col, double *val)
{
    if (!M || !row_ptr) return fail(TSG_ERR_INVALID_ARG, "M/row_ptr is NULL");
    if (r0 < 0 || r1 < r0 || r1 > M->m) return fail(TSG_ERR_INVALID_ARG, "rows [%d, %d) are not inside [0, %d)", r0, r1, M->m);
    if (M->rowptr_bits != 32 && M->rowptr_bits != 64) return fail(TSG_ERR_INVALID_ARG, "M.rowptr_bits must be 32 or 64");
    const bool dev = M->where == TSG_MEM_DEVICE;
    if (dev && !ctx) return fail(TSG_ERR_INVALID_ARG, "device matrix needs a context");
    if (ctx) CUDA_OK(cudaSetDevice(ctx->device));
    const int w = M->rowptr_bits == 64 ? 8 : 4;
    const size_t n = (size_t)(r1 - r0) + 1;
    const char *src = static_cast<const char *>(M->row_ptr) + (size_t)r0 * w;
    if (w == 8) {
        if (dev) CUDA_OK(cudaMemcpy(row_ptr, src, 8 * n, cudaMemcpyDeviceToHost));
        else memcpy(row_ptr, src, 8 * n);
    } else {
        std::vector<int> tmp(n);
        if (dev) CUDA_OK(cudaMemcpy(tmp.data(), src, 4 * n, cudaMemcpyDeviceToHost));
        else memcpy(tmp.data(), src, 4 * n);
        for (size_t i = 0; i < n; ++i) row_ptr[i] = tmp[i];
    }
    const long long e0 = row_ptr[0], e1 = row_ptr[n - 1];
    if (e0 < 0 || e1 < e0 || e1 > M->nnz)
        return fail(TSG_ERR_BAD_INPUT, "row pointers of rows [%d, %d) give entries [%lld, %lld) outside [0, %lld)", r0, r1,
                    e0, e1, (long long)M->nnz);
    const size_t cnt = (size_t)(e1 - e0);
    if (cnt == 0) return TSG_OK;
    if (col) {
        if (dev) CUDA_OK(cudaMemcpy(col, M->col + e0, sizeof(int) * cnt, cudaMemcpyDeviceToHost));
        else memcpy(col, M->col + e0, sizeof(int) * cnt);
    }
    if (val) {
        if (dev) CUDA_OK(cudaMemcpy(val, M->val + e0, sizeof(double) * cnt, cudaMemcpyDeviceToHost));
        else memcpy(val, M->val + e0, sizeof(double) * cnt);
    }
    return TSG_OK;
}


}  // extern "C"

// ---- tile form --------------------------------------------------------------

namespace {
struct TilesOwner {
    tsg_ctx *ctx = nullptr;
    std::vector<void *> blocks;
};

void reset_dev_state(tsg_ctx *ctx)
{
    cudaMemsetAsync(ctx->dstat, 0, sizeof(long long) * ST_SLOTS, ctx->stream);   // the flags inside it too
}

__global__ void k_widen_i32(const int *in, long long *out, long long n)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}
}  // namespace

extern "C" {

tsg_status tsg_tiles_free(tsg_ctx *ctx, tsg_tiles *T)
{
    if (!T) return TSG_OK;
    TilesOwner *o = static_cast<TilesOwner *>(T->owner);
    if (o) {
        tsg_ctx *c = o->ctx ? o->ctx : ctx;
        if (c) {
            cudaSetDevice(c->device);
            for (void *b : o->blocks) cudaFreeAsync(b, c->stream);
            cudaStreamSynchronize(c->stream);
        }
        delete o;
    }
    memset(T, 0, sizeof(*T));
    return TSG_OK;
}

tsg_status tsg_csr_to_tiles(tsg_ctx *ctx, const tsg_csr *A, tsg_tiles *T)
{
    if (!ctx || !T) return fail(TSG_ERR_INVALID_ARG, "ctx/T is NULL");
    tsg_status r = check_csr(A, "A");
    if (r) return r;
    CUDA_OK(cudaSetDevice(ctx->device));
    memset(T, 0, sizeof(*T));
    Pool pool{ctx->pool, ctx->stream};
    TilesOwner *o = new TilesOwner();
    o->ctx = ctx;
    T->owner = o;
    {
        Scratch sc(pool);
        reset_dev_state(ctx);
        DevCSR dA;
        r = stage_operand(ctx, pool, sc, A, ctx->opts.validate != 0, dA);
        TileCSR TA;
        if (!r) r = build_tiles(pool, sc, dA, TA, ctx);
        if (!r) {
            // dstat was zeroed, so the int32 count lands as a valid int64 (little-endian)
            cudaMemcpyAsync(ctx->dstat + ST_TILESB, TA.trp + TA.blkm, sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream);
            r = host_wait(ctx, nullptr);
        }
        if (!r) {
            const long long nb = ctx->hstat[ST_TILESB];
            T->m = dA.m; T->n = dA.n; T->blkm = TA.blkm; T->blkn = TA.blkn; T->numblk = nb; T->nnz = dA.nnz;
            auto get = [&](size_t bytes) { void *p = pool.alloc(bytes); if (p) o->blocks.push_back(p); return p; };
            T->blkrowptr = (int64_t *)get(sizeof(int64_t) * (TA.blkm + 1));
            T->blkcolidx = (int32_t *)get(sizeof(int32_t) * (size_t)(nb + 1));
            T->mask = (uint16_t *)get(sizeof(uint16_t) * (size_t)(nb * TILE + 2));
            T->nnzb = (int64_t *)get(sizeof(int64_t) * (size_t)(nb + 1));
            T->ptr = (uint8_t *)get((size_t)(nb * TILE + 16));
            T->col = (uint8_t *)get((size_t)(dA.nnz + 16));
            T->val = (double *)get(sizeof(double) * (size_t)(dA.nnz + 1));
            if (o->blocks.size() != 7) r = fail(TSG_ERR_OOM, "device pool allocation failed for tiles");
            if (!r) {
                { k_widen_i32<<<(unsigned)((TA.blkm + 1 + 255) / 256), 256, 0, ctx->stream>>>(TA.trp, (long long *)T->blkrowptr, TA.blkm + 1); ::tsg::count_launch(); }
                cudaMemcpyAsync(T->blkcolidx, TA.tcol, sizeof(int) * (size_t)nb, cudaMemcpyDeviceToDevice, ctx->stream);
                masks_to_tile_major_i32(pool, TA.blkm, TA.trp, TA.mask, T->mask);
                cudaError_t e = tiles_payload_a(pool, dA.m, dA.n, dA.rp, dA.col, dA.val, TA, nb, (long long *)T->nnzb,
                                                T->ptr, T->col, T->val, ctx->dflags);
                if (e != cudaSuccess) r = fail(cuda_status(e), "tile payload: %s", cudaGetErrorString(e));
            }
            if (!r) r = host_wait(ctx, nullptr);
        }
    }
    if (r) { tsg_tiles_free(ctx, T); cudaGetLastError(); }
    return r;
}

tsg_status tsg_spgemm_tiles(tsg_ctx *ctx, tsg_op op, const tsg_csr *A, const tsg_csr *B, tsg_tiles *C, tsg_stats *st)
{
    if (!ctx || !C) return fail(TSG_ERR_INVALID_ARG, "ctx/C is NULL");
    CUDA_OK(cudaSetDevice(ctx->device));
    memset(C, 0, sizeof(*C));
    if (st) memset(st, 0, sizeof(*st));
    Pool pool{ctx->pool, ctx->stream};
    PlanData P;
    PhaseTimer tm(ctx, false);
    int *col = nullptr;
    double *val = nullptr;
    tsg_status r;
    {
        Scratch sc(pool);
        r = plan_symbolic(ctx, pool, sc, op, A, B, P, false, st != nullptr && ctx->opts.count_products, tm);
        if (!r) {
            col = pool.alloc_n<int>(P.nnzC);
            val = pool.alloc_n<double>(P.nnzC);
            if (!col || !val) r = fail(TSG_ERR_OOM, "device pool allocation failed for C (%lld entries)", P.nnzC);
        }
        if (!r) r = plan_numeric(ctx, pool, P, P.valA, P.valB, col, val);
    }
    TilesOwner *o = new TilesOwner();
    o->ctx = ctx;
    C->owner = o;
    if (!r) {
        // hand C's tile structure over from the plan
        for (void *p : {(void *)P.crp, (void *)P.ccol}) { P.disown(p); o->blocks.push_back(p); }
        const long long nb = P.numblkC;
        C->m = P.m; C->n = P.n; C->blkm = P.blkm; C->blkn = ceil_div_i(P.n, TILE); C->numblk = nb; C->nnz = P.nnzC;
        C->blkrowptr = (int64_t *)P.crp; C->blkcolidx = P.ccol;
        auto get = [&](size_t bytes) { void *p = pool.alloc(bytes); if (p) o->blocks.push_back(p); return p; };
        C->mask = (uint16_t *)get(sizeof(uint16_t) * (size_t)(nb * TILE + 2));
        if (C->mask) masks_to_tile_major_i64(pool, P.blkm, P.crp, P.cmask, C->mask);
        C->nnzb = (int64_t *)get(sizeof(int64_t) * (size_t)(nb + 1));
        C->ptr = (uint8_t *)get((size_t)(nb * TILE + 16));
        C->col = (uint8_t *)get((size_t)(P.nnzC + 16));
        C->val = (double *)get(sizeof(double) * (size_t)(P.nnzC + 1));
        if (!C->mask || !C->nnzb || !C->ptr || !C->col || !C->val) r = fail(TSG_ERR_OOM, "device pool allocation failed for C tiles");
        if (!r) {
            cudaError_t e = tiles_from_csr_c(pool, P.m, P.blkm, nb, P.crp, P.ccol, P.cmask, P.rowptrC, col, val,
                                             (long long *)C->nnzb, C->ptr, C->col, C->val, ctx->dflags);
            if (e != cudaSuccess) r = fail(cuda_status(e), "tile payload of C: %s", cudaGetErrorString(e));
        }
        if (!r) r = host_wait(ctx, nullptr);
        fill_stats(P, st);
    }
    pool.free(col); pool.free(val);
    P.release(pool);   // after the values' upload, if it is still running
    if (r) tsg_tiles_free(ctx, C);
    cudaStreamSynchronize(ctx->stream);
    cudaGetLastError();
    return r;
}

tsg_status tsg_tiles_to_csr(tsg_ctx *ctx, const tsg_tiles *T, tsg_csr *C)
{
    if (!ctx || !T || !C) return fail(TSG_ERR_INVALID_ARG, "ctx/T/C is NULL");
    CUDA_OK(cudaSetDevice(ctx->device));
    Pool pool{ctx->pool, ctx->stream};
    reset_dev_state(ctx);
    long long *rowptr = pool.alloc_n<long long>(T->m + 1);
    if (!rowptr) return fail(TSG_ERR_OOM, "device pool allocation failed");
    CUDA_OK(csr_from_tiles(pool, T->m, (const long long *)T->blkrowptr, T->blkcolidx, (const long long *)T->nnzb,
                           T->ptr, T->col, T->val, rowptr, nullptr, nullptr, ctx->dflags, false));
    CUDA_OK(cudaMemcpyAsync(ctx->dstat + ST_NNZC, rowptr + T->m, sizeof(long long), cudaMemcpyDeviceToDevice, ctx->stream));
    tsg_status r = host_wait(ctx, nullptr);
    if (r) { pool.free(rowptr); return r; }
    const long long nnz = ctx->hstat[ST_NNZC];
    int *col = pool.alloc_n<int>(nnz);
    double *val = pool.alloc_n<double>(nnz);
    if (!col || !val) { pool.free(rowptr); pool.free(col); pool.free(val); return fail(TSG_ERR_OOM, "device pool allocation failed"); }
    CUDA_OK(csr_from_tiles(pool, T->m, (const long long *)T->blkrowptr, T->blkcolidx, (const long long *)T->nnzb,
                           T->ptr, T->col, T->val, rowptr, col, val, ctx->dflags, true));
    CUDA_OK(cudaStreamSynchronize(ctx->stream));
    OutOwner *o = new OutOwner();
    o->ctx = ctx;
    o->where = TSG_MEM_DEVICE;
    o->blocks = {{rowptr, 0}, {col, 0}, {val, 0}};
    C->m = T->m; C->n = T->n; C->nnz = nnz; C->rowptr_bits = 64; C->where = TSG_MEM_DEVICE;
    C->row_ptr = rowptr; C->col = col; C->val = val; C->owner = o;
    return TSG_OK;
}

tsg_status tsg_tiles_download(tsg_ctx *ctx, const tsg_tiles *T, int64_t *blkrowptr, int32_t *blkcolidx,
                              int64_t *nnzb, uint8_t *ptr, uint8_t *col, double *val, uint16_t *mask)
{
    if (!ctx || !T) return fail(TSG_ERR_INVALID_ARG, "ctx/T is NULL");
    CUDA_OK(cudaSetDevice(ctx->device));
    CUDA_OK(cudaStreamSynchronize(ctx->stream));
    const size_t nb = (size_t)T->numblk;
    if (blkrowptr) CUDA_OK(cudaMemcpy(blkrowptr, T->blkrowptr, sizeof(int64_t) * (size_t)(T->blkm + 1), cudaMemcpyDeviceToHost));
    if (nb && blkcolidx) CUDA_OK(cudaMemcpy(blkcolidx, T->blkcolidx, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost));
    if (nnzb) CUDA_OK(cudaMemcpy(nnzb, T->nnzb, sizeof(int64_t) * (nb + 1), cudaMemcpyDeviceToHost));
    if (nb && ptr) CUDA_OK(cudaMemcpy(ptr, T->ptr, nb * TILE, cudaMemcpyDeviceToHost));
    if (nb && mask) CUDA_OK(cudaMemcpy(mask, T->mask, sizeof(uint16_t) * nb * TILE, cudaMemcpyDeviceToHost));
    if (T->nnz && col) CUDA_OK(cudaMemcpy(col, T->col, (size_t)T->nnz, cudaMemcpyDeviceToHost));
    if (T->nnz && val) CUDA_OK(cudaMemcpy(val, T->val, sizeof(double) * (size_t)T->nnz, cudaMemcpyDeviceToHost));
    return TSG_OK;
}

}  // extern "C"

// ---- batched products ------------------------------------------------------

namespace {

inline long long round16(long long x) { return (x + 15) & ~15ll; }

// Stack `count` operands block-diagonally into one device CSR (rows and
// columns of every instance start on a multiple of 16).  rowoff/coloff give
// each instance's first packed row/column.
tsg_status pack_operands(tsg_ctx *ctx, Pool &pool, Scratch &sc, int count, const tsg_csr *M,
                         const std::vector<long long> &rowoff, const std::vector<long long> &coloff,
                         long long rows_total, long long cols_total, tsg_csr &packed)
{
    long long nnz = 0;
    std::vector<long long> nnzoff(count);
    for (int i = 0; i < count; ++i) { nnzoff[i] = nnz; nnz += M[i].nnz; }
    if (nnz >= (1ll << 31)) return fail(TSG_ERR_NOT_SUPPORTED, "batch operands hold %lld entries; the limit is 2^31-1", nnz);
    if (rows_total >= (1ll << 30) || cols_total >= (1ll << 30))
        return fail(TSG_ERR_NOT_SUPPORTED, "batch is larger than 2^30 rows or columns");
    long long *rp = sc.get<long long>(rows_total + 1);
    int *col = sc.get<int>(nnz);
    double *val = sc.get<double>(nnz);
    if (!rp || !col || !val) return fail(TSG_ERR_OOM, "device pool allocation failed for the packed batch");
    const bool host = M[0].where == TSG_MEM_HOST;
    if (host) {
        // pack on the host into pinned staging, then one copy per array
        const size_t rpb = sizeof(long long) * (size_t)(rows_total + 1);
        long long *hrp = (long long *)pinned_get(ctx, rpb);
        int *hcol = (int *)pinned_get(ctx, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
        double *hval = (double *)pinned_get(ctx, sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
        if (!hrp || !hcol || !hval) return fail(TSG_ERR_OOM, "pinned staging for the batch");
        bool bad = false;
        for (int i = 0; i < count; ++i) {
            const tsg_csr &X = M[i];
            const long long pad = (i + 1 < count ? rowoff[i + 1] : rows_total) - rowoff[i];
            auto rp_at = [&](long long r) -> long long {
                return X.rowptr_bits == 64 ? ((const long long *)X.row_ptr)[r] : (long long)((const int *)X.row_ptr)[r];
            };
            if (rp_at(X.m) != X.nnz) bad = true;
            for (long long r = 0; r < pad; ++r) {
                long long v = X.nnz;                      // padding rows repeat the end
                if (r < X.m) {
                    v = rp_at(r);
                    if (v < 0 || v > X.nnz || (r == 0 && v != 0)) { bad = true; v = v < 0 ? 0 : (v > X.nnz ? X.nnz : v); }
                }
                hrp[rowoff[i] + r] = nnzoff[i] + v;
            }
            for (long long q = 0; q < X.nnz; ++q) {
                int c = X.col[q];
                if ((unsigned)c >= (unsigned)X.n) { bad = true; c = 0; }
                hcol[nnzoff[i] + q] = (int)(c + coloff[i]);
            }
            if (X.nnz > 0) memcpy(hval + nnzoff[i], X.val, sizeof(double) * (size_t)X.nnz);
        }
        hrp[rows_total] = nnz;
        for (long long r = 1; r <= rows_total && !bad; ++r) if (hrp[r] < hrp[r - 1]) bad = true;
        cudaError_t e = cudaMemcpyAsync(rp, hrp, rpb, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && nnz > 0) e = cudaMemcpyAsync(col, hcol, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && nnz > 0) e = cudaMemcpyAsync(val, hval, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        pinned_put(ctx, hrp, rpb);
        pinned_put(ctx, hcol, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
        pinned_put(ctx, hval, sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
        if (e != cudaSuccess) return fail(cuda_status(e), "batch upload: %s", cudaGetErrorString(e));
        if (bad) return fail(TSG_ERR_BAD_INPUT, "an instance's row pointer or column index is out of range");
    } else {
        std::vector<PackDesc> d(count);
        for (int i = 0; i < count; ++i) {
            const tsg_csr &X = M[i];
            d[i].rp = X.row_ptr; d[i].col = X.col; d[i].val = X.val; d[i].rp_bits = X.rowptr_bits;
            d[i].m = X.m; d[i].n = X.n; d[i].nnz = X.nnz; d[i].rowoff = rowoff[i];
            d[i].rowpad = (i + 1 < count ? rowoff[i + 1] : rows_total) - rowoff[i];
            d[i].coloff = coloff[i]; d[i].nnzoff = nnzoff[i];
        }
        PackDesc *dd = sc.get<PackDesc>(count);
        if (!dd) return fail(TSG_ERR_OOM, "device pool allocation failed");
        CUDA_OK(cudaMemcpyAsync(dd, d.data(), sizeof(PackDesc) * (size_t)count, cudaMemcpyHostToDevice, ctx->stream));
        long long most = 0;
        for (int i = 0; i < count; ++i) most = std::max<long long>(most, std::max<long long>(M[i].nnz, d[i].rowpad));
        const int per = (int)std::min<long long>(64, std::max<long long>(1, (most + 8191) / 8192));
        CUDA_OK(batch_pack(pool, dd, count, per, rp, col, val, ctx->dflags));
        CUDA_OK(cudaMemcpyAsync(rp + rows_total, &nnz, sizeof(long long), cudaMemcpyHostToDevice, ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));   // the descriptor and the end value are host stack memory
    }
    packed = tsg_csr{};
    packed.m = (int)rows_total; packed.n = (int)cols_total; packed.nnz = nnz;
    packed.rowptr_bits = 64; packed.where = TSG_MEM_DEVICE;
    packed.row_ptr = rp; packed.col = col; packed.val = val;
    return TSG_OK;
}

}  // namespace

extern "C" {

tsg_status tsg_spgemm_batched(tsg_ctx *ctx, tsg_op op, int32_t count, const tsg_csr *A, const tsg_csr *B,
                              tsg_csr *C, tsg_stats *st)
{
    if (!ctx || !C || (count > 0 && !A)) return fail(TSG_ERR_INVALID_ARG, "ctx/A/C is NULL");
    if (count < 0) return fail(TSG_ERR_INVALID_ARG, "negative count");
    if (op == TSG_OP_AB && count > 0 && !B) return fail(TSG_ERR_INVALID_ARG, "B is NULL for A*B");
    if (C[0].where != TSG_MEM_HOST && C[0].where != TSG_MEM_DEVICE) return fail(TSG_ERR_INVALID_ARG, "C[0].where is not a tsg_mem");
    if (st) memset(st, 0, sizeof(*st));
    if (count == 0) return TSG_OK;
    auto t0 = std::chrono::steady_clock::now();
    CUDA_OK(cudaSetDevice(ctx->device));
    for (int i = 0; i < count; ++i) {
        tsg_status r = check_op(op, &A[i], op == TSG_OP_AB ? &B[i] : nullptr);
        if (r) return r;
        if (A[i].where != A[0].where || (op == TSG_OP_AB && B[i].where != A[0].where))
            return fail(TSG_ERR_INVALID_ARG, "all batch operands must be host, or all device");
        if (A[i].nnz > 0 && !A[i].val) return fail(TSG_ERR_INVALID_ARG, "instance %d has no values", i);
    }
    // layout: rows of A (and C), columns of A (= rows of B), columns of B (and C)
    std::vector<long long> roff(count), koff(count), noff(count);
    long long M = 0, K = 0, N = 0;
    for (int i = 0; i < count; ++i) {
        roff[i] = M; M += round16(A[i].m);
        koff[i] = K; K += round16(A[i].n);
        const int ni = op == TSG_OP_AB ? B[i].n : (op == TSG_OP_AA ? A[i].n : A[i].m);
        noff[i] = N; N += round16(ni);
    }
    Pool pool{ctx->pool, ctx->stream};
    PlanData P;
    PhaseTimer tm(ctx, st && ctx->opts.phase_times);
    int *col = nullptr;
    double *val = nullptr;
    tsg_status r;
    {
        Scratch sc(pool);
        CUDA_OK(cudaMemsetAsync(ctx->dflags, 0, sizeof(int) * FLAG_COUNT, ctx->stream));
        tsg_csr pA{}, pB{};
        r = pack_operands(ctx, pool, sc, count, A, roff, op == TSG_OP_AAT ? koff : (op == TSG_OP_AA ? roff : koff),
                          M, op == TSG_OP_AA ? M : K, pA);
        if (!r && op == TSG_OP_AB) r = pack_operands(ctx, pool, sc, count, B, koff, noff, K, N, pB);
        if (!r) r = plan_symbolic(ctx, pool, sc, op, &pA, op == TSG_OP_AB ? &pB : nullptr, P, false, st != nullptr && ctx->opts.count_products, tm,
                                  false);
        // C's column offset of each packed tile-row's instance: the numeric
        // step writes C_i's columns already rebased
        long long rpn = 0;
        std::vector<UnpackDesc> ud(count);
        std::vector<int> trc((size_t)(M / TILE) + 1, 0);
        for (int i = 0; i < count; ++i) {
            ud[i].rowoff = roff[i]; ud[i].m = A[i].m;
            ud[i].coloff = op == TSG_OP_AAT ? roff[i] : noff[i];
            ud[i].rpoff = rpn; rpn += A[i].m + 1;
            for (long long t = roff[i] / TILE; t < (roff[i] + round16(A[i].m)) / TILE; ++t) trc[(size_t)t] = (int)ud[i].coloff;
        }
        int *d_trc = nullptr;
        if (!r) {
            col = pool.alloc_n<int>(P.nnzC);
            val = pool.alloc_n<double>(P.nnzC);
            d_trc = sc.get<int>((long long)trc.size());
            if (!col || !val || !d_trc) r = fail(TSG_ERR_OOM, "device pool allocation failed for C (%lld entries)", P.nnzC);
        }
        if (!r) {
            CUDA_OK(cudaMemcpyAsync(d_trc, trc.data(), sizeof(int) * trc.size(), cudaMemcpyHostToDevice, ctx->stream));
            r = plan_numeric(ctx, pool, P, P.valA, P.valB, col, val, d_trc);
        }
        tm.mark();  // 4
        // unpack: per-instance row pointers, rebased
        int bits = ctx->opts.out_rowptr_bits;
        if (bits == 0) bits = P.nnzC < (1ll << 31) ? 32 : 64;
        if (!r && bits == 32 && P.nnzC >= (1ll << 31)) r = fail(TSG_ERR_INT32_OVERFLOW, "batch C needs int64 row pointers");
        void *rp_out = nullptr;
        long long *ebase = nullptr;
        if (!r) {
            rp_out = pool.alloc((size_t)rpn * (bits == 64 ? 8 : 4));
            ebase = sc.get<long long>(count);
            UnpackDesc *dud = sc.get<UnpackDesc>(count);
            if (!rp_out || !ebase || !dud) r = fail(TSG_ERR_OOM, "device pool allocation failed (batch outputs)");
            if (!r) {
                CUDA_OK(cudaMemcpyAsync(dud, ud.data(), sizeof(UnpackDesc) * (size_t)count, cudaMemcpyHostToDevice, ctx->stream));
                CUDA_OK(batch_unpack(pool, dud, count, P.rowptrC, rp_out, bits, ebase));
            }
        }
        std::vector<long long> eb(count);
        if (!r) {
            CUDA_OK(cudaMemcpyAsync(eb.data(), ebase, sizeof(long long) * (size_t)count, cudaMemcpyDeviceToHost, ctx->stream));
            CUDA_OK(cudaStreamSynchronize(ctx->stream));
            int hflags[FLAG_COUNT];
            CUDA_OK(cudaMemcpy(hflags, ctx->dflags, sizeof(hflags), cudaMemcpyDeviceToHost));
            if (hflags[FLAG_BAD_INPUT]) r = fail(TSG_ERR_BAD_INPUT, "an instance's row pointer or column index is out of range");
            else if (hflags[FLAG_INTERNAL]) r = fail(TSG_ERR_CUDA, "internal bound check failed on the device");
        }
        if (!r) {
            OutOwner *o = new OutOwner();
            o->ctx = ctx;
            o->refs = count;
            o->where = C[0].where;
            const int w = bits == 64 ? 8 : 4;
            char *hrp = nullptr;
            int *hcol = nullptr;
            double *hval = nullptr;
            if (C[0].where == TSG_MEM_DEVICE) {
                o->blocks = {{rp_out, 0}, {col, 0}, {val, 0}};
            } else {
                const size_t rpb = (size_t)rpn * w, cb = sizeof(int) * (size_t)P.nnzC, vb = sizeof(double) * (size_t)P.nnzC;
                hrp = (char *)pinned_get(ctx, rpb);
                hcol = (int *)pinned_get(ctx, cb);
                hval = (double *)pinned_get(ctx, vb);
                cudaError_t e = (hrp && hcol && hval) ? cudaSuccess : cudaErrorMemoryAllocation;
                if (e == cudaSuccess) e = cudaMemcpyAsync(hrp, rp_out, rpb, cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess && P.nnzC) e = cudaMemcpyAsync(hcol, col, cb, cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess && P.nnzC) e = cudaMemcpyAsync(hval, val, vb, cudaMemcpyDeviceToHost, ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                pool.free(rp_out); pool.free(col); pool.free(val);
                col = nullptr; val = nullptr; rp_out = nullptr;
                if (hrp) o->blocks.push_back({hrp, rpb});
                if (hcol) o->blocks.push_back({hcol, cb});
                if (hval) o->blocks.push_back({hval, vb});
                if (e != cudaSuccess) {
                    o->refs = 1;
                    tsg_csr tmp{};
                    tmp.owner = o;
                    tsg_csr_free(ctx, &tmp);
                    r = fail(cuda_status(e), "batch output copy: %s", cudaGetErrorString(e));
                }
            }
            if (!r) {
                char *rpbase = C[0].where == TSG_MEM_DEVICE ? (char *)rp_out : hrp;
                int *colbase = C[0].where == TSG_MEM_DEVICE ? col : hcol;
                double *valbase = C[0].where == TSG_MEM_DEVICE ? val : hval;
                for (int i = 0; i < count; ++i) {
                    const int ni = op == TSG_OP_AB ? B[i].n : (op == TSG_OP_AA ? A[i].n : A[i].m);
                    const long long nz_i = (i + 1 < count ? eb[i + 1] : P.nnzC) - eb[i];
                    C[i].m = A[i].m; C[i].n = ni; C[i].nnz = nz_i; C[i].rowptr_bits = bits; C[i].where = C[0].where;
                    C[i].row_ptr = rpbase + ud[i].rpoff * w;
                    C[i].col = colbase + eb[i];
                    C[i].val = valbase + eb[i];
                    C[i].owner = o;
                }
                col = nullptr; val = nullptr;
            }
        } else {
            pool.free(rp_out);
        }
    }
    if (r) {
        pool.free(col); pool.free(val);
        P.release(pool);
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
        return r;
    }
    fill_stats(P, st);
    P.release(pool);
    cudaStreamSynchronize(ctx->stream);
    if (st) {
        st->ms_total = ms_since(t0);
        phase_times(ctx, st, tm);
    }
    return TSG_OK;
}

}  // extern "C"

// ---- tile form -> CSR without allocation -----------------------------------
//
// tsg_tiles_to_csr_noalloc runs the two passes of tsg_tiles_to_csr (row counts
// and their scan, then the fill) with its scratch in one file-scope device
// array instead of the context's pool, and writes into caller buffers.
// Scratch layout (bytes), sized for TSG_NOALLOC_MAX_ROWS rows:
//   [0, 32)        device error flags (FLAG_COUNT int32)
//   [128, 132)     scan ticket
//   [256, 4352)    scan look-back status, one uint64 per 2048 rows
//   [4352, ...)    row counts, int32, one per row
namespace {

constexpr long long NA_FLAGS_OFF = 0;
constexpr long long NA_TICKET_OFF = 128;
constexpr long long NA_STATUS_OFF = 256;
constexpr long long NA_STATUS_BYTES = 8ll * ((TSG_NOALLOC_MAX_ROWS + 2047) / 2048);
constexpr long long NA_ROWCNT_OFF = NA_STATUS_OFF + NA_STATUS_BYTES;
constexpr long long NA_SCRATCH_BYTES = (NA_ROWCNT_OFF + 4ll * (TSG_NOALLOC_MAX_ROWS + 1) + 255) / 256 * 256;
static_assert(NA_ROWCNT_OFF % 256 == 0, "row counts start on a 256-byte boundary");
static_assert(FLAG_COUNT * 4 <= NA_TICKET_OFF, "flags fit before the ticket");

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mu;
char *g_na_addr[NA_MAX_DEVICES] = {};

}  // namespace

static __device__ __align__(256) unsigned char tsg_noalloc_scratch[NA_SCRATCH_BYTES];

namespace {

// Device address of the scratch array on `device` (current), resolved with
// cudaGetSymbolAddress at the first call on the device and kept.  Creating
// a context on the device drops the kept address (noalloc_forget), so the
// first call after it resolves it again: a context cannot outlive a reset
// of its device (cudaDeviceReset ends its streams and pool), and after a
// reset the module is loaded anew and the array may sit elsewhere.
tsg_status noalloc_scratch(int device, char **out)
{
    if (device < 0 || device >= NA_MAX_DEVICES) return fail(TSG_ERR_NOT_SUPPORTED, "device %d: no-alloc scratch covers devices 0-%d", device, NA_MAX_DEVICES - 1);
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, tsg_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(TSG_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch) on device %d: %s", device,
                        cudaGetErrorString(e));
        }
        g_na_addr[device] = static_cast<char *>(p);
    }
    *out = g_na_addr[device];
    return TSG_OK;
}

// p is memory that kernels launched on `device` may write: device memory of
// that device, or managed memory (reachable from every device).  Device
// memory of another GPU is refused: without peer access the writes would
// fault, with it they would land on the other GPU.
}  // namespace

void tsg::noalloc_forget(int device)
{
    if (device < 0 || device >= NA_MAX_DEVICES) return;
    std::lock_guard<std::mutex> lk(g_na_mu);
    g_na_addr[device] = nullptr;
}

namespace {

bool is_device_pointer(const void *p, int device)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    if (a.type == cudaMemoryTypeDevice) return a.device == device;
    return a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" {

tsg_status tsg_tiles_to_csr_noalloc(tsg_ctx *ctx, const tsg_tiles *T, int64_t *row_ptr, int32_t *col, double *val)
{
    if (!ctx || !T || !row_ptr) return fail(TSG_ERR_INVALID_ARG, "ctx/T/row_ptr is NULL");
    if (T->m < 0 || T->n < 0 || T->nnz < 0 || T->numblk < 0) return fail(TSG_ERR_INVALID_ARG, "T has a negative size");
    if (T->m > TSG_NOALLOC_MAX_ROWS)
        return fail(TSG_ERR_NOT_SUPPORTED,
                    "tsg_tiles_to_csr_noalloc: T has %d rows, more than its static scratch holds "
                    "(TSG_NOALLOC_MAX_ROWS = %d); use tsg_tiles_to_csr", T->m, TSG_NOALLOC_MAX_ROWS);
    if (T->blkm != (T->m + TILE - 1) / TILE) return fail(TSG_ERR_INVALID_ARG, "T->blkm is not ceil(m/16)");
    if (T->m > 0 && (!T->blkrowptr || !T->nnzb || !T->ptr)) return fail(TSG_ERR_INVALID_ARG, "T's tile arrays are NULL");
    if (T->nnz > 0 && (!T->blkcolidx || !T->col || !T->val)) return fail(TSG_ERR_INVALID_ARG, "T's entry arrays are NULL");
    if (T->nnz > 0 && (!col || !val)) return fail(TSG_ERR_INVALID_ARG, "col/val is NULL for %lld entries", (long long)T->nnz);
    CUDA_OK(cudaSetDevice(ctx->device));
    const int dev = ctx->device;
    if (!is_device_pointer(row_ptr, dev) || (T->nnz > 0 && (!is_device_pointer(col, dev) || !is_device_pointer(val, dev))))
        return fail(TSG_ERR_INVALID_ARG, "row_ptr/col/val must be device memory of the context's device %d", dev);
    char *scr = nullptr;
    tsg_status r = noalloc_scratch(ctx->device, &scr);
    if (r) return r;
    const long long words = scan_status_words(T->m);
    if (8 * words > NA_STATUS_BYTES) return fail(TSG_ERR_CUDA, "no-alloc scan status does not fit its scratch");
    int *flags = reinterpret_cast<int *>(scr + NA_FLAGS_OFF);
    unsigned *ticket = reinterpret_cast<unsigned *>(scr + NA_TICKET_OFF);
    unsigned long long *status = reinterpret_cast<unsigned long long *>(scr + NA_STATUS_OFF);
    int *rowcnt = reinterpret_cast<int *>(scr + NA_ROWCNT_OFF);
    cudaStream_t s = ctx->stream;
    // flags, ticket and look-back status start at zero; the count pass writes every row count
    CUDA_OK(cudaMemsetAsync(scr, 0, (size_t)(NA_STATUS_OFF + 8 * words), s));
    const long long *brp = reinterpret_cast<const long long *>(T->blkrowptr);
    const long long *nnzb = reinterpret_cast<const long long *>(T->nnzb);
    long long *rp = reinterpret_cast<long long *>(row_ptr);
    CUDA_OK(csr_rowcnt_from_tiles(s, T->m, brp, nnzb, T->ptr, rowcnt));
    CUDA_OK(scan_i32_to_i64_in(s, rowcnt, rp, T->m, flags, ticket, status));
    long long total = 0;
    int hflags[FLAG_COUNT];
    CUDA_OK(cudaMemcpyAsync(&total, rp + T->m, sizeof(total), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaStreamSynchronize(s));
    if (hflags[FLAG_TIMEOUT]) return fail(TSG_ERR_DEVICE_TIMEOUT, "a bounded device wait gave up");
    if (hflags[FLAG_INTERNAL] || hflags[FLAG_OVERFLOW]) return fail(TSG_ERR_CUDA, "internal bound check failed on the device");
    // the fill writes exactly `total` entries: it must be the size of the caller's col/val
    if (total != T->nnz)
        return fail(TSG_ERR_BAD_INPUT, "T's tiles hold %lld entries but T->nnz is %lld", total, (long long)T->nnz);
    CUDA_OK(csr_fill_from_tiles(s, T->m, brp, T->blkcolidx, nnzb, T->ptr, T->col, T->val, rp, col, val));
    CUDA_OK(cudaStreamSynchronize(s));
    return TSG_OK;
}

}  // extern "C"

// ---- plans: batched plans, resident results, tuning, graph replay ------------
//
// A plan's numeric step can run entirely on the device: tsg_plan_set_values
// puts new operand values into the plan's resident buffers, tsg_plan_replay
// launches the numeric step (for A*A^T also the gather of A^T's values, for a
// batched plan also the per-instance row pointers) into the plan's resident
// C as one CUDA graph, captured at the first replay, and tsg_plan_result
// hands out device views of C.  tsg_plan_tune times the numeric step's
// variants (threads per tile-row CTA, row walk) on the plan and keeps the
// fastest; all variants give the same bits.

namespace {

// the numeric step of a plan on its resident values into its resident C;
// stream-ordered, no allocation and no host wait (so it can be captured)
// Bin the plan's C tile-rows again with other thresholds (the structure is
// kept; only the bins, their work lists and statistics change).  One host
// wait: the numeric launches need the bins' sizes on the host.
tsg_status plan_rebin(tsg_ctx *ctx, Pool &pool, tsg_plan *pl, int dense_tile_min, int smem_acc_max, int row_acc_max)
{
    PlanData &P = pl->P;
    NumericBinParams bp{dense_tile_min, smem_acc_max, row_acc_max, P.rpA, ctx->opts.rows_global};
    CUDA_OK(cudaMemsetAsync(ctx->dstat + ST_BINS, 0, sizeof(long long) * BS_SLOTS, ctx->stream));
    CUDA_OK(bin_tilerows(pool, P.blkm, P.m, P.crp, P.ccol, P.rowptrC, bp, P.bin, ctx->dstat + ST_BINS, P.binlist,
                         P.rowlist));
    CUDA_OK(cudaMemcpyAsync(ctx->hstat + ST_BINS, ctx->dstat + ST_BINS, sizeof(long long) * BS_SLOTS,
                            cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OK(cudaStreamSynchronize(ctx->stream));
    for (int b = 0; b < BS_SLOTS; ++b) P.bstat[b] = ctx->hstat[ST_BINS + b];
    pl->dense_tile_min = dense_tile_min;
    pl->smem_acc_max = smem_acc_max;
    pl->row_acc_max = row_acc_max;
    if (pl->gexec) { cudaGraphExecDestroy(pl->gexec); pl->gexec = nullptr; }
    return TSG_OK;
}

tsg_status plan_enqueue_numeric(tsg_ctx *ctx, Pool &pool, tsg_plan *pl, int threads, int walk)
{
    PlanData &P = pl->P;
    const double *va = P.valA_buf, *vb = nullptr;
    if (P.op == TSG_OP_AB) vb = P.valB_buf;
    else if (P.op == TSG_OP_AA) vb = va;
    else {
        CUDA_OK(aux_gather(pool, P.perm, va, P.valB_buf, P.nnzA));
        vb = P.valB_buf;
    }
    tsg_status r = plan_numeric(ctx, pool, P, va, vb, pl->rcol, pl->rval, pl->d_trc, threads, walk);
    if (r) return r;
    if (pl->count > 0) {
        CUDA_OK(batch_unpack(pool, pl->d_ud, pl->count, P.rowptrC, pl->rp_out, 64, pl->d_ebase));
    }
    return TSG_OK;
}

tsg_status plan_resident(tsg_plan *pl, Pool &pool)
{
    if (pl->rcol) return TSG_OK;
    pl->rcol = pl->P.own<int>(pool, pl->P.nnzC);
    pl->rval = pl->P.own<double>(pool, pl->P.nnzC);
    if (!pl->rcol || !pl->rval) return fail(TSG_ERR_OOM, "device pool allocation failed for the plan's C");
    return TSG_OK;
}

tsg_status plan_check_flags(tsg_ctx *ctx)
{
    int hflags[FLAG_COUNT];
    CUDA_OK(cudaMemcpy(hflags, ctx->dflags, sizeof(hflags), cudaMemcpyDeviceToHost));
    if (hflags[FLAG_INTERNAL]) return fail(TSG_ERR_CUDA, "internal bound check failed on the device");
    if (hflags[FLAG_BAD_INPUT]) return fail(TSG_ERR_BAD_INPUT, "an operand was out of range");
    return TSG_OK;
}

}  // namespace

extern "C" {

tsg_status tsg_plan_create_batched(tsg_ctx *ctx, tsg_op op, int32_t count, const tsg_csr *A, const tsg_csr *B,
                                   tsg_plan **plan, tsg_stats *st)
{
    if (!ctx || !plan || (count > 0 && !A)) return fail(TSG_ERR_INVALID_ARG, "ctx/A/plan is NULL");
    *plan = nullptr;
    if (count <= 0) return fail(TSG_ERR_INVALID_ARG, "a batched plan needs at least one instance");
    if (op == TSG_OP_AB && !B) return fail(TSG_ERR_INVALID_ARG, "B is NULL for A*B");
    if (st) memset(st, 0, sizeof(*st));
    auto t0 = std::chrono::steady_clock::now();
    CUDA_OK(cudaSetDevice(ctx->device));
    for (int i = 0; i < count; ++i) {
        tsg_status r = check_op(op, &A[i], op == TSG_OP_AB ? &B[i] : nullptr);
        if (r) return r;
        if (A[i].where != A[0].where || (op == TSG_OP_AB && B[i].where != A[0].where))
            return fail(TSG_ERR_INVALID_ARG, "all batch operands must be host, or all device");
        if (A[i].nnz > 0 && !A[i].val) return fail(TSG_ERR_INVALID_ARG, "instance %d has no values", i);
    }
    std::vector<long long> roff(count), koff(count), noff(count);
    long long M = 0, K = 0, N = 0;
    for (int i = 0; i < count; ++i) {
        roff[i] = M; M += round16(A[i].m);
        koff[i] = K; K += round16(A[i].n);
        const int ni = op == TSG_OP_AB ? B[i].n : (op == TSG_OP_AA ? A[i].n : A[i].m);
        noff[i] = N; N += round16(ni);
    }
    Pool pool{ctx->pool, ctx->stream};
    tsg_plan *pl = new tsg_plan();
    pl->ctx = ctx;
    pl->count = count;
    PlanData &P = pl->P;
    PhaseTimer tm(ctx, false);
    tsg_status r;
    {
        Scratch sc(pool);
        CUDA_OK(cudaMemsetAsync(ctx->dflags, 0, sizeof(int) * FLAG_COUNT, ctx->stream));
        tsg_csr pA{}, pB{};
        r = pack_operands(ctx, pool, sc, count, A, roff, op == TSG_OP_AAT ? koff : (op == TSG_OP_AA ? roff : koff),
                          M, op == TSG_OP_AA ? M : K, pA);
        if (!r && op == TSG_OP_AB) r = pack_operands(ctx, pool, sc, count, B, koff, noff, K, N, pB);
        if (!r) r = plan_symbolic(ctx, pool, sc, op, &pA, op == TSG_OP_AB ? &pB : nullptr, P, true, st != nullptr && ctx->opts.count_products, tm,
                                  false);
        if (!r) r = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? TSG_OK : fail(TSG_ERR_CUDA, "plan build failed");
    }
    if (!r) {
        pl->mi.resize(count); pl->ni.resize(count);
        pl->aoff.assign(count + 1, 0); pl->boff.assign(count + 1, 0);
        pl->rpoff.resize(count);
        std::vector<UnpackDesc> ud(count);
        std::vector<int> trc((size_t)(M / TILE) + 1, 0);
        long long rpn = 0;
        for (int i = 0; i < count; ++i) {
            pl->mi[i] = A[i].m;
            pl->ni[i] = op == TSG_OP_AB ? B[i].n : (op == TSG_OP_AA ? A[i].n : A[i].m);
            pl->aoff[i + 1] = pl->aoff[i] + A[i].nnz;
            pl->boff[i + 1] = pl->boff[i] + (op == TSG_OP_AB ? B[i].nnz : 0);
            ud[i].rowoff = roff[i]; ud[i].m = A[i].m;
            ud[i].coloff = op == TSG_OP_AAT ? roff[i] : noff[i];
            ud[i].rpoff = rpn;
            pl->rpoff[i] = rpn;
            rpn += A[i].m + 1;
            for (long long t = roff[i] / TILE; t < (roff[i] + round16(A[i].m)) / TILE; ++t) trc[(size_t)t] = (int)ud[i].coloff;
        }
        pl->d_trc = P.own<int>(pool, (long long)trc.size());
        pl->d_ud = P.own<UnpackDesc>(pool, count);
        pl->rp_out = P.own<long long>(pool, rpn);
        pl->d_ebase = P.own<long long>(pool, count);
        if (!pl->d_trc || !pl->d_ud || !pl->rp_out || !pl->d_ebase) r = fail(TSG_ERR_OOM, "device pool allocation failed (batched plan)");
        if (!r) {
            CUDA_OK(cudaMemcpyAsync(pl->d_trc, trc.data(), sizeof(int) * trc.size(), cudaMemcpyHostToDevice, ctx->stream));
            CUDA_OK(cudaMemcpyAsync(pl->d_ud, ud.data(), sizeof(UnpackDesc) * (size_t)count, cudaMemcpyHostToDevice, ctx->stream));
            CUDA_OK(batch_unpack(pool, pl->d_ud, count, P.rowptrC, pl->rp_out, 64, pl->d_ebase));
            pl->ebase.resize(count);
            CUDA_OK(cudaMemcpyAsync(pl->ebase.data(), pl->d_ebase, sizeof(long long) * (size_t)count, cudaMemcpyDeviceToHost, ctx->stream));
            CUDA_OK(cudaStreamSynchronize(ctx->stream));
            r = plan_check_flags(ctx);
        }
    }
    if (r) {
        P.release(pool);
        cudaStreamSynchronize(ctx->stream);
        cudaGetLastError();
        delete pl;
        return r;
    }
    fill_stats(P, st);
    if (st) st->ms_total = ms_since(t0);
    *plan = pl;
    return TSG_OK;
}

int32_t tsg_plan_count(const tsg_plan *plan) { return plan ? (plan->count > 0 ? plan->count : 1) : 0; }

tsg_status tsg_plan_set_values(tsg_ctx *ctx, tsg_plan *plan, const double *valA, const double *valB, int32_t where)
{
    if (!ctx || !plan) return fail(TSG_ERR_INVALID_ARG, "ctx/plan is NULL");
    if (plan->ctx != ctx) return fail(TSG_ERR_INVALID_ARG, "plan belongs to another context");
    if (where != TSG_MEM_HOST && where != TSG_MEM_DEVICE) return fail(TSG_ERR_INVALID_ARG, "where is not a tsg_mem");
    PlanData &P = plan->P;
    if (P.nnzA > 0 && !valA) return fail(TSG_ERR_INVALID_ARG, "valA is NULL");
    if (P.op == TSG_OP_AB && P.nnzB > 0 && !valB) return fail(TSG_ERR_INVALID_ARG, "valB is NULL for A*B");
    CUDA_OK(cudaSetDevice(ctx->device));
    const cudaMemcpyKind kind = where == TSG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (P.nnzA > 0) CUDA_OK(cudaMemcpyAsync(P.valA_buf, valA, sizeof(double) * (size_t)P.nnzA, kind, ctx->stream));
    if (P.op == TSG_OP_AB && P.nnzB > 0)
        CUDA_OK(cudaMemcpyAsync(P.valB_buf, valB, sizeof(double) * (size_t)P.nnzB, kind, ctx->stream));
    if (where == TSG_MEM_HOST) CUDA_OK(cudaStreamSynchronize(ctx->stream));   // the caller may reuse host memory
    return TSG_OK;
}

tsg_status tsg_plan_replay(tsg_ctx *ctx, tsg_plan *plan)
{
    if (!ctx || !plan) return fail(TSG_ERR_INVALID_ARG, "ctx/plan is NULL");
    if (plan->ctx != ctx) return fail(TSG_ERR_INVALID_ARG, "plan belongs to another context");
    CUDA_OK(cudaSetDevice(ctx->device));
    Pool pool{ctx->pool, ctx->stream};
    if (!plan->gexec) {
        tsg_status r = plan_resident(plan, pool);
        if (r) return r;
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
        CUDA_OK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const long long l0 = g_launches.load(std::memory_order_relaxed);
        cudaError_t me = cudaMemsetAsync(ctx->dflags, 0, sizeof(int) * FLAG_COUNT, ctx->stream);
        r = me == cudaSuccess ? plan_enqueue_numeric(ctx, pool, plan, plan->threads, plan->walk)
                              : fail(TSG_ERR_CUDA, "%s", cudaGetErrorString(me));
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        // launches issued while capturing run at each replay instead
        plan->glaunches = g_launches.load(std::memory_order_relaxed) - l0;
        g_launches.fetch_sub(plan->glaunches, std::memory_order_relaxed);
        if (!r && ce != cudaSuccess) r = fail(TSG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        if (!r) {
            const cudaError_t ie = cudaGraphInstantiate(&plan->gexec, graph, 0);
            if (ie != cudaSuccess) { plan->gexec = nullptr; r = fail(TSG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie)); }
        }
        if (graph) cudaGraphDestroy(graph);
        if (r) { cudaGetLastError(); return r; }
    }
    CUDA_OK(cudaGraphLaunch(plan->gexec, ctx->stream));
    g_launches.fetch_add(plan->glaunches, std::memory_order_relaxed);
    return TSG_OK;
}

tsg_status tsg_plan_result(tsg_ctx *ctx, tsg_plan *plan, int32_t instance, tsg_csr *C)
{
    if (!ctx || !plan || !C) return fail(TSG_ERR_INVALID_ARG, "ctx/plan/C is NULL");
    if (plan->ctx != ctx) return fail(TSG_ERR_INVALID_ARG, "plan belongs to another context");
    const int n = plan->count > 0 ? plan->count : 1;
    if (instance < 0 || instance >= n) return fail(TSG_ERR_INVALID_ARG, "instance %d out of range (%d)", instance, n);
    if (!plan->rcol) return fail(TSG_ERR_INVALID_ARG, "the plan has no result yet: call tsg_plan_replay");
    CUDA_OK(cudaSetDevice(ctx->device));
    CUDA_OK(cudaStreamSynchronize(ctx->stream));
    tsg_status r = plan_check_flags(ctx);
    if (r) return r;
    const PlanData &P = plan->P;
    *C = tsg_csr{};
    C->rowptr_bits = 64;
    C->where = TSG_MEM_DEVICE;
    C->owner = nullptr;   // a view of the plan's memory
    if (plan->count == 0) {
        C->m = P.m; C->n = P.n; C->nnz = P.nnzC;
        C->row_ptr = P.rowptrC; C->col = plan->rcol; C->val = plan->rval;
    } else {
        const long long e0 = plan->ebase[instance];
        const long long e1 = instance + 1 < plan->count ? plan->ebase[instance + 1] : P.nnzC;
        C->m = plan->mi[instance]; C->n = plan->ni[instance]; C->nnz = e1 - e0;
        C->row_ptr = plan->rp_out + plan->rpoff[instance];
        C->col = plan->rcol + e0; C->val = plan->rval + e0;
    }
    return TSG_OK;
}

tsg_status tsg_plan_value_offsets(const tsg_plan *plan, int64_t *a_offsets, int64_t *b_offsets)
{
    if (!plan) return fail(TSG_ERR_INVALID_ARG, "plan is NULL");
    const int n = plan->count > 0 ? plan->count : 1;
    for (int i = 0; i <= n; ++i) {
        if (a_offsets) a_offsets[i] = plan->count > 0 ? plan->aoff[i] : (i ? plan->P.nnzA : 0);
        if (b_offsets) b_offsets[i] = plan->count > 0 ? plan->boff[i] : (i ? (plan->P.op == TSG_OP_AB ? plan->P.nnzB : 0) : 0);
    }
    return TSG_OK;
}

tsg_status tsg_plan_tune(tsg_ctx *ctx, tsg_plan *plan, double *best_ms)
{
    if (!ctx || !plan) return fail(TSG_ERR_INVALID_ARG, "ctx/plan is NULL");
    if (plan->ctx != ctx) return fail(TSG_ERR_INVALID_ARG, "plan belongs to another context");
    CUDA_OK(cudaSetDevice(ctx->device));
    Pool pool{ctx->pool, ctx->stream};
    tsg_status r = plan_resident(plan, pool);
    if (r) return r;
    if (!plan->dense_tile_min) {   // bins as built: the context's thresholds
        plan->dense_tile_min = ctx->opts.dense_tile_min;
        plan->smem_acc_max = ctx->opts.smem_acc_max;
        plan->row_acc_max = ctx->opts.row_acc_max;
    }
    // mean of three timed runs after one warm-up run
    auto time_numeric = [&](int t, int w, float &ms_out) -> tsg_status {
        float tot = 0.f;
        for (int rep = 0; rep < 4; ++rep) {
            CUDA_OK(cudaEventRecord(ctx->ev[6], ctx->stream));
            tsg_status rr = plan_enqueue_numeric(ctx, pool, plan, t, w);
            if (rr) return rr;
            CUDA_OK(cudaEventRecord(ctx->ev[7], ctx->stream));
            CUDA_OK(cudaEventSynchronize(ctx->ev[7]));
            float ms = 0.f;
            CUDA_OK(cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]));
            if (rep > 0) tot += ms;
        }
        ms_out = tot / 3;
        return TSG_OK;
    };
    // 1. threads per tile-row CTA and row walk, on the plan's bins
    const int cand_threads[3] = {128, 256, 512};
    const int cand_walk[3] = {1, 2, 3};
    float best = 1e30f;
    int bt = plan->threads, bw = plan->walk;
    for (int t : cand_threads) {
        for (int w : cand_walk) {
            if (w != 2 && plan->P.dupsafe) continue;   // repeated B columns always take the packed walk
            float ms = 0.f;
            r = time_numeric(t, w, ms);
            if (r) return r;
            if (ms < best) { best = ms; bt = t; bw = w; }
        }
    }
    // 2. the bin thresholds -- which tile-rows take the dense accumulator,
    // which the shared-memory sparse one, which rows the row kernels -- with
    // those settings: every candidate bins the plan again and is timed
    struct Th { int dense, smem, row; };
    const Th base{plan->dense_tile_min, plan->smem_acc_max, plan->row_acc_max};
    const Th cand_th[5] = {{96, base.smem, base.row}, {257, base.smem, base.row}, {base.dense, 12288, base.row},
                           {base.dense, 65535, base.row}, {base.dense, base.smem, 16384}};
    Th bth = base;
    for (const Th &c : cand_th) {
        if (c.dense == base.dense && c.smem == base.smem && c.row == base.row) continue;
        r = plan_rebin(ctx, pool, plan, c.dense, c.smem, c.row);
        if (r) return r;
        float ms = 0.f;
        r = time_numeric(bt, bw, ms);
        if (r) return r;
        if (ms < best * 0.98f) { best = ms; bth = c; }
    }
    r = plan_rebin(ctx, pool, plan, bth.dense, bth.smem, bth.row);
    if (r) return r;
    r = plan_check_flags(ctx);
    if (r) return r;
    plan->threads = bt;
    plan->walk = bw;
    if (plan->gexec) { cudaGraphExecDestroy(plan->gexec); plan->gexec = nullptr; }
    if (best_ms) *best_ms = best;
    return TSG_OK;
}

tsg_status tsg_plan_settings(const tsg_plan *plan, int32_t *threads, int32_t *walk, int32_t *dense_tile_min,
                             int32_t *smem_acc_max, int32_t *row_acc_max)
{
    if (!plan) return fail(TSG_ERR_INVALID_ARG, "plan is NULL");
    const tsg_opts &o = plan->ctx->opts;
    if (threads) *threads = plan->threads > 0 ? plan->threads : o.threads_numeric;
    if (walk) *walk = plan->walk >= 0 ? plan->walk : o.numeric_walk;
    if (dense_tile_min) *dense_tile_min = plan->dense_tile_min ? plan->dense_tile_min : o.dense_tile_min;
    if (smem_acc_max) *smem_acc_max = plan->smem_acc_max ? plan->smem_acc_max : o.smem_acc_max;
    if (row_acc_max) *row_acc_max = plan->row_acc_max ? plan->row_acc_max : o.row_acc_max;
    return TSG_OK;
}

}  // extern "C"

extern "C" tsg_status tsg_tiles_spmv(tsg_ctx *ctx, const tsg_tiles *T, const double *x, double *y)
{
    if (!ctx || !T || !x || !y) return fail(TSG_ERR_INVALID_ARG, "ctx/T/x/y is NULL");
    if (T->m < 0 || T->n < 0 || T->blkm != (T->m + TILE - 1) / TILE) return fail(TSG_ERR_INVALID_ARG, "T is not a tile form");
    CUDA_OK(cudaSetDevice(ctx->device));
    CUDA_OK(tiles_spmv(ctx->stream, T->m, T->blkm, (const long long *)T->blkrowptr, T->blkcolidx,
                       (const long long *)T->nnzb, T->ptr, T->col, T->val, x, T->n, y));
    CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return TSG_OK;
}
