// tsg_scan.cu -- single-pass exclusive prefix scan (decoupled look-back).
//
// Replaces the reference's Thrust scans (utils_cuda_scan.h:249-314,
// spgemm_nsparse_kernel.h:1311), which allocate temporaries and synchronise,
// and its own single-pass scan whose look-back spins without a bound
// (utils_cuda_scan.h:167-170).  Here tiles take an atomic ticket, so a tile
// only ever waits on tiles that are already running; every wait is bounded
// (SPIN_LIMIT polls) and a wait that gives up sets FLAG_TIMEOUT and lets the
// kernel finish, so the host reports TSG_ERR_DEVICE_TIMEOUT instead of hanging.
//
// Roofline: HBM-bound, reads n inputs and writes n+1 outputs once.
#include "tsg_internal.cuh"

namespace tsg {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// status word: bits 62-63 = state (0 empty, 1 tile aggregate, 2 inclusive
// prefix), bits 0-61 = value.
constexpr unsigned long long ST_AGG = 1ull << 62;
constexpr unsigned long long ST_INC = 2ull << 62;
constexpr unsigned long long ST_VAL = (1ull << 62) - 1;

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(SCAN_THREADS)
k_scan(const Tin *__restrict__ in, Tout *__restrict__ out, long long n,
       unsigned long long *status, unsigned *ticket, int *flags, int spin_limit)
{
    __shared__ int s_tile;
    __shared__ long long s_warp[SCAN_THREADS / 32];
    __shared__ long long s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) s_tile = (int)atomicAdd(ticket, 1u);
    __syncthreads();
    const int tile = s_tile;
    const long long base = (long long)tile * SCAN_TILE + (long long)tid * SCAN_ITEMS;

    long long v[SCAN_ITEMS];
    long long tsum = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        long long idx = base + j;
        long long x = (idx < n) ? (long long)in[idx] : 0;
        if (x < 0) { set_flag(flags, FLAG_INTERNAL); x = 0; }
        v[j] = tsum;
        tsum += x;
    }
    // block-wide exclusive scan of the per-thread sums
    long long incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        long long w = (lane < SCAN_THREADS / 32) ? s_warp[lane] : 0;
        long long wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < SCAN_THREADS / 32) s_warp[lane] = wi - w;  // exclusive per warp
        long long aggregate = __shfl_sync(0xffffffffu, wi, SCAN_THREADS / 32 - 1);
        // publish and look back
        volatile unsigned long long *vst = status;
        long long exclusive = 0;
        if (tile == 0) {
            if (lane == 0) { __threadfence(); vst[0] = ST_INC | ((unsigned long long)aggregate & ST_VAL); }
        } else {
            if (lane == 0) { __threadfence(); vst[tile] = ST_AGG | ((unsigned long long)aggregate & ST_VAL); }
            int pred = tile - 1;
            bool done = false;
            while (!done) {
                int look = pred - lane;
                unsigned long long st = ST_INC;  // lanes before tile 0 act as an inclusive 0
                if (look >= 0) {
                    int spins = 0;
                    st = vst[look];
                    while ((st >> 62) == 0) {
                        if (++spins > spin_limit) { set_flag(flags, FLAG_TIMEOUT); st = ST_INC; break; }
                        __nanosleep(64);
                        st = vst[look];
                    }
                }
                unsigned inc_mask = __ballot_sync(0xffffffffu, (st >> 62) == 2);
                int first_inc = inc_mask ? __ffs(inc_mask) - 1 : 32;
                long long contrib = (lane <= first_inc) ? (long long)(st & ST_VAL) : 0;
                contrib = warp_sum_ll(contrib);
                exclusive += contrib;
                if (inc_mask) done = true;
                else pred -= 32;
            }
            if (lane == 0) {
                __threadfence();
                vst[tile] = ST_INC | ((unsigned long long)(exclusive + aggregate) & ST_VAL);
            }
        }
        if (lane == 0) s_prefix = exclusive;
        if (tile == (int)((n + SCAN_TILE - 1) / SCAN_TILE) - 1 && lane == 0) {
            long long total = exclusive + aggregate;
            out[n] = (Tout)total;
            if ((long long)(Tout)total != total) set_flag(flags, FLAG_OVERFLOW);
        }
    }
    __syncthreads();
    const long long off = s_prefix + s_warp[wid] + (incl - tsum);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        long long idx = base + j;
        if (idx < n) out[idx] = (Tout)(off + v[j]);
    }
}

template <typename Tout>
__global__ void k_scan_empty(Tout *out) { out[0] = 0; }

__global__ void k_fill_ones(int *a, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = 1;
}

template <typename Tin, typename Tout>
cudaError_t scan_impl(Pool &pool, const Tin *in, Tout *out, long long n, int *flags)
{
    if (n <= 0) {
        { k_scan_empty<Tout><<<1, 1, 0, pool.stream>>>(out); ::tsg::count_launch(); }
        return cudaGetLastError();
    }
    long long tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles > (1ll << 30)) return cudaErrorInvalidValue;
    size_t bytes = sizeof(unsigned long long) * (size_t)tiles + 16;
    char *scratch = static_cast<char *>(pool.alloc(bytes));
    if (!scratch) return pool.err;
    unsigned *ticket = reinterpret_cast<unsigned *>(scratch);
    unsigned long long *status = reinterpret_cast<unsigned long long *>(scratch + 16);
    cudaError_t e = cudaMemsetAsync(scratch, 0, bytes, pool.stream);
    if (e != cudaSuccess) { pool.free(scratch); return e; }
    { k_scan<Tin, Tout><<<(unsigned)tiles, SCAN_THREADS, 0, pool.stream>>>(in, out, n, status, ticket, flags, SPIN_LIMIT); ::tsg::count_launch(); }
    e = cudaGetLastError();
    pool.free(scratch);
    return e;
}

}  // namespace

cudaError_t scan_i32_to_i64(Pool &pool, const int *in, long long *out, long long n, int *flags)
{ return scan_impl<int, long long>(pool, in, out, n, flags); }
cudaError_t scan_i32_to_i32(Pool &pool, const int *in, int *out, long long n, int *flags)
{ return scan_impl<int, int>(pool, in, out, n, flags); }
cudaError_t scan_i64_to_i64(Pool &pool, const long long *in, long long *out, long long n, int *flags)
{ return scan_impl<long long, long long>(pool, in, out, n, flags); }

long long scan_status_words(long long n) { return n > 0 ? (n + SCAN_TILE - 1) / SCAN_TILE : 0; }

// The same scan with its look-back state in caller-provided device memory:
// `ticket` (one word) and `status` (scan_status_words(n) words), both zero on
// entry.  Allocates nothing.
cudaError_t scan_i32_to_i64_in(cudaStream_t s, const int *in, long long *out, long long n, int *flags,
                               unsigned *ticket, unsigned long long *status)
{
    if (n <= 0) {
        { k_scan_empty<long long><<<1, 1, 0, s>>>(out); ::tsg::count_launch(); }
        return cudaGetLastError();
    }
    const long long tiles = scan_status_words(n);
    if (tiles > (1ll << 30)) return cudaErrorInvalidValue;
    { k_scan<int, long long><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, n, status, ticket, flags, SPIN_LIMIT); ::tsg::count_launch(); }
    return cudaGetLastError();
}

// The bounded-wait check behind tsg_check_bounded_wait: the scan of n ones
// with the ticket starting at 1, so that no CTA takes tile 0 and tile 0's
// sum is never published.  Tile 1 (and every tile whose look-back reaches
// tile 0) waits for it until spin_limit polls, then sets FLAG_TIMEOUT and
// finishes.  Bounds: the grid has `tiles` CTAs, which take tiles 1..tiles,
// so `status` needs tiles + 1 words (the last CTA's tile publishes into word
// `tiles`; its items all lie past n and are neither read nor written).
cudaError_t scan_unpublished_tile(Pool &pool, long long n, int spin_limit, int *flags)
{
    if (n <= 0 || spin_limit < 1) return cudaErrorInvalidValue;
    const long long tiles = scan_status_words(n);
    if (tiles > (1ll << 20)) return cudaErrorInvalidValue;
    int *in = pool.alloc_n<int>(n);
    long long *out = pool.alloc_n<long long>(n + 1);
    char *scratch = static_cast<char *>(pool.alloc(16 + sizeof(unsigned long long) * (size_t)(tiles + 1)));
    cudaError_t e = (in && out && scratch) ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, 16 + sizeof(unsigned long long) * (size_t)(tiles + 1), pool.stream);
    if (e == cudaSuccess) { k_fill_ones<<<(unsigned)((n + 255) / 256), 256, 0, pool.stream>>>(in, n); ::tsg::count_launch(); }
    if (e == cudaSuccess) e = cudaGetLastError();
    unsigned *ticket = reinterpret_cast<unsigned *>(scratch);
    unsigned long long *status = reinterpret_cast<unsigned long long *>(scratch + 16);
    const unsigned one = 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(ticket, &one, sizeof(one), cudaMemcpyHostToDevice, pool.stream);
    if (e == cudaSuccess) {
        k_scan<int, long long><<<(unsigned)tiles, SCAN_THREADS, 0, pool.stream>>>(in, out, n, status, ticket, flags, spin_limit);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(pool.stream);   // `one` is host stack memory
    pool.free(in); pool.free(out); pool.free(scratch);
    return e;
}

}  // namespace tsg
