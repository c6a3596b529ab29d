// tsg_internal.cuh -- shared definitions of the GB300 tiled SpGEMM kernels.
//
// Layout in HBM (all device arrays come from the context's stream-ordered pool):
//   CSR operand   rp (int64, m+1, clamped copy of the caller's int32/int64
//                 pointer), col (int32, nnz), val (f64, nnz)
//   tile-CSR      trp (int32, blkm+1), tcol (int32, numblk, sorted per
//                 tile-row), mask (uint16, 16 per tile, bit 15-c for local
//                 column c -- main_spgemm-col.cu:5215)
//   C tiles       crp (int64, blkm+1), ccol (int32), cmask (uint16, 16 per tile)
//   C CSR         rowptr (int64, m+1), col (int32), val (f64)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tsg {

constexpr int TILE = 16;

// Device error flags (one int32 array per context, read back at the host
// waits).  Kernels never trap: they record and return.
enum DevFlag : int {
    FLAG_BAD_INPUT = 0,    // row pointer or column index out of range
    FLAG_TIMEOUT = 1,      // a bounded wait in the scan gave up
    FLAG_INTERNAL = 2,     // an internal bound check failed (a library bug)
    FLAG_OVERFLOW = 3,     // a count did not fit its index type
    FLAG_COUNT = 8
};

// Bounded-wait limit for the decoupled-lookback scan (spins with nanosleep;
// about a quarter second before giving up).
constexpr int SPIN_LIMIT = 1 << 22;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ int warp_min_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int warp_max_int(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Inclusive warp scan.
__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// OR a 16-bit row mask into the uint16 array viewed as 32-bit words (the
// arrays hold 16 masks per tile, so the word view is always in bounds).
__device__ __forceinline__ void atomic_or_mask16(uint16_t *mask, long long idx, unsigned bits) {
    unsigned *w = reinterpret_cast<unsigned *>(mask) + (idx >> 1);
    atomicOr(w, bits << ((idx & 1) * 16));
}

// first e in [lo, hi) with col[e] >= key (col sorted on [lo, hi)), probing
// lo, lo+1, lo+3, lo+7, ... before a binary search of the last gap
__device__ __forceinline__ int gallop_lower_bound(const int *__restrict__ col, int lo, int hi, int key)
{
    int step = 1, a = lo, b = hi;
    while (true) {
        const int probe = a + step - 1;
        if (probe >= hi) break;
        if (col[probe] >= key) { b = probe; break; }
        a = probe + 1;
        step <<= 1;
    }
    while (a < b) {
        const int md = (a + b) >> 1;
        if (col[md] < key) a = md + 1; else b = md;
    }
    return a;
}

// First index in [lo, hi) whose value is >= key (hi if none), by a 32-way
// search of the warp: each round every lane probes one point.
__device__ __forceinline__ int warp_lower_bound(const int *__restrict__ a, int lo, int hi, int key, int lane)
{
    while (hi - lo > 32) {
        const int step = (hi - lo + 31) >> 5;
        const int idx = lo + lane * step;
        const unsigned m = __ballot_sync(0xffffffffu, idx >= hi || a[idx] >= key);
        const int f = m ? __ffs(m) - 1 : 32;
        const int nlo = f == 0 ? lo : lo + (f - 1) * step + 1;
        hi = min(hi, lo + f * step);
        lo = nlo;
    }
    const int idx = lo + lane;
    const unsigned m = __ballot_sync(0xffffffffu, idx < hi && a[idx] >= key);
    return m ? lo + __ffs(m) - 1 : hi;
}

__device__ __forceinline__ void set_flag(int *flags, int which) {
    atomicOr(flags + which, 1);
}

}  // namespace tsg

// ---- host-side helpers shared by the .cu files --------------------------------
namespace tsg {

// Every kernel launch site calls this (process-wide counter behind
// tsg_launch_count), so benchmarks count launches instead of estimating them.
void count_launch();

// Fault injection (tsg_inject_alloc_failure): true when this allocation of
// `kind` (0: device pool, 1: pinned host) is the one armed to fail.
bool alloc_should_fail(int kind);

// Stream-ordered allocations from the context's memory pool.  The pool keeps
// freed memory cached (release threshold = max), so steady-state calls do no
// cudaMalloc.  alloc() returns nullptr and sets `err` on failure.
struct Pool {
    cudaMemPool_t pool = nullptr;
    cudaStream_t stream = nullptr;
    cudaError_t err = cudaSuccess;
    void *alloc(size_t bytes) {
        if (bytes == 0) bytes = 16;
        if (alloc_should_fail(0)) { err = cudaErrorMemoryAllocation; return nullptr; }
        void *p = nullptr;
        cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool, stream);
        if (e != cudaSuccess) { err = e; cudaGetLastError(); return nullptr; }
        return p;
    }
    template <class T> T *alloc_n(long long n) { return static_cast<T *>(alloc(sizeof(T) * (size_t)(n > 0 ? n : 1))); }
    void free(void *p) { if (p) cudaFreeAsync(p, stream); }
};

struct TileCSR {
    int m = 0, n = 0, blkm = 0, blkn = 0;
    long long cap = 0;          // allocated tile capacity (an upper bound of numblk)
    int *trp = nullptr;         // blkm+1 tile-row pointer
    int *tcol = nullptr;        // cap sorted tile columns
    uint16_t *mask = nullptr;   // 16*cap row masks
    // optional bitmap of each tile-row's tile columns (step 1's bitmap path):
    // tile-row k's words cover [tcol_first & ~31, tcol_last] at bmw[bmoff[k], bmoff[k+1]);
    // tile-rows wider than 4,096 tile columns have none
    long long *bmoff = nullptr; // blkm+1
    unsigned *bmw = nullptr;
};

// Bitmaps of T's tile-rows (T.bmoff / T.bmw, allocated by the caller:
// blkm+1 offsets and tile_bitmap_words_bound(T) words).
long long tile_bitmap_words_bound(const TileCSR &T);
cudaError_t tile_bitmaps(Pool &pool, TileCSR &T, long long *wcount, int *flags);

// Exclusive scans (decoupled look-back, one pass): out[i] = sum_{j<i} in[j]
// and out[n] = total.  The int32-output form flags FLAG_OVERFLOW on overflow.
cudaError_t scan_i32_to_i64(Pool &pool, const int *in, long long *out, long long n, int *flags);
cudaError_t scan_i32_to_i32(Pool &pool, const int *in, int *out, long long n, int *flags);
cudaError_t scan_i64_to_i64(Pool &pool, const long long *in, long long *out, long long n, int *flags);

inline int ceil_div_i(long long a, long long b) { return (int)((a + b - 1) / b); }

// A CSR row pointer as the caller gave it: int64 (p64) or int32 (p32).
struct RowPtr {
    const long long *p64 = nullptr;
    const int *p32 = nullptr;
    __host__ __device__ __forceinline__ long long operator[](long long i) const {
        return p64 ? p64[i] : (long long)p32[i];
    }
};

// The small-product path (tsg_small.cu): rows of A that meet at most
// SMALL_MAX_PRODUCTS entries of B, one warp per row of C.  small_count
// writes each row's entry count (0 for rows over the limit) and adds the
// rows over the limit to stat[0], the products to stat[1], and sets stat[2]
// when a row does not fit one warp round (32 products); small_fill
// writes C's columns and values at rowptrC (nothing when rowptrC[m] > cap);
// with `kept` non-null rowptrC is a row pointer kept from an earlier call:
// rows that do not match it add 1 to kept[0] (products to kept[1]);
// rp_out (optional) gets rowptrC as the caller's int32 or int64 row pointer;
// one_round (with `kept`): a variant without shared memory for shapes
// whose rows all fit one round (a row that does not counts in kept[0]).
// ka = A's columns (= B's rows), nb = B's columns.
constexpr int SMALL_MAX_PRODUCTS = 128;
// The operands' row pointers are clamped into [0, nnz] where they are
// read; with `check` (the kept-row-pointer fill on operands not validated
// before) the fill also validates A's row pointer and columns as the
// validation kernel does, and B's (kb rows) when B is not A.
struct SmallOperands {
    RowPtr rpA, rpB;
    const int *colA = nullptr, *colB = nullptr;
    const double *valA = nullptr, *valB = nullptr;
    int m = 0, ka = 0, kb = 0, nb = 0;    // A: m x ka; B: kb x nb
    long long nnzA = 0, nnzB = 0;
    bool check = false, b_is_a = false;
};
cudaError_t small_count(Pool &pool, const SmallOperands &o, int *rowcnt, unsigned long long *stat);
cudaError_t small_fill(Pool &pool, const SmallOperands &o, const long long *rowptrC, long long cap, int *colC,
                       double *valC, int *flags, unsigned long long *kept = nullptr, void *rp_out = nullptr,
                       int rp_bits = 32, bool one_round = false);

// One instance of a batched product, as the pack/unpack kernels see it.
struct PackDesc {
    const void *rp;          // instance row pointer (int32 or int64), device
    const int *col;          // instance columns, device
    const double *val;       // instance values, device (may be null)
    int rp_bits;
    int m, n;                // instance shape (n: column bound for validation)
    long long nnz;
    long long rowoff;        // first packed row (multiple of 16)
    long long rowpad;        // packed rows reserved (m rounded up to 16)
    long long coloff;        // added to the instance's column indices
    long long nnzoff;        // first packed entry
};

struct UnpackDesc {
    long long rowoff;        // first packed row of C_i
    int m;                   // rows of C_i
    long long coloff;        // C_i's first packed column (the numeric step subtracts it)
    long long rpoff;         // first entry of C_i's row pointer in the output array
};

// per = CTAs per instance (grid y)
cudaError_t batch_pack(Pool &pool, const PackDesc *d_desc, int count, int per, long long *rp, int *col, double *val,
                       int *flags);
cudaError_t batch_unpack(Pool &pool, const UnpackDesc *d_desc, int count, const long long *rowptrC, void *rp_out,
                         int rp_bits, long long *ebase);

}  // namespace tsg
