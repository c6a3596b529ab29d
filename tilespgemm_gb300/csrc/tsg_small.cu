// tsg_small.cu -- the small-product path of tsg_spgemm: C = A*B row by row,
// one warp per row of C, the row kept in a shared-memory hash table (or, for
// rows of at most 32 products, in the warp's registers).
//
// The tiled pipeline (conversion, two symbolic steps, binned numeric step)
// costs some 27 launches and three host waits per call, which is most of
// the time of a product of a few million intermediate products (a 2D
// Laplacian on a 256x256 grid: 1.6 M products).  Products whose every row of
// A meets at most SMALL_MAX_PRODUCTS entries of B take this path instead:
//   k_small_count  per row, the distinct columns among its products (hash
//                  insertions) -> rowcnt; rows over the limit are counted in
//                  stat[0] (the caller then takes the tiled path), the
//                  products in stat[1]
//   (the look-back scan of rowcnt gives C's row pointer)
//   k_small_fill   per row, the same walk accumulating values, then the row's
//                  entries written in column order.  With `kept` (C's row
//                  pointer kept from the last call of the same shape, no
//                  count pass before it) a row whose entries differ from the
//                  kept count, or that is over the limit, adds 1 to kept[0]
//                  (the caller then runs the count pass), the products go
//                  to kept[1].
// The row's products are dealt 32 at a time in A's order then B's (lane =
// position in the concatenation of the B rows of up to 32 A entries); lanes
// of one round that meet in one output apply in lane order, so every entry
// of C sees exactly the sequence fma(a_ik, b_kj, c) over k in A's row order,
// as in the tiled path and the oracle: the two paths give identical values.
// The reference has no such path; its per-call setup is the overhead
// (main_spgemm-col.cu:4529-4774) that this path removes for small products.
#include "tsg_internal.cuh"

namespace tsg {

namespace {

constexpr int SH_WARPS = 8;                    // rows per CTA (one warp each)
constexpr int SH_BITS = 8;
constexpr int SH_CAP = 1 << SH_BITS;           // hash slots per warp
static_assert(SMALL_MAX_PRODUCTS * 2 <= SH_CAP, "the table stays at most half full");

__device__ __forceinline__ int sh_hash(int col) { return (int)(((unsigned)col * 2654435761u) >> (32 - SH_BITS)); }

// slot of `col` in the warp's table, inserting it if absent (fresh: it was);
// -1 if the table is full (not reached: at most SMALL_MAX_PRODUCTS keys)
__device__ __forceinline__ int sh_insert(int *key, int col, bool &fresh)
{
    int h = sh_hash(col);
    fresh = false;
    for (int probe = 0; probe < SH_CAP; ++probe) {
        const int old = atomicCAS(key + h, -1, col);
        if (old == -1) { fresh = true; return h; }
        if (old == col) return h;
        h = (h + 1) & (SH_CAP - 1);
    }
    return -1;
}

// Up to 32 A entries of row r, lane q < na holding entry q's B row
// [bs, bs + len) (len clamped to SMALL_MAX_PRODUCTS + 1, empty for an
// out-of-range column of A; B's row pointers clamped into [0, nnzB], so
// that an unchecked row pointer reads nothing outside B).
struct Batch {
    long long bs = 0;
    int len = 0;
};

__device__ __forceinline__ Batch load_batch(const SmallOperands &o, long long p, int na, int lane, int *flags, int &k)
{
    Batch b;
    k = -1;
    if (lane < na) {
        k = o.colA[p + lane];
        if (o.check && (unsigned)k >= (unsigned)o.ka) set_flag(flags, FLAG_BAD_INPUT);
        if ((unsigned)k < (unsigned)o.ka) {
            const RowPtr rpB = o.rpB;
            const long long nnzB = o.nnzB;
            const long long s0 = rpB[k], s1 = rpB[k + 1];
            b.bs = s0 < 0 ? 0 : (s0 > nnzB ? nnzB : s0);
            const long long l = (s1 > nnzB ? nnzB : s1) - b.bs;
            b.len = (int)(l < 0 ? 0 : (l > SMALL_MAX_PRODUCTS + 1 ? SMALL_MAX_PRODUCTS + 1 : l));
        } else {
            k = -1;
        }
    }
    return b;
}

// Row r's entries [a0, a1) of A, clamped into [0, nnzA]; with `check` the
// row pointer is validated as the validation kernel does (bounds, order,
// first 0, last nnzA: lane 0 flags FLAG_BAD_INPUT).
__device__ __forceinline__ void row_span(RowPtr rp, int r, int m, long long nnz, bool check, int lane, int *flags,
                                         long long &a0, long long &a1)
{
    const long long v0 = rp[r], v1 = rp[r + 1];
    if (check && lane == 0) {
        const bool bad = v0 < 0 || v0 > nnz || v1 < v0 || v1 > nnz || (r == 0 && v0 != 0) || (r == m - 1 && v1 != nnz);
        if (bad) set_flag(flags, FLAG_BAD_INPUT);
    }
    a0 = v0 < 0 ? 0 : (v0 > nnz ? nnz : v0);
    a1 = v1 < a0 ? a0 : (v1 > nnz ? nnz : v1);
}

// the lane whose B row holds position f of the concatenation (last lane
// whose exclusive offset is at or before f)
__device__ __forceinline__ int owner_lane(int off, int f)
{
    int q = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const int oc = __shfl_sync(0xffffffffu, off, q + step);
        if (oc <= f) q += step;
    }
    return q;
}

// Rows whose products fit one round (at most 32, from at most 32 A
// entries) skip the table: the 32 lanes' keys are sorted across the warp
// (bitonic network on shuffles), equal columns then sit in adjacent lanes
// in product order, and the first lane of each run of equal columns starts
// an entry of C.
template <typename K>
__device__ __forceinline__ K warp_sort_up(K key, int lane)
{
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const K other = __shfl_xor_sync(0xffffffffu, key, j);
            const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
            key = keep_min ? (other < key ? other : key) : (other > key ? other : key);
        }
    }
    return key;
}

// One round's products sorted by (column, product index f = lane): lane
// i gets the i-th smallest, its column, and the A and B values of the lane
// that held it; live = false for the lanes past the products (c0 < 0).
template <typename K>
__device__ __forceinline__ void sort_products(int c0, double a, double bv, int lane, bool &live, int &col, double &sa,
                                              double &sb)
{
    K key = c0 >= 0 ? (((K)(unsigned)c0 << 5) | (K)(unsigned)lane) : ~(K)0;
    key = warp_sort_up(key, lane);
    live = key != ~(K)0;
    const int src = (int)(key & 31u);
    col = (int)(key >> 5);
    sa = __shfl_sync(0xffffffffu, a, src);
    sb = __shfl_sync(0xffffffffu, bv, src);
}

__global__ void __launch_bounds__(SH_WARPS * 32)
k_small_count(SmallOperands o, int *rowcnt, unsigned long long *stat)
{
    __shared__ int s_key[SH_WARPS][SH_CAP];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * SH_WARPS + warp;
    if (r >= o.m) return;
    const int *__restrict__ colB = o.colB;
    const int nb = o.nb;
    int *key = s_key[warp];
    bool table = false;      // the hash table is set up on the first batch that needs it
    long long a0, a1;
    row_span(o.rpA, r, o.m, o.nnzA, false, lane, nullptr, a0, a1);
    int cnt = 0, P = 0;
    bool over = false;
    for (long long pb = a0; pb < a1; pb += 32) {
        const int na = (int)min(32ll, a1 - pb);
        int k;
        const Batch b = load_batch(o, pb, na, lane, nullptr, k);
        const int incl = warp_incl_scan(b.len, lane);
        const int T = __shfl_sync(0xffffffffu, incl, 31);
        P += T;
        if (P > SMALL_MAX_PRODUCTS) { over = true; break; }
        const int off = incl - b.len;
        if (a1 - a0 <= 32 && T <= 32) {
            // one round: sort the columns, count the runs
            const int q = owner_lane(off, lane);
            const long long e = __shfl_sync(0xffffffffu, b.bs, q) + (lane - __shfl_sync(0xffffffffu, off, q));
            unsigned key = 0xffffffffu;
            if (lane < T) {
                const int col = colB[e];
                if ((unsigned)col < (unsigned)nb) key = (unsigned)col;
            }
            key = warp_sort_up(key, lane);
            const unsigned prev = __shfl_up_sync(0xffffffffu, key, 1);
            const bool head = key != 0xffffffffu && (lane == 0 || prev != key);
            const unsigned heads = __ballot_sync(0xffffffffu, head);   // every lane takes part
            cnt = lane == 0 ? __popc(heads) : 0;
            break;
        }
        if (!table) {
            for (int t = lane; t < SH_CAP; t += 32) key[t] = -1;
            __syncwarp();
            table = true;
        }
        for (int base = 0; base < T; base += 32) {
            const int f = base + lane;
            const int q = owner_lane(off, f);
            const long long e = __shfl_sync(0xffffffffu, b.bs, q) + (f - __shfl_sync(0xffffffffu, off, q));
            if (f < T) {
                const int col = colB[e];
                if ((unsigned)col < (unsigned)nb) {
                    bool fresh;
                    sh_insert(key, col, fresh);
                    cnt += fresh ? 1 : 0;
                }
            }
        }
    }
    cnt = warp_sum_int(cnt);
    if (lane == 0) {
        rowcnt[r] = over ? 0 : cnt;
        if (over) atomicAdd(stat, 1ull);
        else if (P) atomicAdd(stat + 1, (unsigned long long)P);
        // stat[2]: a row that does not fit one round (more than 32 products or A entries)
        if (!over && (P > 32 || a1 - a0 > 32) && stat[2] == 0) atomicMax(stat + 2, 1ull);
    }
}

// ONE: every row is expected to fit one round (a kept shape whose rows all
// did): no hash tables, so no shared memory and more warps per SM; a row
// that does not fit is reported through `kept` like a changed row.
template <bool ONE>
__global__ void __launch_bounds__(SH_WARPS * 32, ONE ? 6 : 1)
k_small_fill(SmallOperands o, const long long *__restrict__ rowptrC, long long cap, int *colC, double *valC,
             int *flags, unsigned long long *kept, void *rp_out, int rp_bits)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * SH_WARPS + warp;
    if (o.check && !o.b_is_a) {
        // B's row pointer and columns, checked across the whole grid
        const long long stride = (long long)gridDim.x * blockDim.x;
        const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        bool bad = false;
        for (long long i = t0; i <= o.kb; i += stride) {
            const long long v = o.rpB[i];
            bad |= v < 0 || v > o.nnzB || (i == 0 && v != 0) || (i == o.kb && v != o.nnzB) || (i < o.kb && o.rpB[i + 1] < v);
        }
        for (long long q = t0; q < o.nnzB; q += stride) bad |= (unsigned)o.colB[q] >= (unsigned)o.nb;
        if (bad) set_flag(flags, FLAG_BAD_INPUT);
    }
    const int m = o.m;
    if (r >= m) return;
    const int *__restrict__ colB = o.colB;
    const double *__restrict__ valA = o.valA;
    const double *__restrict__ valB = o.valB;
    const int nb = o.nb;
    const long long Rb = rowptrC[r], Re = rowptrC[r + 1];
    // C larger than the buffers: nothing is written (the caller sees nnzC
    // and runs this pass again into buffers of that size)
    if (rowptrC[m] > cap) return;
    if (rp_out && lane == 0) {   // the caller's row pointer, in its type
        if (rp_bits == 64) {
            static_cast<long long *>(rp_out)[r] = Rb;
            if (r == m - 1) static_cast<long long *>(rp_out)[m] = Re;
        } else {
            static_cast<int *>(rp_out)[r] = (int)Rb;
            if (r == m - 1) static_cast<int *>(rp_out)[m] = (int)Re;
        }
    }
    long long a0, a1;
    row_span(o.rpA, r, m, o.nnzA, o.check, lane, flags, a0, a1);
    if (a1 - a0 <= 32) {
        const int na = (int)(a1 - a0);
        int k;
        const Batch b = load_batch(o, a0, na, lane, flags, k);
        const int incl = warp_incl_scan(b.len, lane);
        const int T = __shfl_sync(0xffffffffu, incl, 31);
        if (T <= 32) {
            // one round: lane f holds product f (A's order, then B's); the
            // keys (column, f) sorted across the warp put each column's
            // products in adjacent lanes in product order, and the run's
            // first lane applies them in that order
            const double av = (lane < na && k >= 0) ? valA[a0 + lane] : 0.0;
            const int off = incl - b.len;
            const int q = owner_lane(off, lane);
            const long long e = __shfl_sync(0xffffffffu, b.bs, q) + (lane - __shfl_sync(0xffffffffu, off, q));
            const double a = __shfl_sync(0xffffffffu, av, q);
            int c0 = -1;
            double bv = 0.0;
            if (lane < T) {
                const int cb = colB[e];
                if ((unsigned)cb < (unsigned)nb) {
                    c0 = cb;
                    bv = valB[e];
                }
            }
            // 32-bit keys when B's columns leave room for the 5 bits of f
            bool live;
            int col;
            double sa, sb;
            if (nb <= (1 << 26)) sort_products<unsigned>(c0, a, bv, lane, live, col, sa, sb);
            else sort_products<unsigned long long>(c0, a, bv, lane, live, col, sa, sb);
            const int pcol = __shfl_up_sync(0xffffffffu, col, 1);
            const bool head = live && (lane == 0 || pcol != col);
            const unsigned heads = __ballot_sync(0xffffffffu, head);
            const int n = __popc(heads);
            if ((long long)n != Re - Rb) {
                if (lane == 0) {
                    if (kept) atomicAdd(kept, 1ull);
                    else set_flag(flags, FLAG_INTERNAL);
                }
                return;
            }
            if (kept && lane == 0 && T) atomicAdd(kept + 1, (unsigned long long)T);
            // run of lane i: lanes i, i+1, ... while the column stays col
            double acc = 0.0;
            bool more = head;
            for (int j = 0; __any_sync(0xffffffffu, more); ++j) {
                const int cj = __shfl_down_sync(0xffffffffu, col, j);
                const bool lj = __shfl_down_sync(0xffffffffu, live ? 1 : 0, j) != 0;
                const double aj = __shfl_down_sync(0xffffffffu, sa, j), bj = __shfl_down_sync(0xffffffffu, sb, j);
                more = more && lane + j < 32 && lj && cj == col;
                if (more) acc = fma(aj, bj, acc);
            }
            if (head) {
                const int rank = __popc(heads & lanemask_lt());
                colC[Rb + rank] = col;
                valC[Rb + rank] = acc;
            }
            return;
        }
    }
    if constexpr (ONE) {
        if (lane == 0) atomicAdd(kept, 1ull);   // not one round: the caller counts again
        return;
    } else {
    __shared__ int s_key[SH_WARPS][SH_CAP];
    __shared__ double s_val[SH_WARPS][SH_CAP];
    __shared__ int s_ck[SH_WARPS][SMALL_MAX_PRODUCTS];
    __shared__ double s_cv[SH_WARPS][SMALL_MAX_PRODUCTS];
    int *key = s_key[warp];
    double *val = s_val[warp];
    for (int t = lane; t < SH_CAP; t += 32) { key[t] = -1; val[t] = 0.0; }
    __syncwarp();
    int P = 0;
    for (long long pb = a0; pb < a1; pb += 32) {
        const int na = (int)min(32ll, a1 - pb);
        int k;
        const Batch b = load_batch(o, pb, na, lane, flags, k);
        const double av = (lane < na && k >= 0) ? valA[pb + lane] : 0.0;
        const int incl = warp_incl_scan(b.len, lane);
        const int T = __shfl_sync(0xffffffffu, incl, 31);
        P += T;
        if (P > SMALL_MAX_PRODUCTS) {   // counted as over the limit: the row is empty here
            if (kept && lane == 0) atomicAdd(kept, 1ull);
            return;
        }
        const int off = incl - b.len;
        for (int base = 0; base < T; base += 32) {
            const int f = base + lane;
            const int q = owner_lane(off, f);
            const long long e = __shfl_sync(0xffffffffu, b.bs, q) + (f - __shfl_sync(0xffffffffu, off, q));
            const double a = __shfl_sync(0xffffffffu, av, q);
            int slot = -1;
            double bv = 0.0;
            if (f < T) {
                const int col = colB[e];
                if ((unsigned)col < (unsigned)nb) {
                    bool fresh;
                    slot = sh_insert(key, col, fresh);
                    bv = valB[e];
                }
            }
            // lanes on one output apply in lane order (A's order, then B's)
            const unsigned peers = __match_any_sync(0xffffffffu, slot >= 0 ? slot : -2 - lane);
            const int rank = __popc(peers & lanemask_lt());
            if (!__any_sync(0xffffffffu, rank > 0)) {
                if (slot >= 0) val[slot] = fma(a, bv, val[slot]);
            } else {
                const int rounds = __reduce_max_sync(0xffffffffu, (unsigned)__popc(peers));
                for (int q2 = 0; q2 < rounds; ++q2) {
                    if (q2 == rank && slot >= 0) val[slot] = fma(a, bv, val[slot]);
                    __syncwarp();
                }
            }
            __syncwarp();
        }
    }
    // the row's entries, compacted in slot order, then each to its rank by column
    int *ck = s_ck[warp];
    double *cv = s_cv[warp];
    int n = 0;
    for (int t0 = 0; t0 < SH_CAP; t0 += 32) {
        const int t = t0 + lane;
        const int kk = key[t];
        const unsigned bal = __ballot_sync(0xffffffffu, kk >= 0);
        if (kk >= 0) {
            const int p = n + __popc(bal & lanemask_lt());
            if (p < SMALL_MAX_PRODUCTS) { ck[p] = kk; cv[p] = val[t]; }
        }
        n += __popc(bal);
    }
    __syncwarp();
    if ((long long)n != Re - Rb || n > SMALL_MAX_PRODUCTS) {
        if (lane == 0) {
            if (kept) atomicAdd(kept, 1ull);
            else set_flag(flags, FLAG_INTERNAL);
        }
        return;
    }
    if (kept && lane == 0 && P) atomicAdd(kept + 1, (unsigned long long)P);
    for (int p = lane; p < n; p += 32) {
        const int c = ck[p];
        int rank = 0;
        for (int j = 0; j < n; ++j) rank += ck[j] < c ? 1 : 0;
        colC[Rb + rank] = c;
        valC[Rb + rank] = cv[p];
    }
    }
}

}  // namespace

cudaError_t small_count(Pool &pool, const SmallOperands &o, int *rowcnt, unsigned long long *stat)
{
    if (o.m <= 0) return cudaSuccess;
    k_small_count<<<(unsigned)((o.m + SH_WARPS - 1) / SH_WARPS), SH_WARPS * 32, 0, pool.stream>>>(o, rowcnt, stat);
    ::tsg::count_launch();
    return cudaGetLastError();
}

cudaError_t small_fill(Pool &pool, const SmallOperands &o, const long long *rowptrC, long long cap, int *colC,
                       double *valC, int *flags, unsigned long long *kept, void *rp_out, int rp_bits, bool one_round)
{
    const int m = o.m;
    if (m <= 0) {   // C's row pointer is the single 0
        if (!rp_out) return cudaSuccess;
        return cudaMemsetAsync(rp_out, 0, rp_bits == 64 ? 8 : 4, pool.stream);
    }
    const unsigned grid = (unsigned)((m + SH_WARPS - 1) / SH_WARPS);
    if (one_round && kept)
        k_small_fill<true><<<grid, SH_WARPS * 32, 0, pool.stream>>>(o, rowptrC, cap, colC, valC, flags, kept, rp_out,
                                                                    rp_bits);
    else
        k_small_fill<false><<<grid, SH_WARPS * 32, 0, pool.stream>>>(o, rowptrC, cap, colC, valC, flags, kept, rp_out,
                                                                     rp_bits);
    ::tsg::count_launch();
    return cudaGetLastError();
}

}  // namespace tsg
