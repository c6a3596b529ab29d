// tsg_numeric.cu -- step 3: FP64 numeric accumulation and the CSR write of C.
//
// Reference: stir_spgemm_step4_cuda_kernel_smem_v3 (main_spgemm-col.cu:2094-2397,
// sparse tiles: warp per C tile, products added into the tile's sorted local
// column list found by linear search, shared-memory atomicAdd(double)) and
// stir_spgemm_step4_cuda_kernel_dns_noatomic_halfwarp (:3386-3755, dense
// tiles: 16x16 FP64 shared accumulator).  The reference writes C in tile form
// and stops; this step writes CSR directly.
//
// GB300 design.  On this part FP64 FMA issue is the ceiling (about 0.6 T
// FMA/s, and an FMA warp instruction costs the same with idle lanes), so each
// intermediate product is exactly one DFMA, with no other FP64 instruction in
// the loop.  One CTA owns a C tile-row (16 rows); step 2 already fixed every
// output's position: for C tile (i,j) and local row r, the row's entries are
// the set bits of mask[j][r], and an output column c of that row sits at
//     offset(j, r) + popc(mask[j][r] >> (16 - c))
// inside the tile-row's CSR segment (a perfect hash keyed by the masks).  The
// CTA keeps the tile-row's whole CSR segment of values in shared memory,
// each warp owns C rows (so no two warps touch one output), and for every
// A entry (R,k) the warp's lanes take B row k's entries, which have distinct
// columns, so one DFMA instruction updates distinct outputs.  When B's rows
// repeat columns the packed walk instead gives each lane one (A entry, B
// entry) pair of the row's flattened pair sequence and orders lanes that
// meet in one output (it fills the lanes when B's rows are short too, but
// measured slower there: these loops are latency-bound, not DFMA-bound).  Per output the products are applied in
// A's row order, then B's row order: the same order as the CPU reference
// (thmkl_dcsrmultcsr.c:52-91), so with FMA rounding the two agree bit for bit.
// The epilogue streams the segment's values out coalesced and expands the
// masks into column indices.  Dense tile-rows (mean tile nnz >= a threshold)
// use 16x16 dense accumulators instead (position = slot*256 + r*16 + c).
// Tile-rows too large for one CTA's shared memory take one CTA per row
// (k_numeric_rows), and rows too large for that accumulate in C's value
// array (k_numeric_wide).
//
// Roofline: the DFMA issue rate bounds the loop (2 FLOP per intermediate
// product); HBM traffic is A and B once (B rows are re-read from L2) plus
// 12 bytes per C entry written.
#include "tsg_numeric.cuh"

#include <algorithm>
#include <climits>

namespace tsg {

namespace {

__device__ __forceinline__ int lower_bound_dev(const int *a, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// dense accumulators: 16 doubles per (row, tile) padded to 17, so lanes on
// different tiles with the same local column use different banks
constexpr int DPAD = 17;

// word[r*S + s] packs, for C tile s and local row r, the offset of the
// tile's row segment inside the tile-row's CSR segment (top 16 bits) and the
// row mask (low 16 bits)
// Bank swizzles.  The accumulator index p is permuted inside aligned groups
// of 16 (p ^ ((p >> 4) & 15)): regular column strides (stencils put a B
// row's outputs 16 apart) would otherwise land on one bank.  The map index
// is permuted inside groups of 64 halfwords for the same reason (tile
// columns of neighbouring planes sit 2^k apart).  Both are bijections that
// keep the index inside its group, so the arrays are rounded up to 16 / 64.
__device__ __forceinline__ int acc_swz(int p) { return p ^ ((p >> 4) & 15); }
__device__ __forceinline__ unsigned map_swz(unsigned o) { return o ^ (((o >> 6) & 31u) << 1); }

__device__ __forceinline__ int rank_in_row(unsigned w, int c) {
    return (int)(w >> 16) + __popc((w & 0xffffu) >> (TILE - c));
}

struct TileRowSmem {
    const int *scol;
    const unsigned *word;
    const unsigned short *map;
    double *acc;
    int S, jbase, span, nacc;
};

template <bool DENSE, bool MAP>
__device__ __forceinline__ int out_pos(const TileRowSmem &t, const unsigned *wrow, int r, int col) {
    const unsigned off = (unsigned)((col >> 4) - t.jbase);
    if (off >= (unsigned)t.span) return -1;
    int s;
    if (MAP) {
        s = (int)t.map[map_swz(off)];          // 0xffff marks a column with no C tile
        if (s >= t.S) return -1;
    } else {
        s = lower_bound_dev(t.scol, t.S, col >> 4);
        if (s >= t.S || t.scol[s] != (col >> 4)) return -1;
    }
    const int p = DENSE ? (r * t.S + s) * DPAD + (col & 15) : acc_swz(rank_in_row(wrow[s], col & 15));
    return (unsigned)p < (unsigned)t.nacc ? p : -1;
}

// out_pos for the map layout without early exits: every read uses an index
// clamped into its array, and the checks combine into one predicate, so the
// compiler selects instead of branching (a product costs about 80 warp
// instructions with the branches, 13 of them branches).  -1: not in C.
template <bool DENSE>
__device__ __forceinline__ int out_pos_map(const TileRowSmem &t, const unsigned *wrow, int r, int col) {
    const unsigned off = (unsigned)((col >> 4) - t.jbase);
    const bool in = off < (unsigned)t.span;
    const int s = (int)t.map[map_swz(in ? off : 0u)];   // 0xffff marks a column with no C tile
    const bool sok = in && (unsigned)s < (unsigned)t.S;
    const int c = col & 15;
    const int p = DENSE ? (r * t.S + s) * DPAD + c : acc_swz(rank_in_row(wrow[sok ? s : 0], c));
    return sok && (unsigned)p < (unsigned)t.nacc ? p : -1;
}

// One C row: the warp walks A's row in order; for each A entry its lanes
// take the B row's entries (distinct columns, so distinct outputs).  B rows
// of up to 32 entries (one per lane) take a path without a loop.
template <bool DENSE, bool MAP>
__device__ __forceinline__ void numeric_row(const NumericArgs &g, const TileRowSmem &t, int r0, int r, int lane)
{
    const int R = r0 + r;
    const unsigned *wrow = t.word + r * t.S;
    const int pa0 = (int)g.rpA[R], pa1 = (int)g.rpA[R + 1];
    double *acc = t.acc;
    bool bad = false;
    for (int pb = pa0; pb < pa1; pb += 32) {
        const int na = min(32, pa1 - pb);
        int bs = 0, be = 0;
        double av = 0.0;
        if (lane < na) {
            const int k = g.colA[pb + lane];
            av = g.valA[pb + lane];
            bs = (int)g.rpB[k];
            be = (int)g.rpB[k + 1];
        }
        for (int q = 0; q < na; ++q) {
            const double a = __shfl_sync(0xffffffffu, av, q);
            const int b0 = __shfl_sync(0xffffffffu, bs, q);
            const int b1 = __shfl_sync(0xffffffffu, be, q);
            if (MAP && b1 - b0 <= 32) {   // uniform
                if (b1 <= b0) continue;
                // every lane loads and updates: idle lanes re-read the row's
                // last entry and update the spare slot acc[nacc]
                const bool live = b0 + lane < b1;
                const int e = live ? b0 + lane : b1 - 1;
                const int col = g.colB[e];
                const double b = g.valB[e];
                const int pos = out_pos_map<DENSE>(t, wrow, r, col);
                bad |= live && pos < 0;
                const int pi = (live && pos >= 0) ? pos : t.nacc;
                acc[pi] = fma(a, b, acc[pi]);
                continue;
            }
            for (int e = b0 + lane; e < b1; e += 32) {
                const int col = g.colB[e];
                const double b = g.valB[e];
                const int pos = out_pos<DENSE, MAP>(t, wrow, r, col);
                if (pos < 0) { bad = true; continue; }
                acc[pos] = fma(a, b, acc[pos]);
            }
        }
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

// Packed walk of one C row: the row's (A entry, B entry) pairs, in A's row
// order then B's row order, are taken 32 at a time, one per lane, whatever
// the lengths of the B rows.  Lanes whose pairs hit the same output --
// repeated columns in a B row, or different A entries meeting in one column
// -- apply their products in lane order, which is pair order, so each
// output still sees A's row order, then B's.  This is the walk for B
// operands with repeated columns.  pos_of(col) gives the accumulator index
// of column col: -1 flags an error (not in C's pattern), other negative
// values skip the pair (a column outside the caller's range).
template <class Acc, class PosFn>
__device__ __forceinline__ void row_walk_packed(const NumericArgs &g, int R, int lane, Acc *acc, PosFn pos_of)
{
    const int pa0 = (int)g.rpA[R], pa1 = (int)g.rpA[R + 1];
    bool bad = false;
    for (int pb = pa0; pb < pa1; pb += 32) {
        const int na = min(32, pa1 - pb);
        int bs = 0, len = 0;
        double av = 0.0;
        if (lane < na) {
            const int k = g.colA[pb + lane];
            av = g.valA[pb + lane];
            bs = (int)g.rpB[k];
            len = (int)g.rpB[k + 1] - bs;
        }
        const int incl = warp_incl_scan(len, lane);
        const int off = incl - len;
        const int T = __shfl_sync(0xffffffffu, incl, 31);
        for (int base = 0; base < T; base += 32) {
            const int tt = base + lane;
            // q = last lane whose pair range starts at or before tt (non-empty when tt < T)
            int q = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int oc = __shfl_sync(0xffffffffu, off, q + step);
                if (oc <= tt) q += step;
            }
            const int e = __shfl_sync(0xffffffffu, bs, q) + tt - __shfl_sync(0xffffffffu, off, q);
            const double a = __shfl_sync(0xffffffffu, av, q);
            long long pos = -2;
            double b = 0.0;
            if (tt < T) {
                b = g.valB[e];
                pos = pos_of(g.colB[e]);
                if (pos == -1) bad = true;
            }
            const unsigned peers = __match_any_sync(0xffffffffu, pos >= 0 ? pos : -3ll - lane);
            const int rank = __popc(peers & lanemask_lt());
            if (!__any_sync(0xffffffffu, rank > 0)) {
                if (pos >= 0) acc[pos] = fma(a, b, acc[pos]);
            } else {
                const int rounds = __reduce_max_sync(0xffffffffu, __popc(peers));
                for (int q2 = 0; q2 < rounds; ++q2) {
                    if (q2 == rank && pos >= 0) acc[pos] = fma(a, b, acc[pos]);
                    __syncwarp();
                }
            }
            __syncwarp();
        }
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

// The (A entry, 32-entry chunk) pairs of up to 32 A entries, lane q holding
// entry q's value av and B segment [bs, be): walked in order, the next
// pair's B loads issued before the current pair's update; only columns in
// [lo, hi) are applied.
template <class Acc, class PosFn>
__device__ __forceinline__ void walk_segments(const NumericArgs &g, int lane, int na, double av, int bs, int be,
                                              int lo, int hi, Acc *acc, PosFn pos_of, bool &bad)
{
    {
        // first non-empty pair
        int q = 0, eb = __shfl_sync(0xffffffffu, bs, 0), ee = __shfl_sync(0xffffffffu, be, 0);
        double a = __shfl_sync(0xffffffffu, av, 0);
        while (eb >= ee && ++q < na) {
            eb = __shfl_sync(0xffffffffu, bs, q);
            ee = __shfl_sync(0xffffffffu, be, q);
            a = __shfl_sync(0xffffffffu, av, q);
        }
        int col = INT_MAX;
        double b = 0.0;
        if (q < na && eb + lane < ee) { col = g.colB[eb + lane]; b = g.valB[eb + lane]; }
        while (q < na) {
            int nq = q, neb = eb + 32, nee = ee;
            double na_ = a;
            while (neb >= nee && ++nq < na) {
                neb = __shfl_sync(0xffffffffu, bs, nq);
                nee = __shfl_sync(0xffffffffu, be, nq);
                na_ = __shfl_sync(0xffffffffu, av, nq);
            }
            int ncol = INT_MAX;
            double nb = 0.0;
            if (nq < na && neb + lane < nee) { ncol = g.colB[neb + lane]; nb = g.valB[neb + lane]; }
            if (col >= lo && col < hi) {
                const long long pos = pos_of(col);
                if (pos < 0) bad = true;
                else acc[pos] = fma(a, b, acc[pos]);
            }
            __syncwarp();
            q = nq; eb = neb; ee = nee; a = na_;
            col = ncol; b = nb;
        }
    }
}

// One warp applies row R's products whose column lies in [lo, hi), in A's
// row order then B's (lanes over one B row; B rows without repeated
// columns).  A's entries are taken 32 at a time, one per lane: with sorted
// B rows each lane first cuts its B row to [lo, hi) by two binary searches
// (all lanes at once), then the warp walks the (A entry, 32-entry chunk)
// pairs in order with the next pair's loads issued before the current
// pair's updates.  Without sorted B rows every entry is tested instead.
template <class Acc, class PosFn>
__device__ __forceinline__ void row_walk_range(const NumericArgs &g, int R, int lane, int lo, int hi, Acc *acc,
                                               PosFn pos_of)
{
    const int pa0 = (int)g.rpA[R], pa1 = (int)g.rpA[R + 1];
    bool bad = false;
    for (int pb = pa0; pb < pa1; pb += 32) {
        const int na = min(32, pa1 - pb);
        int bs = 0, be = 0;
        double av = 0.0;
        if (lane < na) {
            const int k = g.colA[pb + lane];
            av = g.valA[pb + lane];
            bs = (int)g.rpB[k];
            be = (int)g.rpB[k + 1];
            if (g.b_sorted) {
                int l = bs, h = be;
                while (l < h) { const int md = (l + h) >> 1; if (g.colB[md] < lo) l = md + 1; else h = md; }
                bs = l; h = be;
                while (l < h) { const int md = (l + h) >> 1; if (g.colB[md] < hi) l = md + 1; else h = md; }
                be = l;
            }
        }
        walk_segments(g, lane, na, av, bs, be, lo, hi, acc, pos_of, bad);
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

// numeric_row with B's entries loaded one step ahead:
// the warp walks the (A entry, 32-entry chunk of its B row) pairs in order
// and issues the next pair's loads before the current pair's shared-memory
// update, so the L2 latency of B overlaps the accumulator work.  Order of the
// updates per output is unchanged (A's row order, then B's row order).
template <bool DENSE, bool MAP>
__device__ __forceinline__ void numeric_row_prefetch(const NumericArgs &g, const TileRowSmem &t, int r0, int r, int lane)
{
    const int R = r0 + r;
    const unsigned *wrow = t.word + r * t.S;
    const int pa0 = (int)g.rpA[R], pa1 = (int)g.rpA[R + 1];
    double *acc = t.acc;
    bool bad = false;
    for (int pb = pa0; pb < pa1; pb += 32) {
        const int na = min(32, pa1 - pb);
        int bs = 0, be = 0;
        double av = 0.0;
        if (lane < na) {
            const int k = g.colA[pb + lane];
            av = g.valA[pb + lane];
            bs = (int)g.rpB[k];
            be = (int)g.rpB[k + 1];
        }
        // first non-empty pair
        int q = 0, eb = __shfl_sync(0xffffffffu, bs, 0), ee = __shfl_sync(0xffffffffu, be, 0);
        double a = __shfl_sync(0xffffffffu, av, 0);
        while (eb >= ee && ++q < na) {
            eb = __shfl_sync(0xffffffffu, bs, q);
            ee = __shfl_sync(0xffffffffu, be, q);
            a = __shfl_sync(0xffffffffu, av, q);
        }
        int col = 0;
        double b = 0.0;
        bool ok = false;
        if (q < na && eb + lane < ee) { ok = true; col = g.colB[eb + lane]; b = g.valB[eb + lane]; }
        while (q < na) {
            // next pair (uniform across the warp)
            int nq = q, neb = eb + 32, nee = ee;
            double na_ = a;
            while (neb >= nee && ++nq < na) {
                neb = __shfl_sync(0xffffffffu, bs, nq);
                nee = __shfl_sync(0xffffffffu, be, nq);
                na_ = __shfl_sync(0xffffffffu, av, nq);
            }
            int ncol = 0;
            double nb = 0.0;
            bool nok = false;
            if (nq < na && neb + lane < nee) { nok = true; ncol = g.colB[neb + lane]; nb = g.valB[neb + lane]; }
            if (ok) {
                const int pos = out_pos<DENSE, MAP>(t, wrow, r, col);
                if (pos < 0) bad = true;
                else acc[pos] = fma(a, b, acc[pos]);
            }
            q = nq; eb = neb; ee = nee; a = na_;
            col = ncol; b = nb; ok = nok;
        }
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

// WALK: 0 lanes over one B row per A entry, 1 packed (repeated B columns),
// 2 as 0 with B's entries loaded one step ahead (more registers, fewer warps)
template <int NT, bool DENSE, int WALK>
__global__ void __launch_bounds__(NT, (WALK == 0 ? 2048 : 1024) / NT)
k_numeric_smem(NumericArgs g, int mybin)
{
    constexpr int NWARP = NT / 32;
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int i = g.binlist[(long long)mybin * g.blkm + blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = i * TILE;
    const int rows = min(TILE, g.m - r0);
    const long long c0 = g.crp[i];
    const int S = (int)(g.crp[i + 1] - c0);
    const long long R0 = g.rowptrC[r0];
    const int nnz_tr = (int)(g.rowptrC[r0 + rows] - R0);
    const int jbase = g.ccol[c0];
    const int span = g.ccol[c0 + S - 1] - jbase + 1;
    const bool use_map = span <= MAP_MAX;

    int *scol = reinterpret_cast<int *>(s_raw);
    unsigned *word = reinterpret_cast<unsigned *>(s_raw + align16((long long)S * 4));
    unsigned short *map = reinterpret_cast<unsigned short *>(s_raw + align16((long long)S * 4) + align16((long long)S * TILE * 4));
    double *acc = reinterpret_cast<double *>(s_raw + align16((long long)S * 4) + align16((long long)S * TILE * 4) +
                                             (use_map ? map_bytes(span) : 0));

    if (use_map) {
        const int span64 = (span + 63) & ~63;
        for (int t = tid; t < span64; t += NT) map[t] = 0xffffu;
        __syncthreads();
    }
    for (int s = tid; s < S; s += NT) {
        int j = g.ccol[c0 + s];
        scol[s] = j;
        if (use_map) map[map_swz((unsigned)(j - jbase))] = (unsigned short)s;
    }
    // packed words, row-major (word[r*S + s]) so that lanes on different
    // tiles of one row hit different banks: per row, exclusive scan of popc
    // over the tile-row's tiles
    for (int r = warp; r < TILE; r += NWARP) {
        int run = (r < rows) ? (int)(g.rowptrC[r0 + r] - R0) : 0;
        for (int sb = 0; sb < S; sb += 32) {
            const int s = sb + lane;
            unsigned mk = (s < S) ? (unsigned)g.cmask[c0 * TILE + (long long)r * S + s] : 0u;
            int c = __popc(mk);
            int incl = warp_incl_scan(c, lane);
            if (s < S) word[r * S + s] = ((unsigned)(run + incl - c) << 16) | mk;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
    const int nacc = DENSE ? S * TILE * DPAD : (nnz_tr + 15) & ~15;
    {
        unsigned long long *z = reinterpret_cast<unsigned long long *>(acc);
        for (int t = tid; t < nacc; t += NT) z[t] = 0ull;
    }
    __syncthreads();

    // warp w owns rows w, w+NWARP, ...
    TileRowSmem t{scol, word, map, acc, S, jbase, span, nacc};
    for (int r = warp; r < rows; r += NWARP) {
        if (WALK == 1) {
            const unsigned *wrow = word + r * S;
            if (use_map)
                row_walk_packed(g, r0 + r, lane, acc, [&](int col) -> long long { return out_pos<DENSE, true>(t, wrow, r, col); });
            else
                row_walk_packed(g, r0 + r, lane, acc, [&](int col) -> long long { return out_pos<DENSE, false>(t, wrow, r, col); });
        } else if (WALK == 2) {
            if (use_map) numeric_row_prefetch<DENSE, true>(g, t, r0, r, lane);
            else numeric_row_prefetch<DENSE, false>(g, t, r0, r, lane);
        } else if (use_map) {
            numeric_row<DENSE, true>(g, t, r0, r, lane);
        } else {
            numeric_row<DENSE, false>(g, t, r0, r, lane);
        }
    }
    __syncthreads();

    // epilogue: values (coalesced for the sparse layout) and column indices
    if (!DENSE) {
        for (int p = tid; p < nnz_tr; p += NT) g.valC[R0 + p] = acc[acc_swz(p)];
    }
    const int cshift = g.tr_coloff ? g.tr_coloff[i] : 0;
    for (int r = warp; r < rows; r += NWARP) {
        for (int s = lane; s < S; s += 32) {
            const unsigned w = word[r * S + s];
            unsigned mk = w & 0xffffu;
            long long dst = R0 + (w >> 16);
            const int jb = scol[s] * TILE - cshift;
            while (mk) {
                const int b = 31 - __clz(mk);   // highest bit = smallest local column
                const int c = TILE - 1 - b;
                if (!g.cols_done) g.colC[dst] = jb + c;
                if (DENSE) g.valC[dst] = acc[(r * S + s) * DPAD + c];
                ++dst;
                mk &= ~(1u << b);
            }
        }
    }
}


// ---- rows of tile-rows too large for one CTA (BIN_ROWS) --------------------

// Shared-memory view of one C row (row r of tile-row i): the row's packed
// words word[S] ((offset in the row << 16) | mask), the slot map or the
// tile columns, and the accumulator.  Built by the CTA's nthr threads.
struct RowSmem {
    unsigned *word;
    unsigned short *map;
    int *scol;
    double *acc;
    int S, jbase, span, nacc;
    bool use_map;
};

__device__ __forceinline__ RowSmem row_smem_build(const NumericArgs &g, unsigned char *s_raw, int i, int r,
                                                  int nnz_r, int tid, int nthr, int *s_part)
{
    RowSmem w;
    const long long c0 = g.crp[i];
    w.S = (int)(g.crp[i + 1] - c0);
    w.jbase = g.ccol[c0];
    w.span = g.ccol[c0 + w.S - 1] - w.jbase + 1;
    w.use_map = w.span <= MAP_MAX;
    w.word = reinterpret_cast<unsigned *>(s_raw);
    unsigned char *p1 = s_raw + align16((long long)w.S * 4);
    w.map = w.use_map ? reinterpret_cast<unsigned short *>(p1) : nullptr;
    w.scol = w.use_map ? nullptr : reinterpret_cast<int *>(p1);
    w.acc = reinterpret_cast<double *>(p1 + (w.use_map ? map_bytes(w.span) : align16((long long)w.S * 4)));
    w.nacc = (nnz_r + 15) & ~15;
    const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
    if (w.use_map) {
        const int span64 = (w.span + 63) & ~63;
        for (int t = tid; t < span64; t += nthr) w.map[t] = 0xffffu;
        if (nw > 1) __syncthreads(); else __syncwarp();
    }
    for (int s = tid; s < w.S; s += nthr) {
        const int j = g.ccol[c0 + s];
        if (w.use_map) w.map[map_swz((unsigned)(j - w.jbase))] = (unsigned short)s;
        else w.scol[s] = j;
    }
    // packed words: warp k scans slots [k*seg, (k+1)*seg); a prefix over the
    // warps' totals (s_part) gives each segment's start offset
    const uint16_t *mrow = g.cmask + c0 * TILE + (long long)r * w.S;
    const int seg = (((w.S + nw - 1) / nw) + 31) & ~31;
    const int s0 = min(w.S, warp * seg), s1 = min(w.S, s0 + seg);
    int tot = 0;
    for (int s = s0 + lane; s < s1; s += 32) tot += __popc((unsigned)mrow[s]);
    tot = warp_sum_int(tot);
    int run = 0;
    if (nw > 1) {
        if (lane == 0) s_part[warp] = tot;
        __syncthreads();
        for (int k = 0; k < warp; ++k) run += s_part[k];
    }
    for (int sb = s0; sb < s1; sb += 32) {
        const int s = sb + lane;
        const unsigned mk = (s < s1) ? (unsigned)mrow[s] : 0u;
        const int c = __popc(mk);
        const int incl = warp_incl_scan(c, lane);
        if (s < s1) w.word[s] = ((unsigned)(run + incl - c) << 16) | mk;
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    {
        unsigned long long *z = reinterpret_cast<unsigned long long *>(w.acc);
        for (int t = tid; t < w.nacc; t += nthr) z[t] = 0ull;
    }
    if (nw > 1) __syncthreads(); else __syncwarp();
    return w;
}

__device__ __forceinline__ long long row_pos(const RowSmem &w, int col) {
    const unsigned off = (unsigned)((col >> 4) - w.jbase);
    if (off >= (unsigned)w.span) return -1;
    int s;
    if (w.use_map) {
        s = (int)w.map[map_swz(off)];
        if (s >= w.S) return -1;
    } else {
        s = lower_bound_dev(w.scol, w.S, col >> 4);
        if (s >= w.S || w.scol[s] != (col >> 4)) return -1;
    }
    const unsigned wd = w.word[s];
    const int c = col & 15;
    if (!((wd >> (TILE - 1 - c)) & 1u)) return -1;
    const int p = rank_in_row(wd, c);
    return p < w.nacc ? acc_swz(p) : -1;
}

// values (coalesced) and column indices of one row from its accumulator
__device__ __forceinline__ void row_epilogue(const NumericArgs &g, const RowSmem &w, int i, long long Rb, int nnz_r,
                                             int tid, int nthr)
{
    for (int p = tid; p < nnz_r; p += nthr) g.valC[Rb + p] = w.acc[acc_swz(p)];
    if (g.cols_done) return;
    const int cshift = g.tr_coloff ? g.tr_coloff[i] : 0;
    const long long c0 = g.crp[i];
    for (int s = tid; s < w.S; s += nthr) {
        const unsigned wd = w.word[s];
        unsigned mk = wd & 0xffffu;
        long long dst = Rb + (wd >> 16);
        const int jb = (w.use_map ? g.ccol[c0 + s] : w.scol[s]) * TILE - cshift;
        while (mk) {
            const int b = 31 - __clz(mk);   // highest bit = smallest local column
            g.colC[dst] = jb + (TILE - 1 - b);
            ++dst;
            mk &= ~(1u << b);
        }
    }
}

// One single-warp CTA per row of row class ROW_S or ROW_M: the row's CSR
// segment of values in shared memory, addressed by the slot map + the row's
// packed words, then streamed out.  The class bounds the shared memory of
// its launch, so short rows keep a high occupancy.
__global__ void __launch_bounds__(32, 32)
k_numeric_rows(NumericArgs g, int cls, bool packed)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int R = g.rowlist[(long long)cls * g.m + blockIdx.x];
    const int i = R >> 4, r = R & (TILE - 1);
    const int lane = threadIdx.x;
    const long long Rb = g.rowptrC[R];
    const int nnz_r = (int)(g.rowptrC[R + 1] - Rb);
    const RowSmem w = row_smem_build(g, s_raw, i, r, nnz_r, lane, 32, nullptr);
    TileRowSmem t{w.scol, w.word, w.map, w.acc, w.S, w.jbase, w.span, w.nacc};
    if (packed) row_walk_packed(g, R, lane, w.acc, [&](int col) -> long long { return row_pos(w, col); });
    else if (w.use_map) numeric_row_prefetch<false, true>(g, t, R, 0, lane);
    else numeric_row_prefetch<false, false>(g, t, R, 0, lane);
    __syncwarp();
    row_epilogue(g, w, i, Rb, nnz_r, lane, 32);
}

// One CTA of WPR warps per row of class `cls` (accumulator in shared
// memory): the row's entries are split into WPR column ranges of about
// equal size, and warp w applies, in A's row order, only the products whose
// column falls in its range -- disjoint outputs per warp, so the order per
// output is unchanged.  More warps per row means more warps per SM for the
// same shared memory.
template <int WPR>
__global__ void __launch_bounds__(WPR * 32)
k_numeric_rows_split(NumericArgs g, int cls, bool packed)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ int s_part[WPR];
    const int R = g.rowlist[(long long)cls * g.m + blockIdx.x];
    const int i = R >> 4, r = R & (TILE - 1);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long Rb = g.rowptrC[R];
    const int nnz_r = (int)(g.rowptrC[R + 1] - Rb);
    const RowSmem w = row_smem_build(g, s_raw, i, r, nnz_r, tid, WPR * 32, s_part);
    // warp's range: the slots whose row offset lies in [e_lo, e_hi)
    auto first_slot = [&](int e) {
        int lo = 0, hi = w.S;
        while (lo < hi) { const int md = (lo + hi) >> 1; if ((int)(w.word[md] >> 16) < e) lo = md + 1; else hi = md; }
        return lo;
    };
    const long long c0 = g.crp[i];
    auto slot_col = [&](int s) { return (w.use_map ? g.ccol[c0 + s] : w.scol[s]) * TILE; };
    const int sa = first_slot((int)((long long)nnz_r * warp / WPR));
    const int sb = warp + 1 < WPR ? first_slot((int)((long long)nnz_r * (warp + 1) / WPR)) : w.S;
    const int lo = warp == 0 ? INT_MIN : (sa < w.S ? slot_col(sa) : INT_MAX);
    const int hi = sb < w.S ? slot_col(sb) : INT_MAX;
    if (lo < hi) {
        if (packed)
            row_walk_packed(g, R, lane, w.acc, [&](int col) -> long long {
                return (col >= lo && col < hi) ? row_pos(w, col) : -2ll; });
        else
            row_walk_range(g, R, lane, lo, hi, w.acc, [&](int col) -> long long { return row_pos(w, col); });
    }
    __syncthreads();
    row_epilogue(g, w, i, Rb, nnz_r, tid, WPR * 32);
}

// ---- rows too large for a shared-memory accumulator (ROW_WIDE) -------------

// column indices of row R of C (one warp) from its masks.  COALESCE: tile
// rows of more than four entries are written one output position per lane
// (coalesced stores; more shuffles per entry), which pays when many warps
// share the GPU; a lone long row is bound by the length of its warp's chain
// and writes a tile row per lane.
template <bool COALESCE>
__device__ __forceinline__ void row_cols(const NumericArgs &g, int R, int lane)
{
    const int i = R >> 4, r = R & (TILE - 1);
    const int cshift = g.tr_coloff ? g.tr_coloff[i] : 0;
    const long long c0 = g.crp[i];
    const int S = (int)(g.crp[i + 1] - c0);
    const long long Rb = g.rowptrC[R];
    const uint16_t *mrow = g.cmask + c0 * TILE + (long long)r * S;
    const long long nnz_r = g.rowptrC[R + 1] - Rb;
    long long run = 0;
    // 128 slots per round: all their loads issued before any is used; the
    // walk ends with the row's last entry (the tile-row's later tiles, which
    // other rows use, hold nothing of this row)
    for (int sb = 0; sb < S && run < nnz_r; sb += 128) {
        unsigned mkv[4];
        int jbv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int s = sb + 32 * u + lane;
            mkv[u] = s < S ? (unsigned)mrow[s] : 0u;
            jbv[u] = s < S ? g.ccol[c0 + s] * TILE - cshift : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const unsigned mk = mkv[u];
            if (!__ballot_sync(0xffffffffu, mk != 0u)) continue;   // 32 tiles without an entry of this row
            const int cnt = __popc(mk);
            const int incl = warp_incl_scan(cnt, lane);
            const int excl = incl - cnt;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            if constexpr (COALESCE) {
                if (__reduce_max_sync(0xffffffffu, (unsigned)cnt) > 4) {
                    // one output position per lane (coalesced stores): its
                    // slot t is the first lane whose inclusive count exceeds
                    // it, its column the k-th set column of that slot's mask
                    for (int p0 = 0; p0 < total; p0 += 32) {
                        const int p = p0 + lane;
                        int t = 0;
#pragma unroll
                        for (int step = 16; step; step >>= 1)
                            if (__shfl_sync(0xffffffffu, incl, t + step - 1) <= p) t += step;
                        const unsigned mt = __shfl_sync(0xffffffffu, mk, t);
                        const int jt = __shfl_sync(0xffffffffu, jbv[u], t);
                        const int k = p - __shfl_sync(0xffffffffu, excl, t);
                        int x = 0;   // the largest x with popc(columns < x) <= k
#pragma unroll
                        for (int step = 8; step; step >>= 1)
                            if (__popc(mt >> (TILE - (x + step))) <= k) x += step;
                        if (p < total) g.colC[Rb + run + p] = jt + x;
                    }
                    run += total;
                    continue;
                }
            }
            // few entries per tile row: each lane writes its own (a store
            // per entry, consecutive lanes at consecutive positions)
            unsigned m = mk;
            long long dst = Rb + run + excl;
            while (m) {
                const int b = 31 - __clz(m);   // highest bit = smallest local column
                g.colC[dst++] = jbv[u] + (TILE - 1 - b);
                m &= ~(1u << b);
            }
            run += total;
        }
    }
}

// per wide row (one warp each): column indices (the wide kernel zeroes the
// values window by window)
__global__ void __launch_bounds__(256)
k_global_prep(NumericArgs g, int cls, long long nrows)
{
    const long long k = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    if (k >= nrows) return;
    row_cols<false>(g, g.rowlist[(long long)cls * g.m + k], threadIdx.x & 31);
}

// Column indices of every row of C before the numeric kernels.  One CTA per
// tile-row; a tile-row of at most COLS_NARROW C tiles gets a half-warp per
// row, which expands one tile at a time with lane = column in the tile, so
// each store instruction writes one contiguous run of the row.  Wider
// tile-rows are listed for k_cols_wide (a warp per row).
constexpr int COLS_NARROW = 32;
constexpr int COLS_WIDE_GRID = 152 * 8;

__global__ void __launch_bounds__(256)
k_cols_tr(NumericArgs g, int *wide_list, int *wide_n)
{
    const int i = blockIdx.x;
    const long long c0 = g.crp[i];
    const int S = (int)(g.crp[i + 1] - c0);
    if (S == 0) return;
    const int tid = threadIdx.x;
    if (S > COLS_NARROW) {
        if (tid == 0) wide_list[atomicAdd(wide_n, 1)] = i;
        return;
    }
    const int hl = tid & 15, r = tid >> 4;
    const int R = i * TILE + r;
    if (R >= g.m) return;                       // whole half-warps leave together
    const unsigned hmask = 0xffffu << (tid & 16);
    const int cshift = g.tr_coloff ? g.tr_coloff[i] : 0;
    const long long Rb = g.rowptrC[R];
    const uint16_t *mrow = g.cmask + c0 * TILE + (long long)r * S;
    int run = 0;
    for (int sb = 0; sb < S; sb += 16) {
        const int sl = sb + hl;
        const unsigned mk = sl < S ? (unsigned)mrow[sl] : 0u;
        const int jb = sl < S ? g.ccol[c0 + sl] * TILE - cshift : 0;
        const int cnt = __popc(mk);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
            const int t = __shfl_up_sync(hmask, incl, o, 16);
            if (hl >= o) incl += t;
        }
        const int excl = incl - cnt;
        const int nt = min(16, S - sb);
        for (int t = 0; t < nt; ++t) {
            const unsigned mt = __shfl_sync(hmask, mk, t, 16);
            const int jt = __shfl_sync(hmask, jb, t, 16);
            const int et = __shfl_sync(hmask, excl, t, 16);
            if ((mt >> (TILE - 1 - hl)) & 1u)   // local column hl is bit 15 - hl
                g.colC[Rb + run + et + __popc(mt >> (TILE - hl))] = jt + hl;
        }
        run += __shfl_sync(hmask, incl, 15, 16);
    }
}

// rows of the tile-rows k_cols_tr listed: a warp per row over the whole GPU
__global__ void __launch_bounds__(256)
k_cols_wide(NumericArgs g, const int *wide_list, const int *wide_n)
{
    const long long nrows = (long long)(*wide_n) * TILE;
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long k = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; k < nrows; k += nw) {
        const int R = wide_list[k >> 4] * TILE + (int)(k & (TILE - 1));
        if (R < g.m) row_cols<true>(g, R, threadIdx.x & 31);
    }
}

constexpr int WIDE_W = 512;    // tile columns per window of the wide-row kernels (accumulator in C)
constexpr int WIDE_WARP_BYTES = WIDE_W * (4 + 2);   // shared memory per warp
constexpr size_t WIDE_SMEM = (size_t)ROW_WARPS * WIDE_WARP_BYTES;
// windows with the accumulator in shared memory: tile columns and entries
constexpr int WS_W = 256, WS_E = 256;
// Wide rows with more A entries than LONG_NA (all of them, measured
// fastest) are cut into parts of at most LONG_W tile columns, each part one
// warp's work anywhere on the GPU (k_long_walk); their B rows' cut points
// come from a table built once.
constexpr int LONG_NA = 0;
constexpr int LONG_MINP = 32;        // parts of such a row at least (more warps than the per-row kernel's 8)
constexpr int LONG_GRID = 152 * 5;   // CTAs of the part walk: five per SM
constexpr int LONG_MIN_TILES = 1024; // C's tile columns from which wide rows take the parts path
constexpr long long LONG_TAB_MAX = 1ll << 31;   // cut-table entries (8 GB) beyond which long rows stay per row
constexpr int LONG_W = 512;     // tile columns per part at most
constexpr int LONG_ACC = 128;   // a part's entries up to which its accumulators sit in the warp's shared memory
constexpr int LONG_WARP_BYTES = LONG_W * 4 + LONG_ACC * 8;
static_assert(LONG_W * TILE <= 65536, "a part's offsets fit 16 bits");
constexpr size_t LONG_SMEM = (size_t)ROW_WARPS * LONG_WARP_BYTES;
static_assert(4 * WS_W + 8 * WS_E <= WIDE_WARP_BYTES, "shared-memory windows fit the warp's share");

// A wide row's share [t0, t1) of tile columns, for A rows of up to 32
// entries and sorted B rows: windows of at most WS_W tile columns and WS_E
// entries, each with its mask/offset table and its values in the warp's
// shared memory, written out to C in one coalesced pass.  Lane q keeps A
// entry q and a cursor into its B row: one binary search for the share's
// first column, then each window takes the B entries from the cursor on
// while their columns stay below the window's end (one ballot per 32), so
// no window searches the B rows.  A entries follow one another in order
// (with a warp barrier between them), so per output the products come in
// A's row order, then B's.  (Longer A rows keep the accumulator in C: with
// small windows their B rows would be searched again for every window.)
__device__ __noinline__ void wide_windows_smem(const NumericArgs &g, int R, int lane, unsigned char *wbase,
                                               const uint16_t *mrow, const int *tcol, int S, long long Rb, int nnz_r,
                                               int cshift, int t0, int t1, int pa0, int na)
{
    unsigned short *w_msk = reinterpret_cast<unsigned short *>(wbase);
    unsigned short *w_off = w_msk + WS_W;
    double *w_acc = reinterpret_cast<double *>(wbase + 4 * WS_W);
    for (int t = lane; t < WS_W; t += 32) w_msk[t] = 0;
    int cur = 0, bend = 0;
    double av = 0.0;
    if (lane < na) {
        const int k = g.colA[pa0 + lane];
        av = g.valA[pa0 + lane];
        cur = (int)g.rpB[k];
        bend = (int)g.rpB[k + 1];
        const int key = t0 * TILE;
        int h = bend;
        while (cur < h) { const int md = (cur + h) >> 1; if (g.colB[md] < key) cur = md + 1; else h = md; }
    }
    __syncwarp();
    bool bad = false;
    int sa = warp_lower_bound(tcol, 0, S, t0, lane);
    // C offset of the share's first entry; each window then starts where the last ended
    long long wg = sa < S ? Rb + warp_lower_bound(g.colC + Rb, 0, nnz_r, tcol[sa] * TILE - cshift, lane) : Rb;
    while (sa < S && tcol[sa] < t1) {
        const int j0 = tcol[sa];
        const int jlim = (int)min((long long)t1, (long long)j0 + WS_W);
        // the window: slots from sa while the tile column is below jlim and
        // the entries fit; tile columns and masks loaded 128 slots at a time
        int nwin = 0, s = sa;
        bool more = true;
        while (more) {
            int tcv[4];
            unsigned mkv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int ss = s + 32 * u + lane;
                tcv[u] = ss < S ? tcol[ss] : INT_MAX;
                mkv[u] = ss < S ? (unsigned)mrow[ss] : 0u;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (more) {
                    const bool inr = tcv[u] < jlim;
                    const int c = inr ? __popc(mkv[u]) : 0;
                    const int incl = warp_incl_scan(c, lane);
                    const bool ok = inr && nwin + incl <= WS_E;
                    const int nok = __popc(__ballot_sync(0xffffffffu, ok));
                    if (ok && mkv[u]) {
                        w_msk[tcv[u] - j0] = (unsigned short)mkv[u];
                        w_off[tcv[u] - j0] = (unsigned short)(nwin + incl - c);
                    }
                    if (nok > 0) nwin += __shfl_sync(0xffffffffu, incl, nok - 1);
                    s += nok;
                    if (nok < 32) more = false;
                }
            }
        }
        const int sb = s;
        // B columns from the next slot's tile column on belong to later windows
        const int tnext = sb < S ? tcol[sb] : INT_MAX;
        const int hi = (tnext < t1) ? tnext * TILE : (t1 == INT_MAX ? INT_MAX : t1 * TILE);
        for (int t = lane; t < nwin; t += 32) w_acc[t] = 0.0;
        __syncwarp();
        // the B entries of one A entry from position c0 on, below hi
        auto segment = [&](int c0, int bq, double a) -> int {
            for (;;) {
                const int e = c0 + lane;
                int col = INT_MAX;
                double b = 0.0;
                if (e < bq) { col = g.colB[e]; b = g.valB[e]; }
                const bool in = col < hi;
                if (in) {
                    const int t = (col >> 4) - j0, cc = col & 15;
                    const unsigned mk = (unsigned)t < (unsigned)WS_W ? w_msk[t] : 0u;
                    if ((mk >> (TILE - 1 - cc)) & 1u) {
                        const int p = w_off[t] + __popc(mk >> (TILE - cc));
                        w_acc[p] = fma(a, b, w_acc[p]);
                    } else {
                        bad = true;
                    }
                }
                const int n = __popc(__ballot_sync(0xffffffffu, in));
                c0 += n;
                if (n < 32) return c0;
            }
        };
        for (int q = 0; q < na; ++q) {
            const int c1 = segment(__shfl_sync(0xffffffffu, cur, q), __shfl_sync(0xffffffffu, bend, q),
                                   __shfl_sync(0xffffffffu, av, q));
            if (lane == q) cur = c1;
            __syncwarp();
        }
        for (int t = lane; t < nwin; t += 32) g.valC[wg + t] = w_acc[t];
        wg += nwin;
        for (int ss = sa + lane; ss < sb; ss += 32) {
            const int tc = tcol[ss];
            if (tc - j0 < WS_W) w_msk[tc - j0] = 0;
        }
        __syncwarp();
        sa = sb;
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

// One CTA of ROW_WARPS warps per wide row; the values accumulate in place in
// C (columns written by k_global_prep, values zeroed per window here).  The row's entries are
// split into ROW_WARPS column ranges of about equal size (read off C's
// column indices), and warp w walks its range in windows of at most WIDE_W
// tile columns: for a window it tabulates, by tile column, the row's mask
// and the offset of its segment in the row (the warp's own 12 KB of shared
// memory), then applies A's row in order, each A entry's B row restricted
// to the window.  Ranges and windows are disjoint in columns, so per output
// the products still come in A's row order.
template <int WPR>
__global__ void __launch_bounds__(ROW_WARPS * 32, 4)
k_numeric_wide(NumericArgs g, int cls, long long nrows, bool packed, const unsigned char *handled)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *wbase = s_raw + (size_t)warp * WIDE_WARP_BYTES;   // this warp's shared memory
    unsigned *s_off = reinterpret_cast<unsigned *>(wbase);
    unsigned short *s_msk = reinterpret_cast<unsigned short *>(wbase + (size_t)WIDE_W * 4);
    // WPR warps per row: ROW_WARPS (one row per CTA, the warps split its
    // entries) or 1 (ROW_WARPS rows per CTA, one warp each)
    const long long idx = WPR == 1 ? (long long)blockIdx.x * ROW_WARPS + warp : (long long)blockIdx.x;
    if (idx >= nrows) return;
    const int part = WPR == 1 ? 0 : warp;
    const int R = g.rowlist[(long long)cls * g.m + idx];
    if (handled && handled[idx]) return;   // k_long_walk's row
    const int i = R >> 4, r = R & (TILE - 1);
    const long long c0 = g.crp[i];
    const int S = (int)(g.crp[i + 1] - c0);
    const long long Rb = g.rowptrC[R];
    const int nnz_r = (int)(g.rowptrC[R + 1] - Rb);
    const uint16_t *mrow = g.cmask + c0 * TILE + (long long)r * S;
    const int *tcol = g.ccol + c0;
    const int cshift = g.tr_coloff ? g.tr_coloff[i] : 0;
    // this warp's entries [e0, e1) and their tile columns [t0, t1)
    const int e0 = (int)((long long)nnz_r * part / WPR), e1 = (int)((long long)nnz_r * (part + 1) / WPR);
    if (e0 >= e1) return;
    const int t0 = (g.colC[Rb + e0] + cshift) >> 4;
    const int t1 = e1 < nnz_r ? (g.colC[Rb + e1] + cshift) >> 4 : INT_MAX;
    if (t0 >= t1) return;   // the range starts inside the previous warp's last tile column
    {
        const int pa0 = (int)g.rpA[R], pa1 = (int)g.rpA[R + 1];
        if (!packed && g.b_sorted && pa1 - pa0 <= 32) {
            wide_windows_smem(g, R, lane, wbase, mrow, tcol, S, Rb, nnz_r, cshift, t0, t1, pa0, pa1 - pa0);
            return;
        }
    }
    for (int t = lane; t < WIDE_W; t += 32) s_msk[t] = 0;
    __syncwarp();
    int sa = warp_lower_bound(tcol, 0, S, t0, lane);
    while (sa < S && tcol[sa] < t1) {
        const int j0 = tcol[sa];
        const int jend = (int)min((long long)t1, (long long)j0 + WIDE_W);
        const int sb = warp_lower_bound(tcol, sa, S, jend, lane);
        // offset of the window's first entry in the row, from C's columns
        unsigned run = (unsigned)warp_lower_bound(g.colC + Rb, 0, nnz_r, j0 * TILE - cshift, lane);
        for (int s = sa; s < sb; s += 32) {
            const int ss = s + lane;
            const unsigned mk = ss < sb ? (unsigned)mrow[ss] : 0u;
            const int c = __popc(mk);
            const int incl = warp_incl_scan(c, lane);
            if (mk) {
                const int t = tcol[ss] - j0;
                s_off[t] = run + incl - c;
                s_msk[t] = (unsigned short)mk;
                // the segment's values zeroed just before the walk updates
                // them, so they are still in L2 then
                const long long dst = Rb + run + incl - c;
                for (int q = 0; q < c; ++q) g.valC[dst + q] = 0.0;
            }
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        __syncwarp();
        const int lo = j0 * TILE, hi = jend * TILE;
        auto pos_of = [&](int col) -> long long {
            const int t = (col >> 4) - j0, cc = col & 15;
            const unsigned mk = s_msk[t];
            return ((mk >> (TILE - 1 - cc)) & 1u) ? Rb + s_off[t] + __popc(mk >> (TILE - cc)) : -1ll;
        };
        if (packed)
            row_walk_packed(g, R, lane, g.valC, [&](int col) -> long long {
                return (col >= lo && col < hi) ? pos_of(col) : -2ll; });
        else
            row_walk_range(g, R, lane, lo, hi, g.valC, pos_of);
        for (int ss = sa + lane; ss < sb; ss += 32) s_msk[tcol[ss] - j0] = 0;
        __syncwarp();
        sa = sb;
    }
}

// ---- wide rows of long A rows: parts and the cut table ---------------------
//
// A row's span of tile columns [T0, T1] (from C's first and last column) is
// cut into P = max(ceil(span / LONG_W), LONG_MINP) parts of Wp = ceil(span /
// P) tile columns.  The cut table holds, for each A entry p of the row and each part
// boundary j = 0..P, the first entry of B's row k_p whose column is at or
// past the boundary (at [j * na + p], so a part reads its 32 A entries
// coalesced).  A part is one warp's work anywhere on the GPU: a window of
// the per-row kernel (mask/offset table by tile column, values accumulated
// in C) whose B segments come straight from the table -- no search of B on
// the walk's path, and a row with thousands of A entries spreads over many
// warps instead of eight.  Parts hold disjoint columns and each walks A's
// entries in order, so per output the products come in A's row order, then
// B's.

struct LongRow {
    int na, pa0, P, T0, Wp, cshift, nnz_r;
    long long Rb;
};

// A long row's walk data, computed once per call (k_long_list, k_long_fit)
struct LongRowDesc {
    long long Rb;        // the row's first entry of C
    long long c0;        // its tile-row's first C tile
    long long tab_off;   // its cut table
    int R, pa0, na, T0, Wp, cshift, S, nnz_r;
};
// A part of a long row (k_long_parts): the row (l < 0: skipped), the part's
// index j, its C tile slots [sa, sb) and its first entry of C in the row
struct LongPart {
    int l, j, sa, sb, first, pad0, pad1, pad2;
};
static_assert(sizeof(LongPart) == 32, "two 16-byte loads");

__device__ __forceinline__ LongRow long_row(const NumericArgs &g, int R)
{
    LongRow L;
    L.pa0 = (int)g.rpA[R];
    L.na = (int)g.rpA[R + 1] - L.pa0;
    L.Rb = g.rowptrC[R];
    L.nnz_r = (int)(g.rowptrC[R + 1] - L.Rb);
    L.cshift = g.tr_coloff ? g.tr_coloff[R >> 4] : 0;
    L.P = 0; L.T0 = 0; L.Wp = 1;
    if (L.na > LONG_NA && L.nnz_r > 0) {
        L.T0 = (g.colC[L.Rb] + L.cshift) >> 4;
        const int span = ((g.colC[L.Rb + L.nnz_r - 1] + L.cshift) >> 4) - L.T0 + 1;
        L.P = max((span + LONG_W - 1) / LONG_W, min(span, LONG_MINP));
        L.Wp = (span + L.P - 1) / L.P;
        L.P = (span + L.Wp - 1) / L.Wp;   // no empty trailing part
    }
    return L;
}

// per wide row: 1 when its A row is long enough for the parts path
__global__ void __launch_bounds__(256)
k_long_flag(NumericArgs g, int cls, long long nrows, int *flag)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= nrows) return;
    flag[idx] = long_row(g, g.rowlist[(long long)cls * g.m + idx]).P > 0 ? 1 : 0;
}

// the long rows in order (l = lpos[idx]): wide-row index, row, parts, A
// entries and cut-table size; entries past the last long row stay zero
__global__ void __launch_bounds__(256)
k_long_list(NumericArgs g, int cls, long long nrows, const int *lpos, int *lidx, int *lrow, int *parts, int *nas,
            long long *tabsz, LongRowDesc *rdesc)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= nrows || lpos[idx + 1] == lpos[idx]) return;
    const int R = g.rowlist[(long long)cls * g.m + idx];
    const LongRow L = long_row(g, R);
    const int l = lpos[idx];
    lidx[l] = (int)idx;
    lrow[l] = R;
    parts[l] = L.P;
    nas[l] = L.na;
    tabsz[l] = (long long)L.na * (L.P + 1);
    LongRowDesc d;
    d.Rb = L.Rb;
    d.c0 = g.crp[R >> 4];
    d.tab_off = 0;   // set by k_long_fit
    d.R = R; d.pa0 = L.pa0; d.na = L.na; d.T0 = L.T0; d.Wp = L.Wp; d.cshift = L.cshift;
    d.S = (int)(g.crp[(R >> 4) + 1] - d.c0);
    d.nnz_r = L.nnz_r;
    rdesc[l] = d;
}

// rows whose cut table fits the allocation take the parts path
// (handled[idx] = 1); the others stay with k_numeric_wide
__global__ void __launch_bounds__(256)
k_long_fit(long long nrows, const int *lpos, const int *lidx, const long long *tab_off, long long cap,
           unsigned char *handled, unsigned char *lfit, LongRowDesc *rdesc)
{
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (l >= nrows || l >= lpos[nrows]) return;
    const bool fit = tab_off[l + 1] <= cap;
    lfit[l] = fit ? 1 : 0;
    handled[lidx[l]] = fit ? 1 : 0;
    rdesc[l].tab_off = tab_off[l];
}

// first index in [lo, hi) whose value is >= key (one thread's binary search)
__device__ __forceinline__ int lb_range(const int *__restrict__ a, int lo, int hi, int key)
{
    while (lo < hi) {
        const int md = (lo + hi) >> 1;
        if (a[md] < key) lo = md + 1; else hi = md;
    }
    return lo;
}

// Every part's walk data, so that a part of the walk starts from two loads:
// one warp per long row, lanes over its parts -- the part's C tile slots
// [sa, sb) of the tile-row and its first entry of C within the row (binary
// searches of the tile columns and of the row's columns).  Parts of rows
// whose cut table did not fit get l = -1 (the walk skips them).
__global__ void __launch_bounds__(256)
k_long_parts(NumericArgs g, long long nrows, const int *lpos, const unsigned char *lfit, const int *part_off,
             const LongRowDesc *rdesc, LongPart *pdesc)
{
    const int lane = threadIdx.x & 31;
    const long long nw = (long long)gridDim.x * 8, w0 = blockIdx.x * 8LL + (threadIdx.x >> 5);
    const long long nl = lpos[nrows];
    for (long long l = w0; l < nl; l += nw) {
        const LongRowDesc d = rdesc[l];
        const int p0 = part_off[l], np = part_off[l + 1] - p0;
        const bool fit = lfit[l] != 0;
        const int *tcol = g.ccol + d.c0;
        for (int j = lane; j < np; j += 32) {
            LongPart pt;
            pt.l = fit ? (int)l : -1;
            pt.j = j;
            pt.sa = pt.sb = pt.first = 0;
            if (fit) {
                const int wlo = d.T0 + j * d.Wp;
                pt.sa = lb_range(tcol, 0, d.S, wlo);
                pt.sb = lb_range(tcol, pt.sa, d.S, wlo + d.Wp);
                pt.first = lb_range(g.colC + d.Rb, 0, d.nnz_r, wlo * TILE - d.cshift);
            }
            pdesc[p0 + j] = pt;
        }
    }
}

// last l in [0, n) with off[l] <= v (off nondecreasing, off[0] <= v)
template <typename T>
__device__ __forceinline__ long long last_le(const T *off, long long n, long long v)
{
    long long lo = 0, hi = n - 1;
    while (lo < hi) { const long long md = (lo + hi + 1) >> 1; if ((long long)off[md] <= v) lo = md; else hi = md - 1; }
    return lo;
}

// the cut table: each warp a contiguous run of the long rows' A entries
// (na_off: prefix of their counts), lanes over an entry's boundaries
__global__ void __launch_bounds__(256)
k_long_cuts(NumericArgs g, long long nrows, const int *lrow, const unsigned char *lfit, const long long *na_off,
            const long long *tab_off, int *tab)
{
    const int lane = threadIdx.x & 31;
    const long long nw = (long long)gridDim.x * 8, w = blockIdx.x * 8LL + (threadIdx.x >> 5);
    const long long total = na_off[nrows];
    const long long ch = (total + nw - 1) / nw;
    const long long e0 = w * ch, e1 = min(total, e0 + ch);
    if (e0 >= e1) return;
    long long l = last_le(na_off, nrows, e0);
    int R = lrow[l];
    LongRow L = long_row(g, R);
    for (long long e = e0; e < e1; ++e) {
        while (na_off[l + 1] <= e) { ++l; R = lrow[l]; L = long_row(g, R); }
        if (!lfit[l]) continue;
        const int p = (int)(e - na_off[l]);
        const int k = g.colA[L.pa0 + p];
        const int bs = (int)g.rpB[k], be = (int)g.rpB[k + 1];
        int *t = tab + tab_off[l];
        for (int j = lane; j <= L.P; j += 32) {
            int v;
            if (j == 0) v = bs;
            else if (j == L.P) v = be;
            else {
                const int key = (L.T0 + j * L.Wp) * TILE;
                int lo = bs, hi = be;
                while (lo < hi) { const int md = (lo + hi) >> 1; if (g.colB[md] < key) lo = md + 1; else hi = md; }
                v = lo;
            }
            t[(long long)j * L.na + p] = v;
        }
    }
}

// the walk: each warp takes the next part from a counter until none is
// left (parts differ widely in cost, so a static share would leave warps
// idle behind the hub rows' parts)
__global__ void __launch_bounds__(ROW_WARPS * 32, 5)
k_long_walk(NumericArgs g, long long nrows, const int *part_off, const LongRowDesc *__restrict__ rdesc,
            const LongPart *__restrict__ pdesc, const int *tab, unsigned long long *next_part)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *wbase = s_raw + (size_t)warp * LONG_WARP_BYTES;
    unsigned short *s_off = reinterpret_cast<unsigned short *>(wbase);   // < LONG_W * TILE
    unsigned short *s_msk = reinterpret_cast<unsigned short *>(wbase + (size_t)LONG_W * 2);
    double *s_acc = reinterpret_cast<double *>(wbase + (size_t)LONG_W * 4);
    for (int t = lane; t < LONG_W; t += 32) s_msk[t] = 0;
    __syncwarp();
    const long long nparts = part_off[nrows];
    bool bad = false;
    for (;;) {
        // one part per fetch (consecutive parts of a hub row are all heavy:
        // taking several at a time left warps busy behind the rest)
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(next_part, 1ull);
        const long long gp = (long long)__shfl_sync(0xffffffffu, t, 0);
        if (gp >= nparts) break;
        const LongPart pt = pdesc[gp];   // the part's long row, tile slots and first entry (k_long_parts)
        if (pt.l < 0) continue;
        const LongRowDesc L = rdesc[pt.l];
        const int j = pt.j;
        const int r = L.R & (TILE - 1);
        const int S = L.S;
        const uint16_t *mrow = g.cmask + L.c0 * TILE + (long long)r * S;
        const int *tcol = g.ccol + L.c0;
        const int wlo = L.T0 + j * L.Wp, whi = wlo + L.Wp;   // tile columns [wlo, whi)
        const int sa = pt.sa, sb = pt.sb;
        if (sa >= sb) continue;
        // the part's entries of C: [Rb + first, Rb + first + E); s_off
        // holds each tile's offset among them
        const unsigned first = (unsigned)pt.first;
        unsigned run = 0;
        for (int s = sa; s < sb; s += 32) {
            const int ss = s + lane;
            const unsigned mk = ss < sb ? (unsigned)mrow[ss] : 0u;
            const int c = __popc(mk);
            const int incl = warp_incl_scan(c, lane);
            if (mk) {
                const int t = tcol[ss] - wlo;
                s_off[t] = (unsigned short)(run + incl - c);
                s_msk[t] = (unsigned short)mk;
            }
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        const int E = (int)run;
        double *gacc = g.valC + L.Rb + first;
        // accumulators zeroed just before the walk: in the warp's shared
        // memory when the part's entries fit there (written out after it),
        // else in C's values
        const bool sm = E <= LONG_ACC;
        for (int q = lane; q < E; q += 32) {
            if (sm) s_acc[q] = 0.0; else gacc[q] = 0.0;
        }
        __syncwarp();
        if (E > 0) {
            auto pos_of = [&](int col) -> int {
                const int t = (col >> 4) - wlo, cc = col & 15;
                const unsigned mk = s_msk[t];
                return ((mk >> (TILE - 1 - cc)) & 1u) ? (int)s_off[t] + __popc(mk >> (TILE - cc)) : -1;
            };
            const int *tb = tab + L.tab_off;
            for (int pb = 0; pb < L.na; pb += 32) {
                const int nb = min(32, L.na - pb);
                int bs = 0, be = 0;
                double av = 0.0;
                if (lane < nb) {
                    av = g.valA[L.pa0 + pb + lane];
                    bs = tb[(long long)j * L.na + pb + lane];
                    be = tb[(long long)(j + 1) * L.na + pb + lane];
                }
                if (sm) walk_segments(g, lane, nb, av, bs, be, wlo * TILE, whi * TILE, s_acc, pos_of, bad);
                else walk_segments(g, lane, nb, av, bs, be, wlo * TILE, whi * TILE, gacc, pos_of, bad);
            }
            if (sm) {
                __syncwarp();
                for (int q = lane; q < E; q += 32) gacc[q] = s_acc[q];
            }
        }
        for (int ss = sa + lane; ss < sb; ss += 32) s_msk[tcol[ss] - wlo] = 0;
        __syncwarp();
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

template <int NT, bool DENSE, int WALK>
cudaError_t set_smem_attr() {
    cudaError_t e = cudaFuncSetAttribute(k_numeric_smem<NT, DENSE, WALK>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LARGE);
    // the whole unified L1 as shared memory, so occupancy is set by the
    // tile-row's actual request, not by a smaller carveout
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_numeric_smem<NT, DENSE, WALK>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    return e;
}

template <int NT>
cudaError_t launch_smem(const NumericArgs &a, int bin, long long nrows, long long smem, bool dense, int walk,
                        cudaStream_t s) {
    const unsigned grid = (unsigned)nrows;
#define TSG_L(D, W) { k_numeric_smem<NT, D, W><<<grid, NT, smem, s>>>(a, bin); ::tsg::count_launch(); }
    if (dense) { if (walk == 1) TSG_L(true, 1) else if (walk == 2) TSG_L(true, 2) else TSG_L(true, 0) }
    else { if (walk == 1) TSG_L(false, 1) else if (walk == 2) TSG_L(false, 2) else TSG_L(false, 0) }
#undef TSG_L
    return cudaGetLastError();
}

}  // namespace

cudaError_t numeric_init_attributes()
{
    cudaError_t e = cudaSuccess;
#define TSG_SET(NT)                                                    \
    if (e == cudaSuccess) e = set_smem_attr<NT, false, 0>();           \
    if (e == cudaSuccess) e = set_smem_attr<NT, false, 1>();           \
    if (e == cudaSuccess) e = set_smem_attr<NT, false, 2>();           \
    if (e == cudaSuccess) e = set_smem_attr<NT, true, 0>();            \
    if (e == cudaSuccess) e = set_smem_attr<NT, true, 1>();            \
    if (e == cudaSuccess) e = set_smem_attr<NT, true, 2>();
    TSG_SET(128)
    TSG_SET(256)
    TSG_SET(512)
#undef TSG_SET
    const void *fs[6] = {(const void *)k_numeric_rows, (const void *)k_numeric_rows_split<ROW_WARPS>,
                         (const void *)k_numeric_rows_split<4>, (const void *)k_numeric_rows_split<2>,
                         (const void *)k_numeric_wide<ROW_WARPS>, (const void *)k_numeric_wide<1>};
    for (const void *f : fs) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LARGE);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    }
    return e;
}

namespace {

// scratch of the parts path (pool memory, released after the walk)
struct LongScratch {
    int *flag = nullptr, *lpos = nullptr, *lidx = nullptr, *lrow = nullptr, *parts = nullptr, *nas = nullptr,
        *part_off = nullptr;
    long long *tabsz = nullptr, *na_off = nullptr, *tab_off = nullptr;
    unsigned char *handled = nullptr, *lfit = nullptr;
    int *tab = nullptr;
    unsigned long long *next_part = nullptr;   // the walk's work counter
    LongRowDesc *rdesc = nullptr;              // per long row (n at most)
    LongPart *pdesc = nullptr;                 // per part
};

void long_release(Pool &pool, LongScratch &L)
{
    for (void *p : {(void *)L.flag, (void *)L.lpos, (void *)L.lidx, (void *)L.lrow, (void *)L.parts, (void *)L.nas,
                    (void *)L.part_off, (void *)L.tabsz, (void *)L.na_off, (void *)L.tab_off, (void *)L.handled,
                    (void *)L.lfit, (void *)L.tab, (void *)L.next_part, (void *)L.rdesc, (void *)L.pdesc})
        pool.free(p);
    L = LongScratch{};
}

// the long rows' list, part and A-entry prefixes, and the cut table
cudaError_t long_prepare(Pool &pool, const NumericArgs &a, int cls, long long n, long long tab_bound,
                         long long parts_bound, LongScratch &L)
{
    cudaStream_t s = pool.stream;
    L.flag = pool.alloc_n<int>(n + 1);
    L.lpos = pool.alloc_n<int>(n + 1);
    L.lidx = pool.alloc_n<int>(n);
    L.handled = pool.alloc_n<unsigned char>(n);
    L.lfit = pool.alloc_n<unsigned char>(n);
    L.lrow = pool.alloc_n<int>(n);
    L.parts = pool.alloc_n<int>(n + 1);
    L.nas = pool.alloc_n<int>(n + 1);
    L.part_off = pool.alloc_n<int>(n + 1);
    L.tabsz = pool.alloc_n<long long>(n + 1);
    L.na_off = pool.alloc_n<long long>(n + 1);
    L.tab_off = pool.alloc_n<long long>(n + 1);
    L.next_part = pool.alloc_n<unsigned long long>(1);
    L.rdesc = pool.alloc_n<LongRowDesc>(n);
    if (!L.flag || !L.lpos || !L.lidx || !L.handled || !L.lfit || !L.lrow || !L.parts || !L.nas || !L.part_off ||
        !L.tabsz || !L.na_off || !L.tab_off || !L.next_part || !L.rdesc) {
        const cudaError_t err = pool.err != cudaSuccess ? pool.err : cudaErrorMemoryAllocation;
        long_release(pool, L);
        return err;
    }
    cudaError_t e = cudaMemsetAsync(L.parts, 0, sizeof(int) * (size_t)n, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(L.next_part, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(L.handled, 0, (size_t)n, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(L.lfit, 0, (size_t)n, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(L.nas, 0, sizeof(int) * (size_t)n, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(L.tabsz, 0, sizeof(long long) * (size_t)n, s);
    const unsigned gb = (unsigned)((n + 255) / 256);
    if (e == cudaSuccess) { k_long_flag<<<gb, 256, 0, s>>>(a, cls, n, L.flag); ::tsg::count_launch(); e = cudaGetLastError(); }
    if (e == cudaSuccess) e = scan_i32_to_i32(pool, L.flag, L.lpos, n, a.flags);
    if (e == cudaSuccess) {
        k_long_list<<<gb, 256, 0, s>>>(a, cls, n, L.lpos, L.lidx, L.lrow, L.parts, L.nas, L.tabsz, L.rdesc);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = scan_i32_to_i32(pool, L.parts, L.part_off, n, a.flags);
    if (e == cudaSuccess) e = scan_i32_to_i64(pool, L.nas, L.na_off, n, a.flags);
    if (e == cudaSuccess) e = scan_i64_to_i64(pool, L.tabsz, L.tab_off, n, a.flags);
    // the cut table: its exact size when the stream can wait for it, else
    // the bound (inside a graph capture)
    // (and the parts' descriptors: their exact count, or the bound)
    long long cap = tab_bound, nparts = parts_bound;
    if (e == cudaSuccess) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        e = cudaStreamIsCapturing(s, &cs);
        if (e == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
            long long need = 0;
            int np = 0;
            e = cudaMemcpyAsync(&need, L.tab_off + n, sizeof(long long), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(&np, L.part_off + n, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            cap = std::min(tab_bound, need);
            nparts = np;
        }
    }
    if (e == cudaSuccess) {
        L.tab = pool.alloc_n<int>(cap);
        L.pdesc = pool.alloc_n<LongPart>(nparts);
        if (!L.tab || !L.pdesc) e = pool.err != cudaSuccess ? pool.err : cudaErrorMemoryAllocation;
    }
    if (e == cudaSuccess) {
        k_long_fit<<<gb, 256, 0, s>>>(n, L.lpos, L.lidx, L.tab_off, cap, L.handled, L.lfit, L.rdesc);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_long_parts<<<LONG_GRID * 2, 256, 0, s>>>(a, n, L.lpos, L.lfit, L.part_off, L.rdesc, L.pdesc);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_long_cuts<<<LONG_GRID * 2, 256, 0, s>>>(a, n, L.lrow, L.lfit, L.na_off, L.tab_off, L.tab);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) long_release(pool, L);
    return e;
}

}  // namespace

cudaError_t numeric_cols(Pool &pool, const NumericArgs &a)
{
    if (a.m <= 0 || a.blkm <= 0) return cudaSuccess;
    int *wide = pool.alloc_n<int>((long long)a.blkm + 1);
    if (!wide) return cudaErrorMemoryAllocation;
    int *wide_n = wide + a.blkm;
    cudaError_t e = cudaMemsetAsync(wide_n, 0, sizeof(int), pool.stream);
    if (e == cudaSuccess) {
        k_cols_tr<<<(unsigned)a.blkm, 256, 0, pool.stream>>>(a, wide, wide_n);
        ::tsg::count_launch();
        k_cols_wide<<<COLS_WIDE_GRID, 256, 0, pool.stream>>>(a, wide, wide_n);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    pool.free(wide);
    return e;
}

cudaError_t numeric_run(Pool &pool, const NumericArgs &a, const long long *binstat, int walk, int threads,
                        int row_warps, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join)
{
    const bool packed = walk == 1;
    const long long *counts = binstat, *req = binstat + NBIN;
    const long long *rcnt = binstat + BS_ROWCNT, *rreq = binstat + BS_ROWREQ;
    cudaError_t e = cudaSuccess;
    // two streams when there are rows besides the tile-row bins' (disjoint
    // rows of C, joined at the end): the bins -- and, with wide rows, the
    // shared-memory row classes -- run on the side stream
    const bool wide = rcnt[ROW_WIDE] > 0 || rcnt[ROW_WIDE1] > 0;
    const bool rows = rcnt[ROW_S] > 0 || rcnt[ROW_M] > 0 || rcnt[ROW_L] > 0;
    bool bins = false;
    for (int b = BIN_SPARSE_S; b <= BIN_DENSE_L; ++b) bins = bins || counts[b] > 0;
    const bool split = side && (wide || (rows && bins));
    cudaStream_t s = pool.stream;
    if (split) {
        e = cudaEventRecord(fork, pool.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork, 0);
        if (e != cudaSuccess) return e;
        s = side;
    }
    for (int b = BIN_SPARSE_S; b <= BIN_DENSE_L && e == cudaSuccess; ++b) {
        if (counts[b] == 0) continue;
        const bool dense = b >= BIN_DENSE_S;
        const long long smem = req[b];
        // bins whose shared memory leaves one or two CTAs per SM run 16 warps, one per row
        const int nt = (b == BIN_SPARSE_S || b == BIN_DENSE_S) ? threads : std::max(threads, 512);
        if (nt == 128) e = launch_smem<128>(a, b, counts[b], smem, dense, walk, s);
        else if (nt == 512) e = launch_smem<512>(a, b, counts[b], smem, dense, walk, s);
        else e = launch_smem<256>(a, b, counts[b], smem, dense, walk, s);
    }
    if (split && !wide) {   // the row classes on the main stream beside the bins
        if (e == cudaSuccess) e = cudaEventRecord(join, side);
        s = pool.stream;
    }
    for (int c = ROW_S; c <= ROW_M && e == cudaSuccess; ++c) {
        if (rcnt[c] == 0) continue;
        const unsigned g = (unsigned)rcnt[c];
        const size_t sm = (size_t)rreq[c];
        if (row_warps >= 8) { k_numeric_rows_split<ROW_WARPS><<<g, ROW_WARPS * 32, sm, s>>>(a, c, packed); ::tsg::count_launch(); }
        else if (row_warps >= 4) { k_numeric_rows_split<4><<<g, 128, sm, s>>>(a, c, packed); ::tsg::count_launch(); }
        else if (row_warps == 2) { k_numeric_rows_split<2><<<g, 64, sm, s>>>(a, c, packed); ::tsg::count_launch(); }
        else { k_numeric_rows<<<g, 32, sm, s>>>(a, c, packed); ::tsg::count_launch(); }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && rcnt[ROW_L] > 0) {
        { k_numeric_rows_split<ROW_WARPS><<<(unsigned)rcnt[ROW_L], ROW_WARPS * 32, (size_t)rreq[ROW_L], s>>>(a, ROW_L, packed); ::tsg::count_launch(); }
        e = cudaGetLastError();
    }
    if (split && wide) {
        if (e == cudaSuccess) e = cudaEventRecord(join, side);
        s = pool.stream;
    }
    for (int c = ROW_WIDE; c <= ROW_WIDE1 && e == cudaSuccess; ++c) {
        const long long n = rcnt[c];
        if (n == 0) continue;
        if (!a.cols_done) { k_global_prep<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(a, c, n); ::tsg::count_launch(); }
        // rows of long A rows: parts over the whole GPU (measured faster than
        // eight warps per row from C widths of 1,024 tile columns on); the
        // cut table gets at most LONG_TAB_MAX entries (rows past it stay
        // with k_numeric_wide)
        const long long pmax = std::max<long long>(((long long)(a.n + TILE - 1) / TILE + LONG_W - 1) / LONG_W, LONG_MINP);
        // ... and at most a quarter of the device's free memory
        size_t free_b = 0, total_b = 0;
        long long tab_cap = LONG_TAB_MAX;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) tab_cap = std::min<long long>(tab_cap, (long long)(free_b / 16));
        const long long tab_bound = std::min<long long>(tab_cap, a.nnzA * (pmax + 1));
        const bool parts = c == ROW_WIDE && a.b_sorted && !packed &&
                           ((long long)a.n + TILE - 1) / TILE >= LONG_MIN_TILES;
        LongScratch L{};
        if (parts) {
            e = long_prepare(pool, a, c, n, tab_bound, n * pmax, L);
            if (e != cudaSuccess) break;
        }
        if (c == ROW_WIDE) { k_numeric_wide<ROW_WARPS><<<(unsigned)n, ROW_WARPS * 32, WIDE_SMEM, s>>>(a, c, n, packed, L.handled); ::tsg::count_launch(); }
        else { k_numeric_wide<1><<<(unsigned)((n + ROW_WARPS - 1) / ROW_WARPS), ROW_WARPS * 32, WIDE_SMEM, s>>>(a, c, n, packed, nullptr); ::tsg::count_launch(); }
        if (parts) {
            { k_long_walk<<<LONG_GRID, ROW_WARPS * 32, LONG_SMEM, s>>>(a, n, L.part_off, L.rdesc, L.pdesc, L.tab, L.next_part); ::tsg::count_launch(); }
            long_release(pool, L);
        }
        e = cudaGetLastError();
    }
    if (split) {
        // joined after a failure too, so that nothing the caller frees on the
        // main stream is still in use by the side stream's kernels
        cudaError_t e2 = cudaEventRecord(join, side);
        if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(pool.stream, join, 0);
        if (e == cudaSuccess) e = e2;
    }
    return e;
}

}  // namespace tsg
