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
// columns, so one DFMA instruction updates distinct outputs (rows with
// duplicate column indices in B take the DUPSAFE variant, which serialises
// equal targets in B's entry order).  Per output the products are applied in
// A's row order, then B's row order: the same order as the CPU reference
// (thmkl_dcsrmultcsr.c:52-91), so with FMA rounding the two agree bit for bit.
// The epilogue streams the segment's values out coalesced and expands the
// masks into column indices.  Dense tile-rows (mean tile nnz >= a threshold)
// use 16x16 dense accumulators instead (position = slot*256 + r*16 + c).
// Tile-rows too large for shared memory accumulate in C's value array.
//
// Roofline: the DFMA issue rate bounds the loop (2 FLOP per intermediate
// product); HBM traffic is A and B once (B rows are re-read from L2) plus
// 12 bytes per C entry written.
#include "tsg_numeric.cuh"

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

// slot of tile column j in the tile-row (-1 if it is not one of its tiles)
__device__ __forceinline__ int slot_of(int j, int jbase, int span, bool use_map, const unsigned short *map,
                                       const int *scol, int S) {
    const unsigned off = (unsigned)(j - jbase);
    if (off >= (unsigned)span) return -1;
    if (use_map) {
        const int s = (int)map[map_swz(off)];          // 0xffff marks a column with no C tile
        return s < S ? s : -1;
    }
    const int s = lower_bound_dev(scol, S, j);
    return (s < S && scol[s] == j) ? s : -1;
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

// One C row: the warp walks A's row in order; for each A entry its lanes
// take the B row's entries (distinct columns, so distinct outputs).
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

// numeric_row for B operands with repeated columns in a row: lanes that
// would update the same output are serialised in B's entry order.
template <bool DENSE>
__device__ __forceinline__ void numeric_row_dupsafe(const NumericArgs &g, const TileRowSmem &t, bool use_map, int r0,
                                                    int r, int lane)
{
    const int R = r0 + r;
    const unsigned *wrow = t.word + r * t.S;
    const int pa0 = (int)g.rpA[R], pa1 = (int)g.rpA[R + 1];
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
        for (int q0 = 0; q0 < na; ++q0) {
            const double a = __shfl_sync(0xffffffffu, av, q0);
            const int b0 = __shfl_sync(0xffffffffu, bs, q0);
            const int b1 = __shfl_sync(0xffffffffu, be, q0);
            for (int eb = b0; eb < b1; eb += 32) {
                const int e = eb + lane;
                const bool ok = e < b1;
                const unsigned act = __ballot_sync(0xffffffffu, ok);
                if (ok) {
                    const int col = g.colB[e];
                    const double b = g.valB[e];
                    const int j = col >> 4, c = col & 15;
                    const int s = slot_of(j, t.jbase, t.span, use_map, t.map, t.scol, t.S);
                    int pos = -1;
                    if (s >= 0) pos = DENSE ? (r * t.S + s) * DPAD + c : acc_swz(rank_in_row(wrow[s], c));
                    const bool okpos = (unsigned)pos < (unsigned)t.nacc;
                    if (!okpos) { set_flag(g.flags, FLAG_INTERNAL); pos = -1 - lane; }
                    const unsigned peers = __match_any_sync(act, pos);
                    const int rank = __popc(peers & lanemask_lt());
                    const int rounds = __reduce_max_sync(act, __popc(peers));
                    for (int q = 0; q < rounds; ++q) {
                        if (q == rank && okpos) t.acc[pos] = fma(a, b, t.acc[pos]);
                        __syncwarp(act);
                    }
                }
            }
        }
    }
}

template <int NT, bool DENSE, bool DUPSAFE>
__global__ void __launch_bounds__(NT, 2048 / NT)
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
        if (DUPSAFE) numeric_row_dupsafe<DENSE>(g, t, use_map, r0, r, lane);
        else if (use_map) numeric_row<DENSE, true>(g, t, r0, r, lane);
        else numeric_row<DENSE, false>(g, t, r0, r, lane);
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
                g.colC[dst] = jb + c;
                if (DENSE) g.valC[dst] = acc[(r * S + s) * DPAD + c];
                ++dst;
                mk &= ~(1u << b);
            }
        }
    }
}

// ---- tile-rows whose rows fit shared memory one at a time -------------------

// numeric_row for the row kernel, with B's entries loaded one step ahead:
// the warp walks the (A entry, 32-entry chunk of its B row) pairs in order
// and issues the next pair's loads before the current pair's shared-memory
// update, so the L2 latency of B overlaps the accumulator work.  Order of the
// updates per output is unchanged (A's row order, then B's row order).
template <bool MAP>
__device__ __forceinline__ void numeric_row_prefetch(const NumericArgs &g, const TileRowSmem &t, int R, int lane)
{
    const unsigned *wrow = t.word;
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
                const int pos = out_pos<false, MAP>(t, wrow, 0, col);
                if (pos < 0) bad = true;
                else acc[pos] = fma(a, b, acc[pos]);
            }
            q = nq; eb = neb; ee = nee; a = na_;
            col = ncol; b = nb; ok = nok;
        }
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

// One single-warp CTA per C row of a tile-row in bin `mybin` (a BIN_ROWS_*
// size class): the row's CSR segment of values in shared memory, addressed
// as in the tile-row kernel (slot map + this row's packed words), then
// streamed out.  Used where the whole tile-row's segment does not fit: each
// CTA holds one row, so the shared memory in use scales with the row, and
// the rows of one tile-row run on different SMs.
template <bool DUPSAFE>
__global__ void __launch_bounds__(32, 32)
k_numeric_rows(NumericArgs g, int mybin)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int i = g.binlist[(long long)mybin * g.blkm + (blockIdx.x >> 4)];
    const int r = blockIdx.x & (TILE - 1);
    const int R = i * TILE + r;
    if (R >= g.m) return;
    const int lane = threadIdx.x;
    const long long c0 = g.crp[i];
    const int S = (int)(g.crp[i + 1] - c0);
    const long long Rb = g.rowptrC[R];
    const int nnz_r = (int)(g.rowptrC[R + 1] - Rb);
    if (nnz_r == 0) return;
    const int jbase = g.ccol[c0];
    const int span = g.ccol[c0 + S - 1] - jbase + 1;
    const bool use_map = span <= MAP_MAX;

    unsigned *word = reinterpret_cast<unsigned *>(s_raw);
    unsigned char *p1 = s_raw + align16((long long)S * 4);
    unsigned short *map = use_map ? reinterpret_cast<unsigned short *>(p1) : nullptr;
    int *scol = use_map ? nullptr : reinterpret_cast<int *>(p1);
    double *acc = reinterpret_cast<double *>(p1 + (use_map ? map_bytes(span) : align16((long long)S * 4)));

    if (use_map) {
        const int span64 = (span + 63) & ~63;
        for (int t = lane; t < span64; t += 32) map[t] = 0xffffu;
        __syncwarp();
    }
    for (int s = lane; s < S; s += 32) {
        const int j = g.ccol[c0 + s];
        if (use_map) map[map_swz((unsigned)(j - jbase))] = (unsigned short)s;
        else scol[s] = j;
    }
    int run = 0;
    for (int sb = 0; sb < S; sb += 32) {
        const int s = sb + lane;
        const unsigned mk = (s < S) ? (unsigned)g.cmask[c0 * TILE + (long long)r * S + s] : 0u;
        const int c = __popc(mk);
        const int incl = warp_incl_scan(c, lane);
        if (s < S) word[s] = ((unsigned)(run + incl - c) << 16) | mk;
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    const int nacc = (nnz_r + 15) & ~15;
    {
        unsigned long long *z = reinterpret_cast<unsigned long long *>(acc);
        for (int t = lane; t < nacc; t += 32) z[t] = 0ull;
    }
    __syncwarp();
    TileRowSmem t{scol, word, map, acc, S, jbase, span, nacc};
    if (DUPSAFE) numeric_row_dupsafe<false>(g, t, use_map, R, 0, lane);
    else if (use_map) numeric_row_prefetch<true>(g, t, R, lane);
    else numeric_row_prefetch<false>(g, t, R, lane);
    __syncwarp();
    for (int p = lane; p < nnz_r; p += 32) g.valC[Rb + p] = acc[acc_swz(p)];
    const int cshift = g.tr_coloff ? g.tr_coloff[i] : 0;
    for (int s = lane; s < S; s += 32) {
        const unsigned w = word[s];
        unsigned mk = w & 0xffffu;
        long long dst = Rb + (w >> 16);
        const int jb = (use_map ? g.ccol[c0 + s] : scol[s]) * TILE - cshift;
        while (mk) {
            const int b = 31 - __clz(mk);   // highest bit = smallest local column
            g.colC[dst] = jb + (TILE - 1 - b);
            ++dst;
            mk &= ~(1u << b);
        }
    }
}

// ---- rows too large for a shared-memory accumulator ----------------------

// per row of a global-bin tile-row: column indices and zeroed values
__global__ void __launch_bounds__(256)
k_global_prep(NumericArgs g)
{
    const int i = g.binlist[(long long)BIN_GLOBAL * g.blkm + blockIdx.x];
    const int cshift = g.tr_coloff ? g.tr_coloff[i] : 0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = i * TILE, rows = min(TILE, g.m - r0);
    const long long c0 = g.crp[i];
    const int S = (int)(g.crp[i + 1] - c0);
    for (int r = warp; r < rows; r += 8) {
        const long long Rb = g.rowptrC[r0 + r];
        long long run = 0;
        for (int sb = 0; sb < S; sb += 32) {
            const int s = sb + lane;
            unsigned mk = (s < S) ? (unsigned)g.cmask[c0 * TILE + (long long)r * S + s] : 0u;
            const int c = __popc(mk);
            const int incl = warp_incl_scan(c, lane);
            long long dst = Rb + run + incl - c;
            const int jb = (s < S) ? g.ccol[c0 + s] * TILE - cshift : 0;
            while (mk) {
                const int b = 31 - __clz(mk);
                g.colC[dst] = jb + (TILE - 1 - b);
                g.valC[dst] = 0.0;
                ++dst;
                mk &= ~(1u << b);
            }
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

constexpr int WIDE_W = 4096;   // tile columns per window of the wide-row kernel

// One single-warp CTA per C row of a global-bin tile-row; the values
// accumulate in place in C (zeroed by k_global_prep).  The row's tile
// columns are walked in windows of WIDE_W tile columns: for a window the
// CTA tabulates, by tile column, the row's mask and the offset of its
// segment in the row (shared memory, 24 KB), then applies A's row in order,
// each A entry's B row restricted to the window's columns (found by a warp
// search, then scanned until it leaves the window).  Per output the
// products still come in A's row order.
template <bool DUPSAFE>
__global__ void __launch_bounds__(32, 16)
k_numeric_wide(NumericArgs g)
{
    __shared__ unsigned s_off[WIDE_W];
    __shared__ unsigned short s_msk[WIDE_W];
    const int i = g.binlist[(long long)BIN_GLOBAL * g.blkm + (blockIdx.x >> 4)];
    const int r = blockIdx.x & (TILE - 1);
    const int R = i * TILE + r;
    if (R >= g.m) return;
    const int lane = threadIdx.x;
    const long long c0 = g.crp[i];
    const int S = (int)(g.crp[i + 1] - c0);
    const long long Rb = g.rowptrC[R];
    if (g.rowptrC[R + 1] == Rb) return;
    for (int t = lane; t < WIDE_W; t += 32) s_msk[t] = 0;
    __syncwarp();
    const uint16_t *mrow = g.cmask + c0 * TILE + (long long)r * S;
    const int *tcol = g.ccol + c0;
    const int pa0 = (int)g.rpA[R], pa1 = (int)g.rpA[R + 1];
    unsigned run = 0;     // entries of the row before tile slot s
    bool bad = false;
    int s = 0;
    while (s < S) {
        // the window starts at the row's next tile with entries
        {
            int f = -1;
            while (s < S) {
                const int ss = s + lane;
                const unsigned nz = __ballot_sync(0xffffffffu, ss < S && mrow[ss] != 0);
                if (nz) { f = __ffs(nz) - 1; break; }
                s += 32;
            }
            if (f < 0) break;
            s += f;
        }
        const int j0 = tcol[s];
        int se = s;
        for (;;) {
            const int ss = se + lane;
            const bool in = ss < S && tcol[ss] < j0 + WIDE_W;
            const unsigned mk = in ? (unsigned)mrow[ss] : 0u;
            const int c = __popc(mk);
            const int incl = warp_incl_scan(c, lane);
            if (mk) { const int t = tcol[ss] - j0; s_off[t] = run + incl - c; s_msk[t] = (unsigned short)mk; }
            run += __shfl_sync(0xffffffffu, incl, 31);
            const int cnt = __popc(__ballot_sync(0xffffffffu, in));   // in-window slots are a prefix
            se += cnt;
            if (cnt < 32) break;
        }
        __syncwarp();
        const int lo = j0 * TILE, hi = (j0 + WIDE_W) * TILE;
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
                const int b1 = __shfl_sync(0xffffffffu, be, q);
                const int b0 = warp_lower_bound(g.colB, __shfl_sync(0xffffffffu, bs, q), b1, lo, lane);
                for (int eb = b0; eb < b1; eb += 32) {
                    const int e = eb + lane;
                    const int col = e < b1 ? g.colB[e] : INT_MAX;
                    const bool ok = col < hi;
                    long long pos = -1;
                    double b = 0.0;
                    if (ok) {
                        b = g.valB[e];
                        const int t = (col >> 4) - j0, cc = col & 15;
                        const unsigned mk = s_msk[t];
                        if ((mk >> (TILE - 1 - cc)) & 1u) pos = Rb + s_off[t] + __popc(mk >> (TILE - cc));
                        else bad = true;
                    }
                    if (!DUPSAFE) {
                        if (pos >= 0) g.valC[pos] = fma(a, b, g.valC[pos]);
                    } else {
                        const unsigned act = __activemask();
                        const unsigned peers = __match_any_sync(act, pos >= 0 ? pos : -1 - lane);
                        const int rank = __popc(peers & lanemask_lt());
                        const int rounds = __reduce_max_sync(act, __popc(peers));
                        for (int q2 = 0; q2 < rounds; ++q2) {
                            if (q2 == rank && pos >= 0) g.valC[pos] = fma(a, b, g.valC[pos]);
                            __syncwarp(act);
                        }
                    }
                    if (__ballot_sync(0xffffffffu, !ok)) break;   // the rest of B's row is past the window
                }
                __syncwarp();
            }
        }
        for (int ss = s + lane; ss < se; ss += 32) s_msk[tcol[ss] - j0] = 0;
        __syncwarp();
        s = se;
    }
    if (bad) set_flag(g.flags, FLAG_INTERNAL);
}

template <int NT, bool DENSE, bool DUPSAFE>
cudaError_t set_smem_attr() {
    cudaError_t e = cudaFuncSetAttribute(k_numeric_smem<NT, DENSE, DUPSAFE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LARGE);
    // the whole unified L1 as shared memory, so occupancy is set by the
    // tile-row's actual request, not by a smaller carveout
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_numeric_smem<NT, DENSE, DUPSAFE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    return e;
}

template <int NT>
cudaError_t launch_smem(const NumericArgs &a, int bin, long long nrows, long long smem, bool dense, bool dup,
                        cudaStream_t s) {
    const unsigned grid = (unsigned)nrows;
    if (dense) {
        if (dup) { k_numeric_smem<NT, true, true><<<grid, NT, smem, s>>>(a, bin); ::tsg::count_launch(); }
        else { k_numeric_smem<NT, true, false><<<grid, NT, smem, s>>>(a, bin); ::tsg::count_launch(); }
    } else {
        if (dup) { k_numeric_smem<NT, false, true><<<grid, NT, smem, s>>>(a, bin); ::tsg::count_launch(); }
        else { k_numeric_smem<NT, false, false><<<grid, NT, smem, s>>>(a, bin); ::tsg::count_launch(); }
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t numeric_init_attributes()
{
    cudaError_t e = cudaSuccess;
#define TSG_SET(NT)                                                    \
    if (e == cudaSuccess) e = set_smem_attr<NT, false, false>();       \
    if (e == cudaSuccess) e = set_smem_attr<NT, false, true>();        \
    if (e == cudaSuccess) e = set_smem_attr<NT, true, false>();        \
    if (e == cudaSuccess) e = set_smem_attr<NT, true, true>();
    TSG_SET(128)
    TSG_SET(256)
    TSG_SET(512)
#undef TSG_SET
    for (int d = 0; d < 2 && e == cudaSuccess; ++d) {
        const void *f = d ? (const void *)k_numeric_rows<true> : (const void *)k_numeric_rows<false>;
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LARGE);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    }
    return e;
}

cudaError_t numeric_run(Pool &pool, const NumericArgs &a, const long long *counts, const long long *req,
                        bool dupsafe, int threads)
{
    cudaStream_t s = pool.stream;
    cudaError_t e = cudaSuccess;
    for (int b = BIN_SPARSE_S; b <= BIN_DENSE_L && e == cudaSuccess; ++b) {
        if (counts[b] == 0) continue;
        const bool dense = (b == BIN_DENSE_S || b == BIN_DENSE_L);
        const long long smem = req[b];
        if (threads == 128) e = launch_smem<128>(a, b, counts[b], smem, dense, dupsafe, s);
        else if (threads == 512) e = launch_smem<512>(a, b, counts[b], smem, dense, dupsafe, s);
        else e = launch_smem<256>(a, b, counts[b], smem, dense, dupsafe, s);
    }
    for (int b = BIN_ROWS_S; b <= BIN_ROWS_L && e == cudaSuccess; ++b) {
        if (counts[b] == 0) continue;
        const unsigned g = (unsigned)(counts[b] * TILE);
        const size_t smem = (size_t)req[b];
        if (dupsafe) { k_numeric_rows<true><<<g, 32, smem, s>>>(a, b); ::tsg::count_launch(); }
        else { k_numeric_rows<false><<<g, 32, smem, s>>>(a, b); ::tsg::count_launch(); }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && counts[BIN_GLOBAL] > 0) {
        { k_global_prep<<<(unsigned)counts[BIN_GLOBAL], 256, 0, s>>>(a); ::tsg::count_launch(); }
        const unsigned g = (unsigned)(counts[BIN_GLOBAL] * TILE);
        if (dupsafe) { k_numeric_wide<true><<<g, 32, 0, s>>>(a); ::tsg::count_launch(); }
        else { k_numeric_wide<false><<<g, 32, 0, s>>>(a); ::tsg::count_launch(); }
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace tsg
