// tsg_symbolic.cu -- step 2: per-tile row masks of C, C's row counts, and
// the binning of C's tile-rows for the numeric step.
//
// Reference: stir_spgemm_step3_cuda_kernel_2level (main_spgemm-col.cu:997-1325)
// finds, for every C tile, the matched (A tile, B tile) pairs by binary
// search and ORs maskB[colA] into maskC[rowA] with shared-memory atomics;
// __popc gives per-row counts.  Here one CTA owns a C tile-row: it walks the
// row's A tiles (i,k) and, for each, B's tile-row k, so every matched pair is
// visited exactly once with no search for partners.  For a pair, row r of
// the C tile gets OR over the set bits c of maskA[r] of maskB[c] (a 16x16
// boolean tile product on row masks).  The C tile-row's masks live in
// shared memory (global-memory atomics for tile-rows with very many tiles).
//
// Outputs: cmask (16 uint16 per C tile) and rowcnt[m] (nnz of each C row; a
// scan turns it into C's row pointer).  The numeric bins of C's tile-rows
// are chosen afterwards from the finished structure (bin_tilerows).
// Roofline: integer work with L1/L2-resident reads of the B masks; the
// compulsory HBM traffic is writing 32 bytes of mask per C tile.
#include "tsg_internal.cuh"
#include "tsg_numeric.cuh"

#include <climits>

namespace tsg {

namespace {

__device__ __forceinline__ int lower_bound_i(const int *a, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

constexpr int ENTRY_WALK_MAX = 3;   // mean A entries per A tile up to which step 2 walks A's rows by entry

// Tile-row i's A tiles hold ENTRY_WALK_MAX entries or fewer on average: step
// 2 then walks A's rows entry by entry (k_step2_entries) instead of tile by
// tile, as the per-tile transpose would cost more than the entries.
__device__ __forceinline__ bool entry_walk(const long long *erpA, const int *arp, int i, int rows) {
    const long long nea = erpA[(long long)i * TILE + rows] - erpA[(long long)i * TILE];
    return nea <= (long long)ENTRY_WALK_MAX * (arp[i + 1] - arp[i]);
}

// OR `bits` into 16-bit mask idx of a uint16 array in shared memory (word atomics)
__device__ __forceinline__ void smask_or(unsigned short *m, int idx, unsigned bits) {
    atomicOr(reinterpret_cast<unsigned *>(m) + (idx >> 1), bits << ((idx & 1) * 16));
}

// slot of tile column j in C's tile-row: direct map over the row's window
// when it is narrow, binary search otherwise; -1 if j is not one of its
// tiles.  The map holds, for every column of the window, its tile's slot or
// 0xffff, so a mapped slot needs no check against the tile columns.
__device__ __forceinline__ int c_slot(int j, int jbase, int span, const unsigned short *map, const int *scol, int S) {
    const unsigned off = (unsigned)(j - jbase);
    if (off >= (unsigned)span) return -1;
    if (map) {
        const int s = (int)map[off];
        return s < S ? s : -1;
    }
    const int s = lower_bound_i(scol, S, j);
    return (s < S && scol[s] == j) ? s : -1;
}

// Masks accumulate in shared memory (tile-rows with at most `smax` tiles).
// Work split: a warp takes one A tile (i,k) at a time and its lanes the B
// tiles of B's tile-row k.  The A tile is transposed once (16 ballots give,
// for every local column c, the set of rows that use it); then for each c,
// uniformly across the warp, every lane ORs its B tile's row c into the
// rows of that set -- one shared atomicOr per A entry and B tile, no search,
// no per-element branching on the B side.
template <int NT>
__global__ void __launch_bounds__(NT)
k_step2(int blkm, int m, const int *__restrict__ arp, const int *__restrict__ acol,
        const uint16_t *__restrict__ amask, const int *__restrict__ brp, const int *__restrict__ bcol,
        const uint16_t *__restrict__ bmask, const long long *__restrict__ crp, const int *__restrict__ ccol,
        uint16_t *cmask, int *rowcnt, int smin, int smax, int map_cap, int *flags, const int *__restrict__ rows_list,
        const long long *__restrict__ erpB, const int *__restrict__ ecolB, const long long *__restrict__ erpA)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ long long s_rowtot[TILE];
    const int i = rows_list[blockIdx.x];
    if (i >= blkm) return;
    const long long c0 = crp[i];
    const int S = (int)(crp[i + 1] - c0);
    if (S <= smin || S > smax) return;
    const int rows = min(TILE, m - i * TILE);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int jbase = S > 0 ? ccol[c0] : 0;
    const int span = S > 0 ? ccol[c0 + S - 1] - jbase + 1 : 0;
    if (fused_handles(span, S)) return;     // done by the fused warp kernel
    if (entry_walk(erpA, arp, i, rows)) return;   // sparse A tiles: k_step2_entries
    unsigned short *smask = reinterpret_cast<unsigned short *>(s_raw);          // [16][S]
    int *wcol = reinterpret_cast<int *>(s_raw + align16((long long)S * TILE * 2));
    unsigned short *map = nullptr;
    if (span <= map_cap)
        map = reinterpret_cast<unsigned short *>(s_raw + align16((long long)S * TILE * 2) + align16((long long)S * 4));
    const int *scol = wcol;
    {
        unsigned *z = reinterpret_cast<unsigned *>(smask);
        for (int t = tid; t < (S * TILE + 1) / 2; t += NT) z[t] = 0u;
        for (int t = tid; t < S; t += NT) wcol[t] = ccol[c0 + t];
        if (map) {
            for (int t = tid; t < span; t += NT) map[t] = 0xffffu;
            __syncthreads();
            for (int t = tid; t < S; t += NT) map[ccol[c0 + t] - jbase] = (unsigned short)t;
        }
    }
    if (tid < TILE) s_rowtot[tid] = 0;
    __syncthreads();

    const int a0 = arp[i], a1 = arp[i + 1], na = a1 - a0;
    bool bad = false;
    for (int a = a0 + warp; a < a1; a += (NT / 32)) {
        const int kt = acol[a];
        const int q0 = brp[kt], nq = brp[kt + 1] - q0;
        // transpose the A tile: colrows[c] = rows r whose mask has local column c
        const unsigned ma = (lane < TILE) ? (unsigned)amask[(long long)a0 * TILE + (long long)lane * na + (a - a0)] : 0u;
        unsigned colrows[TILE];
#pragma unroll
        for (int c = 0; c < TILE; ++c) colrows[c] = __ballot_sync(0xffffffffu, (ma >> (TILE - 1 - c)) & 1u) & 0xffffu;
        // A tiles with few entries: visit the B rows of the A tile's local
        // columns element by element (an entry (kt*16+c, col) sets bit
        // 15-(col&15) of C's tile col>>4 in the rows that use c) instead of
        // all nq B tiles; the masks are the same either way
        const unsigned acols = __brev(__reduce_or_sync(0xffffffffu, ma)) >> 16;   // bit c: local column c used
        int eb0 = 0, eb1 = 0;   // operands hold < 2^31 entries
        if (lane < TILE && ((acols >> lane) & 1u)) { eb0 = (int)erpB[kt * TILE + lane]; eb1 = (int)erpB[kt * TILE + lane + 1]; }
        const int elem_iters = warp_sum_int((eb1 - eb0 + 31) >> 5);
        if (elem_iters <= 3 * ((nq + 31) >> 5)) {
            for (unsigned cs = acols; cs; cs &= cs - 1) {
                const int c = __ffs(cs) - 1;
                const int e0 = __shfl_sync(0xffffffffu, eb0, c), e1 = __shfl_sync(0xffffffffu, eb1, c);
                const unsigned rowsc = __ballot_sync(0xffffffffu, (ma >> (TILE - 1 - c)) & 1u) & 0xffffu;
                for (int e = e0 + lane; e < e1; e += 32) {
                    const int col = ecolB[e];
                    const int sl = c_slot(col >> 4, jbase, span, map, scol, S);
                    if (sl < 0) { bad = true; continue; }
                    const unsigned bit = 0x8000u >> (col & 15);
                    for (unsigned rs = rowsc; rs; rs &= rs - 1) {
                        const int r = __ffs(rs) - 1;
                        smask_or(smask, r * S + sl, bit);
                    }
                }
            }
            continue;
        }
        for (int qb = 0; qb < nq; qb += 32) {
            const int q = qb + lane;
            const bool ok = q < nq;
            int sl = -1;
            if (ok) {
                sl = c_slot(bcol[q0 + q], jbase, span, map, scol, S);
                if (sl < 0) bad = true;
            }
            const uint16_t *bq = bmask + (long long)q0 * TILE + q;   // row c of B tile q at bq[c*nq]
            unsigned brow[TILE];
#pragma unroll
            for (int c = 0; c < TILE; ++c) brow[c] = (colrows[c] != 0u && sl >= 0) ? (unsigned)bq[c * nq] : 0u;
#pragma unroll
            for (int c = 0; c < TILE; ++c) {
                unsigned rowsc = colrows[c];
                const unsigned b = brow[c];
                while (rowsc) {
                    const int r = __ffs(rowsc) - 1;
                    rowsc &= rowsc - 1;
                    if (!b) continue;
                    smask_or(smask, r * S + sl, b);
                }
            }
        }
    }
    if (bad) set_flag(flags, FLAG_INTERNAL);
    __syncthreads();

    // both smask and cmask are row-major ([r][s]) within the tile-row
    for (int t = tid; t < S * TILE; t += NT) cmask[c0 * TILE + t] = smask[t];
    for (int r = warp; r < TILE; r += (NT / 32)) {
        int c = 0;
        for (int s = lane; s < S; s += 32) {
            c += __popc((unsigned)smask[r * S + s]);
        }
        c = warp_sum_int(c);
        if (lane == 0) {
            if (r < rows) rowcnt[i * TILE + r] = c;
            s_rowtot[r] = c;
        }
    }
}

// Tile-rows with more than `smin` C tiles: the tile slots are taken in
// windows of `smax`; per window the row masks accumulate in shared memory
// (OR does not depend on order) and are then written out.  Every window
// walks the tile-row's A tiles again, with each B tile-row (tile path) or
// B row (element path) restricted to the window's tile columns by a warp
// search.
template <int NT>
__global__ void __launch_bounds__(NT)
k_step2_win(int blkm, int m, const int *__restrict__ arp, const int *__restrict__ acol,
            const uint16_t *__restrict__ amask, const int *__restrict__ brp, const int *__restrict__ bcol,
            const uint16_t *__restrict__ bmask, const long long *__restrict__ crp, const int *__restrict__ ccol,
            uint16_t *cmask, int *rowcnt, int smin, int smax, int *flags, const int *__restrict__ rows_list,
            const long long *__restrict__ erpB, const int *__restrict__ ecolB, const long long *__restrict__ erpA)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ long long s_rowtot[TILE];
    const int i = rows_list[blockIdx.x];
    if (i >= blkm) return;
    const long long c0 = crp[i];
    const int S = (int)(crp[i + 1] - c0);
    if (S <= smin) return;
    const int rows = min(TILE, m - i * TILE);
    if (entry_walk(erpA, arp, i, rows)) return;   // sparse A tiles: k_step2_entries
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned short *smask = reinterpret_cast<unsigned short *>(s_raw);                       // [16][smax]
    int *wcol = reinterpret_cast<int *>(s_raw + align16((long long)smax * TILE * 2));        // [smax]
    unsigned short *map = reinterpret_cast<unsigned short *>(s_raw + align16((long long)smax * TILE * 2) +
                                                              align16((long long)smax * 4));  // [MAP_MAX]
    if (tid < TILE) s_rowtot[tid] = 0;
    const int a0 = arp[i], a1 = arp[i + 1], na = a1 - a0;
    bool bad = false;
    for (int s0 = 0; s0 < S; s0 += smax) {
        const int SW = min(smax, S - s0);
        {
            unsigned *z = reinterpret_cast<unsigned *>(smask);
            for (int t = tid; t < (SW * TILE + 1) / 2; t += NT) z[t] = 0u;
        }
        for (int t = tid; t < SW; t += NT) wcol[t] = ccol[c0 + s0 + t];
        __syncthreads();
        const int jlo = wcol[0], jhi = wcol[SW - 1];
        const bool use_map = jhi - jlo + 1 <= (int)MAP_MAX;
        if (use_map) {
            for (int t = tid; t < jhi - jlo + 1; t += NT) map[t] = 0xffffu;
            __syncthreads();
            for (int t = tid; t < SW; t += NT) map[wcol[t] - jlo] = (unsigned short)t;
        }
        __syncthreads();
        const int wspan = jhi - jlo + 1;
        for (int a = a0 + warp; a < a1; a += (NT / 32)) {
            const int kt = acol[a];
            const int q0 = brp[kt], nq = brp[kt + 1] - q0;
            const unsigned ma = (lane < TILE) ? (unsigned)amask[(long long)a0 * TILE + (long long)lane * na + (a - a0)] : 0u;
            const unsigned acols = __brev(__reduce_or_sync(0xffffffffu, ma)) >> 16;
            int eb0 = 0, eb1 = 0;
            if (lane < TILE && ((acols >> lane) & 1u)) { eb0 = (int)erpB[kt * TILE + lane]; eb1 = (int)erpB[kt * TILE + lane + 1]; }
            const int elem_iters = warp_sum_int((eb1 - eb0 + 31) >> 5);
            if (elem_iters <= 3 * ((nq + 31) >> 5)) {
                for (unsigned cs = acols; cs; cs &= cs - 1) {
                    const int c = __ffs(cs) - 1;
                    const int e1 = __shfl_sync(0xffffffffu, eb1, c);
                    const int e0 = warp_lower_bound(ecolB, __shfl_sync(0xffffffffu, eb0, c), e1, jlo * TILE, lane);
                    const unsigned rowsc = __ballot_sync(0xffffffffu, (ma >> (TILE - 1 - c)) & 1u) & 0xffffu;
                    for (int eb = e0; eb < e1; eb += 32) {
                        const int e = eb + lane;
                        const int col = e < e1 ? ecolB[e] : INT_MAX;
                        const bool ok = (col >> 4) <= jhi;
                        if (ok) {
                            const int sl = c_slot(col >> 4, jlo, wspan, use_map ? map : nullptr, wcol, SW);
                            if (sl < 0) bad = true;
                            else {
                                const unsigned bit = 0x8000u >> (col & 15);
                                for (unsigned rs = rowsc; rs; rs &= rs - 1) smask_or(smask, (__ffs(rs) - 1) * SW + sl, bit);
                            }
                        }
                        if (__ballot_sync(0xffffffffu, !ok)) break;
                    }
                }
                continue;
            }
            unsigned colrows[TILE];
#pragma unroll
            for (int c = 0; c < TILE; ++c) colrows[c] = __ballot_sync(0xffffffffu, (ma >> (TILE - 1 - c)) & 1u) & 0xffffu;
            const int qs = warp_lower_bound(bcol, q0, q0 + nq, jlo, lane) - q0;
            for (int qb = qs; qb < nq; qb += 32) {
                const int q = qb + lane;
                const int j = q < nq ? bcol[q0 + q] : INT_MAX;
                const bool ok = j <= jhi;
                int sl = -1;
                if (ok) {
                    sl = c_slot(j, jlo, wspan, use_map ? map : nullptr, wcol, SW);
                    if (sl < 0) bad = true;
                }
                const uint16_t *bq = bmask + (long long)q0 * TILE + q;   // row c of B tile q at bq[c*nq]
                unsigned brow[TILE];
#pragma unroll
                for (int c = 0; c < TILE; ++c) brow[c] = (colrows[c] != 0u && sl >= 0) ? (unsigned)bq[c * nq] : 0u;
#pragma unroll
                for (int c = 0; c < TILE; ++c) {
                    unsigned rowsc = colrows[c];
                    const unsigned b = brow[c];
                    while (rowsc) {
                        const int r = __ffs(rowsc) - 1;
                        rowsc &= rowsc - 1;
                        if (b) smask_or(smask, r * SW + sl, b);
                    }
                }
                if (__ballot_sync(0xffffffffu, !ok)) break;
            }
        }
        __syncthreads();
        for (int t = tid; t < SW * TILE; t += NT) {
            const int r = t / SW, sl = t - r * SW;
            cmask[c0 * TILE + (long long)r * S + s0 + sl] = smask[t];
        }
        for (int r = warp; r < TILE; r += (NT / 32)) {
            int c = 0;
            for (int sl = lane; sl < SW; sl += 32) c += __popc((unsigned)smask[r * SW + sl]);
            c = warp_sum_int(c);
            if (lane == 0) s_rowtot[r] += c;
        }
        __syncthreads();
    }
    if (bad) set_flag(flags, FLAG_INTERNAL);
    __syncthreads();
    if (tid < rows) rowcnt[i * TILE + tid] = (int)s_rowtot[tid];
}

// ---- tile-rows of sparse A tiles: A's entries one by one -------------------
//
// An entry (r, k) of A's tile-row sets, for every entry (k, col) of B's row
// k, bit 15-(col&15) of row r's mask in C's tile col>>4.  The tile-row's
// entries are taken in batches of up to EB; work is spread over the CTA's
// warps in units of 32 consecutive B entries of one A entry (a block scan
// over the entries' unit counts gives each warp an equal share), so a few
// long B rows do not hold the other warps at the CTA's barrier.  Tile-rows
// with more tiles than one window of shared masks are taken in windows;
// with sorted B rows each entry keeps a cursor into its B row from window
// to window (when the batch holds the whole tile-row) and a galloping
// search finds where its segment in the window ends.  Unsorted B rows are
// tested entry by entry in every window.
constexpr int EB = 1024;   // A entries per batch

__device__ __forceinline__ int block_excl_scan(int *v, int n, int *s_wsum, int tid, int nt)
{
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    __syncthreads();   // v was written under another thread mapping
    const int per = (n + nt - 1) / nt;
    const int b = min(n, tid * per), e = min(n, b + per);
    int loc = 0;
    for (int j = b; j < e; ++j) loc += v[j];
    const int incl = warp_incl_scan(loc, lane);
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    int pre = 0, total = 0;
    for (int w = 0; w < nw; ++w) {
        const int x = s_wsum[w];
        if (w < warp) pre += x;
        total += x;
    }
    int run = pre + incl - loc;
    for (int j = b; j < e; ++j) { const int x = v[j]; v[j] = run; run += x; }
    if (tid == 0) v[n] = total;
    __syncthreads();
    return total;
}

// shared memory of k_step2_entries: masks, tile columns, map, entry state
__host__ __device__ inline size_t step2e_smem(int slots, int map_cap) {
    return (size_t)(align16((long long)slots * TILE * 2) + align16((long long)slots * 4) +
                    align16((long long)map_cap * 2) + 4ll * (4 * EB + 1) + EB);
}

template <int NT>
__global__ void __launch_bounds__(NT)
k_step2_entries(int blkm, int m, const int *__restrict__ arp, const long long *__restrict__ crp,
                const int *__restrict__ ccol, uint16_t *cmask, int *rowcnt, int smin, int smax, int wslots, int map_cap,
                int *flags,
                const int *__restrict__ rows_list, const long long *__restrict__ erpB, const int *__restrict__ ecolB,
                const long long *__restrict__ erpA, const int *__restrict__ ecolA, int b_sorted)
{
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ long long s_rowtot[TILE];
    __shared__ int s_wsum[NW];
    __shared__ int s_rs[TILE + 1];
    const int i = rows_list[blockIdx.x];
    if (i >= blkm) return;
    const long long c0 = crp[i];
    const int S = (int)(crp[i + 1] - c0);
    if (S <= smin || S > smax) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int span = ccol[c0 + S - 1] - ccol[c0] + 1;
    if (fused_handles(span, S)) return;     // done by the fused warp kernel
    const int rows = min(TILE, m - i * TILE);
    if (!entry_walk(erpA, arp, i, rows)) return;   // dense A tiles: the tile kernels
    const int SW = min(S, wslots);
    unsigned short *smask = reinterpret_cast<unsigned short *>(s_raw);                      // [16][SW]
    int *wcol = reinterpret_cast<int *>(s_raw + align16((long long)SW * TILE * 2));         // [SW]
    unsigned short *map = reinterpret_cast<unsigned short *>(reinterpret_cast<unsigned char *>(wcol) +
                                                             align16((long long)SW * 4));   // [map_cap]
    int *e_cur = reinterpret_cast<int *>(reinterpret_cast<unsigned char *>(map) + align16((long long)map_cap * 2));
    int *e_end = e_cur + EB, *e_wend = e_end + EB, *e_pre = e_wend + EB;                     // e_pre: EB + 1
    unsigned char *e_row = reinterpret_cast<unsigned char *>(e_pre + EB + 1);
    if (tid <= TILE) s_rs[tid] = (int)erpA[(long long)i * TILE + min(tid, rows)];
    if (tid < TILE) s_rowtot[tid] = 0;
    __syncthreads();
    const int p0 = s_rs[0], p1 = s_rs[TILE];
    const bool keep = p1 - p0 <= EB && b_sorted;   // cursors carried from window to window
    bool bad = false;
    for (int s0 = 0; s0 < S; s0 += SW) {
        const int nsl = min(SW, S - s0);
        {
            unsigned *z = reinterpret_cast<unsigned *>(smask);
            for (int t = tid; t < (nsl * TILE + 1) / 2; t += NT) z[t] = 0u;
            for (int t = tid; t < nsl; t += NT) wcol[t] = ccol[c0 + s0 + t];
        }
        __syncthreads();
        const int jlo = wcol[0], jhi = wcol[nsl - 1];
        const int wspan = jhi - jlo + 1;
        const bool use_map = wspan <= map_cap;
        if (use_map) {
            for (int t = tid; t < wspan; t += NT) map[t] = 0xffffu;
            __syncthreads();
            for (int t = tid; t < nsl; t += NT) map[wcol[t] - jlo] = (unsigned short)t;
        }
        const int cfirst = jlo * TILE, climit = (jhi + 1) * TILE;
        const bool last = s0 + SW >= S;
        for (int pb0 = p0; pb0 < p1; pb0 += EB) {
            const int nb = min(EB, p1 - pb0);
            for (int t = tid; t < nb; t += NT) {
                const int p = pb0 + t;
                int cur, end;
                if (keep && s0 > 0) {
                    cur = e_wend[t];
                    end = e_end[t];
                } else {
                    const int k = ecolA[p];
                    cur = (int)erpB[k];
                    end = (int)erpB[k + 1];
                    if (s0 > 0 && b_sorted) cur = gallop_lower_bound(ecolB, cur, end, cfirst);
                    int r = 0;
                    while (s_rs[r + 1] <= p) ++r;
                    e_row[t] = (unsigned char)r;
                }
                const int wend = (b_sorted && !last) ? gallop_lower_bound(ecolB, cur, end, climit) : end;
                e_cur[t] = cur;
                e_end[t] = end;
                e_wend[t] = wend;
                e_pre[t] = (wend - cur + 31) >> 5;
            }
            // (the scan's first barrier also orders the map and state writes above)
            const int U = block_excl_scan(e_pre, nb, s_wsum, tid, NT);
            const int u0 = (int)((long long)U * warp / NW), u1 = (int)((long long)U * (warp + 1) / NW);
            if (u0 < u1) {
                int lo = 0, hi = nb - 1;   // last entry whose units start at or before u0
                while (lo < hi) { const int md = (lo + hi + 1) >> 1; if (e_pre[md] <= u0) lo = md; else hi = md - 1; }
                // unit u's B entry for this lane (its A entry tt; -1: past
                // the segment's end); the next unit's column is loaded before
                // the current unit's update (OR does not depend on order)
                auto unit_entry = [&](int u, int &tt) -> int {
                    while (e_pre[tt + 1] <= u) ++tt;
                    const int e = e_cur[tt] + ((u - e_pre[tt]) << 5) + lane;
                    return e < e_wend[tt] ? e : -1;
                };
                int t = lo;
                int e = unit_entry(u0, t);
                int col = e >= 0 ? ecolB[e] : 0;
                for (int u = u0; u < u1; ++u) {
                    int tn = t, en = -1, coln = 0;
                    if (u + 1 < u1) {
                        en = unit_entry(u + 1, tn);
                        if (en >= 0) coln = ecolB[en];
                    }
                    if (e >= 0) {
                        if (col >= cfirst && col < climit) {
                            const int sl = c_slot(col >> 4, jlo, wspan, use_map ? map : nullptr, wcol, nsl);
                            if (sl < 0) bad = true;
                            else smask_or(smask, (int)e_row[t] * nsl + sl, 0x8000u >> (col & 15));
                        } else if (b_sorted) {
                            bad = true;   // a sorted segment lies inside its window
                        }
                    }
                    t = tn; e = en; col = coln;
                }
            }
            __syncthreads();
        }
        // the window's masks out (row-major within the tile-row) and row counts
        for (int r = warp; r < TILE; r += NW) {
            int c = 0;
            for (int sl = lane; sl < nsl; sl += 32) {
                const unsigned short v = smask[r * nsl + sl];
                cmask[c0 * TILE + (long long)r * S + s0 + sl] = v;
                c += __popc((unsigned)v);
            }
            c = warp_sum_int(c);
            if (lane == 0) s_rowtot[r] += c;
        }
        __syncthreads();
    }
    if (bad) set_flag(flags, FLAG_INTERNAL);
    __syncthreads();
    if (tid < rows) rowcnt[i * TILE + tid] = (int)s_rowtot[tid];
}

}  // namespace

constexpr int S2_SMAX = 4096;   // tiles per tile-row (or window) handled with shared-memory masks

constexpr int S2_SMALL = 1024;  // tile-rows of up to this many tiles: 256-thread CTAs with less shared memory
constexpr int S2E_WIN = 2048;   // tiles per window of k_step2_entries (two CTAs per SM)
constexpr int S2W_WIN = 4096;   // tiles per window of k_step2_win

namespace {
size_t step2_smem(int slots, int map_cap) {
    return (size_t)(align16((long long)slots * TILE * 2) + align16((long long)slots * 4) + align16((long long)map_cap * 2));
}
template <class K>
cudaError_t step2_attr(K kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)step2_smem(S2_SMAX, MAP_MAX));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    return e;
}
}  // namespace

cudaError_t symbolic_init_attributes()
{
    cudaError_t e = step2_attr(k_step2<256>);
    if (e == cudaSuccess) e = step2_attr(k_step2<512>);
    if (e == cudaSuccess) e = step2_attr(k_step2_win<512>);
    for (const void *f : {(const void *)k_step2_entries<256>, (const void *)k_step2_entries<512>}) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)step2e_smem(S2_SMAX, MAP_MAX));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    }
    return e;
}

// The deferred tile-rows (too many tiles or too wide a window for the fused
// warp kernel): up to S2_SMALL tiles in 256-thread CTAs, up to S2_SMAX in
// 512-thread CTAs (one per SM at that shared memory, so more warps per
// CTA), beyond that in windows.  Each launch walks the whole defer list and
// skips the tile-rows of the other classes.
cudaError_t step2_masks(Pool &pool, const TileCSR &A, const TileCSR &B, int m, int blkm, const long long *crp,
                        const int *ccol, uint16_t *cmask, int *rowcnt, int max_tiles_per_row, int max_span,
                        int *flags, const int *defer_list, int ndefer, const long long *erpB,
                        const int *ecolB, const long long *erpA, const int *ecolA, bool b_sorted,
                        cudaStream_t side, cudaEvent_t fork, cudaEvent_t join)
{
    cudaStream_t s = pool.stream;
    if (blkm <= 0 || ndefer <= 0) return cudaSuccess;
    const int map_cap = max_span < (int)MAP_MAX ? max_span : (int)MAP_MAX;
    // the windowed kernel takes few, long tile-rows: it runs on the side
    // stream beside the other classes (disjoint tile-rows) and is joined at
    // the end, so its CTAs do not leave the rest of the GPU idle
    const bool win = max_tiles_per_row > S2_SMAX;
    if (win) {
        cudaError_t e = cudaEventRecord(fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork, 0);
        if (e == cudaSuccess) {
            k_step2_win<512><<<ndefer, 512, step2_smem(S2W_WIN, MAP_MAX), side>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol,
                                                      B.mask, crp, ccol, cmask, rowcnt, S2_SMAX, S2W_WIN, flags, defer_list, erpB, ecolB, erpA);
            ::tsg::count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(join, side);
        if (e != cudaSuccess) return e;
    }
    {
        const int slots = max_tiles_per_row < S2_SMALL ? max_tiles_per_row : S2_SMALL;
        { k_step2<256><<<ndefer, 256, step2_smem(slots, map_cap), s>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol, B.mask, crp, ccol,
                                                   cmask, rowcnt, 0, S2_SMALL, map_cap, flags, defer_list,
                                                   erpB, ecolB, erpA); ::tsg::count_launch(); }
        { k_step2_entries<256><<<ndefer, 256, step2e_smem(slots, map_cap), s>>>(blkm, m, A.trp, crp, ccol, cmask, rowcnt, 0, S2_SMALL,
                                                   S2_SMALL, map_cap, flags, defer_list,
                                                   erpB, ecolB, erpA, ecolA, b_sorted ? 1 : 0); ::tsg::count_launch(); }
    }
    if (max_tiles_per_row > S2_SMALL) {
        const int slots = max_tiles_per_row < S2_SMAX ? max_tiles_per_row : S2_SMAX;
        { k_step2<512><<<ndefer, 512, step2_smem(slots, map_cap), s>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol, B.mask, crp, ccol,
                                                   cmask, rowcnt, S2_SMALL, S2_SMAX, map_cap, flags, defer_list,
                                                   erpB, ecolB, erpA); ::tsg::count_launch(); }
        const int wslots = max_tiles_per_row < S2E_WIN ? max_tiles_per_row : S2E_WIN;
        const int wmap = max_tiles_per_row > S2E_WIN ? (int)MAP_MAX : map_cap;
        { k_step2_entries<512><<<ndefer, 512, step2e_smem(wslots, wmap), s>>>(blkm, m, A.trp, crp, ccol, cmask, rowcnt, S2_SMALL, INT_MAX,
                                                   S2E_WIN, wmap, flags, defer_list,
                                                   erpB, ecolB, erpA, ecolA, b_sorted ? 1 : 0); ::tsg::count_launch(); }
    }
    if (win) {
        const cudaError_t e = cudaStreamWaitEvent(s, join, 0);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// ---- numeric bins of C's tile-rows ------------------------------------------

namespace {

constexpr int BIN_THREADS = 256;
constexpr int BIN_SCAN_THREADS = 1024;

// Rank of this thread's tile-row among the CTA's tile-rows of the same bin
// (index order), and per warp the count of each bin in s_wcnt[warp][bin].
__device__ __forceinline__ int bin_rank(int b, int lane, int warp, int (*s_wcnt)[NBIN])
{
    int rank = 0;
#pragma unroll
    for (int k = 0; k < NBIN; ++k) {
        const unsigned mk = __ballot_sync(0xffffffffu, b == k);
        if (b == k) rank = __popc(mk & lanemask_lt());
        if (lane == 0) s_wcnt[warp][k] = __popc(mk);
    }
    return rank;
}

// 1/3: one thread per C tile-row -- its bin from the finished structure
// (tile count, tile-column window, entries: numeric_classify); per CTA the
// count of each bin, and the bins' shared-memory maxima (one global atomic
// per CTA and bin).
__global__ void __launch_bounds__(BIN_THREADS)
k_bin_classify(int blkm, int m, const long long *__restrict__ crp, const int *__restrict__ ccol,
               const long long *__restrict__ rowptrC, NumericBinParams bp, unsigned char *bin, long long *binstat,
               int *ccount)
{
    constexpr int NWB = BIN_THREADS / 32;
    __shared__ int s_wcnt[NWB][NBIN];
    __shared__ long long s_req[NBIN];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < NBIN) s_req[tid] = 0;
    __syncthreads();
    const int i = blockIdx.x * BIN_THREADS + tid;
    int b = -1;
    if (i < blkm) {
        const long long c0 = crp[i], S = crp[i + 1] - c0;
        const int r0 = i * TILE, rows = min(TILE, m - r0);
        const long long nnz_tr = rowptrC[r0 + rows] - rowptrC[r0];
        const long long span = S > 0 ? (long long)ccol[c0 + S - 1] - ccol[c0] + 1 : 0;
        long long req = 0;
        numeric_classify(bp, S, nnz_tr, span, b, req);
        bin[i] = (unsigned char)b;
        if (req) atomicMax(&s_req[b], req);
    }
    bin_rank(b, lane, warp, s_wcnt);
    __syncthreads();
    if (tid < NBIN) {
        int tot = 0;
        for (int w = 0; w < NWB; ++w) tot += s_wcnt[w][tid];
        ccount[(long long)blockIdx.x * NBIN + tid] = tot;
        if (s_req[tid]) atomicMax(&binstat[NBIN + tid], s_req[tid]);
    }
}

// 2/3: one CTA per bin -- exclusive scan of the CTAs' counts (in place) and
// the bin's total
__global__ void __launch_bounds__(BIN_SCAN_THREADS)
k_bin_offsets(int nblocks, int *ccount, long long *binstat)
{
    __shared__ int s_part[BIN_SCAN_THREADS / 32];
    const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    long long run = 0;
    for (int base = 0; base < nblocks; base += BIN_SCAN_THREADS) {
        const int j = base + tid;
        const int v = j < nblocks ? ccount[(long long)j * NBIN + b] : 0;
        const int incl = warp_incl_scan(v, lane);
        if (lane == 31) s_part[warp] = incl;
        __syncthreads();
        int woff = 0, tot = 0;
        for (int w = 0; w < BIN_SCAN_THREADS / 32; ++w) {
            if (w < warp) woff += s_part[w];
            tot += s_part[w];
        }
        if (j < nblocks) ccount[(long long)j * NBIN + b] = (int)(run + woff + incl - v);
        run += tot;
        __syncthreads();
    }
    if (tid == 0) binstat[b] = run;
}

// 3/3: the bins' work lists in tile-row order (CTA offset + warp offset +
// rank), and the row classes of the rows of BIN_ROWS tile-rows
__global__ void __launch_bounds__(BIN_THREADS)
k_bin_scatter(int blkm, int m, const long long *__restrict__ crp, const int *__restrict__ ccol,
              const long long *__restrict__ rowptrC, NumericBinParams bp, const unsigned char *__restrict__ bin,
              const int *__restrict__ ccount, long long *binstat, int *binlist, int *rowlist)
{
    constexpr int NWB = BIN_THREADS / 32;
    __shared__ int s_wcnt[NWB][NBIN];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int i = blockIdx.x * BIN_THREADS + tid;
    const int b = i < blkm ? (int)bin[i] : -1;
    const int rank = bin_rank(b, lane, warp, s_wcnt);
    __syncthreads();
    if (b < 0) return;
    int woff = 0;
    for (int w = 0; w < warp; ++w) woff += s_wcnt[w][b];
    binlist[(long long)b * blkm + ccount[(long long)blockIdx.x * NBIN + b] + woff + rank] = i;
    if (b == BIN_ROWS) {   // rare: heavy tile-rows; their rows one by one
        const long long c0 = crp[i], S = crp[i + 1] - c0;
        const long long span = S > 0 ? (long long)ccol[c0 + S - 1] - ccol[c0] + 1 : 0;
        const int r0 = i * TILE, rows = min(TILE, m - r0);
        for (int r = 0; r < rows; ++r)
            record_row(bp, S, rowptrC[r0 + r + 1] - rowptrC[r0 + r], span, r0 + r, m, binstat, rowlist);
    }
}

}  // namespace

// The bins' lists keep C's tile-rows in index order, so that the numeric
// kernels' CTAs that run together work on neighbouring tile-rows and share
// B's rows in L2 (lists in the order the tile-rows were finished, or by
// CTAs in atomic order, measured up to 35 % slower numeric steps).
cudaError_t bin_tilerows(Pool &pool, int blkm, int m, const long long *crp, const int *ccol, const long long *rowptrC,
                         const NumericBinParams &bp, unsigned char *bin, long long *binstat, int *binlist, int *rowlist)
{
    if (blkm <= 0) return cudaSuccess;
    const int nblocks = (blkm + BIN_THREADS - 1) / BIN_THREADS;
    int *ccount = pool.alloc_n<int>((long long)nblocks * NBIN);
    if (!ccount) return pool.err;
    cudaStream_t s = pool.stream;
    k_bin_classify<<<nblocks, BIN_THREADS, 0, s>>>(blkm, m, crp, ccol, rowptrC, bp, bin, binstat, ccount);
    ::tsg::count_launch();
    k_bin_offsets<<<NBIN, BIN_SCAN_THREADS, 0, s>>>(nblocks, ccount, binstat);
    ::tsg::count_launch();
    k_bin_scatter<<<nblocks, BIN_THREADS, 0, s>>>(blkm, m, crp, ccol, rowptrC, bp, bin, ccount, binstat, binlist,
                                                   rowlist);
    ::tsg::count_launch();
    const cudaError_t e = cudaGetLastError();
    pool.free(ccount);
    return e;
}

}  // namespace tsg
