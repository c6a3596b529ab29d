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
// Outputs: cmask (16 uint16 per C tile), rowcnt[m] (nnz of each C row; a
// scan turns it into C's row pointer), bin[blkm] (numeric bin of each C
// tile-row) and per-bin counters/shared-memory sizes in `binstat`.
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

// OR over the set bits (15-c) of `ma` of B tile q's row c masks
__device__ __forceinline__ unsigned or_rows(unsigned ma, const uint16_t *__restrict__ bmask, long long q) {
    unsigned acc = 0;
    while (ma) {
        int b = __ffs(ma) - 1;      // bit b <-> local column 15-b
        acc |= bmask[q * TILE + (TILE - 1 - b)];
        ma &= ma - 1;
    }
    return acc;
}

constexpr int STG = 64;   // B tiles staged per warp at a time
constexpr int ENTRY_WALK_MAX = 3;   // mean A entries per A tile up to which step 2 walks A's rows by entry
constexpr int ENTRY_B_MAX = 64;     // ...taking there the B rows of at most this many entries

// OR `bits` into 16-bit mask idx of a uint16 array in shared memory (word atomics)
__device__ __forceinline__ void smask_or(unsigned short *m, int idx, unsigned bits) {
    atomicOr(reinterpret_cast<unsigned *>(m) + (idx >> 1), bits << ((idx & 1) * 16));
}

// slot of tile column j in C's tile-row: direct map over the row's window
// when it is narrow, binary search otherwise; -1 if j is not one of its tiles
__device__ __forceinline__ int c_slot(int j, int jbase, int span, const unsigned short *map, const int *scol, int S) {
    const unsigned off = (unsigned)(j - jbase);
    if (off >= (unsigned)span) return -1;
    const int s = map ? (int)map[off] : lower_bound_i(scol, S, j);
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
        uint16_t *cmask, int *rowcnt, int smin, int smax, int map_cap, NumericBinParams bp, unsigned char *bin,
        long long *binstat, int *binlist, int *rowlist, int *flags, const int *__restrict__ rows_list,
        const long long *__restrict__ erpB, const int *__restrict__ ecolB, const long long *__restrict__ erpA,
        const int *__restrict__ ecolA)
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
    // A tiles of a few entries each: walk A's rows entry by entry instead
    // (warp w takes rows w, w + NT/32, ...; lanes take the B row of each
    // entry), skipping the per-tile transpose.  Entries whose B row is
    // longer than ENTRY_B_MAX are left to the tile walk below, which then
    // takes only those (OR does not depend on order): there B's tile masks
    // cover many of the row's entries per operation.
    const long long nea = erpA[(long long)i * TILE + rows] - erpA[(long long)i * TILE];
    const bool by_entry = nea <= (long long)ENTRY_WALK_MAX * na;
    bool has_long = !by_entry;
    if (by_entry) {
        for (int r = warp; r < rows; r += (NT / 32)) {
            const int p0 = (int)erpA[(long long)i * TILE + r], p1 = (int)erpA[(long long)i * TILE + r + 1];
            for (int pb = p0; pb < p1; pb += 32) {
                const int cnt = min(32, p1 - pb);
                int bs = 0, be = 0;
                if (lane < cnt) {
                    const int k = ecolA[pb + lane];
                    bs = (int)erpB[k];
                    be = (int)erpB[k + 1];
                }
                if (be - bs > ENTRY_B_MAX) has_long = true;
                for (int q = 0; q < cnt; ++q) {
                    const int e0 = __shfl_sync(0xffffffffu, bs, q), e1 = __shfl_sync(0xffffffffu, be, q);
                    if (e1 - e0 > ENTRY_B_MAX) continue;
                    for (int e = e0 + lane; e < e1; e += 32) {
                        const int col = ecolB[e];
                        const int sl = c_slot(col >> 4, jbase, span, map, scol, S);
                        if (sl < 0) { bad = true; continue; }
                        smask_or(smask, r * S + sl, 0x8000u >> (col & 15));
                    }
                }
            }
        }
    }
    has_long = __syncthreads_or(has_long);
    for (int a = a0 + warp; a < a1 && has_long; a += (NT / 32)) {
        const int kt = acol[a];
        const int q0 = brp[kt], nq = brp[kt + 1] - q0;
        // transpose the A tile: colrows[c] = rows r whose mask has local column c
        unsigned ma = (lane < TILE) ? (unsigned)amask[(long long)a0 * TILE + (long long)lane * na + (a - a0)] : 0u;
        if (by_entry) {
            // only the columns whose B rows the entry walk left (a used
            // column names a row of B, so the row pointer reads stay in range)
            const unsigned used = __brev(__reduce_or_sync(0xffffffffu, ma)) >> 16;
            const bool lng = lane < TILE && ((used >> lane) & 1u) &&
                             erpB[kt * TILE + lane + 1] - erpB[kt * TILE + lane] > ENTRY_B_MAX;
            ma &= __brev(__ballot_sync(0xffffffffu, lng)) >> 16;
            if (!__any_sync(0xffffffffu, ma != 0u)) continue;
        }
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
    __syncthreads();
    __shared__ int s_bin;
    if (tid == 0) {
        long long nnz_tr = 0;
        for (int r = 0; r < TILE; ++r) nnz_tr += s_rowtot[r];
        int b;
        long long req = 0;
        numeric_classify(bp, S, nnz_tr, span, b, req);
        bin[i] = (unsigned char)b;
        record_bin(b, req, i, blkm, binstat, binlist);
        s_bin = b;
    }
    __syncthreads();
    if (s_bin == BIN_ROWS && tid < rows) record_row(bp, S, s_rowtot[tid], span, i * TILE + tid, m, binstat, rowlist);
}

// Tile-rows with more than `smax` C tiles: the tile slots are taken in
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
            uint16_t *cmask, int *rowcnt, int smax, NumericBinParams bp, unsigned char *bin,
            long long *binstat, int *binlist, int *rowlist, int *flags, const int *__restrict__ rows_list,
            const long long *__restrict__ erpB, const int *__restrict__ ecolB)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ long long s_rowtot[TILE];
    const int i = rows_list[blockIdx.x];
    if (i >= blkm) return;
    const long long c0 = crp[i];
    const int S = (int)(crp[i + 1] - c0);
    if (S <= smax) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int span = ccol[c0 + S - 1] - ccol[c0] + 1;
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
    const int rows = min(TILE, m - i * TILE);
    __shared__ int s_bin;
    if (tid == 0) {
        long long nnz_tr = 0;
        for (int r = 0; r < TILE; ++r) {
            if (r < rows) rowcnt[i * TILE + r] = (int)s_rowtot[r];
            nnz_tr += s_rowtot[r];
        }
        int b;
        long long req = 0;
        numeric_classify(bp, S, nnz_tr, span, b, req);
        bin[i] = (unsigned char)b;
        record_bin(b, req, i, blkm, binstat, binlist);
        s_bin = b;
    }
    __syncthreads();
    if (s_bin == BIN_ROWS && tid < rows) record_row(bp, S, s_rowtot[tid], span, i * TILE + tid, m, binstat, rowlist);
}

}  // namespace

constexpr int S2_SMAX = 4096;   // tiles per tile-row (or window) handled with shared-memory masks

constexpr int S2_SMALL = 1024;  // tile-rows of up to this many tiles: 256-thread CTAs with less shared memory

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
    return e;
}

// The deferred tile-rows (too many tiles or too wide a window for the fused
// warp kernel): up to S2_SMALL tiles in 256-thread CTAs, up to S2_SMAX in
// 512-thread CTAs (one per SM at that shared memory, so more warps per
// CTA), beyond that in windows.  Each launch walks the whole defer list and
// skips the tile-rows of the other classes.
cudaError_t step2_masks(Pool &pool, const TileCSR &A, const TileCSR &B, int m, int blkm, const long long *crp,
                        const int *ccol, uint16_t *cmask, int *rowcnt, int max_tiles_per_row, int max_span,
                        const NumericBinParams &bp, unsigned char *bin, long long *binstat, int *binlist,
                        int *rowlist, int *flags, const int *defer_list, int ndefer, const long long *erpB,
                        const int *ecolB, const long long *erpA, const int *ecolA)
{
    cudaStream_t s = pool.stream;
    if (blkm <= 0 || ndefer <= 0) return cudaSuccess;
    const int map_cap = max_span < (int)MAP_MAX ? max_span : (int)MAP_MAX;
    {
        const int slots = max_tiles_per_row < S2_SMALL ? max_tiles_per_row : S2_SMALL;
        { k_step2<256><<<ndefer, 256, step2_smem(slots, map_cap), s>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol, B.mask, crp, ccol,
                                                   cmask, rowcnt, 0, S2_SMALL, map_cap, bp, bin, binstat, binlist, rowlist, flags, defer_list,
                                                   erpB, ecolB, erpA, ecolA); ::tsg::count_launch(); }
    }
    if (max_tiles_per_row > S2_SMALL) {
        const int slots = max_tiles_per_row < S2_SMAX ? max_tiles_per_row : S2_SMAX;
        { k_step2<512><<<ndefer, 512, step2_smem(slots, map_cap), s>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol, B.mask, crp, ccol,
                                                   cmask, rowcnt, S2_SMALL, S2_SMAX, map_cap, bp, bin, binstat, binlist, rowlist, flags, defer_list,
                                                   erpB, ecolB, erpA, ecolA); ::tsg::count_launch(); }
    }
    if (max_tiles_per_row > S2_SMAX) {
        { k_step2_win<512><<<ndefer, 512, step2_smem(S2_SMAX, MAP_MAX), s>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol, B.mask, crp, ccol,
                                                      cmask, rowcnt, S2_SMAX, bp, bin, binstat, binlist, rowlist, flags, defer_list,
                                                      erpB, ecolB); ::tsg::count_launch(); }
    }
    return cudaGetLastError();
}

}  // namespace tsg
