// tsg_tiles.cu -- CSR preparation, CSR -> 16x16 tile structure, the
// tile-level symbolic product (step 1), and the stable CSR transpose used
// for A*A^T.
//
// Both the conversion and step 1 are "sorted union of small integer keys per
// tile-row": the tile columns touched by 16 CSR rows (conversion,
// main_spgemm-col.cu:44-120 + :4976-4985), or the union over A's tiles (i,k)
// of B's tile-row k (step 1, main_spgemm-col.cu:122-188 and :572-627; the
// reference runs nsparse hash SpGEMM on the tile pattern for it,
// spgemm_nsparse_kernel.h:221-311, 1171-1438).  Here one warp owns a
// tile-row and sets bits in a shared-memory bitmap over the row's key window
// [min, max]; popc gives the count, a warp scan of per-word popc gives each
// key its rank, so the list comes out sorted with no sort and no hash.  Rows
// whose window exceeds 4096 keys go to a CTA-wide kernel that walks the
// window in 65,536-key chunks (any width).
//
// Row masks are stored per tile-row in row-major order: the masks of the
// tile-row whose tiles are t0..t1-1 occupy [16*t0, 16*t1), local row r of
// tile t at 16*t0 + r*(t1-t0) + (t-t0), so lanes that walk a tile-row's
// tiles read one row's masks contiguously.  (The reference's tile format,
// 16 masks per tile, is produced only when a caller asks for tile form.)
//
// Roofline: HBM-bound; the conversion reads each CSR column index twice
// (count pass, fill pass) and writes 36 bytes per tile.
#include "tsg_internal.cuh"
#include "tsg_numeric.cuh"
#include <algorithm>
#include <climits>

namespace tsg {

namespace {

constexpr int NW = 128;                 // narrow bitmap: 128 words = 4096 keys per warp
constexpr int WPC = 8;                  // warps per CTA in the narrow kernels
constexpr int WIDE_WORDS = 2048;        // wide bitmap chunk: 65,536 keys
constexpr int WIDE_GRID = 1216;         // CTAs of the wide union (grid-stride over the wide tile-rows): 8 per SM
constexpr int WIDE_THREADS = 256;
constexpr int WIDE_SMEM = WIDE_WORDS * 4 * 2;  // bitmap + word prefix

// ---- key sources --------------------------------------------------------

// Tile columns of the entries of one tile-row of a CSR matrix.
struct CsrKeys {
    static constexpr bool kHasOrRange = false;
    struct Params { const long long *rp; const int *col; int m, n; };
    const long long *rp; const int *col; int n, r0, r1;
    __device__ CsrKeys(const Params &p, int row)
        : rp(p.rp), col(p.col), n(p.n), r0(row * TILE), r1(min(p.m, row * TILE + TILE)) {}
    __device__ void bounds(int start, int stride, int &kmin, int &kmax) const {
        for (long long q = rp[r0] + start; q < rp[r1]; q += stride) {
            int c = col[q];
            if ((unsigned)c < (unsigned)n) { kmin = min(kmin, c >> 4); kmax = max(kmax, c >> 4); }
        }
    }
    template <class F> __device__ void each(int start, int stride, F &&f) const {
        for (int r = r0; r < r1; ++r) {
            const long long e = rp[r + 1];
            for (long long q = rp[r] + start; q < e; q += stride) {
                int c = col[q];
                if ((unsigned)c < (unsigned)n) f(c >> 4, r - r0, c & 15);
            }
        }
    }
    __device__ void or_bits(unsigned *bm, int kbase, int lane) const {
        each(lane, 32, [&](int key, int, int) {
            const int o = key - kbase;
            atomicOr(&bm[o >> 5], 1u << (o & 31));
        });
    }
};

// Tile columns of C's tile-row i: union over A's tiles (i,k) of B's tile-row k.
struct UnionKeys {
    static constexpr bool kHasOrRange = true;
    struct Params {
        const int *arp; const int *acol; const int *brp; const int *bcol;
        const long long *bmoff = nullptr; const unsigned *bmw = nullptr;   // B's tile-row bitmaps, if built
        // the wide tile-rows' window bitmaps, kept by the count pass for the
        // fill pass (wpr words per entry of the wide list), if there is room
        unsigned *wbm = nullptr; long long wpr = 0;
    };
    const int *arp, *acol, *brp, *bcol; const long long *bmoff; const unsigned *bmw; int i;
    __device__ UnionKeys(const Params &p, int row)
        : arp(p.arp), acol(p.acol), brp(p.brp), bcol(p.bcol), bmoff(p.bmoff), bmw(p.bmw), i(row) {}
    __device__ void bounds(int start, int stride, int &kmin, int &kmax) const {
        for (int a = arp[i] + start; a < arp[i + 1]; a += stride) {
            int k = acol[a];
            int q0 = brp[k], q1 = brp[k + 1];
            if (q1 > q0) { kmin = min(kmin, bcol[q0]); kmax = max(kmax, bcol[q1 - 1]); }
        }
    }
    template <class F> __device__ void each(int start, int stride, F &&f) const {
        for (int a = arp[i]; a < arp[i + 1]; ++a) {
            int k = acol[a];
            const int q1 = brp[k + 1];
            for (int q = brp[k] + start; q < q1; q += stride) f(bcol[q], 0, 0);
        }
    }
    // CTA-wide: OR the keys in [c0, c0 + span) (c0 a multiple of 32) into bm
    // (bit o stands for key c0 + o); warps take A tiles, and per A tile B's
    // tile-row bitmap goes in word by word when it has fewer words than keys
    __device__ void or_range(unsigned *bm, long long c0, long long span, int warp, int nwarps, int lane) const {
        const int a0 = arp[i], a1 = arp[i + 1];
        for (int a = a0 + warp; a < a1; a += nwarps) {
            const int k = acol[a];
            const int q0 = brp[k], q1 = brp[k + 1];
            if (q1 <= q0) continue;
            long long w0 = 0, w1 = 0;
            if (bmoff) { w0 = bmoff[k]; w1 = bmoff[k + 1]; }
            if (w1 > w0 && w1 - w0 < q1 - q0) {
                const long long base = (long long)(bcol[q0] & ~31) - c0;   // bit 0 of word w0, relative to c0
                for (long long w = w0 + lane; w < w1; w += 32) {
                    const long long o = base + ((w - w0) << 5);
                    if (o >= 0 && o < span) {
                        const unsigned x = bmw[w];
                        if (x) atomicOr(&bm[o >> 5], x);
                    }
                }
            } else {
                for (int q = q0 + lane; q < q1; q += 32) {
                    const long long o = (long long)bcol[q] - c0;
                    if (o >= 0 && o < span) atomicOr(&bm[o >> 5], 1u << (o & 31));
                }
            }
        }
    }
    // OR the keys into a warp's bitmap bm whose bit o stands for key kbase+o
    // (kbase a multiple of 32): per A tile, B's tile-row bitmap word by word
    // when it has fewer words than keys, else key by key.  The A tiles' B
    // tile-row descriptors are fetched 32 at a time, one per lane.
    __device__ void or_bits(unsigned *bm, int kbase, int lane) const {
        const int a0 = arp[i], a1 = arp[i + 1];
        for (int ab = a0; ab < a1; ab += 32) {
            const int nac = min(32, a1 - ab);
            int q0 = 0, q1 = 0, d = 0;
            long long w0 = 0, w1 = 0;
            if (lane < nac) {
                const int k = acol[ab + lane];
                q0 = brp[k]; q1 = brp[k + 1];
                if (bmoff) { w0 = bmoff[k]; w1 = bmoff[k + 1]; }
                if (q1 > q0) d = ((bcol[q0] & ~31) - kbase) >> 5;
            }
            for (int t = 0; t < nac; ++t) {
                const int tq0 = __shfl_sync(0xffffffffu, q0, t), tq1 = __shfl_sync(0xffffffffu, q1, t);
                const long long tw0 = __shfl_sync(0xffffffffu, w0, t), tw1 = __shfl_sync(0xffffffffu, w1, t);
                if (tw1 > tw0 && tw1 - tw0 < tq1 - tq0) {
                    const int td = __shfl_sync(0xffffffffu, d, t);
                    for (long long w = tw0 + lane; w < tw1; w += 32) {
                        const unsigned x = bmw[w];
                        if (x) atomicOr(&bm[td + (int)(w - tw0)], x);
                    }
                } else {
                    for (int q = tq0 + lane; q < tq1; q += 32) {
                        const int o = bcol[q] - kbase;
                        atomicOr(&bm[o >> 5], 1u << (o & 31));
                    }
                }
            }
        }
    }
};

// ---- narrow path: one warp per tile-row ----------------------------------

template <class KS>
__global__ void __launch_bounds__(WPC * 32)
k_union_count(typename KS::Params P, int nrows, int *cnt, int *wide_list, int *wide_n, int *stat, int *defer_list,
              int *defer_n, int defer_S)
{
    __shared__ unsigned s_bm[WPC][NW + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * WPC + warp;
    if (row >= nrows) return;
    KS ks(P, row);
    int kmin = INT_MAX, kmax = -1;
    ks.bounds(lane, 32, kmin, kmax);
    kmin = warp_min_int(kmin);
    kmax = warp_max_int(kmax);
    if (kmax < kmin) { if (lane == 0) cnt[row] = 0; return; }
    const long long span = (long long)kmax - kmin + 1;
    if (stat && lane == 0) atomicMax(stat + 1, (int)span);
    if (span > NW * 32) {
        if (lane == 0) {
            cnt[row] = 0;
            wide_list[atomicAdd(wide_n, 1)] = row;
            if (defer_list) defer_list[atomicAdd(defer_n, 1)] = row;
        }
        return;
    }
    unsigned *bm = s_bm[warp];
    const int kbase = kmin & ~31;
    const int nwords = ((kmax - kbase) >> 5) + 1;     // at most NW + 1
    for (int w = lane; w < nwords; w += 32) bm[w] = 0;
    __syncwarp();
    ks.or_bits(bm, kbase, lane);
    __syncwarp();
    int c = 0;
    for (int w = lane; w < nwords; w += 32) c += __popc(bm[w]);
    c = warp_sum_int(c);
    if (lane == 0) {
        cnt[row] = c;
        if (stat) atomicMax(stat, c);
        if (defer_list && c > defer_S) defer_list[atomicAdd(defer_n, 1)] = row;
    }
}

// tile-rows of up to this many tiles build their masks in shared memory
// (the warp's 16 x FILL_SMEM_TILES row masks), the rest with global atomics
constexpr int FILL_SMEM_TILES = 64;

template <class KS, bool MASK, typename TP>
__global__ void __launch_bounds__(WPC * 32)
k_union_fill(typename KS::Params P, int nrows, const TP *rowptr, int *out, uint16_t *mask)
{
    __shared__ unsigned s_bm[WPC][NW];
    __shared__ unsigned short s_pref[WPC][NW];
    __shared__ unsigned s_mw[MASK ? WPC : 1][MASK ? FILL_SMEM_TILES * TILE / 2 : 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * WPC + warp;
    if (row >= nrows) return;
    KS ks(P, row);
    int kmin = INT_MAX, kmax = -1;
    ks.bounds(lane, 32, kmin, kmax);
    kmin = warp_min_int(kmin);
    kmax = warp_max_int(kmax);
    if (kmax < kmin) return;
    const long long span = (long long)kmax - kmin + 1;
    if (span > NW * 32) return;  // handled by the wide kernel
    unsigned *bm = s_bm[warp];
    unsigned short *pref = s_pref[warp];
    const int nwords = (int)((span + 31) >> 5);
    for (int w = lane; w < nwords; w += 32) bm[w] = 0;
    __syncwarp();
    ks.each(lane, 32, [&](int key, int, int) {
        int o = key - kmin;
        atomicOr(&bm[o >> 5], 1u << (o & 31));
    });
    __syncwarp();
    const int wpl = (nwords + 31) >> 5;
    const int w0 = min(nwords, lane * wpl), w1 = min(nwords, w0 + wpl);
    int lc = 0;
    for (int w = w0; w < w1; ++w) lc += __popc(bm[w]);
    const int incl = warp_incl_scan(lc, lane);
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const long long base = (long long)rowptr[row];
    int run = incl - lc;
    for (int w = w0; w < w1; ++w) {
        unsigned x = bm[w];
        pref[w] = (unsigned short)run;
        while (x) {
            int b = __ffs(x) - 1;
            out[base + run] = kmin + w * 32 + b;
            ++run;
            x &= x - 1;
        }
    }
    if (MASK) {
        unsigned *mw = reinterpret_cast<unsigned *>(mask) + base * 8;
        if (total <= FILL_SMEM_TILES) {
            // the row masks in shared memory (16 x total halfwords, row-major),
            // written out once: no global atomics
            unsigned *sw = s_mw[warp];
            for (int t = lane; t < total * 8; t += 32) sw[t] = 0u;
            __syncwarp();
            ks.each(lane, 32, [&](int key, int r, int c) {
                const int o = key - kmin, w = o >> 5;
                const int idx = r * total + pref[w] + __popc(bm[w] & ((1u << (o & 31)) - 1u));
                atomicOr(&sw[idx >> 1], (1u << (TILE - 1 - c)) << ((idx & 1) * 16));
            });
            __syncwarp();
            for (int t = lane; t < total * 8; t += 32) mw[t] = sw[t];
        } else {
            // zero this tile-row's masks, then OR the entries in
            for (int t = lane; t < total * 8; t += 32) mw[t] = 0u;
            __syncwarp();
            ks.each(lane, 32, [&](int key, int r, int c) {
                int o = key - kmin, w = o >> 5;
                int slot = pref[w] + __popc(bm[w] & ((1u << (o & 31)) - 1u));
                atomic_or_mask16(mask, base * TILE + (long long)r * total + slot, 1u << (TILE - 1 - c));
            });
        }
    }
}

// ---- fused step-1 fill + step 2 (narrow tile-rows) -------------------------

constexpr int FWPC = 4;                 // warps per CTA
constexpr int FUSED_ENTRY_WALK_MAX = 3; // mean A entries per A tile up to which A's rows are walked by entry,
constexpr int FUSED_ENTRY_B_MAX = 64;   // ...taking there the B rows of at most this many entries
constexpr int FSW = FUSED_MAX_TILES;    // most C tiles per tile-row handled here
static_assert(NW * 32 == FUSED_MAX_SPAN, "fused window");

// One warp per C tile-row whose tile-column window is at most 4096 wide and
// which has at most FSW tiles: it writes the row's sorted tile columns (step
// 1) and then, in the same warp, its row masks (step 2): for each A tile
// (i,k), lanes take B's tiles (k,j) -- the bitmap rank of j is its slot --
// and for every nonzero row r of the A tile OR together the B rows named by
// A's row mask (masks read coalesced from the row-major layout).  Lanes hold
// distinct slots, so the accumulation in shared memory needs no atomics.
// Then per-row popcounts give C's row counts and the numeric bin.
__global__ void __launch_bounds__(FWPC * 32)
k_sym_fused(UnionKeys::Params P, int blkm, int m, const long long *__restrict__ crp, int *ccol,
            const uint16_t *__restrict__ amaskT, const uint16_t *__restrict__ bmaskT, uint16_t *cmask, int *rowcnt,
            int *flags,
            const long long *__restrict__ erpB, const int *__restrict__ ecolB, const long long *__restrict__ erpA,
            const int *__restrict__ ecolA)
{
    __shared__ unsigned s_bm[FWPC][NW + 1];
    __shared__ unsigned short s_pref[FWPC][NW + 1];
    __shared__ unsigned short s_msk[FWPC][TILE * FSW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * FWPC + warp;
    if (row >= blkm) return;
    UnionKeys ks(P, row);
    int kmin = INT_MAX, kmax = -1;
    ks.bounds(lane, 32, kmin, kmax);
    kmin = warp_min_int(kmin);
    kmax = warp_max_int(kmax);
    const long long c0 = crp[row];
    const int S = (int)(crp[row + 1] - c0);
    const long long span = kmax >= kmin ? (long long)kmax - kmin + 1 : 0;
    if (span > NW * 32) return;   // wide: the wide fill writes its columns, the CTA step-2 kernel its masks
    const int rows = min(TILE, m - row * TILE);
    unsigned *bm = s_bm[warp];
    unsigned short *pref = s_pref[warp];
    unsigned short *msk = s_msk[warp];
    // bit o of bm stands for tile column kbase + o (kbase a multiple of 32)
    const int kbase = kmin & ~31;
    const int nwords = ((kmax - kbase) >> 5) + 1;     // at most NW + 1
    const int wbits = nwords * 32;
    for (int w = lane; w < nwords; w += 32) bm[w] = 0;
    if (S <= FSW)
        for (int t = lane; t < S * TILE; t += 32) msk[t] = 0;
    __syncwarp();
    ks.or_bits(bm, kbase, lane);
    __syncwarp();
    {   // sorted tile columns + per-word ranks
        const int wpl = (nwords + 31) >> 5;
        const int w0 = min(nwords, lane * wpl), w1 = min(nwords, w0 + wpl);
        int lc = 0;
        for (int w = w0; w < w1; ++w) lc += __popc(bm[w]);
        const int incl = warp_incl_scan(lc, lane);
        int run = incl - lc;
        for (int w = w0; w < w1; ++w) {
            unsigned x = bm[w];
            pref[w] = (unsigned short)run;
            while (x) {
                const int b = __ffs(x) - 1;
                ccol[c0 + run] = kbase + w * 32 + b;
                ++run;
                x &= x - 1;
            }
        }
    }
    __syncwarp();
    if (S > FSW) return;          // masks and counts of this tile-row: CTA step-2 kernel
    const int a0 = P.arp[row], a1 = P.arp[row + 1], na = a1 - a0;
    bool bad = false;
    // A tiles of a few entries each: A's rows entry by entry, lanes over the
    // B row of each entry (no per-tile transpose).  Entries whose B row is
    // longer than FUSED_ENTRY_B_MAX are left to the tile walk, which then
    // takes only those (OR does not depend on order).
    const long long ea0 = erpA[(long long)row * TILE];
    const bool by_entry = erpA[(long long)row * TILE + rows] - ea0 <= (long long)FUSED_ENTRY_WALK_MAX * na;
    bool has_long = !by_entry;
    if (by_entry) {
        unsigned *mw = reinterpret_cast<unsigned *>(msk);
        const int p0 = (int)ea0, p1 = (int)erpA[(long long)row * TILE + rows];
        // lane l <= rows holds the start of row l; an entry's row is the
        // number of row starts at or before it, less one
        const int rstart = lane <= rows ? (int)erpA[(long long)row * TILE + lane] : INT_MAX;
        for (int pb = p0; pb < p1; pb += 32) {
            const int cnt = min(32, p1 - pb);
            int bs = 0, be = 0;
            if (lane < cnt) {
                const int k = ecolA[pb + lane];
                bs = (int)erpB[k];
                be = (int)erpB[k + 1];
            }
            if (be - bs > FUSED_ENTRY_B_MAX) has_long = true;
            for (int q = 0; q < cnt; ++q) {
                const int r = __popc(__ballot_sync(0xffffffffu, rstart <= pb + q)) - 1;
                const int e0 = __shfl_sync(0xffffffffu, bs, q), e1 = __shfl_sync(0xffffffffu, be, q);
                if (e1 - e0 > FUSED_ENTRY_B_MAX) continue;
                for (int e = e0 + lane; e < e1; e += 32) {
                    const int col = ecolB[e];
                    const int o = (col >> 4) - kbase;
                    int slot = -1;
                    if (o >= 0 && o < wbits) {
                        const int w = o >> 5;
                        slot = pref[w] + __popc(bm[w] & ((1u << (o & 31)) - 1u));
                    }
                    if (slot < 0 || slot >= S) { bad = true; continue; }
                    const int idx = r * S + slot;
                    atomicOr(mw + (idx >> 1), (0x8000u >> (col & 15)) << ((idx & 1) * 16));
                }
            }
        }
    }
    __syncwarp();
    has_long = __any_sync(0xffffffffu, has_long);
    for (int ab = a0; ab < a1 && has_long; ab += 32) {
        // up to 32 A tiles at once, one per lane: B's tile-row, the columns
        // the A tile uses (bit c: local column c; with the entry walk only
        // those whose B row it left), and what the element path would cost
        // over those columns (32-entry chunks of their B rows)
        const int nac = min(32, a1 - ab);
        int q0l = 0, nql = 0, ktl = 0, eitl = 0;
        unsigned colsl = 0u;
        if (lane < nac) {
            const int a = ab + lane;
            ktl = P.acol[a];
            q0l = P.brp[ktl];
            nql = P.brp[ktl + 1] - q0l;
            const uint4 *at = reinterpret_cast<const uint4 *>(amaskT + (long long)a * TILE);
            const uint4 x0 = at[0], x1 = at[1];
            unsigned u = x0.x | x0.y | x0.z | x0.w | x1.x | x1.y | x1.z | x1.w;
            u = (u | (u >> 16)) & 0xffffu;               // bit 15-c: column c used
            colsl = __brev(u) >> 16;                      // bit c: column c used
            for (unsigned cs = colsl; cs; cs &= cs - 1) {
                const int c = __ffs(cs) - 1;
                const long long len = erpB[(long long)ktl * TILE + c + 1] - erpB[(long long)ktl * TILE + c];
                if (by_entry && len <= FUSED_ENTRY_B_MAX) colsl &= ~(1u << c);   // the entry walk did it
                else eitl += (int)((len + 31) >> 5);
            }
        }
        // the next A tile's row masks are loaded while the current one is walked
        unsigned ma_next = (lane < TILE) ? (unsigned)amaskT[(long long)ab * TILE + lane] : 0u;
        for (int t = 0; t < nac; ++t) {
            const int q0 = __shfl_sync(0xffffffffu, q0l, t), nq = __shfl_sync(0xffffffffu, nql, t);
            const int kt = __shfl_sync(0xffffffffu, ktl, t);
            const unsigned acols = __shfl_sync(0xffffffffu, colsl, t);
            const int elem_iters = __shfl_sync(0xffffffffu, eitl, t);
            unsigned ma = ma_next;
            if (t + 1 < nac) ma_next = (lane < TILE) ? (unsigned)amaskT[(long long)(ab + t + 1) * TILE + lane] : 0u;
            if (!acols) continue;
            ma &= __brev(acols) >> 16;                    // row masks restricted to those columns
            // A tiles with few entries: B's rows element by element (as in the
            // CTA step-2 kernel); lanes may then share a slot, so word atomics
            if (elem_iters <= 3 * ((nq + 31) >> 5)) {
                int eb0 = 0, eb1 = 0;   // operands hold < 2^31 entries
                if (lane < TILE && ((acols >> lane) & 1u)) {
                    eb0 = (int)erpB[(long long)kt * TILE + lane];
                    eb1 = (int)erpB[(long long)kt * TILE + lane + 1];
                }
                unsigned *mw = reinterpret_cast<unsigned *>(msk);
                __syncwarp();
                for (unsigned cs = acols; cs; cs &= cs - 1) {
                    const int c = __ffs(cs) - 1;
                    const int e0 = __shfl_sync(0xffffffffu, eb0, c), e1 = __shfl_sync(0xffffffffu, eb1, c);
                    const unsigned rowsc = __ballot_sync(0xffffffffu, (ma >> (TILE - 1 - c)) & 1u) & 0xffffu;
                    for (int e = e0 + lane; e < e1; e += 32) {
                        const int o = (ecolB[e] >> 4) - kbase;
                        int slot = -1;
                        if (o >= 0 && o < wbits) {
                            const int w = o >> 5;
                            slot = pref[w] + __popc(bm[w] & ((1u << (o & 31)) - 1u));
                        }
                        if (slot < 0 || slot >= S) { bad = true; continue; }
                        const unsigned bit = 0x8000u >> (ecolB[e] & 15);
                        for (unsigned rs = rowsc; rs; rs &= rs - 1) {
                            const int idx = (__ffs(rs) - 1) * S + slot;
                            atomicOr(mw + (idx >> 1), bit << ((idx & 1) * 16));
                        }
                    }
                }
                __syncwarp();
                continue;
            }
            // tile path: lanes take B's tiles (k,j) -- the bitmap rank of j
            // is the slot of C tile (i,j) -- and load each tile's 16 row
            // masks at once (tile-major copy: two 16-byte loads); then per
            // column c of the A tile the rows of A that use it (a ballot,
            // uniform) get B's row c OR'ed in.  Lanes hold distinct slots,
            // so the shared-memory updates need no atomics.
            unsigned colrows[TILE];
#pragma unroll
            for (int c = 0; c < TILE; ++c)
                colrows[c] = ((acols >> c) & 1u) ? __ballot_sync(0xffffffffu, (ma >> (TILE - 1 - c)) & 1u) & 0xffffu : 0u;
            for (int qb = 0; qb < nq; qb += 32) {
                const int q = qb + lane;
                int slot = -1;
                if (q < nq) {
                    const int o = P.bcol[q0 + q] - kbase;
                    if (o >= 0 && o < wbits) {
                        const int w = o >> 5;
                        slot = pref[w] + __popc(bm[w] & ((1u << (o & 31)) - 1u));
                    }
                    if (slot < 0 || slot >= S) { bad = true; slot = -1; }
                }
                uint4 lo = make_uint4(0u, 0u, 0u, 0u), hi = lo;
                if (slot >= 0) {
                    const uint4 *bt = reinterpret_cast<const uint4 *>(bmaskT + (long long)(q0 + q) * TILE);
                    lo = bt[0];
                    hi = bt[1];
                }
                const unsigned bw[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
                for (int c = 0; c < TILE; ++c) {
                    const unsigned b = (bw[c >> 1] >> ((c & 1) * 16)) & 0xffffu;
                    if (!b) continue;
                    for (unsigned rws = colrows[c]; rws; rws &= rws - 1) {
                        const int r = __ffs(rws) - 1;
                        msk[r * S + slot] |= (unsigned short)b;
                    }
                }
            }
        }
    }
    __syncwarp();
    for (int t = lane; t < S * TILE; t += 32) cmask[c0 * TILE + t] = msk[t];
    for (int r = 0; r < rows; ++r) {
        int c = 0;
        for (int sl = lane; sl < S; sl += 32) c += __popc((unsigned)msk[r * S + sl]);
        c = warp_sum_int(c);
        if (lane == 0) rowcnt[row * TILE + r] = c;
    }
    if (bad) set_flag(flags, FLAG_INTERNAL);
}

// Row-major masks of each tile-row -> 16 consecutive masks per tile (the
// reference's layout).  One warp per tile-row.
template <typename TP>
__global__ void k_masks_to_tile_major(int blkm, const TP *__restrict__ rowptr, const uint16_t *__restrict__ src,
                                      uint16_t *dst)
{
    // lanes take tiles: each gathers its tile's 16 row masks (loads of one
    // row of the tile-row are coalesced across the lanes) and writes them as
    // two 16-byte stores (32 contiguous bytes per tile; dst is 32-byte aligned)
    const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= blkm) return;
    const long long b = (long long)rowptr[row];
    const long long nt = (long long)rowptr[row + 1] - b;
    for (long long t = lane; t < nt; t += 32) {
        unsigned w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            w[k] = (unsigned)src[b * TILE + (2 * k) * nt + t] | ((unsigned)src[b * TILE + (2 * k + 1) * nt + t] << 16);
        uint4 *d = reinterpret_cast<uint4 *>(dst + (b + t) * TILE);
        d[0] = make_uint4(w[0], w[1], w[2], w[3]);
        d[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// ---- wide path: one CTA per tile-row, chunked window ----------------------

__device__ __forceinline__ int block_reduce_min(int v, int *sred) {
    v = warp_min_int(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sred[warp] = v;
    __syncthreads();
    int r = INT_MAX;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = min(r, sred[w]);
    __syncthreads();
    return r;
}
__device__ __forceinline__ int block_reduce_max(int v, int *sred) {
    v = warp_max_int(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sred[warp] = v;
    __syncthreads();
    int r = -1;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = max(r, sred[w]);
    __syncthreads();
    return r;
}
__device__ __forceinline__ long long block_reduce_sum_ll(long long v, long long *sred) {
    v = warp_sum_ll(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sred[warp] = v;
    __syncthreads();
    long long r = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sred[w];
    __syncthreads();
    return r;
}

// FILL=false: count (cnt[row]); FILL=true: sorted list + optional masks.
template <class KS, bool FILL, bool MASK, typename TP>
__global__ void __launch_bounds__(WIDE_THREADS)
k_union_wide(typename KS::Params P, const int *wide_list, const int *wide_n, int *cnt, int *stat_max,
             const TP *rowptr, int *out, uint16_t *mask, int *next)
{
    extern __shared__ unsigned s_dyn[];
    unsigned *bm = s_dyn;
    int *pref = reinterpret_cast<int *>(s_dyn + WIDE_WORDS);
    __shared__ int s_red[WIDE_THREADS / 32];
    __shared__ long long s_redll[WIDE_THREADS / 32];
    __shared__ int s_wsum[WIDE_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nw = *wide_n;
    __shared__ int s_next;
    // each CTA takes the next wide tile-row from a counter (their costs differ widely)
    for (;;) {
        if (tid == 0) s_next = atomicAdd(next, 1);
        __syncthreads();
        const int wi = s_next;
        if (wi >= nw) break;
        const int row = wide_list[wi];
        KS ks(P, row);
        int kmin = INT_MAX, kmax = -1;
        ks.bounds(tid, WIDE_THREADS, kmin, kmax);
        kmin = block_reduce_min(kmin, s_red);
        kmax = block_reduce_max(kmax, s_red);
        long long base = 0, ntiles = 0;
        if (FILL) {
            base = (long long)rowptr[row];
            ntiles = (long long)rowptr[row + 1] - base;
            if (MASK) {
                unsigned *mw = reinterpret_cast<unsigned *>(mask) + base * 8;
                for (long long t = tid; t < ntiles * 8; t += WIDE_THREADS) mw[t] = 0u;
                __syncthreads();
            }
        }
        long long run = 0;
        // chunks start on a multiple of 32 so that B's bitmap words align
        for (long long c0 = kmin & ~31ll; c0 <= kmax; c0 += (long long)WIDE_WORDS * 32) {
            const long long span = min((long long)WIDE_WORDS * 32, (long long)kmax - c0 + 1);
            const int nwords = (int)((span + 31) >> 5);
            // the window's bitmap in global memory (count pass: stored, fill
            // pass: loaded instead of taking the union again)
            unsigned *gbm = nullptr;
            if constexpr (KS::kHasOrRange)
                if (P.wbm) gbm = P.wbm + (long long)wi * P.wpr + ((c0 - (kmin & ~31ll)) >> 5);
            if (FILL && gbm) {
                for (int w = tid; w < nwords; w += WIDE_THREADS) bm[w] = gbm[w];
                __syncthreads();
            } else {
                for (int w = tid; w < nwords; w += WIDE_THREADS) bm[w] = 0;
                __syncthreads();
                if constexpr (KS::kHasOrRange) {
                    ks.or_range(bm, c0, span, warp, WIDE_THREADS / 32, lane);
                } else {
                    ks.each(tid, WIDE_THREADS, [&](int key, int, int) {
                        long long o = (long long)key - c0;
                        if (o >= 0 && o < span) atomicOr(&bm[o >> 5], 1u << (o & 31));
                    });
                }
                __syncthreads();
                if (!FILL && gbm)
                    for (int w = tid; w < nwords; w += WIDE_THREADS) gbm[w] = bm[w];
            }
            const int wpt = (nwords + WIDE_THREADS - 1) / WIDE_THREADS;
            const int w0 = min(nwords, tid * wpt), w1 = min(nwords, w0 + wpt);
            int lc = 0;
            for (int w = w0; w < w1; ++w) lc += __popc(bm[w]);
            if (!FILL) {
                run += block_reduce_sum_ll(lc, s_redll);
                continue;
            }
            // block exclusive scan of lc
            int incl = warp_incl_scan(lc, lane);
            if (lane == 31) s_wsum[warp] = incl;
            __syncthreads();
            int woff = 0, chunk_total = 0;
            for (int w = 0; w < WIDE_THREADS / 32; ++w) {
                if (w < warp) woff += s_wsum[w];
                chunk_total += s_wsum[w];
            }
            int r2 = woff + incl - lc;
            for (int w = w0; w < w1; ++w) {
                unsigned x = bm[w];
                pref[w] = r2;
                while (x) {
                    int b = __ffs(x) - 1;
                    out[base + run + r2] = (int)(c0 + w * 32 + b);
                    ++r2;
                    x &= x - 1;
                }
            }
            __syncthreads();
            if (MASK) {
                ks.each(tid, WIDE_THREADS, [&](int key, int r, int c) {
                    long long o = (long long)key - c0;
                    if (o >= 0 && o < span) {
                        int w = (int)(o >> 5);
                        long long slot = run + pref[w] + __popc(bm[w] & ((1u << (o & 31)) - 1u));
                        atomic_or_mask16(mask, base * TILE + r * ntiles + slot, 1u << (TILE - 1 - c));
                    }
                });
            }
            run += chunk_total;
            __syncthreads();
        }
        if (!FILL && tid == 0) {
            cnt[row] = (int)run;
            if (stat_max) { atomicMax(stat_max, (int)run); atomicMax(stat_max + 1, kmax - kmin + 1); }
        }
        __syncthreads();
    }
}

// ---- preparation ----------------------------------------------------------

// One launch: thread i <= m checks and copies row pointer i (clamped to
// [0, nnz], int64); with `col` (validation on) the grid also strides over
// the column indices, checking each against n.
template <typename Tr>
__global__ void k_prepare_rowptr(const Tr *__restrict__ rp, long long m, long long nnz, long long *out, int *flags,
                                 const int *__restrict__ col, int n)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i <= m) {
        const long long v = (long long)rp[i];
        bool bad = (v < 0 || v > nnz) || (i == 0 && v != 0) || (i == m && v != nnz);
        if (i < m && (long long)rp[i + 1] < v) bad = true;
        if (bad) set_flag(flags, FLAG_BAD_INPUT);
        out[i] = v < 0 ? 0 : (v > nnz ? nnz : v);
    }
    if (!col) return;
    bool bad = false;
    for (long long q = i; q < nnz; q += (long long)gridDim.x * blockDim.x) bad |= ((unsigned)col[q] >= (unsigned)n);
    if (bad) set_flag(flags, FLAG_BAD_INPUT);
}

// ---- stable transpose (CSR of A^T), LSD radix sort of (column, position) --

constexpr int RADIX_THREADS = 256;
constexpr int RADIX_ITEMS = 8;
constexpr int RADIX_CHUNK = RADIX_THREADS * RADIX_ITEMS;
constexpr int RADIX_BITS = 8;
constexpr int RADIX_BINS = 1 << RADIX_BITS;

// per-chunk digit histogram; counts laid out digit-major (digit * nchunks + chunk)
__global__ void __launch_bounds__(RADIX_THREADS)
k_radix_hist(const int *__restrict__ keys, long long n, int shift, int nchunks, int *counts)
{
    __shared__ int s_h[RADIX_BINS];
    for (int d = threadIdx.x; d < RADIX_BINS; d += RADIX_THREADS) s_h[d] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * RADIX_CHUNK;
    for (int j = threadIdx.x; j < RADIX_CHUNK; j += RADIX_THREADS) {
        long long q = base + j;
        if (q < n) atomicAdd(&s_h[((unsigned)keys[q] >> shift) & (RADIX_BINS - 1)], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX_BINS; d += RADIX_THREADS)
        counts[(long long)d * nchunks + blockIdx.x] = s_h[d];
}

// stable scatter: items are ranked in input order within the chunk
// (warp-contiguous sub-chunks, lanes striped inside each 32-item step)
__global__ void __launch_bounds__(RADIX_THREADS)
k_radix_scatter(const int *__restrict__ kin, const int *__restrict__ vin, int *kout, int *vout,
                long long n, int shift, int nchunks, const int *__restrict__ offsets)
{
    constexpr int NWARP = RADIX_THREADS / 32;
    __shared__ int s_cnt[NWARP][RADIX_BINS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < NWARP * RADIX_BINS; d += RADIX_THREADS) (&s_cnt[0][0])[d] = 0;
    __syncthreads();
    const long long wbase = (long long)blockIdx.x * RADIX_CHUNK + (long long)warp * (RADIX_ITEMS * 32);
    int key[RADIX_ITEMS], val[RADIX_ITEMS], dig[RADIX_ITEMS], loc[RADIX_ITEMS];
#pragma unroll
    for (int it = 0; it < RADIX_ITEMS; ++it) {
        long long q = wbase + it * 32 + lane;
        bool ok = q < n;
        key[it] = ok ? kin[q] : 0;
        val[it] = ok ? vin[q] : 0;
        int d = ok ? (int)(((unsigned)key[it] >> shift) & (RADIX_BINS - 1)) : RADIX_BINS;  // RADIX_BINS = none
        dig[it] = d;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & lanemask_lt());
        int leader = __ffs(peers) - 1;
        int before = 0;
        if (ok) before = s_cnt[warp][d];
        __syncwarp();
        loc[it] = before + rank;
        if (ok && lane == leader) s_cnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // exclusive scan over warps, per digit
    for (int d = threadIdx.x; d < RADIX_BINS; d += RADIX_THREADS) {
        int run = 0;
        for (int w = 0; w < NWARP; ++w) { int c = s_cnt[w][d]; s_cnt[w][d] = run; run += c; }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < RADIX_ITEMS; ++it) {
        long long q = wbase + it * 32 + lane;
        if (q < n) {
            int d = dig[it];
            long long dst = (long long)offsets[(long long)d * nchunks + blockIdx.x] + s_cnt[warp][d] + loc[it];
            kout[dst] = key[it];
            vout[dst] = val[it];
        }
    }
}

__global__ void k_iota_and_keys(const int *__restrict__ col, long long nnz, int n, int *keys, int *vals)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nnz; q += (long long)gridDim.x * blockDim.x) {
        int c = col[q];
        keys[q] = ((unsigned)c < (unsigned)n) ? c : n - 1;  // invalid input is flagged elsewhere
        vals[q] = (int)q;
    }
}

// row index of every entry (warp per row)
__global__ void k_expand_rows(const long long *__restrict__ rp, int m, int *rowof)
{
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= m) return;
    for (long long q = rp[row] + lane; q < rp[row + 1]; q += 32) rowof[q] = row;
}

// column histogram -> transposed row lengths
__global__ void k_col_hist(const int *__restrict__ keys_sorted, long long nnz, int *len)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nnz; q += (long long)gridDim.x * blockDim.x)
        atomicAdd(&len[keys_sorted[q]], 1);
}

__global__ void k_gather_transposed(const int *__restrict__ perm, const int *__restrict__ rowof,
                                    const double *__restrict__ val, long long nnz, int *tcol, double *tval)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nnz; q += (long long)gridDim.x * blockDim.x) {
        int p = perm[q];
        tcol[q] = rowof[p];
        tval[q] = val[p];
    }
}

__global__ void k_i32_to_i64(const int *in, long long *out, long long n)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}

inline unsigned grid_for(long long n, int threads, long long cap = 152ll * 32) {
    long long g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// the wide kernel over the list; its work counter is the int after the
// list's length (wide_n[1]), zeroed here
template <class KS, bool FILL, bool MASK, typename TP>
cudaError_t launch_union_wide(Pool &pool, typename KS::Params P, const int *wide, int *wide_n, int *cnt,
                              int *stat, const TP *rowptr, int *out, uint16_t *mask)
{
    cudaError_t e = cudaMemsetAsync(wide_n + 1, 0, sizeof(int), pool.stream);
    if (e == cudaSuccess) {
        k_union_wide<KS, FILL, MASK, TP><<<WIDE_GRID, WIDE_THREADS, WIDE_SMEM, pool.stream>>>(P, wide, wide_n, cnt, stat,
                                                                                          rowptr, out, mask, wide_n + 1);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    return e;
}

// Count (+ scan into rowptr_out) and/or fill.  `wide` (nrows+2 ints: the
// list of rows too wide for one warp, its length, and the wide kernel's work
// counter) is written by the count pass and read by the fill pass, so the
// two may be separate calls.
template <class KS, typename TP>
cudaError_t union_structure(Pool &pool, typename KS::Params P, int nrows, int *cnt_scratch, int *wide,
                            TP *rowptr_out, int *out_cols, uint16_t *mask, int *flags, int *stat,
                            cudaError_t (*scan)(Pool &, const int *, TP *, long long, int *),
                            bool do_count, bool do_fill, int *defer = nullptr, int defer_S = 0)
{
    cudaStream_t s = pool.stream;
    int *wide_n = wide + nrows;
    cudaError_t e = cudaSuccess;
    const unsigned g = (unsigned)((nrows + WPC - 1) / WPC);
    if (do_count) {
        e = cudaMemsetAsync(wide_n, 0, sizeof(int), s);
        if (e != cudaSuccess) return e;
        if (nrows > 0) {
            { k_union_count<KS><<<g, WPC * 32, 0, s>>>(P, nrows, cnt_scratch, wide, wide_n, stat, defer,
                                                      defer ? defer + nrows : nullptr, defer_S); ::tsg::count_launch(); }
            e = launch_union_wide<KS, false, false, TP>(pool, P, wide, wide_n, cnt_scratch, stat, nullptr, nullptr,
                                                        nullptr);
        }
        if (e == cudaSuccess) e = scan(pool, cnt_scratch, rowptr_out, nrows, flags);
    }
    if (e == cudaSuccess && do_fill && nrows > 0 && out_cols) {
        if (mask) {
            { k_union_fill<KS, true, TP><<<g, WPC * 32, 0, s>>>(P, nrows, rowptr_out, out_cols, mask); ::tsg::count_launch(); }
            e = launch_union_wide<KS, true, true, TP>(pool, P, wide, wide_n, nullptr, nullptr, rowptr_out, out_cols, mask);
        } else {
            { k_union_fill<KS, false, TP><<<g, WPC * 32, 0, s>>>(P, nrows, rowptr_out, out_cols, nullptr); ::tsg::count_launch(); }
            e = launch_union_wide<KS, true, false, TP>(pool, P, wide, wide_n, nullptr, nullptr, rowptr_out, out_cols,
                                                       nullptr);
        }
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

template <class KS, bool FILL, bool MASK, typename TP>
cudaError_t set_wide_smem() {
    return cudaFuncSetAttribute(k_union_wide<KS, FILL, MASK, TP>, cudaFuncAttributeMaxDynamicSharedMemorySize, WIDE_SMEM);
}

}  // namespace

cudaError_t tiles_init_attributes()
{
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = set_wide_smem<CsrKeys, false, false, int>();
    if (e == cudaSuccess) e = set_wide_smem<CsrKeys, true, true, int>();
    if (e == cudaSuccess) e = set_wide_smem<CsrKeys, true, false, int>();
    if (e == cudaSuccess) e = set_wide_smem<UnionKeys, false, false, long long>();
    if (e == cudaSuccess) e = set_wide_smem<UnionKeys, true, false, long long>();
    if (e == cudaSuccess) e = set_wide_smem<UnionKeys, true, true, long long>();
    return e;
}

cudaError_t prepare_csr(Pool &pool, const void *rp, int rp_bits, const int *col, int m, int n, long long nnz,
                        long long *rp_out, int *flags, bool check_cols)
{
    cudaStream_t s = pool.stream;
    const int *cc = check_cols && nnz > 0 ? col : nullptr;
    // threads for every row pointer, and up to one per column index
    const unsigned g = std::max<unsigned>((unsigned)((m + 1 + 255) / 256), cc ? (unsigned)grid_for(nnz, 256) : 1u);
    if (rp_bits == 64) k_prepare_rowptr<long long><<<g, 256, 0, s>>>((const long long *)rp, m, nnz, rp_out, flags, cc, n);
    else k_prepare_rowptr<int><<<g, 256, 0, s>>>((const int *)rp, m, nnz, rp_out, flags, cc, n);
    ::tsg::count_launch();
    return cudaGetLastError();
}

// CSR -> tile structure (tile-row pointer, sorted tile columns, masks).
// T.trp/tcol/mask must be allocated by the caller (tcol, mask with an upper
// bound of the tile count: min(nnz, blkm*blkn)).
cudaError_t csr_to_tile_structure(Pool &pool, const long long *rp, const int *col, TileCSR &T, bool masks,
                                  int *flags, int *stat)
{
    int *cnt = pool.alloc_n<int>(T.blkm + 1);
    int *wide = pool.alloc_n<int>(T.blkm + 2);
    cudaError_t e = (cnt && wide) ? cudaSuccess : pool.err;
    CsrKeys::Params P{rp, col, T.m, T.n};
    if (e == cudaSuccess)
        e = union_structure<CsrKeys, int>(pool, P, T.blkm, cnt, wide, T.trp, T.tcol, masks ? T.mask : nullptr,
                                          flags, stat, scan_i32_to_i32, true, true);
    pool.free(cnt);
    pool.free(wide);
    return e;
}

// Step 1: C's tile-row pointer (crp, int64; count pass) and C's sorted tile
// columns (fill pass, ccol).  cnt and wide (blkm+1 and blkm+2 ints) carry state
// from the count pass to the fill pass; stat[0] gets the largest tile count
// of a tile-row and stat[1] the widest tile-column window.
// defer (blkm+1 ints, count pass only): the tile-rows the fused warp kernel
// leaves to the CTA step-2 kernel (too wide, or more than FUSED_MAX_TILES
// tiles), then their number; the caller zeroes defer[blkm] first.
namespace {

// Words of each tile-row's bitmap (0 for tile-rows wider than the narrow
// window, which never take the bitmap path).
__global__ void k_bitmap_words(const int *__restrict__ trp, const int *__restrict__ tcol, int blk, long long *nw)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= blk) return;
    const int t0 = trp[k], t1 = trp[k + 1];
    long long w = 0;
    if (t1 > t0) {
        const int lo = tcol[t0] & ~31, hi = tcol[t1 - 1];
        if (hi - lo < NW * 32) w = ((hi - lo) >> 5) + 1;
    }
    nw[k] = w;
}

// one warp per tile-row: set the bits of its tile columns (words zeroed before)
__global__ void k_bitmap_fill(const int *__restrict__ trp, const int *__restrict__ tcol, int blk,
                              const long long *__restrict__ bmoff, unsigned *bmw)
{
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= blk) return;
    const long long w0 = bmoff[k];
    if (bmoff[k + 1] == w0) return;
    const int t0 = trp[k], t1 = trp[k + 1];
    const int lo = tcol[t0] & ~31;
    for (int t = t0 + lane; t < t1; t += 32) {
        const int o = tcol[t] - lo;
        atomicOr(&bmw[w0 + (o >> 5)], 1u << (o & 31));
    }
}

}  // namespace

long long tile_bitmap_words_bound(const TileCSR &T)
{
    const long long per = std::min<long long>(NW + 1, (long long)T.blkn / 32 + 2);
    return (long long)T.blkm * per + 1;
}

cudaError_t tile_bitmaps(Pool &pool, TileCSR &T, long long *wcount, int *flags)
{
    cudaStream_t s = pool.stream;
    if (T.blkm <= 0) return cudaSuccess;
    { k_bitmap_words<<<(unsigned)((T.blkm + 255) / 256), 256, 0, s>>>(T.trp, T.tcol, T.blkm, wcount); ::tsg::count_launch(); }
    cudaError_t e = scan_i64_to_i64(pool, wcount, T.bmoff, T.blkm, flags);
    if (e == cudaSuccess) e = cudaMemsetAsync(T.bmw, 0, sizeof(unsigned) * (size_t)tile_bitmap_words_bound(T), s);
    if (e == cudaSuccess) { k_bitmap_fill<<<(unsigned)((T.blkm * 32LL + 255) / 256), 256, 0, s>>>(T.trp, T.tcol, T.blkm, T.bmoff, T.bmw); ::tsg::count_launch(); }
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

cudaError_t tile_symbolic(Pool &pool, const TileCSR &A, const TileCSR &B, long long *crp, int *ccol, int *cnt,
                          int *wide, int *flags, int *stat, bool count_pass, int *defer, unsigned *wbm, long long wpr)
{
    UnionKeys::Params P{A.trp, A.tcol, B.trp, B.tcol, B.bmoff, B.bmw, wbm, wpr};
    return union_structure<UnionKeys, long long>(pool, P, A.blkm, cnt, wide, crp, ccol, nullptr, flags, stat,
                                                 scan_i32_to_i64, count_pass, !count_pass, defer, FUSED_MAX_TILES);
}

// Step 1 fill and step 2 for the tile-rows one warp can hold (k_sym_fused),
// then the sorted tile columns of the wide tile-rows (their masks and counts
// come from step2_masks's CTA kernel).
cudaError_t symbolic_fill_fused(Pool &pool, const TileCSR &A, const TileCSR &B, int m, const long long *crp,
                                int *ccol, uint16_t *cmask, int *rowcnt, int *cnt, int *wide, int *flags,
                                const long long *erpB, const int *ecolB, const long long *erpA, const int *ecolA,
                                unsigned *wbm, long long wpr)
{
    cudaStream_t s = pool.stream;
    if (A.blkm <= 0) return cudaSuccess;
    UnionKeys::Params P{A.trp, A.tcol, B.trp, B.tcol, B.bmoff, B.bmw, wbm, wpr};
    // the kernel reads the 16 row masks of a tile at once: tile-major copies
    // of A's and B's masks (one copy when B is A)
    uint16_t *amT = pool.alloc_n<uint16_t>(A.cap * TILE + 16);
    uint16_t *bmT = (A.mask == B.mask) ? amT : pool.alloc_n<uint16_t>(B.cap * TILE + 16);
    cudaError_t e = (amT && bmT) ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = masks_to_tile_major_i32(pool, A.blkm, A.trp, A.mask, amT);
    if (e == cudaSuccess && bmT != amT) e = masks_to_tile_major_i32(pool, B.blkm, B.trp, B.mask, bmT);
    if (e == cudaSuccess) {
        k_sym_fused<<<(unsigned)((A.blkm + FWPC - 1) / FWPC), FWPC * 32, 0, s>>>(P, A.blkm, m, crp, ccol, amT, bmT,
                                                                           cmask, rowcnt, flags, erpB, ecolB, erpA, ecolA);
        ::tsg::count_launch();
        e = cudaGetLastError();
    }
    if (bmT && bmT != amT) pool.free(bmT);
    pool.free(amT);
    (void)cnt;
    if (e == cudaSuccess)
        e = launch_union_wide<UnionKeys, true, false, long long>(pool, P, wide, wide + A.blkm, nullptr, nullptr, crp, ccol,
                                                                 nullptr);
    return e;
}

cudaError_t masks_to_tile_major_i32(Pool &pool, int blkm, const int *rowptr, const uint16_t *src, uint16_t *dst)
{
    if (blkm <= 0) return cudaSuccess;
    { k_masks_to_tile_major<int><<<(unsigned)((blkm + 7) / 8), 256, 0, pool.stream>>>(blkm, rowptr, src, dst); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t masks_to_tile_major_i64(Pool &pool, int blkm, const long long *rowptr, const uint16_t *src, uint16_t *dst)
{
    if (blkm <= 0) return cudaSuccess;
    { k_masks_to_tile_major<long long><<<(unsigned)((blkm + 7) / 8), 256, 0, pool.stream>>>(blkm, rowptr, src, dst); ::tsg::count_launch(); }
    return cudaGetLastError();
}

// Stable CSR transpose: (tp, tcol, tval) = CSR of A^T (n x m).
cudaError_t csr_transpose(Pool &pool, const long long *rp, const int *col, const double *val, int m, int n,
                          long long nnz, long long *tp, int *tcol, double *tval, int *perm, int *flags)
{
    cudaStream_t s = pool.stream;
    cudaError_t e = cudaSuccess;
    int *len = pool.alloc_n<int>(n + 1);
    if (!len) return pool.err;
    if (nnz == 0) {
        e = cudaMemsetAsync(len, 0, sizeof(int) * (size_t)(n + 1), s);
        if (e == cudaSuccess) e = scan_i32_to_i64(pool, len, tp, n, flags);
        pool.free(len);
        return e;
    }
    int *k0 = pool.alloc_n<int>(nnz), *v0 = pool.alloc_n<int>(nnz);
    int *k1 = pool.alloc_n<int>(nnz), *v1 = pool.alloc_n<int>(nnz);
    int *rowof = pool.alloc_n<int>(nnz);
    const int nchunks = (int)((nnz + RADIX_CHUNK - 1) / RADIX_CHUNK);
    int *counts = pool.alloc_n<int>((long long)RADIX_BINS * nchunks + 1);
    if (!k0 || !v0 || !k1 || !v1 || !rowof || !counts) {
        e = pool.err ? pool.err : cudaErrorMemoryAllocation;
    } else {
        { k_iota_and_keys<<<grid_for(nnz, 256), 256, 0, s>>>(col, nnz, n, k0, v0); ::tsg::count_launch(); }
        int bits = 1;
        while (bits < 31 && (1ll << bits) < (long long)n) ++bits;
        for (int shift = 0; shift < bits && e == cudaSuccess; shift += RADIX_BITS) {
            { k_radix_hist<<<nchunks, RADIX_THREADS, 0, s>>>(k0, nnz, shift, nchunks, counts); ::tsg::count_launch(); }
            e = scan_i32_to_i32(pool, counts, counts, (long long)RADIX_BINS * nchunks, flags);
            if (e != cudaSuccess) break;
            { k_radix_scatter<<<nchunks, RADIX_THREADS, 0, s>>>(k0, v0, k1, v1, nnz, shift, nchunks, counts); ::tsg::count_launch(); }
            int *t = k0; k0 = k1; k1 = t;
            t = v0; v0 = v1; v1 = t;
        }
        if (e == cudaSuccess) {
            { k_expand_rows<<<(unsigned)((m + 7) / 8), 256, 0, s>>>(rp, m, rowof); ::tsg::count_launch(); }
            e = cudaMemsetAsync(len, 0, sizeof(int) * (size_t)(n + 1), s);
        }
        if (e == cudaSuccess) {
            { k_col_hist<<<grid_for(nnz, 256), 256, 0, s>>>(k0, nnz, len); ::tsg::count_launch(); }
            e = scan_i32_to_i64(pool, len, tp, n, flags);
        }
        if (e == cudaSuccess) {
            { k_gather_transposed<<<grid_for(nnz, 256), 256, 0, s>>>(v0, rowof, val, nnz, tcol, tval); ::tsg::count_launch(); }
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && perm)   // entry q of A^T is entry perm[q] of A
            e = cudaMemcpyAsync(perm, v0, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToDevice, s);
    }
    pool.free(k0); pool.free(v0); pool.free(k1); pool.free(v1);
    pool.free(rowof); pool.free(counts); pool.free(len);
    return e;
}

cudaError_t i32_to_i64(Pool &pool, const int *in, long long *out, long long n)
{
    if (n <= 0) return cudaSuccess;
    { k_i32_to_i64<<<(unsigned)((n + 255) / 256), 256, 0, pool.stream>>>(in, out, n); ::tsg::count_launch(); }
    return cudaGetLastError();
}

}  // namespace tsg
