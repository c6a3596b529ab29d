// tsg_numeric.cuh -- numeric-step bins shared by step 2 (which classifies
// C's tile-rows) and the numeric kernels.
#pragma once
#include "tsg_internal.cuh"

namespace tsg {

// Numeric bins of C's tile-rows (the nsparse-style binning of
// spgemm_nsparse_kernel.h:4-14 / the reference's tile bins at
// main_spgemm-col.cu:26-29, here chosen per tile-row by accumulator size):
enum NumericBin : int {
    BIN_EMPTY = 0,      // no entries
    BIN_SPARSE_S = 1,   // mask-rank accumulator in shared memory, <= SMEM_SMALL bytes
    BIN_SPARSE_M = 2,   // same, <= SMEM_MEDIUM bytes (two CTAs per SM)
    BIN_SPARSE_L = 3,   // same, <= SMEM_LARGE bytes (one CTA per SM)
    BIN_DENSE_S = 4,    // dense 16x16 tile accumulators in shared memory, <= SMEM_SMALL
    BIN_DENSE_M = 5,    // same, <= SMEM_MEDIUM
    BIN_DENSE_L = 6,    // same, <= SMEM_LARGE
    BIN_ROWS = 7,       // too large for one CTA: each of its rows is classed on its own (RowClass)
    NBIN = 8
};

// Classes of the rows of BIN_ROWS tile-rows; each class is one launch over a
// list of rows, so a few long rows set neither the shared memory nor the
// duration of the rest.
enum RowClass : int {
    ROW_S = 0,          // single-warp CTA, row accumulator in shared memory, <= ROWS_SMALL bytes
    ROW_M = 1,          // same, <= ROWS_MEDIUM bytes
    ROW_L = 2,          // ROW_WARPS warps per row, each a column range of it, <= SMEM_LARGE bytes
    ROW_WIDE = 3,       // accumulator in C's value array, ROW_WARPS warps over column windows
    ROW_WIDE1 = 4,      // accumulator in C's value array, one warp per row (rows_global)
    NROWCLS = 5
};
constexpr int ROW_WARPS = 8;

// C tile-rows whose masks the fused warp kernel builds (step 1 fill + step 2
// in one warp): tile-column window at most FUSED_MAX_SPAN, at most
// FUSED_MAX_TILES tiles.  The rest go to the CTA step-2 kernel.
constexpr int FUSED_MAX_SPAN = 4096;
constexpr int FUSED_MAX_TILES = 160;
__host__ __device__ inline bool fused_handles(long long span, long long S) {
    return span <= FUSED_MAX_SPAN && S <= FUSED_MAX_TILES;
}

constexpr long long SMEM_SMALL = 48 * 1024;
constexpr long long SMEM_MEDIUM = 100 * 1024;
constexpr long long SMEM_LARGE = 200 * 1024;
constexpr long long MAP_MAX = 8192;   // direct tile-column -> slot map when the window is this narrow
// size classes of the row kernels
constexpr long long ROWS_SMALL = 24 * 1024;
constexpr long long ROWS_MEDIUM = 64 * 1024;

struct NumericBinParams {
    int dense_tile_min;   // mean C-tile nnz at which a tile-row uses dense accumulators
    int smem_acc_max;     // largest tile-row (entries) accumulated in shared memory
    int row_acc_max;      // largest row (entries) accumulated in shared memory by the row kernel
    const long long *rpA; // A's row pointer (row classes weigh C's row against A's row)
    int rows_global;      // rows of the shared-memory row classes accumulate in C's values instead
};

__host__ __device__ inline long long align16(long long x) { return (x + 15) & ~15ll; }

// bytes of the tile-column -> slot map (uint16 entries, window rounded up to
// the 64-entry swizzle groups)
__host__ __device__ inline long long map_bytes(long long span) { return align16(((span + 63) & ~63ll) * 2); }

// Shared-memory layout of a tile-row in the numeric kernels:
//   int   scol[S]       C tile columns
//   u32   word[S*16]    (offset of the tile's row segment inside the tile-row << 16) | row mask
//   u16   map[span64]   tile column - scol[0] -> slot, swizzled (only when span <= MAP_MAX)
//   f64   acc[...]      nnz_tr entries rounded to 16, swizzled (sparse) or S*16*17 (dense, rows padded to 17),
//                       then 16 more: the first of them takes the updates of idle lanes
__host__ __device__ inline long long numeric_smem_bytes(long long S, long long nnz_tr, long long span, bool dense) {
    long long b = align16(S * 4) + align16(S * TILE * 4) + (span <= MAP_MAX ? map_bytes(span) : 0);
    return b + (dense ? S * TILE * 17 * 8 : ((nnz_tr + 15) & ~15ll) * 8) + TILE * 8;
}

// Shared-memory layout of one C row in the row kernel: word[S] (the row's
// packed words), then the map as above when the window is narrow, else the
// tile columns scol[S] (binary search), then acc[row nnz rounded to 16].
__host__ __device__ inline long long numeric_row_smem_bytes(long long S, long long row_nnz, long long span) {
    return align16(S * 4) + (span <= MAP_MAX ? map_bytes(span) : align16(S * 4)) + ((row_nnz + 15) & ~15ll) * 8;
}

// Bin of a C tile-row from its tile count S, entries nnz_tr and tile-column
// window span; req = its shared-memory bytes.
__host__ __device__ inline void numeric_classify(const NumericBinParams &bp, long long S, long long nnz_tr, long long span,
                                                 int &bin, long long &req) {
    req = 0;
    if (nnz_tr == 0) { bin = BIN_EMPTY; return; }
    const long long dreq = numeric_smem_bytes(S, nnz_tr, span, true);
    const long long sreq = numeric_smem_bytes(S, nnz_tr, span, false);
    if (nnz_tr >= (long long)bp.dense_tile_min * S && dreq <= SMEM_LARGE && nnz_tr < 65536) {
        bin = dreq <= SMEM_SMALL ? BIN_DENSE_S : dreq <= SMEM_MEDIUM ? BIN_DENSE_M : BIN_DENSE_L;
        req = dreq;
    } else if (nnz_tr <= bp.smem_acc_max && sreq <= SMEM_LARGE && nnz_tr < 65536) {
        bin = sreq <= SMEM_SMALL ? BIN_SPARSE_S : sreq <= SMEM_MEDIUM ? BIN_SPARSE_M : BIN_SPARSE_L;
        req = sreq;
    } else {
        bin = BIN_ROWS;
    }
}

// Rows this long, with this many entries per entry of A's row (so B's rows
// are long), go to the wide kernel: eight warps then share the row's
// products, each over its column range, while one warp would walk long B
// rows alone (measured faster on R-MAT A*A^T; rows of short B rows stay in
// shared memory).
constexpr long long WIDE_MIN_ROW = 1536;
constexpr long long WIDE_MIN_RATIO = 96;

// Class of one row of a BIN_ROWS tile-row (a_len: entries of A's row);
// req = its shared-memory bytes.
__host__ __device__ inline int numeric_row_class(const NumericBinParams &bp, long long S, long long row_nnz,
                                                 long long span, long long a_len, long long &req) {
    req = numeric_row_smem_bytes(S, row_nnz, span);
    const bool long_b = row_nnz >= WIDE_MIN_ROW && row_nnz >= WIDE_MIN_RATIO * a_len;
    if (row_nnz <= bp.row_acc_max && row_nnz < 65536 && !long_b) {
        if (req <= ROWS_MEDIUM) {
            if (bp.rows_global) { req = 0; return ROW_WIDE1; }
            return req <= ROWS_SMALL ? ROW_S : ROW_M;
        }
        if (req <= SMEM_LARGE) return ROW_L;
    }
    req = 0;
    return ROW_WIDE;
}

// Layout of the per-call bin statistics (device, then copied to the host):
// [0, NBIN) tile-rows per bin, [NBIN, 2 NBIN) largest shared memory per bin,
// then rows per row class and largest shared memory per row class.
constexpr int BS_ROWCNT = 2 * NBIN;
constexpr int BS_ROWREQ = 2 * NBIN + NROWCLS;
constexpr int BS_SLOTS = 2 * NBIN + 2 * NROWCLS;

// The record of one row R of a BIN_ROWS tile-row (one thread per row).
__device__ __forceinline__ void record_row(const NumericBinParams &bp, long long S, long long row_nnz, long long span,
                                           int R, int m, long long *binstat, int *rowlist) {
    if (row_nnz == 0) return;
    long long req;
    const int c = numeric_row_class(bp, S, row_nnz, span, bp.rpA[R + 1] - bp.rpA[R], req);
    const unsigned long long pos = atomicAdd((unsigned long long *)&binstat[BS_ROWCNT + c], 1ull);
    rowlist[(long long)c * m + (long long)pos] = R;
    if (req) atomicMax((long long *)&binstat[BS_ROWREQ + c], req);
}

struct NumericArgs {
    int m, blkm;
    const long long *rpA; const int *colA; const double *valA;
    const long long *rpB; const int *colB; const double *valB;
    const long long *crp; const int *ccol; const uint16_t *cmask;
    const long long *rowptrC; int *colC; double *valC;
    const unsigned char *bin;
    const int *binlist;   // tile-rows of bin b at binlist[b * blkm + 0 .. counts[b])
    const int *rowlist;   // rows of row class c at rowlist[c * m + 0 .. rowcounts[c])
    bool b_sorted;        // B's rows have strictly increasing columns (column-range searches allowed)
    const int *tr_coloff; // per tile-row, subtracted from the column indices written (batched products); may be null
    int *flags;
    long long nnzA;       // entries of A (bounds the wide rows' cut table)
    int n;                // columns of C
    bool cols_done;       // colC already written (numeric_cols): the kernels write values only
};

cudaError_t step2_masks(Pool &pool, const TileCSR &A, const TileCSR &B, int m, int blkm, const long long *crp,
                        const int *ccol, uint16_t *cmask, int *rowcnt, int max_tiles_per_row, int max_span,
                        int *flags, const int *defer_list, int ndefer, const long long *erpB,
                        const int *ecolB, const long long *erpA, const int *ecolA, bool b_sorted,
                        cudaStream_t side, cudaEvent_t fork, cudaEvent_t join);

// Launch the numeric kernels of every non-empty bin and row class.
// binstat is step 2's statistics (layout above), copied to the host.
// walk: 0 lanes over one B row per A entry, 1 packed (repeated B columns),
// 2 as 0 with B loads one step ahead (tile-row kernels); row_warps: warps
// per row for the shared-memory row classes ROW_S / ROW_M (1, 2 or 4)
// side/fork/join: a second stream and two events; with wide rows the other
// classes run there concurrently (side may be null: one stream)
// Column indices of every row of C from the masks (one warp per row), so
// that they can leave the device while the numeric kernels run; the numeric
// step then runs with a.cols_done set.
cudaError_t numeric_cols(Pool &pool, const NumericArgs &a);

cudaError_t numeric_run(Pool &pool, const NumericArgs &a, const long long *binstat, int walk, int threads,
                        int row_warps, cudaStream_t side = nullptr, cudaEvent_t fork = nullptr,
                        cudaEvent_t join = nullptr);

cudaError_t symbolic_fill_fused(Pool &pool, const TileCSR &A, const TileCSR &B, int m, const long long *crp,
                                int *ccol, uint16_t *cmask, int *rowcnt, int *cnt, int *wide, int *flags,
                                const long long *erpB, const int *ecolB, const long long *erpA, const int *ecolA,
                                unsigned *wbm, long long wpr);

// Numeric bins of C's tile-rows (bin[blkm], per-bin work lists and
// statistics in binstat, row classes of BIN_ROWS tile-rows in rowlist), from
// C's tile structure and row pointer once step 2 and its scan are done.
cudaError_t bin_tilerows(Pool &pool, int blkm, int m, const long long *crp, const int *ccol, const long long *rowptrC,
                         const NumericBinParams &bp, unsigned char *bin, long long *binstat, int *binlist, int *rowlist);
cudaError_t masks_to_tile_major_i32(Pool &pool, int blkm, const int *rowptr, const uint16_t *src, uint16_t *dst);
cudaError_t masks_to_tile_major_i64(Pool &pool, int blkm, const long long *rowptr, const uint16_t *src, uint16_t *dst);

cudaError_t symbolic_init_attributes();
cudaError_t numeric_init_attributes();

}  // namespace tsg
