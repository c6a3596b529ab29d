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
    BIN_SPARSE_L = 2,   // same, <= SMEM_LARGE bytes (one CTA per SM)
    BIN_DENSE_S = 3,    // dense 16x16 tile accumulators in shared memory, <= SMEM_SMALL
    BIN_DENSE_L = 4,    // same, <= SMEM_LARGE
    BIN_ROWS_S = 5,     // one warp (CTA) per C row, the row's accumulator in shared memory, <= ROWS_SMALL bytes
    BIN_ROWS_M = 6,     // same, <= ROWS_MEDIUM bytes
    BIN_ROWS_L = 7,     // same, <= SMEM_LARGE bytes
    BIN_GLOBAL = 8,     // accumulator in C's value array (any size)
    NBIN = 9
};

// C tile-rows whose masks the fused warp kernel builds (step 1 fill + step 2
// in one warp): tile-column window at most FUSED_MAX_SPAN, at most
// FUSED_MAX_TILES tiles.  The rest go to the CTA step-2 kernel.
constexpr int FUSED_MAX_SPAN = 4096;
constexpr int FUSED_MAX_TILES = 160;
__host__ __device__ inline bool fused_handles(long long span, long long S) {
    return span <= FUSED_MAX_SPAN && S <= FUSED_MAX_TILES;
}

constexpr long long SMEM_SMALL = 48 * 1024;
constexpr long long SMEM_LARGE = 200 * 1024;
constexpr long long MAP_MAX = 8192;   // direct tile-column -> slot map when the window is this narrow
// size classes of the one-row-per-CTA kernel (each class is one launch, so a
// few large rows do not set the shared memory, and the occupancy, of all)
constexpr long long ROWS_SMALL = 24 * 1024;
constexpr long long ROWS_MEDIUM = 64 * 1024;

struct NumericBinParams {
    int dense_tile_min;   // mean C-tile nnz at which a tile-row uses dense accumulators
    int smem_acc_max;     // largest tile-row (entries) accumulated in shared memory
    int row_acc_max;      // largest row (entries) accumulated in shared memory by the row kernel
};

__host__ __device__ inline long long align16(long long x) { return (x + 15) & ~15ll; }

// bytes of the tile-column -> slot map (uint16 entries, window rounded up to
// the 64-entry swizzle groups)
__host__ __device__ inline long long map_bytes(long long span) { return align16(((span + 63) & ~63ll) * 2); }

// Shared-memory layout of a tile-row in the numeric kernels:
//   int   scol[S]       C tile columns
//   u32   word[S*16]    (offset of the tile's row segment inside the tile-row << 16) | row mask
//   u16   map[span64]   tile column - scol[0] -> slot, swizzled (only when span <= MAP_MAX)
//   f64   acc[...]      nnz_tr entries rounded to 16, swizzled (sparse) or S*16*17 (dense, rows padded to 17)
__host__ __device__ inline long long numeric_smem_bytes(long long S, long long nnz_tr, long long span, bool dense) {
    long long b = align16(S * 4) + align16(S * TILE * 4) + (span <= MAP_MAX ? map_bytes(span) : 0);
    return b + (dense ? S * TILE * 17 * 8 : ((nnz_tr + 15) & ~15ll) * 8);
}

// Shared-memory layout of one C row in the row kernel: word[S] (the row's
// packed words), then the map as above when the window is narrow, else the
// tile columns scol[S] (binary search), then acc[row nnz rounded to 16].
__host__ __device__ inline long long numeric_row_smem_bytes(long long S, long long row_nnz, long long span) {
    return align16(S * 4) + (span <= MAP_MAX ? map_bytes(span) : align16(S * 4)) + ((row_nnz + 15) & ~15ll) * 8;
}

// Bin of a C tile-row from its tile count S, entries nnz_tr, tile-column
// window span and largest row max_row; req = its shared-memory bytes.
__host__ __device__ inline void numeric_classify(const NumericBinParams &bp, long long S, long long nnz_tr, long long span,
                                                 long long max_row, int &bin, long long &req) {
    req = 0;
    if (nnz_tr == 0) { bin = BIN_EMPTY; return; }
    const long long dreq = numeric_smem_bytes(S, nnz_tr, span, true);
    const long long sreq = numeric_smem_bytes(S, nnz_tr, span, false);
    if (nnz_tr >= (long long)bp.dense_tile_min * S && dreq <= SMEM_LARGE && nnz_tr < 65536) {
        bin = dreq <= SMEM_SMALL ? BIN_DENSE_S : BIN_DENSE_L;
        req = dreq;
    } else if (nnz_tr <= bp.smem_acc_max && sreq <= SMEM_LARGE && nnz_tr < 65536) {
        bin = sreq <= SMEM_SMALL ? BIN_SPARSE_S : BIN_SPARSE_L;
        req = sreq;
    } else if (max_row <= bp.row_acc_max && numeric_row_smem_bytes(S, max_row, span) <= SMEM_LARGE &&
               max_row < 65536) {
        req = numeric_row_smem_bytes(S, max_row, span);
        bin = req <= ROWS_SMALL ? BIN_ROWS_S : (req <= ROWS_MEDIUM ? BIN_ROWS_M : BIN_ROWS_L);
    } else {
        bin = BIN_GLOBAL;
    }
}

struct NumericArgs {
    int m, blkm;
    const long long *rpA; const int *colA; const double *valA;
    const long long *rpB; const int *colB; const double *valB;
    const long long *crp; const int *ccol; const uint16_t *cmask;
    const long long *rowptrC; int *colC; double *valC;
    const unsigned char *bin;
    const int *binlist;   // tile-rows of bin b at binlist[b * blkm + 0 .. counts[b])
    const int *tr_coloff; // per tile-row, subtracted from the column indices written (batched products); may be null
    int *flags;
};

cudaError_t step2_masks(Pool &pool, const TileCSR &A, const TileCSR &B, int m, int blkm, const long long *crp,
                        const int *ccol, uint16_t *cmask, int *rowcnt, int max_tiles_per_row, int max_span,
                        const NumericBinParams &bp, unsigned char *bin, long long *binstat, int *binlist,
                        int *flags, const int *defer_list, int ndefer, const long long *erpB, const int *ecolB);

// Launch the numeric kernels of every non-empty bin.  counts/req are the
// per-bin tile-row counts and maximum shared-memory sizes from step 2.
cudaError_t numeric_run(Pool &pool, const NumericArgs &a, const long long *counts, const long long *req,
                        bool dupsafe, int threads);

cudaError_t symbolic_fill_fused(Pool &pool, const TileCSR &A, const TileCSR &B, int m, const long long *crp,
                                int *ccol, uint16_t *cmask, int *rowcnt, unsigned char *bin,
                                const NumericBinParams &bp, long long *binstat, int *binlist, int *cnt, int *wide,
                                int *flags, const long long *erpB, const int *ecolB);
cudaError_t masks_to_tile_major_i32(Pool &pool, int blkm, const int *rowptr, const uint16_t *src, uint16_t *dst);
cudaError_t masks_to_tile_major_i64(Pool &pool, int blkm, const long long *rowptr, const uint16_t *src, uint16_t *dst);

cudaError_t symbolic_init_attributes();
cudaError_t numeric_init_attributes();

}  // namespace tsg
