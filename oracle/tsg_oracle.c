/*
 * tsg_oracle.c -- CPU oracle for the tiled FP64 SpGEMM path (C = A*B, A*A, A*A^T).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, not the product: only
 * tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py load
 * it.  The CUDA library under tilespgemm_gb300/ never calls into it and has no
 * CPU fallback.
 *
 * Every routine restates, in its own code, an algorithm of the reference
 * project YuyaoNiu/TileSpGEMM; the file:line it follows is given at each
 * function.  Parity of this restatement is pinned by tests/golden/ fixtures
 * generated from the reference's own C code (see tests/golden/make_golden.py).
 *
 * Conventions shared with the reference (common.h:30-32, main_spgemm-col.cu):
 *   - tiles are 16x16 (BLOCK_SIZE 16);
 *   - a tile's row mask has bit (15 - c) set for local column c
 *     (main_spgemm-col.cu:5215, :5331);
 *   - A's packed local index is (r << 4) | c (main_spgemm-col.cu:5214);
 *   - per-tile row pointers are 16 bytes; rows past the last real row of a
 *     partial tile-row are padded with the tile's total (:5225-5228).
 *
 * Index widths: CSR row pointers are int64 here (the product supports C with
 * more than 2^31 entries); column indices are int32; tile counts are int32.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TILE 16

/* ------------------------------------------------------------------------ */
/* 1. CSR Gustavson SpGEMM in the reference's accumulation order            */
/* ------------------------------------------------------------------------ */

/*
 * Row nnz of C = A*B (structural: an entry exists when any product lands on
 * it, even if the values cancel), following thmkl_dcsrmultcsr.c:12-41
 * (request == 1).  crp[0..m] receives the exclusive prefix (int64).
 */
int orc_spgemm_rownnz(int m, int n, const int64_t *arp, const int32_t *acol,
                      const int64_t *brp, const int32_t *bcol, int64_t *crp)
{
    int bad = 0;
#pragma omp parallel reduction(|:bad)
    {
        int64_t *stamp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
        for (int j = 0; j < n; ++j) stamp[j] = -1;
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < m; ++i) {
            int64_t cnt = 0;
            for (int64_t p = arp[i]; p < arp[i + 1]; ++p) {
                int k = acol[p];
                for (int64_t q = brp[k]; q < brp[k + 1]; ++q) {
                    int j = bcol[q];
                    if (j < 0 || j >= n) { bad = 1; continue; }
                    if (stamp[j] != i) { stamp[j] = i; ++cnt; }
                }
            }
            crp[i + 1] = cnt;
        }
        free(stamp);
    }
    crp[0] = 0;
    for (int i = 0; i < m; ++i) crp[i + 1] += crp[i];
    return bad ? -1 : 0;
}

static void sort_int_asc(int32_t *a, int64_t len)
{
    /* insertion sort for short runs, shell sort otherwise (no libc qsort
     * callback overhead, deterministic) */
    if (len < 48) {
        for (int64_t i = 1; i < len; ++i) {
            int32_t v = a[i];
            int64_t j = i - 1;
            while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
            a[j + 1] = v;
        }
        return;
    }
    int64_t gap = 1;
    while (gap < len / 3) gap = gap * 3 + 1;
    for (; gap > 0; gap /= 3)
        for (int64_t i = gap; i < len; ++i) {
            int32_t v = a[i];
            int64_t j = i;
            while (j >= gap && a[j - gap] > v) { a[j] = a[j - gap]; j -= gap; }
            a[j] = v;
        }
}

/*
 * Values of C = A*B into the structure from orc_spgemm_rownnz, following
 * thmkl_dcsrmultcsr.c:52-91 (request == 0): for row i, walk A's row in CSR
 * order, for each entry walk B's row in CSR order, accumulate into a dense
 * per-row accumulator, emit columns in ascending order.  Each product is one
 * fused multiply-add acc = fma(a, b, acc), the same rounding the CUDA path
 * uses, so for identical operand order the two agree bit for bit.
 * cbound (optional) receives sum |a||b| per entry, the scale of the
 * per-entry tolerance used by the tests.
 */
int orc_spgemm_fill(int m, int n, const int64_t *arp, const int32_t *acol, const double *aval,
                    const int64_t *brp, const int32_t *bcol, const double *bval,
                    const int64_t *crp, int32_t *ccol, double *cval, double *cbound)
{
#pragma omp parallel
    {
        int64_t *stamp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
        double *acc = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        double *bnd = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        for (int j = 0; j < n; ++j) stamp[j] = -1;
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < m; ++i) {
            int64_t base = crp[i], cnt = 0;
            for (int64_t p = arp[i]; p < arp[i + 1]; ++p) {
                int k = acol[p];
                double a = aval[p];
                for (int64_t q = brp[k]; q < brp[k + 1]; ++q) {
                    int j = bcol[q];
                    if (stamp[j] != i) {
                        stamp[j] = i;
                        acc[j] = 0.0;
                        bnd[j] = 0.0;
                        ccol[base + cnt++] = j;
                    }
                    acc[j] = fma(a, bval[q], acc[j]);
                    bnd[j] += fabs(a) * fabs(bval[q]);
                }
            }
            sort_int_asc(ccol + base, cnt);
            for (int64_t t = 0; t < cnt; ++t) {
                int j = ccol[base + t];
                cval[base + t] = acc[j];
                if (cbound) cbound[base + t] = bnd[j];
            }
        }
        free(stamp); free(acc); free(bnd);
    }
    return 0;
}

/*
 * Rows rows[0..nr) of C = A*B, computed exactly as orc_spgemm_rownnz and
 * orc_spgemm_fill compute them (thmkl_dcsrmultcsr.c:12-41, :52-91), for
 * checking a sample of rows of a product too large to compute whole on the
 * CPU.  With ccol == NULL, crp[0..nr] receives the exclusive prefix of the
 * listed rows' entry counts; otherwise row t's columns (ascending), values
 * and sum |a||b| bounds go to ccol/cval/cbound from crp[t].  Rows are taken
 * one at a time by the threads (a few hub rows can hold most of the work).
 * Returns -1 when a listed row or a B column is out of range.
 */
int orc_spgemm_rows(int nr, const int32_t *rows, int m, int n, const int64_t *arp, const int32_t *acol,
                    const double *aval, const int64_t *brp, const int32_t *bcol, const double *bval,
                    int64_t *crp, int32_t *ccol, double *cval, double *cbound)
{
    int bad = 0;
#pragma omp parallel reduction(|:bad)
    {
        int64_t *stamp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
        double *acc = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        double *bnd = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        for (int j = 0; j < n; ++j) stamp[j] = -1;
#pragma omp for schedule(dynamic, 1)
        for (int t = 0; t < nr; ++t) {
            const int i = rows[t];
            if (i < 0 || i >= m) { bad = 1; continue; }
            int64_t cnt = 0;
            const int64_t base = ccol ? crp[t] : 0;
            for (int64_t p = arp[i]; p < arp[i + 1]; ++p) {
                const int k = acol[p];
                const double a = aval ? aval[p] : 0.0;
                for (int64_t q = brp[k]; q < brp[k + 1]; ++q) {
                    const int j = bcol[q];
                    if (j < 0 || j >= n) { bad = 1; continue; }
                    if (stamp[j] != t) {
                        stamp[j] = t;
                        if (ccol) { acc[j] = 0.0; bnd[j] = 0.0; ccol[base + cnt] = j; }
                        ++cnt;
                    }
                    if (ccol) {
                        acc[j] = fma(a, bval[q], acc[j]);
                        bnd[j] += fabs(a) * fabs(bval[q]);
                    }
                }
            }
            if (!ccol) { crp[t + 1] = cnt; continue; }
            sort_int_asc(ccol + base, cnt);
            for (int64_t u = 0; u < cnt; ++u) {
                const int j = ccol[base + u];
                cval[base + u] = acc[j];
                if (cbound) cbound[base + u] = bnd[j];
            }
        }
        free(stamp); free(acc); free(bnd);
    }
    if (!ccol) {
        crp[0] = 0;
        for (int t = 0; t < nr; ++t) crp[t + 1] += crp[t];
    }
    return bad ? -1 : 0;
}

/*
 * Faithful restatement of thmkl_dcsrmultcsr (thmkl_dcsrmultcsr.c:7-95), the
 * reference's OpenMP CPU SpGEMM, kept for TIMING as the CPU baseline: per row
 * it allocates and clears dense flag (and value) arrays of length k (the
 * column count of C), which makes every row cost O(k).  int32 row pointers as
 * in the reference.  Rows [r0, r1) only, so that a bounded sample of a large
 * matrix can be timed; ic must hold r1 - r0 + 1 entries (relative pointers).
 * request == 1: symbolic (ic); request == 0: numeric (jc, c).
 */
void orc_thmkl_rows(int request, int r0, int r1, int k,
                    const double *a, const int32_t *ja, const int32_t *ia,
                    const double *b, const int32_t *jb, const int32_t *ib,
                    double *c, int32_t *jc, int32_t *ic)
{
    if (request == 1) {
#pragma omp parallel for
        for (int rid = r0; rid < r1; rid++) {
            int32_t *flag = (int32_t *)malloc((size_t)k * sizeof(int32_t));
            memset(flag, 0, (size_t)k * sizeof(int32_t));
            for (int32_t p = ia[rid]; p < ia[rid + 1]; p++) {
                int32_t rb = ja[p];
                for (int32_t q = ib[rb]; q < ib[rb + 1]; q++) flag[jb[q]] = 1;
            }
            int32_t nz = 0;
            for (int cc = 0; cc < k; cc++) nz += (flag[cc] == 1);
            ic[rid - r0] = nz;
            free(flag);
        }
        int32_t run = 0;
        for (int r = 0; r < r1 - r0; r++) { int32_t v = ic[r]; ic[r] = run; run += v; }
        ic[r1 - r0] = run;
    } else {
#pragma omp parallel for
        for (int rid = r0; rid < r1; rid++) {
            int32_t *flag = (int32_t *)malloc((size_t)k * sizeof(int32_t));
            double *dv = (double *)malloc((size_t)k * sizeof(double));
            memset(flag, 0, (size_t)k * sizeof(int32_t));
            memset(dv, 0, (size_t)k * sizeof(double));
            for (int32_t p = ia[rid]; p < ia[rid + 1]; p++) {
                int32_t rb = ja[p];
                double va = a[p];
                for (int32_t q = ib[rb]; q < ib[rb + 1]; q++) {
                    flag[jb[q]] = 1;
                    dv[jb[q]] += va * b[q];
                }
            }
            int32_t nz = 0, base = ic[rid - r0];
            for (int cc = 0; cc < k; cc++)
                if (flag[cc] == 1) { jc[base + nz] = cc; c[base + nz] = dv[cc]; nz++; }
            free(flag);
            free(dv);
        }
    }
}

/* Stable CSR -> CSC (= CSR of the transpose), following utils.h:158-195. */
void orc_transpose(int m, int n, const int64_t *rp, const int32_t *col, const double *val,
                   int64_t *tp, int32_t *trow, double *tval)
{
    memset(tp, 0, sizeof(int64_t) * (size_t)(n + 1));
    for (int64_t p = 0; p < rp[m]; ++p) tp[col[p] + 1]++;
    for (int j = 0; j < n; ++j) tp[j + 1] += tp[j];
    int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    memcpy(cur, tp, sizeof(int64_t) * (size_t)n);
    for (int i = 0; i < m; ++i)
        for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
            int64_t d = cur[col[p]]++;
            trow[d] = i;
            if (val && tval) tval[d] = val[p];
        }
    free(cur);
}

/* ------------------------------------------------------------------------ */
/* 2. CSR -> 16x16 tile conversion (tile-CSR), main_spgemm-col.cu:44-120,   */
/*    :4968-5240                                                             */
/* ------------------------------------------------------------------------ */

/*
 * Tile-row pointer of the tile-CSR form: number of distinct tile columns
 * touched by each tile-row (blocknnz / blkmessage, main_spgemm-col.cu:44-120).
 * blkrowptr has ceil(m/16)+1 entries.  Returns the tile count.
 */
int64_t orc_tile_rowptr(int m, int n, const int64_t *rp, const int32_t *col, int32_t *blkrowptr)
{
    int blkm = (m + TILE - 1) / TILE, blkn = (n + TILE - 1) / TILE;
    int32_t *stamp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(blkn > 0 ? blkn : 1));
    for (int j = 0; j < blkn; ++j) stamp[j] = -1;
    int64_t total = 0;
    blkrowptr[0] = 0;
    for (int bi = 0; bi < blkm; ++bi) {
        int r0 = bi * TILE, r1 = r0 + TILE < m ? r0 + TILE : m;
        int32_t cnt = 0;
        for (int64_t p = rp[r0]; p < rp[r1]; ++p) {
            int j = col[p] / TILE;
            if (stamp[j] != bi) { stamp[j] = bi; ++cnt; }
        }
        total += cnt;
        blkrowptr[bi + 1] = (int32_t)total;
    }
    free(stamp);
    return total;
}

/*
 * Fill the tile-CSR payload (main_spgemm-col.cu:4976-4985 for the sorted tile
 * column list, :5055-5085 for per-tile nnz offsets, :5130-5240 for the
 * payload).  Within a tile, entries are grouped by local row; inside a row
 * they keep CSR order.  Outputs (any payload pointer may be NULL):
 *   blkcolidx[numblk]   sorted tile columns per tile-row
 *   nnzb[numblk+1]      exclusive prefix of per-tile nnz
 *   ptr[16*numblk]      per-tile row starts (uint8), padded with the total
 *   idx[nnz]            packed (r<<4)|c         (A's form, :5214)
 *   lcol[nnz]           local column c          (the Col array, :5219)
 *   tval[nnz]           values in tile order
 *   mask[16*numblk]     bit 15-c per local row  (:5215)
 */
void orc_tile_fill(int m, int n, const int64_t *rp, const int32_t *col, const double *val,
                   const int32_t *blkrowptr, int32_t *blkcolidx, int32_t *nnzb,
                   uint8_t *ptr, uint8_t *idx, uint8_t *lcol, double *tval, uint16_t *mask)
{
    int blkm = (m + TILE - 1) / TILE, blkn = (n + TILE - 1) / TILE;
    int32_t *slot = (int32_t *)malloc(sizeof(int32_t) * (size_t)(blkn > 0 ? blkn : 1));
    int32_t *stamp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(blkn > 0 ? blkn : 1));
    for (int j = 0; j < blkn; ++j) stamp[j] = -1;
    int64_t numblk = blkrowptr[blkm];
    int32_t *cnt = (int32_t *)calloc((size_t)(numblk > 0 ? numblk : 1) * TILE, sizeof(int32_t));
    int32_t *cur = (int32_t *)calloc((size_t)(numblk > 0 ? numblk : 1), sizeof(int32_t));
    /* sorted tile columns */
    for (int bi = 0; bi < blkm; ++bi) {
        int r0 = bi * TILE, r1 = r0 + TILE < m ? r0 + TILE : m;
        int32_t b = blkrowptr[bi], w = b;
        for (int64_t p = rp[r0]; p < rp[r1]; ++p) {
            int j = col[p] / TILE;
            if (stamp[j] != bi) { stamp[j] = bi; blkcolidx[w++] = j; }
        }
        sort_int_asc(blkcolidx + b, w - b);
    }
    for (int j = 0; j < blkn; ++j) stamp[j] = -1;
    /* per (tile, local row) counts */
    for (int bi = 0; bi < blkm; ++bi) {
        int r0 = bi * TILE, r1 = r0 + TILE < m ? r0 + TILE : m;
        for (int32_t t = blkrowptr[bi]; t < blkrowptr[bi + 1]; ++t) {
            slot[blkcolidx[t]] = t;
            stamp[blkcolidx[t]] = bi;
        }
        for (int r = r0; r < r1; ++r)
            for (int64_t p = rp[r]; p < rp[r + 1]; ++p)
                cnt[(int64_t)slot[col[p] / TILE] * TILE + (r - r0)]++;
    }
    /* tile offsets and padded row starts */
    int64_t run = 0;
    for (int bi = 0; bi < blkm; ++bi) {
        int rows = (bi == blkm - 1) ? m - bi * TILE : TILE;
        for (int32_t t = blkrowptr[bi]; t < blkrowptr[bi + 1]; ++t) {
            nnzb[t] = (int32_t)run;
            int32_t in_tile = 0;
            for (int r = 0; r < TILE; ++r) {
                if (ptr) ptr[(int64_t)t * TILE + r] = (uint8_t)in_tile;  /* rows >= rows: padded */
                if (r < rows) in_tile += cnt[(int64_t)t * TILE + r];
            }
            run += in_tile;
        }
    }
    if (numblk >= 0) nnzb[numblk] = (int32_t)run;
    if (mask && numblk > 0) memset(mask, 0, sizeof(uint16_t) * (size_t)numblk * TILE);
    /* scatter in CSR order */
    for (int bi = 0; bi < blkm; ++bi) {
        int r0 = bi * TILE, r1 = r0 + TILE < m ? r0 + TILE : m;
        for (int32_t t = blkrowptr[bi]; t < blkrowptr[bi + 1]; ++t) {
            slot[blkcolidx[t]] = t;
            cur[t] = 0;
        }
        for (int r = r0; r < r1; ++r) {
            int lr = r - r0;
            for (int64_t p = rp[r]; p < rp[r + 1]; ++p) {
                int j = col[p] / TILE, c = col[p] - j * TILE;
                int32_t t = slot[j];
                int64_t d = (int64_t)nnzb[t] + (ptr ? ptr[(int64_t)t * TILE + lr] : 0) + cur[t];
                if (!ptr) {  /* compute row start without the ptr array */
                    int32_t s = 0;
                    for (int q = 0; q < lr; ++q) s += cnt[(int64_t)t * TILE + q];
                    d = (int64_t)nnzb[t] + s + cur[t];
                }
                cur[t]++;
                if (idx) idx[d] = (uint8_t)((lr << 4) | c);
                if (lcol) lcol[d] = (uint8_t)c;
                if (tval) tval[d] = val[p];
                if (mask) mask[(int64_t)t * TILE + lr] |= (uint16_t)(1u << (TILE - 1 - c));
            }
            /* rows are consumed in order, so reset the per-row cursor */
            for (int32_t t = blkrowptr[bi]; t < blkrowptr[bi + 1]; ++t) cur[t] = 0;
        }
    }
    free(slot); free(stamp); free(cnt); free(cur);
}

/*
 * B in the reference's tile-CSC form (main_spgemm-col.cu:5003-5040 for the
 * structure, :5086-5124 for per-tile nnz, :5242-5351 for the payload).  It is
 * the tile-CSR conversion of B's CSC (the transpose) with each tile
 * transposed back, so that inside a tile the entries are grouped by B's local
 * row with ascending local column.  Inputs: B's CSC (tp, trow, tval) with
 * kB = rows of B, nB = columns of B.  Outputs as orc_tile_fill, indexed in
 * tile-CSC order (tile-columns, each with tiles sorted by tile-row):
 * colptr[ceil(nB/16)+1], rowidx[numblk], nnzb, ptr (rows of B, padded with
 * the tile total), lcol (local column), tval, mask.
 */
void orc_tile_csc_fill(int kB, int nB, const int64_t *tp, const int32_t *trow, const double *tvalin,
                       const int32_t *colptr, int32_t *rowidx, int32_t *nnzb,
                       uint8_t *ptr, uint8_t *lcol, double *tval, uint16_t *mask)
{
    /* tile-CSR of B^T gives the structure and, per tile, entries grouped by
     * B's local column in CSC order; then regroup each tile by B's local row. */
    int64_t numblk = colptr[(nB + TILE - 1) / TILE];
    int64_t nnz = tp[nB];
    uint8_t *tptr = (uint8_t *)malloc((size_t)(numblk > 0 ? numblk : 1) * TILE);
    uint8_t *tidx = (uint8_t *)malloc((size_t)(nnz > 0 ? nnz : 1));
    double *tv = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    orc_tile_fill(nB, kB, tp, trow, tvalin, colptr, rowidx, nnzb, tptr, tidx, NULL, tv, NULL);
    if (mask && numblk > 0) memset(mask, 0, sizeof(uint16_t) * (size_t)numblk * TILE);
    int blkk = (kB + TILE - 1) / TILE;
    for (int64_t t = 0; t < numblk; ++t) {
        int32_t b = nnzb[t], e = nnzb[t + 1];
        int rows = (rowidx[t] == blkk - 1) ? kB - rowidx[t] * TILE : TILE;
        int32_t cnt[TILE + 1];
        memset(cnt, 0, sizeof(cnt));
        /* in tidx, the high nibble is B's local column, the low nibble B's local row */
        for (int32_t p = b; p < e; ++p) cnt[tidx[p] & 15]++;
        int32_t start[TILE], s = 0;
        for (int r = 0; r < TILE; ++r) {
            start[r] = s;
            if (ptr) ptr[t * TILE + r] = (uint8_t)s;
            if (r < rows) s += cnt[r];
        }
        /* stable by B's local column (the CSC order already walks columns in order) */
        for (int32_t p = b; p < e; ++p) {
            int r = tidx[p] & 15, c = tidx[p] >> 4;
            int32_t d = b + start[r]++;
            if (lcol) lcol[d] = (uint8_t)c;
            if (tval) tval[d] = tv[p];
            if (mask) mask[t * TILE + r] |= (uint16_t)(1u << (TILE - 1 - c));
        }
    }
    free(tptr); free(tidx); free(tv);
}

/* ------------------------------------------------------------------------ */
/* 3. Tile-level SpGEMM steps (the reference's CPU goldens)                 */
/* ------------------------------------------------------------------------ */

/*
 * C's tile structure: tile (i, j) exists when tile-row i of A and tile-column
 * j of B share a tile index (main_spgemm-col.cu:122-188 `step1` counts them,
 * :572-627 `step2` lists them in ascending j).  Restated as the union over
 * A's tiles (i, k) of B's tile-row k, which is the same set.  B is given in
 * tile-CSR (browptr, bcolidx).  blkrowptrC has blkmA+1 int64 entries;
 * when blkcolidxC is NULL only the pointer is produced.  Returns numblkC.
 */
int64_t orc_tile_symbolic(int blkmA, const int32_t *arowptr, const int32_t *acolidx,
                          int blknB, const int32_t *browptr, const int32_t *bcolidx,
                          int64_t *blkrowptrC, int32_t *blkcolidxC)
{
    uint8_t *flag = (uint8_t *)calloc((size_t)(blknB > 0 ? blknB : 1), 1);
    int64_t total = 0;
    blkrowptrC[0] = 0;
    for (int i = 0; i < blkmA; ++i) {
        for (int32_t p = arowptr[i]; p < arowptr[i + 1]; ++p) {
            int k = acolidx[p];
            for (int32_t q = browptr[k]; q < browptr[k + 1]; ++q) flag[bcolidx[q]] = 1;
        }
        for (int j = 0; j < blknB; ++j)
            if (flag[j]) {
                if (blkcolidxC) blkcolidxC[total] = j;
                ++total;
                flag[j] = 0;
            }
        blkrowptrC[i + 1] = total;
    }
    free(flag);
    return total;
}

/*
 * Per-tile structure and values of C (main_spgemm-col.cu:899-994 `step3` for
 * the per-tile nnz, :4073-4179 `step4` for column indices, row pointers and
 * values).  For tile (i, j) the matched pairs (A tile (i,k), B tile (k,j)) are
 * found by merging A's tile-row i with B's tile-column j (B in tile-CSC form),
 * products are accumulated into a dense 16x16 tile in pair order, then the
 * tile is compacted row by row in ascending local column.  Structurally empty
 * tiles (matched pairs whose element patterns do not meet) get nnz 0, mask 0
 * and row pointers 0.
 * Inputs: A tile-CSR payload (nnzbA, ptrA, lcolA, valA), B tile-CSC payload.
 * Outputs: nnzbC[numblkC+1] (exclusive prefix), maskC[16*numblkC],
 * ptrC[16*numblkC]; when colC/valC are non-NULL also the payload
 * (nnzbC must then already hold the prefix from a first call).
 * Returns nnzC.
 */
int64_t orc_tile_numeric(int mA, int blkmA, const int32_t *arowptr, const int32_t *acolidx,
                         const int32_t *nnzbA, const uint8_t *ptrA, const uint8_t *lcolA, const double *valA,
                         const int32_t *bcolptr, const int32_t *browidx,
                         const int32_t *nnzbB, const uint8_t *ptrB, const uint8_t *lcolB, const double *valB,
                         const int64_t *blkrowptrC, const int32_t *blkcolidxC,
                         int64_t *nnzbC, uint16_t *maskC, uint8_t *ptrC, uint8_t *colC, double *valC)
{
    int fill = (colC != NULL || valC != NULL);
    int64_t numblkC = blkrowptrC[blkmA];
    int64_t run = 0;
    for (int i = 0; i < blkmA; ++i) {
        int rows = (i == blkmA - 1) ? mA - i * TILE : TILE;
        for (int64_t t = blkrowptrC[i]; t < blkrowptrC[i + 1]; ++t) {
            int j = blkcolidxC[t];
            uint8_t hit[TILE * TILE];
            double acc[TILE * TILE];
            memset(hit, 0, sizeof(hit));
            memset(acc, 0, sizeof(acc));
            int32_t pa = arowptr[i], ea = arowptr[i + 1];
            int32_t pb = bcolptr[j], eb = bcolptr[j + 1];
            while (pa < ea && pb < eb) {
                int ka = acolidx[pa], kb = browidx[pb];
                if (ka < kb) { ++pa; continue; }
                if (kb < ka) { ++pb; continue; }
                for (int r = 0; r < rows; ++r) {
                    int32_t s = ptrA[(int64_t)pa * TILE + r];
                    int32_t e = (r == TILE - 1) ? nnzbA[pa + 1] - nnzbA[pa] : ptrA[(int64_t)pa * TILE + r + 1];
                    for (int32_t x = s; x < e; ++x) {
                        int c = lcolA[nnzbA[pa] + x];
                        double av = valA ? valA[nnzbA[pa] + x] : 0.0;
                        int32_t sb = ptrB[(int64_t)pb * TILE + c];
                        int32_t ebb = (c == TILE - 1) ? nnzbB[pb + 1] - nnzbB[pb] : ptrB[(int64_t)pb * TILE + c + 1];
                        for (int32_t y = sb; y < ebb; ++y) {
                            int cc = lcolB[nnzbB[pb] + y];
                            hit[r * TILE + cc] = 1;
                            if (fill && valA && valB) acc[r * TILE + cc] += av * valB[nnzbB[pb] + y];
                        }
                    }
                }
                ++pa; ++pb;
            }
            int64_t cnt = 0;
            for (int r = 0; r < TILE; ++r) {
                uint16_t mk = 0;
                if (ptrC) ptrC[t * TILE + r] = (uint8_t)cnt;
                for (int c = 0; c < TILE; ++c)
                    if (hit[r * TILE + c]) {
                        mk |= (uint16_t)(1u << (TILE - 1 - c));
                        if (fill) {
                            if (colC) colC[nnzbC[t] + cnt] = (uint8_t)c;
                            if (valC) valC[nnzbC[t] + cnt] = acc[r * TILE + c];
                        }
                        ++cnt;
                    }
                if (maskC) maskC[t * TILE + r] = mk;
            }
            if (!fill) nnzbC[t] = run;
            run += cnt;
        }
    }
    if (!fill) nnzbC[numblkC] = run;
    return run;
}

/*
 * Tile form of C -> CSR (the conversion the reference lacks; it is the
 * inverse of the tile fill above).  Row R = 16 i + r of C is the
 * concatenation, over C's tiles of tile-row i in ascending tile column, of
 * that tile's local row r.  crp must hold m+1 int64.
 */
void orc_tiles_to_csr(int m, int blkm, const int64_t *blkrowptrC, const int32_t *blkcolidxC,
                      const int64_t *nnzbC, const uint8_t *ptrC, const uint8_t *colC, const double *valC,
                      int64_t *crp, int32_t *ccol, double *cval)
{
    int64_t w = 0;
    crp[0] = 0;
    for (int i = 0; i < blkm; ++i) {
        int rows = (i == blkm - 1) ? m - i * TILE : TILE;
        for (int r = 0; r < rows; ++r) {
            for (int64_t t = blkrowptrC[i]; t < blkrowptrC[i + 1]; ++t) {
                int64_t s = ptrC[t * TILE + r];
                int64_t e = (r == TILE - 1) ? nnzbC[t + 1] - nnzbC[t] : ptrC[t * TILE + r + 1];
                if (e < s) e = s;  /* padded rows of a partial tile-row */
                for (int64_t x = s; x < e; ++x) {
                    if (ccol) ccol[w] = blkcolidxC[t] * TILE + colC[nnzbC[t] + x];
                    if (cval) cval[w] = valC[nnzbC[t] + x];
                    ++w;
                }
            }
            crp[i * TILE + r + 1] = w;
        }
    }
}

/* Intermediate-product count nnzCub = sum over A's entries (i,k) of nnz(B row k)
 * (main_spgemm-col.cu:4949-4957). */
int64_t orc_nnzcub(int m, const int64_t *arp, const int32_t *acol, const int64_t *brp)
{
    int64_t s = 0;
    for (int64_t p = 0; p < arp[m]; ++p) s += brp[acol[p] + 1] - brp[acol[p]];
    return s;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int t)
{
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}
