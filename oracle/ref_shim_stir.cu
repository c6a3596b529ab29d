/*
 * ref_shim_stir.cu -- TEST INFRASTRUCTURE ONLY (builds the reference, never shipped).
 *
 * Compiles the reference project's active source file (main_spgemm-col.cu of
 * YuyaoNiu/TileSpGEMM, taken unmodified from the reference checkout via the
 * include path) and exposes its host-side CPU golden routines with C linkage,
 * so that tests/golden/make_golden.py can call them through ctypes:
 *   blocknnz / blkmessage  main_spgemm-col.cu:44-120  (tile-row pointer, tile columns)
 *   quick_sort_key         utils.h:134-155
 *   matrix_transposition   utils.h:158-195  (CSR -> CSC; B = A^T for A*A^T)
 *   step1 / step2          main_spgemm-col.cu:122-188, :572-627  (C tile structure)
 *   step3 / step4          main_spgemm-col.cu:899-994, :4073-4179 (C tile nnz, payload)
 *   mmio_allinone          mmio_highlevel.h:593-759  (Matrix Market load path)
 *   mm_write_mtx_crd       mmio.h:780-850  (Matrix Market writer; real general here)
 * The reference's main() is renamed by the build recipe and never runs.
 */
#include "main_spgemm-col.cu"

extern "C" {
void ref_blocknnz(int *rbnum, int *cbnum, int *col, int *rowptr, int m, int n, int *blknnz)
{ blocknnz(rbnum, cbnum, col, rowptr, m, n, blknnz); }
void ref_blkmessage(int *rbnum, int *cbnum, int *col, int *rowptr, int m, int n, int *blkrowptr, int *blkcolidx)
{ blkmessage(rbnum, cbnum, col, rowptr, m, n, blkrowptr, blkcolidx); }
void ref_quick_sort_key(int *key, int len) { quick_sort_key(key, len); }
void ref_matrix_transposition(int m, int n, int nnz, int *rp, int *col, double *val, int *trow, int *tp, double *tval)
{ matrix_transposition(m, n, nnz, rp, col, val, trow, tp, tval); }
void ref_step1(int *arp, int *aci, int blkmA, int blknA, int *bcp, int *bri, int blkmB, int blknB, int *crp, int *numblkC)
{ step1(arp, aci, blkmA, blknA, bcp, bri, blkmB, blknB, crp, numblkC); }
void ref_step2(int *arp, int *aci, int blkmA, int blknA, int *bcp, int *bri, int blkmB, int blknB, int *crp, int *cci)
{ step2(arp, aci, blkmA, blknA, bcp, bri, blkmB, blknB, crp, cci); }
void ref_step3(int *arp, int *aci, int blkmA, int blknA, int *nnzbA, int mA,
               double *valA, unsigned char *colA, unsigned char *ptrA,
               int *bcp, int *bri, int blkmB, int blknB, int *nnzbB,
               double *valB, unsigned char *colB, unsigned char *ptrB,
               int *crp, int *cci, int *nnzbC, int *nnzC)
{ step3(arp, aci, blkmA, blknA, nnzbA, mA, valA, colA, ptrA, bcp, bri, blkmB, blknB, nnzbB, valB, colB, ptrB, crp, cci, nnzbC, nnzC); }
void ref_step4(int *arp, int *aci, int blkmA, int blknA, int *nnzbA, int mA,
               double *valA, unsigned char *colA, unsigned char *ptrA,
               int *bcp, int *bri, int blkmB, int blknB, int *nnzbB,
               double *valB, unsigned char *colB, unsigned char *ptrB,
               int *crp, int *cci, int *nnzbC, double *valC, unsigned char *colC, unsigned char *ptrC)
{ step4(arp, aci, blkmA, blknA, nnzbA, mA, valA, colA, ptrA, bcp, bri, blkmB, blknB, nnzbB, valB, colB, ptrB, crp, cci, nnzbC, valC, colC, ptrC); }
int ref_mmio_allinone(int *m, int *n, int *nnz, int *isSym, int **rp, int **col, double **val, char *fn)
{ return mmio_allinone(m, n, nnz, isSym, rp, col, val, fn); }
void ref_free(void *p) { free(p); }
int ref_mm_write_mtx_crd(char *fn, int M, int N, int nz, int *I, int *J, double *val)
{
    MM_typecode code;
    mm_initialize_typecode(&code);
    mm_set_matrix(&code);
    mm_set_coordinate(&code);
    mm_set_real(&code);
    mm_set_general(&code);
    return mm_write_mtx_crd(fn, M, N, nz, I, J, val, code);
}
}
