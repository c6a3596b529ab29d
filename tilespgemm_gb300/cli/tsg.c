/*
 * tsg -- command-line front end of libtilespgemm with the interface of the
 * reference's driver (main_spgemm-col.cu:4821-5577, run as
 * `./test -d <dev> <A.mtx>`), written in plain C against include/tilespgemm.h
 * only.
 *
 *   tsg -d <device> [--aat] [--keep-values] [--repeat R] [--csv FILE] A.mtx
 *
 * Like the reference it loads A (tsg_load_mtx, the semantics of
 * mmio_allinone), overwrites A's values with i % 10 (main_spgemm-col.cu:
 * 4895-4896; --keep-values keeps the file's), refuses A*A on a non-square A
 * and A*A^T on a symmetric A (:4887-4891, :4917-4921), counts the
 * intermediate products nnzCub (:4949-4957), runs the SpGEMM R times (20,
 * REPEAT_NUM) on A resident on the device, takes the minimum time (:4777-
 * 4785), and appends
 *   filename,rowA,colA,nnzA,nnzCub,nnzC,compression_rate,time_ms,gflops
 * to results_tile.csv (:5554-5559) with gflops = 2 nnzCub / time (:4787)
 * and compression_rate = nnzCub / nnzC (:4782).  The reference picks A*A or
 * A*A^T at compile time (`#define AAT`, :24); here it is --aat.  Its timed
 * region starts from tile arrays already on the device and stops before
 * tile -> CSR; here it covers the whole CSR-in, CSR-out call with A on the
 * device (tsg_csr_to_device) and C left there.
 *
 * Exit status: 0 after a run or after a refusal the reference also makes
 * (it returns 0 there too), 1 on a library error (message on stderr), 2 on
 * bad arguments.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "tilespgemm.h"

#define REPEAT_DEFAULT 20

static double now_ms(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static int usage(const char *prog)
{
    fprintf(stderr, "Run the code by '%s -d 0 [--aat] [--keep-values] [--repeat R] [--csv FILE] matrix.mtx'.\n", prog);
    return 2;
}

static int lib_error(const char *what)
{
    fprintf(stderr, "%s: %s\n", what, tsg_last_error());
    return 1;
}

int main(int argc, char **argv)
{
    int device_id = 0, aat = 0, keep_values = 0, repeat = REPEAT_DEFAULT, have_dev = 0;
    const char *filename = NULL, *csv = "results_tile.csv";
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "-d") && i + 1 < argc) { device_id = atoi(argv[++i]); have_dev = 1; }
        else if (!strcmp(argv[i], "--aat")) aat = 1;
        else if (!strcmp(argv[i], "--keep-values")) keep_values = 1;
        else if (!strcmp(argv[i], "--repeat") && i + 1 < argc) repeat = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--csv") && i + 1 < argc) csv = argv[++i];
        else if (argv[i][0] == '-') return usage(argv[0]);
        else filename = argv[i];
    }
    if (!have_dev || !filename || repeat < 1) return usage(argv[0]);
    printf("device_id = %i\n", device_id);
    printf("MAT: -------------- %s --------------\n", filename);

    tsg_csr A;
    memset(&A, 0, sizeof(A));
    int32_t symmetric = 0;
    const double t0 = now_ms();
    if (tsg_load_mtx(filename, &A, &symmetric) != TSG_OK) return lib_error("loading the matrix");
    printf("input matrix A: ( %i, %i ) nnz = %lld\n loadfile time    = %4.5f sec\n", A.m, A.n, (long long)A.nnz,
           (now_ms() - t0) / 1000.0);
    if (!aat && A.m != A.n) {
        printf("matrix squaring must have rowA == colA. Exit.\n");
        tsg_csr_free(NULL, &A);
        return 0;
    }
    if (aat && A.m == A.n && symmetric) {
        printf("matrix AAT does not do symmetric matrix. Exit.\n");
        tsg_csr_free(NULL, &A);
        return 0;
    }
    if (!keep_values)
        for (int64_t i = 0; i < A.nnz; ++i) A.val[i] = (double)(i % 10);

    tsg_ctx *ctx = NULL;
    if (tsg_create(&ctx, device_id, NULL) != TSG_OK) {
        tsg_csr_free(NULL, &A);
        return lib_error("creating the context");
    }
    int rc = 0;
    tsg_csr Ad;
    memset(&Ad, 0, sizeof(Ad));
    const tsg_op op = aat ? TSG_OP_AAT : TSG_OP_AA;
    double best = -1.0;
    long long nnz_cub = 0, nnz_c = 0;
    if (tsg_csr_to_device(ctx, &A, &Ad) != TSG_OK) { rc = lib_error("uploading A"); goto done; }
    for (int r = 0; r < repeat; ++r) {
        tsg_csr C;
        memset(&C, 0, sizeof(C));
        C.where = TSG_MEM_DEVICE;
        tsg_stats st;
        const double t1 = now_ms();
        if (tsg_spgemm(ctx, op, &Ad, NULL, &C, &st) != TSG_OK) { rc = lib_error("SpGEMM"); goto done; }
        const double ms = now_ms() - t1;   /* the call returns with C complete */
        nnz_cub = st.nnz_cub;
        nnz_c = C.nnz;
        if (best < 0.0 || ms < best) best = ms;
        tsg_csr_free(ctx, &C);
    }
    {
        const double gflops = 2.0 * (double)nnz_cub / (best * 1e6);
        const double compression = nnz_c > 0 ? (double)nnz_cub / (double)nnz_c : 0.0;
        printf("SpGEMM nnzCub = %lld\n", nnz_cub);
        printf("%s C = A*A%s: nnzC = %lld, compression rate = %.3f, min of %d runs = %.3f ms, gflops = %.2f\n",
               filename, aat ? "^T" : "", nnz_c, compression, repeat, best, gflops);
        FILE *fout = fopen(csv, "a");
        if (fout == NULL) {
            printf("Writing results fails.\n");
        } else {
            fprintf(fout, "%s,%i,%i,%lld,%lld,%lld,%f,%f,%f\n", filename, A.m, A.n, (long long)A.nnz, nnz_cub, nnz_c,
                    compression, best, gflops);
            fclose(fout);
        }
    }
done:
    tsg_csr_free(ctx, &Ad);
    tsg_destroy(ctx);
    tsg_csr_free(NULL, &A);
    return rc;
}
