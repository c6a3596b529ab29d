// tsg_aux.cu -- small reductions used by the pipeline, and the conversions
// between CSR and the reference's tile format:
//   tiles_payload_a   CSR -> tile payload (nnz offsets, uint8 row starts,
//                     local columns, values) in the layout of the reference's
//                     host conversion main_spgemm-col.cu:5055-5240
//   tiles_from_csr_c  C's CSR + tile masks -> C's tile payload, the layout
//                     stepall_cuda_new leaves on the device (:4586-4735)
//   csr_from_tiles    any tile matrix -> CSR (the tile -> CSR output)
// Roofline: all HBM-bound copies/gathers (read once, write once).
#include "tsg_internal.cuh"

namespace tsg {

namespace {

__device__ __forceinline__ int lower_bound_aux(const int *a, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void k_nnzcub(const long long *__restrict__ rpA, const int *__restrict__ colA, int m,
                         const long long *__restrict__ rpB, int kB, unsigned long long *out)
{
    __shared__ unsigned long long s[8];
    unsigned long long acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        for (long long p = rpA[i]; p < rpA[i + 1]; ++p) {
            int k = colA[p];
            if ((unsigned)k < (unsigned)kB) acc += (unsigned long long)(rpB[k + 1] - rpB[k]);
        }
    acc = (unsigned long long)warp_sum_ll((long long)acc);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        atomicAdd(out, t);
    }
}

__global__ void k_mask_popc(const int *__restrict__ trp, int blkm, const uint16_t *__restrict__ mask,
                            unsigned long long *out)
{
    const long long nt = trp[blkm];
    const unsigned *mw = reinterpret_cast<const unsigned *>(mask);
    unsigned long long acc = 0;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nt * 8; w += (long long)gridDim.x * blockDim.x)
        acc += __popc(mw[w]);
    acc = (unsigned long long)warp_sum_ll((long long)acc);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// Is every row's column sequence strictly increasing?  Pass 1 marks the
// first entry of every non-empty row in a bitmap over the entries; pass 2
// compares each entry with the next unless the next starts a row, and
// counts the descents (coalesced over the entries).
__global__ void k_mark_row_starts(const long long *__restrict__ rp, int m, unsigned *starts)
{
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R < m; R += (long long)gridDim.x * blockDim.x) {
        const long long p = rp[R];
        if (rp[R + 1] > p) atomicOr(&starts[p >> 5], 1u << (p & 31));
    }
}

// pairs (q, q+1) inside one row with col[q] >= col[q+1]; each thread takes
// DESC_PER consecutive pairs, so the warp's reduction is paid once per
// DESC_PER entries (one per entry took 65 us on 23 M entries)
constexpr int DESC_PER = 8;
__global__ void k_count_descents(const int *__restrict__ col, long long nnz, const unsigned *__restrict__ starts,
                                 unsigned long long *out)
{
    unsigned long long cnt = 0;
    const long long stride = (long long)gridDim.x * blockDim.x * DESC_PER;
    for (long long q0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * DESC_PER; q0 + 1 < nnz; q0 += stride) {
        int prev = col[q0];
#pragma unroll
        for (int j = 1; j <= DESC_PER; ++j) {
            const long long n1 = q0 + j;
            if (n1 < nnz) {
                const int cur = col[n1];
                if (!((starts[n1 >> 5] >> (n1 & 31)) & 1u) && prev >= cur) ++cnt;
                prev = cur;
            }
        }
    }
    cnt = (unsigned long long)warp_sum_ll((long long)cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(out, cnt);
}

__global__ void k_copy_scalars(const long long *a, long long *da, const int *b, long long *db, const int *c, long long *dc)
{
    if (threadIdx.x == 0) { *da = *a; *db = *b; *dc = *c; }
}

__global__ void k_rowptr_narrow(const long long *in, int *out, long long n)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int)in[i];
}

// ---- C tiles from C's CSR ------------------------------------------------

// per-tile nnz of C from its row-major masks (warp per tile-row)
__global__ void k_tile_nnz_rm(int blkm, const long long *__restrict__ crp, const uint16_t *__restrict__ cmask, int *tn)
{
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= blkm) return;
    const long long c0 = crp[i];
    const int S = (int)(crp[i + 1] - c0);
    for (int s = lane; s < S; s += 32) {
        int c = 0;
        for (int r = 0; r < TILE; ++r) c += __popc((unsigned)cmask[c0 * TILE + (long long)r * S + s]);
        tn[c0 + s] = c;
    }
}

// one CTA per C tile-row; warp per row, lanes over the tile-row's tiles
__global__ void __launch_bounds__(256)
k_tile_payload_c(int m, const long long *__restrict__ crp, const int *__restrict__ ccol,
                 const uint16_t *__restrict__ cmask, const long long *__restrict__ rowptr,
                 const int *__restrict__ col, const double *__restrict__ val, const long long *__restrict__ nnzb,
                 uint8_t *ptr, uint8_t *lcol, double *tval)
{
    const int i = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = i * TILE, rows = min(TILE, m - r0);
    const long long c0 = crp[i];
    const int S = (int)(crp[i + 1] - c0);
    const uint16_t *mk_rm = cmask + c0 * TILE;     // row r of tile s at mk_rm[r*S + s]
    // row starts inside each tile
    for (int s = threadIdx.x; s < S; s += blockDim.x) {
        int run = 0;
        for (int r = 0; r < TILE; ++r) {
            ptr[(c0 + s) * TILE + r] = (uint8_t)run;
            run += __popc((unsigned)mk_rm[r * S + s]);
        }
    }
    for (int r = warp; r < rows; r += 8) {
        const long long Rb = rowptr[r0 + r];
        int run = 0;
        for (int sb = 0; sb < S; sb += 32) {
            const int s = sb + lane;
            unsigned mk = (s < S) ? (unsigned)mk_rm[r * S + s] : 0u;
            int c = __popc(mk);
            int incl = warp_incl_scan(c, lane);
            if (s < S && c) {
                int before = 0;
                for (int q = 0; q < r; ++q) before += __popc((unsigned)mk_rm[q * S + s]);
                const long long src = Rb + run + incl - c;
                const long long dst = nnzb[c0 + s] + before;
                for (int x = 0; x < c; ++x) {
                    lcol[dst + x] = (uint8_t)(col[src + x] & 15);
                    tval[dst + x] = val[src + x];
                }
            }
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

// ---- A's tile payload ------------------------------------------------------

// per (tile, local row) entry counts; warp per CSR row
__global__ void k_a_counts(int m, const long long *__restrict__ rp, const int *__restrict__ col, int n,
                           const int *__restrict__ trp, const int *__restrict__ tcol, int *cnt16)
{
    const int R = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (R >= m) return;
    const int i = R / TILE, r = R - i * TILE;
    const int t0 = trp[i], S = trp[i + 1] - t0;
    for (long long p = rp[R] + lane; p < rp[R + 1]; p += 32) {
        int c = col[p];
        if ((unsigned)c >= (unsigned)n) continue;
        int s = lower_bound_aux(tcol + t0, S, c >> 4);
        atomicAdd(&cnt16[(long long)(t0 + s) * TILE + r], 1);
    }
}

__global__ void k_a_ptr(long long numblk, int blkm, const int *__restrict__ trp, const int *__restrict__ cnt16,
                        int *tn, uint8_t *ptr, int m, int *flags)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < numblk; t += (long long)gridDim.x * blockDim.x) {
        int run = 0;
        for (int r = 0; r < TILE; ++r) {
            if (run > 255) set_flag(flags, FLAG_OVERFLOW);
            ptr[t * TILE + r] = (uint8_t)run;
            run += cnt16[t * TILE + r];
        }
        tn[t] = run;
    }
    (void)blkm; (void)trp; (void)m;
}

// scatter in CSR order; a warp owns a row, so per-(tile,row) cursors advance
// deterministically
__global__ void k_a_scatter(int m, const long long *__restrict__ rp, const int *__restrict__ col,
                            const double *__restrict__ val, int n, const int *__restrict__ trp,
                            const int *__restrict__ tcol, const long long *__restrict__ nnzb,
                            const uint8_t *__restrict__ ptr, int *cur16, uint8_t *lcol, double *tval)
{
    const int R = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (R >= m) return;
    const int i = R / TILE, r = R - i * TILE;
    const int t0 = trp[i], S = trp[i + 1] - t0;
    for (long long pb = rp[R]; pb < rp[R + 1]; pb += 32) {
        const long long p = pb + lane;
        const bool ok = p < rp[R + 1];
        int c = ok ? col[p] : -1;
        const bool valid = ok && (unsigned)c < (unsigned)n;
        int t = valid ? t0 + lower_bound_aux(tcol + t0, S, c >> 4) : -1 - lane;
        unsigned peers = __match_any_sync(0xffffffffu, t);
        int rank = __popc(peers & lanemask_lt());
        int before = valid ? cur16[(long long)t * TILE + r] : 0;
        __syncwarp();
        if (valid) {
            long long dst = nnzb[t] + ptr[(long long)t * TILE + r] + before + rank;
            lcol[dst] = (uint8_t)(c & 15);
            tval[dst] = val[p];
            if (lane == __ffs(peers) - 1) cur16[(long long)t * TILE + r] = before + __popc(peers);
        }
        __syncwarp();
    }
}

// ---- tiles -> CSR ----------------------------------------------------------

__device__ __forceinline__ int tile_row_len(const uint8_t *ptr, const long long *nnzb, long long t, int r) {
    int s = ptr[t * TILE + r];
    int e = (r == TILE - 1) ? (int)(nnzb[t + 1] - nnzb[t]) : ptr[t * TILE + r + 1];
    return e > s ? e - s : 0;
}

// y = T x on the tile form (the consumer the reference's CCSB SpMV is,
// ccsb_spmv.h:11-252): one warp per tile-row, a lane pair per row, each lane
// of the pair taking every other entry of the row's segment in each tile;
// the tile's 16 entries of x are staged in shared memory.
__global__ void __launch_bounds__(256)
k_tiles_spmv(int m, int blkm, const long long *__restrict__ brp, const int *__restrict__ bcol,
             const long long *__restrict__ nnzb, const uint8_t *__restrict__ ptr, const uint8_t *__restrict__ lcol,
             const double *__restrict__ tval, const double *__restrict__ x, int n, double *y)
{
    __shared__ double s_x[8][TILE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * 8 + warp;
    if (i >= blkm) return;
    const int r = lane >> 1, half = lane & 1;
    double sum = 0.0;
    for (long long t = brp[i]; t < brp[i + 1]; ++t) {
        const int jb = bcol[t] * TILE;
        if (lane < TILE) s_x[warp][lane] = (jb + lane < n) ? x[jb + lane] : 0.0;
        __syncwarp();
        const long long base = nnzb[t];
        const int s = ptr[t * TILE + r];
        const int e = (r == TILE - 1) ? (int)(nnzb[t + 1] - base) : ptr[t * TILE + r + 1];
        for (int q = s + half; q < e; q += 2) sum = fma(tval[base + q], s_x[warp][lcol[base + q] & 15], sum);
        __syncwarp();
    }
    sum += __shfl_xor_sync(0xffffffffu, sum, 1);
    const int R = i * TILE + r;
    if (half == 0 && R < m) y[R] = sum;
}

__global__ void k_csr_rowcnt_from_tiles(int m, const long long *__restrict__ brp, const long long *__restrict__ nnzb,
                                        const uint8_t *__restrict__ ptr, int *rowcnt)
{
    const int R = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (R >= m) return;
    const int i = R / TILE, r = R - i * TILE;
    int c = 0;
    for (long long t = brp[i] + lane; t < brp[i + 1]; t += 32) c += tile_row_len(ptr, nnzb, t, r);
    c = warp_sum_int(c);
    if (lane == 0) rowcnt[R] = c;
}

__global__ void k_csr_fill_from_tiles(int m, const long long *__restrict__ brp, const int *__restrict__ bcol,
                                      const long long *__restrict__ nnzb, const uint8_t *__restrict__ ptr,
                                      const uint8_t *__restrict__ lcol, const double *__restrict__ tval,
                                      const long long *__restrict__ rowptr, int *col, double *val)
{
    const int R = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (R >= m) return;
    const int i = R / TILE, r = R - i * TILE;
    long long run = rowptr[R];
    for (long long tb = brp[i]; tb < brp[i + 1]; tb += 32) {
        const long long t = tb + lane;
        int len = (t < brp[i + 1]) ? tile_row_len(ptr, nnzb, t, r) : 0;
        int incl = warp_incl_scan(len, lane);
        if (len) {
            const long long src = nnzb[t] + ptr[t * TILE + r];
            const long long dst = run + incl - len;
            const int jb = bcol[t] * TILE;
            for (int x = 0; x < len; ++x) {
                col[dst + x] = jb + lcol[src + x];
                val[dst + x] = tval[src + x];
            }
        }
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
}

// FP64 FMA throughput probe: 8 independent FMA chains per thread (the
// operands keep the values finite); nothing but DFMA in the loop.
__global__ void __launch_bounds__(256) k_fp64_peak(double *out, int iters, double a, double b)
{
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_gather(const int *__restrict__ perm, const double *__restrict__ src, double *dst, long long n)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        dst[q] = src[perm[q]];
}

// ---- batched products: block-diagonal packing -----------------------------

// gridDim.y CTAs per instance (blockIdx.x): shifted row pointer (padding
// rows repeat the end), shifted columns, copied values; row pointers and
// columns are validated
__global__ void __launch_bounds__(256)
k_batch_pack(const PackDesc *__restrict__ descs, long long *rp, int *col, double *val, int *flags)
{
    const PackDesc d = descs[blockIdx.x];
    const long long t0 = (long long)blockIdx.y * blockDim.x + threadIdx.x, ts = (long long)gridDim.y * blockDim.x;
    bool bad = false;
    for (long long r = t0; r < d.rowpad; r += ts) {
        long long v;
        if (r < d.m) {
            v = d.rp_bits == 64 ? ((const long long *)d.rp)[r] : (long long)((const int *)d.rp)[r];
            const long long nx = d.rp_bits == 64 ? ((const long long *)d.rp)[r + 1] : (long long)((const int *)d.rp)[r + 1];
            if (v < 0 || nx < v || nx > d.nnz || (r == 0 && v != 0)) bad = true;
            v = v < 0 ? 0 : (v > d.nnz ? d.nnz : v);
        } else {
            v = d.nnz;
        }
        rp[d.rowoff + r] = d.nnzoff + v;
    }
    if (t0 == 0 && d.m > 0) {
        const long long last = d.rp_bits == 64 ? ((const long long *)d.rp)[d.m] : (long long)((const int *)d.rp)[d.m];
        if (last != d.nnz) bad = true;
    }
    for (long long q = t0; q < d.nnz; q += ts) {
        int c = d.col[q];
        if ((unsigned)c >= (unsigned)d.n) { bad = true; c = 0; }
        col[d.nnzoff + q] = (int)(c + d.coloff);
        if (d.val) val[d.nnzoff + q] = d.val[q];
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) set_flag(flags, FLAG_BAD_INPUT);
}

// one CTA per instance: C_i's row pointer rebased to 0 and its first entry
template <typename TR>
__global__ void __launch_bounds__(256)
k_batch_unpack(const UnpackDesc *__restrict__ descs, const long long *__restrict__ rowptrC, TR *rp_out,
               long long *ebase)
{
    const UnpackDesc d = descs[blockIdx.x];
    const long long e0 = rowptrC[d.rowoff];
    if (threadIdx.x == 0) ebase[blockIdx.x] = e0;
    for (long long r = threadIdx.x; r <= d.m; r += blockDim.x) rp_out[d.rpoff + r] = (TR)(rowptrC[d.rowoff + r] - e0);
}

inline unsigned g256(long long n) {
    long long g = (n + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152ll * 64) g = 152ll * 64;
    return (unsigned)g;
}

}  // namespace

cudaError_t fp64_peak(cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, double *gflops)
{
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = sms * 8, threads = 256, iters = 2000;
    double *out = nullptr;
    e = cudaMallocAsync(&out, sizeof(double) * blocks * threads, s);
    if (e != cudaSuccess) return e;
    double best = 0.0;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
        cudaEventRecord(e0, s);
        { k_fp64_peak<<<blocks, threads, 0, s>>>(out, iters, 1.0000001, 1e-9); ::tsg::count_launch(); }
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        const double flop = 2.0 * 8.0 * iters * (double)blocks * threads;
        if (rep > 0 && ms > 0.f) best = best > flop / (ms * 1e6) ? best : flop / (ms * 1e6);
    }
    cudaFreeAsync(out, s);
    cudaStreamSynchronize(s);
    *gflops = best;
    return e;
}

cudaError_t aux_nnzcub(Pool &pool, const long long *rpA, const int *colA, int m, const long long *rpB, int kB,
                       unsigned long long *out)
{
    if (m <= 0) return cudaSuccess;
    { k_nnzcub<<<g256(m), 256, 0, pool.stream>>>(rpA, colA, m, rpB, kB, out); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t aux_rows_increasing(Pool &pool, const long long *rp, const int *col, int m, long long nnz,
                                unsigned long long *out)
{
    if (m <= 0 || nnz <= 1) return cudaSuccess;
    const long long words = (nnz + 31) / 32 + 1;
    unsigned *starts = pool.alloc_n<unsigned>(words);
    if (!starts) return pool.err;
    cudaError_t e = cudaMemsetAsync(starts, 0, sizeof(unsigned) * (size_t)words, pool.stream);
    if (e == cudaSuccess) { k_mark_row_starts<<<g256(m), 256, 0, pool.stream>>>(rp, m, starts); ::tsg::count_launch(); }
    if (e == cudaSuccess) { k_count_descents<<<g256((nnz + DESC_PER - 1) / DESC_PER), 256, 0, pool.stream>>>(col, nnz, starts, out); ::tsg::count_launch(); }
    if (e == cudaSuccess) e = cudaGetLastError();
    pool.free(starts);
    return e;
}

cudaError_t aux_mask_popc(Pool &pool, const int *trp, int blkm, const uint16_t *mask, unsigned long long *out)
{
    { k_mask_popc<<<152 * 4, 256, 0, pool.stream>>>(trp, blkm, mask, out); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t aux_copy_scalars(Pool &pool, const long long *a, long long *da, const int *b, long long *db,
                             const int *c, long long *dc)
{
    { k_copy_scalars<<<1, 32, 0, pool.stream>>>(a, da, b, db, c, dc); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t aux_gather(Pool &pool, const int *perm, const double *src, double *dst, long long n)
{
    if (n <= 0) return cudaSuccess;
    { k_gather<<<g256(n), 256, 0, pool.stream>>>(perm, src, dst, n); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t batch_pack(Pool &pool, const PackDesc *d_desc, int count, int per, long long *rp, int *col, double *val,
                       int *flags)
{
    if (count <= 0) return cudaSuccess;
    const dim3 grid((unsigned)count, (unsigned)(per < 1 ? 1 : per));
    { k_batch_pack<<<grid, 256, 0, pool.stream>>>(d_desc, rp, col, val, flags); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t batch_unpack(Pool &pool, const UnpackDesc *d_desc, int count, const long long *rowptrC, void *rp_out,
                         int rp_bits, long long *ebase)
{
    if (count <= 0) return cudaSuccess;
    if (rp_bits == 64) { k_batch_unpack<long long><<<count, 256, 0, pool.stream>>>(d_desc, rowptrC, (long long *)rp_out, ebase); ::tsg::count_launch(); }
    else { k_batch_unpack<int><<<count, 256, 0, pool.stream>>>(d_desc, rowptrC, (int *)rp_out, ebase); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t aux_rowptr_narrow(Pool &pool, const long long *in, int *out, long long n)
{
    if (n <= 0) return cudaSuccess;
    { k_rowptr_narrow<<<(unsigned)((n + 255) / 256), 256, 0, pool.stream>>>(in, out, n); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t tiles_from_csr_c(Pool &pool, int m, int blkm, long long numblk, const long long *crp, const int *ccol,
                             const uint16_t *cmask, const long long *rowptr, const int *col, const double *val,
                             long long *nnzb, uint8_t *ptr, uint8_t *lcol, double *tval, int *flags)
{
    int *tn = pool.alloc_n<int>(numblk + 1);
    if (!tn) return pool.err;
    if (blkm > 0) { k_tile_nnz_rm<<<(unsigned)((blkm + 7) / 8), 256, 0, pool.stream>>>(blkm, crp, cmask, tn); ::tsg::count_launch(); }
    cudaError_t e = scan_i32_to_i64(pool, tn, nnzb, numblk, flags);
    if (e == cudaSuccess && blkm > 0)
        { k_tile_payload_c<<<blkm, 256, 0, pool.stream>>>(m, crp, ccol, cmask, rowptr, col, val, nnzb, ptr, lcol, tval); ::tsg::count_launch(); }
    if (e == cudaSuccess) e = cudaGetLastError();
    pool.free(tn);
    return e;
}

cudaError_t tiles_payload_a(Pool &pool, int m, int n, const long long *rp, const int *col, const double *val,
                            const TileCSR &T, long long numblk, long long *nnzb, uint8_t *ptr, uint8_t *lcol,
                            double *tval, int *flags)
{
    int *cnt16 = pool.alloc_n<int>(numblk * TILE + 1);
    int *cur16 = pool.alloc_n<int>(numblk * TILE + 1);
    int *tn = pool.alloc_n<int>(numblk + 1);
    cudaError_t e = (cnt16 && cur16 && tn) ? cudaSuccess : pool.err;
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt16, 0, sizeof(int) * (size_t)(numblk * TILE + 1), pool.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(cur16, 0, sizeof(int) * (size_t)(numblk * TILE + 1), pool.stream);
    const unsigned gr = (unsigned)((m + 7) / 8);
    if (e == cudaSuccess && m > 0) { k_a_counts<<<gr, 256, 0, pool.stream>>>(m, rp, col, n, T.trp, T.tcol, cnt16); ::tsg::count_launch(); }
    if (e == cudaSuccess && numblk > 0) { k_a_ptr<<<g256(numblk), 256, 0, pool.stream>>>(numblk, T.blkm, T.trp, cnt16, tn, ptr, m, flags); ::tsg::count_launch(); }
    if (e == cudaSuccess) e = scan_i32_to_i64(pool, tn, nnzb, numblk, flags);
    if (e == cudaSuccess && m > 0)
        { k_a_scatter<<<gr, 256, 0, pool.stream>>>(m, rp, col, val, n, T.trp, T.tcol, nnzb, ptr, cur16, lcol, tval); ::tsg::count_launch(); }
    if (e == cudaSuccess) e = cudaGetLastError();
    pool.free(cnt16); pool.free(cur16); pool.free(tn);
    return e;
}

// The two passes of csr_from_tiles as separate launches on `s`, into
// caller-provided row counts (m entries) and outputs; they allocate nothing.
cudaError_t csr_rowcnt_from_tiles(cudaStream_t s, int m, const long long *brp, const long long *nnzb,
                                  const uint8_t *ptr, int *rowcnt)
{
    if (m > 0) { k_csr_rowcnt_from_tiles<<<(unsigned)((m + 7) / 8), 256, 0, s>>>(m, brp, nnzb, ptr, rowcnt); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t csr_fill_from_tiles(cudaStream_t s, int m, const long long *brp, const int *bcol, const long long *nnzb,
                                const uint8_t *ptr, const uint8_t *lcol, const double *tval, const long long *rowptr,
                                int *col, double *val)
{
    if (m > 0) { k_csr_fill_from_tiles<<<(unsigned)((m + 7) / 8), 256, 0, s>>>(m, brp, bcol, nnzb, ptr, lcol, tval, rowptr, col, val); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t tiles_spmv(cudaStream_t s, int m, int blkm, const long long *brp, const int *bcol, const long long *nnzb,
                       const uint8_t *ptr, const uint8_t *lcol, const double *tval, const double *x, int n, double *y)
{
    if (blkm > 0) { k_tiles_spmv<<<(unsigned)((blkm + 7) / 8), 256, 0, s>>>(m, blkm, brp, bcol, nnzb, ptr, lcol, tval, x, n, y); ::tsg::count_launch(); }
    return cudaGetLastError();
}

cudaError_t csr_from_tiles(Pool &pool, int m, const long long *brp, const int *bcol, const long long *nnzb,
                           const uint8_t *ptr, const uint8_t *lcol, const double *tval, long long *rowptr, int *col,
                           double *val, int *flags, bool fill)
{
    const unsigned gr = (unsigned)((m + 7) / 8);
    if (!fill) {
        int *rowcnt = pool.alloc_n<int>(m + 1);
        if (!rowcnt) return pool.err;
        if (m > 0) { k_csr_rowcnt_from_tiles<<<gr, 256, 0, pool.stream>>>(m, brp, nnzb, ptr, rowcnt); ::tsg::count_launch(); }
        cudaError_t e = scan_i32_to_i64(pool, rowcnt, rowptr, m, flags);
        pool.free(rowcnt);
        return e;
    }
    if (m > 0) { k_csr_fill_from_tiles<<<gr, 256, 0, pool.stream>>>(m, brp, bcol, nnzb, ptr, lcol, tval, rowptr, col, val); ::tsg::count_launch(); }
    return cudaGetLastError();
}

}  // namespace tsg
