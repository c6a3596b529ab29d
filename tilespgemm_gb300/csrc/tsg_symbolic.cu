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

namespace tsg {

namespace {

constexpr int S2_THREADS = 256;
constexpr int S2_WARPS = S2_THREADS / 32;

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

// GLOBAL = false: masks accumulate in shared memory (tile-rows with at most
// `smax` tiles); GLOBAL = true: in cmask with global atomics (the rest).
template <bool GLOBAL>
__global__ void __launch_bounds__(S2_THREADS)
k_step2(int blkm, int m, const int *__restrict__ arp, const int *__restrict__ acol,
        const uint16_t *__restrict__ amask, const int *__restrict__ brp, const int *__restrict__ bcol,
        const uint16_t *__restrict__ bmask, const long long *__restrict__ crp, const int *__restrict__ ccol,
        uint16_t *cmask, int *rowcnt, int smax, NumericBinParams bp, unsigned char *bin,
        long long *binstat, int *flags)
{
    extern __shared__ unsigned s_dyn[];
    __shared__ int s_rows[S2_WARPS][TILE];
    __shared__ unsigned s_rmask[S2_WARPS][TILE];
    __shared__ long long s_rowtot[TILE];
    const int i = blockIdx.x;
    if (i >= blkm) return;
    const long long c0 = crp[i];
    const int S = (int)(crp[i + 1] - c0);
    if (GLOBAL ? (S <= smax) : (S > smax)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned *smask = s_dyn;                                   // S*16 (shared path)
    const int *scol = GLOBAL ? (ccol + c0) : reinterpret_cast<const int *>(s_dyn + S * TILE);
    if (!GLOBAL) {
        int *wcol = reinterpret_cast<int *>(s_dyn + S * TILE);
        for (int t = tid; t < S * TILE; t += S2_THREADS) smask[t] = 0u;
        for (int t = tid; t < S; t += S2_THREADS) wcol[t] = ccol[c0 + t];
    } else {
        unsigned *mw = reinterpret_cast<unsigned *>(cmask) + c0 * 8;
        for (long long t = tid; t < (long long)S * 8; t += S2_THREADS) mw[t] = 0u;
    }
    if (tid < TILE) s_rowtot[tid] = 0;
    __syncthreads();

    const int a0 = arp[i], a1 = arp[i + 1];
    for (int a = a0 + warp; a < a1; a += S2_WARPS) {
        const int kt = acol[a];
        const int q0 = brp[kt], nq = brp[kt + 1] - q0;
        // compact the nonzero rows of A tile a
        unsigned ma = (lane < TILE) ? amask[(long long)a * TILE + lane] : 0u;
        unsigned nzr = __ballot_sync(0xffffffffu, ma != 0u);
        if (ma) {
            int pos = __popc(nzr & lanemask_lt());
            s_rows[warp][pos] = lane;
            s_rmask[warp][pos] = ma;
        }
        __syncwarp();
        const int nrow = __popc(nzr);
        const int total = nrow * nq;
        for (int idx = lane; idx < total; idx += 32) {
            const int t = idx / nq;
            const long long q = q0 + (idx - t * nq);
            const int r = s_rows[warp][t];
            unsigned acc = or_rows(s_rmask[warp][t], bmask, q);
            if (acc) {
                const int key = bcol[q];
                const int s = lower_bound_i(scol, S, key);
                if (s >= S || scol[s] != key) { set_flag(flags, FLAG_INTERNAL); continue; }
                if (GLOBAL) atomic_or_mask16(cmask, (c0 + s) * TILE + r, acc);
                else atomicOr(&smask[s * TILE + r], acc);
            }
        }
        __syncwarp();
    }
    __syncthreads();
    if (GLOBAL) __threadfence();

    const int rows = min(TILE, m - i * TILE);
    // write masks (shared path) and count rows
    if (!GLOBAL) {
        unsigned *mw = reinterpret_cast<unsigned *>(cmask) + c0 * 8;
        for (int t = tid; t < S * 8; t += S2_THREADS)
            mw[t] = (smask[2 * t] & 0xffffu) | (smask[2 * t + 1] << 16);
    }
    for (int r = warp; r < TILE; r += S2_WARPS) {
        int c = 0;
        for (int s = lane; s < S; s += 32) {
            unsigned mk = GLOBAL ? (unsigned)__ldcg(cmask + (c0 + s) * TILE + r) : smask[s * TILE + r];
            c += __popc(mk & 0xffffu);
        }
        c = warp_sum_int(c);
        if (lane == 0) {
            if (r < rows) rowcnt[i * TILE + r] = c;
            s_rowtot[r] = c;
        }
    }
    __syncthreads();
    if (tid == 0) {
        long long nnz_tr = 0;
        for (int r = 0; r < TILE; ++r) nnz_tr += s_rowtot[r];
        const long long span = S > 0 ? (long long)scol[S - 1] - scol[0] + 1 : 0;
        int b;
        long long req = 0;
        numeric_classify(bp, S, nnz_tr, span, b, req);
        bin[i] = (unsigned char)b;
        atomicAdd((unsigned long long *)&binstat[b], 1ull);
        atomicMax((long long *)&binstat[NBIN + b], req);
    }
}

}  // namespace

cudaError_t symbolic_init_attributes()
{
    return cudaFuncSetAttribute(k_step2<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2048 * (TILE * 4 + 4) + 16);
}

cudaError_t step2_masks(Pool &pool, const TileCSR &A, const TileCSR &B, int m, int blkm, const long long *crp,
                        const int *ccol, uint16_t *cmask, int *rowcnt, int max_tiles_per_row,
                        const NumericBinParams &bp, unsigned char *bin, long long *binstat, int *flags)
{
    cudaStream_t s = pool.stream;
    if (blkm <= 0) return cudaSuccess;
    // shared path: up to `smax` tiles per tile-row, (16*4 + 4) bytes per tile
    const int smax = 2048;
    const int s_used = max_tiles_per_row < smax ? max_tiles_per_row : smax;
    const size_t smem = (size_t)s_used * (TILE * 4 + 4) + 16;
    { k_step2<false><<<blkm, S2_THREADS, smem, s>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol, B.mask, crp, ccol,
                                                   cmask, rowcnt, smax, bp, bin, binstat, flags); ::tsg::count_launch(); }
    if (max_tiles_per_row > smax)
        { k_step2<true><<<blkm, S2_THREADS, 0, s>>>(blkm, m, A.trp, A.tcol, A.mask, B.trp, B.tcol, B.mask, crp, ccol,
                                                   cmask, rowcnt, smax, bp, bin, binstat, flags); ::tsg::count_launch(); }
    return cudaGetLastError();
}

}  // namespace tsg
