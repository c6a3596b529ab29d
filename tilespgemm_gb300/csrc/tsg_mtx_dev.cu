// tsg_mtx_dev.cu -- Matrix Market data lines parsed on the device
// (tsg_load_mtx_device), with the semantics of the host loader and of the
// reference's mmio_allinone (mmio_highlevel.h:593-759): one entry per data
// line, blank lines skipped, 1-based indices, pattern -> 1.0, integer ->
// (double)(int), complex -> real part; symmetric / hermitian files mirrored
// (the diagonal once), each row in file order with a mirrored entry at the
// file position of its source.
//
//   k_nl_count / k_nl_pos   newlines per 4 KB chunk, then each line's end
//   k_parse_lines           one thread per line: blank, an entry parsed
//                           here, or a line left to the host (anything but
//                           plain decimal numbers inside the exact range
//                           below, and anything malformed: the host parses
//                           those lines with the host loader's line reader)
//   k_take_entries          entries in file order (a scan over the lines),
//                           the first NZ kept; out-of-range indices and
//                           mirrors outside the matrix flagged; the host
//                           lines listed
//   k_emit                  the entries and their mirrors in file order, as
//                           the single row of a 1 x M matrix whose stable
//                           transpose (csr_transpose) is the CSR.
// Decimal values are converted exactly when their significand has at most
// 19 digits, is at most 2^53 and the decimal exponent is within [-22, 22]:
// then the significand and 10^|e| are exact doubles and one IEEE multiply
// or divide rounds correctly (Clinger's fast path, "How to read floating
// point numbers accurately", 1990).  Other values go to the host's strtod.
#include "tsg_internal.cuh"

#include <climits>

namespace tsg {

namespace {

constexpr int NL_THREADS = 256;
constexpr int NL_BYTES = 16;                         // bytes per thread (one 16-byte load)
constexpr long long NL_CHUNK = NL_THREADS * NL_BYTES;

__device__ __forceinline__ bool dev_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }
__device__ __forceinline__ bool dev_digit(char c) { return c >= '0' && c <= '9'; }

// the 16 bytes of thread t of chunk b (zero past the end)
__device__ __forceinline__ uint4 chunk_bytes(const char *text, long long n, long long c0)
{
    if (c0 + NL_BYTES <= n) return *reinterpret_cast<const uint4 *>(text + c0);
    unsigned w[4] = {0u, 0u, 0u, 0u};
    for (int k = 0; k < NL_BYTES && c0 + k < n; ++k) w[k >> 2] |= (unsigned)(unsigned char)text[c0 + k] << ((k & 3) * 8);
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ int newlines_in(uint4 v)
{
    const unsigned nl = 0x0a0a0a0au;
    return (__popc(__vcmpeq4(v.x, nl)) + __popc(__vcmpeq4(v.y, nl)) + __popc(__vcmpeq4(v.z, nl)) +
            __popc(__vcmpeq4(v.w, nl))) >> 3;
}

__global__ void __launch_bounds__(NL_THREADS)
k_nl_count(const char *__restrict__ text, long long n, int *cnt)
{
    __shared__ int s_w[NL_THREADS / 32];
    const long long c0 = (long long)blockIdx.x * NL_CHUNK + (long long)threadIdx.x * NL_BYTES;
    int c = warp_sum_int(newlines_in(chunk_bytes(text, n, c0)));
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < NL_THREADS / 32; ++w) t += s_w[w];
        cnt[blockIdx.x] = t;
    }
}

// ends[k] = position of the k-th newline (chunk_off: newlines before each chunk)
__global__ void __launch_bounds__(NL_THREADS)
k_nl_pos(const char *__restrict__ text, long long n, const long long *__restrict__ chunk_off, long long *ends)
{
    __shared__ int s_w[NL_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long c0 = (long long)blockIdx.x * NL_CHUNK + (long long)threadIdx.x * NL_BYTES;
    const uint4 v = chunk_bytes(text, n, c0);
    const int c = newlines_in(v);
    const int incl = warp_incl_scan(c, lane);
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    int pre = 0;
    for (int w = 0; w < warp; ++w) pre += s_w[w];
    long long k = chunk_off[blockIdx.x] + pre + incl - c;
    const unsigned w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int b = 0; b < NL_BYTES; ++b)
        if (((w4[b >> 2] >> ((b & 3) * 8)) & 0xffu) == 0x0au && c0 + b < n) ends[k++] = c0 + b;
}

// strtoll-like: [blanks][+|-]digits; false (the host decides) otherwise or on overflow
__device__ bool dev_long(const char *&q, const char *e, long long &x)
{
    while (q < e && dev_blank(*q)) ++q;
    if (q >= e) return false;
    bool neg = false;
    if (*q == '+' || *q == '-') { neg = *q == '-'; ++q; }
    if (q >= e || !dev_digit(*q)) return false;
    unsigned long long v = 0;
    while (q < e && dev_digit(*q)) {
        if (v > (ULLONG_MAX - 9) / 10) return false;
        v = v * 10 + (unsigned)(*q - '0');
        ++q;
    }
    if (v > (neg ? (1ull << 63) : (1ull << 63) - 1)) return false;
    x = neg ? (long long)(0ull - v) : (long long)v;
    return true;
}

__constant__ double c_pow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                   1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// A plain decimal [blanks][+|-]digits[.digits][(e|E)[+|-]digits] inside the
// exact range (see the top of the file): true and the correctly rounded
// value; false leaves the token to the host (strtod also reads hex, inf,
// nan and longer significands, and reports malformed ones).
__device__ bool dev_double(const char *&q, const char *e, double &x)
{
    while (q < e && dev_blank(*q)) ++q;
    if (q >= e) return false;
    bool neg = false;
    if (*q == '+' || *q == '-') { neg = *q == '-'; ++q; }
    unsigned long long w = 0;
    int nd = 0, e10 = 0;
    bool any = false;
    while (q < e && dev_digit(*q)) {
        any = true;
        if (w != 0 || *q != '0') {
            if (nd >= 19) return false;
            w = w * 10 + (unsigned)(*q - '0');
            ++nd;
        }
        ++q;
    }
    if (q < e && *q == '.') {
        ++q;
        while (q < e && dev_digit(*q)) {
            any = true;
            if (w != 0 || *q != '0') {
                if (nd >= 19) return false;
                w = w * 10 + (unsigned)(*q - '0');
                ++nd;
            }
            --e10;
            ++q;
        }
    }
    if (!any) return false;
    if (q < e && (*q == 'e' || *q == 'E')) {
        ++q;
        bool eneg = false;
        if (q < e && (*q == '+' || *q == '-')) { eneg = *q == '-'; ++q; }
        if (q >= e || !dev_digit(*q)) return false;
        int ev = 0;
        while (q < e && dev_digit(*q)) {
            if (ev > 100000) return false;
            ev = ev * 10 + (*q - '0');
            ++q;
        }
        e10 += eneg ? -ev : ev;
    }
    if (w == 0) { x = neg ? -0.0 : 0.0; return true; }
    if (w > (1ull << 53) || e10 < -22 || e10 > 22) return false;
    const double d = (double)w;   // exact
    x = e10 >= 0 ? __dmul_rn(d, c_pow10[e10]) : __ddiv_rn(d, c_pow10[-e10]);
    if (neg) x = -x;
    return true;
}

// per line: 0 blank, 1 an entry parsed here, 2 left to the host, 3 an entry
// with an index outside the matrix
__global__ void __launch_bounds__(256)
k_parse_lines(const char *__restrict__ text, const long long *__restrict__ ends, long long lines, int kind,
              long long M, long long N, unsigned char *st, int *ri, int *ci, double *vv)
{
    const long long L = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (L >= lines) return;
    const char *q = text + (L == 0 ? 0 : ends[L - 1] + 1);
    const char *e = text + ends[L];
    while (q < e && dev_blank(*q)) ++q;
    unsigned char s = 0;
    long long i = 0, j = 0;
    double v = 1.0;
    if (q < e) {
        bool good = dev_long(q, e, i) && dev_long(q, e, j);
        if (good) {
            if (kind == 0) good = dev_double(q, e, v);                       // real
            else if (kind == 1) { double vim; good = dev_double(q, e, v) && dev_double(q, e, vim); }   // complex
            else if (kind == 2) { long long iv; good = dev_long(q, e, iv); v = (double)(int)iv; }      // integer
        }
        while (good && q < e && dev_blank(*q)) ++q;
        s = (good && q == e) ? 1 : 2;
        if (s == 1 && (i < 1 || i > M || j < 1 || j > N)) s = 3;
    }
    st[L] = s;
    ri[L] = s == 1 ? (int)(i - 1) : 0;
    ci[L] = s == 1 ? (int)(j - 1) : 0;
    vv[L] = v;
}

__global__ void k_is_entry(const unsigned char *__restrict__ st, long long lines, int *flag)
{
    const long long L = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (L < lines) flag[L] = st[L] != 0 ? 1 : 0;
}

// bad[0]: an entry among the first NZ outside the matrix; bad[1]: a mirror
// outside it (symmetric files); host lines among the first NZ entries:
// their entry numbers and line numbers at hpos (atomic count hn)
__global__ void k_take_entries(const unsigned char *__restrict__ st, const long long *__restrict__ tpos, long long lines,
                               long long NZ, long long M, bool symm, const int *__restrict__ lri,
                               const int *__restrict__ lci, const double *__restrict__ lvv, int *ri, int *ci, double *vv,
                               unsigned long long *hn, long long *ht, long long *hl, int *bad)
{
    const long long L = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (L >= lines || st[L] == 0) return;
    const long long t = tpos[L];
    if (t >= NZ) return;
    if (st[L] == 3) { atomicOr(bad, 1); return; }
    if (st[L] == 2) {
        const unsigned long long h = atomicAdd(hn, 1ull);
        ht[h] = t;
        hl[h] = L;
        return;
    }
    ri[t] = lri[L];
    ci[t] = lci[L];
    vv[t] = lvv[L];
    if (symm && lri[L] != lci[L] && lci[L] >= M) atomicOr(bad + 1, 1);
}

// the host's entries (t, i, j, v) into place
__global__ void k_patch(long long n, const long long *__restrict__ ht, const int *__restrict__ hi,
                        const int *__restrict__ hj, const double *__restrict__ hv, int *ri, int *ci, double *vv)
{
    const long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (h >= n) return;
    const long long t = ht[h];
    ri[t] = hi[h];
    ci[t] = hj[h];
    vv[t] = hv[h];
}

__global__ void k_emit_count(const int *__restrict__ ri, const int *__restrict__ ci, long long NZ, bool symm, int *cnt)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < NZ) cnt[t] = (symm && ri[t] != ci[t]) ? 2 : 1;
}

// entry t (and its mirror right after it) at eoff[t]: key = row, col, value
__global__ void k_emit(const int *__restrict__ ri, const int *__restrict__ ci, const double *__restrict__ vv, long long NZ,
                       bool symm, const long long *__restrict__ eoff, int *key, int *col, double *val)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= NZ) return;
    const long long d = eoff[t];
    key[d] = ri[t];
    col[d] = ci[t];
    val[d] = vv[t];
    if (symm && ri[t] != ci[t]) {
        key[d + 1] = ci[t];
        col[d + 1] = ri[t];
        val[d + 1] = vv[t];
    }
}

// the byte spans [start, end) of the host's lines
__global__ void k_host_spans(long long n, const long long *__restrict__ hl, const long long *__restrict__ ends,
                             long long *span)
{
    const long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (h >= n) return;
    const long long L = hl[h];
    span[2 * h] = L == 0 ? 0 : ends[L - 1] + 1;
    span[2 * h + 1] = ends[L];
}

__global__ void k_gather_i32(const int *__restrict__ perm, const int *__restrict__ src, int *dst, long long n)
{
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[perm[k]];
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

cudaError_t mtx_lines(Pool &pool, const char *text, long long n, long long *&ends, long long &lines, int *flags)
{
    cudaStream_t s = pool.stream;
    const long long chunks = (n + NL_CHUNK - 1) / NL_CHUNK;
    ends = nullptr;
    lines = 0;
    if (chunks == 0) return cudaSuccess;
    int *cnt = pool.alloc_n<int>(chunks + 1);
    long long *off = pool.alloc_n<long long>(chunks + 1);
    cudaError_t e = (cnt && off) ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) { k_nl_count<<<(unsigned)chunks, NL_THREADS, 0, s>>>(text, n, cnt); ::tsg::count_launch(); e = cudaGetLastError(); }
    if (e == cudaSuccess) e = scan_i32_to_i64(pool, cnt, off, chunks, flags);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&lines, off + chunks, sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && lines > 0) {
        ends = pool.alloc_n<long long>(lines);
        if (!ends) e = cudaErrorMemoryAllocation;
        else { k_nl_pos<<<(unsigned)chunks, NL_THREADS, 0, s>>>(text, n, off, ends); ::tsg::count_launch(); e = cudaGetLastError(); }
    }
    pool.free(cnt); pool.free(off);
    return e;
}

cudaError_t mtx_parse(Pool &pool, const char *text, const long long *ends, long long lines, int kind, long long M,
                      long long N, unsigned char *st, int *lri, int *lci, double *lvv)
{
    if (lines <= 0) return cudaSuccess;
    k_parse_lines<<<blocks_for(lines, 256), 256, 0, pool.stream>>>(text, ends, lines, kind, M, N, st, lri, lci, lvv);
    ::tsg::count_launch();
    return cudaGetLastError();
}

cudaError_t mtx_number_entries(Pool &pool, const unsigned char *st, long long lines, long long *tpos, int *flags)
{
    if (lines <= 0) return cudaSuccess;
    int *f = pool.alloc_n<int>(lines);
    if (!f) return cudaErrorMemoryAllocation;
    k_is_entry<<<blocks_for(lines, 256), 256, 0, pool.stream>>>(st, lines, f);
    ::tsg::count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = scan_i32_to_i64(pool, f, tpos, lines, flags);
    pool.free(f);
    return e;
}

cudaError_t mtx_take(Pool &pool, const unsigned char *st, const long long *tpos, long long lines, long long NZ,
                     long long M, bool symm, const int *lri, const int *lci, const double *lvv, int *ri, int *ci,
                     double *vv, unsigned long long *hn, long long *ht, long long *hl, int *bad)
{
    if (lines <= 0) return cudaSuccess;
    k_take_entries<<<blocks_for(lines, 256), 256, 0, pool.stream>>>(st, tpos, lines, NZ, M, symm, lri, lci, lvv, ri, ci,
                                                                   vv, hn, ht, hl, bad);
    ::tsg::count_launch();
    return cudaGetLastError();
}

cudaError_t mtx_patch(Pool &pool, long long n, const long long *ht, const int *hi, const int *hj, const double *hv,
                      int *ri, int *ci, double *vv)
{
    if (n <= 0) return cudaSuccess;
    k_patch<<<blocks_for(n, 256), 256, 0, pool.stream>>>(n, ht, hi, hj, hv, ri, ci, vv);
    ::tsg::count_launch();
    return cudaGetLastError();
}

cudaError_t mtx_emit(Pool &pool, const int *ri, const int *ci, long long NZ, bool symm, int *cnt, long long *eoff,
                     int *flags)
{
    if (NZ <= 0) return cudaMemsetAsync(eoff, 0, sizeof(long long), pool.stream);
    k_emit_count<<<blocks_for(NZ, 256), 256, 0, pool.stream>>>(ri, ci, NZ, symm, cnt);
    ::tsg::count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = scan_i32_to_i64(pool, cnt, eoff, NZ, flags);
    return e;
}

cudaError_t mtx_emit_fill(Pool &pool, const int *ri, const int *ci, const double *vv, long long NZ, bool symm,
                          const long long *eoff, int *key, int *col, double *val)
{
    if (NZ <= 0) return cudaSuccess;
    k_emit<<<blocks_for(NZ, 256), 256, 0, pool.stream>>>(ri, ci, vv, NZ, symm, eoff, key, col, val);
    ::tsg::count_launch();
    return cudaGetLastError();
}

cudaError_t mtx_host_spans(Pool &pool, long long n, const long long *hl, const long long *ends, long long *span)
{
    if (n <= 0) return cudaSuccess;
    k_host_spans<<<blocks_for(n, 256), 256, 0, pool.stream>>>(n, hl, ends, span);
    ::tsg::count_launch();
    return cudaGetLastError();
}

cudaError_t gather_i32(Pool &pool, const int *perm, const int *src, int *dst, long long n)
{
    if (n <= 0) return cudaSuccess;
    k_gather_i32<<<blocks_for(n, 256), 256, 0, pool.stream>>>(perm, src, dst, n);
    ::tsg::count_launch();
    return cudaGetLastError();
}

}  // namespace tsg
