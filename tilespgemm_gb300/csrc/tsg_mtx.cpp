// tsg_mtx.cpp -- Matrix Market load path (tsg_load_mtx).
//
// Restates the semantics of the reference's loader mmio_allinone
// (mmio_highlevel.h:593-759, using mm_read_banner mmio.h:400-496 and
// mm_read_mtx_crd_size mmio.h:561-590):
//   - banner "%%MatrixMarket matrix coordinate <real|complex|integer|pattern>
//     <general|symmetric|hermitian|skew-symmetric>" (tokens after the first
//     are case-insensitive);
//   - comment lines start with '%'; the size line holds M N NNZ;
//   - entries are 1-based; pattern -> 1.0, integer -> double, complex -> real
//     part;
//   - symmetric and hermitian files are mirrored with the same value (the
//     diagonal once), skew-symmetric files are not mirrored;
//   - per row, entries keep file order (a mirrored entry (j,i) lands in row
//     j at the file position of its source); nothing is sorted or merged.
// Differences, all of which the reference turns into undefined behaviour:
// 'array' files, indices outside [1,M]x[1,N], and truncated data lines are
// rejected with TSG_ERR_BAD_MTX.
//
// The data lines of large files are parsed by several host threads, each
// over a run of whole lines, when every data line holds exactly one entry;
// otherwise (an entry split over lines, extra tokens, a malformed line) the
// file is read again token by token, as the reference's fscanf does, so the
// result and the error are the same either way.  TSG_MTX_THREADS sets the
// thread count (1: token by token only); by default one thread per 4 MB of
// data, at most the host's hardware threads.
#include "tilespgemm.h"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace tsg {
void set_last_error(const char *msg);
void *make_malloc_owner(void *a, void *b, void *c);
}
#include "tsg_mtx.h"

namespace {

bool read_file(const char *path, std::string &out)
{
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    // one allocation when the size is known (a regular file), then chunks
    // for whatever else arrives
    if (fseek(f, 0, SEEK_END) == 0) {
        const long sz = ftell(f);
        if (sz > 0) out.reserve((size_t)sz + 1);
        rewind(f);
    }
    std::vector<char> buf(1 << 20);
    size_t got;
    while ((got = fread(buf.data(), 1, buf.size(), f)) > 0) out.append(buf.data(), got);
    fclose(f);
    return true;
}

std::string lower(std::string s)
{
    for (auto &ch : s) ch = (char)tolower((unsigned char)ch);
    return s;
}

struct Cursor {
    const char *p, *end;
    void skip_ws() { while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p; }
    bool read_long(long long &v) {
        skip_ws();
        if (p >= end) return false;
        char *e = nullptr;
        errno = 0;
        v = strtoll(p, &e, 10);
        if (e == p || errno) return false;
        p = e;
        return true;
    }
    bool read_double(double &v) {
        skip_ws();
        if (p >= end) return false;
        char *e = nullptr;
        v = strtod(p, &e);
        if (e == p) return false;
        p = e;
        return true;
    }
};

tsg_status bad(const char *msg)
{
    tsg::set_last_error(msg);
    return TSG_ERR_BAD_MTX;
}

enum ValueKind { V_REAL, V_COMPLEX, V_INT, V_PATTERN };
static_assert((int)V_REAL == (int)tsg::MTX_REAL && (int)V_COMPLEX == (int)tsg::MTX_COMPLEX &&
              (int)V_INT == (int)tsg::MTX_INTEGER && (int)V_PATTERN == (int)tsg::MTX_PATTERN, "value kinds");

// The entries of the data lines in [p, end), one per line (blank lines
// skipped), in file order, 0-based.  ok = false when a line is not exactly
// one entry (the caller then reads the file token by token); first_bad = the
// run's first entry outside the M x N matrix (stored as 0, 0), or -1.
struct LineRun {
    std::vector<int> i, j;
    std::vector<double> v;
    long long first_bad = -1;
    bool ok = true;
};

inline bool blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

}  // namespace

namespace tsg {

// One data line [p, e) (no newline inside; the byte at e is not a digit):
// false unless it is exactly one entry of the given value kind (i, j
// 1-based as written; v: pattern 1.0, integer as (double)(int), complex the
// real part).  Blank lines are the caller's.
bool mtx_line(const char *p, const char *e, int kind, long long &i, long long &j, double &v)
{
    const char *q = p;
    auto tok_long = [&](long long &x) {
        while (q < e && blank(*q)) ++q;
        if (q >= e) return false;
        char *t = nullptr;
        errno = 0;
        x = strtoll(q, &t, 10);
        if (t == q || errno || t > e) return false;
        q = t;
        return true;
    };
    auto tok_double = [&](double &x) {
        while (q < e && blank(*q)) ++q;
        if (q >= e) return false;
        char *t = nullptr;
        x = strtod(q, &t);
        if (t == q || t > e) return false;
        q = t;
        return true;
    };
    i = j = 0;
    v = 1.0;
    double vim = 0.0;
    bool good = tok_long(i) && tok_long(j);
    if (good && kind == V_REAL) good = tok_double(v);
    else if (good && kind == V_COMPLEX) good = tok_double(v) && tok_double(vim);
    else if (good && kind == V_INT) { long long iv = 0; good = tok_long(iv); v = (double)(int)iv; }
    while (good && q < e && blank(*q)) ++q;
    return good && q == e;
}

}  // namespace tsg

namespace {

void parse_lines(const char *p, const char *end, ValueKind kind, long long M, long long N, LineRun &out)
{
    // room for one entry per line, allocated once (threads growing vectors
    // side by side spent their time in the kernel's page mapping)
    const size_t lines = (size_t)std::count(p, end, '\n') + 1;
    out.i.reserve(lines);
    out.j.reserve(lines);
    out.v.reserve(lines);
    while (p < end) {
        const char *e = (const char *)memchr(p, '\n', (size_t)(end - p));
        if (!e) e = end;
        const char *q = p;
        while (q < e && blank(*q)) ++q;
        if (q < e) {
            long long i = 0, j = 0;
            double v = 1.0;
            if (!tsg::mtx_line(q, e, kind, i, j, v)) { out.ok = false; return; }
            if (i < 1 || i > M || j < 1 || j > N) {
                if (out.first_bad < 0) out.first_bad = (long long)out.i.size();
                i = j = 1;
            }
            out.i.push_back((int)(i - 1));
            out.j.push_back((int)(j - 1));
            out.v.push_back(v);
        }
        p = e + 1;
    }
}

int mtx_threads(size_t data_bytes)
{
    if (const char *env = getenv("TSG_MTX_THREADS")) {
        const long t = strtol(env, nullptr, 10);
        if (t >= 1) return (int)std::min<long>(t, 256);
    }
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    return (int)std::min<size_t>(hw, std::max<size_t>(1, data_bytes / (4u << 20)));
}

// Data lines [p, end) parsed by `nt` threads into ri/ci/vv (the first NZ
// entries, checked like the token reader checks them).  Returns false when
// a line is not one entry: nothing is decided then.
bool parse_parallel(const char *p, const char *end, int nt, ValueKind kind, long long M, long long N, long long NZ,
                    std::vector<int> &ri, std::vector<int> &ci, std::vector<double> &vv, tsg_status &st)
{
    std::vector<const char *> cut((size_t)nt + 1);
    cut[0] = p;
    cut[(size_t)nt] = end;
    for (int k = 1; k < nt; ++k) {   // run k starts after the first newline at or past its even share
        const char *c = p + (size_t)(end - p) * (size_t)k / (size_t)nt;
        if (c < cut[(size_t)k - 1]) c = cut[(size_t)k - 1];
        const char *nl = (const char *)memchr(c, '\n', (size_t)(end - c));
        cut[(size_t)k] = nl ? nl + 1 : end;
    }
    std::vector<LineRun> run((size_t)nt);
    std::vector<std::thread> th;
    for (int k = 1; k < nt; ++k)
        th.emplace_back(parse_lines, cut[(size_t)k], cut[(size_t)k + 1], kind, M, N, std::ref(run[(size_t)k]));
    parse_lines(cut[0], cut[1], kind, M, N, run[0]);
    for (auto &t : th) t.join();
    // entries past the first NZ are never read by the token reader, so a
    // malformed line after them does not matter; one before them does
    long long have = 0;
    for (int k = 0; k < nt && have < NZ; ++k) {
        if (!run[(size_t)k].ok) return false;
        have += (long long)run[(size_t)k].i.size();
    }
    long long t = 0;
    for (int k = 0; k < nt && t < NZ; ++k) {
        const LineRun &r = run[(size_t)k];
        const long long take = std::min<long long>((long long)r.i.size(), NZ - t);
        if (r.first_bad >= 0 && r.first_bad < take) { st = bad("entry index outside the matrix"); return true; }
        std::copy(r.i.begin(), r.i.begin() + take, ri.begin() + t);
        std::copy(r.j.begin(), r.j.begin() + take, ci.begin() + t);
        std::copy(r.v.begin(), r.v.begin() + take, vv.begin() + t);
        t += take;
    }
    st = t < NZ ? bad("truncated data line") : TSG_OK;
    return true;
}

}  // namespace

namespace tsg {

// The banner, comments and size line of a Matrix Market text (ending with
// '\n'): sizes, value kind, symmetry; `cursor` = the offset just past the
// size line's NZ, and, when the rest of that line is blank, `data` = the
// offset of the first data line (lines = true).
tsg_status mtx_header(const std::string &text, MtxHeader &h)
{
    const char *p = text.data(), *end = text.data() + text.size();
    // banner line
    const char *nl = (const char *)memchr(p, '\n', (size_t)(end - p));
    std::string line(p, nl ? (size_t)(nl - p) : (size_t)(end - p));
    char tok[5][1025];
    if (line.size() > 1024 || sscanf(line.c_str(), "%1024s %1024s %1024s %1024s %1024s", tok[0], tok[1], tok[2], tok[3], tok[4]) != 5)
        return bad("premature end of the banner line");
    if (strncmp(tok[0], "%%MatrixMarket", 14) != 0) return bad("no %%MatrixMarket banner");
    const std::string mtx = lower(tok[1]), crd = lower(tok[2]), type = lower(tok[3]), sym = lower(tok[4]);
    if (mtx != "matrix") return bad("unsupported object (not 'matrix')");
    if (crd == "array") return bad("'array' (dense) Matrix Market files are not supported");
    if (crd != "coordinate") return bad("unsupported storage (not 'coordinate')");
    const bool is_real = type == "real", is_complex = type == "complex", is_int = type == "integer", is_pat = type == "pattern";
    if (!is_real && !is_complex && !is_int && !is_pat) return bad("unsupported data type");
    h.symm = (sym == "symmetric" || sym == "hermitian");
    if (!h.symm && sym != "general" && sym != "skew-symmetric") return bad("unsupported symmetry");
    h.kind = is_real ? V_REAL : is_complex ? V_COMPLEX : is_int ? V_INT : V_PATTERN;
    p = nl ? nl + 1 : end;
    // skip comment lines, then blank lines, to the size line
    while (p < end && *p == '%') {
        const char *e = (const char *)memchr(p, '\n', (size_t)(end - p));
        p = e ? e + 1 : end;
    }
    Cursor cur{p, end};
    if (!cur.read_long(h.M) || !cur.read_long(h.N) || !cur.read_long(h.NZ)) return bad("bad size line");
    if (h.M < 0 || h.N < 0 || h.NZ < 0 || h.M > INT32_MAX - 1 || h.N > INT32_MAX - 1 || h.NZ > INT32_MAX)
        return bad("sizes out of range");
    h.cursor = (size_t)(cur.p - text.data());
    // the rest of the size line must be blank for the line readers
    const char *dp = cur.p;
    while (dp < end && blank(*dp)) ++dp;
    h.lines = dp < end && *dp == '\n';
    h.data = h.lines ? (size_t)(dp + 1 - text.data()) : text.size();
    return TSG_OK;
}

bool mtx_read_file(const char *path, std::string &out)
{
    if (!read_file(path, out)) return false;
    out.push_back('\n');   // strtod/strtoll and the line readers stop at the end
    return true;
}

}  // namespace tsg

extern "C" tsg_status tsg_load_mtx(const char *path, tsg_csr *out, int32_t *is_symmetric)
{
    if (!path || !out) {
        tsg::set_last_error("path/out is NULL");
        return TSG_ERR_INVALID_ARG;
    }
    memset(out, 0, sizeof(*out));
    std::string text;
    if (!tsg::mtx_read_file(path, text)) return bad("could not open the Matrix Market file");
    const char *end = text.data() + text.size();
    tsg::MtxHeader h;
    tsg_status hst = tsg::mtx_header(text, h);
    if (hst != TSG_OK) return hst;
    const long long M = h.M, N = h.N, NZ = h.NZ;
    const bool symm = h.symm;
    const ValueKind kind = (ValueKind)h.kind;
    const bool is_real = kind == V_REAL, is_complex = kind == V_COMPLEX, is_int = kind == V_INT;
    Cursor cur{text.data() + h.cursor, end};
    std::vector<int> ri((size_t)NZ), ci((size_t)NZ);
    std::vector<double> vv((size_t)NZ);
    const int nt = NZ > 0 ? mtx_threads((size_t)(end - cur.p)) : 1;
    tsg_status pst = TSG_OK;
    if (nt > 1 && h.lines && parse_parallel(text.data() + h.data, end, nt, kind, M, N, NZ, ri, ci, vv, pst)) {
        if (pst != TSG_OK) return pst;
    } else for (long long t = 0; t < NZ; ++t) {
        long long i = 0, j = 0;
        double v = 1.0, vim = 0.0;
        if (!cur.read_long(i) || !cur.read_long(j)) return bad("truncated data line");
        if (is_real) { if (!cur.read_double(v)) return bad("truncated data line"); }
        else if (is_complex) { if (!cur.read_double(v) || !cur.read_double(vim)) return bad("truncated data line"); }
        else if (is_int) { long long iv; if (!cur.read_long(iv)) return bad("truncated data line"); v = (double)(int)iv; }
        if (i < 1 || i > M || j < 1 || j > N) return bad("entry index outside the matrix");
        ri[(size_t)t] = (int)(i - 1);
        ci[(size_t)t] = (int)(j - 1);
        vv[(size_t)t] = v;
    }
    // counts, then fill in file order (mirrors right after their source).
    // With several threads, thread k owns the rows [M k / nt, M (k+1) / nt)
    // and walks every entry in file order, so each row keeps file order.
    auto by_rows = [&](auto &&fn) {
        if (nt <= 1) { fn(0ll, M); return; }
        std::vector<std::thread> th;
        for (int k = 1; k < nt; ++k) th.emplace_back(fn, M * k / nt, M * (k + 1) / nt);
        fn(0ll, M / nt);
        for (auto &t : th) t.join();
    };
    for (long long t = 0; symm && t < NZ; ++t)
        if (ri[(size_t)t] != ci[(size_t)t] && ci[(size_t)t] >= M) return bad("symmetric entry mirrored outside the matrix");
    std::vector<long long> cnt((size_t)M + 1, 0);
    by_rows([&](long long r0, long long r1) {
        for (long long t = 0; t < NZ; ++t) {
            const long long i = ri[(size_t)t], j = ci[(size_t)t];
            if (i >= r0 && i < r1) cnt[(size_t)i]++;
            if (symm && i != j && j >= r0 && j < r1) cnt[(size_t)j]++;
        }
    });
    long long total = 0;
    for (long long r = 0; r < M; ++r) { long long c = cnt[(size_t)r]; cnt[(size_t)r] = total; total += c; }
    cnt[(size_t)M] = total;
    if (total > INT32_MAX) {
        tsg::set_last_error("more than 2^31-1 entries after mirroring");
        return TSG_ERR_NOT_SUPPORTED;
    }
    int *rp = (int *)malloc(sizeof(int) * (size_t)(M + 1));
    int *col = (int *)malloc(sizeof(int) * (size_t)(total > 0 ? total : 1));
    double *val = (double *)malloc(sizeof(double) * (size_t)(total > 0 ? total : 1));
    if (!rp || !col || !val) {
        free(rp); free(col); free(val);
        tsg::set_last_error("host allocation failed");
        return TSG_ERR_OOM;
    }
    for (long long r = 0; r <= M; ++r) rp[r] = (int)cnt[(size_t)r];
    by_rows([&](long long r0, long long r1) {   // cnt[r] becomes row r's next free slot
        for (long long t = 0; t < NZ; ++t) {
            const int i = ri[(size_t)t], j = ci[(size_t)t];
            if (i >= r0 && i < r1) {
                const long long d = cnt[(size_t)i]++;
                col[d] = j;
                val[d] = vv[(size_t)t];
            }
            if (symm && i != j && j >= r0 && j < r1) {
                const long long d = cnt[(size_t)j]++;
                col[d] = i;
                val[d] = vv[(size_t)t];
            }
        }
    });
    out->m = (int32_t)M;
    out->n = (int32_t)N;
    out->nnz = total;
    out->rowptr_bits = 32;
    out->where = TSG_MEM_HOST;
    out->row_ptr = rp;
    out->col = col;
    out->val = val;
    out->owner = tsg::make_malloc_owner(rp, col, val);
    if (is_symmetric) *is_symmetric = symm ? 1 : 0;
    return TSG_OK;
}

// Write a host CSR as a Matrix Market coordinate file, in the format of the
// reference's writer mm_write_mtx_crd (mmio.h:780-850): banner
// "%%MatrixMarket matrix coordinate real general", the size line "M N NNZ",
// then one "i j value" line per entry with 1-based indices, in CSR order.
// Values use the reference's "%20.16g" unless `exact`, which writes 17
// significant digits so that the file loads back to the same doubles.
// Large matrices are formatted by several host threads (TSG_MTX_THREADS, or
// one per 256 K entries up to the hardware threads) in waves of about a
// million entries per thread, written in row order: the bytes are the same.
namespace {

long long rp_at(const tsg_csr *M, long long i)
{
    return M->rowptr_bits == 64 ? ((const long long *)M->row_ptr)[i] : (long long)((const int *)M->row_ptr)[i];
}

// the first row r in [lo, hi] whose row pointer is at least `target`
long long row_at(const tsg_csr *M, long long lo, long long hi, long long target)
{
    while (lo < hi) {
        const long long mid = lo + (hi - lo) / 2;
        if (rp_at(M, mid) < target) lo = mid + 1; else hi = mid;
    }
    return lo;
}

void format_rows(const tsg_csr *M, long long r0, long long r1, const char *fmt, std::string &out)
{
    out.clear();
    char line[128];
    for (long long i = r0; i < r1; ++i) {
        const long long p1 = rp_at(M, i + 1);
        for (long long p = rp_at(M, i); p < p1; ++p) {
            const int len = snprintf(line, sizeof line, fmt, (int)(i + 1), M->col[p] + 1, M->val[p]);
            out.append(line, (size_t)len);
        }
    }
}

}  // namespace

extern "C" tsg_status tsg_write_mtx(const char *path, const tsg_csr *M, int32_t exact)
{
    if (!path || !M) { tsg::set_last_error("path/M is NULL"); return TSG_ERR_INVALID_ARG; }
    if (M->where != TSG_MEM_HOST) { tsg::set_last_error("tsg_write_mtx takes a host matrix"); return TSG_ERR_INVALID_ARG; }
    if (M->m < 0 || M->n < 0 || M->nnz < 0 || (M->rowptr_bits != 32 && M->rowptr_bits != 64) || !M->row_ptr ||
        (M->nnz > 0 && (!M->col || !M->val))) {
        tsg::set_last_error("M is not a valid CSR");
        return TSG_ERR_INVALID_ARG;
    }
    // the row pointer is checked whole before anything is written
    bool rp_ok = rp_at(M, 0) >= 0;
    for (long long i = 0; i < M->m && rp_ok; ++i) rp_ok = rp_at(M, i + 1) >= rp_at(M, i);
    if (rp_ok) rp_ok = rp_at(M, M->m) <= M->nnz;
    if (!rp_ok) { tsg::set_last_error("M's row pointer is not monotone within [0, nnz]"); return TSG_ERR_INVALID_ARG; }
    FILE *f = fopen(path, "wb");
    if (!f) { tsg::set_last_error("cannot open the output file"); return TSG_ERR_INVALID_ARG; }
    char head[128];
    const int hlen = snprintf(head, sizeof head, "%%%%MatrixMarket matrix coordinate real general\n%d %d %lld\n", M->m,
                              M->n, (long long)M->nnz);
    bool ok = fwrite(head, 1, (size_t)hlen, f) == (size_t)hlen;
    const char *fmt = exact ? "%d %d %.17g\n" : "%d %d %20.16g\n";
    const long long entries = rp_at(M, M->m) - rp_at(M, 0);
    int nt = 0;
    if (const char *env = getenv("TSG_MTX_THREADS")) nt = (int)std::min(256l, strtol(env, nullptr, 10));
    if (nt < 1) {
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        nt = (int)std::min<long long>(hw, std::max<long long>(1, entries / (256 << 10)));
    }
    const long long wave = (long long)nt << 20;   // entries per wave
    std::vector<std::string> buf((size_t)nt);
    for (long long a = 0; a < M->m && ok;) {
        long long b = row_at(M, a, M->m, rp_at(M, a) + wave);
        if (b <= a) b = a + 1;
        // the wave's rows in nt slices of about equal entries
        std::vector<long long> cut((size_t)nt + 1);
        cut[0] = a;
        cut[(size_t)nt] = b;
        const long long e0 = rp_at(M, a), e1 = rp_at(M, b);
        for (int k = 1; k < nt; ++k) cut[(size_t)k] = std::max(cut[(size_t)k - 1], row_at(M, a, b, e0 + (e1 - e0) * k / nt));
        std::vector<std::thread> th;
        for (int k = 1; k < nt; ++k)
            th.emplace_back(format_rows, M, cut[(size_t)k], cut[(size_t)k + 1], fmt, std::ref(buf[(size_t)k]));
        format_rows(M, cut[0], cut[1], fmt, buf[0]);
        for (auto &t : th) t.join();
        for (int k = 0; k < nt && ok; ++k) ok = fwrite(buf[(size_t)k].data(), 1, buf[(size_t)k].size(), f) == buf[(size_t)k].size();
        a = b;
    }
    if (fclose(f) != 0) ok = false;
    if (!ok) { tsg::set_last_error("writing the Matrix Market file failed"); return TSG_ERR_INVALID_ARG; }
    return TSG_OK;
}
