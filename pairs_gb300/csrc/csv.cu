// Particle CSV input parsed on the device.
//
// Replaces the reference's read_particle_data (runtime/read_from_file.hpp:33-116): the
// file is one particle per line, its fields in the declared property order (a vector
// property takes 3 fields, a matrix 9, a quaternion 4), numbers read as std::stod /
// std::stoi read them, and a particle is kept when its position lies inside the domain
// (x >= min and x < max - 1e-5 on every axis, runtime/domain/regular_6d_stencil.cpp:96-100)
// or its flags mark it infinite, fixed or global.  Lines that hold only white space are
// skipped (the reference would create a particle from such a line with every property
// left unset).
//
// The host reads the file's bytes; everything after that runs here:
//   1. line index: newlines counted per 4 KB chunk, the counts scanned, each chunk's
//      newline offsets written to line_start (one ballot-compacted pass per chunk);
//   2. one thread per line parses its fields into a column-major table of doubles and
//      decides whether the particle is kept;
//   3. the kept rows are scanned and compacted into the caller's table.
//
// Numbers.  A field is read as std::stod reads it: leading white space, an optional
// sign, "inf"/"infinity"/"nan" in any case, or digits with an optional point and an
// optional exponent; trailing characters end the number.  The value is the correctly
// rounded double of the decimal (round to nearest, ties to even):
//   * up to 15-16 significant digits (w < 2^53) and |exponent| <= 22: one FP64 multiply
//     or divide of two exact operands (Clinger's fast path);
//   * up to 19 significant digits and |exponent| <= 80: exact integer arithmetic on 256
//     bits (w * 5^q, or floor((w << s) / 5^n) with a sticky remainder) rounded to 53 bits;
//   * anything else (more than 19 significant digits that are not all zero, or a larger
//     exponent) is counted as out of the exact range and fails the call, as does a
//     field without digits, a missing field or an integer outside int32 (std::stoi
//     throws for the last two).
#include <math.h>

#include "common.cuh"

namespace pg {

int scan_exclusive_i32(const int32_t *in, int n, int32_t *out, int32_t *block_sums, cudaStream_t st);
int64_t scan_block_sums_len(int n);

constexpr int kCsvChunk = 4096;               // bytes per block of the line index
constexpr int kCsvThreads = 256;              // 16 bytes per thread
constexpr int kCsvMaxFields = 64;

struct CsvWs {
    int32_t *chunk_count;    // [nchunks + 1] newlines per chunk, then their exclusive scan
    int32_t *chunk_base;
    int32_t *line_start;     // [lines + 1]
    int32_t *keep;           // [lines + 1]
    int32_t *row;            // [lines + 1]
    int32_t *block_sums;
    int32_t *status;         // [4]: bad line (min), out-of-range numbers, rows, spare
    double *temp;            // [nfields * lines]
};

static size_t csv_align(size_t x) { return (x + 255) & ~(size_t) 255; }

static int64_t nchunks_of(int64_t bytes) { return (bytes + kCsvChunk - 1) / kCsvChunk; }

static size_t csv_ws_layout(int64_t bytes, int64_t lines, int32_t nfields, char *base, CsvWs *w) {
    const int64_t nc = nchunks_of(bytes);
    const int64_t scan_n = (nc > lines ? nc : lines) + 1;
    size_t off = 0;
    auto take = [&](size_t b) { char *p = base ? base + off : nullptr; off += csv_align(b); return p; };
    CsvWs t;
    t.status = (int32_t *) take(4 * sizeof(int32_t));
    t.chunk_count = (int32_t *) take((size_t) (nc + 1) * 4);
    t.chunk_base = (int32_t *) take((size_t) (nc + 1) * 4);
    t.block_sums = (int32_t *) take((size_t) scan_block_sums_len((int) scan_n) * 4);
    t.line_start = (int32_t *) take((size_t) (lines + 1) * 4);
    t.keep = (int32_t *) take((size_t) (lines + 1) * 4);
    t.row = (int32_t *) take((size_t) (lines + 1) * 4);
    t.temp = (double *) take((size_t) nfields * (size_t) lines * 8);
    if(w) { *w = t; }
    return off;
}

// ------------------------------------------------------------------ line index

__device__ __forceinline__ int newlines16(const char *text, int64_t bytes, int64_t at, unsigned &mask) {
    mask = 0u;
    for(int k = 0; k < 16; k++) {
        const int64_t p = at + k;
        if(p < bytes && text[p] == '\n') { mask |= 1u << k; }
    }
    return __popc(mask);
}

__device__ __forceinline__ int block_exclusive(int v, int &total) {
    __shared__ int warp_tot[kCsvThreads / 32 + 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = v;
    for(int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if(lane >= o) { incl += t; }
    }
    if(lane == 31) { warp_tot[w] = incl; }
    __syncthreads();
    if(threadIdx.x == 0) {
        int run = 0;
        for(int k = 0; k < kCsvThreads / 32; k++) { const int x = warp_tot[k]; warp_tot[k] = run; run += x; }
        warp_tot[kCsvThreads / 32] = run;
    }
    __syncthreads();
    total = warp_tot[kCsvThreads / 32];
    return incl - v + warp_tot[w];
}

__global__ void __launch_bounds__(kCsvThreads) k_csv_count(const char *text, int64_t bytes, int32_t *chunk_count) {
    const int64_t at = (int64_t) blockIdx.x * kCsvChunk + 16 * threadIdx.x;
    unsigned m;
    const int c = newlines16(text, bytes, at, m);
    int total;
    block_exclusive(c, total);
    if(threadIdx.x == 0) { chunk_count[blockIdx.x] = total; }
}

// line_start[0] = 0; the k-th newline of the file (at byte p) starts line k + 1 at p + 1
__global__ void __launch_bounds__(kCsvThreads) k_csv_lines(const char *text, int64_t bytes, const int32_t *chunk_base,
                                                           int32_t *line_start) {
    const int64_t at = (int64_t) blockIdx.x * kCsvChunk + 16 * threadIdx.x;
    unsigned m;
    const int c = newlines16(text, bytes, at, m);
    int total;
    int k = chunk_base[blockIdx.x] + block_exclusive(c, total);
    while(m) {
        const int b = __ffs(m) - 1;
        m &= m - 1;
        line_start[k + 1] = (int32_t) (at + b + 1);
        k++;
    }
    if(blockIdx.x == 0 && threadIdx.x == 0) { line_start[0] = 0; }
}

// ------------------------------------------------------------------ numbers

__device__ __forceinline__ bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f';
}

__device__ __forceinline__ char lower(char c) { return (c >= 'A' && c <= 'Z') ? (char) (c + 32) : c; }

// powers of ten exact in FP64 (10^0 .. 10^22) and of five exact in 64 bits (5^0 .. 5^27)
__device__ __forceinline__ double pow10_exact(int k) {
    double r = 1.0;
    for(int i = 0; i < k; i++) { r *= 10.0; }     // every partial product is exact for k <= 22
    return r;
}

__device__ __forceinline__ unsigned long long pow5(int k) {
    unsigned long long r = 1ull;
    for(int i = 0; i < k; i++) { r *= 5ull; }
    return r;
}

// Unsigned integers of 4 x 64 bits (little-endian words), enough for w * 5^80 or
// (w << s) with s + 64 < 256.
struct U256 { unsigned long long w[4]; };

__device__ __forceinline__ void u_mul(U256 &x, unsigned long long m) {
    unsigned long long carry = 0ull;
    for(int k = 0; k < 4; k++) {
        const unsigned __int128 t = (unsigned __int128) x.w[k] * m + carry;
        x.w[k] = (unsigned long long) t;
        carry = (unsigned long long) (t >> 64);
    }
}

// x = floor(x / d); returns whether the remainder is non-zero
__device__ __forceinline__ bool u_div(U256 &x, unsigned long long d) {
    unsigned long long r = 0ull;
    for(int k = 3; k >= 0; k--) {
        const unsigned __int128 t = ((unsigned __int128) r << 64) | x.w[k];
        x.w[k] = (unsigned long long) (t / d);
        r = (unsigned long long) (t % d);
    }
    return r != 0ull;
}

__device__ __forceinline__ int u_bitlen(const U256 &x) {
    for(int k = 3; k >= 0; k--) {
        if(x.w[k]) { return 64 * k + 64 - __clzll((long long) x.w[k]); }
    }
    return 0;
}

__device__ __forceinline__ bool u_bit(const U256 &x, int i) { return (x.w[i >> 6] >> (i & 63)) & 1ull; }

__device__ __forceinline__ bool u_any_below(const U256 &x, int i) {      // any bit of x below bit i
    for(int k = 0; k < 4; k++) {
        const int lo = 64 * k;
        if(lo >= i) { break; }
        const int nb = i - lo;
        const unsigned long long m = nb >= 64 ? ~0ull : ((1ull << nb) - 1ull);
        if(x.w[k] & m) { return true; }
    }
    return false;
}

// x * 2^e2 rounded to the nearest double (ties to even); `sticky`: the exact value lies
// strictly above x * 2^e2 (a remainder below x's last bit was dropped).  x > 0.
__device__ double round_to_double(const U256 &x, int e2, bool sticky) {
    const int bl = u_bitlen(x);
    unsigned long long m = 0ull;
    int e;
    if(bl <= 53) {
        m = x.w[0];                              // exact (sticky is false on every path that gets here)
        e = e2;
    } else {
        const int sh = bl - 53;
        for(int i = 0; i < 53; i++) { m |= (unsigned long long) u_bit(x, sh + i) << i; }
        const bool half = u_bit(x, sh - 1);
        const bool below = sticky || u_any_below(x, sh - 1);
        e = e2 + sh;
        if(half && (below || (m & 1ull))) {
            m++;
            if(m == (1ull << 53)) { m >>= 1; e++; }
        }
    }
    return ldexp((double) m, e);
}

constexpr int kCsvMaxExp10 = 80;               // |decimal exponent| of the exact paths

struct CsvNum {
    double v;
    int status;              // 0 ok, 1 no number, 2 outside the exact conversion range
};

__device__ CsvNum parse_real(const char *s, int len) {
    CsvNum r; r.v = 0.0; r.status = 1;
    int i = 0;
    while(i < len && is_space(s[i])) { i++; }
    bool neg = false;
    if(i < len && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; i++; }
    // inf / infinity / nan
    if(i + 3 <= len) {
        const char a = lower(s[i]), b = lower(s[i + 1]), c = lower(s[i + 2]);
        if(a == 'i' && b == 'n' && c == 'f') { r.v = neg ? -INFINITY : INFINITY; r.status = 0; return r; }
        if(a == 'n' && b == 'a' && c == 'n') { r.v = neg ? -NAN : NAN; r.status = 0; return r; }
    }
    unsigned long long w = 0ull;
    int nd = 0, q = 0;
    bool any = false, dropped = false;
    while(i < len && s[i] >= '0' && s[i] <= '9') {
        const int d = s[i] - '0';
        any = true;
        if(w == 0ull && d == 0) {
            // leading zero
        } else if(nd < 19) {
            w = w * 10ull + (unsigned long long) d; nd++;
        } else {
            q++;
            if(d != 0) { dropped = true; }
        }
        i++;
    }
    if(i < len && s[i] == '.') {
        i++;
        while(i < len && s[i] >= '0' && s[i] <= '9') {
            const int d = s[i] - '0';
            any = true;
            if(w == 0ull && d == 0) {
                q--;
            } else if(nd < 19) {
                w = w * 10ull + (unsigned long long) d; nd++; q--;
            } else if(d != 0) {
                dropped = true;
            }
            i++;
        }
    }
    if(!any) { return r; }
    if(i < len && (s[i] == 'e' || s[i] == 'E')) {
        int j = i + 1;
        bool eneg = false;
        if(j < len && (s[j] == '+' || s[j] == '-')) { eneg = s[j] == '-'; j++; }
        if(j < len && s[j] >= '0' && s[j] <= '9') {
            int ex = 0;
            while(j < len && s[j] >= '0' && s[j] <= '9') {
                if(ex < 100000) { ex = ex * 10 + (s[j] - '0'); }
                j++;
            }
            q += eneg ? -ex : ex;
        }
    }
    r.status = 0;
    if(w == 0ull) { r.v = neg ? -0.0 : 0.0; return r; }
    if(dropped) { r.status = 2; return r; }
    double v;
    if(w < (1ull << 53) && q >= -22 && q <= 22) {
        v = q >= 0 ? (double) w * pow10_exact(q) : (double) w / pow10_exact(-q);
    } else if(q >= 0 && q <= kCsvMaxExp10) {
        U256 x = {{w, 0ull, 0ull, 0ull}};
        for(int k = q; k > 0; k -= 27) { u_mul(x, pow5(k < 27 ? k : 27)); }
        v = round_to_double(x, q, false);
    } else if(q < 0 && q >= -kCsvMaxExp10) {
        const int n = -q;
        U256 p5 = {{1ull, 0ull, 0ull, 0ull}};
        for(int k = n; k > 0; k -= 27) { u_mul(p5, pow5(k < 27 ? k : 27)); }
        const int bl_w = 64 - __clzll((long long) w), bl_d = u_bitlen(p5);
        const int sh = 62 + bl_d - bl_w;            // >= 1; w << sh has 62 + bl_d <= 250 bits
        U256 x = {{0ull, 0ull, 0ull, 0ull}};
        x.w[sh >> 6] = w << (sh & 63);
        if((sh & 63) != 0 && (sh >> 6) + 1 < 4) { x.w[(sh >> 6) + 1] = w >> (64 - (sh & 63)); }
        bool sticky = false;                        // floor(x / 5^n) in steps of 5^27: Q in [2^61, 2^63)
        for(int k = n; k > 0; k -= 27) { sticky |= u_div(x, pow5(k < 27 ? k : 27)); }
        v = round_to_double(x, -sh - n, sticky);
    } else {
        r.status = 2;
        return r;
    }
    r.v = neg ? -v : v;
    return r;
}

// std::stoi: white space, optional sign, at least one digit, the value within int32
__device__ CsvNum parse_int(const char *s, int len) {
    CsvNum r; r.v = 0.0; r.status = 1;
    int i = 0;
    while(i < len && is_space(s[i])) { i++; }
    bool neg = false;
    if(i < len && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; i++; }
    long long x = 0;
    bool any = false;
    while(i < len && s[i] >= '0' && s[i] <= '9') {
        any = true;
        if(x <= 10000000000ll) { x = x * 10 + (s[i] - '0'); }
        i++;
    }
    if(!any) { return r; }
    x = neg ? -x : x;
    if(x < -2147483648ll || x > 2147483647ll) { return r; }
    r.v = (double) x;
    r.status = 0;
    return r;
}

// ------------------------------------------------------------------ parse, keep, compact

struct CsvArgs {
    const char *text;
    int64_t bytes;
    int32_t lines;
    int32_t nfields;
    int32_t kinds[kCsvMaxFields];
    int32_t pos_field, flags_field, filter;
    double lo[3], hi_small[3];   // hi - 1e-5, rounded as the reference rounds it
};

__global__ void k_csv_parse(CsvArgs a, const int32_t *line_start, int32_t *keep, double *temp, int32_t *status) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if(l >= a.lines) { return; }
    const int64_t s = line_start[l];
    int64_t e = l + 1 < a.lines ? (int64_t) line_start[l + 1] - 1 : a.bytes;     // the newline is not part of it
    if(e > a.bytes) { e = a.bytes; }
    const char *t = a.text;
    bool blank = true;
    for(int64_t p = s; p < e; p++) {
        if(!is_space(t[p])) { blank = false; break; }
    }
    int k = 0;
    if(!blank) {
        int64_t p = s;
        bool bad = false;
        int flags = 0;
        double pos[3] = {0.0, 0.0, 0.0};
        for(int f = 0; f < a.nfields; f++) {
            if(p > e) { bad = true; break; }               // the line ran out of fields
            int64_t q = p;
            while(q < e && t[q] != ',') { q++; }
            const int len = (int) (q - p);
            const CsvNum v = a.kinds[f] == PG_CSV_INT ? parse_int(t + p, len) : parse_real(t + p, len);
            if(v.status == 1) { bad = true; break; }
            if(v.status == 2) { atomicAdd(&status[1], 1); }
            temp[(size_t) f * a.lines + l] = v.v;
            if(f == a.flags_field) { flags = (int) v.v; }
            if(a.pos_field >= 0 && f >= a.pos_field && f < a.pos_field + 3) { pos[f - a.pos_field] = v.v; }
            p = q + 1;
        }
        if(bad) {
            atomicMin(&status[0], l);
        } else {
            bool inside = true;
            if(a.filter && a.pos_field >= 0) {
                for(int d = 0; d < 3; d++) { inside = inside && pos[d] >= a.lo[d] && pos[d] < a.hi_small[d]; }
            }
            k = (inside || (flags & (kFlagInfinite | kFlagFixed | 8))) ? 1 : 0;
        }
    }
    keep[l] = k;
}

__global__ void k_csv_compact(int32_t lines, int32_t nfields, const int32_t *keep, const int32_t *row,
                              const double *temp, double *table, int32_t max_rows) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if(l >= lines || !keep[l]) { return; }
    const int r = row[l];
    if(r >= max_rows) { return; }
    for(int f = 0; f < nfields; f++) { table[(size_t) f * max_rows + r] = temp[(size_t) f * lines + l]; }
}

// ------------------------------------------------------------------ host side

int64_t csv_count_bytes(int64_t bytes) {
    if(bytes < 0) { return -1; }
    return (int64_t) csv_ws_layout(bytes, 0, 0, nullptr, nullptr);
}

int csv_count_lines(const char *text, int64_t bytes, int64_t *lines, pg_workspace ws, cudaStream_t st) {
    if(!lines || bytes < 0 || bytes >= INT32_MAX || (bytes > 0 && !text)) { return PG_ERR_ARGUMENT; }
    if(!ws.ptr || ws.bytes < csv_count_bytes(bytes)) { return PG_ERR_ARGUMENT; }
    CsvWs w;
    csv_ws_layout(bytes, 0, 0, (char *) ws.ptr, &w);
    const int64_t nc = nchunks_of(bytes);
    int32_t total = 0;
    if(nc > 0) {
        k_csv_count<<<(unsigned) nc, kCsvThreads, 0, st>>>(text, bytes, w.chunk_count); note_launch();
        int rc = scan_exclusive_i32(w.chunk_count, (int) nc, w.chunk_base, w.block_sums, st);
        if(rc) { return rc; }
        if(cudaMemcpyAsync(&total, w.chunk_base + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
           cudaStreamSynchronize(st) != cudaSuccess) {
            return PG_ERR_CUDA;
        }
    }
    // lines: newlines + 1 (a final line without a newline, or an empty one after it)
    *lines = bytes == 0 ? 0 : (int64_t) total + 1;
    return launch_status();
}

int64_t csv_workspace_bytes(int64_t bytes, int64_t lines, int32_t nfields) {
    if(bytes < 0 || lines < 0 || nfields < 1 || nfields > kCsvMaxFields) { return -1; }
    return (int64_t) csv_ws_layout(bytes, lines, nfields, nullptr, nullptr);
}

int csv_parse(const char *text, int64_t bytes, int64_t lines, int32_t nfields, const int32_t *kinds, int32_t pos_field,
              int32_t flags_field, const double *domain_lo, const double *domain_hi, double *table, int32_t max_rows,
              pg_csv_result *result, pg_workspace ws, cudaStream_t st) {
    if(!result || !kinds || nfields < 1 || nfields > kCsvMaxFields || bytes < 0 || bytes >= INT32_MAX) {
        return PG_ERR_ARGUMENT;
    }
    if(lines < 0 || lines >= INT32_MAX || (bytes > 0 && !text) || max_rows < 0 || (max_rows > 0 && !table)) {
        return PG_ERR_ARGUMENT;
    }
    if(pos_field >= 0 && pos_field + 3 > nfields) { return PG_ERR_ARGUMENT; }
    if(flags_field >= nfields || (domain_lo == nullptr) != (domain_hi == nullptr)) { return PG_ERR_ARGUMENT; }
    if(!ws.ptr || ws.bytes < csv_workspace_bytes(bytes, lines, nfields)) { return PG_ERR_ARGUMENT; }
    for(int f = 0; f < nfields; f++) {
        if(kinds[f] != PG_CSV_REAL && kinds[f] != PG_CSV_INT) { return PG_ERR_ARGUMENT; }
    }
    CsvWs w;
    csv_ws_layout(bytes, lines, nfields, (char *) ws.ptr, &w);
    result->rows = 0; result->lines = (int32_t) lines; result->bad_line = -1; result->inexact = 0;
    if(lines == 0) { return PG_OK; }
    CsvArgs a;
    a.text = text; a.bytes = bytes; a.lines = (int32_t) lines; a.nfields = nfields;
    for(int f = 0; f < nfields; f++) { a.kinds[f] = kinds[f]; }
    a.pos_field = pos_field; a.flags_field = flags_field; a.filter = domain_lo != nullptr;
    for(int d = 0; d < 3; d++) {
        a.lo[d] = domain_lo ? domain_lo[d] : 0.0;
        a.hi_small[d] = domain_hi ? domain_hi[d] - 0.00001 : 0.0;
    }
    const int32_t init[4] = {INT32_MAX, 0, 0, 0};
    cudaMemcpyAsync(w.status, init, sizeof(init), cudaMemcpyHostToDevice, st);
    const int64_t nc = nchunks_of(bytes);
    k_csv_count<<<(unsigned) nc, kCsvThreads, 0, st>>>(text, bytes, w.chunk_count); note_launch();
    int rc = scan_exclusive_i32(w.chunk_count, (int) nc, w.chunk_base, w.block_sums, st);
    if(rc) { return rc; }
    k_csv_lines<<<(unsigned) nc, kCsvThreads, 0, st>>>(text, bytes, w.chunk_base, w.line_start); note_launch();
    k_csv_parse<<<blocks_for(lines), kBlock, 0, st>>>(a, w.line_start, w.keep, w.temp, w.status); note_launch();
    rc = scan_exclusive_i32(w.keep, (int) lines, w.row, w.block_sums, st);
    if(rc) { return rc; }
    k_csv_compact<<<blocks_for(lines), kBlock, 0, st>>>((int32_t) lines, nfields, w.keep, w.row, w.temp, table, max_rows);
    note_launch();
    int32_t back[4];
    int32_t rows = 0;
    if(cudaMemcpyAsync(back, w.status, sizeof(back), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaMemcpyAsync(&rows, w.row + lines, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess) {
        return PG_ERR_CUDA;
    }
    result->rows = rows;
    result->bad_line = back[0] == INT32_MAX ? -1 : back[0];
    result->inexact = back[1];
    if(result->bad_line >= 0 || result->inexact > 0) { return PG_ERR_ARGUMENT; }
    if(rows > max_rows) { return PG_ERR_LIMIT; }
    return launch_status();
}

}  // namespace pg
