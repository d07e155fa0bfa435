// Legacy VTK text of the particles, formatted on the device.
//
// The reference writes its particle VTK files from the host with iostreams
// (runtime/vtk.hpp:11-86): POINTS rows "x y z" and the mass rows with std::fixed and
// 8 decimals, CELLS rows "1 k", CELL_TYPES rows "1", skipping infinite shapes.  At
// millions of particles the formatting is the cost, so here every row is formatted by
// its own thread into a fixed-width slot, the row lengths are scanned and the rows
// packed into one contiguous text buffer; the host writes the few header lines and the
// buffer.
//
// The fixed-point conversion is exact: a finite double x = m 2^e gives
// |x| 10^8 = m 5^8 2^(e+8), an integer of at most 72 significant bits shifted by
// e + 8, rounded to the nearest integer with ties to even (the C library's rounding
// of %.8f in the default rounding mode), so the text equals printf("%.8f", x) for
// every |x| < 9.2e10 (larger values return an error).  The sign is printed whenever
// the sign bit is set, as printf does ("-0.00000000").
#include "common.cuh"

namespace pg {

constexpr int kNumWidth = 32;                 // "-" + 11 integer digits + "." + 8 digits, padded
constexpr int kRowWidth = 3 * kNumWidth;      // slot of one row

// Writes x with 8 decimals at p, returns the number of characters, or -1 if |x| is too
// large or not finite.
__host__ __device__ int fmt_fixed8(double x, char *p) {
    unsigned long long bits;
    memcpy(&bits, &x, sizeof bits);
    const bool neg = (bits >> 63) != 0;
    const int bexp = (int) ((bits >> 52) & 0x7ff);
    unsigned long long m = bits & ((1ull << 52) - 1);
    if(bexp == 0x7ff) { return -1; }
    int e;
    if(bexp == 0) { e = -1074; } else { m |= 1ull << 52; e = bexp - 1075; }
    // N = round_half_even(m * 5^8 * 2^(e + 8))
    const unsigned __int128 M = (unsigned __int128) m * 390625u;
    const int s = e + 8;
    unsigned long long N;
    if(M == 0) {
        N = 0;
    } else if(s >= 0) {
        if(s > 40) { return -1; }
        const unsigned __int128 v = M << s;
        if(v >> 63) { return -1; }
        N = (unsigned long long) v;
    } else if(-s >= 127) {
        N = 0;
    } else {
        const int r = -s;
        const unsigned __int128 q = M >> r;
        const unsigned __int128 rem = M - (q << r);
        const unsigned __int128 half = (unsigned __int128) 1 << (r - 1);
        unsigned __int128 n = q;
        if(rem > half || (rem == half && (q & 1))) { n += 1; }
        if(n >> 63) { return -1; }
        N = (unsigned long long) n;
    }
    if(N >= 9200000000000000000ull) { return -1; }
    unsigned long long ip = N / 100000000ull, fp = N % 100000000ull;
    char tmp[24];
    int k = 0;
    do { tmp[k++] = (char) ('0' + ip % 10); ip /= 10; } while(ip);
    int w = 0;
    if(neg) { p[w++] = '-'; }
    while(k) { p[w++] = tmp[--k]; }
    p[w++] = '.';
    for(int d = 7; d >= 0; d--) { p[w + d] = (char) ('0' + fp % 10); fp /= 10; }
    return w + 8;
}

__host__ __device__ int fmt_int(long long v, char *p) {
    char tmp[24];
    int k = 0, w = 0;
    unsigned long long u = v < 0 ? (unsigned long long) (-v) : (unsigned long long) v;
    do { tmp[k++] = (char) ('0' + u % 10); u /= 10; } while(u);
    if(v < 0) { p[w++] = '-'; }
    while(k) { p[w++] = tmp[--k]; }
    return w;
}

// Row k of section `what` (0 points, 1 cells, 2 masses) for particle order[k] into its
// slot; len[k] = characters, or -1 for a value out of range.  The cells row of k names
// index[k] (k when index is null).
__global__ void k_vtk_rows(int what, int n, const int32_t *order, const double *pos, const double *mass,
                           const int32_t *index, char *slots, int32_t *len) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n) { return; }
    const int i = order != nullptr ? order[k] : k;
    char *p = slots + (size_t) k * kRowWidth;
    int w = 0;
    if(what == 0) {
        const double *x = pos + 4 * (size_t) i;
        for(int d = 0; d < 3; d++) {
            const int c = fmt_fixed8(x[d], p + w);
            if(c < 0) { len[k] = -1; return; }
            w += c;
            p[w++] = d < 2 ? ' ' : '\n';
        }
    } else if(what == 1) {
        p[w++] = '1';
        p[w++] = ' ';
        w += fmt_int(index != nullptr ? index[k] : k, p + w);
        p[w++] = '\n';
    } else {
        const int c = fmt_fixed8(mass[i], p);
        if(c < 0) { len[k] = -1; return; }
        w = c;
        p[w++] = '\n';
    }
    len[k] = w;
}

// rows packed at their offsets (an exclusive scan of the lengths), one thread per row
__global__ void k_vtk_pack(int n, const char *slots, const int32_t *len, const int64_t *offset, char *out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n) { return; }
    const int c = len[k];
    const char *src = slots + (size_t) k * kRowWidth;
    char *dst = out + offset[k];
    for(int t = 0; t < c; t++) { dst[t] = src[t]; }
}

int64_t vtk_workspace_bytes(int32_t rows) {
    return rows < 0 ? -1 : (int64_t) rows * (kRowWidth + 4);
}

int vtk_format_rows(int what, int32_t rows, const int32_t *order, const double *pos, const double *mass,
                    const int32_t *index, pg_workspace ws, cudaStream_t st) {
    if(rows < 0 || what < 0 || what > 2 || (what == 0 && !pos) || (what == 2 && !mass)) { return PG_ERR_ARGUMENT; }
    if(ws.ptr == nullptr || ws.bytes < vtk_workspace_bytes(rows)) { return PG_ERR_ARGUMENT; }
    char *slots = reinterpret_cast<char *>(ws.ptr);
    int32_t *len = reinterpret_cast<int32_t *>(slots + (size_t) rows * kRowWidth);
    if(rows > 0) { k_vtk_rows<<<blocks_for(rows), kBlock, 0, st>>>(what, rows, order, pos, mass, index, slots, len); note_launch(); }
    return launch_status();
}

int vtk_pack_rows(int32_t rows, pg_workspace ws, const int64_t *offset, char *out, cudaStream_t st) {
    if(rows < 0 || (rows > 0 && (!offset || !out)) || ws.ptr == nullptr || ws.bytes < vtk_workspace_bytes(rows)) {
        return PG_ERR_ARGUMENT;
    }
    const char *slots = reinterpret_cast<const char *>(ws.ptr);
    const int32_t *len = reinterpret_cast<const int32_t *>(slots + (size_t) rows * kRowWidth);
    if(rows > 0) { k_vtk_pack<<<blocks_for(rows), kBlock, 0, st>>>(rows, slots, len, offset, out); note_launch(); }
    return launch_status();
}

}  // namespace pg
