// The DEM simple-cubic initialiser on the device.
//
// Replaces the reference's dem_sc_grid (runtime/dem_sc_grid.hpp:62-172) on one rank:
// grid points ref + k * spacing (ref = spacing / 2) inside [0, xmax) x [0, ymax) x
// [diameter, zmax), visited x fastest.  Every visited point draws a diameter from a
// default-seeded std::mt19937 (std::uniform_real_distribution over libstdc++'s
// generate_canonical<double, 53>: two 32-bit words per draw); a point inside the domain
// [lo, hi - 1e-5) becomes a sphere with uid = its visit number + 1, radius d / 2, mass
// 4/3 pi r^3 density, velocity (0.1 U(-v0, v0), 0.1 U(-v0, v0), -v0) from two more draws
// of the same engine, and type rand() % ntypes (glibc rand() after the default seed).
//
// The draws of point p start at word 2 (p + 2 * kept_before(p)).  The grid and the
// domain are boxes, so kept_before has a closed form from per-axis prefix counts, and
// one thread per point computes its sphere independently.  The two random sequences
// are generated first: MT19937 by one block (each twist of the 624-word state in four
// dependency phases of parallel updates), glibc's additive generator (r[i] = r[i-3] +
// r[i-31] mod 2^32, output r[i] >> 1) by one thread.  Every FP64 operation is the
// reference's, separately rounded in its order, so the result is bit-identical.
#include <math.h>

#include <vector>

#include "common.cuh"

namespace pg {

constexpr int kMtN = 624;
constexpr int kMtThreads = 640;

// tempered outputs of std::mt19937(5489), words [0, nwords)
__global__ void __launch_bounds__(kMtThreads) k_mt19937(uint32_t *out, int64_t nwords) {
    __shared__ uint32_t mt[kMtN];
    const int i = threadIdx.x;
    if(i == 0) {
        mt[0] = 5489u;
        for(int k = 1; k < kMtN; k++) { mt[k] = 1812433253u * (mt[k - 1] ^ (mt[k - 1] >> 30)) + (uint32_t) k; }
    }
    __syncthreads();
    // phase p updates the words [lo_p, hi_p): each reads mt[i] and mt[i + 1] (old) and
    // mt[(i + 397) % 624] (old in phase 0, new in the later phases)
    const int lo[4] = {0, 227, 454, 623}, hi[4] = {227, 454, 623, 624};
    for(int64_t base = 0; base < nwords; base += kMtN) {
        for(int p = 0; p < 4; p++) {
            uint32_t v = 0u;
            const bool mine = i >= lo[p] && i < hi[p];
            if(mine) {
                const uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % kMtN] & 0x7fffffffu);
                v = mt[(i + 397) % kMtN] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            __syncthreads();                 // every read of this phase before any write
            if(mine) { mt[i] = v; }
            __syncthreads();
        }
        if(i < kMtN && base + i < nwords) {
            uint32_t y = mt[i];
            y ^= y >> 11;
            y ^= (y << 7) & 0x9d2c5680u;
            y ^= (y << 15) & 0xefc60000u;
            y ^= y >> 18;
            out[base + i] = y;
        }
        __syncthreads();
    }
}

// the first `count` outputs of glibc rand() after srand(1)
__global__ void k_glibc_rand(int32_t *out, int64_t count) {
    if(blockIdx.x != 0 || threadIdx.x != 0) { return; }
    uint32_t r[34];
    int32_t w = 1;
    r[0] = 1u;
    for(int i = 1; i < 31; i++) {
        const int32_t hi = w / 127773, lo = w % 127773;
        w = 16807 * lo - 2836 * hi;
        if(w < 0) { w += 2147483647; }
        r[i] = (uint32_t) w;
    }
    for(int i = 31; i < 34; i++) { r[i] = r[i - 31]; }
    // ring of the last 34 values; value i sits at i % 34
    for(int64_t i = 34; i < 344 + count; i++) {
        const uint32_t v = r[(i - 31) % 34] + r[(i - 3) % 34];
        r[i % 34] = v;
        if(i >= 344) { out[i - 344] = (int32_t) (v >> 1); }
    }
}

struct ScGridArgs {
    int nx, ny, nz;                  // visited points per axis
    int kx, ky, kz;                  // of which inside the domain
    const double *axis[3];           // coordinates of the visited points per axis
    const int32_t *inside[3];        // 0/1 per axis point
    const int32_t *before[3];        // inside points below each axis point
    const uint32_t *words;
    const int32_t *rnd;
    double dmin, dmax, v0, density;
    int ntypes;
    double *pos, *vel, *mass, *radius;
    int32_t *type, *uid;
};

__device__ __forceinline__ double canonical(const uint32_t *words, int64_t k) {
    // (a + b * 2^32) / 2^64 with a the first word, rounded once in the sum, below 1
    const double a = (double) words[2 * k], b = (double) words[2 * k + 1];
    const double r = __dmul_rn(__dadd_rn(a, __dmul_rn(b, 4294967296.0)), 0x1p-64);
    return r >= 1.0 ? 0x1.fffffffffffffp-1 : r;
}

__global__ void k_sc_points(ScGridArgs a) {
    const int64_t p = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t npts = (int64_t) a.nx * a.ny * a.nz;
    if(p >= npts) { return; }
    const int ix = (int) (p % a.nx), iy = (int) ((p / a.nx) % a.ny), iz = (int) (p / ((int64_t) a.nx * a.ny));
    const bool in_z = a.inside[2][iz] != 0, in_y = a.inside[1][iy] != 0, in_x = a.inside[0][ix] != 0;
    int64_t kept = (int64_t) a.before[2][iz] * a.ky * a.kx;
    if(in_z) { kept += (int64_t) a.before[1][iy] * a.kx; }
    if(in_z && in_y) { kept += a.before[0][ix]; }
    if(!(in_x && in_y && in_z)) { return; }
    const int64_t first = p + 2 * kept;         // this point's first draw
    const double diam = __dadd_rn(__dmul_rn(canonical(a.words, first), __dsub_rn(a.dmax, a.dmin)), a.dmin);
    const double span = __dsub_rn(a.v0, -a.v0);
    const double vx = __dmul_rn(0.1, __dadd_rn(__dmul_rn(canonical(a.words, first + 1), span), -a.v0));
    const double vy = __dmul_rn(0.1, __dadd_rn(__dmul_rn(canonical(a.words, first + 2), span), -a.v0));
    const double rad = __dmul_rn(diam, 0.5);
    const double c = __dmul_rn(__ddiv_rn(4.0, 3.0), 3.141592653589793);      // (4/3) pi, as the reference
    const double m = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(c, rad), rad), rad), a.density);
    st_d4(a.pos, (int) kept, make_d4(a.axis[0][ix], a.axis[1][iy], a.axis[2][iz], 0.0));
    st_d4(a.vel, (int) kept, make_d4(vx, vy, -a.v0, 0.0));
    a.mass[kept] = m;
    a.radius[kept] = rad;
    a.type[kept] = a.rnd[kept] % a.ntypes;
    a.uid[kept] = (int32_t) (p + 1);
}

// ------------------------------------------------------------------ host side

struct ScAxes {
    std::vector<double> v[3];
    std::vector<int32_t> in[3], before[3];
    int k[3];
};

static void sc_axes(double xmax, double ymax, double zmax, double spacing, double diameter, const double *lo,
                    const double *hi, ScAxes &ax) {
    const double glo[3] = {0.0, 0.0, diameter}, ghi[3] = {xmax, ymax, zmax};
    const double ref = spacing * 0.5;
    for(int d = 0; d < 3; d++) {
        ax.v[d].clear(); ax.in[d].clear(); ax.before[d].clear();
        int k = (int) ceil((glo[d] - ref) / spacing);
        int count = 0;
        for(;; k++) {
            const double x = ref + k * spacing;
            if(!(x >= glo[d] && x < ghi[d])) { break; }
            const bool in = x >= lo[d] && x < hi[d] - 0.00001;
            ax.v[d].push_back(x);
            ax.before[d].push_back(count);
            ax.in[d].push_back(in ? 1 : 0);
            count += in ? 1 : 0;
            if(ax.v[d].size() > (1u << 24)) { break; }
        }
        ax.k[d] = count;
    }
}

static size_t sc_align(size_t x) { return (x + 255) & ~(size_t) 255; }

static size_t sc_axis_bytes(size_t n) { return sc_align(n * 8) + 2 * sc_align(n * 4); }

static size_t sc_ws_bytes(const ScAxes &ax, int64_t npts, int64_t kept) {
    const int64_t draws = npts + 2 * kept;
    return sc_align((size_t) draws * 8) + sc_align((size_t) kept * 4) + sc_axis_bytes(ax.v[0].size()) +
           sc_axis_bytes(ax.v[1].size()) + sc_axis_bytes(ax.v[2].size());
}

int dem_sc_grid_size(double xmax, double ymax, double zmax, double spacing, double diameter, const double *lo,
                     const double *hi, int64_t *npoints, int64_t *nkept, int64_t *ws_bytes) {
    if(!lo || !hi || !npoints || !nkept || !ws_bytes || !(spacing > 0.0) || !isfinite(spacing)) {
        return PG_ERR_ARGUMENT;
    }
    ScAxes ax;
    sc_axes(xmax, ymax, zmax, spacing, diameter, lo, hi, ax);
    *npoints = (int64_t) ax.v[0].size() * ax.v[1].size() * ax.v[2].size();
    *nkept = (int64_t) ax.k[0] * ax.k[1] * ax.k[2];
    *ws_bytes = (int64_t) sc_ws_bytes(ax, *npoints, *nkept);
    return PG_OK;
}

int dem_sc_grid(double xmax, double ymax, double zmax, double spacing, double diameter, double min_diameter,
                double max_diameter, double initial_velocity, double density, int ntypes, const double *lo,
                const double *hi, double *pos, double *vel, double *mass, double *radius, int32_t *type,
                int32_t *uid, int64_t capacity, pg_workspace ws, cudaStream_t st) {
    if(!lo || !hi || !(spacing > 0.0) || !isfinite(spacing) || ntypes < 1) { return PG_ERR_ARGUMENT; }
    ScAxes ax;
    sc_axes(xmax, ymax, zmax, spacing, diameter, lo, hi, ax);
    const int64_t n3[3] = {(int64_t) ax.v[0].size(), (int64_t) ax.v[1].size(), (int64_t) ax.v[2].size()};
    const int64_t npts = n3[0] * n3[1] * n3[2];
    const int64_t kept = (int64_t) ax.k[0] * ax.k[1] * ax.k[2];
    if(kept > capacity || kept >= INT32_MAX || npts >= INT32_MAX) { return PG_ERR_ARGUMENT; }
    if(kept > 0 && (!pos || !vel || !mass || !radius || !type || !uid)) { return PG_ERR_ARGUMENT; }
    if(!ws.ptr || ws.bytes < (int64_t) sc_ws_bytes(ax, npts, kept)) { return PG_ERR_ARGUMENT; }
    if(kept == 0) { return PG_OK; }
    char *base = (char *) ws.ptr;
    const int64_t draws = npts + 2 * kept;
    uint32_t *words = (uint32_t *) base;
    base += sc_align((size_t) draws * 8);
    int32_t *rnd = (int32_t *) base;
    base += sc_align((size_t) kept * 4);
    ScGridArgs a;
    for(int d = 0; d < 3; d++) {
        char *axis = base;
        const size_t n = ax.v[d].size();
        base += sc_axis_bytes(n);
        double *v = (double *) axis;
        int32_t *in = (int32_t *) (axis + sc_align(n * 8));
        int32_t *before = (int32_t *) (axis + sc_align(n * 8) + sc_align(n * 4));
        cudaMemcpyAsync(v, ax.v[d].data(), n * 8, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(in, ax.in[d].data(), n * 4, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(before, ax.before[d].data(), n * 4, cudaMemcpyHostToDevice, st);
        a.axis[d] = v; a.inside[d] = in; a.before[d] = before;
    }
    a.nx = (int) n3[0]; a.ny = (int) n3[1]; a.nz = (int) n3[2];
    a.kx = ax.k[0]; a.ky = ax.k[1]; a.kz = ax.k[2];
    a.words = words; a.rnd = rnd;
    a.dmin = min_diameter; a.dmax = max_diameter; a.v0 = initial_velocity; a.density = density; a.ntypes = ntypes;
    a.pos = pos; a.vel = vel; a.mass = mass; a.radius = radius; a.type = type; a.uid = uid;
    k_mt19937<<<1, kMtThreads, 0, st>>>(words, 2 * draws); note_launch();
    k_glibc_rand<<<1, 1, 0, st>>>(rnd, kept); note_launch();
    k_sc_points<<<blocks_for(npts), kBlock, 0, st>>>(a); note_launch();
    // the axis arrays are host vectors copied asynchronously: wait before they go away
    if(cudaStreamSynchronize(st) != cudaSuccess) { return PG_ERR_CUDA; }
    return launch_status();
}

}  // namespace pg
