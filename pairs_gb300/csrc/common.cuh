// Shared device helpers for the GB300 particle kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pairs_gb300.h"

namespace pg {

// 32-byte particle record (x, y, z, unused) of the double4 layout
struct alignas(32) D4 { double x, y, z, w; };

// The replicas of a batched ensemble that take part in a partial rebuild: particle i
// is left alone when rebuild[replica_of[i]] == 0 (rebuild NULL: every particle takes
// part).  Each replica's particles keep their index range, so the mask applies to a
// particle before and after the binning's permutation alike.
struct RepMask {
    const int32_t *rebuild = nullptr;
    const int32_t *replica_of = nullptr;
    __device__ __forceinline__ bool skip(int i) const { return rebuild != nullptr && rebuild[replica_of[i]] == 0; }
};
__host__ __device__ __forceinline__ D4 make_d4(double x, double y, double z, double w) {
    D4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r;
}

constexpr int kBlock = 256;          // threads per block for per-particle kernels
constexpr int kSMs = 152;            // GB300: 2 dies x 76 SMs
constexpr int kFlagInfinite = 1;     // sim/flags.py:1-5
constexpr int kFlagFixed = 4;

inline int blocks_for(int64_t n, int block = kBlock) {
    return (int) ((n + block - 1) / block);
}

// Kernels launched by this library since load (reported by pg_kernel_launches).
extern unsigned long long g_kernel_launches;
inline void note_launch(int k = 1) { __atomic_fetch_add(&g_kernel_launches, (unsigned long long) k, __ATOMIC_RELAXED); }

// Host-side launch check: returns PG_ERR_CUDA when the last launch failed.
inline int launch_status() {
    return cudaPeekAtLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

// --- FP64 loads/stores of the D4 particle layout -----------------------

__device__ __forceinline__ D4 ld_d4(const double *base, int i) {
    const double2 *p = reinterpret_cast<const double2 *>(base) + 2 * (size_t) i;
    double2 a = __ldg(p), b = __ldg(p + 1);
    return make_d4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ D4 ld_d4_plain(const double *base, int i) {
    const double2 *p = reinterpret_cast<const double2 *>(base) + 2 * (size_t) i;
    double2 a = p[0], b = p[1];
    return make_d4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ void st_d4(double *base, int i, D4 v) {
    double2 *p = reinterpret_cast<double2 *>(base) + 2 * (size_t) i;
    p[0] = make_double2(v.x, v.y);
    p[1] = make_double2(v.z, v.w);
}

__device__ __forceinline__ float4 ld_f4(const float *base, int i) {
    return __ldg(reinterpret_cast<const float4 *>(base) + i);
}

__device__ __forceinline__ void st_f4(float *base, int i, float4 v) {
    reinterpret_cast<float4 *>(base)[i] = v;
}

// --- periodic image codes: 2 bits per dimension, 0 none, 1 +len, 2 -len -------

__device__ __forceinline__ int image_shift(uint32_t code, int d) {
    const uint32_t c = (code >> (2 * d)) & 3u;
    return c == 1u ? 1 : (c == 2u ? -1 : 0);
}

__device__ __forceinline__ uint32_t image_code(int sx, int sy, int sz) {
    auto enc = [](int s) -> uint32_t { return s > 0 ? 1u : (s < 0 ? 2u : 0u); };
    return enc(sx) | (enc(sy) << 2) | (enc(sz) << 4);
}

__device__ __forceinline__ int image_dims(uint32_t code) {
    return ((code & 3u) != 0) + (((code >> 2) & 3u) != 0) + (((code >> 4) & 3u) != 0);
}

// Exact-as-the-reference FP64 squared distance between particle position xi and
// the image fl(xj + s*len) of xj: every operation separately rounded, in the
// generated order (dx*dx + dy*dy) + dz*dz (sim/interaction.py:223-227).
__device__ __forceinline__ double ref_image(double xj, int s, double len) {
    return s == 0 ? xj : __dadd_rn(xj, s > 0 ? len : -len);
}

__device__ __forceinline__ double ref_rsq(double dx, double dy, double dz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Cutoff decision of the FP32 force paths.  The truncated LJ force jumps by |F(rc)|
// (0.039 at rc = 2.5) at the cutoff, so a pair within FP32 rounding of rc that one
// precision counts and the other does not changes a force by that much.  A pair whose
// FP32 rsq lies within a relative band of kCutBand around rc^2 is therefore decided by
// the FP64 path's own test (the reference's rsq of the listed image, FP64 positions):
// both precisions apply the force of exactly the same pairs.
constexpr float kCutBand = 1.0e-5f;

// FP64 position load for a rarely taken branch: volatile, so the compiler neither
// hoists it out of the branch nor keeps it live in registers across a loop
__device__ __forceinline__ D4 ld_d4_rare(const double *base, int i) {
    const double *p = base + 4 * (size_t) i;
    double x, y, z;
    asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "l"(p));
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(z) : "l"(p + 2));
    return make_d4(x, y, z, 0.0);
}

__device__ __forceinline__ bool exact_inside(const double *pos, int i, int j, uint32_t code, const double *len,
                                             double cutoff2) {
    const D4 xi = ld_d4_rare(pos, i), xj = ld_d4_rare(pos, j);
    const double jx = ref_image(xj.x, image_shift(code, 0), len[0]);
    const double jy = ref_image(xj.y, image_shift(code, 1), len[1]);
    const double jz = ref_image(xj.z, image_shift(code, 2), len[2]);
    return ref_rsq(__dsub_rn(xi.x, jx), __dsub_rn(xi.y, jy), __dsub_rn(xi.z, jz)) < cutoff2;
}

__device__ __forceinline__ void red_add_v4(float *addr, float a, float b, float c) {
    // one vector reduction to L2 instead of three scalar atomics (sm_90+)
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};"
                 :: "l"(addr), "f"(a), "f"(b), "f"(c), "f"(0.0f) : "memory");
}

// Queue of near-cutoff pairs (particle, list entry) for a second, FP64-deciding pass.
__device__ __forceinline__ void cut_queue_push(int32_t *count, int2 *rec, int capacity, int i, uint32_t e) {
    const int slot = atomicAdd(count, 1);
    if(slot < capacity) { rec[slot] = make_int2(i, (int) e); }
}

// --- compensated FP32 positions ------------------------------------------------
// hi = x rounded to a multiple of the box quantum q (a power of two chosen so every
// |hi| < 2^24 q): differences of hi values and of hi and len_hi are exact in FP32.
// lo = x - hi in FP32 (|lo| <= q/2).

// float4 index of particle i in pos_hi / pos_lo (interleaved records: stride 2)
__device__ __forceinline__ int hl(const pg_particles &p, int i) { return p.hilo_stride == 2 ? 2 * i : i; }

__device__ __forceinline__ void split_pos(double x, double inv_q, double q, float &hi, float &lo) {
    const double h = rint(x * inv_q) * q;
    hi = (float) h;
    lo = (float) (x - h);
}

// FP32 reciprocal by the hardware approximation (PTX rcp.approx: at most 1 ulp from
// the rounded reciprocal over the normal range), one instruction instead of the
// correctly rounded sequence; the mixed-precision force paths use it.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// --- fixed-point positions (pg_particles.pos_fx) ---------------------------------
// x_fx = round((x - lo) * 2^32 / len) mod 2^32 per axis.  One box length is 2^32
// units, so the wrapped 32-bit difference of two coordinates is the minimum-image
// separation in units, exact as an integer whenever that separation is below half a
// box length; no periodic shift is needed.  The unit (len / 2^32 = 2.5e-8 at len =
// 107.5) is far below the FP32 rounding of a pair distance near 1, and the integer
// difference converts to FP32 with one rounding.

__device__ __forceinline__ int32_t to_fx(double x, double lo, double scale) {
    return (int32_t) (uint32_t) (unsigned long long) __double2ll_rn((x - lo) * scale);
}

__device__ __forceinline__ int4 fx_position(const pg_box &box, double x, double y, double z, int type) {
    return make_int4(to_fx(x, box.lo[0], box.fx_scale[0]), to_fx(y, box.lo[1], box.fx_scale[1]),
                     to_fx(z, box.lo[2], box.fx_scale[2]), type);
}

// fixed-point position on a batched-ensemble replica's own box (2^32 units per length)
__device__ __forceinline__ int4 replica_fx(const pg_replica &R, double x, double y, double z, int type) {
    return make_int4(to_fx(x, R.lo[0], R.fx_scale[0]), to_fx(y, R.lo[1], R.fx_scale[1]),
                     to_fx(z, R.lo[2], R.fx_scale[2]), type);
}

// wrapped difference a - b of two fixed-point coordinates
__device__ __forceinline__ int fx_diff(int32_t a, int32_t b) { return (int) ((uint32_t) a - (uint32_t) b); }

__device__ __forceinline__ int4 ld_i4(const int32_t *base, int i) {
    return __ldg(reinterpret_cast<const int4 *>(base) + i);
}

__device__ __forceinline__ void st_i4(int32_t *base, int i, int4 v) {
    reinterpret_cast<int4 *>(base)[i] = v;
}

// Speculative stepping (see pg_particles.guard): a force pass of step p.step is
// skipped once the guard tripped at a step <= p.step, an integration pass once it
// tripped before p.step.  Every thread reads the same word (one broadcast load).
__device__ __forceinline__ bool frozen_force(const pg_particles &p) {
    return p.guard != nullptr && *((volatile const int32_t *) p.guard) <= p.step;
}

__device__ __forceinline__ bool frozen_integrate(const pg_particles &p) {
    return p.guard != nullptr && *((volatile const int32_t *) p.guard) < p.step;
}

// FP32 Lennard-Jones table (mixed precision kernels), up to 8 types
struct LJTableF {
    int ntypes;
    float cutoff2;
    double cutoff2d;             // the FP64 cutoff test near rc (kCutBand)
    float eps[64];
    float sig6[64];
};

// warp/block reductions
__device__ __forceinline__ double warp_sum(double v) {
    for(int o = 16; o > 0; o >>= 1) { v += __shfl_xor_sync(0xffffffffu, v, o); }
    return v;
}

// The partner of a half-list pair in the particle's own x slab of the stencil is
// kept when it lies above: (x, y, z) of the partner greater in that order, the index
// breaking exact ties.  d = x_i - x_j from the screen is exactly antisymmetric between
// the two sides of a pair (an integer difference in fixed point; in the compensated
// layout the hi difference is exact and round-to-nearest is symmetric in sign), so
// exactly one side keeps the pair.
__device__ __forceinline__ bool partner_above(float dx, float dy, float dz, int i, int j) {
    if(dx != 0.0f) { return dx < 0.0f; }
    if(dy != 0.0f) { return dy < 0.0f; }
    if(dz != 0.0f) { return dz < 0.0f; }
    return j > i;
}

__device__ __forceinline__ int warp_max(int v) {
    for(int o = 16; o > 0; o >>= 1) { v = max(v, __shfl_xor_sync(0xffffffffu, v, o)); }
    return v;
}

// Publish a list build's per-particle count: the largest count of the lanes that
// reach this call together goes to status->max_neighbors and, past the list's
// capacity, sets overflow bit 2.  Lanes past the particle range return early in the
// list kernels, so the maximum is taken over the active lanes only (redux.sync over
// __activemask()) and the lowest of them publishes; a full-mask shuffle would read
// exited lanes.
__device__ __forceinline__ void publish_count(int cnt, int capacity, pg_status *status) {
    const unsigned m = __activemask();
    const int wm = __reduce_max_sync(m, cnt);
    if((threadIdx.x & 31) == (unsigned) (__ffs(m) - 1) && wm > 0) {
        atomicMax(&status->max_neighbors, wm);
        if(wm > capacity) { atomicOr(&status->overflow, 2); }
    }
}

// FP32 squared distance with a fixed operation order (no contraction left to the
// compiler), so that every kernel that screens a pair against the cutoff band takes
// the same decision for it.
__device__ __forceinline__ float pair_rsq(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

}  // namespace pg
