// Shared device helpers for the GB300 particle kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pairs_gb300.h"

namespace pg {

// 32-byte particle record (x, y, z, unused) of the double4 layout
struct alignas(32) D4 { double x, y, z, w; };
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
    float eps[64];
    float sig6[64];
};

// warp/block reductions
__device__ __forceinline__ double warp_sum(double v) {
    for(int o = 16; o > 0; o >>= 1) { v += __shfl_xor_sync(0xffffffffu, v, o); }
    return v;
}

__device__ __forceinline__ int warp_max(int v) {
    for(int o = 16; o > 0; o >>= 1) { v = max(v, __shfl_xor_sync(0xffffffffu, v, o)); }
    return v;
}

}  // namespace pg
