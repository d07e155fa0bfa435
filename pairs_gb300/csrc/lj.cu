// Lennard-Jones pair forces over the Verlet list.
//
// The reference's lennard_jones module (examples/md.py:5-8 lowered by
// sim/interaction.py:222-232 and ir/apply.py:112-125):
//   rsq < rc^2:  sr2 = 1/rsq;  sr6 = sr2^3 sigma6[ti,tj];
//                F_i += delta * 48 sr6 (sr6 - 1/2) sr2 epsilon[ti,tj]
// with a full list (every pair seen from both sides, no atomics) or a half list
// (each interior pair once, the reaction -f applied to the partner with an atomic
// add; pairs through a periodic image are in both lists and get no reaction, as the
// reference's ghost images).
//
// Two precisions:
//   FP64   every operation in double; the cutoff test uses the reference's exact
//          rsq (no fused multiply-add) so the same pairs interact.
//   MIXED  delta from fixed-point positions (2^32 units per box length) or from
//          compensated FP32 positions (hi on a 2^-k grid, lo residual), force
//          arithmetic and accumulation in FP32; optional energy/virial in FP64.
//
// One thread per particle: consecutive threads read consecutive entries of the
// column-major list (coalesced 128-byte rows), partner positions are gathered from
// the cell-sorted arrays (mostly L1/L2 hits).  The list stream is the dominant DRAM
// traffic: 4 bytes per entry, read with the streaming (evict-first) cache hint.
#include <algorithm>

#include "common.cuh"
#include "lj_packed.cuh"

namespace pg {

struct ForceArgs {
    pg_box box;
    pg_particles p;
    pg_neighbor_list list;
    LJTable lj;
    int sync_ref;
    double *energy;
    int32_t *cut_count;          // pairs within the cutoff band (mixed path), and their
    int2 *cut_rec;               // records (particle, list entry)
    int cut_capacity;
};

__device__ __forceinline__ void block_add_energy(double pe, double vir, double *energy) {
    __shared__ double s[2][kBlock / 32];
    pe = warp_sum(pe);
    vir = warp_sum(vir);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if(lane == 0) { s[0][w] = pe; s[1][w] = vir; }
    __syncthreads();
    if(threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for(int k = 0; k < (int) (blockDim.x >> 5); k++) { a += s[0][k]; b += s[1][k]; }
        atomicAdd(&energy[0], a);
        atomicAdd(&energy[1], b);
    }
}

// ---------------------------------------------------------------------------- FP64

template<bool kHalf, bool kOneType, bool kEnergy>
__global__ void __launch_bounds__(kBlock) k_lj_fp64(ForceArgs a) {
    if(frozen_force(a.p)) { return; }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0, vir = 0.0;
    if(i < a.p.n) {
        const bool fixed = a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed);
        double fx = 0.0, fy = 0.0, fz = 0.0;
        if(!fixed) {
            const D4 xi = ld_d4(a.p.pos, i);
            const int ti = kOneType ? 0 : a.p.type[i] * a.lj.ntypes;
            const int cnt = a.list.count[i];
            const int32_t *nb = a.list.nbr + i;
            const int stride = a.list.stride;
            const int since = a.list.steps_since_build;
            for(int k = 0; k < cnt; k++) {
                const uint32_t e = (uint32_t) __ldcs(nb + (size_t) k * stride);
                const int j = (int) (e & PG_NBR_INDEX_MASK);
                const uint32_t code = e >> PG_NBR_INDEX_BITS;
                const double *base = a.p.pos;
                if(a.sync_ref && code != 0u) {
                    const int lag = min(max(image_dims(code) - 1, 0), since);
                    base = lag == 0 ? a.p.pos : (lag == 1 ? a.p.pos_prev1 : a.p.pos_prev2);
                }
                const D4 xj = ld_d4(base, j);
                double jx = xj.x, jy = xj.y, jz = xj.z;
                if(code != 0u) {
                    jx = ref_image(jx, image_shift(code, 0), a.box.len[0]);
                    jy = ref_image(jy, image_shift(code, 1), a.box.len[1]);
                    jz = ref_image(jz, image_shift(code, 2), a.box.len[2]);
                }
                const double dx = __dsub_rn(xi.x, jx), dy = __dsub_rn(xi.y, jy), dz = __dsub_rn(xi.z, jz);
                const double rsq = ref_rsq(dx, dy, dz);
                if(rsq < a.lj.cutoff2) {
                    const int tij = kOneType ? 0 : ti + a.p.type[j];
                    const double sr2 = 1.0 / rsq;
                    const double sr6 = sr2 * sr2 * sr2 * a.lj.sig6[tij];
                    const double f = 48.0 * sr6 * (sr6 - 0.5) * sr2 * a.lj.eps[tij];
                    // separately rounded, in the generated order (tmp = tmp + delta*f)
                    const double ex = __dmul_rn(dx, f), ey = __dmul_rn(dy, f), ez = __dmul_rn(dz, f);
                    fx = __dadd_rn(fx, ex); fy = __dadd_rn(fy, ey); fz = __dadd_rn(fz, ez);
                    if(kHalf && code == 0u) {
                        double *fj = a.p.force + 4 * (size_t) j;
                        atomicAdd(fj + 0, -ex); atomicAdd(fj + 1, -ey); atomicAdd(fj + 2, -ez);
                    }
                    if(kEnergy) {
                        const double w = (kHalf && code == 0u) ? 1.0 : 0.5;
                        pe += w * 4.0 * a.lj.eps[tij] * (sr6 * sr6 - sr6);
                        vir += w * (dx * ex + dy * ey + dz * ez);
                    }
                }
            }
        }
        double *fi = a.p.force + 4 * (size_t) i;
        if(kHalf) {
            atomicAdd(fi + 0, fx); atomicAdd(fi + 1, fy); atomicAdd(fi + 2, fz);
        } else {
            st_d4(a.p.force, i, make_d4(fx, fy, fz, 0.0));
        }
    }
    if(kEnergy) { block_add_energy(pe, vir, a.energy); }
}

// ---------------------------------------------------------------------------- MIXED

// kFixed: positions from pos_fx (fixed point, 2^32 units per box length).  The wrapped
// 32-bit difference of two coordinates is the pair's minimum-image separation, which
// is the listed image's as long as the pair stays closer than half a box length (the
// list is rebuilt long before: the box spans at least 4 cells of r_list), so no image
// shift is applied and one 16-byte load per partner carries position and type.
//
// The list is walked in batches of kBatch entries.  The reaction of a pair is a `red`
// with a memory clobber, which no load may pass, so a plain loop would issue the next
// list load only after the previous pair is done and wait a full DRAM round trip per
// entry.  Here the next batch's entries are loaded before the current batch's pairs
// are computed, and a batch's partner gathers are issued together.
#ifndef PG_LJ_BATCH
#define PG_LJ_BATCH 4
#endif
constexpr int kBatch = PG_LJ_BATCH;

// Pair separation on the mixed path: fixed point (wrapped difference, no image shift)
// or compensated hi/lo with the listed image's exact shift.
template<bool kFixed>
__device__ __forceinline__ void mixed_delta(const ForceArgs &a, int4 fi, float4 hi, float4 lo, int4 fj, float4 hj,
                                            float4 lj, uint32_t code, float &dx, float &dy, float &dz) {
    if(kFixed) {
        dx = (float) fx_diff(fi.x, fj.x) * a.box.fx_unit[0];
        dy = (float) fx_diff(fi.y, fj.y) * a.box.fx_unit[1];
        dz = (float) fx_diff(fi.z, fj.z) * a.box.fx_unit[2];
    } else {
        float dlx = lo.x - lj.x, dly = lo.y - lj.y, dlz = lo.z - lj.z;
        float dhx = hi.x - hj.x, dhy = hi.y - hj.y, dhz = hi.z - hj.z;
        if(code != 0u) {
            const int sx = image_shift(code, 0), sy = image_shift(code, 1), sz = image_shift(code, 2);
            dhx -= sx * a.box.len_hi[0]; dlx -= sx * a.box.len_lo[0];
            dhy -= sy * a.box.len_hi[1]; dly -= sy * a.box.len_lo[1];
            dhz -= sz * a.box.len_hi[2]; dlz -= sz * a.box.len_lo[2];
        }
        dx = dhx + dlx; dy = dhy + dly; dz = dhz + dlz;
    }
}

// Queue a near-cutoff pair for k_lj_cutoff_fixup.  The expected load is a few pairs
// per thousand particles against a capacity of several per particle.
__device__ __forceinline__ void cut_push(const ForceArgs &a, int i, uint32_t e) {
    cut_queue_push(a.cut_count, a.cut_rec, a.cut_capacity, i, e);
}

// FP32 LJ pair force factor f (F_i = delta * f) and sr6
__device__ __forceinline__ float mixed_lj(const ForceArgs &a, int tij, float rsq, float &sr6) {
    const float sr2 = rcp_approx(rsq);
    sr6 = sr2 * sr2 * sr2 * a.lj.sig6f[tij];
    return 48.0f * sr6 * (sr6 - 0.5f) * sr2 * a.lj.epsf[tij];
}

template<bool kHalf, bool kOneType, bool kEnergy, bool kFixed>
__global__ void __launch_bounds__(kBlock) k_lj_mixed(ForceArgs a) {
    if(frozen_force(a.p)) { return; }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0, vir = 0.0;
    if(i < a.p.n) {
        const bool fixed = a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed);
        float fx = 0.0f, fy = 0.0f, fz = 0.0f;
        if(!fixed) {
            float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
            int4 fi = make_int4(0, 0, 0, 0);
            if(kFixed) {
                fi = ld_i4(a.p.pos_fx, i);
            } else {
                hi = ld_f4(a.p.pos_hi, hl(a.p, i));
                lo = ld_f4(a.p.pos_lo, hl(a.p, i));
            }
            const int ti = kOneType ? 0 : (kFixed ? fi.w : __float_as_int(hi.w)) * a.lj.ntypes;
            const int cnt = a.list.count[i];
            const int32_t *nb = a.list.nbr + i;
            const size_t stride = (size_t) a.list.stride;
            const float c2 = a.lj.cutoff2f, band = c2 * kCutBand;
            // one list entry.  A pair inside the band around the cutoff is left out here
            // and queued after its batch (returns true); k_lj_cutoff_fixup decides it in
            // FP64.
            auto pair = [&](uint32_t e, float4 hj, float4 lj, int4 fj) -> bool {
                const int j = (int) (e & PG_NBR_INDEX_MASK);
                const uint32_t code = e >> PG_NBR_INDEX_BITS;
                float dx, dy, dz;
                mixed_delta<kFixed>(a, fi, hi, lo, fj, hj, lj, code, dx, dy, dz);
                const float rsq = pair_rsq(dx, dy, dz);
                const bool near = fabsf(rsq - c2) < band;
                if(rsq < c2 && !near) {
                    const int tij = kOneType ? 0 : ti + (kFixed ? fj.w : __float_as_int(hj.w));
                    float sr6;
                    const float f = mixed_lj(a, tij, rsq, sr6);
                    fx += dx * f; fy += dy * f; fz += dz * f;
                    if(kHalf && code == 0u) { red_add_v4(a.p.force32 + 4 * (size_t) j, -dx * f, -dy * f, -dz * f); }
                    if(kEnergy) {
                        const double w = (kHalf && code == 0u) ? 1.0 : 0.5;
                        pe += w * 4.0 * (double) a.lj.epsf[tij] * ((double) sr6 * (double) sr6 - (double) sr6);
                        vir += w * (double) (rsq * f);
                    }
                }
                return near;
            };
            uint32_t cur[kBatch];
#pragma unroll
            for(int u = 0; u < kBatch; u++) { cur[u] = u < cnt ? (uint32_t) __ldcs(nb + u * stride) : 0u; }
            for(int k0 = 0; k0 < cnt; k0 += kBatch) {
                float4 hj[kBatch], lj[kBatch];
                int4 fj[kBatch];
#pragma unroll
                for(int u = 0; u < kBatch; u++) {
                    const int j = (int) (cur[u] & PG_NBR_INDEX_MASK);      // 0 past the end: a valid row
                    if(kFixed) {
                        fj[u] = ld_i4(a.p.pos_fx, j);
                        hj[u] = lj[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    } else {
                        hj[u] = ld_f4(a.p.pos_hi, hl(a.p, j));
                        lj[u] = ld_f4(a.p.pos_lo, hl(a.p, j));
                        fj[u] = make_int4(0, 0, 0, 0);
                    }
                }
                uint32_t nxt[kBatch];
                const int32_t *nbn = nb + (size_t) (k0 + kBatch) * stride;
#pragma unroll
                for(int u = 0; u < kBatch; u++) {
                    nxt[u] = k0 + kBatch + u < cnt ? (uint32_t) __ldcs(nbn + u * stride) : 0u;
                }
                uint32_t pending = 0u;
#pragma unroll
                for(int u = 0; u < kBatch; u++) {
                    if(k0 + u < cnt && pair(cur[u], hj[u], lj[u], fj[u])) { pending |= 1u << u; }
                }
                if(pending != 0u) {
#pragma unroll
                    for(int u = 0; u < kBatch; u++) {
                        if(pending & (1u << u)) { cut_push(a, i, cur[u]); }
                    }
                }
#pragma unroll
                for(int u = 0; u < kBatch; u++) { cur[u] = nxt[u]; }
            }
        }
        if(kHalf) {
            red_add_v4(a.p.force32 + 4 * (size_t) i, fx, fy, fz);
        } else {
            st_f4(a.p.force32, i, make_float4(fx, fy, fz, 0.0f));
        }
    }
    if(kEnergy) { block_add_energy(pe, vir, a.energy); }
}

// Fixed-point positions without energy sums (every step of the time loop): the pair
// arithmetic of two list entries at a time in packed FP32 (Blackwell's f32x2 multiply,
// add and fused multiply-add: one instruction for both pairs).  Each pair rounds as
// in k_lj_mixed: the squared distance in the order of pair_rsq, so the cutoff band
// holds the same pairs, and the force factor 48 sr6 (sr6 - 1/2) sr2 eps in FP32.
// Measured on a 1M-atom liquid: 4-7% fewer cycles than one entry at a time; half
// lists walk 4 entries per batch, full lists 2.
constexpr int kPackedBlock = 128;

template<bool kHalf, bool kOneType, int kB>
__global__ void __launch_bounds__(kPackedBlock) k_lj_packed(ForceArgs a) {
    if(frozen_force(a.p)) { return; }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.p.n) { return; }
    float3 f = make_float3(0.0f, 0.0f, 0.0f);
    if(!(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed))) {
        f = packed_pairs<kHalf, kOneType, kB, false>(i, ld_i4(a.p.pos_fx, i), a.list.nbr + i, a.list.count[i],
                                                      (size_t) a.list.stride, a.p.pos_fx, a.p.force32, a.box, a.lj,
                                                      a.cut_count, a.cut_rec, a.cut_capacity);
    }
    if(kHalf) {
        red_add_v4(a.p.force32 + 4 * (size_t) i, f.x, f.y, f.z);
    } else {
        st_f4(a.p.force32, i, make_float4(f.x, f.y, f.z, 0.0f));
    }
}

// One pair of the cutoff band (FP32 rsq within kCutBand of rc^2): the FP64 path's own
// test decides it; a pair inside gets its FP32 force (and, through a half list's
// interior entry, the reaction), exactly as the main pass would have applied it.
template<bool kHalf, bool kOneType, bool kEnergy, bool kFixed>
__device__ __forceinline__ void fixup_pair(const ForceArgs &a, int i, uint32_t e) {
    const int j = (int) (e & PG_NBR_INDEX_MASK);
    const uint32_t code = e >> PG_NBR_INDEX_BITS;
    if(!exact_inside(a.p.pos, i, j, code, a.box.len, a.lj.cutoff2)) { return; }
    float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi, hj = hi, lj = hi;
    int4 fi = make_int4(0, 0, 0, 0), fj = fi;
    if(kFixed) {
        fi = ld_i4(a.p.pos_fx, i); fj = ld_i4(a.p.pos_fx, j);
    } else {
        hi = ld_f4(a.p.pos_hi, hl(a.p, i)); lo = ld_f4(a.p.pos_lo, hl(a.p, i));
        hj = ld_f4(a.p.pos_hi, hl(a.p, j)); lj = ld_f4(a.p.pos_lo, hl(a.p, j));
    }
    float dx, dy, dz;
    mixed_delta<kFixed>(a, fi, hi, lo, fj, hj, lj, code, dx, dy, dz);
    const float rsq = pair_rsq(dx, dy, dz);
    const int ti = kFixed ? fi.w : __float_as_int(hi.w), tj = kFixed ? fj.w : __float_as_int(hj.w);
    const int tij = kOneType ? 0 : ti * a.lj.ntypes + tj;
    float sr6;
    const float f = mixed_lj(a, tij, rsq, sr6);
    red_add_v4(a.p.force32 + 4 * (size_t) i, dx * f, dy * f, dz * f);
    if(kHalf && code == 0u) { red_add_v4(a.p.force32 + 4 * (size_t) j, -dx * f, -dy * f, -dz * f); }
    if(kEnergy) {
        const double w = (kHalf && code == 0u) ? 1.0 : 0.5;
        atomicAdd(&a.energy[0], w * 4.0 * (double) a.lj.epsf[tij] * ((double) sr6 * (double) sr6 - (double) sr6));
        atomicAdd(&a.energy[1], w * (double) (rsq * f));
    }
}

// The pairs of the cutoff band, which the main pass left out.  Normally they are the
// queued records.  When more pairs fell in the band than the queue holds (a workspace
// too small for the system), the records past its capacity were dropped, so every list
// is walked again and each band pair is taken from there instead (the screen's
// arithmetic is the main pass's, so it finds exactly the pairs that pass left out).
// A small workspace thus costs time, never a force.
template<bool kHalf, bool kOneType, bool kEnergy, bool kFixed>
__global__ void __launch_bounds__(kBlock) k_lj_cutoff_fixup(ForceArgs a) {
    if(frozen_force(a.p)) { return; }
    const int queued = *a.cut_count;
    const int first = blockIdx.x * blockDim.x + threadIdx.x, step = gridDim.x * blockDim.x;
    if(queued <= a.cut_capacity) {
        for(int r = first; r < queued; r += step) {
            const int2 q = a.cut_rec[r];
            fixup_pair<kHalf, kOneType, kEnergy, kFixed>(a, q.x, (uint32_t) q.y);
        }
        return;
    }
    const float c2 = a.lj.cutoff2f, band = c2 * kCutBand;
    for(int i = first; i < a.p.n; i += step) {
        if(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed)) { continue; }
        float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
        int4 fi = make_int4(0, 0, 0, 0);
        if(kFixed) { fi = ld_i4(a.p.pos_fx, i); }
        else { hi = ld_f4(a.p.pos_hi, hl(a.p, i)); lo = ld_f4(a.p.pos_lo, hl(a.p, i)); }
        const int cnt = a.list.count[i];
        for(int k = 0; k < cnt; k++) {
            const uint32_t e = (uint32_t) a.list.nbr[(size_t) k * a.list.stride + i];
            const int j = (int) (e & PG_NBR_INDEX_MASK);
            float4 hj = make_float4(0.f, 0.f, 0.f, 0.f), lj = hj;
            int4 fj = make_int4(0, 0, 0, 0);
            if(kFixed) { fj = ld_i4(a.p.pos_fx, j); }
            else { hj = ld_f4(a.p.pos_hi, hl(a.p, j)); lj = ld_f4(a.p.pos_lo, hl(a.p, j)); }
            float dx, dy, dz;
            mixed_delta<kFixed>(a, fi, hi, lo, fj, hj, lj, e >> PG_NBR_INDEX_BITS, dx, dy, dz);
            if(fabsf(pair_rsq(dx, dy, dz) - c2) < band) { fixup_pair<kHalf, kOneType, kEnergy, kFixed>(a, i, e); }
        }
    }
}

using KernelFn = void (*)(ForceArgs);

// zero the force array before a half-list pass, and the mixed path's near-cutoff queue
// (skipped like the pass when frozen).  Each thread clears kZeroPer consecutive 16-byte
// records after one read of the guard word (one record per thread: 12.5 us at 1M atoms,
// the stores waiting on each thread's guard load).
constexpr int kZeroPer = 4;

__global__ void k_zero_force(pg_particles p, int fp64, int32_t *cut_count) {
    if(frozen_force(p)) { return; }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t == 0 && cut_count != nullptr) { *cut_count = 0; }
    // 16-byte records: one per particle in FP32, two in FP64
    const int64_t records = fp64 ? 2 * (int64_t) p.n : (int64_t) p.n;
    float4 *base = fp64 ? reinterpret_cast<float4 *>(p.force) : reinterpret_cast<float4 *>(p.force32);
    const int64_t first = (int64_t) blockIdx.x * blockDim.x * kZeroPer + threadIdx.x;
#pragma unroll
    for(int k = 0; k < kZeroPer; k++) {
        const int64_t r = first + (int64_t) k * blockDim.x;
        if(r < records) { base[r] = make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
    }
}

static KernelFn pick_fp64(bool half, bool one, bool en) {
    if(half) {
        if(one) { return en ? k_lj_fp64<true, true, true> : k_lj_fp64<true, true, false>; }
        return en ? k_lj_fp64<true, false, true> : k_lj_fp64<true, false, false>;
    }
    if(one) { return en ? k_lj_fp64<false, true, true> : k_lj_fp64<false, true, false>; }
    return en ? k_lj_fp64<false, false, true> : k_lj_fp64<false, false, false>;
}

struct MixedKernels { KernelFn main, fixup; int block; };

template<bool kHalf, bool kOneType, bool kEnergy, bool kFixed>
static MixedKernels mixed_kernels() {
    if(kFixed && !kEnergy) {
        return {k_lj_packed<kHalf, kOneType, kHalf ? 4 : 2>, k_lj_cutoff_fixup<kHalf, kOneType, kEnergy, kFixed>,
                kPackedBlock};
    }
    return {k_lj_mixed<kHalf, kOneType, kEnergy, kFixed>, k_lj_cutoff_fixup<kHalf, kOneType, kEnergy, kFixed>, kBlock};
}

template<bool kFixed>
static MixedKernels pick_mixed_layout(bool half, bool one, bool en) {
    if(half) {
        if(one) { return en ? mixed_kernels<true, true, true, kFixed>() : mixed_kernels<true, true, false, kFixed>(); }
        return en ? mixed_kernels<true, false, true, kFixed>() : mixed_kernels<true, false, false, kFixed>();
    }
    if(one) { return en ? mixed_kernels<false, true, true, kFixed>() : mixed_kernels<false, true, false, kFixed>(); }
    return en ? mixed_kernels<false, false, true, kFixed>() : mixed_kernels<false, false, false, kFixed>();
}

static MixedKernels pick_mixed(bool half, bool one, bool en, bool fixed) {
    return fixed ? pick_mixed_layout<true>(half, one, en) : pick_mixed_layout<false>(half, one, en);
}

// The mixed path's queue of near-cutoff pairs lives in the caller's workspace: a
// counter, then int2 records (the binning scratch of the same workspace is free
// between rebuilds).  The expected load is about 1.7e-3 pairs per particle with full
// lists and half that with half lists (1e-5 of rc^2 around the cutoff at density
// 0.84); one record is the minimum, and a queue that overflows makes the fixup pass
// walk every list again (k_lj_cutoff_fixup).
constexpr int64_t kCutQueueMin = 256 + 8;
constexpr int kFixupBlocks = 2 * kSMs;

int tile_lj_force(const pg_box *box, const pg_particles *p, const pg_neighbor_list *list, const pg_cells *cells,
                  const LJTableF &lj, double *energy, cudaStream_t st);
int pc_lj_force(const pg_box *box, const pg_particles *p, const pg_neighbor_list *list, const LJTable &lj,
                double *energy, int32_t *cut_count, int2 *cut_rec, int cut_capacity, cudaStream_t st);

int lj_force(const pg_box *box, const pg_particles *p, const pg_cells *cells, const pg_neighbor_list *list,
             const pg_lj_params *lj, int precision, int sync_mode, double *energy, pg_workspace ws, cudaStream_t st) {
    if(!box || !p || !list || !lj) { return PG_ERR_ARGUMENT; }
    if(lj->ntypes < 1 || lj->ntypes > kMaxTypes) { return PG_ERR_ARGUMENT; }
    if(precision != PG_FP64 && precision != PG_MIXED) { return PG_ERR_ARGUMENT; }
    if(precision == PG_FP64 && (!p->pos || !p->force)) { return PG_ERR_ARGUMENT; }
    const bool fixed_point = precision == PG_MIXED && p->pos_fx != nullptr;
    if(precision == PG_MIXED && (!p->force32 || (!fixed_point && (!p->pos_hi || !p->pos_lo)))) { return PG_ERR_ARGUMENT; }
    if(fixed_point && !(box->fx_unit[0] > 0.0f && box->fx_unit[1] > 0.0f && box->fx_unit[2] > 0.0f)) {
        return PG_ERR_ARGUMENT;
    }
    if(lj->ntypes > 1 && !p->type) { return PG_ERR_ARGUMENT; }
    if(sync_mode == PG_SYNC_REFERENCE && (precision != PG_FP64 || !p->pos_prev1 || !p->pos_prev2)) {
        return PG_ERR_ARGUMENT;
    }
    ForceArgs a;
    a.box = *box; a.p = *p; a.list = *list;
    a.cut_count = nullptr; a.cut_rec = nullptr; a.cut_capacity = 0;
    a.sync_ref = sync_mode == PG_SYNC_REFERENCE;
    a.energy = energy;
    a.lj.ntypes = lj->ntypes;
    a.lj.cutoff2 = lj->cutoff2;
    a.lj.cutoff2f = (float) lj->cutoff2;
    for(int k = 0; k < lj->ntypes * lj->ntypes; k++) {
        a.lj.eps[k] = lj->epsilon[k]; a.lj.sig6[k] = lj->sigma6[k];
        a.lj.epsf[k] = (float) lj->epsilon[k]; a.lj.sig6f[k] = (float) lj->sigma6[k];
    }
    const bool half = list->half != 0, one = lj->ntypes == 1, en = energy != nullptr;
    const bool tile = precision == PG_MIXED && list->nbr16 != nullptr;
    const bool pairs = list->pair_table != nullptr;
    if(pairs && (precision != PG_MIXED || !fixed_point || !half || tile)) { return PG_ERR_ARGUMENT; }
    if(tile && (!cells || !p->pos_hi || !p->pos_lo)) { return PG_ERR_ARGUMENT; }
    if(!tile && !list->nbr) { return PG_ERR_ARGUMENT; }
    if(en) { cudaMemsetAsync(energy, 0, 2 * sizeof(double), st); }
    const bool queue = precision == PG_MIXED && !tile;
    if(queue) {
        if(ws.ptr == nullptr || ws.bytes < kCutQueueMin) { return PG_ERR_ARGUMENT; }
        a.cut_count = (int32_t *) ws.ptr;
        a.cut_rec = (int2 *) ((char *) ws.ptr + 256);
        a.cut_capacity = (int) std::min<int64_t>((ws.bytes - 256) / 8, INT32_MAX);
    }
    if(half && p->n > 0) {
        const int64_t records = precision == PG_FP64 ? 2 * (int64_t) p->n : (int64_t) p->n;
        k_zero_force<<<blocks_for(records, kBlock * kZeroPer), kBlock, 0, st>>>(*p, precision == PG_FP64, a.cut_count);
        note_launch();
    } else if(queue) {
        cudaMemsetAsync(a.cut_count, 0, sizeof(int32_t), st);
    }
    if(p->n == 0) { return launch_status(); }
    if(tile) {
        LJTableF tf;
        tf.ntypes = lj->ntypes;
        tf.cutoff2 = (float) lj->cutoff2;
        tf.cutoff2d = lj->cutoff2;
        for(int k = 0; k < lj->ntypes * lj->ntypes; k++) { tf.eps[k] = (float) lj->epsilon[k]; tf.sig6[k] = (float) lj->sigma6[k]; }
        return tile_lj_force(box, p, list, cells, tf, energy, st);
    }
    if(precision == PG_FP64) {
        pick_fp64(half, one, en)<<<blocks_for(p->n), kBlock, 0, st>>>(a); note_launch();
        return launch_status();
    }
    if(pairs) { return pc_lj_force(box, p, list, a.lj, energy, a.cut_count, a.cut_rec, a.cut_capacity, st); }
    const MixedKernels k = pick_mixed(half, one, en, fixed_point);
    k.main<<<blocks_for(p->n, k.block), k.block, 0, st>>>(a); note_launch();
    k.fixup<<<kFixupBlocks, kBlock, 0, st>>>(a); note_launch();
    return launch_status();
}

}  // namespace pg
