// The mixed path's Lennard-Jones pair loop of one particle on fixed-point positions,
// shared by the force kernel (lj.cu) and the persistent time-step kernel (persist.cu).
//
// The pair arithmetic of two list entries runs at a time in packed FP32 (Blackwell's
// f32x2 multiply, add and fused multiply-add: one instruction for both pairs).  Each
// pair rounds as in the one-pair-at-a-time kernel: the squared distance in the order
// of pair_rsq, so the cutoff band holds the same pairs, and the force factor
// 48 sr6 (sr6 - 1/2) sr2 eps in FP32 (examples/md.py:5-8, sim/interaction.py:222-232).
// A pair whose FP32 rsq lies within kCutBand of rc^2 is left out and queued for the
// FP64 decision; a half list's interior pair adds its reaction to the partner with a
// vector reduction (ir/apply.py:112-125).
//
// kCoherent: positions are read with ordinary cached loads instead of the read-only
// path.  A kernel that rewrites the positions while it runs (the persistent kernel,
// between grid barriers) must read them this way: the read-only path may serve data
// cached before the rewrite.
#pragma once

#include "common.cuh"

namespace pg {

constexpr int kMaxTypes = 8;

struct LJTable {
    int ntypes;
    float cutoff2f;
    double cutoff2;
    double eps[kMaxTypes * kMaxTypes];
    double sig6[kMaxTypes * kMaxTypes];
    float epsf[kMaxTypes * kMaxTypes];
    float sig6f[kMaxTypes * kMaxTypes];
};

template<bool kCoherent>
__device__ __forceinline__ int4 ld_fx(const int32_t *base, int i) {
    const int4 *p = reinterpret_cast<const int4 *>(base) + i;
    return kCoherent ? __ldca(p) : __ldg(p);
}

// Forces on particle i (position fi) from its cnt list entries nb[k * stride]; returns
// the sum over the list (half lists: the reactions went to the partners).
template<bool kHalf, bool kOneType, int kB, bool kCoherent>
__device__ __forceinline__ float3 packed_pairs(int i, int4 fi, const int32_t *nb, int cnt, size_t stride,
                                               const int32_t *pos_fx, float *force32, const pg_box &box,
                                               const LJTable &lj, int32_t *cut_count, int2 *cut_rec,
                                               int cut_capacity) {
    static_assert(kB % 2 == 0, "entries are taken in pairs");
    const int ti = kOneType ? 0 : fi.w * lj.ntypes;
    const float c2 = lj.cutoff2f, band = c2 * kCutBand;
    const float2 ux = make_float2(box.fx_unit[0], box.fx_unit[0]);
    const float2 uy = make_float2(box.fx_unit[1], box.fx_unit[1]);
    const float2 uz = make_float2(box.fx_unit[2], box.fx_unit[2]);
    const float2 half2 = make_float2(-0.5f, -0.5f);
    float2 FX = make_float2(0.0f, 0.0f), FY = FX, FZ = FX;
    uint32_t cur[kB];
#pragma unroll
    for(int u = 0; u < kB; u++) { cur[u] = u < cnt ? (uint32_t) __ldcs(nb + u * stride) : 0u; }
    for(int k0 = 0; k0 < cnt; k0 += kB) {
        int4 fj[kB];
#pragma unroll
        for(int u = 0; u < kB; u++) { fj[u] = ld_fx<kCoherent>(pos_fx, (int) (cur[u] & PG_NBR_INDEX_MASK)); }
        uint32_t nxt[kB];
        const int32_t *nbn = nb + (size_t) (k0 + kB) * stride;
#pragma unroll
        for(int u = 0; u < kB; u++) { nxt[u] = k0 + kB + u < cnt ? (uint32_t) __ldcs(nbn + u * stride) : 0u; }
        uint32_t pending = 0u;
#pragma unroll
        for(int u = 0; u < kB; u += 2) {
            const bool va = k0 + u < cnt, vb = k0 + u + 1 < cnt;
            const float2 dX = __fmul2_rn(make_float2((float) fx_diff(fi.x, fj[u].x), (float) fx_diff(fi.x, fj[u + 1].x)), ux);
            const float2 dY = __fmul2_rn(make_float2((float) fx_diff(fi.y, fj[u].y), (float) fx_diff(fi.y, fj[u + 1].y)), uy);
            const float2 dZ = __fmul2_rn(make_float2((float) fx_diff(fi.z, fj[u].z), (float) fx_diff(fi.z, fj[u + 1].z)), uz);
            float2 R = __fmul2_rn(dX, dX);
            R = __ffma2_rn(dY, dY, R);
            R = __ffma2_rn(dZ, dZ, R);
            const bool na = fabsf(R.x - c2) < band, nb2 = fabsf(R.y - c2) < band;
            const bool ia = va && R.x < c2 && !na, ib = vb && R.y < c2 && !nb2;
            float2 sig6, eps48;
            if(kOneType) {
                sig6 = make_float2(lj.sig6f[0], lj.sig6f[0]);
                eps48 = make_float2(48.0f * lj.epsf[0], 48.0f * lj.epsf[0]);
            } else {
                const int ta = ti + fj[u].w, tb = ti + fj[u + 1].w;
                sig6 = make_float2(lj.sig6f[ta], lj.sig6f[tb]);
                eps48 = make_float2(48.0f * lj.epsf[ta], 48.0f * lj.epsf[tb]);
            }
            const float2 S2 = make_float2(rcp_approx(R.x), rcp_approx(R.y));
            const float2 S6 = __fmul2_rn(__fmul2_rn(S2, S2), __fmul2_rn(S2, sig6));
            float2 F = __fmul2_rn(__fmul2_rn(S6, __fadd2_rn(S6, half2)), __fmul2_rn(S2, eps48));
            F.x = ia ? F.x : 0.0f;
            F.y = ib ? F.y : 0.0f;
            FX = __ffma2_rn(dX, F, FX);
            FY = __ffma2_rn(dY, F, FY);
            FZ = __ffma2_rn(dZ, F, FZ);
            if(kHalf) {
                const float2 nF = make_float2(-F.x, -F.y);
                const float2 rX = __fmul2_rn(dX, nF), rY = __fmul2_rn(dY, nF), rZ = __fmul2_rn(dZ, nF);
                if(ia && (cur[u] >> PG_NBR_INDEX_BITS) == 0u) {
                    red_add_v4(force32 + 4 * (size_t) (cur[u] & PG_NBR_INDEX_MASK), rX.x, rY.x, rZ.x);
                }
                if(ib && (cur[u + 1] >> PG_NBR_INDEX_BITS) == 0u) {
                    red_add_v4(force32 + 4 * (size_t) (cur[u + 1] & PG_NBR_INDEX_MASK), rX.y, rY.y, rZ.y);
                }
            }
            if(va && na) { pending |= 1u << u; }
            if(vb && nb2) { pending |= 2u << u; }
        }
        if(pending != 0u) {
#pragma unroll
            for(int u = 0; u < kB; u++) {
                if(pending & (1u << u)) { cut_queue_push(cut_count, cut_rec, cut_capacity, i, cur[u]); }
            }
        }
#pragma unroll
        for(int u = 0; u < kB; u++) { cur[u] = nxt[u]; }
    }
    return make_float3(FX.x + FX.y, FY.x + FY.y, FZ.x + FZ.y);
}

}  // namespace pg
