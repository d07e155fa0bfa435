// Pair-cluster half lists: the mixed path's Verlet list and LJ force on fixed-point
// positions, with the list walked by pairs of particles.
//
// The per-particle half list (nlist.cu, lj.cu) spends its time in the L1 data pipe:
// every entry is one scattered 16-byte partner gather and, inside the cutoff, one
// scattered 16-byte reaction reduction.  Two particles of the same cell have nearly the
// same neighbourhood (the union of two r_list spheres 1 sigma apart is 1.27 spheres), so
// here the two share one list: a cluster is a pair of consecutive particles of one cell
// (a, b = a + 1; the last particle of an odd cell alone), and each entry of the
// cluster's list is a partner j with one bit per member saying whether that member
// stores the pair (j, member).  Per entry the partner is gathered once and one reaction
// reduction carries the sum of both members' pair forces; the two members' pair
// arithmetic is the two lanes of Blackwell's packed f32x2 instructions.
//
// The pair set is the reference's (sim/neighbor_lists.py:21-48): a pair of particles
// closer than r_list, decided by the same FP32 screen and FP64 band test as the
// per-particle build (nlist.cu), each pair stored once.  Which member stores a pair is
// geometric: the one whose partner lies above it in x (minimum-image separation; ties
// y, z, index).  Pairs through a periodic image follow the same rule, so every pair,
// image or not, is stored once and applies its reaction (the reference computes an
// image pair from both sides with no reaction, sim/interaction.py:107-113; the force
// on each particle is the same sum).  Stored above means the stencil is the cells at
// 0..reach_x cells above in x (half-width x cells), 3 x 3 in y and z.
//
// Cluster slots need no scan: cell c with first particle s_c and n_c particles owns
// slots ceil((s_c + c) / 2) + m, m < ceil(n_c / 2).  Consecutive cells' slot ranges are
// disjoint (the base grows by at least ceil(n_c / 2) from one cell to the next), and
// at most (n + ncells) / 2 + 2 slots are used; free slots hold -1.
#include <math.h>

#include "common.cuh"
#include "lj_packed.cuh"

namespace pg {

constexpr int32_t kPcHasB = 1 << 30;                 // table record: a second member
constexpr uint32_t kPcIndexMask = (1u << 30) - 1u;   // table record / entry: particle index
constexpr uint32_t kPcMaskA = 1u << 30;              // entry: the pair (j, first member)
constexpr uint32_t kPcMaskB = 1u << 31;              // entry: the pair (j, second member)
constexpr float kPcScreenBand = 1.0e-4f;             // the build's FP64 band (as nlist.cu)
// force pass: 192 threads, at most 64 registers (5 blocks, 960 threads per SM).  Measured
// at 1M atoms (main pass + fixup): 0.1556 ms, against 0.1638 at 128 threads (8 blocks),
// 0.1556 at 96 threads (10 blocks) or at 128 threads with 72 registers (7 blocks),
// 0.1633 at 80 registers or at 64 threads; the resident warps' partner gathers share L1
constexpr int kPcBlock = 192;
constexpr int kPcBatch = 4;

int64_t pair_slots(int32_t n, int32_t ncells) {
    return n < 0 || ncells < 0 ? -1 : ((int64_t) n + ncells) / 2 + 2;
}

// ------------------------------------------------------------------ cluster table

__global__ void k_pc_table(pg_cells cells, int32_t *table) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if(c >= cells.ncells) { return; }
    const int s = cells.cell_start[c], n = cells.cell_count[c];
    const int base = (int) (((int64_t) s + c + 1) >> 1);
    for(int m = 0; 2 * m < n; m++) {
        table[base + m] = (s + 2 * m) | (2 * m + 1 < n ? kPcHasB : 0);
    }
}

// ------------------------------------------------------------------ build

struct PcBuildArgs {
    pg_box box;
    pg_particles p;
    pg_cells cells;
    pg_neighbor_list list;
    double r_list2;
    float r2_lo, r2_hi;          // screening band, box units squared when kCubic
    const pg_replica *replicas;  // batched ensembles: each slot's box and grid from its replica
    const int32_t *replica_of;
    const int32_t *rebuild;      // batched ensembles: the replicas of a partial rebuild (or NULL)
};

// The FP64 decision of a candidate in the screening band: the reference's separately
// rounded rsq to the stencil's image of the partner (as nlist.cu).  The box lengths are
// the system's, or (batched ensembles) those of particle i's replica, looked up here so
// that the build's loops keep no pointer to them.
__device__ __noinline__ bool pc_exact(const PcBuildArgs &a, int i, int j, int sx, int sy, int sz) {
    const double *len = a.replicas != nullptr ? a.replicas[a.replica_of[i]].len : a.box.len;
    const D4 xi = ld_d4_rare(a.p.pos, i), xj = ld_d4_rare(a.p.pos, j);
    const double dx = __dsub_rn(xi.x, ref_image(xj.x, sx, len[0]));
    const double dy = __dsub_rn(xi.y, ref_image(xj.y, sy, len[1]));
    const double dz = __dsub_rn(xi.z, ref_image(xj.z, sz, len[2]));
    return ref_rsq(dx, dy, dz) < a.r_list2;
}

// Fixed-point z of particle j as an ordering key along its cell column: the coordinate
// in units (0 .. 2^32), except in the column's top cell, where a particle rounded onto
// the box's upper face (z_fx = 2^32 mod 2^32 = 0) counts as 2^32, so that the keys of
// a column's particles, sorted by z within each cell (pg_bin_particles), ascend.
__device__ __forceinline__ int64_t z_key(uint32_t zfx, bool top_cell) {
    return (int64_t) zfx + (top_cell && zfx < 0x80000000u ? (int64_t) 1 << 32 : 0);
}

// One thread per cluster slot: both members' candidates from the stencil of their
// cell, one list entry per partner stored by either member.  Also records the guard's
// reference positions of the members.  The build must follow the binning of the same
// positions (each particle inside its cell, each cell sorted by z).
//
// The stencil is walked by z columns: cells (cx + ox, cy + oy, cz - reach .. cz +
// reach) are one contiguous range of particles sorted by z (or two or three ranges
// where the column wraps around a periodic z face, each with its image shift).  A
// partner in column (ox, oy) lies at least g = the member's lateral distance to that
// column's cells away, so within sqrt(r_list^2 - g^2) in z: each range is entered at
// the first particle of the union of the members' z windows and left at its end (both
// found by binary search on the z keys).  A column out of reach of both members is
// skipped.  The windows are widened by a margin far above the rounding of the
// positions (1e-3 sigma, r_list^2 (1 + 1e-3)); a candidate inside a window is decided
// exactly as before, so the list is the same set with fewer candidates.
//
// The screen takes both members' squared distances to a candidate in one packed f32x2
// chain, and the half-list side (partner above) from the integer differences, whose
// signs are the converted differences' signs.  Entries are streaming stores (evict
// first: 0.463 against 0.469 ms; filling each 8-slot group's rows up to its longest
// list, so that L2 sees whole sectors, measured 0.48 ms and no fewer DRAM bytes).
//
// Measured at 1M atoms (fcc 64^3 liquid): 0.463 ms per build against 0.652 ms with
// one z window of +-r_list for every column; 0.47-0.56 ms at other block sizes and
// register caps (the build runs at 64 registers, 128 threads, 8 blocks per SM).
struct PcWindow {
    double clx_u, cly_u;         // cell lengths in units (x, y)
    float clx, cly;              // cell lengths
    float r2w;                   // window radius squared (r_list^2 widened)
    float scale_z;               // units per length along z
};

constexpr int kPcBuildBlock = 128;

// Batched ensembles (kEns): a slot's box, units and grid come from its replica (the
// cells of replica r are [cell0, cell0 + ncells) of the shared arrays, z fastest), and a
// replica whose grid would visit a stencil cell twice (fewer than 2 reach + 1 cells on an
// axis) sets overflow bit 5 instead of listing.
constexpr int kPcGridTooSmall = 32;

template<bool kCubic, bool kEns>
__global__ void __launch_bounds__(kPcBuildBlock, 8) k_pc_build(PcBuildArgs a, PcWindow w, pg_status *status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= a.list.stride) { return; }
    const int rec = a.list.pair_table[t];
    const int cap = a.list.max_neighbors;
    int cnt = 0;
    if(rec >= 0) {
        const int ia = rec & (int) kPcIndexMask;
        // a replica left alone by a partial rebuild keeps its rows (its cells, and so its
        // slots, are unchanged)
        if(kEns && a.rebuild != nullptr && a.rebuild[a.replica_of[ia]] == 0) { return; }
        const bool has_b = (rec & kPcHasB) != 0;
        const int ib = has_b ? ia + 1 : ia;
        const int4 fa = ld_i4(a.p.pos_fx, ia), fb = ld_i4(a.p.pos_fx, ib);
        st_d4(a.p.pos_ref, ia, ld_d4(a.p.pos, ia));
        st_i4(a.p.ref_fx, ia, fa);
        if(has_b) {
            st_d4(a.p.pos_ref, ib, ld_d4(a.p.pos, ib));
            st_i4(a.p.ref_fx, ib, fb);
        }
        const bool use_a = !(a.p.flags != nullptr && (a.p.flags[ia] & kFlagFixed));
        const bool use_b = has_b && !(a.p.flags != nullptr && (a.p.flags[ib] & kFlagFixed));
        // the grid and box of the slot (the system's, or its replica's)
        int ci = a.cells.particle_cell[ia], cell0 = 0, ncells = a.cells.ncells;
        int dz_ = a.cells.dims[2], dy_ = a.cells.dims[1], dx_ = a.cells.dims[0];
        int rr = a.cells.reach > 1 ? a.cells.reach : 1;
        int rx = a.cells.reach_x > 0 ? a.cells.reach_x : rr;
        float fu[3] = {a.box.fx_unit[0], a.box.fx_unit[1], a.box.fx_unit[2]};
        double clx_u = w.clx_u, cly_u = w.cly_u;
        float clx = w.clx, cly = w.cly, scale_z = w.scale_z;
        bool grid_ok = true;
        if(kEns) {
            const pg_replica &R = a.replicas[a.replica_of[ia]];
            cell0 = R.cell0; ncells = R.ncells; ci -= cell0;
            dx_ = R.dims[0]; dy_ = R.dims[1]; dz_ = R.dims[2];
            rr = R.reach > 1 ? R.reach : 1;
            rx = R.reach_x > 0 ? R.reach_x : rr;
            fu[0] = R.fx_unit[0]; fu[1] = R.fx_unit[1]; fu[2] = R.fx_unit[2];
            clx_u = R.cell_len[0] * R.fx_scale[0]; cly_u = R.cell_len[1] * R.fx_scale[1];
            clx = (float) R.cell_len[0]; cly = (float) R.cell_len[1]; scale_z = (float) R.fx_scale[2];
            // each stencil cell visited once (the half stencil's ox 0 .. rx, oy and oz
            // -rr .. rr): then a pair within r_list (< half a box) is met once, through the
            // image its fixed-point difference gives
            grid_ok = dx_ >= 2 * rx + 1 && dy_ >= 2 * rr + 1 && dz_ >= 2 * rr + 1;
            if(!grid_ok) { atomicOr(&status->overflow, kPcGridTooSmall); }
        }
        if((use_a || use_b) && ci >= 0 && ci < ncells && grid_ok) {
            const int cz = ci % dz_, cy = (ci / dz_) % dy_, cx = ci / (dz_ * dy_);
            const float unit2 = kCubic ? fu[0] * fu[0] : 1.0f;
            const float r2_lo = a.r2_lo / unit2, r2_hi = a.r2_hi / unit2;
            const float2 ux = make_float2(fu[0], fu[0]);
            const float2 uy = make_float2(fu[1], fu[1]);
            const float2 uz = make_float2(fu[2], fu[2]);
            const int stride = a.list.stride;
            int32_t *wp = a.list.nbr + t;
            // the members' z keys in their own cell (b follows a in z order)
            const bool own_top = cz == dz_ - 1;
            const int64_t za = z_key((uint32_t) fa.z, own_top), zb = z_key((uint32_t) fb.z, own_top);
            // the members' offsets inside their cell in x and y (a member rounded onto the
            // box's upper face wraps to 0 units; the wrapped difference keeps it at the top)
            const uint32_t ex = (uint32_t) (unsigned long long) llrint(cx * clx_u);
            const uint32_t ey = (uint32_t) (unsigned long long) llrint(cy * cly_u);
            const float xa = (float) (int) ((uint32_t) fa.x - ex) * fu[0];
            const float xb = (float) (int) ((uint32_t) fb.x - ex) * fu[0];
            const float ya = (float) (int) ((uint32_t) fa.y - ey) * fu[1];
            const float yb = (float) (int) ((uint32_t) fb.y - ey) * fu[1];
            constexpr float kMargin = 1.0e-3f;
            // column ranges: the unwrapped cells, then the cells wrapped below / above
            const int z_lo = cz - rr < 0 ? 0 : cz - rr, z_hi = cz + rr > dz_ - 1 ? dz_ - 1 : cz + rr;
            // one candidate j (position fj) of the stencil cell at x offset ox, image (sx, sy, sz)
            auto candidate = [&](int j, int4 fj, int ox, int sx, int sy, int sz) {
                const int dxa = fx_diff(fa.x, fj.x), dya = fx_diff(fa.y, fj.y), dza = fx_diff(fa.z, fj.z);
                const int dxb = fx_diff(fb.x, fj.x), dyb = fx_diff(fb.y, fj.y), dzb = fx_diff(fb.z, fj.z);
                float2 X = make_float2((float) dxa, (float) dxb), Y = make_float2((float) dya, (float) dyb);
                float2 Z = make_float2((float) dza, (float) dzb);
                if(!kCubic) { X = __fmul2_rn(X, ux); Y = __fmul2_rn(Y, uy); Z = __fmul2_rn(Z, uz); }
                float2 R = __fmul2_rn(X, X);
                R = __ffma2_rn(Y, Y, R);
                R = __ffma2_rn(Z, Z, R);
                // a partner in a higher x slab lies above; in the own slab the separation
                // decides (exactly one side of a pair keeps it, as partner_above)
                const bool above_a = ox > 0 || (dxa != 0 ? dxa < 0 : (dya != 0 ? dya < 0 : (dza != 0 ? dza < 0 : j > ia)));
                const bool above_b = ox > 0 || (dxb != 0 ? dxb < 0 : (dyb != 0 ? dyb < 0 : (dzb != 0 ? dzb < 0 : j > ib)));
                bool ka = use_a && j != ia && above_a && R.x <= r2_hi;
                bool kb = use_b && j != ib && above_b && R.y <= r2_hi;
                if(ka && !(R.x < r2_lo)) { ka = pc_exact(a, ia, j, sx, sy, sz); }
                if(kb && !(R.y < r2_lo)) { kb = pc_exact(a, ib, j, sx, sy, sz); }
                if(ka || kb) {
                    if(cnt < cap) {
                        __stcs(wp, (int32_t) ((uint32_t) j | (ka ? kPcMaskA : 0u) | (kb ? kPcMaskB : 0u)));
                        wp += stride;
                    }
                    cnt++;
                }
            };
            for(int ox = 0; ox <= rx; ox++) {
                int nx = cx + ox, sx = 0;
                if(nx >= dx_) { nx -= dx_; sx = 1; }
                const float gxa = ox == 0 ? 0.0f : fmaxf(ox * clx - xa - kMargin, 0.0f);
                const float gxb = ox == 0 ? 0.0f : fmaxf(ox * clx - xb - kMargin, 0.0f);
                for(int oy = -rr; oy <= rr; oy++) {
                    int ny = cy + oy, sy = 0;
                    if(ny < 0) { ny += dy_; sy = -1; } else if(ny >= dy_) { ny -= dy_; sy = 1; }
                    const float gya = oy == 0 ? 0.0f
                                              : fmaxf((oy < 0 ? ya + (-oy - 1) * cly : oy * cly - ya) - kMargin, 0.0f);
                    const float gyb = oy == 0 ? 0.0f
                                              : fmaxf((oy < 0 ? yb + (-oy - 1) * cly : oy * cly - yb) - kMargin, 0.0f);
                    const float qa = use_a ? w.r2w - gxa * gxa - gya * gya : -1.0f;
                    const float qb = use_b ? w.r2w - gxb * gxb - gyb * gyb : -1.0f;
                    if(qa < 0.0f && qb < 0.0f) { continue; }
                    int64_t w_lo = INT64_MAX, w_hi = INT64_MIN;
                    if(qa >= 0.0f) {
                        const int64_t h = (int64_t) (sqrtf(qa) * scale_z) + 16;
                        w_lo = za - h; w_hi = za + h;
                    }
                    if(qb >= 0.0f) {
                        const int64_t h = (int64_t) (sqrtf(qb) * scale_z) + 16;
                        w_lo = min(w_lo, zb - h); w_hi = max(w_hi, zb + h);
                    }
                    const int col = cell0 + (nx * dy_ + ny) * dz_;
                    for(int seg = 0; seg < 3; seg++) {
                        int c0, c1, sz;
                        if(seg == 0) { c0 = z_lo; c1 = z_hi; sz = 0; }
                        else if(seg == 1) { c0 = cz - rr + dz_; c1 = dz_ - 1; sz = -1; }   // wrapped below
                        else { c0 = 0; c1 = cz + rr - dz_; sz = 1; }                          // wrapped above
                        if(c0 > c1) { continue; }
                        const int b = a.cells.cell_start[col + c0];
                        const int e = a.cells.cell_start[col + c1] + a.cells.cell_count[col + c1];
                        const bool top = c1 == dz_ - 1;
                        const int64_t shift = (int64_t) sz * ((int64_t) 1 << 32);
                        // the window's particles [lo, hi): first key + shift >= w_lo, first > w_hi
                        const int ts = top ? a.cells.cell_start[col + dz_ - 1] : e;
                        int lo = b, hi = e;
                        while(lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            const int64_t k = z_key((uint32_t) __ldg(a.p.pos_fx + 4 * (size_t) mid + 2), mid >= ts) + shift;
                            if(k < w_lo) { lo = mid + 1; } else { hi = mid; }
                        }
                        int end = e;
                        for(int l = lo; l < end;) {
                            const int mid = (l + end) >> 1;
                            const int64_t k = z_key((uint32_t) __ldg(a.p.pos_fx + 4 * (size_t) mid + 2), mid >= ts) + shift;
                            if(k <= w_hi) { l = mid + 1; } else { end = mid; }
                        }
                        // two candidates per iteration: their loads and arithmetic overlap
                        int j = lo;
                        for(; j + 1 < end; j += 2) {
                            const int4 f0 = ld_i4(a.p.pos_fx, j), f1 = ld_i4(a.p.pos_fx, j + 1);
                            candidate(j, f0, ox, sx, sy, sz);
                            candidate(j + 1, f1, ox, sx, sy, sz);
                        }
                        if(j < end) { candidate(j, ld_i4(a.p.pos_fx, j), ox, sx, sy, sz); }
                    }
                }
            }
        }
    }
    a.list.count[t] = cnt < cap ? cnt : cap;
    publish_count(cnt, cap, status);
}

// ------------------------------------------------------------------ force

struct PcForceArgs {
    pg_box box;
    pg_particles p;
    pg_neighbor_list list;
    LJTable lj;
    double *energy;
    int32_t *cut_count;          // pairs within the cutoff band, queued (particle, partner)
    int2 *cut_rec;
    int cut_capacity;
    const pg_replica *replicas;  // batched ensembles: each slot's units from its replica
    const int32_t *replica_of;
};

// the fixed-point units and box lengths of particle i (the system's, or its replica's)
template<bool kEns>
__device__ __forceinline__ void pc_units(const PcForceArgs &a, int i, float u[3], const double **len) {
    if(kEns) {
        const pg_replica &R = a.replicas[a.replica_of[i]];
        u[0] = R.fx_unit[0]; u[1] = R.fx_unit[1]; u[2] = R.fx_unit[2];
        *len = R.len;
    } else {
        u[0] = a.box.fx_unit[0]; u[1] = a.box.fx_unit[1]; u[2] = a.box.fx_unit[2];
        *len = a.box.len;
    }
}

__device__ __forceinline__ void pc_block_energy(double pe, double vir, double *energy) {
    __shared__ double s[2][kPcBlock / 32];
    pe = warp_sum(pe);
    vir = warp_sum(vir);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if(lane == 0) { s[0][w] = pe; s[1][w] = vir; }
    __syncthreads();
    if(threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for(int k = 0; k < kPcBlock / 32; k++) { x += s[0][k]; y += s[1][k]; }
        atomicAdd(&energy[0], x);
        atomicAdd(&energy[1], y);
    }
}

// The pair forces of one cluster slot.  Lane x of every packed value is the first
// member's pair with the entry's partner, lane y the second's.  Each pair rounds as
// in the per-particle kernels (the squared distance in the order of pair_rsq, the
// factor 48 sr6 (sr6 - 1/2) sr2 eps in FP32, examples/md.py:5-8); a pair within
// kCutBand of rc^2 is queued for the FP64 decision of k_pc_fixup.
template<bool kOneType, bool kEnergy, bool kEns>
__global__ void __launch_bounds__(kPcBlock, 5) k_pc_lj(PcForceArgs a) {
    if(frozen_force(a.p)) { return; }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int rec = t < a.list.stride ? a.list.pair_table[t] : -1;
    double pe = 0.0, vir = 0.0;
    if(rec >= 0) {
        const int ia = rec & (int) kPcIndexMask;
        const bool has_b = (rec & kPcHasB) != 0;
        const int ib = has_b ? ia + 1 : ia;
        const int4 fa = ld_i4(a.p.pos_fx, ia), fb = ld_i4(a.p.pos_fx, ib);
        const int ta = kOneType ? 0 : fa.w * a.lj.ntypes, tb = kOneType ? 0 : fb.w * a.lj.ntypes;
        const int cnt = a.list.count[t];
        const int32_t *nb = a.list.nbr + t;
        const size_t stride = (size_t) a.list.stride;
        const float c2 = a.lj.cutoff2f, band = c2 * kCutBand;
        float fu[3];
        const double *len;
        pc_units<kEns>(a, ia, fu, &len);
        const float2 ux = make_float2(fu[0], fu[0]);
        const float2 uy = make_float2(fu[1], fu[1]);
        const float2 uz = make_float2(fu[2], fu[2]);
        const float2 half2 = make_float2(-0.5f, -0.5f);
        float2 FX = make_float2(0.0f, 0.0f), FY = FX, FZ = FX;
        uint32_t cur[kPcBatch];
#pragma unroll
        for(int u = 0; u < kPcBatch; u++) { cur[u] = u < cnt ? (uint32_t) __ldcs(nb + u * stride) : 0u; }
        for(int k0 = 0; k0 < cnt; k0 += kPcBatch) {
            int4 fj[kPcBatch];
#pragma unroll
            for(int u = 0; u < kPcBatch; u++) { fj[u] = ld_i4(a.p.pos_fx, (int) (cur[u] & kPcIndexMask)); }
            uint32_t nxt[kPcBatch];
            const int32_t *nbn = nb + (size_t) (k0 + kPcBatch) * stride;
#pragma unroll
            for(int u = 0; u < kPcBatch; u++) {
                nxt[u] = k0 + kPcBatch + u < cnt ? (uint32_t) __ldcs(nbn + u * stride) : 0u;
            }
            uint32_t pend_a = 0u, pend_b = 0u;
#pragma unroll
            for(int u = 0; u < kPcBatch; u++) {
                const bool valid = k0 + u < cnt;
                const bool ma = valid && (cur[u] & kPcMaskA) != 0u, mb = valid && (cur[u] & kPcMaskB) != 0u;
                const float2 dX = __fmul2_rn(make_float2((float) fx_diff(fa.x, fj[u].x), (float) fx_diff(fb.x, fj[u].x)), ux);
                const float2 dY = __fmul2_rn(make_float2((float) fx_diff(fa.y, fj[u].y), (float) fx_diff(fb.y, fj[u].y)), uy);
                const float2 dZ = __fmul2_rn(make_float2((float) fx_diff(fa.z, fj[u].z), (float) fx_diff(fb.z, fj[u].z)), uz);
                float2 R = __fmul2_rn(dX, dX);
                R = __ffma2_rn(dY, dY, R);
                R = __ffma2_rn(dZ, dZ, R);
                const bool na = fabsf(R.x - c2) < band, nbd = fabsf(R.y - c2) < band;
                const bool ina = ma && R.x < c2 && !na, inb = mb && R.y < c2 && !nbd;
                float2 sig6, eps48;
                if(kOneType) {
                    sig6 = make_float2(a.lj.sig6f[0], a.lj.sig6f[0]);
                    eps48 = make_float2(48.0f * a.lj.epsf[0], 48.0f * a.lj.epsf[0]);
                } else {
                    const int pa = ta + fj[u].w, pb = tb + fj[u].w;
                    sig6 = make_float2(a.lj.sig6f[pa], a.lj.sig6f[pb]);
                    eps48 = make_float2(48.0f * a.lj.epsf[pa], 48.0f * a.lj.epsf[pb]);
                }
                const float2 S2 = make_float2(rcp_approx(R.x), rcp_approx(R.y));
                const float2 S6 = __fmul2_rn(__fmul2_rn(S2, S2), __fmul2_rn(S2, sig6));
                float2 F = __fmul2_rn(__fmul2_rn(S6, __fadd2_rn(S6, half2)), __fmul2_rn(S2, eps48));
                F.x = ina ? F.x : 0.0f;
                F.y = inb ? F.y : 0.0f;
                FX = __ffma2_rn(dX, F, FX);
                FY = __ffma2_rn(dY, F, FY);
                FZ = __ffma2_rn(dZ, F, FZ);
                if(ina || inb) {
                    const float2 px = __fmul2_rn(dX, F), py = __fmul2_rn(dY, F), pz = __fmul2_rn(dZ, F);
                    red_add_v4(a.p.force32 + 4 * (size_t) (cur[u] & kPcIndexMask), -(px.x + px.y), -(py.x + py.y),
                               -(pz.x + pz.y));
                    if(kEnergy) {
                        const int pa = kOneType ? 0 : ta + fj[u].w, pb = kOneType ? 0 : tb + fj[u].w;
                        if(ina) {
                            pe += 4.0 * (double) a.lj.epsf[pa] * ((double) S6.x * (double) S6.x - (double) S6.x);
                            vir += (double) (R.x * F.x);
                        }
                        if(inb) {
                            pe += 4.0 * (double) a.lj.epsf[pb] * ((double) S6.y * (double) S6.y - (double) S6.y);
                            vir += (double) (R.y * F.y);
                        }
                    }
                }
                if(ma && na) { pend_a |= 1u << u; }
                if(mb && nbd) { pend_b |= 1u << u; }
            }
            if((pend_a | pend_b) != 0u) {
#pragma unroll
                for(int u = 0; u < kPcBatch; u++) {
                    const int j = (int) (cur[u] & kPcIndexMask);
                    if(pend_a & (1u << u)) { cut_queue_push(a.cut_count, a.cut_rec, a.cut_capacity, ia, (uint32_t) j); }
                    if(pend_b & (1u << u)) { cut_queue_push(a.cut_count, a.cut_rec, a.cut_capacity, ib, (uint32_t) j); }
                }
            }
#pragma unroll
            for(int u = 0; u < kPcBatch; u++) { cur[u] = nxt[u]; }
        }
        red_add_v4(a.p.force32 + 4 * (size_t) ia, FX.x, FY.x, FZ.x);
        if(has_b) { red_add_v4(a.p.force32 + 4 * (size_t) ib, FX.y, FY.y, FZ.y); }
    }
    if(kEnergy) { pc_block_energy(pe, vir, a.energy); }
}

// One pair of the cutoff band, decided by the FP64 path's own test on the image of the
// partner nearest the particle (the image the reference's ghost carries; the pair is
// far closer than half a box), then applied as the main pass would have: the FP32 force
// on the particle and its reaction on the partner.
template<bool kOneType, bool kEnergy, bool kEns>
__device__ void pc_fixup_pair(const PcForceArgs &a, int i, int j) {
    float fu[3];
    const double *len;
    pc_units<kEns>(a, i, fu, &len);
    const D4 xi = ld_d4_rare(a.p.pos, i), xj = ld_d4_rare(a.p.pos, j);
    const double di[3] = {xi.x - xj.x, xi.y - xj.y, xi.z - xj.z};
    int s[3];
    for(int d = 0; d < 3; d++) {
        const double h = 0.5 * len[d];
        s[d] = di[d] > h ? 1 : (di[d] < -h ? -1 : 0);
    }
    const double dx = __dsub_rn(xi.x, ref_image(xj.x, s[0], len[0]));
    const double dy = __dsub_rn(xi.y, ref_image(xj.y, s[1], len[1]));
    const double dz = __dsub_rn(xi.z, ref_image(xj.z, s[2], len[2]));
    if(!(ref_rsq(dx, dy, dz) < a.lj.cutoff2)) { return; }
    const int4 fi = ld_i4(a.p.pos_fx, i), fj = ld_i4(a.p.pos_fx, j);
    const float ex = __fmul_rn((float) fx_diff(fi.x, fj.x), fu[0]);
    const float ey = __fmul_rn((float) fx_diff(fi.y, fj.y), fu[1]);
    const float ez = __fmul_rn((float) fx_diff(fi.z, fj.z), fu[2]);
    const float rsq = pair_rsq(ex, ey, ez);
    const int tij = kOneType ? 0 : fi.w * a.lj.ntypes + fj.w;
    const float s2 = rcp_approx(rsq);
    const float s6 = __fmul_rn(__fmul_rn(s2, s2), __fmul_rn(s2, a.lj.sig6f[tij]));
    const float f = __fmul_rn(__fmul_rn(s6, __fadd_rn(s6, -0.5f)), __fmul_rn(s2, 48.0f * a.lj.epsf[tij]));
    red_add_v4(a.p.force32 + 4 * (size_t) i, ex * f, ey * f, ez * f);
    red_add_v4(a.p.force32 + 4 * (size_t) j, -(ex * f), -(ey * f), -(ez * f));
    if(kEnergy) {
        atomicAdd(&a.energy[0], 4.0 * (double) a.lj.epsf[tij] * ((double) s6 * (double) s6 - (double) s6));
        atomicAdd(&a.energy[1], (double) (rsq * f));
    }
}

// The band pairs the main pass left out: the queued records, or, when more pairs fell
// in the band than the queue holds, every cluster list walked again with the main
// pass's screen arithmetic (which finds exactly the pairs it left out).
template<bool kOneType, bool kEnergy, bool kEns>
__global__ void __launch_bounds__(kBlock) k_pc_fixup(PcForceArgs a) {
    if(frozen_force(a.p)) { return; }
    const int queued = *a.cut_count;
    const int first = blockIdx.x * blockDim.x + threadIdx.x, step = gridDim.x * blockDim.x;
    if(queued <= a.cut_capacity) {
        for(int r = first; r < queued; r += step) {
            const int2 q = a.cut_rec[r];
            pc_fixup_pair<kOneType, kEnergy, kEns>(a, q.x, q.y);
        }
        return;
    }
    const float c2 = a.lj.cutoff2f, band = c2 * kCutBand;
    for(int t = first; t < a.list.stride; t += step) {
        const int rec = a.list.pair_table[t];
        if(rec < 0) { continue; }
        const int ia = rec & (int) kPcIndexMask;
        const int ib = (rec & kPcHasB) != 0 ? ia + 1 : ia;
        const int4 fa = ld_i4(a.p.pos_fx, ia), fb = ld_i4(a.p.pos_fx, ib);
        float fu[3];
        const double *len;
        pc_units<kEns>(a, ia, fu, &len);
        const int cnt = a.list.count[t];
        for(int k = 0; k < cnt; k++) {
            const uint32_t e = (uint32_t) a.list.nbr[(size_t) k * a.list.stride + t];
            const int j = (int) (e & kPcIndexMask);
            const int4 fj = ld_i4(a.p.pos_fx, j);
            for(int m = 0; m < 2; m++) {
                if(!(e & (m == 0 ? kPcMaskA : kPcMaskB))) { continue; }
                const int4 fm = m == 0 ? fa : fb;
                const float ex = __fmul_rn((float) fx_diff(fm.x, fj.x), fu[0]);
                const float ey = __fmul_rn((float) fx_diff(fm.y, fj.y), fu[1]);
                const float ez = __fmul_rn((float) fx_diff(fm.z, fj.z), fu[2]);
                if(fabsf(pair_rsq(ex, ey, ez) - c2) < band) {
                    pc_fixup_pair<kOneType, kEnergy, kEns>(a, m == 0 ? ia : ib, j);
                }
            }
        }
    }
}

// ------------------------------------------------------------------ host side

bool fixed_point_screen(const pg_box *box, const pg_particles *p, const pg_cells *cells);

int pc_build(const pg_box *box, const pg_particles *p, const pg_cells *cells, pg_neighbor_list *list, double r_list2,
             pg_status *status, cudaStream_t st) {
    if(!list->half || !fixed_point_screen(box, p, cells)) { return PG_ERR_ARGUMENT; }
    if((int64_t) list->stride < pair_slots(p->n, cells->ncells) || p->n >= (1 << 30)) { return PG_ERR_ARGUMENT; }
    PcBuildArgs a;
    a.box = *box; a.p = *p; a.cells = *cells; a.list = *list; a.r_list2 = r_list2;
    a.r2_lo = (float) r_list2 * (1.0f - kPcScreenBand);
    a.r2_hi = (float) r_list2 * (1.0f + kPcScreenBand);
    a.replicas = nullptr; a.replica_of = nullptr; a.rebuild = nullptr;
    cudaMemsetAsync(list->pair_table, 0xff, (size_t) list->stride * sizeof(int32_t), st);
    if(cells->ncells > 0) {
        k_pc_table<<<blocks_for(cells->ncells), kBlock, 0, st>>>(*cells, list->pair_table); note_launch();
    }
    PcWindow w;
    w.clx_u = cells->cell_len[0] * box->fx_scale[0];
    w.cly_u = cells->cell_len[1] * box->fx_scale[1];
    w.clx = (float) cells->cell_len[0];
    w.cly = (float) cells->cell_len[1];
    w.r2w = (float) (r_list2 * (1.0 + 1.0e-3));
    w.scale_z = (float) box->fx_scale[2];
    const bool cubic = box->fx_unit[0] == box->fx_unit[1] && box->fx_unit[1] == box->fx_unit[2];
    const int grid = blocks_for(list->stride, kPcBuildBlock);
    if(cubic) { k_pc_build<true, false><<<grid, kPcBuildBlock, 0, st>>>(a, w, status); }
    else { k_pc_build<false, false><<<grid, kPcBuildBlock, 0, st>>>(a, w, status); }
    note_launch();
    return launch_status();
}

constexpr int kPcFixupBlocks = 2 * kSMs;

template<bool kEns>
static void pc_force_launch(const PcForceArgs &a, bool one, bool en, cudaStream_t st) {
    const int grid = blocks_for(a.list.stride, kPcBlock);
    if(one) {
        if(en) { k_pc_lj<true, true, kEns><<<grid, kPcBlock, 0, st>>>(a); k_pc_fixup<true, true, kEns><<<kPcFixupBlocks, kBlock, 0, st>>>(a); }
        else { k_pc_lj<true, false, kEns><<<grid, kPcBlock, 0, st>>>(a); k_pc_fixup<true, false, kEns><<<kPcFixupBlocks, kBlock, 0, st>>>(a); }
    } else {
        if(en) { k_pc_lj<false, true, kEns><<<grid, kPcBlock, 0, st>>>(a); k_pc_fixup<false, true, kEns><<<kPcFixupBlocks, kBlock, 0, st>>>(a); }
        else { k_pc_lj<false, false, kEns><<<grid, kPcBlock, 0, st>>>(a); k_pc_fixup<false, false, kEns><<<kPcFixupBlocks, kBlock, 0, st>>>(a); }
    }
    note_launch(2);
}

int pc_lj_force(const pg_box *box, const pg_particles *p, const pg_neighbor_list *list, const LJTable &lj,
                double *energy, int32_t *cut_count, int2 *cut_rec, int cut_capacity, cudaStream_t st) {
    if(!list->half || !p->pos_fx || !list->nbr || !list->count || !cut_count) { return PG_ERR_ARGUMENT; }
    PcForceArgs a;
    a.box = *box; a.p = *p; a.list = *list; a.lj = lj;
    a.energy = energy; a.cut_count = cut_count; a.cut_rec = cut_rec; a.cut_capacity = cut_capacity;
    a.replicas = nullptr; a.replica_of = nullptr;
    pc_force_launch<false>(a, lj.ntypes == 1, energy != nullptr, st);
    return launch_status();
}

// ------------------------------------------------------------------ batched ensembles

// Pair-cluster half lists over every replica of a batched ensemble: the table of slots
// over the shared cell arrays (a cell's slots depend only on its start and index), then
// the build with each slot's box, units and grid from its replica.  Every replica needs
// at least 2 reach + 1 cells per axis (else overflow bit 5); e->cubic promises cubic boxes.
int ens_pc_build(const pg_ensemble *e, const pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
                 double r_list2, pg_status *status, cudaStream_t st) {
    if(!e || !p || !cells || !list || !status || !list->half || !list->pair_table || !list->nbr || !list->count ||
       !p->pos || !p->pos_fx || !p->ref_fx || !p->pos_ref) {
        return PG_ERR_ARGUMENT;
    }
    if((int64_t) list->stride < pair_slots(p->n, cells->ncells) || p->n >= (1 << 30)) { return PG_ERR_ARGUMENT; }
    PcBuildArgs a;
    a.box = pg_box{}; a.p = *p; a.cells = *cells; a.list = *list; a.r_list2 = r_list2;
    a.r2_lo = (float) r_list2 * (1.0f - kPcScreenBand);
    a.r2_hi = (float) r_list2 * (1.0f + kPcScreenBand);
    a.replicas = e->replicas; a.replica_of = e->replica_of; a.rebuild = e->rebuild;
    cudaMemsetAsync(list->pair_table, 0xff, (size_t) list->stride * sizeof(int32_t), st);
    if(cells->ncells > 0) {
        k_pc_table<<<blocks_for(cells->ncells), kBlock, 0, st>>>(*cells, list->pair_table); note_launch();
    }
    PcWindow w = {};
    w.r2w = (float) (r_list2 * (1.0 + 1.0e-3));
    // cubic replicas screen in their own fixed-point units; replicas of other shapes in lengths
    const int grid = blocks_for(list->stride, kPcBuildBlock);
    if(e->cubic) { k_pc_build<true, true><<<grid, kPcBuildBlock, 0, st>>>(a, w, status); }
    else { k_pc_build<false, true><<<grid, kPcBuildBlock, 0, st>>>(a, w, status); }
    note_launch();
    return launch_status();
}

int ens_pc_force(const pg_ensemble *e, const pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                 int32_t *cut_count, int2 *cut_rec, int cut_capacity, cudaStream_t st) {
    if(!e || !lj || !list->half || !p->pos_fx || !list->nbr || !list->count || !list->pair_table || !cut_count ||
       lj->ntypes < 1 || lj->ntypes > kMaxTypes) {
        return PG_ERR_ARGUMENT;
    }
    PcForceArgs a;
    a.box = pg_box{}; a.p = *p; a.list = *list;
    a.lj.ntypes = lj->ntypes;
    a.lj.cutoff2 = lj->cutoff2;
    a.lj.cutoff2f = (float) lj->cutoff2;
    for(int k = 0; k < lj->ntypes * lj->ntypes; k++) {
        a.lj.eps[k] = lj->epsilon[k]; a.lj.sig6[k] = lj->sigma6[k];
        a.lj.epsf[k] = (float) lj->epsilon[k]; a.lj.sig6f[k] = (float) lj->sigma6[k];
    }
    a.energy = nullptr; a.cut_count = cut_count; a.cut_rec = cut_rec; a.cut_capacity = cut_capacity;
    a.replicas = e->replicas; a.replica_of = e->replica_of;
    pc_force_launch<true>(a, lj->ntypes == 1, false, st);
    return launch_status();
}

}  // namespace pg
