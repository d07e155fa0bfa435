// Batched ensemble: hundreds of independent periodic LJ replicas of uneven size,
// advanced by one launch per phase (bin, list, force, integrate, thermo) for all of
// them.
//
// The reference runs one system per generated program; every replica here follows
// the same modules as the single-system path (cells.cu, nlist.cu, lj.cu,
// integrate.cu), with the box, cell grid and FP32 position grid looked up per
// particle from the replica table.  Particles of replica r occupy [first, first+n)
// of the concatenated arrays and its cells [cell0, cell0+ncells) of the shared cell
// arrays; binning sorts by global cell, so replica ranges never mix.
//
// Small replicas would leave most SMs idle as separate launches (a 500-atom replica
// is two blocks); batched, every phase is one grid over all ~4M particles.  The
// force kernel can give each particle tpa threads (1, 2, 4 or 8) that split its
// list and combine with shuffles; the list layout interleaves tpa entries per
// particle so those threads read consecutive words.  Pair-cluster half lists
// (pairlist.cu) serve replicas too, each row on its replica's box and grid.  The
// host-side autotuner picks tpa, the block size, the stencil reach (27 cells of
// >= r_list, 125 cells of >= r_list/2, or per replica) and the list layout by timing
// them on the ensemble itself.
//
// Partial rebuilds (pg_ensemble.rebuild): binning and list build touch only the
// flagged replicas; the others keep their particle order, cells and list rows, so each
// replica rebuilds on its own displacement cycle.
#include "common.cuh"
#include "persist.cuh"

namespace pg {

int bin_prepare(int32_t n, int32_t ncells, pg_workspace ws, int32_t **count, cudaStream_t st);
int bin_finish(int32_t n, int32_t ncells, pg_workspace ws, pg_particles *p, pg_cells *cells, pg_status *status,
               cudaStream_t st, int32_t **perm_out, const pg_box *split_box, RepMask mask,
               const pg_replica *split_replicas);

// the replicas of a partial rebuild (e.rebuild), as a mask over particles
__host__ __device__ __forceinline__ RepMask ens_mask(const pg_ensemble &e) {
    RepMask m;
    m.rebuild = e.rebuild;
    m.replica_of = e.replica_of;
    return m;
}

constexpr float kEnsBand = 1.0e-4f;

struct EnsArgs {
    pg_ensemble e;
    pg_particles p;
    pg_cells cells;
    pg_neighbor_list list;
    double r_list2;
    float r2_lo, r2_hi;
    int ntypes;
    float cutoff2;
    double cutoff2d;             // FP64 cutoff test near rc (kCutBand)
    int32_t *cut_count;          // queue of near-cutoff pairs (particle, list entry)
    int2 *cut_rec;
    int cut_capacity;
    float eps[64];
    float sig6[64];
    // integration
    double dt, kick, half_skin2;
    float half_skin2_lo, half_skin2_hi;
    int32_t step;
    int drift;
    pg_status *status;
};

// ------------------------------------------------------------------ binning

__global__ void __launch_bounds__(kBlock) k_ens_count(EnsArgs a, int32_t *count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.p.n || ens_mask(a.e).skip(i)) { return; }
    const pg_replica &R = a.e.replicas[a.e.replica_of[i]];
    D4 x = ld_d4_plain(a.p.pos, i);
    double c3[3] = {x.x, x.y, x.z};
    bool moved = false, finite = true;
    for(int d = 0; d < 3; d++) {
        if(!isfinite(c3[d])) { finite = false; }
        const double lo = R.lo[d], hi = __dadd_rn(R.lo[d], R.len[d]);
        if(c3[d] < lo) { c3[d] = __dadd_rn(c3[d], R.len[d]); moved = true; }
        else if(c3[d] > hi) { c3[d] = __dadd_rn(c3[d], -R.len[d]); moved = true; }
    }
    if(moved) {
        x.x = c3[0]; x.y = c3[1]; x.z = c3[2];
        st_d4(a.p.pos, i, x);
    }
    int cell;
    if(!finite) {
        atomicExch(&a.status->nonfinite, 1);
        cell = a.e.ncells;
    } else {
        // multiplied by the inverse, floor and conversion in one round-down conversion
        // (a division per axis made this pass FP64-bound: 301 us at 3.7M atoms)
        int idx = 0;
        for(int d = 0; d < 3; d++) {
            int c = __double2int_rd(__dmul_rn(__dsub_rn(c3[d], R.lo[d]), R.inv_cell_len[d]));
            c = c < 0 ? 0 : (c >= R.dims[d] ? R.dims[d] - 1 : c);
            idx = idx * R.dims[d] + c;
        }
        cell = R.cell0 + idx;
    }
    a.cells.particle_cell[i] = cell;
    atomicAdd(&count[cell], 1);
}

// A partial rebuild: the cells of a replica left alone keep their counts (one block per
// replica), so the scan gives every cell its old start; its particles stay where they are.
__global__ void __launch_bounds__(kBlock) k_ens_count_keep(EnsArgs a, int32_t *count) {
    if(a.e.rebuild[blockIdx.x] != 0) { return; }
    const pg_replica &R = a.e.replicas[blockIdx.x];
    for(int c = threadIdx.x; c < R.ncells; c += blockDim.x) { count[R.cell0 + c] = a.cells.cell_count[R.cell0 + c]; }
}

// fixed-point position on a replica's own box (2^32 units per box length)
__device__ __forceinline__ int4 ens_fx(const pg_replica &R, const D4 &x, int type) {
    return replica_fx(R, x.x, x.y, x.z, type);
}

// ------------------------------------------------------------------ list build

__device__ __forceinline__ float ens_delta(float hi_i, float lo_i, float hi_j, float lo_j, int s, float len_hi,
                                           float len_lo) {
    const float sh = s == 0 ? 0.0f : (s > 0 ? len_hi : -len_hi);
    const float sl = s == 0 ? 0.0f : (s > 0 ? len_lo : -len_lo);
    return __fadd_rn(__fsub_rn(__fsub_rn(hi_i, hi_j), sh), __fsub_rn(__fsub_rn(lo_i, lo_j), sl));
}

// a periodic stencil coordinate c in [-dims, 2 dims): neighbour cell and image shift
// (offsets beyond one box are skipped by the caller; replicas are larger than
// 2 r_list, so they hold no partner)
__device__ __forceinline__ void wrap_cell(int c, int dims, int &nc, int &s) {
    nc = c; s = 0;
    if(nc < 0) { nc += dims; s = -1; }
    else if(nc >= dims) { nc -= dims; s = 1; }
}

__global__ void __launch_bounds__(kBlock) k_ens_list(EnsArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.p.n || ens_mask(a.e).skip(i)) { return; }      // a replica left alone keeps its list
    const D4 xi = ld_d4(a.p.pos, i);
    st_d4(a.p.pos_ref, i, xi);
    const float4 hi = ld_f4(a.p.pos_hi, hl(a.p, i)), lo = ld_f4(a.p.pos_lo, hl(a.p, i));
    if(a.p.ref_fx != nullptr) {
        st_i4(a.p.ref_fx, i, ld_i4(a.p.pos_fx, i));
    } else {
        st_f4(a.p.ref_hi, i, hi);
        st_f4(a.p.ref_lo, i, lo);
    }
    const pg_replica &R = a.e.replicas[a.e.replica_of[i]];
    const int tpa = a.e.tpa;
    int cnt = 0;
    const int ci = a.cells.particle_cell[i] - R.cell0;
    if(ci >= 0 && ci < R.ncells) {
        const int dz_ = R.dims[2], dy_ = R.dims[1], dx_ = R.dims[0], rr = R.reach;
        const int rx = R.reach_x > 0 ? R.reach_x : rr;
        const int cz = ci % dz_, cy = (ci / dz_) % dy_, cx = ci / (dz_ * dy_);
        const int stride = a.list.stride, cap = a.list.max_neighbors;
        // fixed-point screen where the replica's grid keeps every candidate's stencil
        // image within half a box (at least 2 reach + 2 cells per axis; see
        // nlist.cu), the compensated one elsewhere
        const bool fxs = a.p.pos_fx != nullptr && dx_ >= 2 * rx + 2 && dy_ >= 2 * rr + 2 && dz_ >= 2 * rr + 2;
        const int4 fi = fxs ? ld_i4(a.p.pos_fx, i) : make_int4(0, 0, 0, 0);
        int32_t *wp = a.list.nbr + (size_t) i * tpa;       // entry 0 of the interleaved layout
        const size_t row_step = (size_t) stride * tpa - (size_t) (tpa - 1);
        for(int ox = -rx; ox <= rx; ox++) {
            if(ox < -dx_ || ox > dx_) { continue; }
            int nx, sx;
            wrap_cell(cx + ox, dx_, nx, sx);
            for(int oy = -rr; oy <= rr; oy++) {
                if(oy < -dy_ || oy > dy_) { continue; }
                int ny, sy;
                wrap_cell(cy + oy, dy_, ny, sy);
                for(int oz = -rr; oz <= rr; oz++) {
                    if(oz < -dz_ || oz > dz_) { continue; }
                    int nz, sz;
                    wrap_cell(cz + oz, dz_, nz, sz);
                    const int c = R.cell0 + (nx * dy_ + ny) * dz_ + nz;
                    const uint32_t code = image_code(sx, sy, sz) << PG_NBR_INDEX_BITS;
                    // half lists as the single-system build (nlist.cu): an interior pair
                    // once, stored by the particle whose partner lies above it in x (cells
                    // of lower x skipped, the own x slab tested per candidate); a pair
                    // through an image from both sides
                    if(a.list.half && code == 0u && ox < 0) { continue; }
                    const bool slab = a.list.half && code == 0u && ox == 0;
                    const int b = a.cells.cell_start[c], e = b + a.cells.cell_count[c];
                    for(int j = b; j < e; j++) {
                        if(j == i && code == 0u) { continue; }
                        float fx, fy, fz;
                        if(fxs) {
                            const int4 fj = ld_i4(a.p.pos_fx, j);
                            fx = (float) fx_diff(fi.x, fj.x) * R.fx_unit[0];
                            fy = (float) fx_diff(fi.y, fj.y) * R.fx_unit[1];
                            fz = (float) fx_diff(fi.z, fj.z) * R.fx_unit[2];
                        } else {
                            const float4 hj = ld_f4(a.p.pos_hi, hl(a.p, j)), lj = ld_f4(a.p.pos_lo, hl(a.p, j));
                            fx = ens_delta(hi.x, lo.x, hj.x, lj.x, sx, R.len_hi[0], R.len_lo[0]);
                            fy = ens_delta(hi.y, lo.y, hj.y, lj.y, sy, R.len_hi[1], R.len_lo[1]);
                            fz = ens_delta(hi.z, lo.z, hj.z, lj.z, sz, R.len_hi[2], R.len_lo[2]);
                        }
                        if(slab && !partner_above(fx, fy, fz, i, j)) { continue; }
                        const float r2f = fx * fx + fy * fy + fz * fz;
                        bool keep;
                        if(r2f < a.r2_lo) { keep = true; }
                        else if(r2f > a.r2_hi) { keep = false; }
                        else {
                            const D4 xj = ld_d4(a.p.pos, j);
                            const double ddx = __dsub_rn(xi.x, ref_image(xj.x, sx, R.len[0]));
                            const double ddy = __dsub_rn(xi.y, ref_image(xj.y, sy, R.len[1]));
                            const double ddz = __dsub_rn(xi.z, ref_image(xj.z, sz, R.len[2]));
                            keep = ref_rsq(ddx, ddy, ddz) < a.r_list2;
                        }
                        if(keep) {
                            if(cnt < cap) {
                                *wp = (int32_t) (code | (uint32_t) j);
                                wp += ((cnt + 1) & (tpa - 1)) == 0 ? row_step : 1;
                            }
                            cnt++;
                        }
                    }
                }
            }
        }
    }
    a.list.count[i] = cnt < a.list.max_neighbors ? cnt : a.list.max_neighbors;
    publish_count(cnt, a.list.max_neighbors, a.status);
}

// ------------------------------------------------------------------ force

__device__ __forceinline__ float ens_lj(const EnsArgs &a, int tij, float rsq) {
    const float sr2 = rcp_approx(rsq);
    const float sr6 = sr2 * sr2 * sr2 * a.sig6[tij];
    return 48.0f * sr6 * (sr6 - 0.5f) * sr2 * a.eps[tij];
}

// Entries are taken in batches of kEnsBatch per thread: the batch's list words and
// partner positions are loaded before its pairs are computed.  A pair within kCutBand
// of the cutoff is queued for k_ens_cutoff_fixup, which decides it in FP64.
constexpr int kEnsBatch = 4;

// The replica's FP32 units and periodic shifts, held in registers by the force pass:
// read through the replica table in the pair loop, they would be loaded again after
// every reaction `red`, whose memory clobber the compiler cannot see past.
struct RepLen {
    float u[3];                  // fixed-point unit per axis
    float h[3], l[3];            // len_hi, len_lo
};

__device__ __forceinline__ RepLen rep_len(const pg_replica &R) {
    RepLen L;
    for(int d = 0; d < 3; d++) { L.u[d] = R.fx_unit[d]; L.h[d] = R.len_hi[d]; L.l[d] = R.len_lo[d]; }
    return L;
}

// A pair's separation: fixed point (wrapped difference in the replica's units, no
// image shift) or compensated hi/lo with the listed image's exact shift.
template<bool kFixed>
__device__ __forceinline__ void ens_pair_delta(const RepLen &L, const int4 &fi, const float4 &hi, const float4 &lo,
                                               const int4 &fj, const float4 &hj, const float4 &lj, uint32_t code,
                                               float &dx, float &dy, float &dz) {
    if(kFixed) {
        dx = (float) fx_diff(fi.x, fj.x) * L.u[0];
        dy = (float) fx_diff(fi.y, fj.y) * L.u[1];
        dz = (float) fx_diff(fi.z, fj.z) * L.u[2];
    } else {
        float dhx = hi.x - hj.x, dhy = hi.y - hj.y, dhz = hi.z - hj.z;
        float dlx = lo.x - lj.x, dly = lo.y - lj.y, dlz = lo.z - lj.z;
        if(code != 0u) {
            const int sx = image_shift(code, 0), sy = image_shift(code, 1), sz = image_shift(code, 2);
            dhx -= sx * L.h[0]; dlx -= sx * L.l[0];
            dhy -= sy * L.h[1]; dly -= sy * L.l[1];
            dhz -= sz * L.h[2]; dlz -= sz * L.l[2];
        }
        dx = dhx + dlx; dy = dhy + dly; dz = dhz + dlz;
    }
}

// fixed-point record of particle i: through the read-only path, or (kCoherent) through
// L2 only, for a kernel that rewrites the positions while it runs (persistent steps)
template<bool kCoherent>
__device__ __forceinline__ int4 ens_ld_fx(const int32_t *base, int i) {
    const int4 *p = reinterpret_cast<const int4 *>(base) + i;
    return kCoherent ? __ldcg(p) : __ldg(p);
}

// The pair forces of item g (particle g / TPA, lane g % TPA); every lane of a warp calls
// it (the lanes of a particle combine with shuffles), items past the particles idle.
template<int TPA, bool kOneType, bool kFixed, bool kCoherent>
__device__ __forceinline__ void ens_force_item(const EnsArgs &a, int g) {
    const int i = g / TPA, t = g % TPA;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    if(i < a.p.n) {
        float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
        int4 fi = make_int4(0, 0, 0, 0);
        if(kFixed) { fi = ens_ld_fx<kCoherent>(a.p.pos_fx, i); }
        else { hi = ld_f4(a.p.pos_hi, hl(a.p, i)); lo = ld_f4(a.p.pos_lo, hl(a.p, i)); }
        const RepLen L = rep_len(a.e.replicas[a.e.replica_of[i]]);
        const int ti = kOneType ? 0 : (kFixed ? fi.w : __float_as_int(hi.w)) * a.ntypes;
        const int cnt = a.list.count[i];
        const int rows = cnt > t ? (cnt - t + TPA - 1) / TPA : 0;      // this lane's entries
        const int32_t *nb = a.list.nbr + (size_t) i * TPA + t;
        const size_t row = (size_t) a.list.stride * TPA;
        const float c2 = a.cutoff2, band = c2 * kCutBand;
        for(int r0 = 0; r0 < rows; r0 += kEnsBatch) {
            uint32_t e[kEnsBatch];
            float4 hj[kEnsBatch], lj[kEnsBatch];
            int4 fj[kEnsBatch];
#pragma unroll
            for(int u = 0; u < kEnsBatch; u++) {
                e[u] = r0 + u < rows ? (uint32_t) __ldcs(nb + (r0 + u) * row) : 0u;
            }
#pragma unroll
            for(int u = 0; u < kEnsBatch; u++) {
                const int j = (int) (e[u] & PG_NBR_INDEX_MASK);
                if(kFixed) {
                    fj[u] = ens_ld_fx<kCoherent>(a.p.pos_fx, j);
                    hj[u] = lj[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                } else {
                    hj[u] = ld_f4(a.p.pos_hi, hl(a.p, j));
                    lj[u] = ld_f4(a.p.pos_lo, hl(a.p, j));
                    fj[u] = make_int4(0, 0, 0, 0);
                }
            }
            uint32_t pending = 0u;
#pragma unroll
            for(int u = 0; u < kEnsBatch; u++) {
                if(r0 + u >= rows) { continue; }
                float dx, dy, dz;
                ens_pair_delta<kFixed>(L, fi, hi, lo, fj[u], hj[u], lj[u], e[u] >> PG_NBR_INDEX_BITS, dx, dy, dz);
                const float rsq = pair_rsq(dx, dy, dz);
                const bool near = fabsf(rsq - c2) < band;
                if(rsq < c2 && !near) {
                    const int tj = kFixed ? fj[u].w : __float_as_int(hj[u].w);
                    const float f = ens_lj(a, kOneType ? 0 : ti + tj, rsq);
                    fx += dx * f; fy += dy * f; fz += dz * f;
                    if(a.list.half && (e[u] >> PG_NBR_INDEX_BITS) == 0u) {
                        red_add_v4(a.p.force32 + 4 * (size_t) (e[u] & PG_NBR_INDEX_MASK), -dx * f, -dy * f, -dz * f);
                    }
                }
                if(near) { pending |= 1u << u; }
            }
            if(pending != 0u) {
#pragma unroll
                for(int u = 0; u < kEnsBatch; u++) {
                    if(pending & (1u << u)) { cut_queue_push(a.cut_count, a.cut_rec, a.cut_capacity, i, e[u]); }
                }
            }
        }
    }
    if(TPA > 1) {
        for(int o = TPA / 2; o > 0; o >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o);
            fy += __shfl_xor_sync(0xffffffffu, fy, o);
            fz += __shfl_xor_sync(0xffffffffu, fz, o);
        }
    }
    if(i < a.p.n && t == 0) {
        if(a.list.half) { red_add_v4(a.p.force32 + 4 * (size_t) i, fx, fy, fz); }   // reactions add too
        else { st_f4(a.p.force32, i, make_float4(fx, fy, fz, 0.0f)); }
    }
}

template<int TPA, bool kOneType, bool kFixed>
__global__ void k_ens_force(EnsArgs a) {
    if(frozen_force(a.p)) { return; }
    ens_force_item<TPA, kOneType, kFixed, false>(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// One pair of the cutoff band: the FP64 test of the single-system FP64 path decides;
// a pair inside adds its FP32 force (full lists: no reaction).
// the FP64 cutoff test of a listed image through L2-only loads (persistent steps)
__device__ __forceinline__ bool exact_inside_coherent(const double *pos, int i, int j, uint32_t code, const double *len,
                                                      double cutoff2) {
    const double2 *pi = reinterpret_cast<const double2 *>(pos + 4 * (size_t) i);
    const double2 *pj = reinterpret_cast<const double2 *>(pos + 4 * (size_t) j);
    const double2 ai = __ldcg(pi), bi = __ldcg(pi + 1), aj = __ldcg(pj), bj = __ldcg(pj + 1);
    const double jx = ref_image(aj.x, image_shift(code, 0), len[0]);
    const double jy = ref_image(aj.y, image_shift(code, 1), len[1]);
    const double jz = ref_image(bj.x, image_shift(code, 2), len[2]);
    return ref_rsq(__dsub_rn(ai.x, jx), __dsub_rn(ai.y, jy), __dsub_rn(bi.x, jz)) < cutoff2;
}

template<bool kOneType, bool kFixed, bool kCoherent = false>
__device__ __forceinline__ void ens_fixup_pair(const EnsArgs &a, int i, uint32_t e) {
    const int j = (int) (e & PG_NBR_INDEX_MASK);
    const uint32_t code = e >> PG_NBR_INDEX_BITS;
    const pg_replica &R = a.e.replicas[a.e.replica_of[i]];
    if(kCoherent ? !exact_inside_coherent(a.p.pos, i, j, code, R.len, a.cutoff2d)
                 : !exact_inside(a.p.pos, i, j, code, R.len, a.cutoff2d)) { return; }
    float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi, hj = hi, lj = hi;
    int4 fi = make_int4(0, 0, 0, 0), fj = fi;
    if(kFixed) {
        fi = ens_ld_fx<kCoherent>(a.p.pos_fx, i); fj = ens_ld_fx<kCoherent>(a.p.pos_fx, j);
    } else {
        hi = ld_f4(a.p.pos_hi, hl(a.p, i)); lo = ld_f4(a.p.pos_lo, hl(a.p, i));
        hj = ld_f4(a.p.pos_hi, hl(a.p, j)); lj = ld_f4(a.p.pos_lo, hl(a.p, j));
    }
    float dx, dy, dz;
    ens_pair_delta<kFixed>(rep_len(R), fi, hi, lo, fj, hj, lj, code, dx, dy, dz);
    const int ti = kFixed ? fi.w : __float_as_int(hi.w), tj = kFixed ? fj.w : __float_as_int(hj.w);
    const int tij = kOneType ? 0 : ti * a.ntypes + tj;
    const float f = ens_lj(a, tij, pair_rsq(dx, dy, dz));
    red_add_v4(a.p.force32 + 4 * (size_t) i, dx * f, dy * f, dz * f);
    if(a.list.half && code == 0u) { red_add_v4(a.p.force32 + 4 * (size_t) j, -dx * f, -dy * f, -dz * f); }
}

// The cutoff band's pairs, left out by the force pass: the queued records, or, when
// the queue overflowed (more band pairs than the workspace holds), every list walked
// again with the force pass's screen (see k_lj_cutoff_fixup).
template<bool kOneType, bool kFixed>
__global__ void __launch_bounds__(kBlock) k_ens_cutoff_fixup(EnsArgs a) {
    if(frozen_force(a.p)) { return; }
    const int queued = *a.cut_count;
    const int first = blockIdx.x * blockDim.x + threadIdx.x, step = gridDim.x * blockDim.x;
    if(queued <= a.cut_capacity) {
        for(int r = first; r < queued; r += step) {
            const int2 q = a.cut_rec[r];
            ens_fixup_pair<kOneType, kFixed>(a, q.x, (uint32_t) q.y);
        }
        return;
    }
    const float c2 = a.cutoff2, band = c2 * kCutBand;
    const int tpa = a.e.tpa;
    const size_t row = (size_t) a.list.stride * tpa;
    for(int i = first; i < a.p.n; i += step) {
        float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
        int4 fi = make_int4(0, 0, 0, 0);
        if(kFixed) { fi = ld_i4(a.p.pos_fx, i); }
        else { hi = ld_f4(a.p.pos_hi, hl(a.p, i)); lo = ld_f4(a.p.pos_lo, hl(a.p, i)); }
        const RepLen L = rep_len(a.e.replicas[a.e.replica_of[i]]);
        const int cnt = a.list.count[i];
        for(int k = 0; k < cnt; k++) {
            const uint32_t e = (uint32_t) a.list.nbr[(size_t) (k / tpa) * row + (size_t) i * tpa + k % tpa];
            const int j = (int) (e & PG_NBR_INDEX_MASK);
            float4 hj = make_float4(0.f, 0.f, 0.f, 0.f), lj = hj;
            int4 fj = make_int4(0, 0, 0, 0);
            if(kFixed) { fj = ld_i4(a.p.pos_fx, j); }
            else { hj = ld_f4(a.p.pos_hi, hl(a.p, j)); lj = ld_f4(a.p.pos_lo, hl(a.p, j)); }
            float dx, dy, dz;
            ens_pair_delta<kFixed>(L, fi, hi, lo, fj, hj, lj, e >> PG_NBR_INDEX_BITS, dx, dy, dz);
            if(fabsf(pair_rsq(dx, dy, dz) - c2) < band) { ens_fixup_pair<kOneType, kFixed>(a, i, e); }
        }
    }
}

// ------------------------------------------------------------------ integrate

// grid point nearest x, rounded in FP64 (|lo| <= q/2)
__device__ __forceinline__ void ens_resplit(double x, float q, float iq, float &hi, float &lo) {
    split_pos(x, (double) iq, (double) q, hi, lo);
}

// The integration of particle i (k_ens_integrate); returns whether its guard tripped.
// kCoherent: the force is read through L2 only (the persistent steps, where other
// blocks' reactions wrote it during the launch).
template<bool kCoherent>
__device__ __forceinline__ bool ens_integrate_item(const EnsArgs &a, int i) {
    bool tripped = false;
    if(i < a.p.n) {
        // a coherent load: with half lists this pass then zeroes the force (it is the last
        // reader before the next force pass, which accumulates reactions into zeros), and a
        // read-only-cache load could be moved past that store
        const float4 f = kCoherent ? __ldcg(reinterpret_cast<const float4 *>(a.p.force32) + i)
                                   : reinterpret_cast<const float4 *>(a.p.force32)[i];
        const double m = a.p.mass[i];
        const double c = m == 1.0 ? a.kick : a.kick / m;
        D4 v = ld_d4_plain(a.p.vel, i);
        v.x = fma(c, (double) f.x, v.x);
        v.y = fma(c, (double) f.y, v.y);
        v.z = fma(c, (double) f.z, v.z);
        st_d4(a.p.vel, i, v);
        if(a.drift) {
            D4 x = ld_d4_plain(a.p.pos, i);
            x.x = fma(a.dt, v.x, x.x);
            x.y = fma(a.dt, v.y, x.y);
            x.z = fma(a.dt, v.z, x.z);
            st_d4(a.p.pos, i, x);
            const pg_replica &R = a.e.replicas[a.e.replica_of[i]];
            const int type = a.p.type != nullptr ? a.p.type[i] : 0;
            float dx, dy, dz;
            if(a.p.pos_fx != nullptr) {
                // fixed point only: hi/lo are split again at the next binning, which is
                // the only reader of them
                const int4 xf = ens_fx(R, x, type);
                st_i4(a.p.pos_fx, i, xf);
                const int4 rf = ld_i4(a.p.ref_fx, i);
                dx = (float) fx_diff(xf.x, rf.x) * R.fx_unit[0];
                dy = (float) fx_diff(xf.y, rf.y) * R.fx_unit[1];
                dz = (float) fx_diff(xf.z, rf.z) * R.fx_unit[2];
            } else {
                const float q = (float) R.quantum, iq = 1.0f / q;
                float4 h, l;
                ens_resplit(x.x, q, iq, h.x, l.x);
                ens_resplit(x.y, q, iq, h.y, l.y);
                ens_resplit(x.z, q, iq, h.z, l.z);
                h.w = __int_as_float(type);
                l.w = 0.0f;
                st_f4(a.p.pos_hi, hl(a.p, i), h);
                st_f4(a.p.pos_lo, hl(a.p, i), l);
                const float4 rh = ld_f4(a.p.ref_hi, i);
                const float4 rl = ld_f4(a.p.ref_lo, i);
                dx = (h.x - rh.x) + (l.x - rl.x);
                dy = (h.y - rh.y) + (l.y - rl.y);
                dz = (h.z - rh.z) + (l.z - rl.z);
            }
            const float d2 = dx * dx + dy * dy + dz * dz;
            if(d2 > a.half_skin2_hi) {
                tripped = true;
            } else if(d2 > a.half_skin2_lo) {
                const D4 r = ld_d4_plain(a.p.pos_ref, i);
                const double ex = x.x - r.x, ey = x.y - r.y, ez = x.z - r.z;
                tripped = (ex * ex + ey * ey + ez * ez) > a.half_skin2;
            }
            // the zeroing comes last: a store right after the load of the same force
            // held back every later load until that load had returned (342 vs 134 us
            // per launch at 3.7M atoms)
            if(a.e.half) { st_f4(a.p.force32, i, make_float4(0.0f, 0.0f, 0.0f, 0.0f)); }
        }
    }
    return tripped;
}

__global__ void __launch_bounds__(kBlock) k_ens_integrate(EnsArgs a) {
    if(a.drift ? frozen_integrate(a.p) : frozen_force(a.p)) { return; }
    const bool tripped = ens_integrate_item<false>(a, blockIdx.x * blockDim.x + threadIdx.x);
    if(__any_sync(0xffffffffu, tripped) && (threadIdx.x & 31) == 0) {
        atomicMin(&a.status->guard_tripped, a.step);
    }
}

// The replicas of the next partial rebuild: those with a particle whose displacement
// since the replica's last list build (the guard's FP32 measure: fixed point, or the
// hi/lo pair) exceeds sqrt(thresh2), or is not a number.  One thread per particle over
// flags zeroed before; a flag already set is not stored again.  thresh2 below the
// guard's skin^2 / 4 selects every replica the guard tripped on.
__global__ void __launch_bounds__(kBlock) k_ens_select(EnsArgs a, float thresh2, int32_t *rebuild) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.p.n) { return; }
    const int r = a.e.replica_of[i];
    const pg_replica &R = a.e.replicas[r];
    float dx, dy, dz;
    if(a.p.pos_fx != nullptr) {
        const int4 xf = ld_i4(a.p.pos_fx, i), rf = ld_i4(a.p.ref_fx, i);
        dx = (float) fx_diff(xf.x, rf.x) * R.fx_unit[0];
        dy = (float) fx_diff(xf.y, rf.y) * R.fx_unit[1];
        dz = (float) fx_diff(xf.z, rf.z) * R.fx_unit[2];
    } else {
        const float4 h = ld_f4(a.p.pos_hi, hl(a.p, i)), l = ld_f4(a.p.pos_lo, hl(a.p, i));
        const float4 rh = ld_f4(a.p.ref_hi, i), rl = ld_f4(a.p.ref_lo, i);
        dx = (h.x - rh.x) + (l.x - rl.x);
        dy = (h.y - rh.y) + (l.y - rl.y);
        dz = (h.z - rh.z) + (l.z - rl.z);
    }
    const float d2 = dx * dx + dy * dy + dz * dz;
    if(!(d2 <= thresh2) && rebuild[r] == 0) { rebuild[r] = 1; }
}

__global__ void k_ens_select_all(int nreplicas, int32_t *rebuild) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if(r < nreplicas) { rebuild[r] = 1; }
}

// ------------------------------------------------------------------ persistent steps

// The plain steps of a chunk in one cooperative launch (pg_ensemble_steps): for each
// step the integration (two half kicks, drift, fixed-point records, the FP64 guard),
// a grid barrier, the force pass, a barrier, the cutoff band's FP64 decisions, a
// barrier -- the arithmetic of k_ens_integrate, k_ens_force and k_ens_cutoff_fixup,
// every replica at once.  Data other blocks rewrite during the launch (fixed-point
// and FP64 positions, forces) is read through L2 only.  A trip in the integration of
// step r ends the launch before the force of step r, as the separate kernels skip
// themselves; a barrier that waits past the time limit sets status->overflow bit 16
// and every block leaves (persist.cuh).
constexpr int kEnsPersistBlock = 128;

struct EnsStepsArgs {
    EnsArgs a;
    PersistWs ws;
    int32_t first, nsteps;
    unsigned long long limit_ns;
};

template<int TPA, bool kOneType>
__global__ void __launch_bounds__(kEnsPersistBlock) k_ens_steps(EnsStepsArgs s) {
    const EnsArgs &a = s.a;
    const unsigned nblocks = gridDim.x;
    const int first = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int n = a.p.n;
    const volatile int32_t *guard = &a.status->guard_tripped;
    const float c2 = a.cutoff2, band = c2 * kCutBand;
    for(int k = 0; k < s.nsteps; k++) {
        const int32_t r = s.first + k;
        if(*guard < r) { break; }                    // a trip before this step froze the state
        if(first == 0) { *s.ws.cut_count = 0; }
        for(int base = 0; base < n; base += stride) {
            const bool tripped = ens_integrate_item<true>(a, base + first);
            if(__any_sync(0xffffffffu, tripped) && (threadIdx.x & 31) == 0) {
                atomicMin(&a.status->guard_tripped, r);
            }
        }
        if(!grid_barrier(s.ws, nblocks, s.limit_ns, a.status)) { break; }
        if(*guard <= r) { break; }                   // the host rebuilds at the trip step
        for(int base = 0; base < n * TPA; base += stride) {
            ens_force_item<TPA, kOneType, true, true>(a, base + first);
        }
        if(!grid_barrier(s.ws, nblocks, s.limit_ns, a.status)) { break; }
        const int queued = *reinterpret_cast<volatile const int32_t *>(s.ws.cut_count);
        if(queued <= s.ws.capacity) {
            for(int q = first; q < queued; q += stride) {
                const int2 rec = s.ws.records[q];
                ens_fixup_pair<kOneType, true, true>(a, rec.x, (uint32_t) rec.y);
            }
        } else {
            // more band pairs than the queue holds: every list again (k_ens_cutoff_fixup)
            const size_t row = (size_t) a.list.stride * TPA;
            for(int i = first; i < n; i += stride) {
                const int4 fi = ens_ld_fx<true>(a.p.pos_fx, i);
                const RepLen L = rep_len(a.e.replicas[a.e.replica_of[i]]);
                const int cnt = a.list.count[i];
                for(int m = 0; m < cnt; m++) {
                    const uint32_t e = (uint32_t) a.list.nbr[(size_t) (m / TPA) * row + (size_t) i * TPA + m % TPA];
                    const int4 fj = ens_ld_fx<true>(a.p.pos_fx, (int) (e & PG_NBR_INDEX_MASK));
                    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
                    float dx, dy, dz;
                    ens_pair_delta<true>(L, fi, z4, z4, fj, z4, z4, e >> PG_NBR_INDEX_BITS, dx, dy, dz);
                    if(fabsf(pair_rsq(dx, dy, dz) - c2) < band) { ens_fixup_pair<kOneType, true, true>(a, i, e); }
                }
            }
        }
        if(!grid_barrier(s.ws, nblocks, s.limit_ns, a.status)) { break; }
    }
}

// ------------------------------------------------------------------ thermo

__global__ void __launch_bounds__(kBlock) k_ens_thermo(EnsArgs a, double *out) {
    const pg_replica &R = a.e.replicas[blockIdx.x];
    double acc = 0.0;
    for(int i = R.first + threadIdx.x; i < R.first + R.n; i += blockDim.x) {
        const D4 v = ld_d4(a.p.vel, i);
        const double s = __dadd_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)), __dmul_rn(v.z, v.z));
        acc += __dmul_rn(a.p.mass[i], s);
    }
    __shared__ double red[kBlock / 32];
    acc = warp_sum(acc);
    if((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = acc; }
    __syncthreads();
    if(threadIdx.x == 0) {
        double sum = 0.0;
        for(int w = 0; w < (int) (blockDim.x >> 5); w++) { sum += red[w]; }
        out[2 * blockIdx.x] = sum * (1.0 / (double) (R.n * 3 - 3));
        out[2 * blockIdx.x + 1] = sum;
    }
}

// ------------------------------------------------------------------ host side

static bool ens_ok(const pg_ensemble *e, const pg_particles *p) {
    return e && p && e->replicas && e->replica_of && e->nreplicas > 0 && e->ncells >= 1 && p->n >= 0 &&
           p->n <= p->capacity &&
           (e->tpa == 1 || e->tpa == 2 || e->tpa == 4 || e->tpa == 8) && e->block >= 64 && e->block <= 512 &&
           e->block % 32 == 0;
}

int ensemble_bin(const pg_ensemble *e, pg_particles *p, pg_cells *cells, pg_workspace ws, pg_status *status,
                 cudaStream_t st) {
    // hi/lo layouts are optional with fixed-point positions (the pair-cluster path reads none)
    if(!ens_ok(e, p) || !cells || !status || !p->pos || (!p->pos_fx && (!p->pos_hi || !p->pos_lo)) ||
       (!p->pos_hi) != (!p->pos_lo) || cells->ncells != e->ncells) {
        return PG_ERR_ARGUMENT;
    }
    const int n = p->n;
    int32_t *count = nullptr;
    int rc = bin_prepare(n, e->ncells, ws, &count, st);
    if(rc) { return rc; }
    EnsArgs a = {};
    a.e = *e; a.p = *p; a.cells = *cells; a.status = status;
    if(e->rebuild != nullptr) {
        // a partial rebuild: the cell arrays must hold the last binning of every replica
        if(!cells->cell_count || !cells->cell_start) { return PG_ERR_ARGUMENT; }
        k_ens_count_keep<<<e->nreplicas, kBlock, 0, st>>>(a, count); note_launch();
    }
    if(n > 0) { k_ens_count<<<blocks_for(n), kBlock, 0, st>>>(a, count); note_launch(); }
    // the copy back refreshes hi/lo and the fixed-point records on each replica's grid
    return bin_finish(n, e->ncells, ws, p, cells, status, st, nullptr, nullptr, ens_mask(*e), e->replicas);
}

int ens_pc_build(const pg_ensemble *e, const pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
                 double r_list2, pg_status *status, cudaStream_t st);
int ens_pc_force(const pg_ensemble *e, const pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                 int32_t *cut_count, int2 *cut_rec, int cut_capacity, cudaStream_t st);

int ensemble_build_lists(const pg_ensemble *e, pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
                         double r_list2, pg_status *status, cudaStream_t st) {
    if(list != nullptr && list->pair_table != nullptr) {
        // pair-cluster half lists (pairlist.cu), each slot on its replica's box and grid
        if(!ens_ok(e, p) || !cells || (e->half == 0) || cells->ncells != e->ncells) { return PG_ERR_ARGUMENT; }
        list->steps_since_build = 0;
        return ens_pc_build(e, p, cells, list, r_list2, status, st);
    }
    if(!ens_ok(e, p) || !cells || !list || !list->nbr || !list->count || !status || !p->pos_ref || !p->pos_hi ||
       !p->pos_lo || (p->ref_fx != nullptr ? !p->pos_fx : (!p->ref_hi || !p->ref_lo)) || list->stride < p->n ||
       p->n >= (1 << PG_NBR_INDEX_BITS) || (list->half != 0) != (e->half != 0)) {
        return PG_ERR_ARGUMENT;
    }
    EnsArgs a = {};
    a.e = *e; a.p = *p; a.cells = *cells; a.list = *list; a.status = status;
    a.r_list2 = r_list2;
    a.r2_lo = (float) r_list2 * (1.0f - kEnsBand);
    a.r2_hi = (float) r_list2 * (1.0f + kEnsBand);
    if(p->n > 0) { k_ens_list<<<blocks_for(p->n), kBlock, 0, st>>>(a); note_launch(); }
    return launch_status();
}

template<int TPA>
static void launch_force(const EnsArgs &a, int n, int block, bool one, bool fixed, cudaStream_t st) {
    const int64_t threads = (int64_t) n * TPA;
    const int grid = (int) ((threads + block - 1) / block);
    if(fixed) {
        if(one) { k_ens_force<TPA, true, true><<<grid, block, 0, st>>>(a); }
        else { k_ens_force<TPA, false, true><<<grid, block, 0, st>>>(a); }
    } else {
        if(one) { k_ens_force<TPA, true, false><<<grid, block, 0, st>>>(a); }
        else { k_ens_force<TPA, false, false><<<grid, block, 0, st>>>(a); }
    }
    note_launch();
}

int ensemble_force(const pg_ensemble *e, const pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                   pg_workspace ws, cudaStream_t st) {
    const bool fixed = p->pos_fx != nullptr;
    if(!ens_ok(e, p) || !list || !list->nbr || !list->count || !lj || (!fixed && (!p->pos_hi || !p->pos_lo)) ||
       !p->force32 || lj->ntypes < 1 || lj->ntypes > 8 || (lj->ntypes > 1 && !p->type) ||
       (list->half != 0) != (e->half != 0)) {
        return PG_ERR_ARGUMENT;
    }
    EnsArgs a = {};
    a.e = *e; a.p = *p; a.list = *list;
    a.ntypes = lj->ntypes;
    a.cutoff2 = (float) lj->cutoff2;
    a.cutoff2d = lj->cutoff2;
    for(int k = 0; k < lj->ntypes * lj->ntypes; k++) {
        a.eps[k] = (float) lj->epsilon[k];
        a.sig6[k] = (float) lj->sigma6[k];
    }
    if(p->n == 0) { return PG_OK; }
    // queue of near-cutoff pairs in the workspace (scratch between binnings)
    // (one record at least; an overflowing queue makes the fixup walk every list)
    if(ws.ptr == nullptr || ws.bytes < 256 + 8) { return PG_ERR_ARGUMENT; }
    a.cut_count = (int32_t *) ws.ptr;
    a.cut_rec = (int2 *) ((char *) ws.ptr + 256);
    a.cut_capacity = (int) ((ws.bytes - 256) / 8 < INT32_MAX ? (ws.bytes - 256) / 8 : INT32_MAX);
    cudaMemsetAsync(a.cut_count, 0, sizeof(int32_t), st);
    if(list->pair_table != nullptr) {            // pair-cluster half lists (pairlist.cu)
        return ens_pc_force(e, p, list, lj, a.cut_count, a.cut_rec, a.cut_capacity, st);
    }
    const bool one = lj->ntypes == 1;
    switch(e->tpa) {
        case 1: launch_force<1>(a, p->n, e->block, one, fixed, st); break;
        case 2: launch_force<2>(a, p->n, e->block, one, fixed, st); break;
        case 4: launch_force<4>(a, p->n, e->block, one, fixed, st); break;
        default: launch_force<8>(a, p->n, e->block, one, fixed, st); break;
    }
    if(fixed) {
        if(one) { k_ens_cutoff_fixup<true, true><<<2 * kSMs, kBlock, 0, st>>>(a); }
        else { k_ens_cutoff_fixup<false, true><<<2 * kSMs, kBlock, 0, st>>>(a); }
    } else {
        if(one) { k_ens_cutoff_fixup<true, false><<<2 * kSMs, kBlock, 0, st>>>(a); }
        else { k_ens_cutoff_fixup<false, false><<<2 * kSMs, kBlock, 0, st>>>(a); }
    }
    note_launch();
    return launch_status();
}

int ensemble_integrate(const pg_ensemble *e, pg_particles *p, double dt, int kicks, int drift, double half_skin2,
                       int32_t step, pg_status *status, cudaStream_t st) {
    const bool fixed = p->pos_fx != nullptr;
    if(!ens_ok(e, p) || !p->pos || !p->vel || !p->mass || !p->force32 || (!fixed && (!p->pos_hi || !p->pos_lo)) ||
       !status || (kicks != 1 && kicks != 2) ||
       (drift && (!p->pos_ref || (fixed ? !p->ref_fx : (!p->ref_hi || !p->ref_lo))))) {
        return PG_ERR_ARGUMENT;
    }
    EnsArgs a = {};
    a.e = *e; a.p = *p; a.status = status;
    a.dt = dt;
    a.kick = kicks * (dt * 0.5);
    a.half_skin2 = half_skin2;
    a.half_skin2_lo = (float) (half_skin2 * (1.0 - 1e-3));
    a.half_skin2_hi = (float) (half_skin2 * (1.0 + 1e-3));
    a.step = step;
    a.drift = drift;
    if(p->n > 0) { k_ens_integrate<<<blocks_for(p->n), kBlock, 0, st>>>(a); note_launch(); }
    return launch_status();
}

int ensemble_steps(const pg_ensemble *e, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                   double dt, double half_skin2, int32_t first, int32_t nsteps, pg_status *status, pg_workspace ws,
                   double timeout_s, cudaStream_t st) {
    if(!ens_ok(e, p) || !list || !list->nbr || !list->count || !lj || !status || nsteps < 0 || !p->pos || !p->vel ||
       !p->mass || !p->force32 || !p->pos_fx || !p->ref_fx || !p->pos_ref || lj->ntypes < 1 || lj->ntypes > 8 ||
       (lj->ntypes > 1 && !p->type) || (list->half != 0) != (e->half != 0)) {
        return PG_ERR_ARGUMENT;
    }
    if(ws.ptr == nullptr || ws.bytes < 256 + 8 || list->pair_table != nullptr) { return PG_ERR_ARGUMENT; }
    const bool one = lj->ntypes == 1;
    typedef void (*Kernel)(EnsStepsArgs);
    Kernel k;
    int slot;
    switch(e->tpa) {
        case 1: k = one ? k_ens_steps<1, true> : k_ens_steps<1, false>; slot = 0; break;
        case 2: k = one ? k_ens_steps<2, true> : k_ens_steps<2, false>; slot = 1; break;
        case 4: k = one ? k_ens_steps<4, true> : k_ens_steps<4, false>; slot = 2; break;
        default: k = one ? k_ens_steps<8, true> : k_ens_steps<8, false>; slot = 3; break;
    }
    int grid = 0;
    const int rc = cooperative_grid(8 + 2 * slot + (one ? 1 : 0), (const void *) k, kEnsPersistBlock, &grid);
    if(rc != PG_OK) { return rc; }
    if(nsteps == 0 || p->n == 0) { return PG_OK; }         // (a call of no steps only prepares the launch)
    EnsStepsArgs sa = {};
    EnsArgs &a = sa.a;
    a.e = *e; a.p = *p; a.list = *list; a.status = status;
    a.ntypes = lj->ntypes;
    a.cutoff2 = (float) lj->cutoff2;
    a.cutoff2d = lj->cutoff2;
    for(int t = 0; t < lj->ntypes * lj->ntypes; t++) {
        a.eps[t] = (float) lj->epsilon[t];
        a.sig6[t] = (float) lj->sigma6[t];
    }
    a.dt = dt;
    a.kick = 2.0 * (dt * 0.5);
    a.drift = 1;
    a.half_skin2 = half_skin2;
    a.half_skin2_lo = (float) (half_skin2 * (1.0 - 1e-3));
    a.half_skin2_hi = (float) (half_skin2 * (1.0 + 1e-3));
    sa.ws = persist_ws(ws.ptr, ws.bytes);
    a.cut_count = sa.ws.cut_count;
    a.cut_rec = sa.ws.records;
    a.cut_capacity = sa.ws.capacity;
    sa.first = first;
    sa.nsteps = nsteps;
    sa.limit_ns = timeout_ns(timeout_s);
    cudaMemsetAsync(ws.ptr, 0, 256, st);                    // queue count, barrier words, abort word
    void *args[] = {&sa};
    if(cudaLaunchCooperativeKernel((const void *) k, grid, kEnsPersistBlock, args, 0, st) != cudaSuccess) {
        return PG_ERR_CUDA;
    }
    note_launch();
    return launch_status();
}

int ensemble_select(const pg_ensemble *e, const pg_particles *p, double thresh2, int32_t *rebuild, cudaStream_t st) {
    const bool fixed = p != nullptr && p->pos_fx != nullptr;
    if(!ens_ok(e, p) || !rebuild || (fixed ? !p->ref_fx : (!p->pos_hi || !p->pos_lo || !p->ref_hi || !p->ref_lo))) {
        return PG_ERR_ARGUMENT;
    }
    EnsArgs a = {};
    a.e = *e; a.p = *p;
    if(thresh2 < 0.0) {
        k_ens_select_all<<<blocks_for(e->nreplicas), kBlock, 0, st>>>(e->nreplicas, rebuild); note_launch();
    } else {
        cudaMemsetAsync(rebuild, 0, (size_t) e->nreplicas * sizeof(int32_t), st);
        if(p->n > 0) { k_ens_select<<<blocks_for(p->n), kBlock, 0, st>>>(a, (float) thresh2, rebuild); note_launch(); }
    }
    return launch_status();
}

int ensemble_thermo(const pg_ensemble *e, const pg_particles *p, double *out, cudaStream_t st) {
    if(!ens_ok(e, p) || !p->vel || !p->mass || !out) { return PG_ERR_ARGUMENT; }
    EnsArgs a = {};
    a.e = *e; a.p = *p;
    k_ens_thermo<<<e->nreplicas, kBlock, 0, st>>>(a, out); note_launch();
    return launch_status();
}

}  // namespace pg
