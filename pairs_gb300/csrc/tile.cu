// Tile-local Verlet lists and forces (mixed precision): shared-memory neighbourhoods.
//
// Particles are sorted by cell, z fastest, so a column of cells (x, y fixed) is one
// contiguous range of particles.  A tile is TZ consecutive cells of one column; its
// neighbourhood -- the 3x3 columns around it, cells z0-1 .. z1 -- is at most 27
// contiguous particle ranges ("segments": per column the main range plus the cells
// that wrap around a periodic z boundary).  One thread block per tile stages the
// neighbourhood's compensated positions (hi, lo) in shared memory, applying each
// segment's periodic image shift while staging (hi + s*len_hi is exact on the hi
// grid), unshifted segments first.
//
// The Verlet list of a tile particle then holds 16-bit shared-memory indices: half
// the list bytes of global indices, and every partner read is a shared-memory load
// instead of an L1/L2 gather.  The staging order depends only on the cell occupancy,
// which is fixed between rebuilds, so the indices the build kernel writes are the
// ones the force kernel stages.
//
// Acceptance is the reference's exact FP64 test (see nlist.cu): FP32 screen on the
// staged positions, FP64 decision (global positions, reference image arithmetic)
// inside a 1e-4 relative band.  Half lists keep an interior pair once (global index
// j > i) and a pair through a periodic image from both sides, as the reference.
#include "common.cuh"

namespace pg {

constexpr int kTileThreads = 256;
constexpr int kMaxSegs = 27;
constexpr float kTileBand = 1.0e-4f;

struct Seg {
    int start, count, base;      // global first particle, particles, first shared slot
    int code;                    // periodic image code (2 bits per dimension)
};

// Per column of the neighbourhood: where its cells are in shared memory.
struct Col {
    int cell0;                   // global cell index of (nx, ny, 0)
    int za, zb;                  // main (unshifted in z) cell range [za, zb]
    int main_seg, low_seg, high_seg;   // segment ids (-1 if none)
};

struct TileArgs {
    pg_box box;
    pg_particles p;
    pg_cells cells;
    pg_neighbor_list list;
    int tz, ntz;                 // cells per tile along z, tiles per column
    int capacity;                // shared-memory slots (particles)
    double r_list2;
    float r2_lo, r2_hi;
    LJTableF lj;
    double *energy;
    pg_status *status;
};

// Enumerate the neighbourhood of tile t into shared tables (one thread), unshifted
// segments first; returns the number of staged particles.  unshifted_slots = the
// shared-memory slots of the unshifted segments (slots [0, unshifted_slots)).
__device__ int tile_layout(const TileArgs &a, int t, Seg *segs, Col *cols, int &nsegs, int &unshifted_slots,
                           int &i_begin, int &i_end, int &cx, int &cy, int &z0, int &z1) {
    const int dx = a.cells.dims[0], dy = a.cells.dims[1], dz = a.cells.dims[2];
    const int zt = t % a.ntz, col = t / a.ntz;
    cy = col % dy; cx = col / dy;
    z0 = zt * a.tz; z1 = min(z0 + a.tz, dz);
    const int c_first = (cx * dy + cy) * dz;
    i_begin = a.cells.cell_start[c_first + z0];
    i_end = a.cells.cell_start[c_first + z1 - 1] + a.cells.cell_count[c_first + z1 - 1];
    Seg tmp[kMaxSegs];
    int n = 0, n_unshifted_segs = 0;
    for(int k = 0; k < 9; k++) {
        cols[k].cell0 = 0; cols[k].za = 0; cols[k].zb = -1;
        cols[k].main_seg = cols[k].low_seg = cols[k].high_seg = -1;
    }
    for(int pass = 0; pass < 2; pass++) {           // pass 0: unshifted, pass 1: shifted
        int k = 0;
        for(int ox = -1; ox <= 1; ox++) {
            int nx = cx + ox, sx = 0;
            if(nx < 0) { if(!a.box.periodic[0]) { k += 3; continue; } nx += dx; sx = -1; }
            else if(nx >= dx) { if(!a.box.periodic[0]) { k += 3; continue; } nx -= dx; sx = 1; }
            for(int oy = -1; oy <= 1; oy++, k++) {
                int ny = cy + oy, sy = 0;
                if(ny < 0) { if(!a.box.periodic[1]) { continue; } ny += dy; sy = -1; }
                else if(ny >= dy) { if(!a.box.periodic[1]) { continue; } ny -= dy; sy = 1; }
                const int cell0 = (nx * dy + ny) * dz;
                Col &cl = cols[k];
                if(pass == 0) {
                    cl.cell0 = cell0;
                    cl.za = max(z0 - 1, 0);
                    cl.zb = min(z1, dz - 1);
                }
                // main range, then the wrapped cells
                for(int part = 0; part < 3; part++) {
                    int za, zb, sz = 0;
                    if(part == 0) { za = cl.za; zb = cl.zb; }
                    else if(part == 1) {
                        if(z0 - 1 >= 0 || !a.box.periodic[2]) { continue; }
                        za = zb = dz - 1; sz = -1;
                    } else {
                        if(z1 < dz || !a.box.periodic[2]) { continue; }
                        za = zb = 0; sz = 1;
                    }
                    const uint32_t code = image_code(sx, sy, sz);
                    if((code == 0u) != (pass == 0)) { continue; }
                    Seg s;
                    s.start = a.cells.cell_start[cell0 + za];
                    s.count = a.cells.cell_start[cell0 + zb] + a.cells.cell_count[cell0 + zb] - s.start;
                    s.code = (int) code;
                    tmp[n] = s;
                    if(part == 0) { cl.main_seg = n; } else if(part == 1) { cl.low_seg = n; } else { cl.high_seg = n; }
                    n++;
                }
            }
        }
        if(pass == 0) { n_unshifted_segs = n; }
    }
    int base = 0;
    unshifted_slots = 0;
    for(int s = 0; s < n; s++) {
        if(s == n_unshifted_segs) { unshifted_slots = base; }
        tmp[s].base = base;
        base += tmp[s].count;
        segs[s] = tmp[s];
    }
    if(n_unshifted_segs == n) { unshifted_slots = base; }
    nsegs = n;
    return base;
}

// Stage hi/lo of every segment into shared memory (sm[2k] = hi, sm[2k+1] = lo).
__device__ void tile_stage(const TileArgs &a, const Seg *segs, int nsegs, float4 *sm) {
    for(int s = 0; s < nsegs; s++) {
        const Seg g = segs[s];
        const int sx = image_shift(g.code, 0), sy = image_shift(g.code, 1), sz = image_shift(g.code, 2);
        const float hx = sx * a.box.len_hi[0], hy = sy * a.box.len_hi[1], hz = sz * a.box.len_hi[2];
        const float lx = sx * a.box.len_lo[0], ly = sy * a.box.len_lo[1], lz = sz * a.box.len_lo[2];
        for(int k = threadIdx.x; k < g.count; k += blockDim.x) {
            float4 h = ld_f4(a.p.pos_hi, g.start + k);
            float4 l = ld_f4(a.p.pos_lo, g.start + k);
            h.x += hx; h.y += hy; h.z += hz;
            l.x += lx; l.y += ly; l.z += lz;
            sm[2 * (g.base + k)] = h;
            sm[2 * (g.base + k) + 1] = l;
        }
    }
}

// ------------------------------------------------------------------ list build

__global__ void __launch_bounds__(kTileThreads) k_tile_build(TileArgs a) {
    extern __shared__ float4 sm[];
    __shared__ Seg segs[kMaxSegs];
    __shared__ Col cols[9];
    __shared__ int meta[10];
    const int t = blockIdx.x;
    if(threadIdx.x == 0) {
        int nsegs, nun, ib, ie, cx, cy, z0, z1;
        const int staged = tile_layout(a, t, segs, cols, nsegs, nun, ib, ie, cx, cy, z0, z1);
        meta[0] = nsegs; meta[1] = nun; meta[2] = ib; meta[3] = ie; meta[4] = staged;
        if(staged > a.capacity) {
            atomicOr(&a.status->overflow, 4);
            atomicMax(&a.status->max_tile_staged, staged);
        }
    }
    __syncthreads();
    const int nsegs = meta[0], ib = meta[2], ie = meta[3], staged = meta[4];
    if(staged > a.capacity) { return; }
    tile_stage(a, segs, nsegs, sm);
    __syncthreads();
    const int dz = a.cells.dims[2];
    const int stride = a.list.stride, cap = a.list.max_neighbors;
    int wmax = 0;
    for(int i = ib + threadIdx.x; i < ie; i += blockDim.x) {
        const float4 hi = ld_f4(a.p.pos_hi, i), lo = ld_f4(a.p.pos_lo, i);
        const D4 xi = ld_d4(a.p.pos, i);
        st_d4(a.p.pos_ref, i, xi);
        st_f4(a.p.ref_hi, i, hi);
        st_f4(a.p.ref_lo, i, lo);
        int cnt = 0;
        const bool fixed = a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed);
        const int z = a.cells.particle_cell[i] % dz;
        uint16_t *out = a.list.nbr16 + i;
        if(!fixed) {
            for(int c = 0; c < 9; c++) {
                const Col cl = cols[c];
                if(cl.main_seg < 0 && cl.low_seg < 0 && cl.high_seg < 0) { continue; }
                for(int oz = -1; oz <= 1; oz++) {
                    const int zc = z + oz;
                    int seg, b, e;
                    if(zc >= 0 && zc < dz && cl.main_seg >= 0 && zc >= cl.za && zc <= cl.zb) {
                        seg = cl.main_seg;
                        const Seg g = segs[seg];
                        const int cg = cl.cell0 + zc;
                        b = g.base + (a.cells.cell_start[cg] - g.start);
                        e = b + a.cells.cell_count[cg];
                    } else if(zc < 0 && cl.low_seg >= 0) {
                        seg = cl.low_seg; b = segs[seg].base; e = b + segs[seg].count;
                    } else if(zc >= dz && cl.high_seg >= 0) {
                        seg = cl.high_seg; b = segs[seg].base; e = b + segs[seg].count;
                    } else {
                        continue;
                    }
                    const Seg g = segs[seg];
                    for(int js = b; js < e; js++) {
                        const int j = g.start + (js - g.base);
                        if(j == i && g.code == 0) { continue; }
                        if(a.list.half && g.code == 0 && j < i) { continue; }
                        const float4 hj = sm[2 * js], lj = sm[2 * js + 1];
                        const float fx = (hi.x - hj.x) + (lo.x - lj.x);
                        const float fy = (hi.y - hj.y) + (lo.y - lj.y);
                        const float fz = (hi.z - hj.z) + (lo.z - lj.z);
                        const float r2f = fx * fx + fy * fy + fz * fz;
                        bool keep;
                        if(r2f < a.r2_lo) { keep = true; }
                        else if(r2f > a.r2_hi) { keep = false; }
                        else {
                            const D4 xj = ld_d4(a.p.pos, j);
                            const double ddx = __dsub_rn(xi.x, ref_image(xj.x, image_shift(g.code, 0), a.box.len[0]));
                            const double ddy = __dsub_rn(xi.y, ref_image(xj.y, image_shift(g.code, 1), a.box.len[1]));
                            const double ddz = __dsub_rn(xi.z, ref_image(xj.z, image_shift(g.code, 2), a.box.len[2]));
                            keep = ref_rsq(ddx, ddy, ddz) < a.r_list2;
                        }
                        if(keep) {
                            if(cnt < cap) { out[(size_t) cnt * stride] = (uint16_t) js; }
                            cnt++;
                        }
                    }
                }
            }
        }
        a.list.count[i] = min(cnt, cap);
        wmax = max(wmax, cnt);
    }
    wmax = warp_max(wmax);
    if((threadIdx.x & 31) == 0 && wmax > 0) {
        atomicMax(&a.status->max_neighbors, wmax);
        if(wmax > cap) { atomicOr(&a.status->overflow, 2); }
    }
}

// ------------------------------------------------------------------ force

__device__ __forceinline__ void red_add_v4_global(float *addr, float a, float b, float c) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};"
                 :: "l"(addr), "f"(a), "f"(b), "f"(c), "f"(0.0f) : "memory");
}

template<bool kHalf, bool kOneType, bool kEnergy>
__global__ void __launch_bounds__(kTileThreads) k_tile_lj(TileArgs a) {
    if(frozen_force(a.p)) { return; }
    extern __shared__ float4 sm[];
    __shared__ Seg segs[kMaxSegs];
    __shared__ Col cols[9];
    __shared__ int meta[10];
    __shared__ double red[2][kTileThreads / 32];
    const int t = blockIdx.x;
    if(threadIdx.x == 0) {
        int nsegs, nun, ib, ie, cx, cy, z0, z1;
        const int staged = tile_layout(a, t, segs, cols, nsegs, nun, ib, ie, cx, cy, z0, z1);
        meta[0] = nsegs; meta[1] = nun; meta[2] = ib; meta[3] = ie; meta[4] = staged;
    }
    __syncthreads();
    const int nsegs = meta[0], nun = meta[1], ib = meta[2], ie = meta[3], staged = meta[4];
    if(staged > a.capacity) { return; }      // cannot happen after a successful build
    float4 *facc = sm + 2 * (size_t) a.capacity;            // half list: per-slot force sums
    tile_stage(a, segs, nsegs, sm);
    if(kHalf) {
        for(int k = threadIdx.x; k < nun; k += blockDim.x) { facc[k] = make_float4(0.f, 0.f, 0.f, 0.f); }
    }
    __syncthreads();
    const int stride = a.list.stride;
    const float c2 = a.lj.cutoff2;
    double pe = 0.0, vir = 0.0;
    const Seg center = segs[cols[4].main_seg];
    for(int i = ib + threadIdx.x; i < ie; i += blockDim.x) {
        float fx = 0.f, fy = 0.f, fz = 0.f;
        const bool fixed = a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed);
        if(!fixed) {
            const float4 hi = ld_f4(a.p.pos_hi, i), lo = ld_f4(a.p.pos_lo, i);
            const int ti = kOneType ? 0 : __float_as_int(hi.w) * a.lj.ntypes;
            const int cnt = a.list.count[i];
            const uint16_t *nb = a.list.nbr16 + i;
            for(int k = 0; k < cnt; k++) {
                const int js = __ldg(nb + (size_t) k * stride);
                const float4 hj = sm[2 * js], lj = sm[2 * js + 1];
                const float dx = (hi.x - hj.x) + (lo.x - lj.x);
                const float dy = (hi.y - hj.y) + (lo.y - lj.y);
                const float dz = (hi.z - hj.z) + (lo.z - lj.z);
                const float rsq = dx * dx + dy * dy + dz * dz;
                if(rsq < c2) {
                    const int tij = kOneType ? 0 : ti + __float_as_int(hj.w);
                    const float sr2 = __frcp_rn(rsq);
                    const float sr6 = sr2 * sr2 * sr2 * a.lj.sig6[tij];
                    const float f = 48.0f * sr6 * (sr6 - 0.5f) * sr2 * a.lj.eps[tij];
                    fx += dx * f; fy += dy * f; fz += dz * f;
                    const bool interior = js < nun;
                    if(kHalf && interior) {
                        atomicAdd(&facc[js].x, -dx * f);
                        atomicAdd(&facc[js].y, -dy * f);
                        atomicAdd(&facc[js].z, -dz * f);
                    }
                    if(kEnergy) {
                        const double w = (kHalf && interior) ? 1.0 : 0.5;
                        pe += w * 4.0 * (double) a.lj.eps[tij] * ((double) sr6 * (double) sr6 - (double) sr6);
                        vir += w * (double) (rsq * f);
                    }
                }
            }
        }
        if(kHalf) {
            const int own = center.base + (i - center.start);
            atomicAdd(&facc[own].x, fx); atomicAdd(&facc[own].y, fy); atomicAdd(&facc[own].z, fz);
        } else {
            st_f4(a.p.force32, i, make_float4(fx, fy, fz, 0.0f));
        }
    }
    if(kHalf) {
        __syncthreads();
        for(int s = 0; s < nsegs; s++) {
            const Seg g = segs[s];
            if(g.code != 0) { continue; }
            for(int k = threadIdx.x; k < g.count; k += blockDim.x) {
                const float4 f = facc[g.base + k];
                if(f.x != 0.f || f.y != 0.f || f.z != 0.f) {
                    red_add_v4_global(a.p.force32 + 4 * (size_t) (g.start + k), f.x, f.y, f.z);
                }
            }
        }
    }
    if(kEnergy) {
        pe = warp_sum(pe); vir = warp_sum(vir);
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        if(lane == 0) { red[0][w] = pe; red[1][w] = vir; }
        __syncthreads();
        if(threadIdx.x == 0) {
            double x = 0.0, y = 0.0;
            for(int k = 0; k < (int) (blockDim.x >> 5); k++) { x += red[0][k]; y += red[1][k]; }
            atomicAdd(&a.energy[0], x);
            atomicAdd(&a.energy[1], y);
        }
    }
}

// ------------------------------------------------------------------ host side

static bool tile_geometry(const pg_cells *cells, const pg_neighbor_list *list, int &tz, int &ntz, int &ntiles) {
    tz = list->tile_z;
    if(tz <= 0) { return false; }
    ntz = (cells->dims[2] + tz - 1) / tz;
    ntiles = cells->dims[0] * cells->dims[1] * ntz;
    return true;
}

static size_t tile_smem(int capacity, bool half) {
    return (size_t) capacity * (half ? 48 : 32);
}

int tile_build(const pg_box *box, const pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
               double r_list2, pg_status *status, cudaStream_t st) {
    if(!box || !p || !cells || !list || !status || !list->nbr16 || !list->count) { return PG_ERR_ARGUMENT; }
    if(!p->pos || !p->pos_hi || !p->pos_lo || !p->pos_ref || !p->ref_hi || !p->ref_lo) { return PG_ERR_ARGUMENT; }
    if(list->stride < p->n || list->tile_capacity <= 0 || list->tile_capacity > 65535) { return PG_ERR_ARGUMENT; }
    for(int d = 0; d < 3; d++) {
        if(cells->cell_len[d] * cells->cell_len[d] < r_list2) { return PG_ERR_ARGUMENT; }
        if(box->periodic[d] && box->len[d] * box->len[d] <= r_list2) { return PG_ERR_ARGUMENT; }
    }
    TileArgs a;
    int ntiles;
    if(!tile_geometry(cells, list, a.tz, a.ntz, ntiles)) { return PG_ERR_ARGUMENT; }
    a.box = *box; a.p = *p; a.cells = *cells; a.list = *list; a.capacity = list->tile_capacity;
    a.r_list2 = r_list2;
    a.r2_lo = (float) r_list2 * (1.0f - kTileBand);
    a.r2_hi = (float) r_list2 * (1.0f + kTileBand);
    a.energy = nullptr; a.status = status;
    list->steps_since_build = 0;
    const size_t smem = tile_smem(a.capacity, false);
    if(cudaFuncSetAttribute(k_tile_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem) != cudaSuccess) {
        return PG_ERR_CUDA;
    }
    if(ntiles > 0) { k_tile_build<<<ntiles, kTileThreads, smem, st>>>(a); note_launch(); }
    return launch_status();
}

using TileKernel = void (*)(TileArgs);

template<bool H, bool O, bool E>
static int launch_tile_lj(TileArgs &a, int ntiles, size_t smem, cudaStream_t st) {
    if(cudaFuncSetAttribute(k_tile_lj<H, O, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem) != cudaSuccess) {
        return PG_ERR_CUDA;
    }
    k_tile_lj<H, O, E><<<ntiles, kTileThreads, smem, st>>>(a); note_launch();
    return launch_status();
}

int tile_lj_force(const pg_box *box, const pg_particles *p, const pg_neighbor_list *list, const pg_cells *cells,
                  const LJTableF &lj, double *energy, cudaStream_t st) {
    TileArgs a;
    int ntiles;
    if(!tile_geometry(cells, list, a.tz, a.ntz, ntiles)) { return PG_ERR_ARGUMENT; }
    a.box = *box; a.p = *p; a.cells = *cells; a.list = *list; a.capacity = list->tile_capacity;
    a.lj = lj; a.energy = energy; a.status = nullptr;
    const bool half = list->half != 0, one = lj.ntypes == 1, en = energy != nullptr;
    const size_t smem = tile_smem(a.capacity, half);
    if(ntiles == 0) { return PG_OK; }
    if(half) {
        if(one) { return en ? launch_tile_lj<true, true, true>(a, ntiles, smem, st) : launch_tile_lj<true, true, false>(a, ntiles, smem, st); }
        return en ? launch_tile_lj<true, false, true>(a, ntiles, smem, st) : launch_tile_lj<true, false, false>(a, ntiles, smem, st);
    }
    if(one) { return en ? launch_tile_lj<false, true, true>(a, ntiles, smem, st) : launch_tile_lj<false, true, false>(a, ntiles, smem, st); }
    return en ? launch_tile_lj<false, false, true>(a, ntiles, smem, st) : launch_tile_lj<false, false, false>(a, ntiles, smem, st);
}

}  // namespace pg
