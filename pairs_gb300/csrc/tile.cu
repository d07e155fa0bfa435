// Tile-local Verlet lists and forces (mixed precision): shared-memory neighbourhoods.
//
// Particles are sorted by cell, z fastest, so a column of cells (x, y fixed) is one
// contiguous range of particles.  A tile is TZ consecutive cells of one column; its
// neighbourhood -- the 3x3 columns around it, cells z0-1 .. z1 -- is at most 27
// contiguous particle ranges ("segments": per column the main range plus the cells
// that wrap around a periodic z boundary), laid out back to back in shared memory,
// unshifted segments first.  Staging applies each segment's periodic image shift
// (hi + s*len_hi is exact on the hi grid).
//
// The Verlet list of a tile particle holds 16-bit shared-memory slot indices: half
// the list bytes of global indices, and every partner read is a shared-memory load
// instead of an L1/L2 gather.  The layout depends only on the cell occupancy, which
// is fixed between rebuilds, so the build computes it once per tile (one thread per
// tile, k_tile_layouts) into tile_table; the list build and every force pass load
// their tile's record cooperatively.
//
// Acceptance is the reference's exact FP64 test (see nlist.cu): FP32 screen, FP64
// decision inside a 1e-4 relative band.  Tile lists are full lists (each pair from
// both sides): no reactions, no atomics, 32 bytes of shared memory per staged
// particle, so two or more tile blocks share an SM.
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

// One tile's layout as stored in tile_table (PG_TILE_RECORD_WORDS int32 words).
struct alignas(16) TileRec {
    Seg segs[kMaxSegs];          // 108 words
    Col cols[9];                 // 54 words
    int nsegs, staged, ib, ie, z0, cx, cy;        // 7 words
    int pad[11];
};
static_assert(sizeof(TileRec) == PG_TILE_RECORD_WORDS * 4, "tile record size");

struct TileArgs {
    pg_box box;
    pg_particles p;
    pg_cells cells;
    pg_neighbor_list list;
    int tz, ntz, ntiles;         // cells per tile along z, tiles per column, tiles
    int capacity;
    double r_list2;
    float r2_lo, r2_hi;
    LJTableF lj;
    double *energy;
    pg_status *status;
};

// Enumerate the neighbourhood of tile t (unshifted segments first).
__device__ void tile_layout(const TileArgs &a, int t, TileRec &r) {
    const int dx = a.cells.dims[0], dy = a.cells.dims[1], dz = a.cells.dims[2];
    const int zt = t % a.ntz, col = t / a.ntz;
    const int cy = col % dy, cx = col / dy;
    const int z0 = zt * a.tz, z1 = min(z0 + a.tz, dz);
    const int c_first = (cx * dy + cy) * dz;
    r.ib = a.cells.cell_start[c_first + z0];
    r.ie = a.cells.cell_start[c_first + z1 - 1] + a.cells.cell_count[c_first + z1 - 1];
    r.z0 = z0; r.cx = cx; r.cy = cy;
    for(int k = 0; k < 11; k++) { r.pad[k] = 0; }
    int n = 0;
    for(int k = 0; k < 9; k++) {
        r.cols[k].cell0 = 0; r.cols[k].za = 0; r.cols[k].zb = -1;
        r.cols[k].main_seg = r.cols[k].low_seg = r.cols[k].high_seg = -1;
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
                Col &cl = r.cols[k];
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
                    Seg &s = r.segs[n];
                    s.start = a.cells.cell_start[cell0 + za];
                    s.count = a.cells.cell_start[cell0 + zb] + a.cells.cell_count[cell0 + zb] - s.start;
                    s.code = (int) code;
                    if(part == 0) { cl.main_seg = n; } else if(part == 1) { cl.low_seg = n; } else { cl.high_seg = n; }
                    n++;
                }
            }
        }
    }
    int base = 0;
    for(int s = 0; s < n; s++) {
        r.segs[s].base = base;
        base += r.segs[s].count;
    }
    for(int s = n; s < kMaxSegs; s++) { r.segs[s].start = r.segs[s].count = r.segs[s].base = r.segs[s].code = 0; }
    r.nsegs = n;
    r.staged = base;
}

__global__ void __launch_bounds__(128) k_tile_layouts(TileArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int staged = 0;
    if(t < a.ntiles) {
        TileRec r;
        tile_layout(a, t, r);
        const int *src = reinterpret_cast<const int *>(&r);
        int *dst = a.list.tile_table + (size_t) t * PG_TILE_RECORD_WORDS;
        for(int w = 0; w < PG_TILE_RECORD_WORDS; w++) { dst[w] = src[w]; }
        staged = r.staged;
    }
    const int wm = warp_max(staged);
    if((threadIdx.x & 31) == 0 && wm > 0) {
        atomicMax(&a.status->max_tile_staged, wm);
        if(wm > a.capacity) { atomicOr(&a.status->overflow, 4); }
    }
}

// The block's tile record into shared memory.
__device__ __forceinline__ void load_tile(const TileArgs &a, int t, TileRec &r) {
    const int4 *src = reinterpret_cast<const int4 *>(a.list.tile_table + (size_t) t * PG_TILE_RECORD_WORDS);
    int4 *dst = reinterpret_cast<int4 *>(&r);
    for(int w = threadIdx.x; w < PG_TILE_RECORD_WORDS / 4; w += blockDim.x) { dst[w] = src[w]; }
}

// Stage hi/lo of every segment into shared memory (sm[2k] = hi, sm[2k+1] = lo).
__device__ void tile_stage(const TileArgs &a, const TileRec &r, float4 *sm) {
    for(int s = 0; s < r.nsegs; s++) {
        const Seg g = r.segs[s];
        const int sx = image_shift(g.code, 0), sy = image_shift(g.code, 1), sz = image_shift(g.code, 2);
        const float hx = sx * a.box.len_hi[0], hy = sy * a.box.len_hi[1], hz = sz * a.box.len_hi[2];
        const float lx = sx * a.box.len_lo[0], ly = sy * a.box.len_lo[1], lz = sz * a.box.len_lo[2];
        for(int k = threadIdx.x; k < g.count; k += blockDim.x) {
            float4 h = ld_f4(a.p.pos_hi, hl(a.p, g.start + k));
            float4 l = ld_f4(a.p.pos_lo, hl(a.p, g.start + k));
            h.x += hx; h.y += hy; h.z += hz;
            l.x += lx; l.y += ly; l.z += lz;
            sm[2 * (g.base + k)] = h;
            sm[2 * (g.base + k) + 1] = l;
        }
    }
}

// ------------------------------------------------------------------ list build

__global__ void __launch_bounds__(kTileThreads) k_tile_build(TileArgs a) {
    __shared__ TileRec r;
    const int t = blockIdx.x;
    load_tile(a, t, r);
    __syncthreads();
    if(r.staged > a.capacity || r.staged > 65535) { return; }
    const int dz = a.cells.dims[2];
    const int stride = a.list.stride, cap = a.list.max_neighbors;
    int wmax = 0;
    for(int i = r.ib + threadIdx.x; i < r.ie; i += blockDim.x) {
        const float4 hi = ld_f4(a.p.pos_hi, hl(a.p, i)), lo = ld_f4(a.p.pos_lo, hl(a.p, i));
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
                const Col cl = r.cols[c];
                if(cl.main_seg < 0 && cl.low_seg < 0 && cl.high_seg < 0) { continue; }
                for(int oz = -1; oz <= 1; oz++) {
                    const int zc = z + oz;
                    int seg, b, e;
                    if(zc >= 0 && zc < dz && cl.main_seg >= 0 && zc >= cl.za && zc <= cl.zb) {
                        seg = cl.main_seg;
                        const Seg g = r.segs[seg];
                        const int cg = cl.cell0 + zc;
                        b = g.base + (a.cells.cell_start[cg] - g.start);
                        e = b + a.cells.cell_count[cg];
                    } else if(zc < 0 && cl.low_seg >= 0) {
                        seg = cl.low_seg; b = r.segs[seg].base; e = b + r.segs[seg].count;
                    } else if(zc >= dz && cl.high_seg >= 0) {
                        seg = cl.high_seg; b = r.segs[seg].base; e = b + r.segs[seg].count;
                    } else {
                        continue;
                    }
                    const Seg g = r.segs[seg];
                    const int sx = image_shift(g.code, 0), sy = image_shift(g.code, 1), sz = image_shift(g.code, 2);
                    const float shx = sx * a.box.len_hi[0], shy = sy * a.box.len_hi[1], shz = sz * a.box.len_hi[2];
                    const float slx = sx * a.box.len_lo[0], sly = sy * a.box.len_lo[1], slz = sz * a.box.len_lo[2];
                    for(int js = b; js < e; js++) {
                        const int j = g.start + (js - g.base);
                        if(j == i && g.code == 0) { continue; }
                        float4 hj = ld_f4(a.p.pos_hi, hl(a.p, j)), lj = ld_f4(a.p.pos_lo, hl(a.p, j));
                        hj.x += shx; hj.y += shy; hj.z += shz;
                        lj.x += slx; lj.y += sly; lj.z += slz;
                        const float fx = (hi.x - hj.x) + (lo.x - lj.x);
                        const float fy = (hi.y - hj.y) + (lo.y - lj.y);
                        const float fz = (hi.z - hj.z) + (lo.z - lj.z);
                        const float r2f = fx * fx + fy * fy + fz * fz;
                        bool keep;
                        if(r2f < a.r2_lo) { keep = true; }
                        else if(r2f > a.r2_hi) { keep = false; }
                        else {
                            const D4 xj = ld_d4(a.p.pos, j);
                            const double ddx = __dsub_rn(xi.x, ref_image(xj.x, sx, a.box.len[0]));
                            const double ddy = __dsub_rn(xi.y, ref_image(xj.y, sy, a.box.len[1]));
                            const double ddz = __dsub_rn(xi.z, ref_image(xj.z, sz, a.box.len[2]));
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

// TPA threads per particle: thread t of a particle takes list entries t, t+TPA, ...
// (consecutive rows of the column-major list, so a warp still reads whole rows)
// and the partial forces are combined with shuffles.
template<int TPA, bool kOneType, bool kEnergy>
__global__ void __launch_bounds__(kTileThreads) k_tile_lj(TileArgs a) {
    if(frozen_force(a.p)) { return; }
    extern __shared__ float4 sm[];
    __shared__ TileRec r;
    __shared__ double red[2][kTileThreads / 32];
    const int t = blockIdx.x;
    load_tile(a, t, r);
    __syncthreads();
    if(r.staged > a.capacity) { return; }      // cannot happen after a successful build
    tile_stage(a, r, sm);
    __syncthreads();
    const int stride = a.list.stride;
    const float c2 = a.lj.cutoff2;
    double pe = 0.0, vir = 0.0;
    const int lane = threadIdx.x % TPA;
    const int per_pass = blockDim.x / TPA;
    const int npass = (r.ie - r.ib + per_pass - 1) / per_pass;
    for(int pass = 0; pass < npass; pass++) {
        const int i = r.ib + pass * per_pass + threadIdx.x / TPA;
        float fx = 0.f, fy = 0.f, fz = 0.f;
        const bool live = i < r.ie && !(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed));
        if(live) {
            const float4 hi = ld_f4(a.p.pos_hi, hl(a.p, i)), lo = ld_f4(a.p.pos_lo, hl(a.p, i));
            const int ti = kOneType ? 0 : __float_as_int(hi.w) * a.lj.ntypes;
            const int cnt = a.list.count[i];
            const uint16_t *nb = a.list.nbr16 + i;
            for(int k = lane; k < cnt; k += TPA) {
                const int js = __ldcs(nb + (size_t) k * stride);
                const float4 hj = sm[2 * js], lj = sm[2 * js + 1];
                const float dx = (hi.x - hj.x) + (lo.x - lj.x);
                const float dy = (hi.y - hj.y) + (lo.y - lj.y);
                const float dz = (hi.z - hj.z) + (lo.z - lj.z);
                const float rsq = dx * dx + dy * dy + dz * dz;
                bool inside = rsq < c2;
                if(fabsf(rsq - c2) < c2 * kCutBand) {
                    // the slot's segment gives the global partner and its image
                    int s = 0;
                    while(s + 1 < r.nsegs && r.segs[s + 1].base <= js) { s++; }
                    const Seg g = r.segs[s];
                    inside = exact_inside(a.p.pos, i, g.start + (js - g.base), (uint32_t) g.code, a.box.len,
                                          a.lj.cutoff2d);
                }
                if(inside) {
                    const int tij = kOneType ? 0 : ti + __float_as_int(hj.w);
                    const float sr2 = rcp_approx(rsq);
                    const float sr6 = sr2 * sr2 * sr2 * a.lj.sig6[tij];
                    const float f = 48.0f * sr6 * (sr6 - 0.5f) * sr2 * a.lj.eps[tij];
                    fx += dx * f; fy += dy * f; fz += dz * f;
                    if(kEnergy) {
                        pe += 0.5 * 4.0 * (double) a.lj.eps[tij] * ((double) sr6 * (double) sr6 - (double) sr6);
                        vir += 0.5 * (double) (rsq * f);
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
        if(lane == 0 && i < r.ie) { st_f4(a.p.force32, i, make_float4(fx, fy, fz, 0.0f)); }
    }
    if(kEnergy) {
        pe = warp_sum(pe); vir = warp_sum(vir);
        const int ln = threadIdx.x & 31, w = threadIdx.x >> 5;
        if(ln == 0) { red[0][w] = pe; red[1][w] = vir; }
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

int tile_build(const pg_box *box, const pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
               double r_list2, pg_status *status, cudaStream_t st) {
    if(!box || !p || !cells || !list || !status || !list->nbr16 || !list->count || !list->tile_table) {
        return PG_ERR_ARGUMENT;
    }
    if(!p->pos || !p->pos_hi || !p->pos_lo || !p->pos_ref || !p->ref_hi || !p->ref_lo) { return PG_ERR_ARGUMENT; }
    if(list->stride < p->n || list->tile_capacity <= 0 || list->half) { return PG_ERR_ARGUMENT; }
    for(int d = 0; d < 3; d++) {
        if(cells->cell_len[d] * cells->cell_len[d] < r_list2) { return PG_ERR_ARGUMENT; }
        if(box->periodic[d] && box->len[d] * box->len[d] <= r_list2) { return PG_ERR_ARGUMENT; }
    }
    TileArgs a;
    if(!tile_geometry(cells, list, a.tz, a.ntz, a.ntiles)) { return PG_ERR_ARGUMENT; }
    a.box = *box; a.p = *p; a.cells = *cells; a.list = *list;
    a.capacity = min(list->tile_capacity, 65535);
    a.r_list2 = r_list2;
    a.r2_lo = (float) r_list2 * (1.0f - kTileBand);
    a.r2_hi = (float) r_list2 * (1.0f + kTileBand);
    a.energy = nullptr; a.status = status;
    list->steps_since_build = 0;
    if(a.ntiles > 0) {
        k_tile_layouts<<<(a.ntiles + 127) / 128, 128, 0, st>>>(a); note_launch();
        k_tile_build<<<a.ntiles, kTileThreads, 0, st>>>(a); note_launch();
    }
    return launch_status();
}

template<int TPA, bool O, bool E>
static int launch_tile_lj(TileArgs &a, size_t smem, cudaStream_t st) {
    if(cudaFuncSetAttribute(k_tile_lj<TPA, O, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem) !=
       cudaSuccess) {
        return PG_ERR_CUDA;
    }
    k_tile_lj<TPA, O, E><<<a.ntiles, kTileThreads, smem, st>>>(a); note_launch();
    return launch_status();
}

template<int TPA>
static int launch_tile_lj_tpa(TileArgs &a, bool one, bool en, size_t smem, cudaStream_t st) {
    if(one) { return en ? launch_tile_lj<TPA, true, true>(a, smem, st) : launch_tile_lj<TPA, true, false>(a, smem, st); }
    return en ? launch_tile_lj<TPA, false, true>(a, smem, st) : launch_tile_lj<TPA, false, false>(a, smem, st);
}

int tile_lj_force(const pg_box *box, const pg_particles *p, const pg_neighbor_list *list, const pg_cells *cells,
                  const LJTableF &lj, double *energy, cudaStream_t st) {
    if(!list->tile_table || list->half || list->tile_capacity <= 0 || list->tile_capacity > 65535) {
        return PG_ERR_ARGUMENT;
    }
    TileArgs a;
    if(!tile_geometry(cells, list, a.tz, a.ntz, a.ntiles)) { return PG_ERR_ARGUMENT; }
    a.box = *box; a.p = *p; a.cells = *cells; a.list = *list; a.capacity = list->tile_capacity;
    a.lj = lj; a.energy = energy; a.status = nullptr;
    const bool one = lj.ntypes == 1, en = energy != nullptr;
    const size_t smem = (size_t) a.capacity * 32;
    if(a.ntiles == 0) { return PG_OK; }
    switch(list->tile_tpa) {
        case 1: return launch_tile_lj_tpa<1>(a, one, en, smem, st);
        case 2: return launch_tile_lj_tpa<2>(a, one, en, smem, st);
        case 4: return launch_tile_lj_tpa<4>(a, one, en, smem, st);
        default: return PG_ERR_ARGUMENT;
    }
}

}  // namespace pg
