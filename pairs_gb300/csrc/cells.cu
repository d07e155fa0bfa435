// Cell binning and counting sort of particles into cell order.
//
// Replaces the reference's build_cell_lists / partition_cell_lists modules
// (sim/cell_lists.py:90-171) and the wrap half of its exchange step
// (sim/comm.py:101-151).  The reference appends particle indices into fixed-size
// per-cell slots (cell_particles[ncells][64]) with one atomic per particle; here the
// particles themselves are permuted into cell order (counting sort: count, scan,
// scatter, per-cell order by z then uid, gather), so every later kernel streams
// contiguous, spatially sorted memory and the cell list is just (start, count).
#include <string.h>

#include "common.cuh"

namespace pg {

// Wrap into the periodic box exactly as the reference's exchange pack does
// (x + mult*len with mult = +1 below lo, -1 above hi), then compute the cell.
// inv_len: 1 / cell_len per axis (host FP64); the cell of a coordinate is
// floor((x - lo) * inv_len), clamped.  Between rebuilds particles stay mostly in cell
// order, so a warp's particles fall into a few cells: one atomic per distinct cell.
//
// The FP64 pipe bounds this pass, so the comparisons with the box faces and the finite
// test are made on the numbers' bit patterns (an integer key that orders like the
// number for every finite value), and floor + conversion is one round-down conversion:
// 18 -> 9 FP64 operations per particle, the same cells.
struct InvLen {
    double v[3];
    long long lo_key[3], hi_key[3];          // order keys of box.lo, box.hi
};

__host__ __device__ __forceinline__ long long order_key(double x) {
    long long b;
    memcpy(&b, &x, sizeof(b));
    if(b == (long long) 0x8000000000000000ULL) { b = 0; }          // -0 compares equal to +0
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

__device__ __forceinline__ bool finite_bits(double x) {
    return (__double_as_longlong(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}

__global__ void k_bin_count(pg_box box, pg_particles p, pg_cells cells, InvLen inv, int32_t *count,
                            pg_status *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= p.n) { return; }
    D4 x = ld_d4_plain(p.pos, i);
    double c3[3] = {x.x, x.y, x.z};
    bool moved = false;
    bool finite = true;
    const bool infinite = p.flags != nullptr && (p.flags[i] & kFlagInfinite);   // half spaces stay put
    for(int d = 0; d < 3; d++) {
        if(!finite_bits(c3[d])) { finite = false; continue; }
        if(box.periodic[d] && !infinite) {
            const long long k = order_key(c3[d]);
            if(k < inv.lo_key[d]) { c3[d] = __dadd_rn(c3[d], box.len[d]); moved = true; }
            else if(k > inv.hi_key[d]) { c3[d] = __dadd_rn(c3[d], -box.len[d]); moved = true; }
        }
    }
    if(moved) {
        x.x = c3[0]; x.y = c3[1]; x.z = c3[2];
        st_d4(p.pos, i, x);
    }
    int cell;
    if(!finite) {
        atomicExch(&status->nonfinite, 1);
        cell = cells.ncells;                       // parked in the extra bucket
    } else if(infinite) {
        cell = cells.ncells;                       // infinite shapes (half spaces) last
    } else {
        int idx = 0;
        for(int d = 0; d < 3; d++) {
            int c = __double2int_rd(__dmul_rn(__dsub_rn(c3[d], box.lo[d]), inv.v[d]));   // floor, saturating
            c = c < 0 ? 0 : (c >= cells.dims[d] ? cells.dims[d] - 1 : c);
            idx = idx * cells.dims[d] + c;
        }
        cell = idx;
    }
    cells.particle_cell[i] = cell;
    const unsigned peers = __match_any_sync(__activemask(), cell);
    if((threadIdx.x & 31) == (unsigned) (__ffs(peers) - 1)) { atomicAdd(&count[cell], __popc(peers)); }
}

// Exclusive scan, three passes over blocks of 1024 entries.
constexpr int kScanBlock = 1024;

__device__ __forceinline__ int block_exclusive_scan(int v, int *smem_warp, int &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
    for(int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if(lane >= o) { incl += t; }
    }
    if(lane == 31) { smem_warp[warp] = incl; }
    __syncthreads();
    if(warp == 0) {
        const int nw = blockDim.x >> 5;
        int w = lane < nw ? smem_warp[lane] : 0;
        int wi = w;
        for(int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, wi, o);
            if(lane >= o) { wi += t; }
        }
        if(lane < nw) { smem_warp[lane] = wi - w; }
        if(lane == nw - 1) { smem_warp[32] = wi; }
    }
    __syncthreads();
    total = smem_warp[32];
    const int res = incl - v + smem_warp[warp];
    __syncthreads();
    return res;
}

__global__ void k_scan_block_sums(const int32_t *in, int n, int32_t *block_sums) {
    __shared__ int s[33];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    int total;
    block_exclusive_scan(v, s, total);
    if(threadIdx.x == 0) { block_sums[blockIdx.x] = total; }
}

__global__ void k_scan_sums(int32_t *block_sums, int nb) {
    __shared__ int s[33];
    int carry = 0;
    for(int base = 0; base < nb; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? block_sums[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, s, total);
        if(i < nb) { block_sums[i] = ex + carry; }
        carry += total;
        __syncthreads();
    }
}

// out[i] = exclusive prefix of in; out[n] = total.  also zeroes cursor[i].
__global__ void k_scan_apply(const int32_t *in, int n, const int32_t *block_sums, int32_t *out,
                             int32_t *cursor) {
    __shared__ int s[33];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    int total;
    const int ex = block_exclusive_scan(v, s, total) + block_sums[blockIdx.x];
    if(i < n) {
        out[i] = ex;
        if(cursor != nullptr) { cursor[i] = 0; }
        if(i == n - 1) { out[n] = ex + v; }
    }
}

// Exclusive scan of n int32 values into out[0 .. n] (out[n] = the total) with the three
// kernels above; block_sums holds scan_block_sums_len(n) values.
int64_t scan_block_sums_len(int n) { return n < 0 ? 0 : ((int64_t) n + kScanBlock - 1) / kScanBlock + 1; }

int scan_exclusive_i32(const int32_t *in, int n, int32_t *out, int32_t *block_sums, cudaStream_t st) {
    if(n <= 0) {
        if(n == 0) { cudaMemsetAsync(out, 0, sizeof(int32_t), st); }
        return n == 0 ? launch_status() : PG_ERR_ARGUMENT;
    }
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    k_scan_block_sums<<<nb, kScanBlock, 0, st>>>(in, n, block_sums); note_launch();
    k_scan_sums<<<1, kScanBlock, 0, st>>>(block_sums, nb); note_launch();
    k_scan_apply<<<nb, kScanBlock, 0, st>>>(in, n, block_sums, out, nullptr); note_launch();
    return launch_status();
}

__global__ void k_scatter(int n, const int32_t *particle_cell, const int32_t *start,
                          int32_t *cursor, int32_t *perm, RepMask mask) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n || mask.skip(i)) { return; }
    const int c = particle_cell[i];
    perm[start[c] + atomicAdd(&cursor[c], 1)] = i;
}

// Order each cell's particles by z, then uid, then index before binning, so the
// result does not depend on the atomic order of the scatter.  The cells of a z column
// are consecutive, so a column's particles are then sorted by z as a whole: the list
// builds take the candidates of a column within a z window.
//
// One thread per particle counts the members of its cell that precede it (a cell holds
// ~10-20 particles) and writes it to that rank; the scatter's unordered cell ranges are
// read from `unordered`.  z enters as a 64-bit integer key that orders like the number
// (-0 taken as +0; NaN, parked in the trailing bucket, above every number), so the
// order is total and the ranks of a cell are distinct.  Every cell is ordered, with or
// without uids (the z windows of the list builds rely on it).  Measured at 1M atoms:
// 37 us against 42 us for an insertion sort per cell over the same data.
__device__ __forceinline__ long long z_order_key(double z) {
    const long long b = __double_as_longlong(__dadd_rn(z, 0.0));
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

__global__ void k_rank_cells(int n, const int32_t *unordered, const int32_t *particle_cell, const int32_t *start,
                             const int32_t *uid, const double *pos, int32_t *perm, pg_status *status,
                             RepMask mask) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if(s >= n) { return; }
    if(mask.skip(s)) { perm[s] = s; return; }     // a replica left alone keeps its order
    const int v = unordered[s];
    const int c = particle_cell[v];
    const int b = start[c], e = start[c + 1];
    const long long kz = z_order_key(pos[4 * (size_t) v + 2]);
    const int ku = uid != nullptr ? uid[v] : 0;
    int rank = 0;
    int m = b;
    for(; m + 4 <= e; m += 4) {                 // four members' loads in flight
        int w[4];
        double z[4];
        int u[4];
#pragma unroll
        for(int q = 0; q < 4; q++) { w[q] = unordered[m + q]; }
#pragma unroll
        for(int q = 0; q < 4; q++) { z[q] = pos[4 * (size_t) w[q] + 2]; u[q] = uid != nullptr ? uid[w[q]] : 0; }
#pragma unroll
        for(int q = 0; q < 4; q++) {
            const long long wz = z_order_key(z[q]);
            rank += (wz < kz || (wz == kz && (u[q] < ku || (u[q] == ku && w[q] < v)))) ? 1 : 0;
        }
    }
    for(; m < e; m++) {
        const int w = unordered[m];
        const long long wz = z_order_key(pos[4 * (size_t) w + 2]);
        const int wu = uid != nullptr ? uid[w] : 0;
        rank += (wz < kz || (wz == kz && (wu < ku || (wu == ku && w < v)))) ? 1 : 0;
    }
    perm[b + rank] = v;
    const int cnt = e - b;
    const unsigned act = __activemask();
    const int wm = __reduce_max_sync(act, cnt);
    if((threadIdx.x & 31) == (unsigned) (__ffs(act) - 1)) { atomicMax(&status->max_cell_count, wm); }
}

// new[k] = old[perm[k]] for element sizes 4, 8, 16, 32 bytes
template<typename T>
__global__ void k_gather(int n, const int32_t *perm, const T *src, T *dst) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k < n) { dst[k] = src[perm[k]]; }
}

struct alignas(32) Blob32 { D4 v; };

int gather_array(int n, const int32_t *perm, const void *src, void *dst, int elem_bytes,
                 cudaStream_t st) {
    const int nb = blocks_for(n);
    switch(elem_bytes) {
        case 4: k_gather<<<nb, kBlock, 0, st>>>(n, perm, (const int32_t *) src, (int32_t *) dst); note_launch(); break;
        case 8: k_gather<<<nb, kBlock, 0, st>>>(n, perm, (const int2 *) src, (int2 *) dst); note_launch(); break;
        case 16: k_gather<<<nb, kBlock, 0, st>>>(n, perm, (const int4 *) src, (int4 *) dst); note_launch(); break;
        case 32: k_gather<<<nb, kBlock, 0, st>>>(n, perm, (const Blob32 *) src, (Blob32 *) dst); note_launch(); break;
        default: return PG_ERR_ARGUMENT;
    }
    return launch_status();
}

__global__ void k_split_positions(pg_box box, pg_particles p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= p.n) { return; }
    const D4 x = ld_d4_plain(p.pos, i);
    const int type = p.type != nullptr ? p.type[i] : 0;
    if(p.pos_hi != nullptr) {
        const double q = box.quantum, iq = 1.0 / q;
        float4 h, l;
        split_pos(x.x, iq, q, h.x, l.x);
        split_pos(x.y, iq, q, h.y, l.y);
        split_pos(x.z, iq, q, h.z, l.z);
        h.w = __int_as_float(type);
        l.w = 0.0f;
        st_f4(p.pos_hi, hl(p, i), h);
        st_f4(p.pos_lo, hl(p, i), l);
    }
    if(p.pos_fx != nullptr) { st_i4(p.pos_fx, i, fx_position(box, x.x, x.y, x.z, type)); }
}

// The permutation applied to every per-particle array in two passes: gather into the
// staging area (new[k] = old[perm[k]], all arrays in one pass over perm), then copy
// back, refreshing the FP32 position layouts (pos_fx, pos_hi/pos_lo) from the new
// positions on the way when a box is given.  Absent arrays (null) are skipped.
struct StageView {
    D4 *pos, *vel;
    double *mass;
    int32_t *type, *uid, *flags, *cell;
};

__host__ __device__ inline StageView stage_view(char *stage, int n) {
    StageView v;
    v.pos = reinterpret_cast<D4 *>(stage);
    v.vel = v.pos + n;
    v.mass = reinterpret_cast<double *>(v.vel + n);
    v.type = reinterpret_cast<int32_t *>(v.mass + n);
    v.uid = v.type + n;
    v.flags = v.uid + n;
    v.cell = v.flags + n;
    return v;
}

__global__ void k_gather_all(int n, const int32_t *perm, pg_particles p, const int32_t *cell, StageView v,
                             RepMask mask) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n || mask.skip(k)) { return; }
    const int s = perm[k];
    v.pos[k] = ld_d4_plain(p.pos, s);
    if(p.vel != nullptr) { v.vel[k] = ld_d4_plain(p.vel, s); }
    if(p.mass != nullptr) { v.mass[k] = p.mass[s]; }
    if(p.type != nullptr) { v.type[k] = p.type[s]; }
    if(p.uid != nullptr) { v.uid[k] = p.uid[s]; }
    if(p.flags != nullptr) { v.flags[k] = p.flags[s]; }
    v.cell[k] = cell[s];
}

// With replicas (a batched ensemble), each particle's layouts are on its replica's grid.
__global__ void k_copy_back_all(int n, pg_particles p, int32_t *cell, StageView v, pg_box box, int split,
                                RepMask mask, const pg_replica *replicas) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n || mask.skip(k)) { return; }
    const D4 x = v.pos[k];
    st_d4(p.pos, k, x);
    if(p.vel != nullptr) { st_d4(p.vel, k, v.vel[k]); }
    if(p.mass != nullptr) { p.mass[k] = v.mass[k]; }
    int type = 0;
    if(p.type != nullptr) { type = v.type[k]; p.type[k] = type; }
    if(p.uid != nullptr) { p.uid[k] = v.uid[k]; }
    if(p.flags != nullptr) { p.flags[k] = v.flags[k]; }
    cell[k] = v.cell[k];
    if(split) {
        const pg_replica *R = replicas != nullptr ? &replicas[mask.replica_of[k]] : nullptr;
        if(p.pos_hi != nullptr) {
            const double q = R != nullptr ? R->quantum : box.quantum, iq = 1.0 / q;
            float4 h, l;
            split_pos(x.x, iq, q, h.x, l.x);
            split_pos(x.y, iq, q, h.y, l.y);
            split_pos(x.z, iq, q, h.z, l.z);
            h.w = __int_as_float(type);
            l.w = 0.0f;
            st_f4(p.pos_hi, hl(p, k), h);
            st_f4(p.pos_lo, hl(p, k), l);
        }
        if(p.pos_fx != nullptr) {
            st_i4(p.pos_fx, k, R != nullptr ? replica_fx(*R, x.x, x.y, x.z, type) : fx_position(box, x.x, x.y, x.z, type));
        }
    }
}

// workspace layout for pg_bin_particles (all offsets 256-byte aligned)
constexpr size_t kStageBytes = 32 + 32 + 8 + 4 + 4 + 4 + 4;   // pos, vel, mass, type, uid, flags, cell

struct BinWs {
    int32_t *count, *start, *cursor, *block_sums, *perm;
    char *stage;                      // staging of every gathered array (kStageBytes per particle)
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t) 255; }

static size_t bin_ws_layout(int32_t n, int32_t ncells, char *base, BinWs *w) {
    const size_t nc = (size_t) ncells + 2;
    const size_t nb = (nc + kScanBlock - 1) / kScanBlock + 1;
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = base ? base + off : nullptr; off += align256(bytes); return p; };
    BinWs tmp;
    tmp.count = (int32_t *) take(nc * 4);
    tmp.start = (int32_t *) take((nc + 1) * 4);
    tmp.cursor = (int32_t *) take(nc * 4);
    tmp.block_sums = (int32_t *) take(nb * 4);
    tmp.perm = (int32_t *) take((size_t) n * 4);
    tmp.stage = take((size_t) n * kStageBytes);
    if(w) { *w = tmp; }
    return off;
}

int64_t bin_workspace_bytes(int32_t n, int32_t ncells) {
    return (int64_t) bin_ws_layout(n, ncells, nullptr, nullptr);
}

const int32_t *bin_permutation(int32_t n, int32_t ncells, pg_workspace ws) {
    if(ws.ptr == nullptr || n < 0 || ncells < 0 || ws.bytes < bin_workspace_bytes(n, ncells)) { return nullptr; }
    BinWs w;
    bin_ws_layout(n, ncells, (char *) ws.ptr, &w);
    return w.perm;
}

// Zero the cell counters of the workspace (the count pass adds into them).
int bin_prepare(int32_t n, int32_t ncells, pg_workspace ws, int32_t **count, cudaStream_t st) {
    if(ws.ptr == nullptr || ws.bytes < bin_workspace_bytes(n, ncells)) { return PG_ERR_ARGUMENT; }
    BinWs w;
    bin_ws_layout(n, ncells, (char *) ws.ptr, &w);
    cudaMemsetAsync(w.count, 0, (size_t) (ncells + 1) * 4, st);
    *count = w.count;
    return PG_OK;
}

// Everything after the count pass: exclusive scan of the counts (ncells cells plus
// the trailing bucket), scatter, per-cell order by z then uid, the permutation of every
// per-particle array of p and of cells->particle_cell, and the cell bookkeeping.
// With a box, the FP32 position layouts of p are refreshed from the new positions.
// With a replica mask, the particles of the replicas left alone keep their places (their
// cells' counts must be in the count array already, so their starts come out unchanged).
// With split_replicas (a batched ensemble; mask.replica_of set), the layouts are refreshed
// on each particle's replica grid.
int bin_finish(int32_t n, int32_t ncells, pg_workspace ws, pg_particles *p, pg_cells *cells, pg_status *status,
               cudaStream_t st, int32_t **perm_out, const pg_box *split_box, RepMask mask,
               const pg_replica *split_replicas) {
    BinWs w;
    bin_ws_layout(n, ncells, (char *) ws.ptr, &w);
    if(perm_out) { *perm_out = w.perm; }
    const int ntot = ncells + 1;
    const int nb = (ntot + kScanBlock - 1) / kScanBlock;
    k_scan_block_sums<<<nb, kScanBlock, 0, st>>>(w.count, ntot, w.block_sums); note_launch();
    k_scan_sums<<<1, kScanBlock, 0, st>>>(w.block_sums, nb); note_launch();
    k_scan_apply<<<nb, kScanBlock, 0, st>>>(w.count, ntot, w.block_sums, w.start, w.cursor); note_launch();
    if(n == 0) { return launch_status(); }
    // the scatter's unordered cell ranges go to the staging area's cell column (the
    // gather fills it later), the ranked order to perm
    const StageView v = stage_view(w.stage, n);
    k_scatter<<<blocks_for(n), kBlock, 0, st>>>(n, cells->particle_cell, w.start, w.cursor, v.cell, mask);
    note_launch();
    k_rank_cells<<<blocks_for(n), kBlock, 0, st>>>(n, v.cell, cells->particle_cell, w.start, p->uid, p->pos, w.perm,
                                                   status, mask);
    note_launch();
    k_gather_all<<<blocks_for(n), kBlock, 0, st>>>(n, w.perm, *p, cells->particle_cell, v, mask); note_launch();
    pg_box box = {};
    if(split_box != nullptr) { box = *split_box; }
    const int split = split_box != nullptr || split_replicas != nullptr ? 1 : 0;
    k_copy_back_all<<<blocks_for(n), kBlock, 0, st>>>(n, *p, cells->particle_cell, v, box, split, mask, split_replicas);
    note_launch();
    // cell bookkeeping for the sorted order
    cudaMemcpyAsync(cells->cell_start, w.start, (size_t) (ntot + 1) * 4, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(cells->cell_count, w.count, (size_t) ntot * 4, cudaMemcpyDeviceToDevice, st);
    return launch_status();
}

// A cell grid the kernels can index: at least one cell of positive, finite length
// along every axis, and ncells the product of the dimensions (the binning clamps a
// coordinate into [0, dims - 1], which is a valid cell only for dims >= 1).
bool grid_ok(const pg_cells *cells) {
    if(cells == nullptr) { return false; }
    int64_t prod = 1;
    for(int d = 0; d < 3; d++) {
        if(cells->dims[d] < 1 || !(cells->cell_len[d] > 0.0) || !isfinite(cells->cell_len[d])) { return false; }
        prod *= cells->dims[d];
        if(prod > INT32_MAX - 4) { return false; }
    }
    return prod == cells->ncells;
}

int bin_particles(const pg_box *box, pg_particles *p, pg_cells *cells, pg_workspace ws,
                  pg_status *status, cudaStream_t st, int32_t **perm_out) {
    if(box == nullptr || p == nullptr || cells == nullptr || status == nullptr) { return PG_ERR_ARGUMENT; }
    if(p->n < 0 || p->n > p->capacity || p->pos == nullptr) { return PG_ERR_ARGUMENT; }
    if(!grid_ok(cells)) { return PG_ERR_ARGUMENT; }
    const int n = p->n;
    int32_t *count = nullptr;
    int rc = bin_prepare(n, cells->ncells, ws, &count, st);
    if(rc) { return rc; }
    if(n > 0) {
        InvLen inv;
        for(int d = 0; d < 3; d++) {
            inv.v[d] = 1.0 / cells->cell_len[d];
            inv.lo_key[d] = order_key(box->lo[d]);
            inv.hi_key[d] = order_key(box->hi[d]);
        }
        k_bin_count<<<blocks_for(n), kBlock, 0, st>>>(*box, *p, *cells, inv, count, status); note_launch();
    }
    const bool split = (p->pos_hi != nullptr && p->pos_lo != nullptr) || p->pos_fx != nullptr;
    return bin_finish(n, cells->ncells, ws, p, cells, status, st, perm_out, split ? box : nullptr, RepMask{}, nullptr);
}

int split_positions(const pg_box *box, pg_particles *p, cudaStream_t st) {
    if(box == nullptr || p == nullptr || (p->pos_hi == nullptr) != (p->pos_lo == nullptr) ||
       (p->pos_hi == nullptr && p->pos_fx == nullptr)) { return PG_ERR_ARGUMENT; }
    if(p->n > 0) { k_split_positions<<<blocks_for(p->n), kBlock, 0, st>>>(*box, *p); note_launch(); }
    return launch_status();
}

}  // namespace pg
