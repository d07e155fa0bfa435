// Persistent time steps of the mixed LJ path: the plain steps between two rebuild
// points in one cooperative launch.
//
// The reference launches every module of every time step as its own kernel and
// synchronises the device after each (src/pairs/code_gen/cgen.py:540-576).  Here the
// steps that need no host decision (no rebuild, no thermo) run inside one kernel whose
// blocks stay resident for the whole chunk:
//
//   for each step r:  integrate   fused final + initial half kicks, FP64 drift,
//                                 fixed-point positions, FP64 displacement guard
//                                 (k_integrate_mixed's arithmetic); half lists also
//                                 zero the force the kick has just read
//                     grid barrier
//                     force       the packed pair loop of k_lj_packed
//                     grid barrier
//                     fixup       the cutoff band's pairs decided in FP64
//                                 (k_lj_cutoff_fixup's arithmetic)
//                     grid barrier
//
// The guard keeps its meaning: a trip in the integration of step r stops the chunk
// before the force of step r, as the separate kernels skip themselves
// (pg_particles.guard).  Every block takes the same decision because the guard only
// changes inside an integration phase, which a barrier closes.
//
// Data that other blocks rewrite during the launch (positions, forces, the FP64
// positions of the fixup) is read with ordinary coherent loads, never through the
// read-only path; each barrier is a release (fence before arriving) and an acquire
// (fence after leaving) for every thread.
//
// A barrier never waits without limit: after `limit_ns` of waiting (2 s by default) a
// block sets status->overflow bit 16 and an abort word, and every block leaves the
// kernel at its next barrier.  pg_grid_barrier_check runs the same barrier with an
// arrival count that can never be reached, so that a test can see the limit work.
#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "lj_packed.cuh"
#include "persist.cuh"

namespace pg {

constexpr int kPersistBlock = 128;

struct StepsArgs {
    pg_box box;
    pg_particles p;
    pg_neighbor_list list;
    LJTable lj;
    double dt, kick, half_skin2;             // kick: two half kicks, dt
    float half_skin2_lo, half_skin2_hi;
    int32_t first, nsteps;
    pg_status *status;
    PersistWs ws;
    unsigned long long limit_ns;
};

__device__ __forceinline__ int32_t guard_word(const StepsArgs &a) {
    return *reinterpret_cast<volatile const int32_t *>(&a.status->guard_tripped);
}

// coherent FP64 position (x, y, z) of particle i
__device__ __forceinline__ double3 ld_pos_coherent(const double *pos, int i) {
    const double2 *q = reinterpret_cast<const double2 *>(pos + 4 * (size_t) i);
    const double2 a = __ldcg(q), b = __ldcg(q + 1);
    return make_double3(a.x, a.y, b.x);
}

// One pair of the cutoff band (k_lj_cutoff_fixup's arithmetic): the FP64 test of the
// FP64 path decides; a pair inside adds its FP32 force (and a half list's reaction).
template<bool kHalf, bool kOneType>
__device__ void band_pair(const StepsArgs &a, int i, uint32_t e) {
    const int j = (int) (e & PG_NBR_INDEX_MASK);
    const uint32_t code = e >> PG_NBR_INDEX_BITS;
    const double3 xi = ld_pos_coherent(a.p.pos, i), xj = ld_pos_coherent(a.p.pos, j);
    const double jx = ref_image(xj.x, image_shift(code, 0), a.box.len[0]);
    const double jy = ref_image(xj.y, image_shift(code, 1), a.box.len[1]);
    const double jz = ref_image(xj.z, image_shift(code, 2), a.box.len[2]);
    if(!(ref_rsq(__dsub_rn(xi.x, jx), __dsub_rn(xi.y, jy), __dsub_rn(xi.z, jz)) < a.lj.cutoff2)) { return; }
    const int4 fi = ld_fx<true>(a.p.pos_fx, i), fj = ld_fx<true>(a.p.pos_fx, j);
    const float dx = (float) fx_diff(fi.x, fj.x) * a.box.fx_unit[0];
    const float dy = (float) fx_diff(fi.y, fj.y) * a.box.fx_unit[1];
    const float dz = (float) fx_diff(fi.z, fj.z) * a.box.fx_unit[2];
    const float rsq = pair_rsq(dx, dy, dz);
    const int tij = kOneType ? 0 : fi.w * a.lj.ntypes + fj.w;
    const float sr2 = rcp_approx(rsq);
    const float sr6 = sr2 * sr2 * sr2 * a.lj.sig6f[tij];
    const float f = 48.0f * sr6 * (sr6 - 0.5f) * sr2 * a.lj.epsf[tij];
    red_add_v4(a.p.force32 + 4 * (size_t) i, dx * f, dy * f, dz * f);
    if(kHalf && code == 0u) { red_add_v4(a.p.force32 + 4 * (size_t) j, -dx * f, -dy * f, -dz * f); }
}

template<bool kHalf, bool kOneType>
__global__ void __launch_bounds__(kPersistBlock) k_lj_steps(StepsArgs a) {
    const unsigned nblocks = gridDim.x;
    const int first = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int n = a.p.n;
    const float c2 = a.lj.cutoff2f, band = c2 * kCutBand;
    for(int s = 0; s < a.nsteps; s++) {
        const int32_t r = a.first + s;
        // ---- integrate: a trip before this step froze the state (k_integrate_mixed)
        if(guard_word(a) < r) { break; }
        if(first == 0) { *a.ws.cut_count = 0; }
        for(int base = 0; base < n; base += stride) {
            const int i = base + first;
            bool tripped = false;
            if(i < n && !(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed))) {
                const float4 f = __ldcg(reinterpret_cast<const float4 *>(a.p.force32) + i);
                if(kHalf) { st_f4(a.p.force32, i, make_float4(0.0f, 0.0f, 0.0f, 0.0f)); }
                const double m = a.p.mass[i];
                const double c = m == 1.0 ? a.kick : a.kick / m;
                D4 v = ld_d4_plain(a.p.vel, i);
                v.x = fma(c, (double) f.x, v.x);
                v.y = fma(c, (double) f.y, v.y);
                v.z = fma(c, (double) f.z, v.z);
                st_d4(a.p.vel, i, v);
                D4 x = ld_d4_plain(a.p.pos, i);
                x.x = fma(a.dt, v.x, x.x);
                x.y = fma(a.dt, v.y, x.y);
                x.z = fma(a.dt, v.z, x.z);
                st_d4(a.p.pos, i, x);
                const int type = a.p.type != nullptr ? a.p.type[i] : 0;
                const int4 xf = fx_position(a.box, x.x, x.y, x.z, type);
                st_i4(a.p.pos_fx, i, xf);
                const int4 rf = ld_i4(a.p.ref_fx, i);
                const float dx = (float) fx_diff(xf.x, rf.x) * a.box.fx_unit[0];
                const float dy = (float) fx_diff(xf.y, rf.y) * a.box.fx_unit[1];
                const float dz = (float) fx_diff(xf.z, rf.z) * a.box.fx_unit[2];
                const float d2 = dx * dx + dy * dy + dz * dz;
                if(d2 > a.half_skin2_hi) {
                    tripped = true;
                } else if(d2 > a.half_skin2_lo) {
                    const D4 rr = ld_d4_plain(a.p.pos_ref, i);
                    const double ex = x.x - rr.x, ey = x.y - rr.y, ez = x.z - rr.z;
                    tripped = (ex * ex + ey * ey + ez * ez) > a.half_skin2;
                }
            } else if(i < n && kHalf) {
                st_f4(a.p.force32, i, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
            }
            if(__any_sync(0xffffffffu, tripped) && (threadIdx.x & 31) == 0) {
                atomicMin(&a.status->guard_tripped, r);
            }
        }
        if(!grid_barrier(a.ws, nblocks, a.limit_ns, a.status)) { break; }
        // ---- force: a trip in this step's integration leaves it to the host
        if(guard_word(a) <= r) { break; }
        for(int i = first; i < n; i += stride) {
            float3 f = make_float3(0.0f, 0.0f, 0.0f);
            if(!(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed))) {
                f = packed_pairs<kHalf, kOneType, kHalf ? 4 : 2, true>(
                    i, ld_fx<true>(a.p.pos_fx, i), a.list.nbr + i, a.list.count[i], (size_t) a.list.stride, a.p.pos_fx,
                    a.p.force32, a.box, a.lj, a.ws.cut_count, a.ws.records, a.ws.capacity);
            }
            if(kHalf) { red_add_v4(a.p.force32 + 4 * (size_t) i, f.x, f.y, f.z); }
            else { st_f4(a.p.force32, i, make_float4(f.x, f.y, f.z, 0.0f)); }
        }
        if(!grid_barrier(a.ws, nblocks, a.limit_ns, a.status)) { break; }
        // ---- the cutoff band's pairs: the queue, or every list again when it overflowed
        const int queued = *reinterpret_cast<volatile const int32_t *>(a.ws.cut_count);
        if(queued <= a.ws.capacity) {
            for(int q = first; q < queued; q += stride) {
                const int2 rec = a.ws.records[q];
                band_pair<kHalf, kOneType>(a, rec.x, (uint32_t) rec.y);
            }
        } else {
            for(int i = first; i < n; i += stride) {
                if(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed)) { continue; }
                const int4 fi = ld_fx<true>(a.p.pos_fx, i);
                for(int k = 0; k < a.list.count[i]; k++) {
                    const uint32_t e = (uint32_t) a.list.nbr[(size_t) k * a.list.stride + i];
                    const int4 fj = ld_fx<true>(a.p.pos_fx, (int) (e & PG_NBR_INDEX_MASK));
                    const float dx = (float) fx_diff(fi.x, fj.x) * a.box.fx_unit[0];
                    const float dy = (float) fx_diff(fi.y, fj.y) * a.box.fx_unit[1];
                    const float dz = (float) fx_diff(fi.z, fj.z) * a.box.fx_unit[2];
                    if(fabsf(pair_rsq(dx, dy, dz) - c2) < band) { band_pair<kHalf, kOneType>(a, i, e); }
                }
            }
        }
        if(!grid_barrier(a.ws, nblocks, a.limit_ns, a.status)) { break; }
    }
}

// A cooperative kernel whose barriers expect `extra` more arrivals than it has blocks:
// with extra > 0 no wait can end, and every block must leave after the time limit.
__global__ void k_barrier_check(PersistWs w, unsigned extra, unsigned long long limit_ns, pg_status *status) {
    for(int k = 0; k < 3; k++) {
        if(!grid_barrier(w, gridDim.x + extra, limit_ns, status)) { return; }
    }
}

typedef void (*StepsKernel)(StepsArgs);

// Blocks of a cooperative launch: as many as the device keeps resident at once (all of
// them must be, for the grid barrier).  Queried once per kernel and device, so that a
// call inside a stream capture issues nothing but the launch.
constexpr int kCoopKernels = 32, kCoopDevices = 64;
static std::atomic<int> g_coop_grid[kCoopKernels][kCoopDevices];

// slots: 0-3 k_lj_steps, 4 k_barrier_check, 8 + k the ensemble's persistent kernels
int cooperative_grid(int slot, const void *kernel, int block, int *grid) {
    int dev = 0;
    if(slot < 0 || slot >= kCoopKernels) { return PG_ERR_ARGUMENT; }
    if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kCoopDevices) { return PG_ERR_CUDA; }
    int g = g_coop_grid[slot][dev].load(std::memory_order_acquire);
    if(g == 0) {
        int sms = 0, coop = 0, per_sm = 0;
        if(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) { return PG_ERR_CUDA; }
        if(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) { return PG_ERR_CUDA; }
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1) {
            return PG_ERR_CUDA;
        }
        g = per_sm * sms;
        g_coop_grid[slot][dev].store(g, std::memory_order_release);
    }
    *grid = g;
    return PG_OK;
}

int lj_steps(const pg_box *box, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj, double dt,
             double half_skin2, int32_t first, int32_t nsteps, pg_status *status, pg_workspace ws, double timeout_s,
             cudaStream_t st) {
    if(!box || !p || !list || !lj || !status || nsteps < 0) { return PG_ERR_ARGUMENT; }
    if(!p->pos || !p->vel || !p->mass || !p->force32 || !p->pos_fx || !p->ref_fx || !p->pos_ref || !list->nbr ||
       !list->count || list->nbr16 != nullptr || list->pair_table != nullptr) {
        return PG_ERR_ARGUMENT;
    }
    if(lj->ntypes < 1 || lj->ntypes > kMaxTypes || (lj->ntypes > 1 && !p->type)) { return PG_ERR_ARGUMENT; }
    if(!(box->fx_unit[0] > 0.0f && box->fx_unit[1] > 0.0f && box->fx_unit[2] > 0.0f)) { return PG_ERR_ARGUMENT; }
    if(ws.ptr == nullptr || ws.bytes < 256 + 8) { return PG_ERR_ARGUMENT; }
    const bool half = list->half != 0, one = lj->ntypes == 1;
    StepsKernel k = half ? (one ? k_lj_steps<true, true> : k_lj_steps<true, false>)
                         : (one ? k_lj_steps<false, true> : k_lj_steps<false, false>);
    int grid = 0;
    const int rc = cooperative_grid((half ? 2 : 0) + (one ? 1 : 0), (const void *) k, kPersistBlock, &grid);
    if(rc != PG_OK) { return rc; }
    if(nsteps == 0 || p->n == 0) { return PG_OK; }         // (a call of no steps only prepares the launch)
    StepsArgs a;
    a.box = *box; a.p = *p; a.list = *list;
    a.lj.ntypes = lj->ntypes;
    a.lj.cutoff2 = lj->cutoff2;
    a.lj.cutoff2f = (float) lj->cutoff2;
    for(int k = 0; k < lj->ntypes * lj->ntypes; k++) {
        a.lj.eps[k] = lj->epsilon[k]; a.lj.sig6[k] = lj->sigma6[k];
        a.lj.epsf[k] = (float) lj->epsilon[k]; a.lj.sig6f[k] = (float) lj->sigma6[k];
    }
    a.dt = dt;
    a.kick = 2.0 * (dt * 0.5);
    a.half_skin2 = half_skin2;
    a.half_skin2_lo = (float) (half_skin2 * (1.0 - 1e-3));
    a.half_skin2_hi = (float) (half_skin2 * (1.0 + 1e-3));
    a.first = first;
    a.nsteps = nsteps;
    a.status = status;
    a.ws = persist_ws(ws.ptr, ws.bytes);
    a.limit_ns = timeout_ns(timeout_s);
    cudaMemsetAsync(ws.ptr, 0, 256, st);                    // queue count, barrier words, abort word
    void *args[] = {&a};
    if(cudaLaunchCooperativeKernel((const void *) k, grid, kPersistBlock, args, 0, st) != cudaSuccess) {
        return PG_ERR_CUDA;
    }
    note_launch();
    return launch_status();
}

int grid_barrier_check(int32_t extra_arrivals, double timeout_s, pg_status *status, pg_workspace ws, cudaStream_t st) {
    if(!status || extra_arrivals < 0 || ws.ptr == nullptr || ws.bytes < 256) { return PG_ERR_ARGUMENT; }
    int grid = 0;
    const int rc = cooperative_grid(4, (const void *) k_barrier_check, kPersistBlock, &grid);
    if(rc != PG_OK) { return rc; }
    cudaMemsetAsync(ws.ptr, 0, 256, st);
    PersistWs w = persist_ws(ws.ptr, ws.bytes);
    unsigned extra = (unsigned) extra_arrivals;
    unsigned long long limit = timeout_ns(timeout_s);
    void *args[] = {&w, &extra, &limit, &status};
    if(cudaLaunchCooperativeKernel((const void *) k_barrier_check, grid, kPersistBlock, args, 0, st) != cudaSuccess) {
        return PG_ERR_CUDA;
    }
    note_launch();
    return launch_status();
}

}  // namespace pg
