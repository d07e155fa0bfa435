// Velocity-Verlet integration, displacement guard and thermo reductions.
//
// Integration restates the reference's user kernels examples/md.py:11-17 with the
// generated operation order (separately rounded, no fused multiply-add):
//   initial:  v = v + ((dt*0.5) * F) / m;   x = x + dt * v
//   final:    v = v + ((dt*0.5) * F) / m
// so that, given the same forces, positions and velocities are bit-identical to
// the reference's.  The FP64 guard |x - x_ref|^2 > (skin/2)^2 is evaluated in the
// same pass (x_ref = positions at the last list build).
//
// Thermo restates runtime/thermo.hpp:11-51: sum m (vx*vx + vy*vy + vz*vz) in FP64
// over a fixed reduction tree (deterministic), T = sum / (3N - 3), kinetic pressure
// T (3N - 3) / (3 V).
#include "common.cuh"

namespace pg {

struct IntArgs {
    pg_box box;
    pg_particles p;
    double dt, h;             // h = dt * 0.5, computed by the caller in FP64
    double half_skin2;
    int32_t step;
    int mixed;
    int from_prev;            // read positions from pos_prev1 (reference image sync)
    int do_initial, do_final; // final kick (of this step) then initial kick + drift
    pg_status *status;
};

__device__ __forceinline__ double3 load_force(const IntArgs &a, int i) {
    if(a.mixed) {
        const float4 f = ld_f4(a.p.force32, i);
        return make_double3((double) f.x, (double) f.y, (double) f.z);
    }
    const D4 f = ld_d4(a.p.force, i);
    return make_double3(f.x, f.y, f.z);
}

__device__ __forceinline__ double kick(double v, double h, double f, double m) {
    // (h*F)/m; dividing by 1.0 is exact, so unit masses skip the (slow) FP64 divide
    const double hf = __dmul_rn(h, f);
    return __dadd_rn(v, m == 1.0 ? hf : __ddiv_rn(hf, m));
}

__global__ void __launch_bounds__(kBlock) k_integrate(IntArgs a) {
    if(a.do_initial ? frozen_integrate(a.p) : frozen_force(a.p)) { return; }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool tripped = false;
    if(i < a.p.n && !(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed))) {
        const double m = a.p.mass[i];
        const double3 f = load_force(a, i);
        D4 v = ld_d4_plain(a.p.vel, i);
        if(a.do_final) {
            v.x = kick(v.x, a.h, f.x, m); v.y = kick(v.y, a.h, f.y, m); v.z = kick(v.z, a.h, f.z, m);
        }
        if(a.do_initial) {
            v.x = kick(v.x, a.h, f.x, m); v.y = kick(v.y, a.h, f.y, m); v.z = kick(v.z, a.h, f.z, m);
            D4 x = ld_d4_plain(a.from_prev ? a.p.pos_prev1 : a.p.pos, i);
            x.x = __dadd_rn(x.x, __dmul_rn(a.dt, v.x));
            x.y = __dadd_rn(x.y, __dmul_rn(a.dt, v.y));
            x.z = __dadd_rn(x.z, __dmul_rn(a.dt, v.z));
            st_d4(a.p.pos, i, x);
            if(a.p.pos_ref != nullptr) {
                const D4 r = ld_d4_plain(a.p.pos_ref, i);
                const double ex = x.x - r.x, ey = x.y - r.y, ez = x.z - r.z;
                tripped = (ex * ex + ey * ey + ez * ez) > a.half_skin2;
            }
            if(a.p.pos_hi != nullptr) {
                const double q = a.box.quantum, iq = 1.0 / q;
                float4 hv, lv;
                split_pos(x.x, iq, q, hv.x, lv.x);
                split_pos(x.y, iq, q, hv.y, lv.y);
                split_pos(x.z, iq, q, hv.z, lv.z);
                hv.w = __int_as_float(a.p.type != nullptr ? a.p.type[i] : 0);
                lv.w = 0.0f;
                st_f4(a.p.pos_hi, hl(a.p, i), hv);
                st_f4(a.p.pos_lo, hl(a.p, i), lv);
            }
            if(a.p.pos_fx != nullptr) {
                st_i4(a.p.pos_fx, i, fx_position(a.box, x.x, x.y, x.z, a.p.type != nullptr ? a.p.type[i] : 0));
            }
        }
        st_d4(a.p.vel, i, v);
    } else if(i < a.p.n && a.from_prev) {
        // fixed particles do not move, but the position ring still advances
        st_d4(a.p.pos, i, ld_d4_plain(a.p.pos_prev1, i));
    }
    if(__any_sync(0xffffffffu, tripped) && (threadIdx.x & 31) == 0) {
        atomicMin(&a.status->guard_tripped, a.step);
    }
}

// ------------------------------------------------------------------ mixed precision
// Mixed-precision step: FP32 forces in, FP64 velocity and position update, compensated
// FP32 positions re-split (or fixed-point positions rounded) from the new FP64
// positions, FP64 displacement guard.
// GB300 issues ~2 FP64 instructions per clock per SM, so FP64 work is kept to what
// the method needs: the kicks of a deferred final half step and the next initial
// half step are merged into one (v += k*(dt/2)*F/m, k = 1 or 2), and the guard is
// screened with the FP32 displacement (hi - hi_ref) + (lo - lo_ref), or the exact
// fixed-point displacement converted to FP32; only particles
// within a relative band of 1e-3 of the threshold are decided by the exact FP64
// test |x - x_ref|^2 > (skin/2)^2, so the outcome is the FP64 test's outcome.

struct MixArgs {
    pg_box box;
    pg_particles p;
    double dt;
    double kick;              // k * dt/2
    float half_skin2_lo, half_skin2_hi;
    double half_skin2;
    int32_t step;
    int drift;                // 0: kick only (a final half step before thermo)
    pg_status *status;
};

// grid point nearest x, rounded in FP64 (|lo| <= q/2)
__device__ __forceinline__ void resplit(double x, float q, float iq, float &hi, float &lo) {
    split_pos(x, (double) iq, (double) q, hi, lo);
}

__global__ void __launch_bounds__(kBlock) k_integrate_mixed(MixArgs a) {
    if(a.drift ? frozen_integrate(a.p) : frozen_force(a.p)) { return; }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool tripped = false;
    if(i < a.p.n && !(a.p.flags != nullptr && (a.p.flags[i] & kFlagFixed))) {
        const float4 f = ld_f4(a.p.force32, i);
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
            // guard, screened in FP32 against the positions of the last list build
            const int type = a.p.type != nullptr ? a.p.type[i] : 0;
            float dx, dy, dz;
            if(a.p.pos_fx != nullptr) {
                const int4 xf = fx_position(a.box, x.x, x.y, x.z, type);
                st_i4(a.p.pos_fx, i, xf);
                const int4 rf = ld_i4(a.p.ref_fx, i);
                dx = (float) fx_diff(xf.x, rf.x) * a.box.fx_unit[0];
                dy = (float) fx_diff(xf.y, rf.y) * a.box.fx_unit[1];
                dz = (float) fx_diff(xf.z, rf.z) * a.box.fx_unit[2];
            } else {
                const float q = (float) a.box.quantum, iq = 1.0f / q;
                float4 h, l;
                resplit(x.x, q, iq, h.x, l.x);
                resplit(x.y, q, iq, h.y, l.y);
                resplit(x.z, q, iq, h.z, l.z);
                h.w = __int_as_float(type);   // type bits
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
        }
    }
    if(__any_sync(0xffffffffu, tripped) && (threadIdx.x & 31) == 0) {
        atomicMin(&a.status->guard_tripped, a.step);
    }
}

int integrate_mixed(const pg_box *box, pg_particles *p, double dt, int kicks, int drift,
                    double half_skin2, int32_t step, pg_status *status, cudaStream_t st) {
    if(!box || !p || !p->pos || !p->vel || !p->mass || !p->force32) { return PG_ERR_ARGUMENT; }
    const bool fx = p->pos_fx != nullptr;
    if(!fx && (!p->pos_hi || !p->pos_lo)) { return PG_ERR_ARGUMENT; }
    if(drift && (!p->pos_ref || !status || (fx ? !p->ref_fx : (!p->ref_hi || !p->ref_lo)))) { return PG_ERR_ARGUMENT; }
    if(kicks < 1 || kicks > 2) { return PG_ERR_ARGUMENT; }
    MixArgs a;
    a.box = *box; a.p = *p; a.dt = dt; a.kick = kicks * (dt * 0.5); a.drift = drift;
    a.half_skin2 = half_skin2;
    a.half_skin2_lo = (float) (half_skin2 * (1.0 - 1e-3));
    a.half_skin2_hi = (float) (half_skin2 * (1.0 + 1e-3));
    a.step = step; a.status = status;
    if(p->n > 0) { k_integrate_mixed<<<blocks_for(p->n), kBlock, 0, st>>>(a); note_launch(); }
    return launch_status();
}

static int launch_integrate(const pg_box *box, pg_particles *p, double dt, int precision,
                            double half_skin2, int32_t step, pg_status *status, int sync_mode,
                            int do_initial, int do_final, cudaStream_t st) {
    if(!box || !p || !p->pos || !p->vel || !p->mass) { return PG_ERR_ARGUMENT; }
    if(precision == PG_FP64 && !p->force) { return PG_ERR_ARGUMENT; }
    if(precision == PG_MIXED && !p->force32) { return PG_ERR_ARGUMENT; }
    if(do_initial && p->pos_ref && !status) { return PG_ERR_ARGUMENT; }
    if(sync_mode == PG_SYNC_REFERENCE && !p->pos_prev1) { return PG_ERR_ARGUMENT; }
    if((p->pos_hi == nullptr) != (p->pos_lo == nullptr)) { return PG_ERR_ARGUMENT; }
    IntArgs a;
    a.box = *box; a.p = *p; a.dt = dt; a.h = dt * 0.5; a.half_skin2 = half_skin2; a.step = step;
    a.mixed = precision == PG_MIXED; a.from_prev = sync_mode == PG_SYNC_REFERENCE && do_initial;
    a.do_initial = do_initial; a.do_final = do_final; a.status = status;
    if(p->n > 0) { k_integrate<<<blocks_for(p->n), kBlock, 0, st>>>(a); note_launch(); }
    return launch_status();
}

int initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision, double half_skin2,
                      int32_t step, pg_status *status, int sync_mode, cudaStream_t st) {
    return launch_integrate(box, p, dt, precision, half_skin2, step, status, sync_mode, 1, 0, st);
}

int final_integrate(const pg_box *box, pg_particles *p, double dt, int precision, cudaStream_t st) {
    return launch_integrate(box, p, dt, precision, 0.0, 0, nullptr, PG_SYNC_EXACT, 0, 1, st);
}

int final_initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision,
                            double half_skin2, int32_t step, pg_status *status, int sync_mode,
                            cudaStream_t st) {
    return launch_integrate(box, p, dt, precision, half_skin2, step, status, sync_mode, 1, 1, st);
}

// ---------------------------------------------------------------------------- thermo

constexpr int kThermoBlocks = 2 * kSMs;     // fixed grid: the reduction tree never changes

__device__ __forceinline__ double block_sum_fixed(double v) {
    __shared__ double s[kBlock / 32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if(lane == 0) { s[w] = v; }
    __syncthreads();
    double t = 0.0;
    if(threadIdx.x == 0) {
        for(int k = 0; k < (int) (blockDim.x >> 5); k++) { t += s[k]; }
    }
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(kBlock) k_ke_partials(pg_particles p, double *partials) {
    double acc = 0.0;
    for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x) {
        const D4 v = ld_d4(p.vel, i);
        const double s = __dadd_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)), __dmul_rn(v.z, v.z));
        acc += __dmul_rn(p.mass[i], s);
    }
    const double t = block_sum_fixed(acc);
    if(threadIdx.x == 0) { partials[blockIdx.x] = t; }
}

__global__ void __launch_bounds__(kBlock) k_ke_finish(const double *partials, int nparts, double t_scale,
                                                      double dof, double p_scale, double *out) {
    double acc = 0.0;
    for(int k = threadIdx.x; k < nparts; k += blockDim.x) { acc += partials[k]; }
    const double sum = block_sum_fixed(acc);
    if(threadIdx.x == 0) {
        const double t = sum * t_scale;
        out[0] = t;
        out[1] = (t * dof) * p_scale;
        out[2] = sum;
    }
}

int64_t thermo_workspace_bytes() { return (int64_t) kThermoBlocks * sizeof(double); }

static void thermo_scales(const pg_box *box, int n, double *t_scale, double *dof, double *p_scale) {
    *dof = (double) (n * 3 - 3);
    *t_scale = 1.0 / *dof;
    *p_scale = 1.0 / 3 / box->len[0] / box->len[1] / box->len[2];
}

int compute_thermo(const pg_box *box, const pg_particles *p, double *out, double *partials,
                   cudaStream_t st) {
    if(!box || !p || !out || !p->vel || !p->mass || !partials || p->n < 2) { return PG_ERR_ARGUMENT; }
    double t_scale, dof, p_scale;
    thermo_scales(box, p->n, &t_scale, &dof, &p_scale);
    k_ke_partials<<<kThermoBlocks, kBlock, 0, st>>>(*p, partials); note_launch();
    k_ke_finish<<<1, kBlock, 0, st>>>(partials, kThermoBlocks, t_scale, dof, p_scale, out); note_launch();
    return launch_status();
}

}  // namespace pg
