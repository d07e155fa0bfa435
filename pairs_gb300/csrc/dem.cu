// DEM: gravity, linear spring-dashpot contacts with tangential history, explicit
// Euler with rotation, in FP64.
//
// Restates the reference's DEM program (examples/dem.py):
//   update_mass_and_inertia  examples/dem.py:6-15, inversed() mapping/keywords.py:129-146
//   gravity                  examples/dem.py:90-92
//   linear_spring_dashpot    examples/dem.py:18-74; geometry sim/interaction.py:234-264
//                            (sphere-sphere and sphere-half-space); contact history
//                            sim/contact_history.py:12-127, mapping/funcs.py:230-265
//   euler                    examples/dem.py:77-87 with the quaternion keywords of
//                            mapping/keywords.py:208-259
// with the generated operation order.  This file is compiled with -fmad=false so
// every FP64 operation is separately rounded, as in the reference's C code.  A
// mixed-precision contact kernel (FP64 geometry, FP32 contact model) serves large
// granular workloads.
//
// GPU organisation: one thread per particle.  Each particle owns its contact
// records (partner uid, sticking flag, tangential spring displacement, impact
// velocity magnitude), as in the reference, so the contact kernel needs no atomics:
// a sphere pair is evaluated from both sides, each side updating its own record.
// Candidates come from a Verlet list with the radius-dependent cutoff r_i + r_j +
// skin; the exact overlap test runs every step.  Half-space walls are the infinite
// particles of the cell grid's trailing bucket and are tested by every sphere.
#include "common.cuh"

namespace pg {

int bin_particles(const pg_box *box, pg_particles *p, pg_cells *cells, pg_workspace ws, pg_status *status,
                  cudaStream_t st, int32_t **perm_out);

constexpr int kDemBlock = 128;
constexpr int kShapeHalfspace = 1;

struct DemArgs {
    pg_box box;
    pg_dem_particles d;
    pg_cells cells;
    pg_neighbor_list list;
    pg_contacts c;
    pg_dem_params prm;
    pg_status *status;
    double half_skin2;
    int32_t step;
    float screen;                // FP32 candidate screen margin (metres), mixed kernel
    float len32[3];              // box lengths in FP32 (mixed kernel's image shifts)
};

// gravity on a sphere, examples/dem.py:90-92 in the generated order (kept in angvel.w
// by the setup kernel: the radius never changes)
__device__ __forceinline__ double sphere_gravity(const pg_dem_params &prm, double r) {
    const double vol = (((4.0 / 3.0) * prm.pi) * r) * r * r;
    return 0.0 - (prm.drho * vol) * prm.gravity;
}

__device__ __forceinline__ D4 ldd(const double *b, int i) { return ld_d4_plain(b, i); }

__device__ __forceinline__ bool dem_frozen(const pg_dem_particles &d, bool integrate) {
    if(d.guard == nullptr) { return false; }
    const int32_t g = *((volatile const int32_t *) d.guard);
    return integrate ? g < d.step : g <= d.step;
}

// ------------------------------------------------------------------ setup

__global__ void k_dem_setup(pg_dem_particles d, pg_dem_params prm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= d.n) { return; }
    st_d4(d.quat, i, make_d4(1.0, 0.0, 0.0, 0.0));
    if(d.shape[i] == 0) {
        // inversed(diagonal_matrix(v)): det = v*(v*v - 0*0) + 0*(...) + 0*(...),
        // entry (0,0) = (1/det) * (v*v - 0*0); the other diagonal entries are equal
        // and the off-diagonal ones +0.
        const double r = d.radius[i];
        const double v = 0.4 * d.mass[i] * r * r;
        const double det = v * ((v * v) - (0.0 * 0.0)) + 0.0 * ((0.0 * 0.0) - (v * 0.0)) +
                           0.0 * ((0.0 * 0.0) - (v * 0.0));
        d.inv_inertia[i] = (1.0 / det) * ((v * v) - (0.0 * 0.0));
    } else {
        d.mass[i] = __longlong_as_double(0x7ff0000000000000ll);
        d.inv_inertia[i] = 0.0;
    }
    // vel.w keeps 1 / mass (0 for half spaces): the kernels read it with the velocity
    // instead of dividing every step (the same IEEE quotient, so FP64 results are
    // unchanged)
    D4 v = ldd(d.vel, i);
    v.w = 1.0 / d.mass[i];
    st_d4(d.vel, i, v);
    // angvel.w keeps the sphere's gravity force on z (0 for half spaces), the value the
    // contact kernels would otherwise recompute from the radius every step
    D4 w = ldd(d.angvel, i);
    w.w = d.shape[i] == 0 ? sphere_gravity(prm, d.radius[i]) : 0.0;
    st_d4(d.angvel, i, w);
}

// ------------------------------------------------------------------ binning

// gather of the arrays the binning does not permute in place, into the spare set
__global__ void k_dem_gather(int n, const int32_t *perm, pg_dem_particles d, pg_dem_particles o, pg_contacts c,
                             pg_contacts oc) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n) { return; }
    const int s = perm[k];
    st_d4(o.vel, k, ldd(d.vel, s));
    st_d4(o.angvel, k, ldd(d.angvel, s));
    st_d4(o.quat, k, ldd(d.quat, s));
    st_d4(o.normal, k, ldd(d.normal, s));
    o.mass[k] = d.mass[s];
    o.radius[k] = d.radius[s];
    o.inv_inertia[k] = d.inv_inertia[s];
    o.shape[k] = d.shape[s];
    if(d.type) { o.type[k] = d.type[s]; }
    const int nc = c.count[s];
    oc.count[k] = nc;
    for(int q = 0; q < nc; q++) {
        const size_t a = (size_t) q * c.stride + s, b = (size_t) q * oc.stride + k;
        oc.partner[b] = c.partner[a];
        oc.sticking[b] = c.sticking[a];
        st_d4(oc.history, (int) b, ldd(c.history, (int) a));
    }
}

// ------------------------------------------------------------------ list build

__global__ void __launch_bounds__(kBlock) k_dem_list(DemArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.d.n) { return; }
    const D4 xi = ldd(a.d.pos, i);
    st_d4(a.d.pos_ref, i, xi);
    if(a.d.pos32 != nullptr) {
        st_f4(a.d.pos32, i, make_float4((float) xi.x, (float) xi.y, (float) xi.z, (float) a.d.radius[i]));
    }
    int cnt = 0;
    const int ci = a.cells.particle_cell[i];
    if(ci < a.cells.ncells && a.d.shape[i] == 0) {
        const double ri = a.d.radius[i];
        const int dz_ = a.cells.dims[2], dy_ = a.cells.dims[1], dx_ = a.cells.dims[0];
        const int cz = ci % dz_, cy = (ci / dz_) % dy_, cx = ci / (dz_ * dy_);
        const int stride = a.list.stride, cap = a.list.max_neighbors;
        for(int ox = -1; ox <= 1; ox++) {
            int nx = cx + ox, sx = 0;
            if(nx < 0) { if(!a.box.periodic[0]) { continue; } nx += dx_; sx = -1; }
            else if(nx >= dx_) { if(!a.box.periodic[0]) { continue; } nx -= dx_; sx = 1; }
            for(int oy = -1; oy <= 1; oy++) {
                int ny = cy + oy, sy = 0;
                if(ny < 0) { if(!a.box.periodic[1]) { continue; } ny += dy_; sy = -1; }
                else if(ny >= dy_) { if(!a.box.periodic[1]) { continue; } ny -= dy_; sy = 1; }
                for(int oz = -1; oz <= 1; oz++) {
                    int nz = cz + oz, sz = 0;
                    if(nz < 0) { if(!a.box.periodic[2]) { continue; } nz += dz_; sz = -1; }
                    else if(nz >= dz_) { if(!a.box.periodic[2]) { continue; } nz -= dz_; sz = 1; }
                    const int c = (nx * dy_ + ny) * dz_ + nz;
                    const int b = a.cells.cell_start[c], e = b + a.cells.cell_count[c];
                    const uint32_t code = image_code(sx, sy, sz);
                    for(int j = b; j < e; j++) {
                        if(j == i && code == 0u) { continue; }
                        const D4 xj = ldd(a.d.pos, j);
                        const double dx = xi.x - ref_image(xj.x, sx, a.box.len[0]);
                        const double dy = xi.y - ref_image(xj.y, sy, a.box.len[1]);
                        const double dz = xi.z - ref_image(xj.z, sz, a.box.len[2]);
                        const double cut = ri + a.d.radius[j] + a.prm.skin;
                        if(dx * dx + dy * dy + dz * dz < cut * cut) {
                            if(cnt < cap) {
                                a.list.nbr[(size_t) cnt * stride + i] =
                                    (int32_t) ((code << PG_NBR_INDEX_BITS) | (uint32_t) j);
                            }
                            cnt++;
                        }
                    }
                }
            }
        }
    }
    a.list.count[i] = min(cnt, a.list.max_neighbors);
    publish_count(cnt, a.list.max_neighbors, a.status);
}

// ------------------------------------------------------------------ contact model

// One contact's spring-dashpot update, examples/dem.py:18-74 once the geometry is
// known: normal n, overlap delta, and the contact point relative to both centres
// (ri = cp - x_i, rj = cp - x_j).  h is the contact's record (tangential spring
// displacement in x, y, z; impact velocity magnitude in w).  T = double follows the
// generated operation order; T = float is the mixed-precision contact model (the
// overlap itself comes from FP64 geometry, see k_dem_force_mixed).
template<typename T>
__device__ void spring_dashpot(const pg_dem_params &p, T inv_mi, T inv_mj, int tij, const T vi[3], const T vj[3],
                               const T wi[3], const T wj[3], const T n[3], const T ri[3], const T rj[3], T delta,
                               int &sticking, T h[4], T facc[3], T tacc[3]) {
    T vwi[3], vwj[3], rel[3], reln[3], relt[3];
    vwi[0] = vi[0] + (wi[1] * ri[2] - wi[2] * ri[1]);
    vwi[1] = vi[1] + (wi[2] * ri[0] - wi[0] * ri[2]);
    vwi[2] = vi[2] + (wi[0] * ri[1] - wi[1] * ri[0]);
    vwj[0] = vj[0] + (wj[1] * rj[2] - wj[2] * rj[1]);
    vwj[1] = vj[1] + (wj[2] * rj[0] - wj[0] * rj[2]);
    vwj[2] = vj[2] + (wj[0] * rj[1] - wj[1] * rj[0]);
    for(int e = 0; e < 3; e++) { rel[e] = -(vwi[e] - vwj[e]); }
    const T vn = rel[0] * n[0] + rel[1] * n[1] + rel[2] * n[2];
    for(int e = 0; e < 3; e++) { reln[e] = vn * n[e]; relt[e] = rel[e] - reln[e]; }
    const T lrt = sqrt(relt[0] * relt[0] + relt[1] * relt[1] + relt[2] * relt[2]);
    const bool cond1a = (sticking == 1) && (lrt < T(1e-08));
    const T meff = T(1.0) / (inv_mi + inv_mj);
    const T pi = T(p.pi), ln_e = T(p.ln_e), kappa = T(p.kappa), dt = T(p.dt);
    T kn, dn;
    if(p.kn > 0.0) {
        // fixed normal stiffness; damping from the restitution relation
        kn = T(p.kn);
        dn = (((-(T(2.0))) * ln_e) * sqrt(meff * kn)) / sqrt((pi * pi) + (ln_e * ln_e));
    } else {
        const T tc = T(p.tc);
        kn = (meff * ((pi * pi) + (ln_e * ln_e))) / (tc * tc);
        dn = ((-(T(2.0))) * meff) * ln_e / tc;
    }
    const T kt = kappa * kn;
    const T tsd0[3] = {h[0], h[1], h[2]};
    const T proj = tsd0[0] * n[0] + tsd0[1] * n[1] + tsd0[2] * n[2];
    T rot[3], nts[3], fTLS[3], fN[3], t[3];
    for(int e = 0; e < 3; e++) { rot[e] = tsd0[e] - n[e] * proj; }
    const T rl2 = rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2];
    const T tl2 = tsd0[0] * tsd0[0] + tsd0[1] * tsd0[1] + tsd0[2] * tsd0[2];
    const T sc = sqrt(tl2 / rl2);
    for(int e = 0; e < 3; e++) {
        const T sel = (rl2 <= T(0.0)) ? T(0.0) : rot[e] * sc;
        nts[e] = dt * relt[e] + sel;
    }
    const T dtn = sqrt(kappa) * dn;
    for(int e = 0; e < 3; e++) { fTLS[e] = kt * nts[e] + dtn * relt[e]; }
    const T fTLS_len = sqrt(fTLS[0] * fTLS[0] + fTLS[1] * fTLS[1] + fTLS[2] * fTLS[2]);
    const T kd = kn * delta;
    for(int e = 0; e < 3; e++) { fN[e] = kd * n[e] + dn * reln[e]; }
    const T fNl = sqrt(fN[0] * fN[0] + fN[1] * fN[1] + fN[2] * fN[2]);
    const T fstat = T(p.friction_static[tij]) * fNl;
    const bool cond1 = cond1a && (fTLS_len < fstat);
    const T fdyn = T(p.friction_dynamic[tij]) * fNl;
    const bool cond2 = (sticking == 1) && (fTLS_len < fdyn);
    const bool slide = (!cond1 && !cond2) && (kt > T(0.0));
    const T ffa = cond1 ? fstat : fdyn;
    const T tl = sqrt(fTLS[0] * fTLS[0] + fTLS[1] * fTLS[1] + fTLS[2] * fTLS[2]);
    const T itl = T(1.0) / tl;
    for(int e = 0; e < 3; e++) { t[e] = (tl > T(0.0)) ? fTLS[e] * itl : T(0.0); }
    T nt[3];
    for(int e = 0; e < 3; e++) { nt[e] = slide ? ((ffa * t[e]) - (dtn * relt[e])) / kt : nts[e]; }
    const T lrel = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2]);
    const T ivm = (h[3] > T(0.0)) ? h[3] : lrel;
    h[0] = nt[0]; h[1] = nt[1]; h[2] = nt[2]; h[3] = ivm;
    sticking = ((cond1 || cond2) || (fTLS_len < fdyn)) ? 1 : 0;
    const T fTabs = (ffa < fTLS_len) ? ffa : fTLS_len;
    T pf[3];
    for(int e = 0; e < 3; e++) { pf[e] = fN[e] + fTabs * t[e]; facc[e] = facc[e] + pf[e]; }
    const T c0 = ri[1] * pf[2] - ri[2] * pf[1];
    const T c1 = ri[2] * pf[0] - ri[0] * pf[2];
    const T c2 = ri[0] * pf[1] - ri[1] * pf[0];
    tacc[0] = tacc[0] + c0;
    tacc[1] = tacc[1] + c1;
    tacc[2] = tacc[2] + c2;
}

// The record of partner uid `uj` (the last matching slot, as the reference's
// search), created with the contact properties' defaults when absent.  Returns -1
// when all `capacity` slots are taken.
__device__ __forceinline__ int dem_slot(const pg_contacts &c, int i, int uj, int &nc, uint32_t used[2]) {
    int id = -1;
    for(int k = 0; k < nc; k++) {
        if(c.partner[(size_t) k * c.stride + i] == uj) { id = k; }
    }
    if(id == -1) {
        if(nc >= c.capacity) { return -1; }
        id = nc++;
        const size_t a = (size_t) id * c.stride + i;
        c.partner[a] = uj;
        c.sticking[a] = 0;
        st_d4(c.history, (int) a, make_d4(0.0, 0.0, 0.0, 0.0));
    }
    used[id >> 5] |= 1u << (id & 31);
    return id;
}

// Look up / create the contact record of partner j, run the model in precision T,
// store the record back.
template<typename T>
__device__ __forceinline__ void dem_contact(const DemArgs &a, int i, int j, const T vi[3], const T wi[3],
                                            T inv_mi, int ti, const T n[3], const T ri[3], const T rj[3], T delta,
                                            int &nc, uint32_t used[2], bool &overflow, T f[3], T t[3]) {
    const int slot = dem_slot(a.c, i, a.d.uid[j], nc, used);
    if(slot < 0) { overflow = true; return; }
    const size_t s = (size_t) slot * a.c.stride + i;
    int sticking = a.c.sticking[s];
    const D4 hd = ldd(a.c.history, (int) s);
    T h[4] = {T(hd.x), T(hd.y), T(hd.z), T(hd.w)};
    const int tij = ti * a.prm.ntypes + (a.d.type ? a.d.type[j] : 0);
    const D4 vj4 = ldd(a.d.vel, j), wj4 = ldd(a.d.angvel, j);
    const T vj[3] = {T(vj4.x), T(vj4.y), T(vj4.z)}, wj[3] = {T(wj4.x), T(wj4.y), T(wj4.z)};
    spring_dashpot<T>(a.prm, inv_mi, T(vj4.w), tij, vi, vj, wi, wj, n, ri, rj, delta, sticking, h, f, t);
    a.c.sticking[s] = sticking;
    st_d4(a.c.history, (int) s, make_d4(h[0], h[1], h[2], h[3]));
}

// drop the records not used this step: the last record moves into the hole and is
// examined in turn (sim/contact_history.py:103-120)
__device__ __forceinline__ void clear_unused(const DemArgs &a, int i, int &nc, uint32_t used[2]) {
    int k = 0;
    while(k < nc) {
        if(!((used[k >> 5] >> (k & 31)) & 1u)) {
            const int last = nc - 1;
            if(last > 0) {
                const size_t dst = (size_t) k * a.c.stride + i, src = (size_t) last * a.c.stride + i;
                a.c.partner[dst] = a.c.partner[src];
                a.c.sticking[dst] = a.c.sticking[src];
                st_d4(a.c.history, (int) dst, ldd(a.c.history, (int) src));
                if((used[last >> 5] >> (last & 31)) & 1u) { used[k >> 5] |= 1u << (k & 31); }
                else { used[k >> 5] &= ~(1u << (k & 31)); }
            }
            nc--;
        } else {
            k++;
        }
    }
}

__device__ __forceinline__ D4 image_of(const DemArgs &a, int j, uint32_t code) {
    D4 xj = ldd(a.d.pos, j);
    if(code != 0u) {
        xj.x = ref_image(xj.x, image_shift(code, 0), a.box.len[0]);
        xj.y = ref_image(xj.y, image_shift(code, 1), a.box.len[1]);
        xj.z = ref_image(xj.z, image_shift(code, 2), a.box.len[2]);
    }
    return xj;
}

__global__ void __launch_bounds__(kDemBlock) k_dem_force(DemArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.d.n || dem_frozen(a.d, false)) { return; }
    if(a.d.flags != nullptr && (a.d.flags[i] & kFlagFixed)) {
        st_d4(a.d.force, i, make_d4(0.0, 0.0, 0.0, 0.0));
        st_d4(a.d.torque, i, make_d4(0.0, 0.0, 0.0, 0.0));
        a.c.count[i] = 0;
        return;
    }
    const D4 xi = ldd(a.d.pos, i), v4 = ldd(a.d.vel, i), w4 = ldd(a.d.angvel, i);
    const double vi[3] = {v4.x, v4.y, v4.z}, wi[3] = {w4.x, w4.y, w4.z};
    const double ri = a.d.radius[i];
    const double inv_mi = v4.w;                  // 1 / mass (pg_dem_setup)
    const int ti = a.d.type ? a.d.type[i] : 0;
    int nc = a.c.count[i];
    uint32_t used[2] = {0u, 0u};
    double fs[3] = {0, 0, 0}, ts[3] = {0, 0, 0}, fh[3] = {0, 0, 0}, th[3] = {0, 0, 0};
    bool overflow = false;
    // sphere-sphere (sim/interaction.py:234-246)
    const int cnt = a.list.count[i];
    for(int k = 0; k < cnt; k++) {
        const uint32_t e = (uint32_t) a.list.nbr[(size_t) k * a.list.stride + i];
        const int j = (int) (e & PG_NBR_INDEX_MASK);
        const D4 xj = image_of(a, j, e >> PG_NBR_INDEX_BITS);
        const double d0 = xi.x - xj.x, d1 = xi.y - xj.y, d2 = xi.z - xj.z;
        const double rsq = d0 * d0 + d1 * d1 + d2 * d2;
        const double rj = a.d.radius[j];
        const double sep = ri + rj;
        if(!(rsq < sep * (sep + 0.0))) { continue; }
        const double dist = sqrt(rsq);
        const double pd = (dist - ri) - rj;
        const double delta = -pd;
        if(delta < 0.0) { continue; }
        const double inv = 1.0 / dist;
        const double n[3] = {d0 * inv, d1 * inv, d2 * inv};
        const double kk = rj + 0.5 * pd;
        const double cp[3] = {xj.x + n[0] * kk, xj.y + n[1] * kk, xj.z + n[2] * kk};
        const double rvi[3] = {cp[0] - xi.x, cp[1] - xi.y, cp[2] - xi.z};
        const double rvj[3] = {cp[0] - xj.x, cp[1] - xj.y, cp[2] - xj.z};
        dem_contact<double>(a, i, j, vi, wi, inv_mi, ti, n, rvi, rvj, delta, nc, used, overflow, fs, ts);
    }
    // sphere-half-space (sim/interaction.py:248-264)
    const int wb = a.cells.cell_start[a.cells.ncells], we = wb + a.cells.cell_count[a.cells.ncells];
    for(int j = wb; j < we; j++) {
        if(a.d.shape[j] != kShapeHalfspace) { continue; }
        const D4 nj = ldd(a.d.normal, j), xj = ldd(a.d.pos, j);
        const double kx = (nj.x * xi.x + nj.y * xi.y) + nj.z * xi.z;
        const double dd = (nj.x * xj.x + nj.y * xj.y) + nj.z * xj.z;
        const double pd = (kx - ri) - dd;
        if(!(pd < 0.0)) { continue; }
        const double delta = -pd;
        if(delta < 0.0) { continue; }
        const double tmp = ri + pd;
        const double n[3] = {nj.x, nj.y, nj.z};
        const double cp[3] = {xi.x - tmp * nj.x, xi.y - tmp * nj.y, xi.z - tmp * nj.z};
        const double rvi[3] = {cp[0] - xi.x, cp[1] - xi.y, cp[2] - xi.z};
        const double rvj[3] = {cp[0] - xj.x, cp[1] - xj.y, cp[2] - xj.z};
        dem_contact<double>(a, i, j, vi, wi, inv_mi, ti, n, rvi, rvj, delta, nc, used, overflow, fh, th);
    }
    clear_unused(a, i, nc, used);
    a.c.count[i] = nc;
    if(overflow) {
        atomicOr(&a.status->overflow, 8);
        atomicMax(&a.status->max_contacts, a.c.capacity + 1);
    }
    // reset to 0, gravity on z (kept in angvel.w), then the contact sums (sphere part +
    // half-space part)
    const double gz = w4.w;
    st_d4(a.d.force, i, make_d4(0.0 + (fs[0] + fh[0]), 0.0 + (fs[1] + fh[1]), gz + (fs[2] + fh[2]), 0.0));
    st_d4(a.d.torque, i, make_d4(0.0 + (ts[0] + th[0]), 0.0 + (ts[1] + th[1]), 0.0 + (ts[2] + th[2]), 0.0));
}

// Mixed precision: the contact geometry in FP64 (overlaps are ~1e-7 of the
// separation, far below FP32 resolution of a distance), everything after it in
// FP32: normal from the FP32 difference vector, overlap from the FP64 numerator
// sep^2 - |d|^2 divided by sep + |d| (no cancellation), contact-point offsets
// relative to the two centres, the spring-dashpot model, friction and the force /
// torque sums.  The integrator stays FP64.
__global__ void __launch_bounds__(kDemBlock) k_dem_force_mixed(DemArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.d.n || dem_frozen(a.d, false)) { return; }
    if(a.d.flags != nullptr && (a.d.flags[i] & kFlagFixed)) {
        st_d4(a.d.force, i, make_d4(0.0, 0.0, 0.0, 0.0));
        st_d4(a.d.torque, i, make_d4(0.0, 0.0, 0.0, 0.0));
        a.c.count[i] = 0;
        return;
    }
    const D4 xi = ldd(a.d.pos, i), v4 = ldd(a.d.vel, i), w4 = ldd(a.d.angvel, i);
    // the FP32 velocities and 1/mass are converted at the first contact: most spheres
    // of a packing touch nothing, and their force is then gravity alone
    float vi[3], wi[3], inv_mi = 0.0f;
    bool touched = false;
    auto convert = [&]() {
        if(touched) { return; }
        vi[0] = (float) v4.x; vi[1] = (float) v4.y; vi[2] = (float) v4.z;
        wi[0] = (float) w4.x; wi[1] = (float) w4.y; wi[2] = (float) w4.z;
        inv_mi = (float) v4.w;
        touched = true;
    };
    const double ri = a.d.radius[i];
    // FP32 screen: a candidate whose FP32 distance exceeds the contact distance by more
    // than the FP32 rounding of the coordinates (a.screen) cannot touch
    const float4 pi32 = ld_f4(a.d.pos32, i);
    const float lx = a.len32[0], ly = a.len32[1], lz = a.len32[2];
    const int ti = a.d.type ? a.d.type[i] : 0;
    int nc = a.c.count[i];
    uint32_t used[2] = {0u, 0u};
    float fs[3] = {0, 0, 0}, ts[3] = {0, 0, 0}, fh[3] = {0, 0, 0}, th[3] = {0, 0, 0};
    bool overflow = false;
    const int cnt = a.list.count[i];
    for(int k = 0; k < cnt; k++) {
        const uint32_t e = (uint32_t) a.list.nbr[(size_t) k * a.list.stride + i];
        const int j = (int) (e & PG_NBR_INDEX_MASK);
        const uint32_t code = e >> PG_NBR_INDEX_BITS;
        {
            const float4 pj = ld_f4(a.d.pos32, j);
            const float fx = pi32.x - (pj.x + image_shift(code, 0) * lx);
            const float fy = pi32.y - (pj.y + image_shift(code, 1) * ly);
            const float fz = pi32.z - (pj.z + image_shift(code, 2) * lz);
            const float lim = pi32.w + pj.w + a.screen;
            if(fx * fx + fy * fy + fz * fz > lim * lim) { continue; }
        }
        const D4 xj = image_of(a, j, code);
        const double d0 = xi.x - xj.x, d1 = xi.y - xj.y, d2 = xi.z - xj.z;
        const double rsq = d0 * d0 + d1 * d1 + d2 * d2;
        const double rj = a.d.radius[j];
        const double sep = ri + rj;
        if(!(rsq < sep * sep)) { continue; }
        const float dist = sqrtf((float) rsq);
        const float delta = (float) (sep * sep - rsq) / ((float) sep + dist);
        const float inv = 1.0f / dist;
        const float df[3] = {(float) d0, (float) d1, (float) d2};
        const float n[3] = {df[0] * inv, df[1] * inv, df[2] * inv};
        const float kk = (float) rj - 0.5f * delta;
        const float rvj[3] = {n[0] * kk, n[1] * kk, n[2] * kk};
        const float rvi[3] = {rvj[0] - df[0], rvj[1] - df[1], rvj[2] - df[2]};
        convert();
        dem_contact<float>(a, i, j, vi, wi, inv_mi, ti, n, rvi, rvj, delta, nc, used, overflow, fs, ts);
    }
    const int wb = a.cells.cell_start[a.cells.ncells], we = wb + a.cells.cell_count[a.cells.ncells];
    for(int j = wb; j < we; j++) {
        if(a.d.shape[j] != kShapeHalfspace) { continue; }
        const D4 nj = ldd(a.d.normal, j), xj = ldd(a.d.pos, j);
        {
            const float pdf = ((float) nj.x * (pi32.x - (float) xj.x) + (float) nj.y * (pi32.y - (float) xj.y)) +
                              (float) nj.z * (pi32.z - (float) xj.z) - pi32.w;
            if(pdf > a.screen) { continue; }
        }
        const double kx = (nj.x * xi.x + nj.y * xi.y) + nj.z * xi.z;
        const double dd = (nj.x * xj.x + nj.y * xj.y) + nj.z * xj.z;
        const double pd = (kx - ri) - dd;
        if(!(pd < 0.0)) { continue; }
        const float delta = (float) (-pd);
        const float tmp = (float) (ri + pd);
        const float n[3] = {(float) nj.x, (float) nj.y, (float) nj.z};
        const float rvi[3] = {-tmp * n[0], -tmp * n[1], -tmp * n[2]};
        const float rvj[3] = {(float) (xi.x - xj.x) + rvi[0], (float) (xi.y - xj.y) + rvi[1],
                              (float) (xi.z - xj.z) + rvi[2]};
        convert();
        dem_contact<float>(a, i, j, vi, wi, inv_mi, ti, n, rvi, rvj, delta, nc, used, overflow, fh, th);
    }
    clear_unused(a, i, nc, used);
    a.c.count[i] = nc;
    if(overflow) {
        atomicOr(&a.status->overflow, 8);
        atomicMax(&a.status->max_contacts, a.c.capacity + 1);
    }
    const double gz = w4.w;                      // gravity on z (pg_dem_setup)
    if(!touched) {
        // no contact: the sums are +0, and gz + 0 = gz (gz is never -0)
        st_d4(a.d.force, i, make_d4(0.0, 0.0, gz, 0.0));
        st_d4(a.d.torque, i, make_d4(0.0, 0.0, 0.0, 0.0));
        return;
    }
    st_d4(a.d.force, i, make_d4((double) (fs[0] + fh[0]), (double) (fs[1] + fh[1]), gz + (double) (fs[2] + fh[2]),
                                0.0));
    st_d4(a.d.torque, i, make_d4((double) (ts[0] + th[0]), (double) (ts[1] + th[1]), (double) (ts[2] + th[2]), 0.0));
}

// ------------------------------------------------------------------ Euler with rotation

// quaternion_to_rotation_matrix (mapping/keywords.py:241-259)
__device__ __forceinline__ void quat_matrix(const double Q[4], double R[9]) {
    R[0] = (1.0 - 2.0 * Q[2] * Q[2]) - 2.0 * Q[3] * Q[3];
    R[1] = 2.0 * (Q[1] * Q[2] - Q[0] * Q[3]);
    R[2] = 2.0 * (Q[1] * Q[3] + Q[0] * Q[2]);
    R[3] = 2.0 * (Q[1] * Q[2] + Q[0] * Q[3]);
    R[4] = (1.0 - 2.0 * Q[1] * Q[1]) - 2.0 * Q[3] * Q[3];
    R[5] = 2.0 * (Q[2] * Q[3] - Q[0] * Q[1]);
    R[6] = 2.0 * (Q[1] * Q[3] - Q[0] * Q[2]);
    R[7] = 2.0 * (Q[2] * Q[3] + Q[0] * Q[1]);
    R[8] = (1.0 - 2.0 * Q[1] * Q[1]) - 2.0 * Q[2] * Q[2];
}

// +0 or -0, tested on the bit pattern (integer work: GB300's FP64 rate is low)
__device__ __forceinline__ bool zero_bits(double v) { return (__double_as_longlong(v) << 1) == 0; }

// kMixed: the mixed path's step, the same FP64 update with fused multiply-adds,
// x + dt v + (dt^2 / 2m) F and v + (dt / m) F; otherwise the generated operation order.
template<bool kMixed>
__global__ void __launch_bounds__(kBlock) k_dem_euler(DemArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool tripped = false;
    if(i < a.d.n && !dem_frozen(a.d, true) && !(a.d.flags != nullptr && (a.d.flags[i] & kFlagFixed))) {
        const double dt = a.prm.dt;
        const D4 X = ldd(a.d.pos, i), V = ldd(a.d.vel, i), W = ldd(a.d.angvel, i);
        const D4 F = ldd(a.d.force, i), T = ldd(a.d.torque, i), Qd = ldd(a.d.quat, i);
        const double Qo[4] = {Qd.x, Qd.y, Qd.z, Qd.w};
        const double im = V.w;                   // 1 / mass (pg_dem_setup)
        const double f3[3] = {F.x, F.y, F.z}, t3[3] = {T.x, T.y, T.z};
        double x3[3] = {X.x, X.y, X.z}, v3[3] = {V.x, V.y, V.z}, w3[3] = {W.x, W.y, W.z};
        if(kMixed) {
            const double c = (0.5 * im) * (dt * dt), b = im * dt;
            for(int e = 0; e < 3; e++) { x3[e] = fma(c, f3[e], fma(dt, v3[e], x3[e])); }
            for(int e = 0; e < 3; e++) { v3[e] = fma(b, f3[e], v3[e]); }
        } else {
            const double h = 0.5 * im;
            for(int e = 0; e < 3; e++) { x3[e] = x3[e] + (((h * f3[e]) * dt) * dt + v3[e] * dt); }
            for(int e = 0; e < 3; e++) { v3[e] = v3[e] + (im * f3[e]) * dt; }
        }
        // No torque and no spin: the rotation yields phi = 0, the identity quaternion,
        // the product q Q = Q bit for bit and, when |Q|^2 is within 1e-8 of one, no
        // renormalisation -- orientation and angular velocity stay as they are, so the
        // FP64 rotation arithmetic is skipped (most spheres of a settling packing).  A
        // sphere that never turned (torque and spin +-0, orientation exactly (1, 0, 0, 0),
        // so |Q|^2 = 1) is recognised from the bit patterns alone.
        const bool never_turned = zero_bits(T.x) && zero_bits(T.y) && zero_bits(T.z) && zero_bits(W.x) &&
                                  zero_bits(W.y) && zero_bits(W.z) &&
                                  __double_as_longlong(Qd.x) == 0x3FF0000000000000ll && zero_bits(Qd.y) &&
                                  zero_bits(Qd.z) && zero_bits(Qd.w);
        const bool still = never_turned ||
                           (T.x == 0.0 && T.y == 0.0 && T.z == 0.0 && W.x == 0.0 && W.y == 0.0 && W.z == 0.0 &&
                            fabs((((Qo[0] * Qo[0] + Qo[1] * Qo[1]) + Qo[2] * Qo[2]) + Qo[3] * Qo[3]) - 1.0) < 1e-08);
        if(!still) {
            double R[9];
            quat_matrix(Qo, R);                  // the rotation matrix of the last step
            const double iI = a.d.inv_inertia[i];
            // inv_inertia * torque with the +0 off-diagonal entries of the reference's matrix
            double av[3], bv[3], wd[3], phi[3];
            av[0] = (iI * t3[0] + 0.0 * t3[1]) + 0.0 * t3[2];
            av[1] = (0.0 * t3[0] + iI * t3[1]) + 0.0 * t3[2];
            av[2] = (0.0 * t3[0] + 0.0 * t3[1]) + iI * t3[2];
            for(int r = 0; r < 3; r++) { bv[r] = (R[r * 3] * av[0] + R[r * 3 + 1] * av[1]) + R[r * 3 + 2] * av[2]; }
            for(int c = 0; c < 3; c++) { wd[c] = (bv[0] * R[c] + bv[1] * R[c + 3]) + bv[2] * R[c + 6]; }
            for(int e = 0; e < 3; e++) { phi[e] = w3[e] * dt + ((0.5 * wd[e]) * dt) * dt; }
            const double lp = sqrt(phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2]);
            double q[4];
            if(fabs(lp) < 1e-06) {
                q[0] = 1.0; q[1] = 0.0; q[2] = 0.0; q[3] = 0.0;
            } else {
                const double ca = cos(lp * 0.5), sa = sin(lp * 0.5), il = 1.0 / lp;
                q[0] = ca; q[1] = sa * (phi[0] * il); q[2] = sa * (phi[1] * il); q[3] = sa * (phi[2] * il);
            }
            const double r_ = ((q[0] * Qo[0] - q[1] * Qo[1]) - q[2] * Qo[2]) - q[3] * Qo[3];
            const double i_ = ((q[0] * Qo[1] + q[1] * Qo[0]) + q[2] * Qo[3]) - q[3] * Qo[2];
            const double j_ = ((q[0] * Qo[2] + q[2] * Qo[0]) + q[3] * Qo[1]) - q[1] * Qo[3];
            const double k_ = ((q[0] * Qo[3] + q[3] * Qo[0]) + q[1] * Qo[2]) - q[2] * Qo[1];
            const double len2 = ((r_ * r_ + i_ * i_) + j_ * j_) + k_ * k_;
            const double il2 = (fabs(len2 - 1.0) < 1e-08) ? 1.0 : 1.0 / sqrt(len2);
            for(int e = 0; e < 3; e++) { w3[e] = w3[e] + wd[e] * dt; }
            st_d4(a.d.angvel, i, make_d4(w3[0], w3[1], w3[2], W.w));
            st_d4(a.d.quat, i, make_d4(r_ * il2, i_ * il2, j_ * il2, k_ * il2));
        }
        st_d4(a.d.pos, i, make_d4(x3[0], x3[1], x3[2], X.w));
        if(a.d.pos32 != nullptr) {
            st_f4(a.d.pos32, i, make_float4((float) x3[0], (float) x3[1], (float) x3[2], (float) a.d.radius[i]));
        }
        st_d4(a.d.vel, i, make_d4(v3[0], v3[1], v3[2], V.w));
        if(a.d.pos_ref != nullptr) {
            // the guard (no counterpart in the reference) with fused multiply-adds
            const D4 r0 = ldd(a.d.pos_ref, i);
            const double ex = x3[0] - r0.x, ey = x3[1] - r0.y, ez = x3[2] - r0.z;
            tripped = fma(ex, ex, fma(ey, ey, ez * ez)) > a.half_skin2;
        }
    }
    if(__any_sync(0xffffffffu, tripped) && (threadIdx.x & 31) == 0) {
        atomicMin(&a.status->guard_tripped, a.step);
    }
}

// ------------------------------------------------------------------ host side

static bool dem_ok(const pg_dem_particles *d) {
    return d && d->n >= 0 && d->n <= d->capacity && d->pos && d->vel && d->angvel && d->force && d->torque &&
           d->quat && d->normal && d->mass && d->radius && d->inv_inertia && d->uid && d->shape;
}

static bool contacts_ok(const pg_contacts *c, const pg_dem_particles *d) {
    return c && c->count && c->partner && c->sticking && c->history && c->capacity >= 1 && c->capacity <= 64 &&
           c->stride >= d->n;
}

int dem_setup(pg_dem_particles *d, const pg_dem_params *prm, cudaStream_t st) {
    if(!dem_ok(d) || !prm) { return PG_ERR_ARGUMENT; }
    if(d->n > 0) { k_dem_setup<<<blocks_for(d->n), kBlock, 0, st>>>(*d, *prm); note_launch(); }
    return launch_status();
}

int dem_bin(const pg_box *box, pg_dem_particles *d, const pg_dem_particles *spare, const pg_contacts *c,
            const pg_contacts *spare_c, pg_cells *cells, pg_workspace ws, pg_status *status, cudaStream_t st) {
    if(!box || !dem_ok(d) || !spare || !dem_ok(spare) || spare->capacity < d->n || !contacts_ok(c, d) ||
       !contacts_ok(spare_c, d) || spare_c->capacity != c->capacity || !cells || !status) {
        return PG_ERR_ARGUMENT;
    }
    if(d->type != nullptr && spare->type == nullptr) { return PG_ERR_ARGUMENT; }
    pg_particles view = {};
    view.n = d->n;
    view.capacity = d->capacity;
    view.pos = d->pos;
    view.uid = d->uid;
    view.flags = d->flags;
    int32_t *perm = nullptr;
    const int rc = bin_particles(box, &view, cells, ws, status, st, &perm);
    if(rc) { return rc; }
    if(d->n > 0) {
        k_dem_gather<<<blocks_for(d->n), kBlock, 0, st>>>(d->n, perm, *d, *spare, *c, *spare_c);
        note_launch();
    }
    return launch_status();
}

bool grid_ok(const pg_cells *cells);

int dem_build_list(const pg_box *box, pg_dem_particles *d, const pg_cells *cells, pg_neighbor_list *list,
                   const pg_dem_params *prm, pg_status *status, cudaStream_t st) {
    if(!box || !dem_ok(d) || !d->pos_ref || !grid_ok(cells) || !list || !list->nbr || !list->count || !prm || !status) {
        return PG_ERR_ARGUMENT;
    }
    if(list->stride < d->n || d->n >= (1 << PG_NBR_INDEX_BITS) || list->max_neighbors < 1) {
        return PG_ERR_ARGUMENT;
    }
    DemArgs a = {};
    a.box = *box; a.d = *d; a.cells = *cells; a.list = *list; a.prm = *prm; a.status = status;
    if(d->n > 0) { k_dem_list<<<blocks_for(d->n), kBlock, 0, st>>>(a); note_launch(); }
    return launch_status();
}

int dem_force(const pg_box *box, const pg_dem_particles *d, const pg_cells *cells, const pg_neighbor_list *list,
              const pg_contacts *c, const pg_dem_params *prm, int precision, pg_status *status, cudaStream_t st) {
    if(!box || !dem_ok(d) || !cells || !list || !list->nbr || !list->count || !contacts_ok(c, d) || !prm ||
       !status) {
        return PG_ERR_ARGUMENT;
    }
    if(prm->ntypes < 1 || prm->ntypes > 4 || list->stride < d->n) { return PG_ERR_ARGUMENT; }
    if(precision != PG_FP64 && precision != PG_MIXED) { return PG_ERR_ARGUMENT; }
    if(precision == PG_MIXED && d->pos32 == nullptr) { return PG_ERR_ARGUMENT; }
    DemArgs a = {};
    a.box = *box; a.d = *d; a.cells = *cells; a.list = *list; a.c = *c; a.prm = *prm; a.status = status;
    // FP32 rounding of coordinates up to |lo| + 2 len (images), of radii and of the
    // distance arithmetic, with a factor 64 of room
    double span = 0.0;
    for(int k = 0; k < 3; k++) { span = fmax(span, fabs(box->lo[k]) + 2.0 * box->len[k]); }
    a.screen = (float) (64.0 * span * 1.1920928955078125e-07);
    for(int k = 0; k < 3; k++) { a.len32[k] = (float) box->len[k]; }
    if(d->n > 0) {
        if(precision == PG_FP64) { k_dem_force<<<blocks_for(d->n, kDemBlock), kDemBlock, 0, st>>>(a); }
        else { k_dem_force_mixed<<<blocks_for(d->n, kDemBlock), kDemBlock, 0, st>>>(a); }
        note_launch();
    }
    return launch_status();
}

int dem_euler(pg_dem_particles *d, const pg_dem_params *prm, int precision, double half_skin2, int32_t step,
              pg_status *status, cudaStream_t st) {
    if(!dem_ok(d) || !prm || !status) { return PG_ERR_ARGUMENT; }
    if(precision != PG_FP64 && precision != PG_MIXED) { return PG_ERR_ARGUMENT; }
    DemArgs a = {};
    a.d = *d; a.prm = *prm; a.status = status; a.half_skin2 = half_skin2; a.step = step;
    if(d->n > 0) {
        if(precision == PG_MIXED) { k_dem_euler<true><<<blocks_for(d->n), kBlock, 0, st>>>(a); }
        else { k_dem_euler<false><<<blocks_for(d->n), kBlock, 0, st>>>(a); }
        note_launch();
    }
    return launch_status();
}

}  // namespace pg
