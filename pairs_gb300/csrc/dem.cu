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
// every FP64 operation is separately rounded, as in the reference's C code.
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
};

__device__ __forceinline__ D4 ldd(const double *b, int i) { return ld_d4_plain(b, i); }

__device__ __forceinline__ bool dem_frozen(const pg_dem_particles &d, bool integrate) {
    if(d.guard == nullptr) { return false; }
    const int32_t g = *((volatile const int32_t *) d.guard);
    return integrate ? g < d.step : g <= d.step;
}

// ------------------------------------------------------------------ setup

__global__ void k_dem_setup(pg_dem_particles d) {
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
    const int wm = warp_max(cnt);
    if((threadIdx.x & 31) == 0 && wm > 0) {
        atomicMax(&a.status->max_neighbors, wm);
        if(wm > a.list.max_neighbors) { atomicOr(&a.status->overflow, 2); }
    }
}

// ------------------------------------------------------------------ contact model

// One contact's spring-dashpot update, examples/dem.py:18-74 once the geometry
// (normal n, contact point cp, overlap delta) is known.  h is the contact's record
// (tangential spring displacement in x, y, z; impact velocity magnitude in w).
__device__ void spring_dashpot(const pg_dem_params &p, double inv_mi, double mj, int tij, const D4 &xi,
                               const D4 &xj, const D4 &vi, const D4 &vj, const D4 &wi, const D4 &wj,
                               const double n[3], const double cp[3], double delta, int &sticking, D4 &h,
                               double facc[3], double tacc[3]) {
    const double ri[3] = {cp[0] - xi.x, cp[1] - xi.y, cp[2] - xi.z};
    const double rj[3] = {cp[0] - xj.x, cp[1] - xj.y, cp[2] - xj.z};
    double vwi[3], vwj[3], rel[3], reln[3], relt[3];
    vwi[0] = vi.x + (wi.y * ri[2] - wi.z * ri[1]);
    vwi[1] = vi.y + (wi.z * ri[0] - wi.x * ri[2]);
    vwi[2] = vi.z + (wi.x * ri[1] - wi.y * ri[0]);
    vwj[0] = vj.x + (wj.y * rj[2] - wj.z * rj[1]);
    vwj[1] = vj.y + (wj.z * rj[0] - wj.x * rj[2]);
    vwj[2] = vj.z + (wj.x * rj[1] - wj.y * rj[0]);
    for(int e = 0; e < 3; e++) { rel[e] = -(vwi[e] - vwj[e]); }
    const double vn = rel[0] * n[0] + rel[1] * n[1] + rel[2] * n[2];
    for(int e = 0; e < 3; e++) { reln[e] = vn * n[e]; relt[e] = rel[e] - reln[e]; }
    const double lrt = sqrt(relt[0] * relt[0] + relt[1] * relt[1] + relt[2] * relt[2]);
    const bool cond1a = (sticking == 1) && (lrt < 1e-08);
    const double meff = 1.0 / (inv_mi + (1.0 / mj));
    const double kn = (meff * ((p.pi * p.pi) + (p.ln_e * p.ln_e))) / (p.tc * p.tc);
    const double kt = p.kappa * kn;
    const double tsd0[3] = {h.x, h.y, h.z};
    const double proj = tsd0[0] * n[0] + tsd0[1] * n[1] + tsd0[2] * n[2];
    double rot[3], nts[3], fTLS[3], fN[3], t[3];
    for(int e = 0; e < 3; e++) { rot[e] = tsd0[e] - n[e] * proj; }
    const double rl2 = rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2];
    const double tl2 = tsd0[0] * tsd0[0] + tsd0[1] * tsd0[1] + tsd0[2] * tsd0[2];
    const double sc = sqrt(tl2 / rl2);
    for(int e = 0; e < 3; e++) {
        const double sel = (rl2 <= 0.0) ? 0.0 : rot[e] * sc;
        nts[e] = p.dt * relt[e] + sel;
    }
    const double dn = ((-(2.0)) * meff) * p.ln_e / p.tc;
    const double dtn = sqrt(p.kappa) * dn;
    for(int e = 0; e < 3; e++) { fTLS[e] = kt * nts[e] + dtn * relt[e]; }
    const double fTLS_len = sqrt(fTLS[0] * fTLS[0] + fTLS[1] * fTLS[1] + fTLS[2] * fTLS[2]);
    const double kd = kn * delta;
    for(int e = 0; e < 3; e++) { fN[e] = kd * n[e] + dn * reln[e]; }
    const double fNl = sqrt(fN[0] * fN[0] + fN[1] * fN[1] + fN[2] * fN[2]);
    const double fstat = p.friction_static[tij] * fNl;
    const bool cond1 = cond1a && (fTLS_len < fstat);
    const double fdyn = p.friction_dynamic[tij] * fNl;
    const bool cond2 = (sticking == 1) && (fTLS_len < fdyn);
    const bool slide = (!cond1 && !cond2) && (kt > 0.0);
    const double ffa = cond1 ? fstat : fdyn;
    const double tl = sqrt(fTLS[0] * fTLS[0] + fTLS[1] * fTLS[1] + fTLS[2] * fTLS[2]);
    const double itl = 1.0 / tl;
    for(int e = 0; e < 3; e++) { t[e] = (tl > 0.0) ? fTLS[e] * itl : 0.0; }
    double nt[3];
    for(int e = 0; e < 3; e++) { nt[e] = slide ? ((ffa * t[e]) - (dtn * relt[e])) / kt : nts[e]; }
    const double lrel = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2]);
    const double ivm = (h.w > 0.0) ? h.w : lrel;
    h = make_d4(nt[0], nt[1], nt[2], ivm);
    sticking = ((cond1 || cond2) || (fTLS_len < fdyn)) ? 1 : 0;
    const double fTabs = (ffa < fTLS_len) ? ffa : fTLS_len;
    double pf[3];
    for(int e = 0; e < 3; e++) { pf[e] = fN[e] + fTabs * t[e]; facc[e] = facc[e] + pf[e]; }
    const double c0 = (cp[1] - xi.y) * pf[2] - (cp[2] - xi.z) * pf[1];
    const double c1 = (cp[2] - xi.z) * pf[0] - (cp[0] - xi.x) * pf[2];
    const double c2 = (cp[0] - xi.x) * pf[1] - (cp[1] - xi.y) * pf[0];
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

__device__ __forceinline__ void dem_contact(const DemArgs &a, int i, int j, const D4 &xi, const D4 &xj,
                                            const D4 &vi, const D4 &wi, double inv_mi, int ti, const double n[3],
                                            const double cp[3], double delta, int &nc, uint32_t used[2],
                                            bool &overflow, double f[3], double t[3]) {
    const int slot = dem_slot(a.c, i, a.d.uid[j], nc, used);
    if(slot < 0) { overflow = true; return; }
    const size_t s = (size_t) slot * a.c.stride + i;
    int sticking = a.c.sticking[s];
    D4 h = ldd(a.c.history, (int) s);
    const int tij = ti * a.prm.ntypes + (a.d.type ? a.d.type[j] : 0);
    spring_dashpot(a.prm, inv_mi, a.d.mass[j], tij, xi, xj, vi, ldd(a.d.vel, j), wi, ldd(a.d.angvel, j), n, cp,
                   delta, sticking, h, f, t);
    a.c.sticking[s] = sticking;
    st_d4(a.c.history, (int) s, h);
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
    const D4 xi = ldd(a.d.pos, i), vi = ldd(a.d.vel, i), wi = ldd(a.d.angvel, i);
    const double ri = a.d.radius[i];
    const double inv_mi = 1.0 / a.d.mass[i];
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
        const uint32_t code = e >> PG_NBR_INDEX_BITS;
        D4 xj = ldd(a.d.pos, j);
        if(code != 0u) {
            xj.x = ref_image(xj.x, image_shift(code, 0), a.box.len[0]);
            xj.y = ref_image(xj.y, image_shift(code, 1), a.box.len[1]);
            xj.z = ref_image(xj.z, image_shift(code, 2), a.box.len[2]);
        }
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
        dem_contact(a, i, j, xi, xj, vi, wi, inv_mi, ti, n, cp, delta, nc, used, overflow, fs, ts);
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
        dem_contact(a, i, j, xi, xj, vi, wi, inv_mi, ti, n, cp, delta, nc, used, overflow, fh, th);
    }
    // drop the records not used this step: the last record moves into the hole and
    // is examined in turn (sim/contact_history.py:103-120)
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
    a.c.count[i] = nc;
    if(overflow) {
        atomicOr(&a.status->overflow, 8);
        atomicMax(&a.status->max_contacts, a.c.capacity + 1);
    }
    // reset to 0, gravity on z, then the contact sums (sphere part + half-space part)
    const double vol = (((4.0 / 3.0) * a.prm.pi) * ri) * ri * ri;
    const double gz = 0.0 - (a.prm.drho * vol) * a.prm.gravity;
    st_d4(a.d.force, i, make_d4(0.0 + (fs[0] + fh[0]), 0.0 + (fs[1] + fh[1]), gz + (fs[2] + fh[2]), 0.0));
    st_d4(a.d.torque, i, make_d4(0.0 + (ts[0] + th[0]), 0.0 + (ts[1] + th[1]), 0.0 + (ts[2] + th[2]), 0.0));
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

__global__ void __launch_bounds__(kBlock) k_dem_euler(DemArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool tripped = false;
    if(i < a.d.n && !dem_frozen(a.d, true) && !(a.d.flags != nullptr && (a.d.flags[i] & kFlagFixed))) {
        const double dt = a.prm.dt;
        const D4 X = ldd(a.d.pos, i), V = ldd(a.d.vel, i), W = ldd(a.d.angvel, i);
        const D4 F = ldd(a.d.force, i), T = ldd(a.d.torque, i), Qd = ldd(a.d.quat, i);
        const double Qo[4] = {Qd.x, Qd.y, Qd.z, Qd.w};
        double R[9];
        quat_matrix(Qo, R);                      // the rotation matrix of the last step
        const double iI = a.d.inv_inertia[i];
        const double im = 1.0 / a.d.mass[i];
        const double h = 0.5 * im;
        const double f3[3] = {F.x, F.y, F.z}, t3[3] = {T.x, T.y, T.z};
        double x3[3] = {X.x, X.y, X.z}, v3[3] = {V.x, V.y, V.z}, w3[3] = {W.x, W.y, W.z};
        for(int e = 0; e < 3; e++) { x3[e] = x3[e] + (((h * f3[e]) * dt) * dt + v3[e] * dt); }
        for(int e = 0; e < 3; e++) { v3[e] = v3[e] + (im * f3[e]) * dt; }
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
        st_d4(a.d.pos, i, make_d4(x3[0], x3[1], x3[2], X.w));
        st_d4(a.d.vel, i, make_d4(v3[0], v3[1], v3[2], 0.0));
        st_d4(a.d.angvel, i, make_d4(w3[0], w3[1], w3[2], 0.0));
        st_d4(a.d.quat, i, make_d4(r_ * il2, i_ * il2, j_ * il2, k_ * il2));
        if(a.d.pos_ref != nullptr) {
            const D4 r0 = ldd(a.d.pos_ref, i);
            const double ex = x3[0] - r0.x, ey = x3[1] - r0.y, ez = x3[2] - r0.z;
            tripped = (ex * ex + ey * ey + ez * ez) > a.half_skin2;
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

int dem_setup(pg_dem_particles *d, cudaStream_t st) {
    if(!dem_ok(d)) { return PG_ERR_ARGUMENT; }
    if(d->n > 0) { k_dem_setup<<<blocks_for(d->n), kBlock, 0, st>>>(*d); note_launch(); }
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

int dem_build_list(const pg_box *box, pg_dem_particles *d, const pg_cells *cells, pg_neighbor_list *list,
                   const pg_dem_params *prm, pg_status *status, cudaStream_t st) {
    if(!box || !dem_ok(d) || !d->pos_ref || !cells || !list || !list->nbr || !list->count || !prm || !status) {
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
              const pg_contacts *c, const pg_dem_params *prm, pg_status *status, cudaStream_t st) {
    if(!box || !dem_ok(d) || !cells || !list || !list->nbr || !list->count || !contacts_ok(c, d) || !prm ||
       !status) {
        return PG_ERR_ARGUMENT;
    }
    if(prm->ntypes < 1 || prm->ntypes > 4 || list->stride < d->n) { return PG_ERR_ARGUMENT; }
    DemArgs a = {};
    a.box = *box; a.d = *d; a.cells = *cells; a.list = *list; a.c = *c; a.prm = *prm; a.status = status;
    if(d->n > 0) { k_dem_force<<<blocks_for(d->n, kDemBlock), kDemBlock, 0, st>>>(a); note_launch(); }
    return launch_status();
}

int dem_euler(pg_dem_particles *d, const pg_dem_params *prm, double half_skin2, int32_t step, pg_status *status,
              cudaStream_t st) {
    if(!dem_ok(d) || !prm || !status) { return PG_ERR_ARGUMENT; }
    DemArgs a = {};
    a.d = *d; a.prm = *prm; a.status = status; a.half_skin2 = half_skin2; a.step = step;
    if(d->n > 0) { k_dem_euler<<<blocks_for(d->n), kBlock, 0, st>>>(a); note_launch(); }
    return launch_status();
}

}  // namespace pg
