/*
 * lj_oracle.c -- CPU restatement of the reference's Lennard-Jones particle path.
 *
 * TEST INFRASTRUCTURE: this file is the oracle the CUDA path is checked against
 * (tests/, __graft_entry__.smoke(), bench.py's CPU baseline).  The product never
 * links or calls it.
 *
 * It restates, in plain C and in the same FP64 operation order, the program the
 * reference's generator emits for its LJ example (examples/md.py) on one rank:
 *
 *   initial state   runtime/copper_fcc_lattice.hpp:18-26 (Park-Miller), :64-145
 *                   (fcc sites in 8^3 sub-boxes), runtime/thermo.hpp:53-97
 *                   (zero momentum, rescale to T)
 *   time loop       sim/simulation.py:387-417 order, sim/timestep.py:36-61 gating
 *                   (rebuild when (ts+1)%every==0 || ts==0; integrate skip_first)
 *   exchange        sim/comm.py:101-151, 223-259, 445-520 (wrap + reorder)
 *   borders         sim/comm.py:57-98 + sim/domain_partitioning.py:65-99 (ghost
 *                   images within one cell spacing of each face, dim by dim)
 *   synchronize     sim/comm.py:46-54, 369-442 (ONE pack over all ghosts, then
 *                   unpack: ghost-of-ghost images read their source ghost before it
 *                   is refreshed, i.e. they lag by one step per extra shifted dim)
 *   cell lists      sim/cell_lists.py:46-134 (grid over [min-s, max+s], cell 0 for
 *                   infinite particles, 27-cell stencil)
 *   neighbour list  sim/neighbor_lists.py:21-48, sim/interaction.py:90-120
 *                   (full: j != i; half: i < j, ghosts always kept)
 *   LJ force        examples/md.py:5-8 via sim/interaction.py:222-232 and
 *                   ir/apply.py:112-125 (half list: reaction on j only if j < nlocal)
 *   integration     examples/md.py:11-17
 *   thermo          runtime/thermo.hpp:11-51
 *
 * Added beyond the reference (it has no such quantities): potential energy and
 * virial of the same truncated, unshifted pair potential, and an `exact` ghost
 * refresh mode that updates images dim by dim so no image lags.
 *
 * Build: cc -O2 -ffp-contract=off -fPIC -shared -fopenmp (see oracle/build.py).
 * -ffp-contract=off keeps every multiply and add separately rounded, as in the
 * generated expression sequence.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FLAG_INFINITE 1
#define FLAG_GHOST    2
#define FLAG_FIXED    4
#define FLAG_GLOBAL   8
#define SHAPE_POINT_MASS 2
#define SUBDOMAIN_SMALL 0.00001          /* runtime/domain/regular_6d_stencil.hpp:6 */

/* ------------------------------------------------------------------------- */
/* Initial state                                                              */
/* ------------------------------------------------------------------------- */

/* Park-Miller minimal standard generator without masking
 * (runtime/copper_fcc_lattice.hpp:18-26). */
static double park_miller(int *seed) {
    const int ia = 16807, im = 2147483647, iq = 127773, ir = 2836;
    int k = (*seed) / iq;
    *seed = ia * (*seed - k * iq) - ir * k;
    if(*seed < 0) { *seed += im; }
    return (1.0 / im) * (*seed);
}

/* fcc lattice of nx*ny*nz unit cells at reduced density rho; visits lattice sites
 * in the reference's sub-box order so particle order, velocities and the rand()
 * stream used for types match (runtime/copper_fcc_lattice.hpp:64-145).  Returns the
 * number of particles written (at most `cap`). */
int lj_fcc_lattice(int nx, int ny, int nz, double rho, int ntypes, int cap,
                   double *pos, double *vel, double *mass, int *type) {
    const double alat = pow(4.0 / rho, 1.0 / 3.0);
    const double xprd = nx * alat, yprd = ny * alat, zprd = nz * alat;
    int ilo = (int) (0.0 / (0.5 * alat) - 1), ihi = (int) (xprd / (0.5 * alat) + 1);
    int jlo = (int) (0.0 / (0.5 * alat) - 1), jhi = (int) (yprd / (0.5 * alat) + 1);
    int klo = (int) (0.0 / (0.5 * alat) - 1), khi = (int) (zprd / (0.5 * alat) + 1);
    ilo = ilo > 0 ? ilo : 0; ihi = ihi < 2 * nx - 1 ? ihi : 2 * nx - 1;
    jlo = jlo > 0 ? jlo : 0; jhi = jhi < 2 * ny - 1 ? jhi : 2 * ny - 1;
    klo = klo > 0 ? klo : 0; khi = khi < 2 * nz - 1 ? khi : 2 * nz - 1;

    const int sub = 8;
    int sx = 0, sy = 0, sz = 0, ox = 0, oy = 0, oz = 0, natoms = 0;
    srand(1);                       /* the reference never seeds rand() */
    while(oz * sub <= khi) {
        const int k = oz * sub + sz, j = oy * sub + sy, i = ox * sub + sx;
        if(((i + j + k) % 2 == 0) && i >= ilo && i <= ihi && j >= jlo && j <= jhi &&
           k >= klo && k <= khi) {
            const double x = 0.5 * alat * i, y = 0.5 * alat * j, z = 0.5 * alat * k;
            if(x >= 0.0 && x < xprd - SUBDOMAIN_SMALL && y >= 0.0 && y < yprd - SUBDOMAIN_SMALL &&
               z >= 0.0 && z < zprd - SUBDOMAIN_SMALL) {
                int n = k * (2 * ny) * (2 * nx) + j * (2 * nx) + i + 1;
                double v[3];
                for(int c = 0; c < 3; c++) {
                    for(int m = 0; m < 5; m++) { park_miller(&n); }
                    v[c] = park_miller(&n);
                }
                if(natoms < cap) {
                    mass[natoms] = 1.0;
                    pos[natoms * 3 + 0] = x; pos[natoms * 3 + 1] = y; pos[natoms * 3 + 2] = z;
                    vel[natoms * 3 + 0] = v[0]; vel[natoms * 3 + 1] = v[1]; vel[natoms * 3 + 2] = v[2];
                    type[natoms] = rand() % ntypes;
                }
                natoms++;
            }
        }
        sx++;
        if(sx == sub) { sx = 0; sy++; }
        if(sy == sub) { sy = 0; sz++; }
        if(sz == sub) { sz = 0; ox++; }
        if(ox * sub > ihi) { ox = 0; oy++; }
        if(oy * sub > jhi) { oy = 0; oz++; }
    }
    return natoms;
}

/* Temperature T = sum m v^2 / (3N-3) (runtime/thermo.hpp:11-51); *press gets the
 * kinetic pressure T*(3N-3)/(3V). */
double lj_temperature(int n, const double *mass, const double *vel, double xprd, double yprd,
                      double zprd, double *press) {
    const double dof = (n * 3 - 3);
    const double t_scale = 1.0 / dof;
    const double p_scale = 1.0 / 3 / xprd / yprd / zprd;
    double t = 0.0;
    for(int i = 0; i < n; i++) {
        t += mass[i] * (vel[i * 3] * vel[i * 3] + vel[i * 3 + 1] * vel[i * 3 + 1] +
                        vel[i * 3 + 2] * vel[i * 3 + 2]);
    }
    t = t * t_scale;
    if(press != NULL) { *press = (t * dof) * p_scale; }
    return t;
}

/* Remove the mean velocity and rescale to `temp` (runtime/thermo.hpp:53-97). */
void lj_adjust_thermo(int n, const double *mass, double *vel, double xprd, double yprd,
                      double zprd, double temp) {
    double vt[3] = {0.0, 0.0, 0.0};
    for(int i = 0; i < n; i++) { for(int d = 0; d < 3; d++) { vt[d] += vel[i * 3 + d]; } }
    for(int d = 0; d < 3; d++) { vt[d] /= n; }
    for(int i = 0; i < n; i++) { for(int d = 0; d < 3; d++) { vel[i * 3 + d] -= vt[d]; } }
    const double t = lj_temperature(n, mass, vel, xprd, yprd, zprd, NULL);
    const double factor = sqrt(temp / t);
    for(int i = 0; i < n; i++) { for(int d = 0; d < 3; d++) { vel[i * 3 + d] *= factor; } }
}

/* ------------------------------------------------------------------------- */
/* Simulation state (one rank, one periodic box)                             */
/* ------------------------------------------------------------------------- */

typedef struct {
    /* configuration */
    int ntypes;
    double eps[64], sig6[64];
    double cutoff2, list2, spacing, dt;
    double lo[3], hi[3], len[3];
    int pbc[3];
    int every;          /* reneighbour period */
    int half;           /* compute_half() */
    int exact_sync;     /* 0: reference ghost refresh (lagging images); 1: per-dim refresh */
    int nthreads;
    /* particles: locals [0, nlocal), ghosts [nlocal, nlocal + nghost) */
    int cap, nlocal, nghost;
    int *uid, *type, *flags, *shape;
    double *mass, *pos, *vel, *force;
    /* halo bookkeeping */
    int nsend_all, nsend[6], nrecv[6], send_off[6], recv_off[6];
    int send_cap;
    int *send_map, *send_mult, *exchg_flag, *copy_to;
    double *buf;        /* staged properties of sent particles */
    int *ibuf;
    /* cell lists */
    int dims[3], ncells, nstencil, stencil[27], cell_cap;
    int *cell_sizes, *cell_particles, *particle_cell;
    /* Verlet lists, AoS [i][k] as the reference's CPU target */
    int neigh_cap;
    int *numneighs, *neighbors;
    int ts;
    int overflow;
} lj_sim;

static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s);
    if(p == NULL) { fprintf(stderr, "lj_oracle: out of memory\n"); abort(); }
    return p;
}

void lj_destroy(lj_sim *s) {
    if(s == NULL) { return; }
    free(s->uid); free(s->type); free(s->flags); free(s->shape);
    free(s->mass); free(s->pos); free(s->vel); free(s->force);
    free(s->send_map); free(s->send_mult); free(s->exchg_flag); free(s->copy_to);
    free(s->buf); free(s->ibuf);
    free(s->cell_sizes); free(s->cell_particles); free(s->particle_cell);
    free(s->numneighs); free(s->neighbors);
    free(s);
}

/* cap: particle capacity including ghosts. */
lj_sim *lj_create(int cap, int ntypes, const double *eps, const double *sig6, double cutoff,
                  double skin, double dt, const double *lo, const double *hi, int every, int half,
                  int exact_sync, int neigh_cap, int nthreads) {
    lj_sim *s = (lj_sim *) xcalloc(1, sizeof(lj_sim));
    s->ntypes = ntypes;
    for(int k = 0; k < ntypes * ntypes && k < 64; k++) { s->eps[k] = eps[k]; s->sig6[k] = sig6[k]; }
    s->cutoff2 = cutoff * cutoff;
    s->spacing = cutoff + skin;
    s->list2 = s->spacing * s->spacing;
    s->dt = dt;
    for(int d = 0; d < 3; d++) {
        s->lo[d] = lo[d]; s->hi[d] = hi[d]; s->len[d] = hi[d] - lo[d]; s->pbc[d] = 1;
    }
    s->every = every; s->half = half; s->exact_sync = exact_sync;
    s->nthreads = nthreads > 0 ? nthreads : 1;
    s->cap = cap;
    s->uid = xcalloc(cap, sizeof(int)); s->type = xcalloc(cap, sizeof(int));
    s->flags = xcalloc(cap, sizeof(int)); s->shape = xcalloc(cap, sizeof(int));
    s->mass = xcalloc(cap, sizeof(double)); s->pos = xcalloc((size_t) cap * 3, sizeof(double));
    s->vel = xcalloc((size_t) cap * 3, sizeof(double));
    s->force = xcalloc((size_t) cap * 3, sizeof(double));
    s->send_cap = cap;
    s->send_map = xcalloc(cap, sizeof(int)); s->send_mult = xcalloc((size_t) cap * 3, sizeof(int));
    s->exchg_flag = xcalloc(cap, sizeof(int)); s->copy_to = xcalloc(cap, sizeof(int));
    s->buf = xcalloc((size_t) cap * 7, sizeof(double)); s->ibuf = xcalloc((size_t) cap * 4, sizeof(int));
    s->particle_cell = xcalloc(cap, sizeof(int));
    s->neigh_cap = neigh_cap;
    s->numneighs = xcalloc(cap, sizeof(int));
    s->neighbors = xcalloc((size_t) cap * neigh_cap, sizeof(int));

    /* grid + stencil (sim/cell_lists.py:46-86) */
    s->ncells = 1;
    for(int d = 0; d < 3; d++) {
        const double dmax = s->hi[d] + s->spacing, dmin = s->lo[d] - s->spacing;
        s->dims[d] = (int) ceil((dmax - dmin) / s->spacing) + 1;
        s->ncells *= s->dims[d];
    }
    s->ncells += 1;
    s->nstencil = 0;
    for(int a = -1; a < 2; a++) {
        for(int b = -1; b < 2; b++) {
            for(int c = -1; c < 2; c++) {
                s->stencil[s->nstencil++] = (a * s->dims[1] + b) * s->dims[2] + c;
            }
        }
    }
    s->cell_cap = 64;
    s->cell_sizes = xcalloc(s->ncells, sizeof(int));
    s->cell_particles = xcalloc((size_t) s->ncells * s->cell_cap, sizeof(int));
    return s;
}

/* Load n local particles (any order); uid must be unique. */
void lj_set_state(lj_sim *s, int n, const int *uid, const int *type, const double *mass,
                  const double *pos, const double *vel) {
    s->nlocal = n; s->nghost = 0; s->ts = 0;
    for(int i = 0; i < n; i++) {
        s->uid[i] = uid[i]; s->type[i] = type[i]; s->mass[i] = mass[i];
        s->flags[i] = 0; s->shape[i] = SHAPE_POINT_MASS;
        for(int d = 0; d < 3; d++) {
            s->pos[i * 3 + d] = pos[i * 3 + d]; s->vel[i * 3 + d] = vel[i * 3 + d];
            s->force[i * 3 + d] = 0.0;
        }
    }
}

/* ---- exchange: wrap particles that left the box, reordering like the reference */

static void exchange_dim(lj_sim *s, int d) {
    s->nsend_all = 0;
    s->nghost = 0;
    for(int j = 0; j <= 2 * d + 1; j++) { s->nsend[j] = 0; s->nrecv[j] = 0; s->send_off[j] = 0; s->recv_off[j] = 0; }
    const int n = s->nlocal + s->nghost;
    for(int i = 0; i < s->nlocal; i++) { s->exchg_flag[i] = 0; }
    for(int side = 0; side < 2; side++) {
        for(int i = 0; i < n; i++) {
            if((s->flags[i] & (FLAG_INFINITE | FLAG_GLOBAL)) != 0) { continue; }
            const double x = s->pos[i * 3 + d];
            if(side == 0 ? (x < s->lo[d]) : (x > s->hi[d])) {
                const int k = s->nsend_all++;
                s->send_map[k] = i;
                s->exchg_flag[i] = 1;
                for(int e = 0; e < 3; e++) { s->send_mult[k * 3 + e] = (e == d) ? (side == 0 ? 1 : -1) : 0; }
                s->nsend[2 * d + side]++;
            }
        }
    }
    s->nrecv[2 * d] = s->nsend[2 * d]; s->nrecv[2 * d + 1] = s->nsend[2 * d + 1];
    /* pack (position shifted by mult * L), comm.py:302-330 */
    const int cnt = s->nsend[2 * d] + s->nsend[2 * d + 1];
    for(int k = 0; k < cnt; k++) {
        const int m = s->send_map[k];
        s->ibuf[k * 4 + 0] = s->uid[m]; s->ibuf[k * 4 + 1] = s->shape[m];
        s->ibuf[k * 4 + 2] = s->flags[m]; s->ibuf[k * 4 + 3] = s->type[m];
        for(int e = 0; e < 3; e++) {
            s->buf[k * 7 + e] = s->pos[m * 3 + e] + s->send_mult[k * 3 + e] * s->len[e];
            s->buf[k * 7 + 4 + e] = s->vel[m * 3 + e];
        }
        s->buf[k * 7 + 3] = s->mass[m];
    }
    /* remove exchanged particles: fill holes from the tail (comm.py:445-506) */
    int send_pos = s->nlocal - 1;
    for(int k = 0; k < s->nsend_all; k++) {
        if(s->send_map[k] < s->nlocal - s->nsend_all) {
            while(s->exchg_flag[send_pos] == 1) { send_pos--; }
            s->copy_to[k] = send_pos;
            send_pos--;
        } else {
            s->copy_to[k] = -1;
        }
    }
    for(int k = 0; k < s->nsend_all; k++) {
        const int src = s->copy_to[k];
        if(src > 0) {            /* the reference tests src > 0 */
            const int dst = s->send_map[k];
            s->uid[dst] = s->uid[src]; s->shape[dst] = s->shape[src]; s->flags[dst] = s->flags[src];
            s->type[dst] = s->type[src]; s->mass[dst] = s->mass[src];
            for(int e = 0; e < 3; e++) {
                s->pos[dst * 3 + e] = s->pos[src * 3 + e]; s->vel[dst * 3 + e] = s->vel[src * 3 + e];
            }
        }
    }
    s->nlocal -= s->nsend_all;
    /* unpack received (= sent, one rank) particles after the locals */
    for(int k = 0; k < cnt; k++) {
        const int t = s->nlocal + k;
        s->uid[t] = s->ibuf[k * 4 + 0]; s->shape[t] = s->ibuf[k * 4 + 1];
        s->flags[t] = s->ibuf[k * 4 + 2]; s->type[t] = s->ibuf[k * 4 + 3];
        s->mass[t] = s->buf[k * 7 + 3];
        for(int e = 0; e < 3; e++) { s->pos[t * 3 + e] = s->buf[k * 7 + e]; s->vel[t * 3 + e] = s->buf[k * 7 + 4 + e]; }
    }
    s->nlocal += cnt;
}

/* ---- borders: ghost images within one spacing of each face, dim by dim */

static int ensure_ghost_room(lj_sim *s, int extra) {
    if(s->nlocal + s->nghost + extra > s->cap || s->nsend_all + extra > s->send_cap) {
        s->overflow = 1;
        return 0;
    }
    return 1;
}

static void borders(lj_sim *s) {
    s->nsend_all = 0;
    s->nghost = 0;
    for(int d = 0; d < 3; d++) {
        s->nsend[2 * d] = s->nsend[2 * d + 1] = 0;
        s->nrecv[2 * d] = s->nrecv[2 * d + 1] = 0;
        if(!s->pbc[d]) { continue; }
        const int n = s->nlocal + s->nghost;
        for(int side = 0; side < 2; side++) {
            for(int i = 0; i < n; i++) {
                if((s->flags[i] & (FLAG_INFINITE | FLAG_GLOBAL)) != 0) { continue; }
                const double x = s->pos[i * 3 + d];
                if(side == 0 ? (x < s->lo[d] + s->spacing) : (x > s->hi[d] - s->spacing)) {
                    if(!ensure_ghost_room(s, 1)) { return; }
                    const int k = s->nsend_all++;
                    s->send_map[k] = i;
                    for(int e = 0; e < 3; e++) { s->send_mult[k * 3 + e] = (e == d) ? (side == 0 ? 1 : -1) : 0; }
                    s->nsend[2 * d + side]++;
                }
            }
        }
        s->nrecv[2 * d] = s->nsend[2 * d]; s->nrecv[2 * d + 1] = s->nsend[2 * d + 1];
        int isend = 0;
        for(int j = 0; j < 2 * d; j++) { isend += s->nsend[j]; }
        s->send_off[2 * d] = s->recv_off[2 * d] = isend;
        s->send_off[2 * d + 1] = s->recv_off[2 * d + 1] = isend + s->nsend[2 * d];
        const int start = s->send_off[2 * d], cnt = s->nsend[2 * d] + s->nsend[2 * d + 1];
        for(int k = start; k < start + cnt; k++) {
            const int m = s->send_map[k];
            s->ibuf[k * 4 + 0] = s->uid[m]; s->ibuf[k * 4 + 1] = s->shape[m];
            s->ibuf[k * 4 + 3] = s->type[m];
            s->buf[k * 7 + 3] = s->mass[m];
            for(int e = 0; e < 3; e++) {
                s->buf[k * 7 + e] = s->pos[m * 3 + e] + s->send_mult[k * 3 + e] * s->len[e];
                s->buf[k * 7 + 4 + e] = s->vel[m * 3 + e];
            }
        }
        for(int k = start; k < start + cnt; k++) {
            const int t = s->nlocal + k;
            s->uid[t] = s->ibuf[k * 4 + 0]; s->shape[t] = s->ibuf[k * 4 + 1];
            s->flags[t] = 0; s->type[t] = s->ibuf[k * 4 + 3]; s->mass[t] = s->buf[k * 7 + 3];
            for(int e = 0; e < 3; e++) { s->pos[t * 3 + e] = s->buf[k * 7 + e]; s->vel[t * 3 + e] = s->buf[k * 7 + 4 + e]; }
        }
        s->nghost += cnt;
    }
}

/* ---- synchronize: refresh ghost positions/velocities from their sources */

static void synchronize(lj_sim *s) {
    if(!s->exact_sync) {
        /* one pack over every ghost, then one unpack (comm.py:369-442) */
        for(int k = 0; k < s->nsend_all; k++) {
            const int m = s->send_map[k];
            for(int e = 0; e < 3; e++) {
                s->buf[k * 7 + e] = s->pos[m * 3 + e] + s->send_mult[k * 3 + e] * s->len[e];
                s->buf[k * 7 + 4 + e] = s->vel[m * 3 + e];
            }
        }
        for(int k = 0; k < s->nsend_all; k++) {
            const int t = s->nlocal + k;
            for(int e = 0; e < 3; e++) { s->pos[t * 3 + e] = s->buf[k * 7 + e]; s->vel[t * 3 + e] = s->buf[k * 7 + 4 + e]; }
        }
    } else {
        /* sources are always created before their images, so refreshing in send
         * order reads every source after its own refresh */
        for(int k = 0; k < s->nsend_all; k++) {
            const int m = s->send_map[k], t = s->nlocal + k;
            for(int e = 0; e < 3; e++) {
                s->pos[t * 3 + e] = s->pos[m * 3 + e] + s->send_mult[k * 3 + e] * s->len[e];
                s->vel[t * 3 + e] = s->vel[m * 3 + e];
            }
        }
    }
}

/* ---- cell lists (sim/cell_lists.py:90-134) */

static int build_cell_lists(lj_sim *s) {
    for(int c = 0; c < s->ncells; c++) { s->cell_sizes[c] = 0; }
    const int n = s->nlocal + s->nghost;
    for(int i = 0; i < n; i++) {
        int flat = 0;
        if(!(s->flags[i] & FLAG_INFINITE)) {
            int idx = 0;
            for(int d = 0; d < 3; d++) {
                const double q = (s->pos[i * 3 + d] - (s->lo[d] - s->spacing)) / s->spacing;
                int c = ((int) q >= 0) ? (int) q : 0;
                c = (c < s->dims[d]) ? c : s->dims[d] - 1;
                idx = (d == 0) ? c : idx * s->dims[d] + c;
            }
            flat = idx + 1;
        }
        if(flat >= 0 && flat < s->ncells) {
            s->particle_cell[i] = flat;
            const int slot = s->cell_sizes[flat]++;
            if(slot >= s->cell_cap) { s->overflow = 2; return 0; }
            s->cell_particles[(size_t) flat * s->cell_cap + slot] = i;
        }
    }
    return 1;
}

/* ---- neighbour lists (sim/neighbor_lists.py:21-48, interaction.py:90-120) */

static void build_neighbor_lists(lj_sim *s) {
    const int nlocal = s->nlocal;
    int overflow = 0;
    #pragma omp parallel for schedule(static) num_threads(s->nthreads) reduction(|:overflow)
    for(int i = 0; i < nlocal; i++) {
        s->numneighs[i] = 0;
        if(s->flags[i] & FLAG_FIXED) { continue; }
        const int ci = s->particle_cell[i];
        const double xi = s->pos[i * 3], yi = s->pos[i * 3 + 1], zi = s->pos[i * 3 + 2];
        int *list = s->neighbors + (size_t) i * s->neigh_cap;
        int nn = 0;
        for(int disp = -1; disp < s->nstencil; disp++) {
            const int nc = (disp < 0) ? 0 : ci + s->stencil[disp];
            if(!(disp < 0 || (nc > 0 && nc < s->ncells))) { continue; }
            const int cnt = s->cell_sizes[nc];
            const int *cp = s->cell_particles + (size_t) nc * s->cell_cap;
            for(int k = 0; k < cnt; k++) {
                const int j = cp[k];
                const int keep = s->half ? (s->shape[j] > SHAPE_POINT_MASS ||
                                            (s->shape[j] == SHAPE_POINT_MASS && i < j))
                                         : (j != i);
                if(!keep) { continue; }
                const double dx = xi - s->pos[j * 3], dy = yi - s->pos[j * 3 + 1], dz = zi - s->pos[j * 3 + 2];
                const double rsq = dx * dx + dy * dy + dz * dz;
                if(rsq < s->list2) {
                    list[nn] = j;
                    if(nn + 2 >= s->neigh_cap) { overflow = 1; } else { nn++; }
                }
            }
        }
        s->numneighs[i] = nn;
    }
    if(overflow) { s->overflow = 3; }
}

/* ---- force (examples/md.py:5-8); energy/virial accumulate per pair if asked */

static void lennard_jones(lj_sim *s, double *pe_out, double *vir_out) {
    const int nlocal = s->nlocal, nt = s->ntypes;
    for(int i = 0; i < nlocal; i++) { for(int e = 0; e < 3; e++) { s->force[i * 3 + e] = 0.0; } }
    double pe = 0.0, vir = 0.0;
    if(!s->half) {
        #pragma omp parallel for schedule(static) num_threads(s->nthreads) reduction(+:pe, vir)
        for(int i = 0; i < nlocal; i++) {
            if(s->flags[i] & FLAG_FIXED) { continue; }
            double fx = 0.0, fy = 0.0, fz = 0.0;
            const double xi = s->pos[i * 3], yi = s->pos[i * 3 + 1], zi = s->pos[i * 3 + 2];
            const int ti = s->type[i] * nt;
            const int *list = s->neighbors + (size_t) i * s->neigh_cap;
            for(int k = 0; k < s->numneighs[i]; k++) {
                const int j = list[k];
                const double dx = xi - s->pos[j * 3], dy = yi - s->pos[j * 3 + 1], dz = zi - s->pos[j * 3 + 2];
                const double rsq = dx * dx + dy * dy + dz * dz;
                if(rsq < s->cutoff2) {
                    const double sr2 = 1.0 / rsq;
                    const double sr6 = sr2 * sr2 * sr2 * s->sig6[ti + s->type[j]];
                    const double f = 48.0 * sr6 * (sr6 - 0.5) * sr2 * s->eps[ti + s->type[j]];
                    fx = fx + dx * f; fy = fy + dy * f; fz = fz + dz * f;
                    if(pe_out) {
                        pe += 0.5 * 4.0 * s->eps[ti + s->type[j]] * (sr6 * sr6 - sr6);
                        vir += 0.5 * (dx * dx * f + dy * dy * f + dz * dz * f);
                    }
                }
            }
            s->force[i * 3] = s->force[i * 3] + fx;
            s->force[i * 3 + 1] = s->force[i * 3 + 1] + fy;
            s->force[i * 3 + 2] = s->force[i * 3 + 2] + fz;
        }
    } else {
        /* Newton's third law on the half list: the reaction goes to j only when j is
         * local (ghost images carry no force); serial, as the reference's CPU code */
        for(int i = 0; i < nlocal; i++) {
            if(s->flags[i] & FLAG_FIXED) { continue; }
            double fx = 0.0, fy = 0.0, fz = 0.0;
            const double xi = s->pos[i * 3], yi = s->pos[i * 3 + 1], zi = s->pos[i * 3 + 2];
            const int ti = s->type[i] * nt;
            const int *list = s->neighbors + (size_t) i * s->neigh_cap;
            for(int k = 0; k < s->numneighs[i]; k++) {
                const int j = list[k];
                const double dx = xi - s->pos[j * 3], dy = yi - s->pos[j * 3 + 1], dz = zi - s->pos[j * 3 + 2];
                const double rsq = dx * dx + dy * dy + dz * dz;
                if(rsq < s->cutoff2) {
                    const double sr2 = 1.0 / rsq;
                    const double sr6 = sr2 * sr2 * sr2 * s->sig6[ti + s->type[j]];
                    const double f = 48.0 * sr6 * (sr6 - 0.5) * sr2 * s->eps[ti + s->type[j]];
                    const double ex = dx * f, ey = dy * f, ez = dz * f;
                    fx = fx + ex; fy = fy + ey; fz = fz + ez;
                    const double w = (j < nlocal) ? 1.0 : 0.5;
                    if(j < nlocal) {
                        s->force[j * 3] += -ex; s->force[j * 3 + 1] += -ey; s->force[j * 3 + 2] += -ez;
                    }
                    if(pe_out) {
                        pe += w * 4.0 * s->eps[ti + s->type[j]] * (sr6 * sr6 - sr6);
                        vir += w * (dx * dx * f + dy * dy * f + dz * dz * f);
                    }
                }
            }
            s->force[i * 3] = s->force[i * 3] + fx;
            s->force[i * 3 + 1] = s->force[i * 3 + 1] + fy;
            s->force[i * 3 + 2] = s->force[i * 3 + 2] + fz;
        }
    }
    if(pe_out) { *pe_out = pe; }
    if(vir_out) { *vir_out = vir; }
}

static void initial_integrate(lj_sim *s) {
    const double h = s->dt * 0.5;
    #pragma omp parallel for schedule(static) num_threads(s->nthreads)
    for(int i = 0; i < s->nlocal; i++) {
        if(s->flags[i] & FLAG_FIXED) { continue; }
        for(int e = 0; e < 3; e++) { s->vel[i * 3 + e] = s->vel[i * 3 + e] + h * s->force[i * 3 + e] / s->mass[i]; }
        for(int e = 0; e < 3; e++) { s->pos[i * 3 + e] = s->pos[i * 3 + e] + s->dt * s->vel[i * 3 + e]; }
    }
}

static void final_integrate(lj_sim *s) {
    const double h = s->dt * 0.5;
    #pragma omp parallel for schedule(static) num_threads(s->nthreads)
    for(int i = 0; i < s->nlocal; i++) {
        if(s->flags[i] & FLAG_FIXED) { continue; }
        for(int e = 0; e < 3; e++) { s->vel[i * 3 + e] = s->vel[i * 3 + e] + h * s->force[i * 3 + e] / s->mass[i]; }
    }
}

/* One iteration of the reference's time loop.  Returns 0, or the overflow code
 * (1 ghosts, 2 cell, 3 neighbour capacity).  When `energy` is given, the force
 * pass also fills energy[0] = potential energy, energy[1] = virial sum r.F. */
int lj_step(lj_sim *s, double *energy) {
    const int ts = s->ts;
    const int rebuild = ((ts + 1) % s->every == 0) || ts == 0;
    s->overflow = 0;
    if(ts > 0) { initial_integrate(s); }
    if(rebuild) {
        for(int d = 0; d < 3; d++) { exchange_dim(s, d); }
        borders(s);
        if(s->overflow) { return s->overflow; }
        if(!build_cell_lists(s)) { return s->overflow; }
        build_neighbor_lists(s);
        if(s->overflow) { return s->overflow; }
    } else {
        synchronize(s);
    }
    lennard_jones(s, energy ? &energy[0] : NULL, energy ? &energy[1] : NULL);
    if(ts > 0) { final_integrate(s); }
    s->ts++;
    return 0;
}

int lj_run(lj_sim *s, int nsteps) {
    for(int k = 0; k < nsteps; k++) {
        const int rc = lj_step(s, NULL);
        if(rc) { return rc; }
    }
    return 0;
}

/* ---- accessors: locals in uid order (uid values are 0..n-1) */

int lj_nlocal(const lj_sim *s) { return s->nlocal; }
int lj_nghost(const lj_sim *s) { return s->nghost; }
int lj_timestep(const lj_sim *s) { return s->ts; }

void lj_get_state(const lj_sim *s, double *pos, double *vel, double *force) {
    for(int i = 0; i < s->nlocal; i++) {
        const int u = s->uid[i];
        for(int e = 0; e < 3; e++) {
            if(pos) { pos[u * 3 + e] = s->pos[i * 3 + e]; }
            if(vel) { vel[u * 3 + e] = s->vel[i * 3 + e]; }
            if(force) { force[u * 3 + e] = s->force[i * 3 + e]; }
        }
    }
}

double lj_thermo(const lj_sim *s, double *press) {
    return lj_temperature(s->nlocal, s->mass, s->vel, s->len[0], s->len[1], s->len[2], press);
}

/* Number of Verlet entries of the last build. */
long lj_list_size(const lj_sim *s) {
    long tot = 0;
    for(int i = 0; i < s->nlocal; i++) { tot += s->numneighs[i]; }
    return tot;
}

/* Verlet entries as (uid_i, uid_j, sx, sy, sz); sx.. is the periodic image of j.
 * Valid right after a rebuild step, when every ghost position is fresh. */
long lj_list_pairs(const lj_sim *s, int *out, long max_pairs) {
    int *owner = (int *) xcalloc(s->nlocal, sizeof(int));
    for(int i = 0; i < s->nlocal; i++) { owner[s->uid[i]] = i; }
    long k = 0;
    for(int i = 0; i < s->nlocal; i++) {
        const int *list = s->neighbors + (size_t) i * s->neigh_cap;
        for(int q = 0; q < s->numneighs[i] && k < max_pairs; q++) {
            const int j = list[q], o = owner[s->uid[j]];
            out[k * 5 + 0] = s->uid[i];
            out[k * 5 + 1] = s->uid[j];
            for(int e = 0; e < 3; e++) {
                out[k * 5 + 2 + e] = (int) lround((s->pos[j * 3 + e] - s->pos[o * 3 + e]) / s->len[e]);
            }
            k++;
        }
    }
    free(owner);
    return k;
}

/* Occupancy of the reference grid: cell_sizes (locals + ghosts) and the local
 * count per cell, both over ncells; returns ncells. */
int lj_cell_counts(const lj_sim *s, int *sizes, int *local_counts, int max_cells) {
    const int nc = s->ncells < max_cells ? s->ncells : max_cells;
    for(int c = 0; c < nc; c++) { sizes[c] = s->cell_sizes[c]; local_counts[c] = 0; }
    for(int i = 0; i < s->nlocal; i++) {
        const int c = s->particle_cell[i];
        if(c >= 0 && c < nc) { local_counts[c]++; }
    }
    return s->ncells;
}

void lj_grid(const lj_sim *s, int *dims) { for(int d = 0; d < 3; d++) { dims[d] = s->dims[d]; } }
