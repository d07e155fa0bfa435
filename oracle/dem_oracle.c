/*
 * dem_oracle.c -- CPU restatement of the reference's DEM particle path.
 *
 * TEST INFRASTRUCTURE: the oracle the CUDA DEM path is checked against.  The
 * product never links or calls it.
 *
 * It restates, in plain C with the same FP64 operation order, the program the
 * reference's generator emits for its DEM example (examples/dem.py) on one rank:
 *
 *   initial state   runtime/dem_sc_grid.hpp:62-172 (simple-cubic grid, diameters and
 *                   velocities from a default-seeded mt19937 through libstdc++'s
 *                   uniform_real_distribution), half spaces from a CSV
 *                   (runtime/read_from_file.hpp:121-203), setup kernel
 *                   update_mass_and_inertia (examples/dem.py:6-15)
 *   time loop       sim/simulation.py:387-417 with a cell-list-only program: every step
 *                   exchange + borders + cell lists + partition by shape, then
 *                   contact-history usage reset, force/torque reset, gravity
 *                   (examples/dem.py:90-92), linear spring-dashpot contact
 *                   (examples/dem.py:18-74 lowered by sim/interaction.py:234-264),
 *                   explicit Euler with rotation (examples/dem.py:77-87), removal of
 *                   unused contact history (sim/contact_history.py:91-127)
 *   contact history sim/contact_history.py:12-17, mapping/funcs.py:230-265: per
 *                   particle slots keyed by partner uid, created with the property
 *                   defaults on first contact
 *   keyword maths   mapping/keywords.py:34-259 (length, dot, cross, normalized,
 *                   select, min, quaternion ops)
 *
 * The reference packs the contact history of a particle leaving through a periodic
 * face after its slot was refilled by the exchange's compaction
 * (sim/comm.py:101-151 order: remove, then pack contact history), so such a
 * particle can take over its filler's contacts.  `exchange_history_fixed = 0`
 * restates that; 1 moves each particle's own history with it.
 *
 * Build: part of oracle/_build/liboracle.so (oracle/build.py), -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define DF_INFINITE 1
#define DF_FIXED    4
#define DF_GLOBAL   8
#define DSHAPE_SPHERE 0
#define DSHAPE_HALFSPACE 1
#define D_SMALL 0.00001
#define D_PI 3.14159265358979323846      /* M_PI of <math.h> */

/* ------------------------------------------------------------------------- */
/* std::mt19937 and libstdc++'s uniform_real_distribution<double>             */
/* ------------------------------------------------------------------------- */

typedef struct { uint32_t mt[624]; int idx; } mt19937;

static void mt_seed(mt19937 *g, uint32_t s) {
    g->mt[0] = s;
    for(int i = 1; i < 624; i++) {
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t) i;
    }
    g->idx = 624;
}

static uint32_t mt_next(mt19937 *g) {
    if(g->idx >= 624) {
        for(int i = 0; i < 624; i++) {
            const uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
            if(y & 1u) { v ^= 0x9908b0dfu; }
            g->mt[i] = v;
        }
        g->idx = 0;
    }
    uint32_t y = g->mt[g->idx++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

/* generate_canonical<double, 53> over a 32-bit engine: two draws, low word first */
static double mt_canonical(mt19937 *g) {
    const double r = 4294967296.0;
    double sum = 0.0, tmp = 1.0;
    for(int k = 0; k < 2; k++) {
        sum += (double) mt_next(g) * tmp;
        tmp *= r;
    }
    double ret = sum / tmp;
    if(ret >= 1.0) { ret = nextafter(1.0, 0.0); }
    return ret;
}

static double mt_uniform(mt19937 *g, double a, double b) {
    return mt_canonical(g) * (b - a) + a;
}

/* ------------------------------------------------------------------------- */

typedef struct {
    /* configuration */
    double lo[3], hi[3], len[3];
    int pbc[3];
    double spacing;              /* cell size (linkedCellWidth) */
    double dt, pi, kappa, ln_e, tc;
    double kn_fixed;             /* > 0: fixed normal stiffness (see dem_set_normal_stiffness) */
    double rho_p, rho_f, g;
    int ntypes;
    double fs[16], fd[16];       /* friction_static / friction_dynamic feature tables */
    int history_fixed;
    /* particles */
    int cap, nlocal, nghost, ccap;
    int *uid, *type, *flags, *shape;
    double *mass, *radius, *pos, *vel, *angvel, *force, *torque, *normal, *inv_inertia, *rot_mat, *rot_quat;
    /* contact history, slots [i * ccap + k] */
    int *num_contacts, *contact_lists, *contact_used, *is_sticking;
    double *tsd, *ivm;
    /* halo */
    int nsend_all, nsend[6], nrecv[6], send_off[6];
    int *send_map, *send_mult, *exchg_flag, *copy_to;
    /* cells */
    int dims[3], ncells, nstencil, stencil[27], cell_cap;
    int *cell_sizes, *cell_particles, *particle_cell, *nshapes;
    int ts;
    int overflow;
} dem_sim;

static void *dcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s);
    if(!p) { fprintf(stderr, "dem_oracle: out of memory\n"); abort(); }
    return p;
}

void dem_destroy(dem_sim *s) {
    if(!s) { return; }
    void *ptrs[] = {s->uid, s->type, s->flags, s->shape, s->mass, s->radius, s->pos, s->vel, s->angvel,
                    s->force, s->torque, s->normal, s->inv_inertia, s->rot_mat, s->rot_quat,
                    s->num_contacts, s->contact_lists, s->contact_used, s->is_sticking, s->tsd, s->ivm,
                    s->send_map, s->send_mult, s->exchg_flag, s->copy_to, s->cell_sizes,
                    s->cell_particles, s->particle_cell, s->nshapes};
    for(size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) { free(ptrs[k]); }
    free(s);
}

dem_sim *dem_create(int cap, const double *lo, const double *hi, const int *pbc, double spacing, double dt,
                    double pi, double kappa, double ln_e, double tc, double rho_p, double rho_f, double g,
                    int ntypes, const double *fs, const double *fd, int ccap, int history_fixed) {
    dem_sim *s = (dem_sim *) dcalloc(1, sizeof(dem_sim));
    for(int d = 0; d < 3; d++) { s->lo[d] = lo[d]; s->hi[d] = hi[d]; s->len[d] = hi[d] - lo[d]; s->pbc[d] = pbc[d]; }
    s->spacing = spacing; s->dt = dt; s->pi = pi; s->kappa = kappa; s->ln_e = ln_e; s->tc = tc;
    s->rho_p = rho_p; s->rho_f = rho_f; s->g = g; s->ntypes = ntypes;
    for(int k = 0; k < ntypes * ntypes && k < 16; k++) { s->fs[k] = fs[k]; s->fd[k] = fd[k]; }
    s->history_fixed = history_fixed;
    s->cap = cap; s->ccap = ccap;
    s->uid = dcalloc(cap, sizeof(int)); s->type = dcalloc(cap, sizeof(int));
    s->flags = dcalloc(cap, sizeof(int)); s->shape = dcalloc(cap, sizeof(int));
    s->mass = dcalloc(cap, sizeof(double)); s->radius = dcalloc(cap, sizeof(double));
    s->pos = dcalloc((size_t) cap * 3, sizeof(double)); s->vel = dcalloc((size_t) cap * 3, sizeof(double));
    s->angvel = dcalloc((size_t) cap * 3, sizeof(double)); s->force = dcalloc((size_t) cap * 3, sizeof(double));
    s->torque = dcalloc((size_t) cap * 3, sizeof(double)); s->normal = dcalloc((size_t) cap * 3, sizeof(double));
    s->inv_inertia = dcalloc((size_t) cap * 9, sizeof(double)); s->rot_mat = dcalloc((size_t) cap * 9, sizeof(double));
    s->rot_quat = dcalloc((size_t) cap * 4, sizeof(double));
    s->num_contacts = dcalloc(cap, sizeof(int));
    s->contact_lists = dcalloc((size_t) cap * ccap, sizeof(int));
    s->contact_used = dcalloc((size_t) cap * ccap, sizeof(int));
    s->is_sticking = dcalloc((size_t) cap * ccap, sizeof(int));
    s->tsd = dcalloc((size_t) cap * ccap * 3, sizeof(double));
    s->ivm = dcalloc((size_t) cap * ccap, sizeof(double));
    s->send_map = dcalloc(cap, sizeof(int)); s->send_mult = dcalloc((size_t) cap * 3, sizeof(int));
    s->exchg_flag = dcalloc(cap, sizeof(int)); s->copy_to = dcalloc(cap, sizeof(int));
    s->particle_cell = dcalloc(cap, sizeof(int));
    s->ncells = 1;
    for(int d = 0; d < 3; d++) {
        const double dmax = s->hi[d] + spacing, dmin = s->lo[d] - spacing;
        s->dims[d] = (int) ceil((dmax - dmin) / spacing) + 1;
        s->ncells *= s->dims[d];
    }
    s->ncells += 1;
    s->nstencil = 0;
    for(int a = -1; a < 2; a++) {
        for(int b = -1; b < 2; b++) {
            for(int c = -1; c < 2; c++) { s->stencil[s->nstencil++] = (a * s->dims[1] + b) * s->dims[2] + c; }
        }
    }
    s->cell_cap = 64;
    s->cell_sizes = dcalloc(s->ncells, sizeof(int));
    s->nshapes = dcalloc((size_t) s->ncells * 2, sizeof(int));
    s->cell_particles = dcalloc((size_t) s->ncells * s->cell_cap, sizeof(int));
    return s;
}

/* Fixed normal stiffness (the batched DEM workload's contact model: k_n given
 * directly instead of through the collision time; 0 restores the example's model). */
void dem_set_normal_stiffness(dem_sim *s, double kn) { s->kn_fixed = kn; }

/* ---- initial state ---------------------------------------------------------- */

/* dem_sc_grid: returns the number of spheres written at [start, ...).  Uses the
 * default-seeded engine the reference keeps as a static, and rand() for types. */
int dem_sc_grid(dem_sim *s, double xmax, double ymax, double zmax, double spacing, double diameter,
                double min_d, double max_d, double v0, double density, int ntypes) {
    mt19937 g;
    mt_seed(&g, 5489u);
    srand(1);
    int last_uid = 1, n = s->nlocal;
    const double gen[6] = {0.0, 0.0, diameter, xmax, ymax, zmax};
    const double ref[3] = {spacing * 0.5, spacing * 0.5, spacing * 0.5};
    const int iret = (int) ceil((0.0 - ref[0]) / spacing);
    const int jret = (int) ceil((0.0 - ref[1]) / spacing);
    const int kret = (int) ceil((diameter - ref[2]) / spacing);
    int i = iret, j = jret, k = kret;
    double pt[3] = {ref[0] + i * spacing, ref[1] + j * spacing, ref[2] + k * spacing};
#define INSIDE(p) ((p)[0] >= gen[0] && (p)[0] < gen[3] && (p)[1] >= gen[1] && (p)[1] < gen[4] && (p)[2] >= gen[2] && (p)[2] < gen[5])
    while(INSIDE(pt)) {
        const double d = mt_uniform(&g, min_d, max_d);
        const int in = pt[0] >= s->lo[0] && pt[0] < s->hi[0] - D_SMALL && pt[1] >= s->lo[1] &&
                       pt[1] < s->hi[1] - D_SMALL && pt[2] >= s->lo[2] && pt[2] < s->hi[2] - D_SMALL;
        if(in && n < s->cap) {
            const double rad = d * 0.5;
            s->uid[n] = last_uid;
            s->radius[n] = rad;
            s->mass[n] = ((4.0 / 3.0) * D_PI) * rad * rad * rad * density;
            for(int e = 0; e < 3; e++) { s->pos[n * 3 + e] = pt[e]; }
            s->vel[n * 3 + 0] = 0.1 * mt_uniform(&g, -v0, v0);
            s->vel[n * 3 + 1] = 0.1 * mt_uniform(&g, -v0, v0);
            s->vel[n * 3 + 2] = -v0;
            s->type[n] = rand() % ntypes;
            s->flags[n] = 0;
            s->shape[n] = DSHAPE_SPHERE;
            n++;
        }
        ++i;
        pt[0] = ref[0] + i * spacing; pt[1] = ref[1] + j * spacing; pt[2] = ref[2] + k * spacing;
        if(!INSIDE(pt)) {
            i = iret; j++;
            pt[0] = ref[0] + i * spacing; pt[1] = ref[1] + j * spacing; pt[2] = ref[2] + k * spacing;
            if(!INSIDE(pt)) {
                j = jret; k++;
                pt[0] = ref[0] + i * spacing; pt[1] = ref[1] + j * spacing; pt[2] = ref[2] + k * spacing;
                if(!INSIDE(pt)) { break; }
            }
        }
        last_uid++;
    }
#undef INSIDE
    const int added = n - s->nlocal;
    s->nlocal = n;
    return added;
}

/* Append one particle (after the grid, e.g. half spaces read from CSV). */
void dem_add_particle(dem_sim *s, int uid, int type, double mass, double radius, const double *pos,
                      const double *vel, const double *normal, int flags, int shape) {
    const int n = s->nlocal++;
    s->uid[n] = uid; s->type[n] = type; s->mass[n] = mass; s->radius[n] = radius;
    s->flags[n] = flags; s->shape[n] = shape;
    for(int e = 0; e < 3; e++) {
        s->pos[n * 3 + e] = pos[e]; s->vel[n * 3 + e] = vel ? vel[e] : 0.0;
        s->normal[n * 3 + e] = normal ? normal[e] : 0.0; s->angvel[n * 3 + e] = 0.0;
    }
}

/* update_mass_and_inertia (examples/dem.py:6-15) with keywords.py:129-146 inversed() */
void dem_setup(dem_sim *s) {
    for(int i = 0; i < s->nlocal; i++) {
        double *R = s->rot_mat + i * 9, *Q = s->rot_quat + i * 4, *I = s->inv_inertia + i * 9;
        for(int e = 0; e < 9; e++) { R[e] = (e % 4 == 0) ? 1.0 : 0.0; }
        Q[0] = 1.0; Q[1] = 0.0; Q[2] = 0.0; Q[3] = 0.0;
        if(s->shape[i] == DSHAPE_SPHERE) {
            const double v = 0.4 * s->mass[i] * s->radius[i] * s->radius[i];
            double m[9];
            for(int e = 0; e < 9; e++) { m[e] = (e % 4 == 0) ? v : 0.0; }
            const double det = m[0] * ((m[4] * m[8]) - (m[7] * m[5])) + m[1] * ((m[5] * m[6]) - (m[8] * m[3])) +
                               m[2] * ((m[3] * m[7]) - (m[4] * m[6]));
            const double id = 1.0 / det;
            I[0] = id * ((m[4] * m[8]) - (m[5] * m[7]));
            I[1] = id * ((m[7] * m[2]) - (m[8] * m[1]));
            I[2] = id * ((m[1] * m[5]) - (m[2] * m[4]));
            I[3] = id * ((m[5] * m[6]) - (m[3] * m[8]));
            I[4] = id * ((m[8] * m[0]) - (m[6] * m[2]));
            I[5] = id * ((m[2] * m[3]) - (m[0] * m[5]));
            I[6] = id * ((m[3] * m[7]) - (m[4] * m[6]));
            I[7] = id * ((m[6] * m[1]) - (m[7] * m[0]));
            I[8] = id * ((m[0] * m[4]) - (m[1] * m[3]));
        } else {
            s->mass[i] = INFINITY;
            for(int e = 0; e < 9; e++) { I[e] = 0.0; }
        }
    }
}

/* ---- halo ------------------------------------------------------------------- */

static void copy_particle(dem_sim *s, int dst, int src, int with_history) {
    s->uid[dst] = s->uid[src]; s->shape[dst] = s->shape[src]; s->flags[dst] = s->flags[src];
    s->mass[dst] = s->mass[src]; s->radius[dst] = s->radius[src]; s->type[dst] = s->type[src];
    memcpy(s->pos + dst * 3, s->pos + src * 3, 3 * sizeof(double));
    memcpy(s->vel + dst * 3, s->vel + src * 3, 3 * sizeof(double));
    memcpy(s->angvel + dst * 3, s->angvel + src * 3, 3 * sizeof(double));
    memcpy(s->normal + dst * 3, s->normal + src * 3, 3 * sizeof(double));
    memcpy(s->inv_inertia + dst * 9, s->inv_inertia + src * 9, 9 * sizeof(double));
    memcpy(s->rot_mat + dst * 9, s->rot_mat + src * 9, 9 * sizeof(double));
    memcpy(s->rot_quat + dst * 4, s->rot_quat + src * 4, 4 * sizeof(double));
    if(with_history) {
        const int nc = s->num_contacts[src];
        for(int k = 0; k < nc; k++) {
            const size_t a = (size_t) dst * s->ccap + k, b = (size_t) src * s->ccap + k;
            s->contact_lists[a] = s->contact_lists[b]; s->contact_used[a] = s->contact_used[b];
            s->is_sticking[a] = s->is_sticking[b]; s->ivm[a] = s->ivm[b];
            memcpy(s->tsd + a * 3, s->tsd + b * 3, 3 * sizeof(double));
        }
        s->num_contacts[dst] = nc;
    }
}

typedef struct {          /* staged copy of a sent particle */
    int uid, shape, flags, type, nc;
    double mass, radius, pos[3], vel[3], angvel[3], normal[3], ii[9], rm[9], rq[4];
    int *cl, *st;
    double *tsd, *ivm;
} staged_t;

static void stage(dem_sim *s, staged_t *b, int m, const int *mult) {
    b->uid = s->uid[m]; b->shape = s->shape[m]; b->flags = s->flags[m]; b->type = s->type[m];
    b->mass = s->mass[m]; b->radius = s->radius[m];
    for(int e = 0; e < 3; e++) {
        b->pos[e] = s->pos[m * 3 + e] + mult[e] * s->len[e];
        b->vel[e] = s->vel[m * 3 + e]; b->angvel[e] = s->angvel[m * 3 + e]; b->normal[e] = s->normal[m * 3 + e];
    }
    memcpy(b->ii, s->inv_inertia + m * 9, sizeof(b->ii));
    memcpy(b->rm, s->rot_mat + m * 9, sizeof(b->rm));
    memcpy(b->rq, s->rot_quat + m * 4, sizeof(b->rq));
}

static void stage_history(dem_sim *s, staged_t *b, int m) {
    b->nc = s->num_contacts[m];
    b->cl = dcalloc(s->ccap, sizeof(int)); b->st = dcalloc(s->ccap, sizeof(int));
    b->tsd = dcalloc((size_t) s->ccap * 3, sizeof(double)); b->ivm = dcalloc(s->ccap, sizeof(double));
    for(int k = 0; k < b->nc; k++) {
        const size_t a = (size_t) m * s->ccap + k;
        b->cl[k] = s->contact_lists[a]; b->st[k] = s->is_sticking[a]; b->ivm[k] = s->ivm[a];
        memcpy(b->tsd + k * 3, s->tsd + a * 3, 3 * sizeof(double));
    }
}

static void unstage(dem_sim *s, const staged_t *b, int t, int with_history) {
    s->uid[t] = b->uid; s->shape[t] = b->shape; s->flags[t] = b->flags; s->type[t] = b->type;
    s->mass[t] = b->mass; s->radius[t] = b->radius;
    memcpy(s->pos + t * 3, b->pos, sizeof(b->pos)); memcpy(s->vel + t * 3, b->vel, sizeof(b->vel));
    memcpy(s->angvel + t * 3, b->angvel, sizeof(b->angvel)); memcpy(s->normal + t * 3, b->normal, sizeof(b->normal));
    memcpy(s->inv_inertia + t * 9, b->ii, sizeof(b->ii)); memcpy(s->rot_mat + t * 9, b->rm, sizeof(b->rm));
    memcpy(s->rot_quat + t * 4, b->rq, sizeof(b->rq));
    if(with_history) {
        s->num_contacts[t] = b->nc;
        for(int k = 0; k < b->nc; k++) {
            const size_t a = (size_t) t * s->ccap + k;
            s->contact_lists[a] = b->cl[k]; s->contact_used[a] = 1;
            s->is_sticking[a] = b->st[k]; s->ivm[a] = b->ivm[k];
            memcpy(s->tsd + a * 3, b->tsd + k * 3, 3 * sizeof(double));
        }
    }
}

static void free_staged(staged_t *b, int n) {
    for(int k = 0; k < n; k++) { free(b[k].cl); free(b[k].st); free(b[k].tsd); free(b[k].ivm); }
    free(b);
}

static void exchange_dim(dem_sim *s, int d) {
    if(!s->pbc[d]) {
        /* a non-periodic dimension never sends on a single rank (pbc flag != 0) */
        return;
    }
    s->nsend_all = 0; s->nghost = 0;
    for(int i = 0; i < s->nlocal; i++) { s->exchg_flag[i] = 0; }
    int cnt = 0;
    for(int side = 0; side < 2; side++) {
        for(int i = 0; i < s->nlocal; i++) {
            if(s->flags[i] & (DF_INFINITE | DF_GLOBAL)) { continue; }
            const double x = s->pos[i * 3 + d];
            if(side == 0 ? (x < s->lo[d]) : (x > s->hi[d])) {
                const int k = s->nsend_all++;
                s->send_map[k] = i; s->exchg_flag[i] = 1;
                for(int e = 0; e < 3; e++) { s->send_mult[k * 3 + e] = (e == d) ? (side == 0 ? 1 : -1) : 0; }
                cnt++;
            }
        }
    }
    staged_t *buf = dcalloc(cnt > 0 ? cnt : 1, sizeof(staged_t));
    for(int k = 0; k < cnt; k++) {
        stage(s, &buf[k], s->send_map[k], s->send_mult + k * 3);
        if(s->history_fixed) { stage_history(s, &buf[k], s->send_map[k]); }
    }
    int send_pos = s->nlocal - 1;
    for(int k = 0; k < s->nsend_all; k++) {
        if(s->send_map[k] < s->nlocal - s->nsend_all) {
            while(s->exchg_flag[send_pos] == 1) { send_pos--; }
            s->copy_to[k] = send_pos; send_pos--;
        } else {
            s->copy_to[k] = -1;
        }
    }
    for(int k = 0; k < s->nsend_all; k++) {
        if(s->copy_to[k] > 0) { copy_particle(s, s->send_map[k], s->copy_to[k], 1); }
    }
    s->nlocal -= s->nsend_all;
    if(!s->history_fixed) {
        /* the reference reads the sent particles' histories after the compaction */
        for(int k = 0; k < cnt; k++) { stage_history(s, &buf[k], s->send_map[k]); }
    }
    for(int k = 0; k < cnt; k++) { unstage(s, &buf[k], s->nlocal + k, 1); }
    s->nlocal += cnt;
    free_staged(buf, cnt);
}

static int borders(dem_sim *s) {
    s->nsend_all = 0; s->nghost = 0;
    for(int d = 0; d < 3; d++) {
        if(!s->pbc[d]) { continue; }
        const int n = s->nlocal + s->nghost;
        int start = s->nsend_all;
        for(int side = 0; side < 2; side++) {
            for(int i = 0; i < n; i++) {
                if(s->flags[i] & (DF_INFINITE | DF_GLOBAL)) { continue; }
                const double x = s->pos[i * 3 + d];
                if(side == 0 ? (x < s->lo[d] + s->spacing) : (x > s->hi[d] - s->spacing)) {
                    if(s->nlocal + s->nghost + (s->nsend_all - start) + 1 > s->cap) { s->overflow = 1; return 0; }
                    const int k = s->nsend_all++;
                    s->send_map[k] = i;
                    for(int e = 0; e < 3; e++) { s->send_mult[k * 3 + e] = (e == d) ? (side == 0 ? 1 : -1) : 0; }
                }
            }
        }
        const int cnt = s->nsend_all - start;
        staged_t *buf = dcalloc(cnt > 0 ? cnt : 1, sizeof(staged_t));
        for(int k = 0; k < cnt; k++) { stage(s, &buf[k], s->send_map[start + k], s->send_mult + (start + k) * 3); }
        for(int k = 0; k < cnt; k++) {
            const int t = s->nlocal + start + k;
            /* ghosts carry uid, type, mass, radius, position, velocities, shape */
            s->uid[t] = buf[k].uid; s->type[t] = buf[k].type; s->mass[t] = buf[k].mass; s->radius[t] = buf[k].radius;
            s->shape[t] = buf[k].shape; s->flags[t] = 0;
            memcpy(s->pos + t * 3, buf[k].pos, 3 * sizeof(double));
            memcpy(s->vel + t * 3, buf[k].vel, 3 * sizeof(double));
            memcpy(s->angvel + t * 3, buf[k].angvel, 3 * sizeof(double));
        }
        free_staged(buf, cnt);
        s->nghost += cnt;
    }
    return 1;
}

/* ---- cells (sim/cell_lists.py:90-171 with two shapes) ------------------------ */

static int build_cells(dem_sim *s) {
    for(int c = 0; c < s->ncells; c++) { s->cell_sizes[c] = 0; }
    const int n = s->nlocal + s->nghost;
    for(int i = 0; i < n; i++) {
        int flat = 0;
        if(!(s->flags[i] & DF_INFINITE)) {
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
    /* partition each cell by shape: spheres (shape id 0) then half spaces (1) */
    for(int c = 0; c < s->ncells; c++) {
        int start = 0, end = 0;
        int *cp = s->cell_particles + (size_t) c * s->cell_cap;
        for(int sh = 0; sh < 2; sh++) {
            const int shape_start = start;
            end = s->cell_sizes[c] - 1;
            s->nshapes[c * 2 + sh] = 0;
            while(start <= end) {
                const int p = cp[start];
                if(s->shape[p] != sh) {
                    if(start != end) { cp[start] = cp[end]; cp[end] = p; }
                    end--;
                } else {
                    start++;
                    s->nshapes[c * 2 + sh] = start - shape_start;
                }
            }
        }
    }
    return 1;
}

/* ---- contact force ------------------------------------------------------------ */

static int contact_slot(dem_sim *s, int i, int uj) {
    int id = -1;
    const int nc = s->num_contacts[i];
    for(int k = 0; k < nc; k++) { if(s->contact_lists[(size_t) i * s->ccap + k] == uj) { id = k; } }
    if(id == -1) {
        id = nc;
        if(nc >= s->ccap) { s->overflow = 3; return -1; }
        s->num_contacts[i] = nc + 1;
        const size_t a = (size_t) i * s->ccap + nc;
        s->contact_lists[a] = uj;
        s->is_sticking[a] = 0;
        s->tsd[a * 3 + 0] = 0.0; s->tsd[a * 3 + 1] = 0.0; s->tsd[a * 3 + 2] = 0.0;
        s->ivm[a] = 0.0;
    }
    s->contact_used[(size_t) i * s->ccap + id] = 1;
    return id;
}

/* The shared part of examples/dem.py:18-74 once the contact geometry is known.
 * n = contact normal, cp = contact point, delta = -penetration depth. */
static void spring_dashpot(dem_sim *s, int i, int j, int cid, const double *n, const double *cp, double delta,
                           double inv_mi, double *facc, double *tacc) {
    const double *xi = s->pos + i * 3, *xj = s->pos + j * 3;
    const double *vi = s->vel + i * 3, *vj = s->vel + j * 3;
    const double *wi = s->angvel + i * 3, *wj = s->angvel + j * 3;
    const size_t a = (size_t) i * s->ccap + cid;
    const int sticking = s->is_sticking[a];
    double ri[3], rj[3], vwi[3], vwj[3], rel[3], reln[3], relt[3];
    for(int e = 0; e < 3; e++) { ri[e] = cp[e] - xi[e]; rj[e] = cp[e] - xj[e]; }
    vwi[0] = vi[0] + (wi[1] * ri[2] - wi[2] * ri[1]);
    vwi[1] = vi[1] + (wi[2] * ri[0] - wi[0] * ri[2]);
    vwi[2] = vi[2] + (wi[0] * ri[1] - wi[1] * ri[0]);
    vwj[0] = vj[0] + (wj[1] * rj[2] - wj[2] * rj[1]);
    vwj[1] = vj[1] + (wj[2] * rj[0] - wj[0] * rj[2]);
    vwj[2] = vj[2] + (wj[0] * rj[1] - wj[1] * rj[0]);
    for(int e = 0; e < 3; e++) { rel[e] = -(vwi[e] - vwj[e]); }
    const double vn = rel[0] * n[0] + rel[1] * n[1] + rel[2] * n[2];
    for(int e = 0; e < 3; e++) { reln[e] = vn * n[e]; relt[e] = rel[e] - reln[e]; }
    const double lrt = sqrt(relt[0] * relt[0] + relt[1] * relt[1] + relt[2] * relt[2]);
    const int cond1a = (sticking == 1) && (lrt < 1e-08);
    const double meff = 1.0 / (inv_mi + (1.0 / s->mass[j]));
    double kn;
    if(s->kn_fixed > 0.0) {
        kn = s->kn_fixed;
    } else {
        kn = (meff * ((s->pi * s->pi) + (s->ln_e * s->ln_e))) / (s->tc * s->tc);
    }
    const double kt = s->kappa * kn;
    double tsd0[3], rot[3], sel1[3], nts[3], fTLS[3], fN[3], t[3];
    for(int e = 0; e < 3; e++) { tsd0[e] = s->tsd[a * 3 + e]; }
    const double proj = tsd0[0] * n[0] + tsd0[1] * n[1] + tsd0[2] * n[2];
    for(int e = 0; e < 3; e++) { rot[e] = tsd0[e] - n[e] * proj; }
    const double rl2 = rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2];
    const double tl2 = tsd0[0] * tsd0[0] + tsd0[1] * tsd0[1] + tsd0[2] * tsd0[2];
    const double sc = sqrt(tl2 / rl2);
    for(int e = 0; e < 3; e++) {
        sel1[e] = (rl2 <= 0.0) ? 0.0 : rot[e] * sc;
        nts[e] = s->dt * relt[e] + sel1[e];
    }
    /* normal damping: from the collision time (examples/dem.py:26), or with a fixed
     * stiffness the same restitution relation solved for the damping,
     * -2 ln(e) sqrt(meff kn) / sqrt(pi^2 + ln(e)^2) */
    const double dn = s->kn_fixed > 0.0
        ? (((-(2.0)) * s->ln_e) * sqrt(meff * kn)) / sqrt((s->pi * s->pi) + (s->ln_e * s->ln_e))
        : ((-(2.0)) * meff) * s->ln_e / s->tc;
    const double dtn = sqrt(s->kappa) * dn;
    for(int e = 0; e < 3; e++) { fTLS[e] = kt * nts[e] + dtn * relt[e]; }
    const double fTLS_len = sqrt(fTLS[0] * fTLS[0] + fTLS[1] * fTLS[1] + fTLS[2] * fTLS[2]);
    const int tij = s->type[i] * s->ntypes + s->type[j];
    const double kd = kn * delta;
    for(int e = 0; e < 3; e++) { fN[e] = kd * n[e] + dn * reln[e]; }
    const double fNl = sqrt(fN[0] * fN[0] + fN[1] * fN[1] + fN[2] * fN[2]);
    const double fstat = s->fs[tij] * fNl;
    const int cond1 = cond1a && (fTLS_len < fstat);
    const double fdyn = s->fd[tij] * fNl;
    const int cond2 = (sticking == 1) && (fTLS_len < fdyn);
    const int c340 = (!cond1 && !cond2) && (kt > 0.0);
    const double ffa = cond1 ? fstat : fdyn;
    const double tl = sqrt(fTLS[0] * fTLS[0] + fTLS[1] * fTLS[1] + fTLS[2] * fTLS[2]);
    const double itl = 1.0 / tl;
    for(int e = 0; e < 3; e++) { t[e] = (tl > 0.0) ? fTLS[e] * itl : 0.0; }
    for(int e = 0; e < 3; e++) {
        const double v = ((ffa * t[e]) - (dtn * relt[e])) / kt;
        s->tsd[a * 3 + e] = c340 ? v : nts[e];
    }
    const double ivm0 = s->ivm[a];
    const double lrel = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2]);
    s->ivm[a] = (ivm0 > 0.0) ? ivm0 : lrel;
    s->is_sticking[a] = ((cond1 || cond2) || (fTLS_len < fdyn)) ? 1 : 0;
    const double fTabs = (ffa < fTLS_len) ? ffa : fTLS_len;
    double pf[3];
    for(int e = 0; e < 3; e++) { pf[e] = fN[e] + fTabs * t[e]; facc[e] = facc[e] + pf[e]; }
    const double c0 = (cp[1] - xi[1]) * pf[2] - (cp[2] - xi[2]) * pf[1];
    const double c1 = (cp[2] - xi[2]) * pf[0] - (cp[0] - xi[0]) * pf[2];
    const double c2 = (cp[0] - xi[0]) * pf[1] - (cp[1] - xi[1]) * pf[0];
    tacc[0] = tacc[0] + c0; tacc[1] = tacc[1] + c1; tacc[2] = tacc[2] + c2;
}

static void contact_forces(dem_sim *s) {
    for(int i = 0; i < s->nlocal; i++) {
        if(s->flags[i] & DF_FIXED) { continue; }
        double ts_[3] = {0, 0, 0}, fs_[3] = {0, 0, 0}, th[3] = {0, 0, 0}, fh[3] = {0, 0, 0};
        const double *xi = s->pos + i * 3;
        const double ri = s->radius[i];
        const double inv_mi = 1.0 / s->mass[i];
        const int ci = s->particle_cell[i];
        for(int sh = 0; sh < 2; sh++) {
            for(int disp = -1; disp < s->nstencil; disp++) {
                const int nc = (disp < 0) ? 0 : ci + s->stencil[disp];
                if(!(disp < 0 || (nc > 0 && nc < s->ncells))) { continue; }
                const int b = sh == 0 ? 0 : s->nshapes[nc * 2];
                const int e_ = b + s->nshapes[nc * 2 + sh];
                const int *cp_ = s->cell_particles + (size_t) nc * s->cell_cap;
                for(int k = b; k < e_; k++) {
                    const int j = cp_[k];
                    if(j == i) { continue; }
                    const double *xj = s->pos + j * 3;
                    double n[3], cp[3], delta;
                    if(sh == 0) {
                        const double d0 = xi[0] - xj[0], d1 = xi[1] - xj[1], d2 = xi[2] - xj[2];
                        const double rsq = d0 * d0 + d1 * d1 + d2 * d2;
                        const double sep = ri + s->radius[j];
                        if(!(rsq < sep * (sep + 0.0))) { continue; }
                        const double dist = sqrt(rsq);
                        const double pd = (dist - ri) - s->radius[j];
                        delta = -pd;
                        if(delta < 0.0) { continue; }
                        const double inv = 1.0 / dist;
                        n[0] = d0 * inv; n[1] = d1 * inv; n[2] = d2 * inv;
                        const double kk = s->radius[j] + 0.5 * pd;
                        for(int e = 0; e < 3; e++) { cp[e] = xj[e] + n[e] * kk; }
                    } else {
                        const double *nj = s->normal + j * 3;
                        const double kx = (nj[0] * xi[0] + nj[1] * xi[1]) + nj[2] * xi[2];
                        const double dd = (nj[0] * xj[0] + nj[1] * xj[1]) + nj[2] * xj[2];
                        const double pd = (kx - ri) - dd;
                        if(!(pd < 0.0)) { continue; }
                        delta = -pd;
                        if(delta < 0.0) { continue; }
                        const double tmp = ri + pd;
                        for(int e = 0; e < 3; e++) { n[e] = nj[e]; cp[e] = xi[e] - tmp * nj[e]; }
                    }
                    const int cid = contact_slot(s, i, s->uid[j]);
                    if(cid < 0) { return; }
                    spring_dashpot(s, i, j, cid, n, cp, delta, inv_mi, sh == 0 ? fs_ : fh, sh == 0 ? ts_ : th);
                }
            }
        }
        for(int e = 0; e < 3; e++) {
            s->torque[i * 3 + e] = s->torque[i * 3 + e] + (ts_[e] + th[e]);
            s->force[i * 3 + e] = s->force[i * 3 + e] + (fs_[e] + fh[e]);
        }
    }
}

static void gravity(dem_sim *s) {
    const double drho = (double) (int) (s->rho_p - s->rho_f);
    for(int i = 0; i < s->nlocal; i++) {
        if(s->flags[i] & DF_FIXED) { continue; }
        const double r = s->radius[i];
        const double vol = (((4.0 / 3.0) * s->pi) * r) * r * r;
        s->force[i * 3 + 2] = s->force[i * 3 + 2] - (drho * vol) * s->g;
    }
}

static void euler(dem_sim *s) {
    const double dt = s->dt;
    for(int i = 0; i < s->nlocal; i++) {
        if(s->flags[i] & DF_FIXED) { continue; }
        double *x = s->pos + i * 3, *v = s->vel + i * 3, *w = s->angvel + i * 3;
        const double *F = s->force + i * 3, *T = s->torque + i * 3;
        double *R = s->rot_mat + i * 9, *Q = s->rot_quat + i * 4;
        const double *Ii = s->inv_inertia + i * 9;
        const double im = 1.0 / s->mass[i];
        const double h = 0.5 * im;
        for(int e = 0; e < 3; e++) { x[e] = x[e] + (((h * F[e]) * dt) * dt + v[e] * dt); }
        for(int e = 0; e < 3; e++) { v[e] = v[e] + (im * F[e]) * dt; }
        double a[3], b[3], wd[3], phi[3];
        for(int r = 0; r < 3; r++) { a[r] = (Ii[r * 3] * T[0] + Ii[r * 3 + 1] * T[1]) + Ii[r * 3 + 2] * T[2]; }
        for(int r = 0; r < 3; r++) { b[r] = (R[r * 3] * a[0] + R[r * 3 + 1] * a[1]) + R[r * 3 + 2] * a[2]; }
        /* vector * transposed(R) (keywords.py:185-189 with the transpose of :117-123):
         * component c = b0 R[c] + b1 R[c+3] + b2 R[c+6] */
        for(int c = 0; c < 3; c++) { wd[c] = (b[0] * R[c] + b[1] * R[c + 3]) + b[2] * R[c + 6]; }
        for(int e = 0; e < 3; e++) { phi[e] = w[e] * dt + ((0.5 * wd[e]) * dt) * dt; }
        const double lp = sqrt(phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2]);
        double q[4];
        if(fabs(lp) < 1e-06) {
            q[0] = 1.0; q[1] = 0.0; q[2] = 0.0; q[3] = 0.0;
        } else {
            const double ca = cos(lp * 0.5), sa = sin(lp * 0.5), il = 1.0 / lp;
            q[0] = ca; q[1] = sa * (phi[0] * il); q[2] = sa * (phi[1] * il); q[3] = sa * (phi[2] * il);
        }
        const double p0 = Q[0], p1 = Q[1], p2 = Q[2], p3 = Q[3];
        const double r_ = ((q[0] * p0 - q[1] * p1) - q[2] * p2) - q[3] * p3;
        const double i_ = ((q[0] * p1 + q[1] * p0) + q[2] * p3) - q[3] * p2;
        const double j_ = ((q[0] * p2 + q[2] * p0) + q[3] * p1) - q[1] * p3;
        const double k_ = ((q[0] * p3 + q[3] * p0) + q[1] * p2) - q[2] * p1;
        const double len2 = ((r_ * r_ + i_ * i_) + j_ * j_) + k_ * k_;
        const double il2 = (fabs(len2 - 1.0) < 1e-08) ? 1.0 : 1.0 / sqrt(len2);
        Q[0] = r_ * il2; Q[1] = i_ * il2; Q[2] = j_ * il2; Q[3] = k_ * il2;
        R[0] = (1.0 - 2.0 * Q[2] * Q[2]) - 2.0 * Q[3] * Q[3];
        R[1] = 2.0 * (Q[1] * Q[2] - Q[0] * Q[3]);
        R[2] = 2.0 * (Q[1] * Q[3] + Q[0] * Q[2]);
        R[3] = 2.0 * (Q[1] * Q[2] + Q[0] * Q[3]);
        R[4] = (1.0 - 2.0 * Q[1] * Q[1]) - 2.0 * Q[3] * Q[3];
        R[5] = 2.0 * (Q[2] * Q[3] - Q[0] * Q[1]);
        R[6] = 2.0 * (Q[1] * Q[3] - Q[0] * Q[2]);
        R[7] = 2.0 * (Q[2] * Q[3] + Q[0] * Q[1]);
        R[8] = (1.0 - 2.0 * Q[1] * Q[1]) - 2.0 * Q[2] * Q[2];
        for(int e = 0; e < 3; e++) { w[e] = w[e] + wd[e] * dt; }
    }
}

static void clear_unused(dem_sim *s) {
    for(int i = 0; i < s->nlocal; i++) {
        int c = 0;
        while(c < s->num_contacts[i]) {
            const size_t a = (size_t) i * s->ccap + c;
            if(s->contact_used[a] == 0) {
                const int last = s->num_contacts[i] - 1;
                if(last > 0) {
                    const size_t b = (size_t) i * s->ccap + last;
                    s->is_sticking[a] = s->is_sticking[b];
                    memcpy(s->tsd + a * 3, s->tsd + b * 3, 3 * sizeof(double));
                    s->ivm[a] = s->ivm[b];
                    s->contact_lists[a] = s->contact_lists[b];
                    s->contact_used[a] = s->contact_used[b];
                }
                s->num_contacts[i] = s->num_contacts[i] - 1;
            } else {
                c++;
            }
        }
    }
}

int dem_step(dem_sim *s) {
    s->overflow = 0;
    for(int d = 0; d < 3; d++) { exchange_dim(s, d); }
    if(!borders(s)) { return s->overflow; }
    if(!build_cells(s)) { return s->overflow; }
    for(int i = 0; i < s->nlocal; i++) {
        for(int c = 0; c < s->num_contacts[i]; c++) { s->contact_used[(size_t) i * s->ccap + c] = 0; }
    }
    for(int i = 0; i < s->nlocal; i++) {
        for(int e = 0; e < 3; e++) { s->force[i * 3 + e] = 0.0; s->torque[i * 3 + e] = 0.0; }
    }
    gravity(s);
    contact_forces(s);
    if(s->overflow) { return s->overflow; }
    euler(s);
    clear_unused(s);
    s->ts++;
    return 0;
}

int dem_nlocal(const dem_sim *s) { return s->nlocal; }

/* State of the spheres and walls ordered by uid (uids need not be dense: the caller
 * passes the sorted uid list it wants). out_* may be NULL. */
void dem_get(const dem_sim *s, int n, const int *uids, double *pos, double *vel, double *angvel, double *force,
             double *torque, double *quat, int *ncontacts) {
    for(int q = 0; q < n; q++) {
        int i = -1;
        for(int k = 0; k < s->nlocal; k++) { if(s->uid[k] == uids[q]) { i = k; break; } }
        if(i < 0) { continue; }
        for(int e = 0; e < 3; e++) {
            if(pos) { pos[q * 3 + e] = s->pos[i * 3 + e]; }
            if(vel) { vel[q * 3 + e] = s->vel[i * 3 + e]; }
            if(angvel) { angvel[q * 3 + e] = s->angvel[i * 3 + e]; }
            if(force) { force[q * 3 + e] = s->force[i * 3 + e]; }
            if(torque) { torque[q * 3 + e] = s->torque[i * 3 + e]; }
        }
        if(quat) { for(int e = 0; e < 4; e++) { quat[q * 4 + e] = s->rot_quat[i * 4 + e]; } }
        if(ncontacts) { ncontacts[q] = s->num_contacts[i]; }
    }
}

/* Raw arrays of local particle k (creation-ordered readback of the initial state). */
void dem_get_initial(const dem_sim *s, int *uid, int *type, int *flags, int *shape, double *mass, double *radius,
                     double *pos, double *vel, double *normal) {
    for(int k = 0; k < s->nlocal; k++) {
        uid[k] = s->uid[k]; type[k] = s->type[k]; flags[k] = s->flags[k]; shape[k] = s->shape[k];
        mass[k] = s->mass[k]; radius[k] = s->radius[k];
        for(int e = 0; e < 3; e++) {
            pos[k * 3 + e] = s->pos[k * 3 + e]; vel[k * 3 + e] = s->vel[k * 3 + e];
            normal[k * 3 + e] = s->normal[k * 3 + e];
        }
    }
}

/* Contact records (uid_i, uid_j, sticking) and (tsd[3], ivm) of every local particle. */
long dem_contacts(const dem_sim *s, int *ids, double *vals, long max) {
    long m = 0;
    for(int i = 0; i < s->nlocal; i++) {
        for(int k = 0; k < s->num_contacts[i] && m < max; k++) {
            const size_t a = (size_t) i * s->ccap + k;
            ids[m * 3 + 0] = s->uid[i]; ids[m * 3 + 1] = s->contact_lists[a]; ids[m * 3 + 2] = s->is_sticking[a];
            vals[m * 4 + 0] = s->tsd[a * 3]; vals[m * 4 + 1] = s->tsd[a * 3 + 1]; vals[m * 4 + 2] = s->tsd[a * 3 + 2];
            vals[m * 4 + 3] = s->ivm[a];
            m++;
        }
    }
    return m;
}
