/*
 * pairs_gb300.h -- C ABI of the GB300 particle hot path (libpairs_gb300.so).
 *
 * One entry point per module of the reference's generated time step that it
 * replaces.  The reference prints each module as a C/CUDA function taking raw
 * pointers and sizes (src/pairs/code_gen/cgen.py:119-251) and calls it from the
 * generated main(); these entry points take the same kind of arguments: plain
 * structs of device pointers, sizes and capacities, plus a cudaStream_t passed as
 * void*.  No C++ or torch type crosses the boundary.
 *
 * Memory: the caller owns every buffer (the Python front end allocates them as
 * torch tensors).  The library allocates nothing; kernels that need scratch take it
 * from pg_workspace (pg_bin_particles_noalloc instead uses a fixed array inside the
 * library).
 *
 * Errors: every entry point returns an int status (PG_OK, or a PG_ERR_* code, or
 * PG_OVERFLOW when a capacity was too small).  On PG_OVERFLOW the needed size is in
 * pg_status (device memory written by the kernel, read by the host after the
 * stream is synchronised) -- the reference's resizes[] protocol
 * (src/pairs/transformations/modules.py:37-205, runtime/devices/device.hpp:63-71).
 * Kernels never trap or assert.
 *
 * Layouts (all device memory, "sorted order" = cell order of the last rebuild):
 *   double4 pos[n]      x, y, z, (unused)          FP64 master positions
 *   double4 vel[n]      vx, vy, vz, (unused)
 *   double4 force[n]    FP64 force (precision PG_FP64)
 *   float4  force32[n]  FP32 force (precision PG_MIXED)
 *   float4  pos_hi[n], pos_lo[n]   compensated FP32 positions: hi on a 2^-k grid so
 *                      hi differences and periodic shifts are exact in FP32, lo the
 *                      FP32 residual x - hi
 *   int4    pos_fx[n]  fixed-point positions (precision PG_MIXED, periodic boxes of
 *                      at least 2 reach + 2 cells per axis): 2^32 units per box length, so
 *                      periodic images need no shift; replaces pos_hi/pos_lo there
 *   int     nbr[k * stride + i]    Verlet entry k of particle i (column-major, as
 *                      the reference's GPU layout, sim/neighbor_lists.py:14); bits
 *                      0-25 the partner index, bits 26-31 the periodic image code
 *                      (2 bits per dimension: 0 none, 1 plus one box, 2 minus one)
 */
#ifndef PAIRS_GB300_H
#define PAIRS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_OK              0
#define PG_OVERFLOW        1     /* a capacity was exceeded; see pg_status */
#define PG_ERR_ARGUMENT   -1     /* invalid argument (sizes, null pointers, alignment) */
#define PG_ERR_CUDA       -2     /* a CUDA call failed (launch or runtime error) */
#define PG_ERR_NONFINITE  -3     /* a non-finite position/velocity/force was found */
#define PG_ERR_LIMIT      -4     /* the input is larger than a fixed-scratch entry point takes */

#define PG_FP64   0              /* FP64 force, FP64 everything */
#define PG_MIXED  1              /* FP32 force on compensated FP32 positions, FP64 integration */

#define PG_SYNC_EXACT      0     /* periodic images always at the partner's current position */
#define PG_SYNC_REFERENCE  1     /* images refreshed like the reference's halo sync:
                                    an image shifted in k>1 dimensions uses the partner's
                                    position from min(k-1, steps since rebuild) steps ago
                                    (src/pairs/sim/comm.py:46-54, 369-442) */

#define PG_NBR_INDEX_BITS 26
#define PG_NBR_INDEX_MASK ((1u << PG_NBR_INDEX_BITS) - 1u)

/* Device-side status, written by kernels (mirrors the reference's resizes[]). */
typedef struct {
    int32_t overflow;            /* bit 0 cells, bit 1 neighbours, bit 2 tile
                                    neighbourhood, bit 3 contacts; bit 4: a grid
                                    barrier of pg_lj_steps or pg_ensemble_steps ran out
                                    of time */
    int32_t max_cell_count;      /* largest cell occupancy seen */
    int32_t max_neighbors;       /* largest per-particle Verlet count seen */
    int32_t nonfinite;           /* set when a non-finite value was met */
    int32_t guard_tripped;       /* first step at which a displacement > skin/2 was seen;
                                    INT32_MAX while none was */
    int32_t max_contacts;        /* DEM contact-history slots needed */
    int32_t max_tile_staged;     /* largest tile neighbourhood seen (overflow bit 2) */
    int32_t pad;
} pg_status;

/* Periodic (or walled) orthorhombic box, sim/domain_partitioning.py:46-57. */
typedef struct {
    double lo[3];
    double hi[3];
    double len[3];               /* hi - lo, as the reference's grid.length() */
    int    periodic[3];
    float  len_hi[3];            /* len split on the compensated FP32 grid */
    float  len_lo[3];
    double quantum;              /* grid step of pos_hi (a power of two) */
    double fx_scale[3];          /* 2^32 / len: fixed-point units per length (pos_fx) */
    float  fx_unit[3];           /* len / 2^32 rounded to FP32: length of one unit */
    int32_t fx_pad_;
} pg_box;

/* Per-particle state, sorted order.  Optional arrays may be NULL. */
typedef struct {
    int32_t n;                   /* particles in use */
    int32_t capacity;
    double *pos;                 /* double4[capacity] */
    double *pos_prev1;           /* double4[capacity], PG_SYNC_REFERENCE only */
    double *pos_prev2;           /* double4[capacity], PG_SYNC_REFERENCE only */
    double *vel;                 /* double4[capacity] */
    double *force;               /* double4[capacity] (PG_FP64) */
    float  *force32;             /* float4[capacity]  (PG_MIXED) */
    float  *pos_hi;              /* float4[capacity]  (PG_MIXED); w = type as float bits */
    float  *pos_lo;              /* float4[capacity]  (PG_MIXED) */
    double *pos_ref;             /* double4[capacity] positions at last rebuild (guard) */
    float  *ref_hi;              /* float4[capacity]  pos_hi at last rebuild (guard screen) */
    float  *ref_lo;              /* float4[capacity]  pos_lo at last rebuild */
    int32_t *pos_fx;             /* int4[capacity] or NULL (PG_MIXED): fixed-point positions,
                                    x_fx = round((x - lo) * fx_scale) mod 2^32 per axis, w =
                                    type.  A box length is 2^32 units, so the wrapped 32-bit
                                    difference of two coordinates is their minimum-image
                                    separation; used instead of pos_hi/pos_lo when every
                                    axis is periodic and has at least 2 reach + 2 cells
                                    (the axis's stencil reach) */
    int32_t *ref_fx;             /* int4[capacity] pos_fx at last rebuild (guard screen) */
    double *mass;                /* [capacity] */
    int32_t *type;               /* [capacity] */
    int32_t *uid;                /* [capacity] user id (the reference's uid property) */
    int32_t *flags;              /* [capacity] reference flag bits: 1 infinite, 4 fixed */
    /* Speculative stepping: when `guard` is not NULL it points at
     * status->guard_tripped; a force pass of time step `step` does nothing once the
     * guard tripped at a step <= `step`, an integration pass once it tripped at a
     * step < `step`.  The host later rebuilds at the tripped step and resumes. */
    const int32_t *guard;
    int32_t step;
    int32_t hilo_stride;         /* 0 or 1: pos_hi and pos_lo are separate float4 arrays;
                                    2: one interleaved array (hi, lo of a particle in one
                                    32-byte record), pos_lo = pos_hi + 4 floats */
} pg_particles;

/* Cell grid over the box, counting-sort layout (cell_start/cell_count). */
typedef struct {
    int32_t dims[3];
    int32_t ncells;
    int32_t reach;               /* Verlet build stencil: cells within `reach` per axis (27 cells
                                    for 1, 125 for 2); 0 is taken as 1 */
    int32_t reach_x;             /* stencil reach along x alone (1 or 2; 0: `reach`).  With
                                    reach 1 and reach_x 2 the cells are half as wide in x and
                                    the stencil has 5 x 3 x 3 cells */
    double  cell_len[3];         /* len[d] / dims[d] >= list radius / reach of axis d */
    int32_t *cell_start;         /* [ncells + 2]: cells, then the bucket of infinite shapes */
    int32_t *cell_count;         /* [ncells + 1] */
    int32_t *particle_cell;      /* [capacity] */
} pg_cells;

/* Verlet list, column-major ELL.  Two entry formats:
 *   nbr   32-bit global partner index + image code (any precision);
 *   nbr16 16-bit slot in the shared-memory neighbourhood of the particle's tile
 *         (mixed precision, full lists; used when not NULL): a tile is tile_z
 *         cells of one z column, its neighbourhood the 3x3 columns around it,
 *         staged with the periodic images applied.  The build writes each tile's
 *         layout (segments of the neighbourhood) to tile_table and the largest
 *         neighbourhood to pg_status.max_tile_staged. */
#define PG_TILE_RECORD_WORDS 180     /* int32 words per tile in tile_table */
typedef struct {
    int32_t stride;              /* >= capacity of particles */
    int32_t max_neighbors;       /* entries per particle */
    int32_t half;                /* 1: interior pairs once (Newton's third law), stored by
                                    the particle whose partner lies above it in x (ties: y,
                                    z, then the higher index); pairs through a periodic image
                                    in both lists */
    int32_t *nbr;                /* [max_neighbors * stride] or NULL */
    int32_t *count;              /* [stride] */
    int32_t steps_since_build;   /* host-maintained, for PG_SYNC_REFERENCE */
    uint16_t *nbr16;             /* [max_neighbors * stride] or NULL */
    int32_t tile_z;              /* cells per tile along z (nbr16 lists) */
    int32_t tile_capacity;       /* build: largest neighbourhood allowed (overflow bit 2
                                    above it); force: slots each block stages (at least
                                    the build's max_tile_staged) */
    int32_t *tile_table;         /* [ntiles * PG_TILE_RECORD_WORDS] */
    int32_t tile_tpa;            /* threads per particle in the tile force kernel: 1, 2, 4 */
    int32_t pad_;
    int32_t *pair_table;         /* [stride] or NULL: pair-cluster half lists (below) */
} pg_neighbor_list;

/* Lennard-Jones parameters per type pair (examples/md.py:5-8, feature tables). */
typedef struct {
    int32_t ntypes;              /* <= 16 */
    double  cutoff2;             /* rc^2 (6.25 for rc = 2.5) */
    double  epsilon[256];        /* [ti * ntypes + tj] */
    double  sigma6[256];
} pg_lj_params;

/* Scratch memory provided by the caller (bytes). */
typedef struct {
    void   *ptr;
    int64_t bytes;
} pg_workspace;

/* One replica of a batched ensemble: its slice of the concatenated particle arrays
 * and of the shared cell arrays, and its own periodic box and cell grid.  Replicas
 * are independent systems; no pair crosses replicas. */
typedef struct {
    int32_t first;               /* particles [first, first + n) */
    int32_t n;
    int32_t cell0;               /* cells [cell0, cell0 + ncells) of the shared cell arrays */
    int32_t ncells;
    int32_t dims[3];
    int32_t reach;               /* stencil reach in cells (cell_len >= r_list / reach) */
    double  lo[3];
    double  len[3];
    double  cell_len[3];
    double  inv_cell_len[3];     /* 1 / cell_len (the binning multiplies by it) */
    double  quantum;             /* grid step of this replica's pos_hi */
    float   len_hi[3];
    float   len_lo[3];
    double  fx_scale[3];         /* 2^32 / len: fixed-point units of this replica's box (pos_fx) */
    float   fx_unit[3];          /* len / 2^32 rounded to FP32 */
    int32_t reach_x;             /* stencil reach along x (0: `reach`); 2 with reach 1: x cells
                                    of >= r_list / 2, a 5 x 3 x 3 stencil */
} pg_replica;

/* A batched ensemble (config: hundreds of independent periodic LJ replicas run by
 * one launch per phase).  The per-particle list layout interleaves `tpa` entries per
 * particle: entry k of particle i is at ((k / tpa) * stride + i) * tpa + k % tpa, so the
 * tpa threads that share a particle read consecutive words.  With list->pair_table set,
 * the lists are pair-cluster half lists over every replica's cells (the layout of
 * pg_build_neighbor_lists; stride >= pg_pair_slots(n, total cells)), tpa and block
 * then unused. */
typedef struct {
    int32_t nreplicas;
    int32_t ncells;              /* cells of all replicas */
    const pg_replica *replicas;  /* device [nreplicas] */
    const int32_t *replica_of;   /* device [capacity]: replica of each particle */
    int32_t tpa;                 /* threads per particle in the force kernel: 1, 2, 4 or 8 */
    int32_t block;               /* threads per block of the force kernel: 64..512 */
    int32_t half;                /* 1: half lists (the list's own flag must agree); the drift
                                    pass of pg_ensemble_integrate then zeroes force32 after its
                                    kick, and the force pass adds reactions into it */
    int32_t cubic;               /* 1: every replica's box is cubic; the pair-cluster build then
                                    screens distances in fixed-point units (0: in lengths) */
    const int32_t *rebuild;      /* device [nreplicas] or NULL: a partial rebuild.  Binning and
                                    list build then touch only the replicas with a nonzero flag
                                    (pg_ensemble_select); the others keep their particle order,
                                    cells and list rows.  The cell arrays must hold the last
                                    binning of every replica.  NULL: every replica. */
} pg_ensemble;

/* DEM particle state, sorted order (the properties of examples/dem.py:144-162).
 * Spheres (shape 0) and half spaces (shape 1, flags infinite|fixed) share the
 * arrays; binning puts half spaces in the trailing bucket of the cell grid.  The
 * reference's rotation matrix is not stored: it is always the matrix of rotation_quat
 * (mapping/keywords.py:241-259), recomputed where needed with the same arithmetic.
 * The reference's 3x3 inverse inertia is diag(inv_inertia) for both shapes. */
typedef struct {
    int32_t n;
    int32_t capacity;
    double *pos;                 /* double4[capacity] */
    double *vel;                 /* double4[capacity] linear velocity; w = 1 / mass, written
                                    by pg_dem_setup (0 for half spaces) */
    double *angvel;              /* double4[capacity] angular velocity; w = the gravity force
                                    on z, 0 - (drho 4/3 pi r^3) g, written by pg_dem_setup
                                    (0 for half spaces) */
    double *force;               /* double4[capacity] */
    double *torque;              /* double4[capacity] */
    double *quat;                /* double4[capacity] rotation quaternion (w, x, y, z) */
    double *normal;              /* double4[capacity] half-space normal */
    double *pos_ref;             /* double4[capacity] positions at the last list build */
    double *mass;                /* [capacity] (+inf for half spaces after setup) */
    double *radius;              /* [capacity] */
    double *inv_inertia;         /* [capacity] diagonal of the inverse inertia tensor */
    int32_t *uid;                /* [capacity] */
    int32_t *type;               /* [capacity] */
    int32_t *flags;              /* [capacity] 1 infinite, 4 fixed, 8 global */
    int32_t *shape;              /* [capacity] 0 sphere, 1 half space */
    float   *pos32;              /* float4[capacity] (x, y, z, radius) in FP32, or NULL; kept
                                    by the list build and Euler for the mixed-precision
                                    contact kernel's candidate screen */
    const int32_t *guard;        /* speculative stepping, as pg_particles.guard */
    int32_t step;
    int32_t pad_;
} pg_dem_particles;

/* Per-particle contact history (sim/contact_history.py:12-17): up to `capacity`
 * records per particle, column-major [slot * stride + particle], keyed by the
 * partner's uid, in creation order (the reference's contact_lists / num_contacts
 * with the properties is_sticking, tangential_spring_displacement and
 * impact_velocity_magnitude of examples/dem.py:159-161). */
typedef struct {
    int32_t capacity;            /* records per particle, <= 64 */
    int32_t stride;              /* >= particle capacity */
    int32_t *count;              /* [stride] records in use */
    int32_t *partner;            /* [capacity * stride] partner uid */
    int32_t *sticking;           /* [capacity * stride] */
    double  *history;            /* double4[capacity * stride]: tangential spring
                                    displacement (x, y, z), impact velocity magnitude */
} pg_contacts;

/* Constants of the DEM program (symbols of examples/dem.py:180-211). */
typedef struct {
    double dt;
    double pi;                   /* the program's `pi` symbol */
    double kappa;                /* tangential / normal stiffness ratio */
    double ln_e;                 /* log of the dry restitution coefficient */
    double tc;                   /* collision time */
    double drho;                 /* densityParticle - densityFluid, in the symbols' type */
    double gravity;
    double skin;                 /* Verlet list skin (list radius r_i + r_j + skin) */
    double kn;                   /* 0: normal stiffness from the collision time tc, as the
                                    example; > 0: this fixed stiffness, damping
                                    -2 ln_e sqrt(meff kn) / sqrt(pi^2 + ln_e^2) */
    int32_t ntypes;              /* <= 4 */
    int32_t pad_;
    double friction_static[16];  /* [ti * ntypes + tj] */
    double friction_dynamic[16];
} pg_dem_params;

/* ---------------------------------------------------------------------------- */

/* Library version and the size of each struct, so a binding can check layouts. */
int pg_version(void);

/* Number of CUDA kernels this library has launched since it was loaded. */
int64_t pg_kernel_launches(void);
int pg_struct_sizes(int64_t *out, int n);

/* Scratch bytes pg_bin_particles / pg_compute_thermo need for n particles. */
int64_t pg_workspace_bytes(int32_t n, int32_t ncells);

/* Wrap particles that left a periodic box back in (x < lo -> x + len, x > hi ->
 * x - len, as the reference's exchange, sim/comm.py:101-151), bin them into the
 * cell grid, and permute every per-particle array into cell order (within a cell by
 * z, then uid; cells are numbered z fastest, so each z column of cells is sorted by z).  Replaces build_cell_lists + partition_cell_lists
 * (sim/cell_lists.py:90-171) and the exchange half of the halo code.
 * The grid must have dims[d] >= 1 and a positive, finite cell_len[d] on every axis
 * and ncells = dims[0]*dims[1]*dims[2]; anything else returns PG_ERR_ARGUMENT before
 * any work is queued. */
int pg_bin_particles(const pg_box *box, pg_particles *p, pg_cells *cells,
                     pg_workspace ws, pg_status *status, void *stream);

/* pg_bin_particles for callers that cannot allocate device memory.  No counterpart
 * in the reference (its generated code allocates its own arrays).
 *
 * Who needs it: a host program that gives this library a fixed device-memory
 * budget at start-up and allows no allocation afterwards, or one that must not
 * stall on (or fail in) a device allocation inside its time loop, cannot make the
 * workspace pg_bin_particles takes.  This entry point takes the same inputs and
 * outputs and no workspace: its scratch is a fixed array inside the library's own
 * device image, which every GPU that loads the library holds until the process
 * exits (about 12.8 MB).  It calls no allocator.
 *
 * Limit: at most PG_NOALLOC_MAX_PARTICLES particles and PG_NOALLOC_MAX_CELLS cells;
 * larger inputs return PG_ERR_LIMIT before any work is queued.
 * The first call on a device looks up the scratch array's device address (once
 * per device, on the calling thread's current device); make that first call
 * before any stream capture begins.
 * Every call shares the one scratch array and leaves its contents behind (the
 * call clears what it needs zeroed itself); calls whose GPU work overlaps, on
 * different streams or from different host threads, race on it: serialise them.
 * The binning permutation of such a call stays in the library's array, so
 * pg_bin_permutation cannot return it: a caller that keeps further per-particle
 * arrays of its own, which it would permute with pg_permute, uses pg_bin_particles
 * with a workspace instead. */
#define PG_NOALLOC_MAX_PARTICLES 131072
#define PG_NOALLOC_MAX_CELLS     65536
int pg_bin_particles_noalloc(const pg_box *box, pg_particles *p, pg_cells *cells, pg_status *status,
                             void *stream);

/* Build the Verlet list within r_list (the reference's build_neighbor_lists,
 * sim/neighbor_lists.py:21-48 with interaction.py:90-120).  The acceptance test
 * rsq < r_list2 is evaluated exactly as the reference: FP64, image position
 * fl(x_j + s*len), delta, (dx*dx + dy*dy) + dz*dz, no fused multiply-add.  Also
 * records pos_ref (and ref_hi/ref_lo or ref_fx) for the displacement guard.  The FP32
 * screen reads pos_fx when it is set and the box allows it (every axis periodic with
 * at least 2 reach + 2 cells), else pos_hi/pos_lo.
 *
 * Pair-cluster half lists (list->pair_table not NULL; half lists on fixed-point
 * positions, PG_MIXED forces): the list is kept per cluster of two consecutive
 * particles of one cell (the last particle of an odd cell alone).  pair_table[t] of
 * cluster slot t is the first particle's index, bit 30 set when particle index + 1 is
 * the second member, or -1 for a free slot; stride must be at least
 * pg_pair_slots(n, ncells).  nbr[k * stride + t] is the partner index in bits 0-29,
 * bit 30 set when the pair (first member, partner) is stored, bit 31 for the second
 * member; count[t] entries.  The pair set is the per-particle half list's, each pair
 * stored once by the member whose partner lies above it in x (minimum image; pairs
 * through a periodic image too), and the force applies every pair's reaction. */
int64_t pg_pair_slots(int32_t n, int32_t ncells);
int pg_build_neighbor_lists(const pg_box *box, const pg_particles *p, const pg_cells *cells,
                            pg_neighbor_list *list, double r_list2, pg_status *status,
                            void *stream);

/* Lennard-Jones forces over the Verlet list (the reference's lennard_jones module:
 * examples/md.py:5-8, sim/interaction.py:222-232, ir/apply.py:112-125).
 * precision PG_FP64 writes p->force, PG_MIXED writes p->force32.  sync_mode selects
 * PG_SYNC_EXACT or PG_SYNC_REFERENCE (FP64 only).  energy, if not NULL, is a device
 * double[2] that receives potential energy and virial sum r.F (FP64 sums).  cells
 * is needed for nbr16 (tile) lists and may be NULL otherwise.  On the PG_MIXED path a
 * pair whose FP32 rsq lies within a relative 1e-5 of the cutoff is decided by the
 * FP64 test of the PG_FP64 path, so both paths apply the force of the same pairs;
 * such pairs are queued in ws and applied by a second kernel.  ws is scratch of at
 * least 256 + 8 bytes; its queue holds (ws.bytes - 256) / 8 pairs.  About 1.7e-3
 * pairs per particle fall in the band with full lists at density 0.84 (half that
 * with half lists), so 256 + 8 * ceil(0.004 * n) bytes leaves a wide margin, and
 * pg_workspace_bytes(n, ncells) always does.  A queue that overflows loses no
 * force: the second kernel then walks every list again for the band's pairs, which
 * costs about one more force pass.  Pair-cluster lists (list->pair_table, see
 * pg_build_neighbor_lists) take the mixed path on fixed-point positions with a half
 * list; one thread walks a cluster's list and computes both members' pairs in the two
 * lanes of packed FP32 instructions. */
int pg_lj_force(const pg_box *box, const pg_particles *p, const pg_cells *cells,
                const pg_neighbor_list *list, const pg_lj_params *lj, int precision, int sync_mode,
                double *energy, pg_workspace ws, void *stream);

/* Plain time steps of the mixed-precision LJ path in one persistent, cooperative
 * launch: for each device step first_step .. first_step + nsteps - 1, the fused final
 * + initial half kicks with the FP64 drift and displacement guard (pg_integrate_mixed
 * with kicks = 2), the force pass on the Verlet list (pg_lj_force) and its FP64
 * decision of the cutoff band, each phase closed by a grid barrier.  Replaces the
 * per-module kernel launches and device synchronisations of the reference's
 * generated time loop (src/pairs/code_gen/cgen.py:540-576) for the steps between two
 * list rebuilds.  Needs fixed-point positions (pos_fx, ref_fx), force32, global
 * per-particle lists (no tile or pair-cluster lists).  The guard keeps its meaning: a trip in the integration of step r ends the
 * launch before the force of step r (status->guard_tripped = r), as the separate
 * kernels would skip themselves.  ws: scratch as for pg_lj_force (its first 256
 * bytes hold the queue count and the barrier words).  No barrier waits longer than
 * barrier_timeout_s (2 s if <= 0): after that the launch ends early with
 * status->overflow bit 4 set and the state of an unfinished step.  A call with
 * nsteps = 0 only prepares the launch (it queries the device once, so make it before
 * a stream capture that will hold such launches). */
int pg_lj_steps(const pg_box *box, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                double dt, double half_skin2, int32_t first_step, int32_t nsteps, pg_status *status,
                pg_workspace ws, double barrier_timeout_s, void *stream);

/* Diagnostic of the grid barrier that pg_lj_steps uses (no counterpart in the
 * reference): a cooperative launch passes three barriers that expect extra_arrivals
 * more blocks than it has.  With extra_arrivals = 0 it returns with status untouched;
 * with more, no wait can end, every block gives up after timeout_s and
 * status->overflow bit 4 is set.  Either way the device stays usable. */
int pg_grid_barrier_check(int32_t extra_arrivals, double timeout_s, pg_status *status, pg_workspace ws,
                          void *stream);

/* Velocity-Verlet half steps of examples/md.py:11-17 (the reference's
 * initial_integrate / final_integrate modules), same operation order:
 *   initial: v = v + ((dt*0.5)*F)/m;  x = x + dt*v      (pre_step, skip_first)
 *   final:   v = v + ((dt*0.5)*F)/m                     (skip_first)
 * precision selects which force array is read.  The initial step also tests every
 * particle's displacement since the last list build against half_skin2 in FP64
 * (the guard; the first offending step is kept in status->guard_tripped) and
 * refreshes pos_hi/pos_lo and pos_fx when present.  With sync_mode PG_SYNC_REFERENCE the caller
 * rotates the position ring first (prev2 <- prev1 <- pos <- old prev2); the kernel
 * then reads pos_prev1 and writes pos. */
int pg_initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision,
                         double half_skin2, int32_t step, int sync_mode, pg_status *status,
                         void *stream);
int pg_final_integrate(const pg_box *box, pg_particles *p, double dt, int precision, void *stream);

/* Final half kick of step k fused with the initial kick + drift of step k+1: one
 * pass instead of two, identical arithmetic to calling both in order. */
int pg_final_initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision,
                               double half_skin2, int32_t step, int sync_mode, pg_status *status,
                               void *stream);

/* Mixed-precision integration (FP32 force in, FP64 velocity/position update):
 * kicks = 1 or 2 half kicks merged into one (v += kicks*(dt/2)*F/m), then, if drift,
 * x += dt*v in FP64, pos_hi/pos_lo re-split (or pos_fx rounded) from the new x, and
 * the FP64 displacement guard (screened in FP32 against ref_hi/ref_lo or ref_fx,
 * decided in FP64 near the threshold) recorded in status->guard_tripped. */
int pg_integrate_mixed(const pg_box *box, pg_particles *p, double dt, int kicks, int drift,
                       double half_skin2, int32_t step, pg_status *status, void *stream);

/* Sum m v^2 over particles (FP64, fixed reduction tree, deterministic) and
 * write out[0] = T = sum/(3N-3), out[1] = kinetic pressure T(3N-3)/(3V), out[2] = sum
 * (runtime/thermo.hpp:11-51).  out is device memory (double[3]). */
int pg_compute_thermo(const pg_box *box, const pg_particles *p, double *out,
                      pg_workspace ws, void *stream);

/* Refresh pos_hi / pos_lo and pos_fx (those present) from pos (after a host upload
 * or a permutation). */
int pg_split_positions(const pg_box *box, pg_particles *p, void *stream);

/* Device address of the permutation of the last pg_bin_particles call that used ws
 * with these sizes (new index k holds old particle perm[k]), or NULL if ws is too
 * small.  No counterpart in the reference, whose exchange moves every property
 * itself: callers that keep further per-particle arrays permute them with it. */
const int32_t *pg_bin_permutation(int32_t n, int32_t ncells, pg_workspace ws);

/* dst[k] = src[perm[k]] for k < n, elements of elem_bytes (4, 8, 16 or 32): applies
 * the last binning permutation to caller-held per-particle arrays. */
int pg_permute(int32_t n, const int32_t *perm, const void *src, void *dst, int elem_bytes,
               void *stream);

/* ---- learned rebuild schedule (no counterpart in the reference, which rebuilds
 * on a fixed period: sim/simulation.py:232-233, sim/timestep.py:47) ----------- */

/* Number of FP32 parameters of the 3-64-64-1 network: W1[64][3] b1[64] W2[64][64]
 * b2[64] W3[64] b3. */
int pg_mlp_param_count(void);

/* Per-cell features [ncells][4]: max|v|*dt/(skin/2), mean(|F|/m)*dt^2/(skin/2),
 * steps_since_build/20, 1 if the cell holds particles else 0. */
int pg_cell_features(const pg_particles *p, const pg_cells *cells, int precision, int32_t steps_since_build,
                     double dt, double half_skin, float *features, void *stream);

/* pg_cell_features of a state just binned by pg_bin_particles, before any force pass:
 * every per-particle array is in the new order except the forces, which the binning
 * leaves in the old one; perm is that binning's permutation (pg_bin_permutation:
 * perm[k] = index before the binning of particle k).  The cells are the new ones. */
int pg_cell_features_binned(const pg_particles *p, const pg_cells *cells, const int32_t *perm, int precision,
                            int32_t steps_since_build, double dt, double half_skin, float *features, void *stream);

/* The cells of one sample (no counterpart in the reference): the ncells feature rows
 * are split into k contiguous groups and each group's row with the largest feature 0
 * (fastest particle) is copied to out[k][4].  ncells >= k. */
int pg_cell_select(const float *features, int32_t ncells, int32_t k, float *out, void *stream);

/* out[c] = network output (log steps until the cell's first displacement > skin/2)
 * for non-empty cells, +inf for empty ones. */
int pg_mlp_forward(const float *params, const float *features, int32_t ncells, float *out, void *stream);

/* result[0] = soft minimum of out (temperature T), result[1] = min (ordered int
 * bits), result[2] = partition sum; result is device float[4]. */
int pg_mlp_softmin(const float *out, int32_t ncells, float temperature, float *result, void *stream);

/* Accumulate the gradient of (P - target_log)^2 (censored: min(P - target_log, 0)^2)
 * into grads[param_count] and the loss into *loss (device). */
int pg_mlp_backward(const float *params, const float *features, const float *out, int32_t ncells,
                    const float *result, float target_log, int censored, float temperature, float *grads,
                    float *loss, void *stream);

/* One Adam step on params with grads * grad_scale; zeroes grads. t counts from 1. */
int pg_mlp_adam(float *params, float *grads, float *m1, float *m2, float lr, float beta1, float beta2,
                float eps, int32_t t, float grad_scale, void *stream);

/* ---- batched ensemble of LJ replicas (no counterpart in the reference, which runs
 * one system per generated program; each replica follows the same modules) ---- */

/* Wrap each particle into its replica's box and bin it into the replica's cells
 * (global cell = cell0 + local cell), sort, permute, and split positions on each
 * replica's grid; pg_bin_particles for every replica at once.  cells->ncells = total
 * cells, cell_start/cell_count sized as for pg_bin_particles.  ws:
 * pg_workspace_bytes(n, total cells).  pos_hi/pos_lo may be NULL with fixed-point
 * positions (then only pos_fx is written).  With e->rebuild set, only the flagged
 * replicas are binned (see pg_ensemble). */
int pg_ensemble_bin(const pg_ensemble *e, pg_particles *p, pg_cells *cells, pg_workspace ws, pg_status *status,
                    void *stream);

/* Verlet lists within r_list for every replica (the stencil of each replica's reach
 * and reach_x), exact FP64 acceptance as pg_build_neighbor_lists, in the
 * tpa-interleaved layout (full or half lists per e->half), or pair-cluster half lists
 * when list->pair_table is set (every replica grid then needs 2 reach + 1 cells per
 * axis, else status->overflow bit 5); records pos_ref and ref_fx (or ref_hi / ref_lo).
 * With e->rebuild set, only the flagged replicas' rows are built. */
int pg_ensemble_build_lists(const pg_ensemble *e, pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
                            double r_list2, pg_status *status, void *stream);

/* Mixed-precision LJ forces for every replica, tpa threads per particle (pair-cluster
 * lists: one thread per row), full or half lists:
 * FP32 on fixed-point positions (p->pos_fx, each replica's box 2^32 units, used when set)
 * or on compensated positions.  Pairs within a relative 1e-5 of the cutoff
 * are decided by the FP64 test, as in pg_lj_force, through a queue in ws (scratch, at
 * least 256 + 8 bytes, sized as for pg_lj_force; the binning workspace serves). */
int pg_ensemble_force(const pg_ensemble *e, const pg_particles *p, const pg_neighbor_list *list,
                      const pg_lj_params *lj, pg_workspace ws, void *stream);

/* pg_integrate_mixed for every replica (each re-splits on its own grid); the guard
 * word takes the first step at which any replica's particle moved > skin/2. */
int pg_ensemble_integrate(const pg_ensemble *e, pg_particles *p, double dt, int kicks, int drift,
                          double half_skin2, int32_t step, pg_status *status, void *stream);

/* The plain steps first .. first + nsteps - 1 of every replica in one cooperative
 * launch: per step pg_ensemble_integrate (two half kicks, drift), pg_ensemble_force
 * and its cutoff-band decisions, separated by grid barriers -- the same arithmetic, in
 * place of 2 nsteps launches under a CUDA graph (the generated code launches and
 * synchronises every module of every step, src/pairs/code_gen/cgen.py:540-576).
 * Needs fixed-point positions (pos_fx, ref_fx) and force32.  A guard trip in the
 * integration of step r ends the launch before the force of step r (status->
 * guard_tripped = r), as the separate kernels would skip themselves.  ws: scratch as
 * for pg_ensemble_force (its first 256 bytes hold the queue count and the barrier
 * words).  No barrier waits longer than timeout_s (2 s when <= 0): then
 * status->overflow gets bit 4 and the state is that of an unfinished step.  A call
 * with nsteps = 0 only prepares the launch (make it before a stream capture). */
int pg_ensemble_steps(const pg_ensemble *e, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                      double dt, double half_skin2, int32_t first, int32_t nsteps, pg_status *status,
                      pg_workspace ws, double timeout_s, void *stream);

/* Per-replica thermo: out[2r] = T_r = sum/(3 n_r - 3), out[2r+1] = sum m v^2 (FP64,
 * one block per replica, fixed order).  out: device double[2 * nreplicas]. */
int pg_ensemble_thermo(const pg_ensemble *e, const pg_particles *p, double *out, void *stream);

/* The replicas of a partial rebuild: rebuild[r] = 1 when a particle of replica r moved
 * more than sqrt(thresh2) since its last list build (the guard's FP32 displacement:
 * fixed point, or the hi/lo pair), or holds a non-finite position; else 0.  thresh2 < 0
 * selects every replica.  With thresh2 below skin^2 / 4 every replica the guard tripped
 * on is selected.  rebuild: device int32[nreplicas].  Replaces nothing in the reference
 * (one system per run); the batched ensemble's per-replica rebuilds. */
int pg_ensemble_select(const pg_ensemble *e, const pg_particles *p, double thresh2, int32_t *rebuild, void *stream);

/* ---- DEM (examples/dem.py) ------------------------------------------------ */

/* Setup kernel update_mass_and_inertia (examples/dem.py:6-15): identity rotation,
 * inv_inertia = the (0,0) entry of inversed(diagonal_matrix(0.4 m r^2)) for spheres
 * (mapping/keywords.py:129-146 arithmetic), mass = +inf and inv_inertia = 0 for half
 * spaces.  Also stores 1 / mass in vel.w and each sphere's gravity force on z
 * (examples/dem.py:90-92 with prm) in angvel.w. */
int pg_dem_setup(pg_dem_particles *d, const pg_dem_params *prm, void *stream);

/* Wrap, bin and sort the DEM particles like pg_bin_particles.  pos, uid, flags and
 * cells->particle_cell are permuted in place; every other per-particle array of d
 * and the contact history c are gathered into `spare` / `spare_c` (same capacities),
 * which the caller then swaps with d / c.  force and torque are not carried (each
 * step recomputes them).  ws: pg_workspace_bytes(n, ncells). */
int pg_dem_bin(const pg_box *box, pg_dem_particles *d, const pg_dem_particles *spare, const pg_contacts *c,
               const pg_contacts *spare_c, pg_cells *cells, pg_workspace ws, pg_status *status, void *stream);

/* Sphere-sphere candidate list: partners j (with periodic image) whose centre lies
 * within r_i + r_j + skin, over the 27 cells around the sphere (cell_len must be at
 * least 2 r_max + skin).  Records pos_ref.  The reference scans the 27 cells every
 * step instead (build_cell_lists only, examples/dem.py:193); the exact contact test
 * below runs every step, so the contacts are the same while no sphere moved more
 * than skin/2 since the build. */
int pg_dem_build_list(const pg_box *box, pg_dem_particles *d, const pg_cells *cells, pg_neighbor_list *list,
                      const pg_dem_params *prm, pg_status *status, void *stream);

/* Gravity with buoyancy (examples/dem.py:90-92) and the linear spring-dashpot
 * contact (examples/dem.py:18-74) against spheres (list) and half spaces (trailing
 * bucket), with contact-history lookup/creation by partner uid
 * (mapping/funcs.py:230-265) and removal of the records not used this step
 * (sim/contact_history.py:91-127).  Writes force and torque.  precision PG_FP64:
 * the generated operation order; PG_MIXED: FP64 contact geometry, FP32 contact
 * model and sums.  Overflow bit 3: a particle needed more than c->capacity records. */
int pg_dem_force(const pg_box *box, const pg_dem_particles *d, const pg_cells *cells,
                 const pg_neighbor_list *list, const pg_contacts *c, const pg_dem_params *prm,
                 int precision, pg_status *status, void *stream);

/* Explicit Euler with rotation (examples/dem.py:77-87), skipping fixed particles,
 * plus the FP64 displacement guard against pos_ref (first step with a displacement
 * above sqrt(half_skin2) kept in status->guard_tripped).  precision PG_FP64: the
 * generated operation order; PG_MIXED: the same FP64 update with fused
 * multiply-adds. */
int pg_dem_euler(pg_dem_particles *d, const pg_dem_params *prm, int precision, double half_skin2, int32_t step,
                 pg_status *status, void *stream);

/* ---- VTK output (runtime/vtk.hpp:11-86, replaces the host loops of vtk_write_data) */

/* Workspace of pg_vtk_format_rows / pg_vtk_pack_rows for `rows` rows: a 96-byte slot
 * per row, then the int32 row lengths (the last 4 * rows bytes); -1 for rows < 0. */
int64_t pg_vtk_workspace_bytes(int32_t rows);

/* Formats row k of one section for particle order[k] (order NULL: k) into its slot and
 * its length into the length array: section 0 "x y z\n" of pos[i] (double4) and section
 * 2 "m\n" of mass[i], each number as printf("%.8f") prints it (exact conversion, ties to
 * even); section 1 "1 index[k]\n" (index NULL: k).  A length of -1 marks a value that
 * %.8f with at most 11 integer digits cannot hold (|x| >= 9.2e10, NaN, infinity).  The
 * caller leaves infinite shapes out of `order` and gives in index[k] the row's index
 * among all particles (vtk.hpp:36-40, 57-60). */
int pg_vtk_format_rows(int section, int32_t rows, const int32_t *order, const double *pos, const double *mass,
                       const int32_t *index, pg_workspace ws, void *stream);

/* Copies the formatted rows to out + offsets[k] (offsets: the exclusive scan of the
 * lengths, int64, device memory), giving the section's text. */
int pg_vtk_pack_rows(int32_t rows, pg_workspace ws, const int64_t *offsets, char *out, void *stream);

/* ---- particle CSV input on the device ---------------------------------------
 * Replaces read_particle_data (runtime/read_from_file.hpp:33-116).  The caller copies
 * the file's bytes to the device (text); the library indexes the lines, parses every
 * field as std::stod (PG_CSV_REAL) or std::stoi (PG_CSV_INT) reads it, keeps a line's
 * particle when its position (fields pos_field .. pos_field + 2) lies in [lo, hi - 1e-5)
 * on every axis (runtime/domain/regular_6d_stencil.cpp:96-100; no filter when domain_lo
 * is NULL) or its flags field (flags_field, or -1) has the infinite, fixed or global bit,
 * and writes the kept rows in file order to table, column-major [nfields * max_rows]
 * (integers as exact doubles).  Lines of white space only are skipped.  A real field is
 * converted to the correctly rounded double (ties to even) for up to 19 significant
 * digits and decimal exponents within +-27 (up to 15 digits: +-22 by one FP64 operation);
 * other numbers are counted in result->inexact.  A missing field, a field without
 * digits or an integer outside int32 sets result->bad_line (0-based, the first such
 * line).  Either returns PG_ERR_ARGUMENT; more kept rows than max_rows return
 * PG_ERR_LIMIT with result->rows the number needed.  Both calls synchronise the stream
 * (they return counts to the host). */
#define PG_CSV_REAL 0
#define PG_CSV_INT  1
typedef struct {
    int32_t rows;                /* particles kept */
    int32_t lines;               /* lines indexed (newlines + 1) */
    int32_t bad_line;            /* first malformed line, or -1 */
    int32_t inexact;             /* real fields outside the exact conversion range */
} pg_csv_result;
int64_t pg_csv_count_bytes(int64_t bytes);
int pg_csv_count_lines(const char *text, int64_t bytes, int64_t *lines, pg_workspace ws, void *stream);
int64_t pg_csv_workspace_bytes(int64_t bytes, int64_t lines, int32_t nfields);
int pg_csv_parse(const char *text, int64_t bytes, int64_t lines, int32_t nfields, const int32_t *kinds,
                 int32_t pos_field, int32_t flags_field, const double *domain_lo, const double *domain_hi,
                 double *table, int32_t max_rows, pg_csv_result *result, pg_workspace ws, void *stream);

/* ---- DEM simple-cubic initialiser on the device -----------------------------
 * Replaces dem_sc_grid (runtime/dem_sc_grid.hpp:62-172) on one rank: spheres on the grid
 * points spacing/2 + k*spacing inside [0, xmax) x [0, ymax) x [diameter, zmax), x
 * fastest; a point inside the domain [lo, hi - 1e-5) is kept with uid = its visit
 * number + 1, a diameter drawn uniformly in [min_diameter, max_diameter) from a
 * default-seeded std::mt19937 (one draw per visited point, libstdc++'s
 * generate_canonical: two 32-bit words per draw), velocity (0.1 U(-v0, v0), 0.1
 * U(-v0, v0), -v0) from two more draws, mass 4/3 pi r^3 density and type rand() %
 * ntypes (glibc rand(), default seed); bit-identical to the reference on one rank.
 * pg_dem_sc_grid_size gives the visited and kept counts and the workspace bytes (host
 * arithmetic only).  Outputs are double4 pos and vel, and per sphere mass, radius,
 * type, uid; capacity is their length.  The call synchronises the stream. */
int pg_dem_sc_grid_size(double xmax, double ymax, double zmax, double spacing, double diameter, const double *lo,
                        const double *hi, int64_t *npoints, int64_t *nkept, int64_t *ws_bytes);
int pg_dem_sc_grid(double xmax, double ymax, double zmax, double spacing, double diameter, double min_diameter,
                   double max_diameter, double initial_velocity, double density, int32_t ntypes, const double *lo,
                   const double *hi, double *pos, double *vel, double *mass, double *radius, int32_t *type,
                   int32_t *uid, int64_t capacity, pg_workspace ws, void *stream);

/* cudaStreamSynchronize, returning PG_OK or PG_ERR_CUDA. */
int pg_stream_sync(void *stream);

#ifdef __cplusplus
}
#endif

#endif
