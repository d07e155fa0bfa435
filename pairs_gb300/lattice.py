"""Initial particle states: the reference's fcc lattice and its thermo adjustment.

Host-side setup (like the reference's runtime, which builds the lattice on the host
before the time loop).  Restates, vectorised and bit-identical in FP64:

* runtime/copper_fcc_lattice.hpp:64-145 -- fcc sites (i+j+k even on a 2n grid of
  a/2) visited in 8^3 sub-box order, per-site Park-Miller velocities
  (:18-26 without masking; seed = site index + 1, five discarded draws before each
  component), mass 1, type = rand() % ntypes in visiting order;
* runtime/thermo.hpp:53-97 -- subtract the mean velocity, rescale to T, with the
  reference's sequential FP64 summation order.

rand() is the C library generator the reference calls unseeded; glibc's is an
additive lagged-Fibonacci generator (r[i] = r[i-3] + r[i-31] mod 2^32, 34 seeded
words from the minimal-standard LCG, first 310 outputs discarded, result r >> 1),
restated here so the type stream matches.
"""
import math

import numpy as np

_IA, _IM, _IQ, _IR = 16807, 2147483647, 127773, 2836


def _park_miller(seed):
    """One Park-Miller step on an int64 array of seeds; returns (seed, value)."""
    k = seed // _IQ
    seed = _IA * (seed - k * _IQ) - _IR * k
    seed = np.where(seed < 0, seed + _IM, seed)
    return seed, (1.0 / _IM) * seed.astype(np.float64)


def glibc_rand(count, seed=1):
    """First `count` outputs of glibc rand() after srand(seed)."""
    r = [0] * 34
    r[0] = seed
    for i in range(1, 31):
        hi, lo = divmod(r[i - 1], 127773)
        w = 16807 * lo - 2836 * hi
        if w < 0:
            w += 2147483647
        r[i] = w
    for i in range(31, 34):
        r[i] = r[i - 31]
    out = []
    buf = r
    total = 344 + count
    for i in range(34, total):
        buf.append((buf[i - 31] + buf[i - 3]) & 0xFFFFFFFF)
        if i >= 344:
            out.append(buf[i] >> 1)
    return np.array(out, dtype=np.int64)


def fcc_sites(nx, ny, nz, rho):
    """Lattice sites of copper_fcc_lattice in the reference's visiting order.

    Returns (i, j, k) integer arrays and the lattice constant."""
    alat = pow(4.0 / rho, 1.0 / 3.0)
    xprd, yprd, zprd = nx * alat, ny * alat, nz * alat
    half = 0.5 * alat
    ihi = min(int(xprd / half + 1), 2 * nx - 1)
    jhi = min(int(yprd / half + 1), 2 * ny - 1)
    khi = min(int(zprd / half + 1), 2 * nz - 1)
    sub = 8
    nox, noy, noz = ihi // sub + 1, jhi // sub + 1, khi // sub + 1
    # order: sx fastest, then sy, sz, ox, oy, oz
    oz, oy, ox, sz, sy, sx = np.meshgrid(np.arange(noz), np.arange(noy), np.arange(nox),
                                         np.arange(sub), np.arange(sub), np.arange(sub), indexing="ij")
    i = (ox * sub + sx).ravel().astype(np.int64)
    j = (oy * sub + sy).ravel().astype(np.int64)
    k = (oz * sub + sz).ravel().astype(np.int64)
    keep = ((i + j + k) % 2 == 0) & (i <= ihi) & (j <= jhi) & (k <= khi)
    i, j, k = i[keep], j[keep], k[keep]
    x, y, z = half * i, half * j, half * k
    small = 0.00001                               # regular_6d_stencil.hpp:6
    inside = (x >= 0.0) & (x < xprd - small) & (y >= 0.0) & (y < yprd - small) & \
             (z >= 0.0) & (z < zprd - small)
    return i[inside], j[inside], k[inside], alat


def copper_fcc_lattice(nx, ny, nz, rho=0.8442, temperature=1.44, ntypes=1):
    """The reference's LJ initial state.  Returns a dict with pos, vel (n, 3) float64,
    mass (n,), type (n,) int32, uid (n,) = creation index, and box (3,)."""
    i, j, k, alat = fcc_sites(nx, ny, nz, rho)
    half = 0.5 * alat
    pos = np.stack([half * i, half * j, half * k], axis=1)
    seed = k * (2 * ny) * (2 * nx) + j * (2 * nx) + i + 1
    vel = np.empty_like(pos)
    for c in range(3):
        for _ in range(5):
            seed, _v = _park_miller(seed)
        seed, vel[:, c] = _park_miller(seed)
    n = len(pos)
    mass = np.ones(n)
    if ntypes > 1:
        typ = (glibc_rand(n) % ntypes).astype(np.int32)
    else:
        typ = np.zeros(n, dtype=np.int32)
    box = np.array([nx * alat, ny * alat, nz * alat])
    adjust_thermo(mass, vel, box, temperature)
    return dict(pos=pos, vel=vel, mass=mass, type=typ, uid=np.arange(n, dtype=np.int32), box=box)


def _seq_sum(a):
    """Left-to-right FP64 sum (the reference's loop order)."""
    return np.cumsum(a)[-1] if len(a) else 0.0


def temperature(mass, vel):
    """T = sum m (vx*vx + vy*vy + vz*vz) / (3N-3), reference summation order."""
    n = len(mass)
    s = mass * ((vel[:, 0] * vel[:, 0] + vel[:, 1] * vel[:, 1]) + vel[:, 2] * vel[:, 2])
    return _seq_sum(s) * (1.0 / (n * 3 - 3))


def adjust_thermo(mass, vel, box, temp):
    """Zero the total momentum (mean velocity) and rescale to `temp`, in place."""
    n = len(mass)
    for c in range(3):
        vel[:, c] -= _seq_sum(vel[:, c]) / n
    t = temperature(mass, vel)
    vel *= np.sqrt(temp / t)


# ---------------------------------------------------------------------------- DEM grid

def _mt19937_words(count, seed=5489):
    """First `count` 32-bit outputs of std::mt19937(seed) (tempered), as uint64."""
    mt = np.zeros(624, dtype=np.uint64)
    mt[0] = seed
    for i in range(1, 624):
        prev = int(mt[i - 1])
        mt[i] = (1812433253 * (prev ^ (prev >> 30)) + i) & 0xFFFFFFFF
    upper, lower, mag = np.uint64(0x80000000), np.uint64(0x7FFFFFFF), np.uint64(0x9908B0DF)
    out = []
    produced = 0

    def twist(lo, hi):
        # mt[i] for i in [lo, hi): reads mt[i+1] (old unless i+1 == 624 -> new mt[0])
        # and mt[(i+397) % 624] (already new when it wrapped below i)
        i = np.arange(lo, hi)
        nxt = mt[(i + 1) % 624]
        y = (mt[i] & upper) | (nxt & lower)
        v = mt[(i + 397) % 624] ^ (y >> np.uint64(1))
        v = np.where((y & np.uint64(1)) != 0, v ^ mag, v)
        mt[lo:hi] = v

    while produced < count:
        twist(0, 227)          # reads old mt[397..623]
        twist(227, 454)        # reads new mt[0..226]
        twist(454, 623)        # reads new mt[227..395]
        twist(623, 624)        # reads new mt[0] and mt[396]
        y = mt.copy()
        y ^= y >> np.uint64(11)
        y ^= (y << np.uint64(7)) & np.uint64(0x9D2C5680)
        y ^= (y << np.uint64(15)) & np.uint64(0xEFC60000)
        y ^= y >> np.uint64(18)
        out.append(y & np.uint64(0xFFFFFFFF))
        produced += 624
    return np.concatenate(out)[:count] if out else np.zeros(0, dtype=np.uint64)


def _canonical(words):
    """libstdc++ generate_canonical<double, 53> over pairs of 32-bit draws (low word
    first): (a + b * 2^32) / 2^64, rounded once in the sum, clamped below 1."""
    a = words[0::2].astype(np.float64)
    b = words[1::2].astype(np.float64)
    r = (a + b * 4294967296.0) / 18446744073709551616.0
    return np.where(r >= 1.0, np.nextafter(1.0, 0.0), r)


def dem_sc_grid(xmax, ymax, zmax, spacing, diameter, min_diameter, max_diameter, initial_velocity, density,
                ntypes, lo=(0.0, 0.0, 0.0), hi=None):
    """Spheres on a simple-cubic grid, the reference's dem_sc_grid
    (runtime/dem_sc_grid.hpp:62-172) on one rank, vectorised and bit-identical.

    Grid points ref + idx*spacing (ref = spacing/2) inside [0, xmax) x [0, ymax) x
    [diameter, zmax), visited x fastest.  Every visited point draws a diameter from a
    default-seeded mt19937 (uniform in [min_diameter, max_diameter)); a point inside
    the domain [lo, hi - 1e-5) becomes a sphere with uid = its visit number + 1, mass
    4/3 pi r^3 density, velocity (0.1 U(-v0, v0), 0.1 U(-v0, v0), -v0) from the same
    engine and type rand() % ntypes."""
    hi = (xmax, ymax, zmax) if hi is None else hi
    gen_lo = (0.0, 0.0, float(diameter))
    gen_hi = (float(xmax), float(ymax), float(zmax))
    ref = spacing * 0.5
    axes = []
    for d in range(3):
        start = int(math.ceil((gen_lo[d] - ref) / spacing))
        idx = []
        k = start
        while True:
            x = ref + k * spacing
            if not (x >= gen_lo[d] and x < gen_hi[d]):
                break
            idx.append(x)
            k += 1
        axes.append(np.array(idx, dtype=np.float64))
    if any(len(a) == 0 for a in axes):
        return dict(pos=np.zeros((0, 3)), vel=np.zeros((0, 3)), mass=np.zeros(0), radius=np.zeros(0),
                    type=np.zeros(0, np.int32), uid=np.zeros(0, np.int32), flags=np.zeros(0, np.int32),
                    shape=np.zeros(0, np.int32))
    zz, yy, xx = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    pts = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)
    npts = len(pts)
    small = 0.00001
    inside = np.ones(npts, dtype=bool)
    for d in range(3):
        inside &= (pts[:, d] >= lo[d]) & (pts[:, d] < hi[d] - small)
    # uniform draws in visiting order: one per point, two more per kept sphere
    per_point = 1 + 2 * inside.astype(np.int64)
    first = np.concatenate([[0], np.cumsum(per_point)[:-1]])
    ndraws = int(per_point.sum())
    u = _canonical(_mt19937_words(2 * ndraws))
    diam = u[first] * (max_diameter - min_diameter) + min_diameter
    v0 = float(initial_velocity)
    keep = np.nonzero(inside)[0]
    vx = 0.1 * (u[first[keep] + 1] * (v0 - (-v0)) + (-v0))
    vy = 0.1 * (u[first[keep] + 2] * (v0 - (-v0)) + (-v0))
    n = len(keep)
    rad = diam[keep] * 0.5
    pi = 3.141592653589793
    mass = ((4.0 / 3.0) * pi) * rad * rad * rad * float(density)
    vel = np.stack([vx, vy, np.full(n, -v0)], axis=1)
    typ = (glibc_rand(n) % ntypes).astype(np.int32) if n else np.zeros(0, np.int32)
    return dict(pos=pts[keep].copy(), vel=vel, mass=mass, radius=rad, type=typ,
                uid=(keep + 1).astype(np.int32), flags=np.zeros(n, np.int32), shape=np.zeros(n, np.int32))


def dem_sc_grid_device(xmax, ymax, zmax, spacing, diameter, min_diameter, max_diameter, initial_velocity, density,
                       ntypes, lo=(0.0, 0.0, 0.0), hi=None, device=None):
    """dem_sc_grid generated on the GPU (pg_dem_sc_grid, csrc/demgrid.cu): the same
    spheres, bit-identical, as torch tensors on the device (pos and vel n x 4, the
    fourth component zero)."""
    import ctypes as C
    import torch
    from . import _capi as A
    lib = A.load()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    hi = (xmax, ymax, zmax) if hi is None else hi
    dlo, dhi = (C.c_double * 3)(*[float(v) for v in lo]), (C.c_double * 3)(*[float(v) for v in hi])
    npts, kept, wsb = C.c_int64(0), C.c_int64(0), C.c_int64(0)
    A.call("pg_dem_sc_grid_size", float(xmax), float(ymax), float(zmax), float(spacing), float(diameter), dlo, dhi,
           C.byref(npts), C.byref(kept), C.byref(wsb))
    n = int(kept.value)
    f64 = dict(dtype=torch.float64, device=dev)
    out = dict(pos=torch.zeros((n, 4), **f64), vel=torch.zeros((n, 4), **f64), mass=torch.zeros(n, **f64),
               radius=torch.zeros(n, **f64), type=torch.zeros(n, dtype=torch.int32, device=dev),
               uid=torch.zeros(n, dtype=torch.int32, device=dev))
    ws = torch.empty(max(int(wsb.value), 16), dtype=torch.uint8, device=dev)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    A.call("pg_dem_sc_grid", float(xmax), float(ymax), float(zmax), float(spacing), float(diameter),
           float(min_diameter), float(max_diameter), float(initial_velocity), float(density), int(ntypes), dlo, dhi,
           ptr(out["pos"]), ptr(out["vel"]), ptr(out["mass"]), ptr(out["radius"]), ptr(out["type"]), ptr(out["uid"]),
           n, A.PgWorkspace(ws.data_ptr(), ws.numel()), C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    out["flags"] = torch.zeros(n, dtype=torch.int32, device=dev)
    out["shape"] = torch.zeros(n, dtype=torch.int32, device=dev)
    return out


# ---------------------------------------------------------------------------- ensembles

def trimmed_fcc(natoms, rho, temperature, uid0=0):
    """One replica of the batched ensemble: the smallest n^3 fcc lattice with
    4 n^3 >= natoms, its first `natoms` sites in the reference's visiting order,
    rescaled into the cubic box L = (natoms / rho)^(1/3); reference velocity rule
    (Park-Miller per site, zero momentum, rescaled to `temperature` over the kept
    atoms), mass 1, one type."""
    n = 1
    while 4 * n ** 3 < natoms:
        n += 1
    i, j, k, _ = fcc_sites(n, n, n, 0.8442)
    i, j, k = i[:natoms], j[:natoms], k[:natoms]
    L = (natoms / rho) ** (1.0 / 3.0)
    half = L / (2 * n)
    pos = np.stack([half * i, half * j, half * k], axis=1)
    seed = k * (2 * n) * (2 * n) + j * (2 * n) + i + 1
    vel = np.empty_like(pos)
    for c in range(3):
        for _ in range(5):
            seed, _v = _park_miller(seed)
        seed, vel[:, c] = _park_miller(seed)
    mass = np.ones(natoms)
    box = np.array([L, L, L])
    adjust_thermo(mass, vel, box, temperature)
    return dict(pos=pos, vel=vel, mass=mass, type=np.zeros(natoms, np.int32),
                uid=np.arange(uid0, uid0 + natoms, dtype=np.int32), box=box)


def ensemble_configs(count=512, nmin=500, nmax=32000, rho=(0.6, 0.9), temperature=(0.7, 1.5), seed=2024):
    """Replica sizes log-uniform in [nmin, nmax], densities and temperatures uniform,
    from numpy's PCG64 with `seed`."""
    g = np.random.default_rng(seed)
    sizes = np.exp(g.uniform(np.log(nmin), np.log(nmax), count)).astype(np.int64)
    rhos = g.uniform(rho[0], rho[1], count)
    temps = g.uniform(temperature[0], temperature[1], count)
    return [dict(natoms=int(s), rho=float(r), temperature=float(t)) for s, r, t in zip(sizes, rhos, temps)]


def dem_random_packing(count, box, rmin, rmax, density, seed=7, spacing=None):
    """`count` spheres, radii uniform in [rmin, rmax], at random non-overlapping
    positions in `box` (lower corner at the origin), filled from the bottom up: one
    sphere per site of a cubic lattice of spacing >= 2 rmax, jittered uniformly by
    up to (spacing/2 - r) per axis so it stays inside its own site cube.  numpy
    PCG64 with `seed`; mass 4/3 pi r^3 density, zero velocity, uid 1..count."""
    s = float(spacing or 2.0 * rmax * 1.05)
    nx, ny, nz = (int(math.floor(box[d] / s)) for d in range(3))
    if nx * ny * nz < count:
        raise ValueError(f"box holds only {nx * ny * nz} sites of spacing {s}")
    g = np.random.default_rng(seed)
    k = np.arange(count)
    ix, iy, iz = k % nx, (k // nx) % ny, k // (nx * ny)
    r = g.uniform(rmin, rmax, count)
    room = (0.5 * s - r)[:, None]
    jitter = g.uniform(-1.0, 1.0, (count, 3)) * room
    pos = (np.stack([ix, iy, iz], axis=1) + 0.5) * s + jitter
    mass = (4.0 / 3.0) * math.pi * r * r * r * density
    return dict(pos=pos, vel=np.zeros((count, 3)), mass=mass, radius=r, type=np.zeros(count, np.int32),
                uid=np.arange(1, count + 1, dtype=np.int32), flags=np.zeros(count, np.int32),
                shape=np.zeros(count, np.int32))


def dem_compressed_fcc(count, rmin, rmax, density, nearest, seed=7):
    """`count` spheres on the sites of an fcc lattice whose nearest-neighbour distance is
    `nearest`, radii uniform in [rmin, rmax] (numpy PCG64 with `seed`), at rest: a
    compressed packing in which a pair of neighbours overlaps whenever r_i + r_j >
    nearest (with radii U[0.4, 0.6] mm and nearest = 1 mm, half of the 12 neighbours).
    The lattice has n x n x 2n unit cells (n the smallest that holds `count`), filled
    from the bottom; sites start half a nearest distance above z = 0.  Returns the
    state (mass 4/3 pi r^3 density, uid 1..count) and the box (x, y periodic lengths
    and the height of the highest site plus half a nearest distance)."""
    a = nearest * math.sqrt(2.0)
    n = int(math.ceil((count / 8.0) ** (1.0 / 3.0)))
    basis = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
    k = np.arange(2 * n * n * n)
    ix, iy, iz = k % n, (k // n) % n, k // (n * n)
    cells = np.stack([ix, iy, iz], axis=1).astype(np.float64)
    sites = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3)
    sites = sites[np.lexsort((sites[:, 0], sites[:, 1], sites[:, 2]))][:count] * a
    sites[:, 2] += 0.5 * nearest
    g = np.random.default_rng(seed)
    r = g.uniform(rmin, rmax, count)
    mass = (4.0 / 3.0) * math.pi * r * r * r * density
    box = (n * a, n * a, float(sites[:, 2].max()) + 0.5 * nearest)
    state = dict(pos=sites, vel=np.zeros((count, 3)), mass=mass, radius=r, type=np.zeros(count, np.int32),
                 uid=np.arange(1, count + 1, dtype=np.int32), flags=np.zeros(count, np.int32),
                 shape=np.zeros(count, np.int32))
    return state, box
