"""ctypes binding of libpairs_gb300.so (the C ABI in include/pairs_gb300.h).

The structs below mirror the header field by field; `check_layout()` compares their
sizes with the library's own sizeof() values at load time.  Every entry point returns
an int status; `call()` turns non-zero codes into exceptions.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpairs_gb300.so")

PG_OK = 0
PG_OVERFLOW = 1
PG_ERR_ARGUMENT = -1
PG_ERR_CUDA = -2
PG_ERR_NONFINITE = -3
PG_ERR_LIMIT = -4
NOALLOC_MAX_PARTICLES = 131072
NOALLOC_MAX_CELLS = 65536

PG_FP64 = 0
PG_MIXED = 1
PG_SYNC_EXACT = 0
PG_SYNC_REFERENCE = 1
NBR_INDEX_BITS = 26


class PgStatus(C.Structure):
    _fields_ = [("overflow", C.c_int32), ("max_cell_count", C.c_int32),
                ("max_neighbors", C.c_int32), ("nonfinite", C.c_int32),
                ("guard_tripped", C.c_int32), ("max_contacts", C.c_int32),
                ("max_tile_staged", C.c_int32), ("pad", C.c_int32)]


class PgBox(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3), ("len", C.c_double * 3),
                ("periodic", C.c_int * 3), ("len_hi", C.c_float * 3), ("len_lo", C.c_float * 3),
                ("quantum", C.c_double), ("fx_scale", C.c_double * 3), ("fx_unit", C.c_float * 3),
                ("fx_pad_", C.c_int32)]


class PgParticles(C.Structure):
    _fields_ = [("n", C.c_int32), ("capacity", C.c_int32),
                ("pos", C.c_void_p), ("pos_prev1", C.c_void_p), ("pos_prev2", C.c_void_p),
                ("vel", C.c_void_p), ("force", C.c_void_p), ("force32", C.c_void_p),
                ("pos_hi", C.c_void_p), ("pos_lo", C.c_void_p), ("pos_ref", C.c_void_p),
                ("ref_hi", C.c_void_p), ("ref_lo", C.c_void_p), ("pos_fx", C.c_void_p),
                ("ref_fx", C.c_void_p),
                ("mass", C.c_void_p), ("type", C.c_void_p), ("uid", C.c_void_p),
                ("flags", C.c_void_p), ("guard", C.c_void_p), ("step", C.c_int32), ("hilo_stride", C.c_int32)]


class PgCells(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("ncells", C.c_int32), ("reach", C.c_int32), ("reach_x", C.c_int32),
                ("cell_len", C.c_double * 3),
                ("cell_start", C.c_void_p), ("cell_count", C.c_void_p),
                ("particle_cell", C.c_void_p)]


class PgNeighborList(C.Structure):
    _fields_ = [("stride", C.c_int32), ("max_neighbors", C.c_int32), ("half", C.c_int32),
                ("nbr", C.c_void_p), ("count", C.c_void_p), ("steps_since_build", C.c_int32),
                ("nbr16", C.c_void_p), ("tile_z", C.c_int32), ("tile_capacity", C.c_int32),
                ("tile_table", C.c_void_p), ("tile_tpa", C.c_int32), ("pad_", C.c_int32),
                ("pair_table", C.c_void_p)]


TILE_RECORD_WORDS = 180


class PgLJParams(C.Structure):
    _fields_ = [("ntypes", C.c_int32), ("cutoff2", C.c_double),
                ("epsilon", C.c_double * 256), ("sigma6", C.c_double * 256)]


class PgWorkspace(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("bytes", C.c_int64)]


class PgDemParticles(C.Structure):
    _fields_ = [("n", C.c_int32), ("capacity", C.c_int32),
                ("pos", C.c_void_p), ("vel", C.c_void_p), ("angvel", C.c_void_p), ("force", C.c_void_p),
                ("torque", C.c_void_p), ("quat", C.c_void_p), ("normal", C.c_void_p), ("pos_ref", C.c_void_p),
                ("mass", C.c_void_p), ("radius", C.c_void_p), ("inv_inertia", C.c_void_p),
                ("uid", C.c_void_p), ("type", C.c_void_p), ("flags", C.c_void_p), ("shape", C.c_void_p),
                ("pos32", C.c_void_p), ("guard", C.c_void_p), ("step", C.c_int32), ("pad_", C.c_int32)]


class PgContacts(C.Structure):
    _fields_ = [("capacity", C.c_int32), ("stride", C.c_int32), ("count", C.c_void_p),
                ("partner", C.c_void_p), ("sticking", C.c_void_p), ("history", C.c_void_p)]


class PgDemParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("pi", C.c_double), ("kappa", C.c_double), ("ln_e", C.c_double),
                ("tc", C.c_double), ("drho", C.c_double), ("gravity", C.c_double), ("skin", C.c_double),
                ("kn", C.c_double),
                ("ntypes", C.c_int32), ("pad_", C.c_int32),
                ("friction_static", C.c_double * 16), ("friction_dynamic", C.c_double * 16)]


class PgReplica(C.Structure):
    _fields_ = [("first", C.c_int32), ("n", C.c_int32), ("cell0", C.c_int32), ("ncells", C.c_int32),
                ("dims", C.c_int32 * 3), ("reach", C.c_int32), ("lo", C.c_double * 3), ("len", C.c_double * 3),
                ("cell_len", C.c_double * 3), ("inv_cell_len", C.c_double * 3), ("quantum", C.c_double),
                ("len_hi", C.c_float * 3),
                ("len_lo", C.c_float * 3), ("fx_scale", C.c_double * 3), ("fx_unit", C.c_float * 3),
                ("reach_x", C.c_int32)]


class PgEnsemble(C.Structure):
    _fields_ = [("nreplicas", C.c_int32), ("ncells", C.c_int32), ("replicas", C.c_void_p),
                ("replica_of", C.c_void_p), ("tpa", C.c_int32), ("block", C.c_int32), ("half", C.c_int32),
                ("cubic", C.c_int32), ("rebuild", C.c_void_p)]


class PgCsvResult(C.Structure):
    _fields_ = [("rows", C.c_int32), ("lines", C.c_int32), ("bad_line", C.c_int32), ("inexact", C.c_int32)]


PG_CSV_REAL, PG_CSV_INT = 0, 1

STRUCTS = [PgStatus, PgBox, PgParticles, PgCells, PgNeighborList, PgLJParams, PgWorkspace, PgDemParticles,
           PgContacts, PgDemParams, PgReplica, PgEnsemble, PgCsvResult]

P = C.POINTER
# name -> (restype, argtypes)
SIGNATURES = {
    "pg_version": (C.c_int, []),
    "pg_kernel_launches": (C.c_int64, []),
    "pg_struct_sizes": (C.c_int, [P(C.c_int64), C.c_int]),
    "pg_workspace_bytes": (C.c_int64, [C.c_int32, C.c_int32]),
    "pg_bin_particles": (C.c_int, [P(PgBox), P(PgParticles), P(PgCells), PgWorkspace, C.c_void_p, C.c_void_p]),
    "pg_bin_particles_noalloc": (C.c_int, [P(PgBox), P(PgParticles), P(PgCells), C.c_void_p, C.c_void_p]),
    "pg_build_neighbor_lists": (C.c_int, [P(PgBox), P(PgParticles), P(PgCells), P(PgNeighborList), C.c_double,
                                          C.c_void_p, C.c_void_p]),
    "pg_lj_force": (C.c_int, [P(PgBox), P(PgParticles), P(PgCells), P(PgNeighborList), P(PgLJParams), C.c_int,
                              C.c_int, C.c_void_p, PgWorkspace, C.c_void_p]),
    "pg_lj_steps": (C.c_int, [P(PgBox), P(PgParticles), P(PgNeighborList), P(PgLJParams), C.c_double, C.c_double,
                              C.c_int32, C.c_int32, C.c_void_p, PgWorkspace, C.c_double, C.c_void_p]),
    "pg_grid_barrier_check": (C.c_int, [C.c_int32, C.c_double, C.c_void_p, PgWorkspace, C.c_void_p]),
    "pg_initial_integrate": (C.c_int, [P(PgBox), P(PgParticles), C.c_double, C.c_int, C.c_double, C.c_int32,
                                       C.c_int, C.c_void_p, C.c_void_p]),
    "pg_final_integrate": (C.c_int, [P(PgBox), P(PgParticles), C.c_double, C.c_int, C.c_void_p]),
    "pg_final_initial_integrate": (C.c_int, [P(PgBox), P(PgParticles), C.c_double, C.c_int, C.c_double,
                                             C.c_int32, C.c_int, C.c_void_p, C.c_void_p]),
    "pg_integrate_mixed": (C.c_int, [P(PgBox), P(PgParticles), C.c_double, C.c_int, C.c_int, C.c_double,
                                     C.c_int32, C.c_void_p, C.c_void_p]),
    "pg_compute_thermo": (C.c_int, [P(PgBox), P(PgParticles), C.c_void_p, PgWorkspace, C.c_void_p]),
    "pg_split_positions": (C.c_int, [P(PgBox), P(PgParticles), C.c_void_p]),
    "pg_permute": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "pg_pair_slots": (C.c_int64, [C.c_int32, C.c_int32]),
    "pg_csv_count_bytes": (C.c_int64, [C.c_int64]),
    "pg_csv_count_lines": (C.c_int, [C.c_void_p, C.c_int64, P(C.c_int64), PgWorkspace, C.c_void_p]),
    "pg_csv_workspace_bytes": (C.c_int64, [C.c_int64, C.c_int64, C.c_int32]),
    "pg_csv_parse": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int32, P(C.c_int32), C.c_int32, C.c_int32,
                               P(C.c_double), P(C.c_double), C.c_void_p, C.c_int32, P(PgCsvResult), PgWorkspace,
                               C.c_void_p]),
    "pg_dem_sc_grid_size": (C.c_int, [C.c_double] * 5 + [P(C.c_double), P(C.c_double), P(C.c_int64),
                                                           P(C.c_int64), P(C.c_int64)]),
    "pg_dem_sc_grid": (C.c_int, [C.c_double] * 9 + [C.c_int32, P(C.c_double), P(C.c_double)] + [C.c_void_p] * 6
                       + [C.c_int64, PgWorkspace, C.c_void_p]),
    "pg_vtk_workspace_bytes": (C.c_int64, [C.c_int32]),
    "pg_vtk_format_rows": (C.c_int, [C.c_int, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     PgWorkspace, C.c_void_p]),
    "pg_vtk_pack_rows": (C.c_int, [C.c_int32, PgWorkspace, C.c_void_p, C.c_void_p, C.c_void_p]),
    "pg_stream_sync": (C.c_int, [C.c_void_p]),
    "pg_mlp_param_count": (C.c_int, []),
    "pg_cell_features": (C.c_int, [P(PgParticles), P(PgCells), C.c_int, C.c_int32, C.c_double, C.c_double,
                                   C.c_void_p, C.c_void_p]),
    "pg_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "pg_mlp_softmin": (C.c_int, [C.c_void_p, C.c_int32, C.c_float, C.c_void_p, C.c_void_p]),
    "pg_bin_permutation": (C.c_void_p, [C.c_int32, C.c_int32, PgWorkspace]),
    "pg_cell_select": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "pg_cell_features_binned": (C.c_int, [P(PgParticles), P(PgCells), C.c_void_p, C.c_int, C.c_int32, C.c_double,
                                          C.c_double, C.c_void_p, C.c_void_p]),
    "pg_mlp_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_float, C.c_int,
                                  C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]),
    "pg_mlp_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_float,
                              C.c_float, C.c_int32, C.c_float, C.c_void_p]),
    "pg_ensemble_bin": (C.c_int, [P(PgEnsemble), P(PgParticles), P(PgCells), PgWorkspace, C.c_void_p,
                                  C.c_void_p]),
    "pg_ensemble_build_lists": (C.c_int, [P(PgEnsemble), P(PgParticles), P(PgCells), P(PgNeighborList),
                                          C.c_double, C.c_void_p, C.c_void_p]),
    "pg_ensemble_force": (C.c_int, [P(PgEnsemble), P(PgParticles), P(PgNeighborList), P(PgLJParams),
                                    PgWorkspace, C.c_void_p]),
    "pg_ensemble_integrate": (C.c_int, [P(PgEnsemble), P(PgParticles), C.c_double, C.c_int, C.c_int, C.c_double,
                                        C.c_int32, C.c_void_p, C.c_void_p]),
    "pg_ensemble_thermo": (C.c_int, [P(PgEnsemble), P(PgParticles), C.c_void_p, C.c_void_p]),
    "pg_ensemble_select": (C.c_int, [P(PgEnsemble), P(PgParticles), C.c_double, C.c_void_p, C.c_void_p]),
    "pg_ensemble_steps": (C.c_int, [P(PgEnsemble), P(PgParticles), P(PgNeighborList), P(PgLJParams), C.c_double,
                                    C.c_double, C.c_int32, C.c_int32, C.c_void_p, PgWorkspace, C.c_double,
                                    C.c_void_p]),
    "pg_dem_setup": (C.c_int, [P(PgDemParticles), P(PgDemParams), C.c_void_p]),
    "pg_dem_bin": (C.c_int, [P(PgBox), P(PgDemParticles), P(PgDemParticles), P(PgContacts), P(PgContacts),
                             P(PgCells), PgWorkspace, C.c_void_p, C.c_void_p]),
    "pg_dem_build_list": (C.c_int, [P(PgBox), P(PgDemParticles), P(PgCells), P(PgNeighborList), P(PgDemParams),
                                    C.c_void_p, C.c_void_p]),
    "pg_dem_force": (C.c_int, [P(PgBox), P(PgDemParticles), P(PgCells), P(PgNeighborList), P(PgContacts),
                               P(PgDemParams), C.c_int, C.c_void_p, C.c_void_p]),
    "pg_dem_euler": (C.c_int, [P(PgDemParticles), P(PgDemParams), C.c_int, C.c_double, C.c_int32, C.c_void_p,
                               C.c_void_p]),
}

_lib = None


class PairsError(RuntimeError):
    pass


class CapacityOverflow(PairsError):
    pass


def load(path=LIB_PATH):
    """Load the library (no GPU needed) and bind every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise PairsError(
            f"{path} is missing: build it with pairs_gb300.build.build() (nvcc, sm_103a). "
            "There is no CPU fallback.")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    check_layout(lib)
    return lib


def check_layout(lib):
    n = lib.pg_struct_sizes(None, 0)
    out = (C.c_int64 * n)()
    lib.pg_struct_sizes(out, n)
    for s, size in zip(STRUCTS, out):
        if C.sizeof(s) != size:
            raise PairsError(f"struct layout mismatch for {s.__name__}: python {C.sizeof(s)} vs C {size}")


_ERR = {PG_ERR_ARGUMENT: "invalid argument", PG_ERR_CUDA: "CUDA error", PG_ERR_NONFINITE: "non-finite state",
        PG_ERR_LIMIT: f"input too large for the fixed scratch (at most {NOALLOC_MAX_PARTICLES} particles and "
                      f"{NOALLOC_MAX_CELLS} cells)"}


def call(name, *args):
    rc = getattr(load(), name)(*args)
    if rc == PG_OVERFLOW:
        raise CapacityOverflow(f"{name}: capacity overflow")
    if rc != PG_OK:
        raise PairsError(f"{name} failed: {_ERR.get(rc, rc)}")
    return rc
