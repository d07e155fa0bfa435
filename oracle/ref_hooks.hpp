/*
 * Dump hooks force-included (g++ -include) into the reference's generated CPU
 * program when oracle/ref_build.py builds it as a test oracle.  Test
 * infrastructure only: the product never includes this file.
 *
 * oracle_hook_init  -- called right after the setup modules (copper_fcc_lattice +
 *                      adjust_thermo or read_particle_data), before the time loop.
 *                      copper_fcc_lattice never assigns `uid`
 *                      (runtime/copper_fcc_lattice.hpp:64-145), so when asked to it
 *                      numbers particles 0..nlocal-1 in creation order; the dump
 *                      then carries the initial state keyed by that uid.
 * oracle_hook_step  -- called after the user modules of time step `ts` (after
 *                      lennard_jones / final_integrate, before compute_thermo,
 *                      generated main loop order of sim/simulation.py:387-417).
 *                      Writes uid, position, linear_velocity, force of the local
 *                      particles; on rebuild steps also the Verlet list mapped to
 *                      (uid_i, uid_j, image shift) and the cell occupancy.
 *
 * Files: <dir>/init.bin and <dir>/step_<ts>.bin, little-endian raw records, read by
 * oracle/ref_dump.py.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <unordered_map>
#include <vector>

namespace oracle_dump {

inline const char *dump_dir() {
    const char *d = std::getenv("PAIRS_ORACLE_DUMP");
    return (d != nullptr && d[0] != '\0') ? d : nullptr;
}

inline int env_int(const char *name, int dflt) {
    const char *v = std::getenv(name);
    return (v != nullptr && v[0] != '\0') ? std::atoi(v) : dflt;
}

inline void put_i32(FILE *f, int32_t v) { fwrite(&v, sizeof(v), 1, f); }

template<typename T>
inline void put_arr(FILE *f, const T *p, size_t n) { if(n) { fwrite(p, sizeof(T), n, f); } }

}  // namespace oracle_dump

static void oracle_hook_init(
    int nlocal, int *uid, int *type, int *flags, double *mass, double *position,
    double *linear_velocity) {

    using namespace oracle_dump;
    if(env_int("PAIRS_ORACLE_SET_UID", 1)) {
        for(int i = 0; i < nlocal; i++) { uid[i] = i; }
    }

    const char *dir = dump_dir();
    if(dir == nullptr) { return; }
    std::string path = std::string(dir) + "/init.bin";
    FILE *f = fopen(path.c_str(), "wb");
    if(f == nullptr) { perror("oracle_hook_init"); std::exit(3); }
    put_i32(f, nlocal);
    put_arr(f, uid, nlocal);
    put_arr(f, type, nlocal);
    put_arr(f, flags, nlocal);
    put_arr(f, mass, nlocal);
    put_arr(f, position, (size_t) nlocal * 3);
    put_arr(f, linear_velocity, (size_t) nlocal * 3);
    fclose(f);
}

/*
 * nb_stride / nb_slot_stride describe the Verlet-list layout the generator chose:
 * CPU target AoS  -> entry k of particle i at neighborlists[i * neighbor_capacity + k]
 * (sim/neighbor_lists.py:14, Layouts.AoS when the target is not a GPU).
 */
static void oracle_hook_step(
    int ts, int rebuilt, int nlocal, int nghost, const double *box_len,
    const int *uid, const double *position, const double *linear_velocity,
    const double *force, const int *numneighs, const int *neighborlists,
    int neighbor_capacity, int ncells, const int *cell_sizes, const int *particle_cell) {

    using namespace oracle_dump;
    const char *dir = dump_dir();
    if(dir == nullptr) { return; }
    const int every = env_int("PAIRS_ORACLE_DUMP_EVERY", 1);
    if(!rebuilt && every > 1 && (ts % every) != 0) { return; }

    char name[64];
    snprintf(name, sizeof(name), "/step_%05d.bin", ts);
    std::string path = std::string(dir) + name;
    FILE *f = fopen(path.c_str(), "wb");
    if(f == nullptr) { perror("oracle_hook_step"); std::exit(3); }

    put_i32(f, ts);
    put_i32(f, rebuilt);
    put_i32(f, nlocal);
    put_i32(f, nghost);
    put_arr(f, uid, nlocal);
    put_arr(f, position, (size_t) nlocal * 3);
    put_arr(f, linear_velocity, (size_t) nlocal * 3);
    put_arr(f, force, (size_t) nlocal * 3);

    if(rebuilt && numneighs != nullptr) {
        std::unordered_map<int, int> owner;
        owner.reserve((size_t) nlocal * 2);
        for(int i = 0; i < nlocal; i++) { owner[uid[i]] = i; }

        std::vector<int32_t> rec;
        for(int i = 0; i < nlocal; i++) {
            for(int k = 0; k < numneighs[i]; k++) {
                const int j = neighborlists[(size_t) i * neighbor_capacity + k];
                const int o = owner.at(uid[j]);
                rec.push_back(uid[i]);
                rec.push_back(uid[j]);
                for(int d = 0; d < 3; d++) {
                    const double s = (position[j * 3 + d] - position[o * 3 + d]) / box_len[d];
                    rec.push_back((int32_t) std::lround(s));
                }
            }
        }
        put_i32(f, (int32_t) (rec.size() / 5));
        put_arr(f, rec.data(), rec.size());

        /* cell occupancy of local particles only (ghost images excluded) */
        std::vector<int32_t> local_count((size_t) ncells, 0);
        for(int i = 0; i < nlocal; i++) {
            const int c = particle_cell[i];
            if(c >= 0 && c < ncells) { local_count[c]++; }
        }
        put_i32(f, ncells);
        put_arr(f, cell_sizes, (size_t) ncells);
        put_arr(f, local_count.data(), (size_t) ncells);
    } else {
        put_i32(f, -1);
    }
    fclose(f);
}

/* DEM dumps (examples/dem.py program): initial state after the setup kernel, and
 * per step the local particles' state plus every contact-history record. */
static void oracle_hook_init_dem(int nlocal, const int *uid, const int *type, const int *flags, const int *shape,
                                 const double *mass, const double *radius, const double *position,
                                 const double *linear_velocity, const double *normal) {
    using namespace oracle_dump;
    const char *dir = dump_dir();
    if(dir == nullptr) { return; }
    std::string path = std::string(dir) + "/init.bin";
    FILE *f = fopen(path.c_str(), "wb");
    if(f == nullptr) { perror("oracle_hook_init_dem"); std::exit(3); }
    put_i32(f, nlocal);
    put_arr(f, uid, nlocal); put_arr(f, type, nlocal); put_arr(f, flags, nlocal); put_arr(f, shape, nlocal);
    put_arr(f, mass, nlocal); put_arr(f, radius, nlocal);
    put_arr(f, position, (size_t) nlocal * 3); put_arr(f, linear_velocity, (size_t) nlocal * 3);
    put_arr(f, normal, (size_t) nlocal * 3);
    fclose(f);
}

static void oracle_hook_step_dem(int ts, int nlocal, const int *uid, const double *position,
                                 const double *linear_velocity, const double *angular_velocity,
                                 const double *force, const double *torque, const double *rotation_quat,
                                 const int *num_contacts, const int *contact_lists, const int *is_sticking,
                                 const double *tsd, const double *ivm, int neighbor_capacity) {
    using namespace oracle_dump;
    const char *dir = dump_dir();
    if(dir == nullptr) { return; }
    const int every = env_int("PAIRS_ORACLE_DUMP_EVERY", 1);
    if(every > 1 && (ts % every) != 0) { return; }
    char name[64];
    snprintf(name, sizeof(name), "/step_%05d.bin", ts);
    std::string path = std::string(dir) + name;
    FILE *f = fopen(path.c_str(), "wb");
    if(f == nullptr) { perror("oracle_hook_step_dem"); std::exit(3); }
    put_i32(f, ts); put_i32(f, nlocal);
    put_arr(f, uid, nlocal);
    put_arr(f, position, (size_t) nlocal * 3); put_arr(f, linear_velocity, (size_t) nlocal * 3);
    put_arr(f, angular_velocity, (size_t) nlocal * 3);
    put_arr(f, force, (size_t) nlocal * 3); put_arr(f, torque, (size_t) nlocal * 3);
    put_arr(f, rotation_quat, (size_t) nlocal * 4);
    std::vector<int32_t> ids;
    std::vector<double> vals;
    for(int i = 0; i < nlocal; i++) {
        for(int k = 0; k < num_contacts[i]; k++) {
            const size_t a = (size_t) i * neighbor_capacity + k;
            ids.push_back(uid[i]); ids.push_back(contact_lists[a]); ids.push_back(is_sticking[a]);
            vals.push_back(tsd[a * 3]); vals.push_back(tsd[a * 3 + 1]); vals.push_back(tsd[a * 3 + 2]);
            vals.push_back(ivm[a]);
        }
    }
    put_i32(f, (int32_t) (ids.size() / 3));
    put_arr(f, ids.data(), ids.size());
    put_arr(f, vals.data(), vals.size());
    fclose(f);
}
