// extern "C" entry points of libpairs_gb300.so (declared in include/pairs_gb300.h).
#include "common.cuh"

namespace pg {
int64_t bin_workspace_bytes(int32_t n, int32_t ncells);
const int32_t *bin_permutation(int32_t n, int32_t ncells, pg_workspace ws);
int bin_particles(const pg_box *box, pg_particles *p, pg_cells *cells, pg_workspace ws,
                  pg_status *status, cudaStream_t st, int32_t **perm_out);
int gather_array(int n, const int32_t *perm, const void *src, void *dst, int elem_bytes, cudaStream_t st);
int split_positions(const pg_box *box, pg_particles *p, cudaStream_t st);
int build_neighbor_lists(const pg_box *box, const pg_particles *p, const pg_cells *cells,
                         pg_neighbor_list *list, double r_list2, pg_status *status, cudaStream_t st);
int lj_force(const pg_box *box, const pg_particles *p, const pg_cells *cells, const pg_neighbor_list *list,
             const pg_lj_params *lj, int precision, int sync_mode, double *energy, pg_workspace ws, cudaStream_t st);
int initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision, double half_skin2,
                      int32_t step, pg_status *status, int sync_mode, cudaStream_t st);
int final_integrate(const pg_box *box, pg_particles *p, double dt, int precision, cudaStream_t st);
int final_initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision,
                            double half_skin2, int32_t step, pg_status *status, int sync_mode,
                            cudaStream_t st);
int64_t thermo_workspace_bytes();
int integrate_mixed(const pg_box *box, pg_particles *p, double dt, int kicks, int drift,
                    double half_skin2, int32_t step, pg_status *status, cudaStream_t st);
int compute_thermo(const pg_box *box, const pg_particles *p, double *out, double *partials,
                   cudaStream_t st);
int cell_features(const pg_particles *p, const pg_cells *cells, const int32_t *perm, int precision, int32_t since, double dt,
                  double half_skin, float *feat, cudaStream_t st);
int mlp_forward(const float *params, const float *feat, int32_t ncells, float *out, cudaStream_t st);
int mlp_softmin(const float *out, int32_t ncells, float temperature, float *result, cudaStream_t st);
int cell_select(const float *features, int32_t ncells, int32_t k, float *out, cudaStream_t st);
int mlp_backward(const float *params, const float *feat, const float *out, int32_t ncells, const float *result,
                 float target_log, int censored, float temperature, float *grads, float *loss, cudaStream_t st);
int mlp_adam(float *params, float *grads, float *m1, float *m2, float lr, float b1, float b2, float eps,
             int32_t t, float scale, cudaStream_t st);
int mlp_param_count();
int ensemble_bin(const pg_ensemble *e, pg_particles *p, pg_cells *cells, pg_workspace ws, pg_status *status,
                 cudaStream_t st);
int ensemble_build_lists(const pg_ensemble *e, pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
                         double r_list2, pg_status *status, cudaStream_t st);
int ensemble_force(const pg_ensemble *e, const pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                   pg_workspace ws, cudaStream_t st);
int ensemble_integrate(const pg_ensemble *e, pg_particles *p, double dt, int kicks, int drift, double half_skin2,
                       int32_t step, pg_status *status, cudaStream_t st);
int ensemble_thermo(const pg_ensemble *e, const pg_particles *p, double *out, cudaStream_t st);
int ensemble_select(const pg_ensemble *e, const pg_particles *p, double thresh2, int32_t *rebuild, cudaStream_t st);
int ensemble_steps(const pg_ensemble *e, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                   double dt, double half_skin2, int32_t first, int32_t nsteps, pg_status *status, pg_workspace ws,
                   double timeout_s, cudaStream_t st);
int lj_steps(const pg_box *box, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj, double dt,
             double half_skin2, int32_t first, int32_t nsteps, pg_status *status, pg_workspace ws, double timeout_s,
             cudaStream_t st);
int grid_barrier_check(int32_t extra_arrivals, double timeout_s, pg_status *status, pg_workspace ws, cudaStream_t st);
int64_t pair_slots(int32_t n, int32_t ncells);
int64_t vtk_workspace_bytes(int32_t rows);
int vtk_format_rows(int what, int32_t rows, const int32_t *order, const double *pos, const double *mass,
                    const int32_t *index, pg_workspace ws, cudaStream_t st);
int vtk_pack_rows(int32_t rows, pg_workspace ws, const int64_t *offset, char *out, cudaStream_t st);
int64_t csv_count_bytes(int64_t bytes);
int dem_sc_grid_size(double xmax, double ymax, double zmax, double spacing, double diameter, const double *lo,
                     const double *hi, int64_t *npoints, int64_t *nkept, int64_t *ws_bytes);
int dem_sc_grid(double xmax, double ymax, double zmax, double spacing, double diameter, double min_diameter,
                double max_diameter, double initial_velocity, double density, int ntypes, const double *lo,
                const double *hi, double *pos, double *vel, double *mass, double *radius, int32_t *type,
                int32_t *uid, int64_t capacity, pg_workspace ws, cudaStream_t st);
int csv_count_lines(const char *text, int64_t bytes, int64_t *lines, pg_workspace ws, cudaStream_t st);
int64_t csv_workspace_bytes(int64_t bytes, int64_t lines, int32_t nfields);
int csv_parse(const char *text, int64_t bytes, int64_t lines, int32_t nfields, const int32_t *kinds, int32_t pos_field,
              int32_t flags_field, const double *domain_lo, const double *domain_hi, double *table, int32_t max_rows,
              pg_csv_result *result, pg_workspace ws, cudaStream_t st);
int dem_setup(pg_dem_particles *d, const pg_dem_params *prm, cudaStream_t st);
int dem_bin(const pg_box *box, pg_dem_particles *d, const pg_dem_particles *spare, const pg_contacts *c,
            const pg_contacts *spare_c, pg_cells *cells, pg_workspace ws, pg_status *status, cudaStream_t st);
int dem_build_list(const pg_box *box, pg_dem_particles *d, const pg_cells *cells, pg_neighbor_list *list,
                   const pg_dem_params *prm, pg_status *status, cudaStream_t st);
int dem_force(const pg_box *box, const pg_dem_particles *d, const pg_cells *cells, const pg_neighbor_list *list,
              const pg_contacts *c, const pg_dem_params *prm, int precision, pg_status *status, cudaStream_t st);
int dem_euler(pg_dem_particles *d, const pg_dem_params *prm, int precision, double half_skin2, int32_t step, pg_status *status,
              cudaStream_t st);
}  // namespace pg

unsigned long long pg::g_kernel_launches = 0;

static inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" {

int pg_version(void) { return 1; }

int64_t pg_kernel_launches(void) { return (int64_t) __atomic_load_n(&pg::g_kernel_launches, __ATOMIC_RELAXED); }

int pg_struct_sizes(int64_t *out, int n) {
    const int64_t sizes[] = {
        (int64_t) sizeof(pg_status), (int64_t) sizeof(pg_box), (int64_t) sizeof(pg_particles),
        (int64_t) sizeof(pg_cells), (int64_t) sizeof(pg_neighbor_list), (int64_t) sizeof(pg_lj_params),
        (int64_t) sizeof(pg_workspace), (int64_t) sizeof(pg_dem_particles), (int64_t) sizeof(pg_contacts),
        (int64_t) sizeof(pg_dem_params), (int64_t) sizeof(pg_replica), (int64_t) sizeof(pg_ensemble),
        (int64_t) sizeof(pg_csv_result),
    };
    const int m = (int) (sizeof(sizes) / sizeof(sizes[0]));
    if(out == nullptr) { return m; }
    for(int k = 0; k < n && k < m; k++) { out[k] = sizes[k]; }
    return m;
}

const int32_t *pg_bin_permutation(int32_t n, int32_t ncells, pg_workspace ws) {
    return pg::bin_permutation(n, ncells, ws);
}

int64_t pg_workspace_bytes(int32_t n, int32_t ncells) {
    const int64_t a = pg::bin_workspace_bytes(n, ncells);
    const int64_t b = pg::thermo_workspace_bytes();
    return a > b ? a : b;
}

int pg_bin_particles(const pg_box *box, pg_particles *p, pg_cells *cells, pg_workspace ws,
                     pg_status *status, void *stream) {
    return pg::bin_particles(box, p, cells, ws, status, S(stream), nullptr);
}

int pg_build_neighbor_lists(const pg_box *box, const pg_particles *p, const pg_cells *cells,
                            pg_neighbor_list *list, double r_list2, pg_status *status, void *stream) {
    return pg::build_neighbor_lists(box, p, cells, list, r_list2, status, S(stream));
}

int pg_lj_force(const pg_box *box, const pg_particles *p, const pg_cells *cells,
                const pg_neighbor_list *list, const pg_lj_params *lj, int precision, int sync_mode,
                double *energy, pg_workspace ws, void *stream) {
    return pg::lj_force(box, p, cells, list, lj, precision, sync_mode, energy, ws, S(stream));
}

int pg_lj_steps(const pg_box *box, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj, double dt,
                double half_skin2, int32_t first_step, int32_t nsteps, pg_status *status, pg_workspace ws,
                double barrier_timeout_s, void *stream) {
    return pg::lj_steps(box, p, list, lj, dt, half_skin2, first_step, nsteps, status, ws, barrier_timeout_s, S(stream));
}

int pg_grid_barrier_check(int32_t extra_arrivals, double timeout_s, pg_status *status, pg_workspace ws,
                          void *stream) {
    return pg::grid_barrier_check(extra_arrivals, timeout_s, status, ws, S(stream));
}

int pg_initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision,
                         double half_skin2, int32_t step, int sync_mode, pg_status *status,
                         void *stream) {
    return pg::initial_integrate(box, p, dt, precision, half_skin2, step, status, sync_mode, S(stream));
}

int pg_final_integrate(const pg_box *box, pg_particles *p, double dt, int precision, void *stream) {
    return pg::final_integrate(box, p, dt, precision, S(stream));
}

int pg_final_initial_integrate(const pg_box *box, pg_particles *p, double dt, int precision,
                               double half_skin2, int32_t step, int sync_mode, pg_status *status,
                               void *stream) {
    return pg::final_initial_integrate(box, p, dt, precision, half_skin2, step, status, sync_mode,
                                       S(stream));
}

int pg_integrate_mixed(const pg_box *box, pg_particles *p, double dt, int kicks, int drift,
                       double half_skin2, int32_t step, pg_status *status, void *stream) {
    return pg::integrate_mixed(box, p, dt, kicks, drift, half_skin2, step, status, S(stream));
}

int pg_compute_thermo(const pg_box *box, const pg_particles *p, double *out, pg_workspace ws,
                      void *stream) {
    if(ws.ptr == nullptr || ws.bytes < pg::thermo_workspace_bytes()) { return PG_ERR_ARGUMENT; }
    return pg::compute_thermo(box, p, out, (double *) ws.ptr, S(stream));
}

int pg_split_positions(const pg_box *box, pg_particles *p, void *stream) {
    return pg::split_positions(box, p, S(stream));
}

int pg_permute(int32_t n, const int32_t *perm, const void *src, void *dst, int elem_bytes, void *stream) {
    if(n < 0 || (n > 0 && (!perm || !src || !dst)) || src == dst) { return PG_ERR_ARGUMENT; }
    if(n == 0) { return PG_OK; }
    return pg::gather_array(n, perm, src, dst, elem_bytes, S(stream));
}

int pg_mlp_param_count(void) { return pg::mlp_param_count(); }

int pg_ensemble_bin(const pg_ensemble *e, pg_particles *p, pg_cells *cells, pg_workspace ws, pg_status *status,
                    void *stream) {
    return pg::ensemble_bin(e, p, cells, ws, status, S(stream));
}

int pg_ensemble_build_lists(const pg_ensemble *e, pg_particles *p, const pg_cells *cells, pg_neighbor_list *list,
                            double r_list2, pg_status *status, void *stream) {
    return pg::ensemble_build_lists(e, p, cells, list, r_list2, status, S(stream));
}

int pg_ensemble_force(const pg_ensemble *e, const pg_particles *p, const pg_neighbor_list *list,
                      const pg_lj_params *lj, pg_workspace ws, void *stream) {
    return pg::ensemble_force(e, p, list, lj, ws, S(stream));
}

int pg_ensemble_integrate(const pg_ensemble *e, pg_particles *p, double dt, int kicks, int drift,
                          double half_skin2, int32_t step, pg_status *status, void *stream) {
    return pg::ensemble_integrate(e, p, dt, kicks, drift, half_skin2, step, status, S(stream));
}

int pg_ensemble_steps(const pg_ensemble *e, pg_particles *p, const pg_neighbor_list *list, const pg_lj_params *lj,
                      double dt, double half_skin2, int32_t first, int32_t nsteps, pg_status *status,
                      pg_workspace ws, double timeout_s, void *stream) {
    return pg::ensemble_steps(e, p, list, lj, dt, half_skin2, first, nsteps, status, ws, timeout_s, S(stream));
}

int pg_ensemble_select(const pg_ensemble *e, const pg_particles *p, double thresh2, int32_t *rebuild, void *stream) {
    return pg::ensemble_select(e, p, thresh2, rebuild, S(stream));
}

int pg_ensemble_thermo(const pg_ensemble *e, const pg_particles *p, double *out, void *stream) {
    return pg::ensemble_thermo(e, p, out, S(stream));
}

int pg_dem_setup(pg_dem_particles *d, const pg_dem_params *prm, void *stream) {
    return pg::dem_setup(d, prm, S(stream));
}

int pg_dem_bin(const pg_box *box, pg_dem_particles *d, const pg_dem_particles *spare, const pg_contacts *c,
               const pg_contacts *spare_c, pg_cells *cells, pg_workspace ws, pg_status *status, void *stream) {
    return pg::dem_bin(box, d, spare, c, spare_c, cells, ws, status, S(stream));
}

int pg_dem_build_list(const pg_box *box, pg_dem_particles *d, const pg_cells *cells, pg_neighbor_list *list,
                      const pg_dem_params *prm, pg_status *status, void *stream) {
    return pg::dem_build_list(box, d, cells, list, prm, status, S(stream));
}

int pg_dem_force(const pg_box *box, const pg_dem_particles *d, const pg_cells *cells,
                 const pg_neighbor_list *list, const pg_contacts *c, const pg_dem_params *prm,
                 int precision, pg_status *status, void *stream) {
    return pg::dem_force(box, d, cells, list, c, prm, precision, status, S(stream));
}

int pg_dem_euler(pg_dem_particles *d, const pg_dem_params *prm, int precision, double half_skin2, int32_t step,
                 pg_status *status, void *stream) {
    return pg::dem_euler(d, prm, precision, half_skin2, step, status, S(stream));
}

int pg_cell_features(const pg_particles *p, const pg_cells *cells, int precision, int32_t steps_since_build,
                     double dt, double half_skin, float *features, void *stream) {
    return pg::cell_features(p, cells, nullptr, precision, steps_since_build, dt, half_skin, features, S(stream));
}

int pg_cell_features_binned(const pg_particles *p, const pg_cells *cells, const int32_t *perm, int precision,
                            int32_t steps_since_build, double dt, double half_skin, float *features, void *stream) {
    if(!perm) { return PG_ERR_ARGUMENT; }
    return pg::cell_features(p, cells, perm, precision, steps_since_build, dt, half_skin, features, S(stream));
}

int pg_cell_select(const float *features, int32_t ncells, int32_t k, float *out, void *stream) {
    return pg::cell_select(features, ncells, k, out, S(stream));
}

int pg_mlp_forward(const float *params, const float *features, int32_t ncells, float *out, void *stream) {
    return pg::mlp_forward(params, features, ncells, out, S(stream));
}

int pg_mlp_softmin(const float *out, int32_t ncells, float temperature, float *result, void *stream) {
    return pg::mlp_softmin(out, ncells, temperature, result, S(stream));
}

int pg_mlp_backward(const float *params, const float *features, const float *out, int32_t ncells,
                    const float *result, float target_log, int censored, float temperature, float *grads,
                    float *loss, void *stream) {
    return pg::mlp_backward(params, features, out, ncells, result, target_log, censored, temperature, grads,
                            loss, S(stream));
}

int pg_mlp_adam(float *params, float *grads, float *m1, float *m2, float lr, float beta1, float beta2,
                float eps, int32_t t, float grad_scale, void *stream) {
    return pg::mlp_adam(params, grads, m1, m2, lr, beta1, beta2, eps, t, grad_scale, S(stream));
}

int64_t pg_pair_slots(int32_t n, int32_t ncells) { return pg::pair_slots(n, ncells); }

int64_t pg_vtk_workspace_bytes(int32_t rows) { return pg::vtk_workspace_bytes(rows); }

int pg_vtk_format_rows(int section, int32_t rows, const int32_t *order, const double *pos, const double *mass,
                       const int32_t *index, pg_workspace ws, void *stream) {
    return pg::vtk_format_rows(section, rows, order, pos, mass, index, ws, S(stream));
}

int pg_vtk_pack_rows(int32_t rows, pg_workspace ws, const int64_t *offsets, char *out, void *stream) {
    return pg::vtk_pack_rows(rows, ws, offsets, out, S(stream));
}

int64_t pg_csv_count_bytes(int64_t bytes) { return pg::csv_count_bytes(bytes); }

int pg_csv_count_lines(const char *text, int64_t bytes, int64_t *lines, pg_workspace ws, void *stream) {
    return pg::csv_count_lines(text, bytes, lines, ws, S(stream));
}

int64_t pg_csv_workspace_bytes(int64_t bytes, int64_t lines, int32_t nfields) {
    return pg::csv_workspace_bytes(bytes, lines, nfields);
}

int pg_csv_parse(const char *text, int64_t bytes, int64_t lines, int32_t nfields, const int32_t *kinds,
                 int32_t pos_field, int32_t flags_field, const double *domain_lo, const double *domain_hi,
                 double *table, int32_t max_rows, pg_csv_result *result, pg_workspace ws, void *stream) {
    return pg::csv_parse(text, bytes, lines, nfields, kinds, pos_field, flags_field, domain_lo, domain_hi, table,
                         max_rows, result, ws, S(stream));
}

int pg_dem_sc_grid_size(double xmax, double ymax, double zmax, double spacing, double diameter, const double *lo,
                        const double *hi, int64_t *npoints, int64_t *nkept, int64_t *ws_bytes) {
    return pg::dem_sc_grid_size(xmax, ymax, zmax, spacing, diameter, lo, hi, npoints, nkept, ws_bytes);
}

int pg_dem_sc_grid(double xmax, double ymax, double zmax, double spacing, double diameter, double min_diameter,
                   double max_diameter, double initial_velocity, double density, int32_t ntypes, const double *lo,
                   const double *hi, double *pos, double *vel, double *mass, double *radius, int32_t *type,
                   int32_t *uid, int64_t capacity, pg_workspace ws, void *stream) {
    return pg::dem_sc_grid(xmax, ymax, zmax, spacing, diameter, min_diameter, max_diameter, initial_velocity, density,
                           ntypes, lo, hi, pos, vel, mass, radius, type, uid, capacity, ws, S(stream));
}

int pg_stream_sync(void *stream) {
    return cudaStreamSynchronize(S(stream)) == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

}  // extern "C"
