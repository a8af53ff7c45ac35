/*
 * pgdg_oracle.h -- C interface of the FP64 CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a serial, canonical-order restatement
 * of the reference's per-time-step particle-grid path
 * (3D_generalized/PGDG_3D_spheric: mpm.cpp, particle_flow.cpp, particle.cpp,
 * level_infor.cpp, cell_list.cpp, mpm_ini.cpp:682-766).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
 * only as the checker.  The product (libpgdg_gpu.so) never links it.
 *
 * The entry points mirror the GPU library's (include/pgdg.h) one to one, with
 * the prefix po_ instead of pgdg_, so tests can swap implementations.
 */
#ifndef PGDG_ORACLE_H
#define PGDG_ORACLE_H
#include "../include/pgdg_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct po_ctx po_ctx;

/* the oracle's own construction of the synthetic workloads (oracle_case.cpp),
 * bit-identical to pgdg_case_setup / _particles / _cells of the GPU library */
int po_case_setup(int config_id, const int32_t* ncell, pgdg_case* out);
int64_t po_case_num_particles(const pgdg_case* cs);
int po_case_particles(const pgdg_case* cs, int config_id, uint64_t seed, pgdg_particles* out);
int po_case_cells(const pgdg_case* cs, pgdg_cells* out);

int po_create(const pgdg_case* cs, po_ctx** out);
int po_destroy(po_ctx* ctx);
int po_set_threads(int n);

int po_upload_particles(po_ctx* ctx, const pgdg_particles* p);
int po_download_particles(po_ctx* ctx, pgdg_particles* p);  /* p->n in: capacity, out: count */
int po_num_particles(po_ctx* ctx, int64_t* n);
int po_upload_cells(po_ctx* ctx, const pgdg_cells* c);
int po_download_cells(po_ctx* ctx, pgdg_cells* c);
/* neighbour lists in canonical index space: entry >= 0 fluid index,
 * -1 dead particle, -(2+b) boundary particle b.  off has n+1 entries. */
int po_upload_lists(po_ctx* ctx, const int64_t* off, const int64_t* ent);
int po_download_lists(po_ctx* ctx, int64_t* off, int64_t* ent, int64_t cap, int64_t* total);
/* cell lists (Cell_list::particle_list) in the same encoding */
int po_download_cell_lists(po_ctx* ctx, int64_t* off, int64_t* ent, int64_t cap, int64_t* total);

int po_set_dt(po_ctx* ctx, double dt);
int po_set_iterate(po_ctx* ctx, int64_t iterate_num);
int po_set_max_v(po_ctx* ctx, double max_v);
int po_get_stats(po_ctx* ctx, pgdg_stats* st);

/* reference methods (MPM::*) */
int po_set_timestep(po_ctx* ctx, double* dt, double* max_v);
int po_used_state_update(po_ctx* ctx);
int po_bin_particles(po_ctx* ctx);           /* Reset_cell_list_info + Map_the_particle_to_tree */
int po_split_particle_fast(po_ctx* ctx);
int po_merge_particle_fast(po_ctx* ctx);
int po_refresh_membership(po_ctx* ctx);      /* Reset/Refresh_neighbor_info(4) */
int po_refresh_neighbors(po_ctx* ctx);       /* Reset/Refresh_neighbor_info(2) */
int po_mls_p2g(po_ctx* ctx);
int po_calculate_limiter(po_ctx* ctx);
int po_grid_acceleration(po_ctx* ctx);
int po_update_grid(po_ctx* ctx, int md);
int po_update_particle(po_ctx* ctx, int md);
int po_run_step(po_ctx* ctx, int64_t n);     /* MPM_run_simulation */
/* Solver::MPM_Solver without output clipping: set_timestep, ++iterate, run_step */
int po_advance(po_ctx* ctx, int nsteps);
int po_totals(po_ctx* ctx, double* out);     /* [F particle mass, particle E, F cell mass, cell E] */
int po_output_point(po_ctx* ctx, double* out5); /* Output_point: bubble extents, phase-2 mass, count */
/* Output_plt_file: Tecplot binary of the particles, ASCII table of the cells (either path may be NULL) */
int po_output_plt(po_ctx* ctx, const char* particle_path, const char* cell_path);

/* batched MGFM with an explicit material table (gamma[m], pinf[m]) */
int po_mgfm_batched(const double* in6, const int8_t* mat2, const double* gam, const double* pinf,
                    int variant, const double* seed, double* out3, int32_t* iters, int64_t n);
double po_root_d(double x, int d);

#ifdef __cplusplus
}
#endif
#endif
