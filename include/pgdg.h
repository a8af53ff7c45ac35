/*
 * pgdg.h -- C ABI of libpgdg_gpu.so, the GB300-native per-time-step
 * particle-grid path of the Particle-Grid DG method (reference: PGDG_p2,
 * program 3D_generalized/PGDG_3D_spheric; file:line citations below are
 * relative to that program unless another program is named).
 *
 * The reference has no plugin or FFI: its boundary is the MPM method set that
 * the driver calls (mpm.h:160-194) with all state inside the MPM object.  Each
 * entry point below replaces one of those methods; the state lives in an opaque
 * context on one GPU.  Every function returns PGDG_OK (0) or a negative
 * PGDG_E* code; pgdg_last_error() describes the last failure.  Calls on one
 * context are stream-ordered and not re-entrant; separate contexts are
 * independent.
 */
#ifndef PGDG_H
#define PGDG_H
#include "pgdg_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pgdg_ctx pgdg_ctx;

/* precision of the grid/particle arithmetic:
 *   FP64      all FP64, evaluated in the oracle's operation order without FMA
 *             contraction (bit-identical to the CPU restatement of the reference)
 *   MIXED     FP32 residual/limiter/G2P/shifting, FP64 MGFM Newton and P2G sums
 *   FP64_FMA  all FP64 with FMA contraction (the plain FP64 GPU path timed
 *             against MIXED) */
enum { PGDG_PREC_FP64 = 0, PGDG_PREC_MIXED = 1, PGDG_PREC_FP64_FMA = 2 };

/* ---- case construction (replaces MPM::Initialize_case, mpm_ini.cpp:33-673) ----
 * config_id 1..4 are the synthetic workloads: 1 2D triple point 112x48,
 * 2 3D cylinder shock-bubble 256x64x64, 3 3D sphere shock-bubble 384x96x96,
 * 4 2D underwater explosion 1024^2.  ncell (may be NULL) overrides the grid. */
int pgdg_case_setup(int config_id, const int32_t* ncell, pgdg_case* out);
int64_t pgdg_case_num_particles(const pgdg_case* cs);
int pgdg_case_particles(const pgdg_case* cs, int config_id, uint64_t seed, pgdg_particles* out);
int pgdg_case_cells(const pgdg_case* cs, pgdg_cells* out);

/* ---- context ---- */
/* MPM::MPM + allocation; capacity = max fluid particles held (0 = automatic).
 * PGDG_EINVAL without touching the GPU for a case it cannot hold: a cell count
 * below 1 on an axis, or (MIXED and FP64_FMA, whose shifting kernel sorts
 * each row of cells with 16-bit cell offsets) more than 65535 cells along the
 * last axis. */
int pgdg_create(const pgdg_case* cs, int precision, int64_t capacity, pgdg_ctx** out);
int pgdg_destroy(pgdg_ctx* ctx);
const char* pgdg_last_error(pgdg_ctx* ctx);
/* MPM::Initialize_case (mpm_ini.cpp:33-673; fluid particles mpm_ini.cpp:170-294,
 * cells mpm_ini.cpp:299-346) on the device: workload config_id is built in
 * place into a context created for the case pgdg_case_setup(config_id, ...)
 * returned, with no host arrays and no upload.  The state equals
 * pgdg_case_particles (same seed) and pgdg_case_cells followed by the two
 * uploads, bit for bit. */
int pgdg_case_build(pgdg_ctx* ctx, int config_id, uint64_t seed);
int pgdg_capacity(pgdg_ctx* ctx, int64_t* cap);

/* ---- data movement (host arrays, canonical particle order) ---- */
int pgdg_upload_particles(pgdg_ctx* ctx, const pgdg_particles* p);
int pgdg_download_particles(pgdg_ctx* ctx, pgdg_particles* p); /* p->n: in capacity, out count */
int pgdg_num_particles(pgdg_ctx* ctx, int64_t* n);
int pgdg_upload_cells(pgdg_ctx* ctx, const pgdg_cells* c);
int pgdg_download_cells(pgdg_ctx* ctx, pgdg_cells* c);
/* Particle_base::neighbor lists, canonical index space (>=0 fluid index,
 * -1 dead particle, -(2+b) boundary particle b); stored[i] says whether the
 * device holds particle i's list (it keeps only the lists split/merge read). */
int pgdg_upload_lists(pgdg_ctx* ctx, const int64_t* off, const int64_t* ent);
int pgdg_download_lists(pgdg_ctx* ctx, int64_t* off, int64_t* ent, int32_t* stored, int64_t cap,
                        int64_t* total);
/* Cell_list::particle_list of every cell (cell_list.h), same encoding */
int pgdg_download_cell_lists(pgdg_ctx* ctx, int64_t* off, int64_t* ent, int64_t cap, int64_t* total);

int pgdg_set_dt(pgdg_ctx* ctx, double dt);                 /* Solver clip of glbl_timestep (solver.cpp:40-44) */
int pgdg_set_iterate(pgdg_ctx* ctx, int64_t iterate_num);
int pgdg_set_max_v(pgdg_ctx* ctx, double max_v);
int pgdg_get_stats(pgdg_ctx* ctx, pgdg_stats* st);
int pgdg_synchronize(pgdg_ctx* ctx);

/* ---- reference methods ---- */
int pgdg_set_timestep(pgdg_ctx* ctx, double* dt, double* max_v);   /* MPM::Set_timestep mpm.cpp:19-57 */
int pgdg_used_state_update(pgdg_ctx* ctx);                         /* mpm.cpp:184-263 */
int pgdg_bin_particles(pgdg_ctx* ctx);                             /* Reset_cell_list_info + Map_the_particle_to_tree mpm.cpp:65-96 */
int pgdg_split_particle_fast(pgdg_ctx* ctx);                       /* mpm.cpp:1036-1417 */
int pgdg_merge_particle_fast(pgdg_ctx* ctx);                       /* mpm.cpp:1536-1706 (one pass) */
int pgdg_refresh_membership(pgdg_ctx* ctx);                        /* Reset/Refresh_neighbor_info(4) mpm.cpp:101-161 */
int pgdg_refresh_neighbors(pgdg_ctx* ctx);                         /* Reset/Refresh_neighbor_info(2) level_infor.cpp:153-195 */
int pgdg_mls_p2g(pgdg_ctx* ctx);                                   /* MPM::MLS_P2G mpm.cpp:274-382 */
int pgdg_calculate_limiter(pgdg_ctx* ctx);                         /* mpm.cpp:392-738 */
int pgdg_grid_acceleration(pgdg_ctx* ctx);                         /* mpm.cpp:747-763 -> particle_flow.cpp:16-405 */
int pgdg_update_grid(pgdg_ctx* ctx, int md);                       /* mpm.cpp:768-830 */
int pgdg_update_particle(pgdg_ctx* ctx, int md);                   /* mpm.cpp:839-853 -> particle_flow.cpp:413-622 */
int pgdg_run_step(pgdg_ctx* ctx, int64_t n);                       /* MPM::MPM_run_simulation mpm_ini.cpp:682-766 */
/* Solver::MPM_Solver (solver.cpp:30-64) without output clipping:
 * nsteps x {Set_timestep, ++iterate_num, MPM_run_simulation}, all on device */
int pgdg_advance(pgdg_ctx* ctx, int nsteps);
/* conservation totals (Triple_point_2phase/mpm_ini.cpp:599-654): particle mass
 * per phase, particle energy, cell mass per phase, cell energy; each summed in
 * double-double and rounded once, so the result does not depend on the order
 * of the addends */
int pgdg_totals(pgdg_ctx* ctx, double* out6);
/* MPM::Output_point (mpm_ini.cpp:774-824) on the device: out5 = the largest and
 * smallest x of the phase-2 particles near the axis (y, z < 2.5 p_sz: the
 * bubble's downstream end and the jet), the smallest x of those away from it
 * (y or z > 4 p_sz: the upstream end), the phase-2 mass sum rho vol, and the
 * number of fluid particles (the rows of pointa.txt and mass.txt); the ends
 * start at the box's left and right x */
int pgdg_output_point(pgdg_ctx* ctx, double* out5);
/* MPM::Output_plt_file (mpm_ini.cpp:832-980): the live particles as a Tecplot
 * binary (#!TDV112, one ordered zone of twelve variables x y z phase vx vy vol
 * rho P |tv| |v| n_neighbor, doubles with phase and n_neighbor int32, stored
 * variable after variable in canonical order) and the cells as the ASCII table
 * (centre, v1 v2 |v|, rho0 rho1, coef[0](1,1) coef[0](1,2), Lim_u[0](0)
 * Lim_u[1](0), alph0 alph1, P; one line per cell, i outer); either path may be
 * NULL.  The solution time is the context's simulated time.  n_neighbor is the
 * flag-2 list size (fluid and boundary particles within 2h, itself included)
 * over the last stage's search coordinates, or the current ones when the
 * particle set changed since.  The state is packed on the device into a
 * snapshot; with async = 0 the call returns once both files are written, with
 * async = 1 as soon as the snapshot is packed, a host thread copying it out and
 * writing while later calls go on (pgdg_output_wait joins it and returns its
 * status; the next pgdg_output_plt and pgdg_destroy wait for it too). */
int pgdg_output_plt(pgdg_ctx* ctx, const char* particle_path, const char* cell_path, int async);
int pgdg_output_wait(pgdg_ctx* ctx);

/* ---- MGFM seed surrogate (new; the reference starts Newton from max(p_l,p_r),
 *      mpm.cpp:893) ----
 * A 12-64-64-64-2 tanh MLP predicting the star pressure and velocity of a
 * two-material Riemann problem, FP32 accumulation.  bf16 = 1: BF16 weights,
 * FP32 activations (CUDA cores); 0: FP32 weights (gradient checks); 2: BF16
 * weights and activations on the tensor cores (tcgen05) for forward passes,
 * training as mode 1.  Parameters are
 * pgdg_surrogate_num_params() floats: weights, biases and the fixed
 * feature/target normalisation.  Array arguments are device pointers unless
 * named *_host. */
typedef struct pgdg_mlp pgdg_mlp;
int pgdg_surrogate_create(int bf16, pgdg_mlp** out);
int pgdg_surrogate_destroy(pgdg_mlp* net);
int pgdg_surrogate_num_params(void);
int pgdg_surrogate_set_params(pgdg_mlp* net, const float* params_host);
int pgdg_surrogate_get_params(pgdg_mlp* net, float* params_host);
int pgdg_surrogate_features(const double* in6, const int8_t* mat2, const double* gam, const double* pinf, float* X,
                            int64_t n);
int pgdg_surrogate_forward(pgdg_mlp* net, const float* X, float* Y, int64_t n);
int pgdg_surrogate_gradients(pgdg_mlp* net, const float* X, const float* T, int64_t n, float* grad_host,
                             double* loss);
int pgdg_surrogate_train_step(pgdg_mlp* net, const float* X, const float* T, int64_t n, float lr, double* loss);
/* attach a surrogate to a context: the mixed-precision step then seeds every
 * interface MGFM solve with it (NULL detaches).  Attaching turns the interface
 * queue on.  Not available on the exact-order FP64 path (PGDG_EINVAL). */
int pgdg_set_surrogate(pgdg_ctx* ctx, pgdg_mlp* net);
/* interface queue (no reference counterpart: MPM::Grid_acceleration calls
 * MGFM inline, particle_flow.cpp:192-204): the residual gathers each stage's
 * two-material interface problems into one batch, solves them together and
 * reads the ghost states back.  Mixed and FP64_FMA paths only. */
int pgdg_set_iface_queue(pgdg_ctx* ctx, int on);
/* copy the last stage's queued problems to the host (in6 n x 6, mat2 n x 2,
 * at most cap entries); *n receives the queue length */
int pgdg_iface_download(pgdg_ctx* ctx, double* in6, int8_t* mat2, int64_t cap, int64_t* n);

/* ---- MGFM interface Riemann solve (mpm.cpp:882-926), batched ----
 * in6: n x (u_l, u_r, p_l, p_r, rho_l, rho_r); mat2: n x (material l, material r)
 * into gam/pinf (nmat entries); out3: n x (rho*_L, p*, u*); iters may be NULL.
 * net == NULL starts Newton from the reference's plain seed; otherwise from the
 * surrogate's prediction, falling back to the plain solve when the seeded one
 * does not converge.  Device pointers; the default stream. */
int pgdg_mgfm_batched(const pgdg_mlp* net, const double* in6, const int8_t* mat2, const double* gam,
                      const double* pinf, int nmat, int variant, double* out3, int32_t* iters, int64_t n);

/* ---- batched MGFM that allocates nothing (no counterpart in the reference) ----
 * The same solve and results as pgdg_mgfm_batched, for callers that cannot
 * allocate device memory: a host driver whose own pool already holds the free
 * device memory (cudaMalloc would fail there), and per-stage callers that
 * cannot absorb the device-wide synchronisation of cudaFree (the allocating
 * entry point frees and regrows its seed buffer when a batch outgrows it).
 * The per-problem seeds live in a fixed device array of
 * PGDG_MGFM_NOALLOC_MAX entries (8 MiB); a larger n returns PGDG_EOVERFLOW
 * before anything is launched.  Nothing in that array is read before it is
 * written, so nothing is cleared.  The first call on a device looks the array
 * up (cudaGetSymbolAddress) and should come before any stream capture.  The
 * address is kept for the life of the process: do not call this entry point
 * again on a device after cudaDeviceReset (or any other teardown of its
 * primary context) in the same process.
 * Overlapping calls on one device (several host threads, or per-thread default
 * streams) share the array and race: serialise them.  A tensor-core network
 * (pgdg_surrogate_create mode 2) is refused (PGDG_EINVAL): its seeds differ from
 * the CUDA-core network this entry point evaluates.  Device pointers; the
 * default stream. */
#define PGDG_MGFM_NOALLOC_MAX (1 << 20)
int pgdg_mgfm_batched_noalloc(const pgdg_mlp* net, const double* in6, const int8_t* mat2, const double* gam,
                              const double* pinf, int nmat, int variant, double* out3, int32_t* iters, int64_t n);

/* ---- CUDA graphs of whole steps (no reference counterpart) ----
 * pgdg_advance replays captured graphs of three steps (one per rotation of
 * the coordinate buffers) when a step reads nothing back on the host: not at
 * the first iteration, not while per-method timing is on, not before the
 * shifting kernel's variant is tuned.  With the interface queue (and the seed
 * surrogate) the stage's problem count stays on the device and sizes the
 * batch there; between calls the host grows the queue when a stage passed half
 * of it, and a stage that outgrows it is solved inline.  Results equal the
 * eager steps bit for bit.  on = 0 runs every step eagerly.  Uploads, queue
 * growth and changes of surrogate, queue or kernel variant drop the graphs. */
int pgdg_set_graphs(pgdg_ctx* ctx, int on);

/* ---- kernel variants (no reference counterpart) ----
 * Some kernels have several implementations with identical results; the
 * context times them on its own state at their first call and keeps the
 * fastest.  kernel: "pst" (the shifting kernel of pgdg_update_particle).
 * variant >= 0 forces that variant, -1 re-tunes at the next call, -2 only
 * queries; *chosen (may be NULL) receives the current choice (-1: not tuned).
 * kernel "p2g_skip": 1 (default) lets pgdg_mls_p2g skip neighbour cells beyond
 * its cut radius while every particle still lies in its bucket's cell (from
 * pgdg_bin_particles until particles move); 0 always visits all 3^d cells.
 * Both give identical sums.  "iface_cap": variant >= 0 fixes the interface
 * queue's capacity at that many problems (a stage beyond it is solved inline;
 * a memory bound for large cases), -1 returns to automatic growth. */
int pgdg_tune(pgdg_ctx* ctx, const char* kernel, int variant, int* chosen);

/* ---- measurement ----
 * pgdg_profile: record CUDA events on the context stream around every method
 * call; pgdg_profile_read returns per-method totals (names ';'-separated, in
 * first-seen order), pgdg_launch_count the number of kernels launched so far,
 * pgdg_time_advance the device time of nsteps steps (events on the context
 * stream, synchronised on both sides). */
int pgdg_profile(pgdg_ctx* ctx, int enable);
int pgdg_profile_read(pgdg_ctx* ctx, char* names, int names_cap, double* ms, int64_t* counts, int cap, int* n);
int pgdg_launch_count(pgdg_ctx* ctx, int64_t* n);
int pgdg_time_advance(pgdg_ctx* ctx, int nsteps, double* ms);
/* the FP32 fused multiply-add rate of the current device, measured by timing
 * independent FFMA chains on every SM with CUDA events (the roofline
 * denominator of the FP32-bound kernels); *ms (may be NULL) receives the
 * timed launch's duration */
int pgdg_fp32_peak(double* tflops, double* ms);
/* the same with the chains as packed pairs (FFMA2, two FP32 multiply-adds per
 * instruction) */
int pgdg_fp32_peak_packed(double* tflops, double* ms);

#ifdef __cplusplus
}
#endif
#endif
