/*
 * pgdg_types.h -- plain-C data formats shared by the GPU library (libpgdg_gpu.so)
 * and the CPU oracle.  Only layouts live here; no algorithm.
 *
 * The layouts mirror the reference's per-particle / per-cell fields
 * (3D_generalized/PGDG_3D_spheric/particle.h:9-106, mpm.h:36-48,52-195) as
 * structure-of-arrays, all FP64 at the boundary.  A device context may store
 * some fields in FP32 internally (mixed precision); the boundary is always FP64.
 */
#ifndef PGDG_TYPES_H
#define PGDG_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGDG_MAX_FLD 3          /* the largest FldNum of a build (glbparam.h:41: 2; Triple_point_3phase: 3) */
#define PGDG_PHASE_BOUNDARY 10  /* boundary particle phase (mpm_ini.cpp:586) */

/* error codes returned by every entry point */
enum {
  PGDG_OK = 0,
  PGDG_EINVAL = -1,
  PGDG_ENOMEM = -2,
  PGDG_ECUDA = -3,
  PGDG_ENONFINITE = -4,
  PGDG_ETIMEOUT = -5,
  PGDG_EOVERFLOW = -6,
  PGDG_ESTATE = -7
};

/* Boundary kind of a domain side.  The 3D_generalized program tags faces with
 * b_mk (mpm_ini.cpp:448-545): 0 interior, 1 wall, -1 inlet (prescribed state),
 * -2 outlet, -3 symmetry.  -4 is the underwater-explosion program's zero-gradient
 * side (2D_cases/PGDG_underwater_explosion/particle_flow.cpp:312-330), which has
 * no lateral velocity mirroring. */
enum {
  PGDG_BC_INTERIOR = 0,
  PGDG_BC_WALL = 1,
  PGDG_BC_INLET = -1,
  PGDG_BC_OUTLET = -2,
  PGDG_BC_SYMMETRY = -3,
  PGDG_BC_TRANSMISSIVE = -4
};

/* MGFM variant: 0 = 3D_generalized (mpm.cpp:882-926: clamps p,rho >= 1e-10,
 * seed max(pl,pr), u* from the pre-update p*), 1 = 2D cases
 * (Triple_point_2phase/mpm.cpp:1373-1416: clamp p >= 0, seed (pl+pr)/2, u*
 * from the final p*). */
enum { PGDG_MGFM_3D = 0, PGDG_MGFM_2D = 1 };

/* Case parameters (replaces the constants hard-coded in MPM::Initialize_case,
 * mpm_ini.cpp:33-673, and the inlet state hard-coded in the face flux,
 * particle_flow.cpp:332-339). */
typedef struct pgdg_case {
  int32_t dim;            /* 2 or 3 */
  int32_t nfld;           /* number of materials: 2, or 3 (the three-material build) */
  int32_t ncell[3];       /* NUM (cells per axis; 1 for z in 2D) */
  int32_t bc[6];          /* boundary kind per side: xL, xR, yL, yR, zL, zR */
  int32_t mgfm_variant;   /* PGDG_MGFM_3D or PGDG_MGFM_2D */
  int32_t merge_iters;    /* merge passes per step (4, mpm_ini.cpp:708) */
  double box_l[3];
  double box_r[3];
  double p_size[3];       /* cell size per axis (px, py, pz) */
  double p_g;             /* nominal cell size */
  double p_sz;            /* particle spacing */
  double gamma[PGDG_MAX_FLD];
  double pinf[PGDG_MAX_FLD];    /* stiffened-gas Pp0 */
  double ini_rho[PGDG_MAX_FLD]; /* density of an absent phase (mpm.cpp:371) */
  double c_ini[PGDG_MAX_FLD];   /* initial cell sound speed (mpm_ini.cpp:94,100) */
  double inlet_rho;
  double inlet_u[3];
  double inlet_p;
  double cfl;             /* 0.3 (particle.cpp:558) */
  double probe[8][3];     /* positivity probe offsets (mpm.cpp:694-719), host-computed */
} pgdg_case;

/* Fluid particles in canonical (particle_fluid) order. */
typedef struct pgdg_particles {
  int64_t n;
  double *coord;   /* n*3 */
  double *v;       /* n*3 */
  double *tv;      /* n*3 */
  double *rhov;    /* n*3 */
  double *vol, *mass, *h, *P, *rho, *E, *c;   /* n */
  double *slope;   /* n*U*D : columns 1..D of coef[0] (row-major u*D+b) */
  int32_t *phase;  /* n : 1..nfld */
  int32_t *mark_in;/* n */
  uint64_t *seq;   /* n : creation rank; canonical order is ascending seq */
} pgdg_particles;

/* Grid cells ("Ele_cen"), lexicographic (i*NY + j)*NZ + k. */
typedef struct pgdg_cells {
  int64_t n;
  double *rho;     /* n*F */
  double *rhov;    /* n*F*3 */
  double *E;       /* n*F */
  double *c;       /* n*F */
  double *ac;      /* n*F */
  double *alph;    /* n*F */
  double *coef;    /* n*F*U*B (row-major u*B+b) */
  double *v;       /* n*3 */
  double *P;       /* n */
  int32_t *ph_state;   /* n*F */
  int32_t *ph_state_b; /* n*F */
  int32_t *used;       /* n */
  /* per-stage transients (download only; may be NULL) */
  double *lim_u;   /* n*F*U */
  double *g_v;     /* n*D*D  (row = velocity component, col = derivative axis) */
  double *dcoef;   /* n*F*U*B */
} pgdg_cells;

/* Run statistics. */
typedef struct pgdg_stats {
  int64_t n_particles;
  int64_t n_split, n_inlet, n_outlet, n_merge;
  int64_t n_affected;
  int64_t mgfm_calls, mgfm_iters, mgfm_maxit_hits;
  int64_t g2p_fallbacks;
  int64_t list_entries;     /* stored neighbour-list entries */
  int64_t iterate_num;
  double dt, max_v, time;
} pgdg_stats;

#ifdef __cplusplus
}
#endif
#endif
