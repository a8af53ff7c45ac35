/*
 * case_builder.cpp -- host-side construction of the synthetic workloads.
 *
 * Restates the structure of MPM::Initialize_case (mpm_ini.cpp:33-673): grid of
 * P1 DG cells, fluid particles on a lattice of spacing p_sz (mpm_ini.cpp:170-294),
 * cell state (mpm_ini.cpp:299-346), face boundary tags (mpm_ini.cpp:352-550).
 * The reference hard-codes one dimensional case per program; here the case is a
 * parameter (pgdg_case) and the four synthetic configurations are built from the
 * shapes and states of the workloads they stand for:
 *   1  2D triple point, [0,7]x[0,3], 112x48, 4 particles/cell with seeded jitter
 *   2  3D Air/He cylindrical shock-bubble, [0,4]x[0,1]^2, 256x64x64, 8 ppc
 *   3  3D Air/He spherical shock-bubble, [0,4]x[0,1]^2, 384x96x96, 8 ppc
 *   4  2D underwater explosion, [-1,1]^2, 1024^2, 4 ppc, stiffened-gas water
 */
#include "../../include/pgdg.h"

#include <cmath>
#include <cstring>

#include "case_math.h"

namespace {

constexpr double PI_REF = 3.1415926;

inline double powern(double a, int n) {
  double r = 1;
  for (int i = 0; i < n; i++) r *= a;
  return r;
}

using namespace pgdg_case_math;

void post_shock(double& rho2, double& u2, double& p2) {
  pgdg_case_math::post_shock(rho2, u2, p2, std::sqrt(1.4 * 1.0 / 1.0));
}

int npart_axis(const pgdg_case* cs, int d) {
  if (d >= cs->dim) return 1;
  return (int)std::lround((cs->box_r[d] - cs->box_l[d]) / cs->p_sz);  /* mpm_ini.cpp:170-173 */
}

}  // namespace

extern "C" {

int pgdg_case_setup(int id, const int32_t* ncell, pgdg_case* cs) {
  if (!cs || id < 1 || id > 5) return PGDG_EINVAL;
  std::memset(cs, 0, sizeof(*cs));
  cs->nfld = 2;
  cs->merge_iters = 4;
  cs->cfl = 0.3;
  int def[3];
  switch (id) {
    case 1:
      cs->dim = 2; def[0] = 112; def[1] = 48; def[2] = 1;
      cs->box_l[0] = 0; cs->box_l[1] = 0; cs->box_r[0] = 7; cs->box_r[1] = 3;
      cs->gamma[0] = 1.5; cs->pinf[0] = 0; cs->ini_rho[0] = 1.0;
      cs->gamma[1] = 1.4; cs->pinf[1] = 0; cs->ini_rho[1] = 0.125;
      for (int s = 0; s < 4; s++) cs->bc[s] = PGDG_BC_WALL;
      cs->mgfm_variant = PGDG_MGFM_2D;
      break;
    case 2:
    case 3:
      cs->dim = 3;
      if (id == 2) { def[0] = 256; def[1] = 64; def[2] = 64; }
      else { def[0] = 384; def[1] = 96; def[2] = 96; }
      cs->box_r[0] = 4; cs->box_r[1] = 1; cs->box_r[2] = 1;
      cs->gamma[0] = 1.4; cs->pinf[0] = 0; cs->ini_rho[0] = 1.0;
      cs->gamma[1] = 1.648; cs->pinf[1] = 0; cs->ini_rho[1] = 0.138;
      cs->bc[0] = PGDG_BC_INLET; cs->bc[1] = PGDG_BC_OUTLET;
      cs->bc[2] = PGDG_BC_SYMMETRY; cs->bc[3] = PGDG_BC_WALL;
      cs->bc[4] = PGDG_BC_SYMMETRY;
      cs->bc[5] = (id == 2) ? PGDG_BC_SYMMETRY : PGDG_BC_WALL;
      cs->mgfm_variant = PGDG_MGFM_3D;
      post_shock(cs->inlet_rho, cs->inlet_u[0], cs->inlet_p);
      break;
    case 5:
      /* the triple point with three materials (Triple_point_3phase/mpm_ini.cpp:
       * 80-97): C1's box, cells, walls and sub-lattice */
      cs->dim = 2; def[0] = 112; def[1] = 48; def[2] = 1;
      cs->nfld = 3;
      cs->box_l[0] = 0; cs->box_l[1] = 0; cs->box_r[0] = 7; cs->box_r[1] = 3;
      cs->gamma[0] = 1.4; cs->pinf[0] = 0; cs->ini_rho[0] = 1.0;
      cs->gamma[1] = 1.5; cs->pinf[1] = 0; cs->ini_rho[1] = 0.125;
      cs->gamma[2] = 1.6; cs->pinf[2] = 0.1; cs->ini_rho[2] = 0.125;
      for (int s = 0; s < 4; s++) cs->bc[s] = PGDG_BC_WALL;
      cs->mgfm_variant = PGDG_MGFM_2D;
      break;
    default:
      cs->dim = 2; def[0] = 1024; def[1] = 1024; def[2] = 1;
      cs->box_l[0] = -1; cs->box_l[1] = -1; cs->box_r[0] = 1; cs->box_r[1] = 1;
      cs->gamma[0] = 7.15; cs->pinf[0] = 3.309e8; cs->ini_rho[0] = 1000.0;
      cs->gamma[1] = 2.0; cs->pinf[1] = 0; cs->ini_rho[1] = 1270.0;
      for (int s = 0; s < 4; s++) cs->bc[s] = PGDG_BC_TRANSMISSIVE;
      cs->mgfm_variant = PGDG_MGFM_2D;
      break;
  }
  for (int d = 0; d < 3; d++) cs->ncell[d] = (ncell && ncell[d] > 0 && d < cs->dim) ? ncell[d] : def[d];
  if (cs->dim == 2) cs->ncell[2] = 1;
  for (int d = 0; d < 3; d++)
    cs->p_size[d] = (d < cs->dim) ? (cs->box_r[d] - cs->box_l[d]) / (double)cs->ncell[d] : 0.0;
  cs->p_g = cs->p_size[0];
  /* p_sz = (px py [pz])^(1/d) / round(p_g / p_sz_init), p_sz_init = p_g / 2
   * (mpm_ini.cpp:55-83): 2^d particles per cell */
  double prod = cs->p_size[0] * cs->p_size[1];
  if (cs->dim == 3) prod = prod * cs->p_size[2];
  double root = (cs->dim == 2) ? std::sqrt(prod) : std::cbrt(prod);
  cs->p_sz = root / std::round(cs->p_g / (cs->p_g / 2.0));
  for (int s = 0; s < cs->nfld; s++) cs->c_ini[s] = std::sqrt(cs->gamma[s] * (cs->pinf[s] + 0) / cs->ini_rho[s]);
  /* positivity probe points (mpm.cpp:694-706) */
  int k = 0;
  for (int jj = 0; jj < 4; jj++) {
    double theta = (jj + 0.5) * PI_REF * 0.5;
    for (int k1 = 0; k1 < (cs->dim == 3 ? 2 : 1); k1++) {
      cs->probe[k][0] = std::sqrt(2.) * cs->p_g * std::cos(theta);
      cs->probe[k][1] = std::sqrt(2.) * cs->p_g * std::sin(theta);
      cs->probe[k][2] = (cs->dim == 3) ? (-0.5 + k1) * cs->p_g : 0.0;
      k++;
    }
  }
  return PGDG_OK;
}

int64_t pgdg_case_num_particles(const pgdg_case* cs) {
  return (int64_t)npart_axis(cs, 0) * npart_axis(cs, 1) * npart_axis(cs, 2);
}

int pgdg_case_particles(const pgdg_case* cs, int id, uint64_t seed, pgdg_particles* out) {
  int64_t n = pgdg_case_num_particles(cs);
  if (!out || out->n < n) return PGDG_EINVAL;
  const int D = cs->dim;
  const int U = D + 2;
  const int NS = U * D;
  int na[3] = {npart_axis(cs, 0), npart_axis(cs, 1), npart_axis(cs, 2)};
  const uint64_t rs = seed ? seed : 20260101ull;
  const double jit = jittered(id) ? cs->p_g / 8.0 : 0.0;
  double vol0 = powern(cs->p_sz, D);
  double h0 = 3.2 / 2. * cs->p_sz;
  double ps[3];
  post_shock(ps[0], ps[1], ps[2]);
  int64_t p = 0;
  for (int i = 0; i < na[0]; i++)
    for (int j = 0; j < na[1]; j++)
      for (int k = 0; k < na[2]; k++, p++) {
        const PState0 s = lattice_particle(id, D, cs->box_l, cs->p_sz, jit, rs, p, i, j, k, vol0, h0, cs->gamma,
                                           cs->pinf, ps);
        for (int d = 0; d < 3; d++) {
          out->coord[3 * p + d] = s.x[d];
          if (out->v) out->v[3 * p + d] = s.u[d];
          if (out->tv) out->tv[3 * p + d] = 0.0;
          out->rhov[3 * p + d] = s.rhov[d];
        }
        out->vol[p] = s.vol;
        out->mass[p] = s.mass;
        out->h[p] = s.h;
        out->P[p] = s.P;
        out->rho[p] = s.rho;
        out->E[p] = s.E;
        out->c[p] = s.c;
        if (out->slope)
          for (int t = 0; t < NS; t++) out->slope[NS * p + t] = 0.0;
        out->phase[p] = s.phase;
        if (out->mark_in) out->mark_in[p] = 0;
        if (out->seq) out->seq[p] = (uint64_t)p;
      }
  out->n = n;
  return PGDG_OK;
}

int pgdg_case_cells(const pgdg_case* cs, pgdg_cells* c) {
  const int D = cs->dim, F = cs->nfld, U = D + 2, B = D + 1;
  int64_t n = (int64_t)cs->ncell[0] * cs->ncell[1] * (D == 3 ? cs->ncell[2] : 1);
  if (!c || c->n != n) return PGDG_EINVAL;
  for (int64_t ci = 0; ci < n; ci++) {
    for (int s = 0; s < F; s++) {
      int64_t q = ci * F + s;
      c->rho[q] = cs->ini_rho[s];
      for (int d = 0; d < 3; d++) c->rhov[q * 3 + d] = 0;
      c->E[q] = 0;
      c->c[q] = cs->c_ini[s];
      if (c->ac) c->ac[q] = 0;
      c->alph[q] = 0;
      for (int t = 0; t < U * B; t++) c->coef[q * U * B + t] = 0;
      c->ph_state[q] = 1;
      c->ph_state_b[q] = 0;
      if (c->lim_u) for (int u = 0; u < U; u++) c->lim_u[q * U + u] = 1.0;
      if (c->dcoef) for (int t = 0; t < U * B; t++) c->dcoef[q * U * B + t] = 0;
    }
    for (int d = 0; d < 3; d++) c->v[3 * ci + d] = 0;
    c->P[ci] = 0;
    if (c->used) c->used[ci] = 1;
    if (c->g_v) for (int t = 0; t < D * D; t++) c->g_v[ci * D * D + t] = 0;
  }
  return PGDG_OK;
}

}  // extern "C"
