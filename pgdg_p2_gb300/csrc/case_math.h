/*
 * case_math.h -- the per-particle mathematics of the synthetic workloads,
 * shared by the host case builder (case_builder.cpp) and the device one
 * (k_case.cu), so that both produce the same bits: each expression is written
 * once, and both translation units are compiled without FMA contraction.
 *
 * Restates the particle set-up of MPM::Initialize_case
 * (3D_generalized/PGDG_3D_spheric/mpm_ini.cpp:170-294): lattice positions
 * (i + 1/2) p_sz, the region each particle lies in, and its primitive state.
 */
#ifndef PGDG_CASE_MATH_H
#define PGDG_CASE_MATH_H
#include <stdint.h>

#ifdef __CUDACC__
#define PGDG_CHD __host__ __device__ inline
#else
#define PGDG_CHD inline
#endif

namespace pgdg_case_math {

/* splitmix64: the state advances by the golden gamma each draw, so draw k
 * (from 0) of a stream seeded s is mix(s + (k + 1) gamma) */
constexpr uint64_t GAMMA = 0x9E3779B97F4A7C15ull;
PGDG_CHD uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
PGDG_CHD double draw_u01(uint64_t seed, uint64_t k) {
  return (double)(mix64(seed + (k + 1) * GAMMA) >> 11) * (1.0 / 9007199254740992.0);
}

/* Mach-1.22 shock into air at rest (gamma 1.4, rho 1, p 1): Rankine-Hugoniot;
 * c1 is the sound speed ahead of the shock */
PGDG_CHD void post_shock(double& rho2, double& u2, double& p2, double c1) {
  const double g = 1.4, M = 1.22, r1 = 1.0, p1 = 1.0;
  double M2 = M * M;
  p2 = p1 * (1.0 + 2.0 * g / (g + 1.0) * (M2 - 1.0));
  rho2 = r1 * (g + 1.0) * M2 / ((g - 1.0) * M2 + 2.0);
  u2 = M * c1 * (1.0 - r1 / rho2);
}

struct Region {
  int phase;
  double rho, p, u[3];
};

/* the region of workload id holding x; ps = (rho2, u2, p2) behind the shock */
PGDG_CHD Region region_of(int id, const double* x, const double* ps) {
  Region r{1, 1.0, 1.0, {0, 0, 0}};
  switch (id) {
    case 1:
      if (x[0] < 1.0) r = {1, 1.0, 1.0, {0, 0, 0}};
      else if (x[1] < 1.5) r = {1, 1.0, 0.1, {0, 0, 0}};
      else r = {2, 0.125, 0.1, {0, 0, 0}};
      break;
    case 2:
    case 3: {
      double d2 = (x[0] - 1.5) * (x[0] - 1.5) + x[1] * x[1];
      if (id == 3) d2 += x[2] * x[2];
      if (x[0] < 1.0) r = {1, ps[0], ps[2], {ps[1], 0, 0}};
      else if (d2 < 0.25 * 0.25) r = {2, 0.138, 1.0, {0, 0, 0}};
      else r = {1, 1.0, 1.0, {0, 0, 0}};
      break;
    }
    case 4: {
      double d2 = x[0] * x[0] + x[1] * x[1];
      if (d2 < 0.3 * 0.3) r = {2, 1270.0, 8.29e8, {0, 0, 0}};
      else r = {1, 1000.0, 1e5, {0, 0, 0}};
      break;
    }
    case 5:
      /* three materials (Triple_point_3phase/mpm_ini.cpp:157-245): lower right
       * phase 1, upper right phase 2, left phase 3 */
      if (x[0] > 1.0 && x[1] < 1.5) r = {1, 1.0, 0.1, {0, 0, 0}};
      else if (x[0] > 1.0) r = {2, 0.125, 0.1, {0, 0, 0}};
      else r = {3, 1.0, 1.0, {0, 0, 0}};
      break;
    default: break;
  }
  return r;
}

/* the triple-point layouts jitter their sub-lattice (seeded, +-p_g/8) */
PGDG_CHD bool jittered(int id) { return id == 1 || id == 5; }

/* the particle at lattice index (i, j, k), number p: position (with the
 * triple point's jitter, draws D p + d of the stream), region and state */
struct PState0 {
  double x[3], u[3], rhov[3];
  double vol, mass, h, P, rho, E, c;
  int phase;
};
PGDG_CHD PState0 lattice_particle(int id, int D, const double* box_l, double p_sz, double jit, uint64_t seed,
                                  int64_t p, int i, int j, int k, double vol0, double h0, const double* gam,
                                  const double* pinf, const double* ps) {
  PState0 s;
  s.x[0] = box_l[0] + (i + 0.5) * p_sz;
  s.x[1] = box_l[1] + (j + 0.5) * p_sz;
  s.x[2] = (D == 3) ? box_l[2] + (k + 0.5) * p_sz : 0.0;
  if (jit > 0)
    for (int d = 0; d < D; d++) s.x[d] += (2.0 * draw_u01(seed, (uint64_t)p * D + d) - 1.0) * jit;
  const Region r = region_of(id, s.x, ps);
  const int ph = r.phase - 1;
  const double g = gam[ph], pf = pinf[ph];
  double vv = 0;
  for (int d = 0; d < 3; d++) {
    s.u[d] = (d < D) ? r.u[d] : 0.0;
    s.rhov[d] = (d < D) ? r.u[d] * r.rho : 0.0;
  }
  for (int d = 0; d < D; d++) vv += r.u[d] * r.u[d];
  s.vol = vol0;
  s.mass = vol0 * r.rho;
  s.h = h0;
  s.P = r.p;
  s.rho = r.rho;
  double E = (r.p + g * pf) / (g - 1);
  E += 0.5 * r.rho * vv;
  s.E = E;
  s.c = sqrt(g * (r.p + pf) / r.rho);
  s.phase = r.phase;
  return s;
}

}  // namespace pgdg_case_math
#endif
