/*
 * oracle_case.cpp -- the oracle's own construction of the synthetic workloads.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  It lets the CPU oracle (the tests'
 * reference and bench.py's CPU arms) build a case without loading the GPU
 * library.  tests/test_case_builder.py checks its output bit for bit against
 * the library's pgdg_case_setup / pgdg_case_particles / pgdg_case_cells.
 *
 * Restatement of MPM::Initialize_case (3D_generalized/PGDG_3D_spheric/
 * mpm_ini.cpp:33-673, cited below without that prefix) with the reference's
 * hard-coded dimensional case replaced by the four synthetic workloads:
 *   - domain, cell count per axis and cell size: mpm_ini.cpp:49-83;
 *   - particle spacing p_sz = (px py [pz])^(1/d) / round(p_g / p_sz_init) with
 *     p_sz_init = p_g / 2 (2^d particles per cell): mpm_ini.cpp:79-83;
 *   - materials gamma / Pp0 / ini_rho / c: mpm_ini.cpp:90-100;
 *   - fluid particles on the lattice (i+1/2) p_sz, looped i, j, k, each given
 *     the state of the region it lies in (the reference's f1 / f2 tests):
 *     mpm_ini.cpp:170-294;
 *   - cells: every phase at ini_rho, zero coefficients, Lim_u 1, ph_state 1:
 *     mpm_ini.cpp:299-346;
 *   - positivity probe offsets at radius sqrt(2) p_g, theta = (j+1/2) pi/2,
 *     z = +-p_g/2: mpm.cpp:694-706.
 * The triple point's lattice carries seeded splitmix64 jitter of +-p_g/8 per
 * axis, drawn per particle in lattice order, axis by axis.
 */
#include "pgdg_oracle.h"

#include <cmath>
#include <cstring>

namespace {

const double PI_REF = 3.1415926; /* glbparam.h:31 */

struct Mix64 {
  uint64_t s;
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

/* state behind a normal shock of Mach number m running into a gas at rest
 * (Rankine-Hugoniot relations for a perfect gas) */
struct Shock { double rho, u, p; };
Shock rankine_hugoniot(double gam, double m, double rho1, double p1) {
  const double m2 = m * m;
  Shock s;
  s.p = p1 * (1.0 + 2.0 * gam / (gam + 1.0) * (m2 - 1.0));
  s.rho = rho1 * (gam + 1.0) * m2 / ((gam - 1.0) * m2 + 2.0);
  const double c1 = std::sqrt(gam * p1 / rho1);
  s.u = m * c1 * (1.0 - rho1 / s.rho);
  return s;
}

struct State { int phase; double rho, p, u0; };

/* the region tests of each workload (the reference's f1 / f2 of mpm_ini.cpp:187-197) */
State initial_state(int id, const double x[3], int dim) {
  if (id == 1) {
    if (x[0] < 1.0) return {1, 1.0, 1.0, 0.0};
    return x[1] < 1.5 ? State{1, 1.0, 0.1, 0.0} : State{2, 0.125, 0.1, 0.0};
  }
  if (id == 5) {
    /* Triple_point_3phase/mpm_ini.cpp:157-245: f1 = x > 1 and y < 1.5 */
    if (x[0] > 1.0 && x[1] < 1.5) return {1, 1.0, 0.1, 0.0};
    return x[0] > 1.0 ? State{2, 0.125, 0.1, 0.0} : State{3, 1.0, 1.0, 0.0};
  }
  if (id == 4) {
    const double r2 = x[0] * x[0] + x[1] * x[1];
    return r2 < 0.3 * 0.3 ? State{2, 1270.0, 8.29e8, 0.0} : State{1, 1000.0, 1e5, 0.0};
  }
  /* 2: helium cylinder along z through (1.5, 0); 3: helium sphere at (1.5, 0, 0) */
  const bool behind_shock = x[0] < 1.0;
  if (behind_shock) {
    const Shock s = rankine_hugoniot(1.4, 1.22, 1.0, 1.0);
    return {1, s.rho, s.p, s.u};
  }
  double r2 = (x[0] - 1.5) * (x[0] - 1.5) + x[1] * x[1];
  if (id == 3 && dim == 3) r2 += x[2] * x[2];
  if (r2 < 0.25 * 0.25) return {2, 0.138, 1.0, 0.0};
  return {1, 1.0, 1.0, 0.0};
}

int lattice_count(const pgdg_case* cs, int d) {
  return d < cs->dim ? (int)std::lround((cs->box_r[d] - cs->box_l[d]) / cs->p_sz) : 1;
}

}  // namespace

extern "C" {

int po_case_setup(int id, const int32_t* ncell, pgdg_case* cs) {
  if (!cs || id < 1 || id > 5) return PGDG_EINVAL;
  std::memset(cs, 0, sizeof(*cs));
  struct Workload {
    int dim, n[3];
    double lo[3], hi[3];
    int nfld;
    double gam[3], pinf[3], rho0[3];
    int bc[6];
    int mgfm;
  };
  const int W = PGDG_BC_WALL, I = PGDG_BC_INLET, O = PGDG_BC_OUTLET, S = PGDG_BC_SYMMETRY,
            T = PGDG_BC_TRANSMISSIVE;
  static const Workload table[5] = {
      {2, {112, 48, 1}, {0, 0, 0}, {7, 3, 0}, 2, {1.5, 1.4}, {0, 0}, {1.0, 0.125}, {W, W, W, W, 0, 0}, PGDG_MGFM_2D},
      {3, {256, 64, 64}, {0, 0, 0}, {4, 1, 1}, 2, {1.4, 1.648}, {0, 0}, {1.0, 0.138}, {I, O, S, W, S, S},
       PGDG_MGFM_3D},
      {3, {384, 96, 96}, {0, 0, 0}, {4, 1, 1}, 2, {1.4, 1.648}, {0, 0}, {1.0, 0.138}, {I, O, S, W, S, W},
       PGDG_MGFM_3D},
      {2, {1024, 1024, 1}, {-1, -1, 0}, {1, 1, 0}, 2, {7.15, 2.0}, {3.309e8, 0}, {1000.0, 1270.0},
       {T, T, T, T, 0, 0}, PGDG_MGFM_2D},
      /* Triple_point_3phase/mpm_ini.cpp:80-97 materials on C1's box */
      {2, {112, 48, 1}, {0, 0, 0}, {7, 3, 0}, 3, {1.4, 1.5, 1.6}, {0, 0, 0.1}, {1.0, 0.125, 0.125},
       {W, W, W, W, 0, 0}, PGDG_MGFM_2D}};
  const Workload& w = table[id - 1];
  cs->dim = w.dim;
  cs->nfld = w.nfld;
  cs->merge_iters = 4; /* mpm_ini.cpp:708 */
  cs->cfl = 0.3;       /* particle.cpp:558 */
  cs->mgfm_variant = w.mgfm;
  for (int s = 0; s < 6; s++) cs->bc[s] = w.bc[s];
  for (int d = 0; d < 3; d++) {
    cs->box_l[d] = w.lo[d];
    cs->box_r[d] = w.hi[d];
    cs->ncell[d] = d < w.dim ? ((ncell && ncell[d] > 0) ? ncell[d] : w.n[d]) : 1;
    cs->p_size[d] = d < w.dim ? (w.hi[d] - w.lo[d]) / (double)cs->ncell[d] : 0.0;
  }
  for (int s = 0; s < w.nfld; s++) {
    cs->gamma[s] = w.gam[s];
    cs->pinf[s] = w.pinf[s];
    cs->ini_rho[s] = w.rho0[s];
    cs->c_ini[s] = std::sqrt(w.gam[s] * (w.pinf[s] + 0) / w.rho0[s]); /* mpm_ini.cpp:94,100 */
  }
  if (id == 2 || id == 3) {
    const Shock s = rankine_hugoniot(1.4, 1.22, 1.0, 1.0);
    cs->inlet_rho = s.rho;
    cs->inlet_u[0] = s.u;
    cs->inlet_p = s.p;
  }
  cs->p_g = cs->p_size[0];
  const double cellvol = w.dim == 3 ? cs->p_size[0] * cs->p_size[1] * cs->p_size[2] : cs->p_size[0] * cs->p_size[1];
  const double edge = w.dim == 3 ? std::cbrt(cellvol) : std::sqrt(cellvol);
  const double p_sz_init = cs->p_g / 2.0;
  cs->p_sz = edge / std::round(cs->p_g / p_sz_init);
  int k = 0;
  for (int j = 0; j < 4; j++) {
    const double theta = (j + 0.5) * PI_REF * 0.5;
    const int nz = w.dim == 3 ? 2 : 1;
    for (int kz = 0; kz < nz; kz++, k++) {
      cs->probe[k][0] = std::sqrt(2.) * cs->p_g * std::cos(theta);
      cs->probe[k][1] = std::sqrt(2.) * cs->p_g * std::sin(theta);
      cs->probe[k][2] = w.dim == 3 ? (-0.5 + kz) * cs->p_g : 0.0;
    }
  }
  return PGDG_OK;
}

int64_t po_case_num_particles(const pgdg_case* cs) {
  return (int64_t)lattice_count(cs, 0) * lattice_count(cs, 1) * lattice_count(cs, 2);
}

int po_case_particles(const pgdg_case* cs, int id, uint64_t seed, pgdg_particles* out) {
  const int64_t n = po_case_num_particles(cs);
  if (!cs || !out || out->n < n) return PGDG_EINVAL;
  const int D = cs->dim, NS = (D + 2) * D;
  const int ni = lattice_count(cs, 0), nj = lattice_count(cs, 1), nk = lattice_count(cs, 2);
  Mix64 rng{seed ? seed : 20260101ull};
  const double jitter = (id == 1 || id == 5) ? cs->p_g / 8.0 : 0.0;
  double vol = 1;
  for (int d = 0; d < D; d++) vol *= cs->p_sz; /* powern(p_sz, DIM) */
  const double ini_h = 3.2 / 2. * cs->p_sz;     /* CELL_RATIO / CUT_OFF * p_sz */
  int64_t q = 0;
  for (int i = 0; i < ni; i++)
    for (int j = 0; j < nj; j++)
      for (int kk = 0; kk < nk; kk++, q++) {
        double x[3] = {cs->box_l[0] + (i + 0.5) * cs->p_sz, cs->box_l[1] + (j + 0.5) * cs->p_sz,
                       D == 3 ? cs->box_l[2] + (kk + 0.5) * cs->p_sz : 0.0};
        if (jitter > 0)
          for (int d = 0; d < D; d++) x[d] += (2.0 * rng.uniform() - 1.0) * jitter;
        const State st = initial_state(id, x, D);
        const int s = st.phase - 1;
        const double g = cs->gamma[s], pinf = cs->pinf[s];
        const double v[3] = {st.u0, 0.0, 0.0};
        double vv = 0;
        for (int d = 0; d < D; d++) vv += v[d] * v[d];
        for (int d = 0; d < 3; d++) {
          out->coord[3 * q + d] = x[d];
          out->rhov[3 * q + d] = d < D ? v[d] * st.rho : 0.0;
          if (out->v) out->v[3 * q + d] = d < D ? v[d] : 0.0;
          if (out->tv) out->tv[3 * q + d] = 0.0;
        }
        out->vol[q] = vol;
        out->mass[q] = vol * st.rho;
        out->h[q] = ini_h;
        out->P[q] = st.p;
        out->rho[q] = st.rho;
        double E = (st.p + g * pinf) / (g - 1);
        E += 0.5 * st.rho * vv;
        out->E[q] = E;
        out->c[q] = std::sqrt(g * (st.p + pinf) / st.rho);
        if (out->slope)
          for (int t = 0; t < NS; t++) out->slope[NS * q + t] = 0.0;
        out->phase[q] = st.phase;
        if (out->mark_in) out->mark_in[q] = 0;
        if (out->seq) out->seq[q] = (uint64_t)q;
      }
  out->n = n;
  return PGDG_OK;
}

int po_case_cells(const pgdg_case* cs, pgdg_cells* c) {
  if (!cs || !c) return PGDG_EINVAL;
  const int D = cs->dim, U = D + 2, B = D + 1, F = cs->nfld;
  const int64_t n = (int64_t)cs->ncell[0] * cs->ncell[1] * (D == 3 ? cs->ncell[2] : 1);
  if (c->n != n) return PGDG_EINVAL;
  for (int64_t ci = 0; ci < n; ci++) {
    for (int s = 0; s < F; s++) {
      const int64_t q = ci * F + s;
      c->rho[q] = cs->ini_rho[s];
      c->E[q] = 0;
      c->c[q] = cs->c_ini[s];
      c->alph[q] = 0;
      c->ph_state[q] = 1;
      c->ph_state_b[q] = 0;
      for (int d = 0; d < 3; d++) c->rhov[3 * q + d] = 0;
      for (int t = 0; t < U * B; t++) c->coef[q * U * B + t] = 0;
      if (c->dcoef)
        for (int t = 0; t < U * B; t++) c->dcoef[q * U * B + t] = 0;
      if (c->lim_u)
        for (int u = 0; u < U; u++) c->lim_u[q * U + u] = 1.0;
      if (c->ac) c->ac[q] = 0;
    }
    for (int d = 0; d < 3; d++) c->v[3 * ci + d] = 0;
    c->P[ci] = 0;
    if (c->used) c->used[ci] = 1;
    if (c->g_v)
      for (int t = 0; t < D * D; t++) c->g_v[ci * D * D + t] = 0;
  }
  return PGDG_OK;
}

}  // extern "C"
