/*
 * pgdg_oracle.cpp -- FP64 CPU oracle of the PGDG per-time-step particle-grid path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; never shipped, never on the product path).
 *
 * A serial, canonical-order restatement of the reference program
 * 3D_generalized/PGDG_3D_spheric (cited below without that prefix), templated on
 * the dimension so the 2D cases run the same algorithm.  Canonical choices where
 * the reference is order-nondeterministic (TBB concurrent_vector push_back) or
 * racy:
 *   - particle_fluid order is creation order (every new particle is appended);
 *   - Map_the_particle_to_tree bins fluid particles in particle_fluid order, then
 *     boundary particles (mpm.cpp:74-96);
 *   - split/merge records are processed in particle_fluid order;
 *   - Update_particle is two-pass: every particle's G2P update (particle_flow.cpp:
 *     413-477) completes before any particle's shifting (particle_flow.cpp:485-622),
 *     which the reference runs in one racy loop (mpm.cpp:839-853);
 *   - pow(x, 1./DIM) is oracle::root_d, a near-correctly-rounded restatement.
 * Sums over small fixed-size vectors are evaluated left to right (the reference
 * uses Eigen 3.4 expression templates, whose order is not pinned here).
 */
#include "pgdg_oracle.h"
#include "oracle_math.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <fstream>
#include <string>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>

#ifndef PO_NFLD
#define PO_NFLD 2
#endif
#endif

using namespace oracle;

struct po_ctx {
  virtual ~po_ctx() {}
  virtual int upload_particles(const pgdg_particles* p) = 0;
  virtual int download_particles(pgdg_particles* p) = 0;
  virtual int64_t num_particles() = 0;
  virtual int upload_cells(const pgdg_cells* c) = 0;
  virtual int download_cells(pgdg_cells* c) = 0;
  virtual int upload_lists(const int64_t* off, const int64_t* ent) = 0;
  virtual int download_lists(int64_t* off, int64_t* ent, int64_t cap, int64_t* total) = 0;
  virtual int download_cell_lists(int64_t* off, int64_t* ent, int64_t cap, int64_t* total) = 0;
  virtual int set_timestep(double* dt, double* max_v) = 0;
  virtual void used_state_update() = 0;
  virtual void bin_particles() = 0;
  virtual void split_particle_fast() = 0;
  virtual void merge_particle_fast() = 0;
  virtual void refresh_membership() = 0;
  virtual void refresh_neighbors() = 0;
  virtual void mls_p2g() = 0;
  virtual void calculate_limiter() = 0;
  virtual void grid_acceleration() = 0;
  virtual void update_grid(int md) = 0;
  virtual void update_particle(int md) = 0;
  virtual void run_step(int64_t n) = 0;
  virtual void totals(double* out) = 0;
  virtual void output_point(double* out) = 0;
  virtual int output_plt(const char* ppath, const char* cpath) = 0;
  double dt = 0, max_v = 1e-7;
  int64_t iterate = 0;
  pgdg_stats st{};
};

namespace {

struct Face {
  double cen[3], n[3], t0[3], t1[3], S;
  int64_t nb;  /* neighbour cell index (valid when bound == 0) */
  int bound;
};

template <int D>
struct OracleT : po_ctx {
  static constexpr int F = PO_NFLD; /* FldNum (glbparam.h:41), fixed per build */
  static constexpr int U = D + 2;
  static constexpr int B = D + 1;
  static constexpr int NS = U * D;  /* stored slopes per particle */
  static constexpr int NF = 2 * D;  /* faces per cell */

  pgdg_case cs;
  int N[3];
  int64_t ncell;
  double vol_max, vol_min, dss0;
  int rad2;  /* flag-2 neighbour scan radius in cells */

  /* ---- fluid particles, by slot (Mypool) ---- */
  std::vector<double> x, x0, v, tv, a, rhov;  /* 3 per slot */
  std::vector<double> vol, vol0, mass, h, P, rho, E, c;
  std::vector<double> sl;                     /* NS per slot: coef[0] columns 1..D */
  std::vector<int> phase, mark_in, mrg, mrg_mark, copy, in_ele;
  std::vector<uint64_t> seq;
  std::vector<std::vector<int>> nbr;          /* neighbour list (refs) */
  std::vector<int> fluid;                     /* particle_fluid */
  std::deque<int> freel;
  uint64_t seq_next = 0;

  /* ---- boundary particles (phase 10), static ---- */
  int64_t nbnd = 0;
  std::vector<double> bx, bn;
  double bvol = 0, brho = 0, bc0 = 0;

  /* ---- cells ---- */
  std::vector<double> ccen;                   /* 3 per cell */
  std::vector<double> crho, crhov, cE, cc, cac, calph, ccoef, ccoef0, cdcoef, clim, cgv, cv, cP, ca;
  std::vector<int> cph, cphb, cused;
  std::vector<int64_t> used_list;
  std::vector<std::vector<int>> clist;        /* Cell_list::particle_list (refs) */
  std::vector<std::vector<int>> cnbr;         /* cell->neighbor (flag 4) */
  double Gp[2], Gw[2];

  static bool is_bnd(int r) { return r <= -2; }
  static int bref(int64_t b) { return -(int)(b + 2); }
  static int64_t bidx(int r) { return -(int64_t)r - 2; }

  explicit OracleT(const pgdg_case* c) : cs(*c) {
    for (int d = 0; d < 3; d++) N[d] = (d < D) ? cs.ncell[d] : 1;
    ncell = (int64_t)N[0] * N[1] * N[2];
    vol_max = powern(cs.p_sz, D) * 1.6;            /* mpm.cpp:1068 */
    vol_min = powern(cs.p_sz, D) * 2. / 3.;        /* mpm.cpp:1540 */
    dss0 = root_d(vol_min, D);                     /* mpm.cpp:1568 */
    double g_p_rt = cs.p_g / cs.p_sz;              /* level_infor.cpp:27 */
    rad2 = (int)std::ceil(CELL_RATIO / g_p_rt);    /* level_infor.cpp:155 */
    Gp[0] = -1. / std::sqrt(3.);
    Gp[1] = 1. / std::sqrt(3.);                    /* mpm_ini.cpp:37-41 */
    Gw[0] = 0.5;
    Gw[1] = 0.5;
    init_cells();
    init_boundary();
  }

  /* ------------------------------------------------------------------ */
  /* geometry                                                           */
  /* ------------------------------------------------------------------ */
  int64_t cidx(int i, int j, int k) const { return ((int64_t)i * N[1] + j) * N[2] + k; }
  void cijk(int64_t ci, int& i, int& j, int& k) const {
    k = (int)(ci % N[2]);
    j = (int)((ci / N[2]) % N[1]);
    i = (int)(ci / ((int64_t)N[1] * N[2]));
  }

  /* get_cell_id (glbfunc.h:161-173) of a coordinate */
  void cell_pos(const double* p, int pos[3]) const {
    for (int d = 0; d < 3; d++) {
      if (d >= D) { pos[d] = 0; continue; }
      double q = std::floor((p[d] - cs.box_l[d]) / cs.p_size[d]);
      int ip;
      if (!(q >= 0)) ip = 0;                 /* also maps NaN to 0 */
      else if (q >= N[d] - 1) ip = N[d] - 1;
      else ip = (int)q;
      pos[d] = ip;
    }
  }
  int64_t cell_of(const double* p) const {
    int pos[3];
    cell_pos(p, pos);
    return cidx(pos[0], pos[1], pos[2]);
  }

  /* Cell_dg face table (mpm_ini.cpp:352-550); face order yL, xR, yR, xL, zL, zR */
  void face(int64_t ci, int f, Face& fc) const {
    int i, j, k;
    cijk(ci, i, j, k);
    const double px = cs.p_size[0], py = cs.p_size[1], pz = cs.p_size[2];
    const double* vr = &ccen[3 * ci];
    for (int d = 0; d < 3; d++) fc.cen[d] = fc.n[d] = fc.t0[d] = fc.t1[d] = 0;
    for (int d = 0; d < D; d++) fc.cen[d] = vr[d];
    int ni = i, nj = j, nk = k;
    int side;
    switch (f) {
      case 0: fc.n[1] = -1; fc.t0[0] = 0.5 * px; fc.t1[2] = 0.5 * pz; fc.cen[1] = vr[1] - 0.5 * py;
        fc.S = (D == 3) ? px * pz : px; nj = j - 1; side = 2; break;
      case 1: fc.n[0] = 1; fc.t0[1] = 0.5 * py; fc.t1[2] = 0.5 * pz; fc.cen[0] = vr[0] + 0.5 * px;
        fc.S = (D == 3) ? py * pz : py; ni = i + 1; side = 1; break;
      case 2: fc.n[1] = 1; fc.t0[0] = -0.5 * px; fc.t1[2] = 0.5 * pz; fc.cen[1] = vr[1] + 0.5 * py;
        fc.S = (D == 3) ? px * pz : px; nj = j + 1; side = 3; break;
      case 3: fc.n[0] = -1; fc.t0[1] = -0.5 * py; fc.t1[2] = 0.5 * pz; fc.cen[0] = vr[0] - 0.5 * px;
        fc.S = (D == 3) ? py * pz : py; ni = i - 1; side = 0; break;
      case 4: fc.n[2] = -1; fc.t0[0] = 0.5 * px; fc.t1[1] = 0.5 * py; fc.cen[2] = vr[2] - 0.5 * pz;
        fc.S = py * px; nk = k - 1; side = 4; break;
      default: fc.n[2] = 1; fc.t0[0] = 0.5 * px; fc.t1[1] = 0.5 * py; fc.cen[2] = vr[2] + 0.5 * pz;
        fc.S = py * px; nk = k + 1; side = 5; break;
    }
    if (D == 2) fc.t1[2] = 0;
    bool inside = ni >= 0 && ni < N[0] && nj >= 0 && nj < N[1] && nk >= 0 && nk < N[2];
    fc.bound = inside ? 0 : cs.bc[side];
    fc.nb = inside ? cidx(ni, nj, nk) : -1;
  }

  void init_cells() {
    ccen.assign(3 * ncell, 0.0);
    crho.assign(ncell * F, 0.0);
    crhov.assign(ncell * F * 3, 0.0);
    cE.assign(ncell * F, 0.0);
    cc.assign(ncell * F, 0.0);
    cac.assign(ncell * F, 0.0);
    calph.assign(ncell * F, 0.0);
    ccoef.assign(ncell * F * U * B, 0.0);
    ccoef0.assign(ncell * F * U * B, 0.0);
    cdcoef.assign(ncell * F * U * B, 0.0);
    clim.assign(ncell * F * U, 1.0);
    cgv.assign(ncell * D * D, 0.0);
    cv.assign(ncell * 3, 0.0);
    cP.assign(ncell, 0.0);
    ca.assign(ncell * 3, 0.0);
    cph.assign(ncell * F, 1);
    cphb.assign(ncell * F, 0);
    cused.assign(ncell, 1);
    clist.assign(ncell, {});
    cnbr.assign(ncell, {});
    for (int64_t ci = 0; ci < ncell; ci++) {
      int i, j, k;
      cijk(ci, i, j, k);
      int idx[3] = {i, j, k};
      for (int d = 0; d < D; d++) ccen[3 * ci + d] = cs.box_l[d] + cs.p_size[d] * (idx[d] + 0.5);
      for (int s = 0; s < F; s++) {
        crho[ci * F + s] = cs.ini_rho[s];
        cc[ci * F + s] = cs.c_ini[s];
      }
    }
    used_list.clear();
    for (int64_t ci = 0; ci < ncell; ci++) used_list.push_back(ci);
  }

  /* boundary particles on the domain's boundary nodes (mpm_ini.cpp:555-620) */
  void init_boundary() {
    bx.clear();
    bn.clear();
    int S2 = (D == 3) ? N[2] : 0;
    for (int sx = 0; sx <= N[0]; ++sx)
      for (int sy = 0; sy <= N[1]; ++sy)
        for (int sz = 0; sz <= S2; ++sz) {
          bool fg = (sx == 0 || sx == N[0] || sy == 0 || sy == N[1]);
          if (D == 3) fg = fg || sz == 0 || sz == N[2];
          if (!fg) continue;
          double p[3] = {cs.box_l[0] + cs.p_size[0] * (sx + 0.), cs.box_l[1] + cs.p_size[1] * (sy + 0.), 0.0};
          if (D == 3) p[2] = cs.box_l[2] + cs.p_size[2] * (sz + 0.);
          double nn[3] = {0, 0, 0};
          if (sx == 0) nn[0] = -1;
          else if (sx == N[0]) nn[0] = 1;
          else if (sy == 0) nn[1] = -1;
          else if (sy == N[1]) nn[1] = 1;
          else if (D == 3 && sz == 0) nn[2] = -1;
          else if (D == 3 && sz == N[2]) nn[2] = 1;
          for (int d = 0; d < 3; d++) {
            bx.push_back(p[d]);
            bn.push_back(nn[d]);
          }
        }
    nbnd = (int64_t)bx.size() / 3;
    bvol = powern(cs.p_sz, D - 1);
    brho = cs.ini_rho[0];
    bc0 = cs.c_ini[0];
  }

  /* ------------------------------------------------------------------ */
  /* particle pool (Mypool.h) and setters (particle.cpp)                */
  /* ------------------------------------------------------------------ */
  int pmalloc() {
    if (!freel.empty()) {
      int s = freel.front();
      freel.pop_front();
      return s;
    }
    int s = (int)vol.size();
    x.resize(3 * (s + 1), 0.0); x0.resize(3 * (s + 1), 0.0); v.resize(3 * (s + 1), 0.0);
    tv.resize(3 * (s + 1), 0.0); a.resize(3 * (s + 1), 0.0); rhov.resize(3 * (s + 1), 0.0);
    vol.push_back(0); vol0.push_back(0); mass.push_back(0); h.push_back(0); P.push_back(0);
    rho.push_back(0); E.push_back(0); c.push_back(0);
    sl.resize(NS * (s + 1), 0.0);
    phase.push_back(0); mark_in.push_back(0); mrg.push_back(0); mrg_mark.push_back(0);
    copy.push_back(-1); in_ele.push_back(-1); seq.push_back(0);
    nbr.emplace_back();
    return s;
  }
  /* Clearup (particle.cpp:61-104); mrg_mark and mark_in are left as they are */
  void clearup(int s) {
    nbr[s].clear();
    P[s] = mass[s] = vol[s] = h[s] = 0;
    for (int d = 0; d < 3; d++) x[3 * s + d] = v[3 * s + d] = a[3 * s + d] = tv[3 * s + d] = rhov[3 * s + d] = 0;
    phase[s] = 0;
    rho[s] = c[s] = E[s] = 0;
    for (int q = 0; q < NS; q++) sl[NS * s + q] = 0;
  }
  void pfree(int s) {
    clearup(s);
    freel.push_back(s);
  }

  /* rho, rhov, E of the parent polynomial at offset dr */
  void poly_state(int p, const double* dr, double& r, double* rv, double& e) const {
    const double* S = &sl[NS * p];
    double acc = 0;
    for (int b = 0; b < D; b++) acc = (b == 0) ? S[0 * D + b] * dr[b] : acc + S[0 * D + b] * dr[b];
    r = rho[p] + acc;
    for (int k = 0; k < D; k++) {
      double ak = 0;
      for (int b = 0; b < D; b++) ak = (b == 0) ? S[(1 + k) * D + b] * dr[b] : ak + S[(1 + k) * D + b] * dr[b];
      rv[k] = rhov[3 * p + k] + ak;
    }
    double ae = 0;
    for (int b = 0; b < D; b++) ae = (b == 0) ? S[(U - 1) * D + b] * dr[b] : ae + S[(U - 1) * D + b] * dr[b];
    e = E[p] + ae;
  }
  double sqnorm_head(const double* w) const {
    double s = w[0] * w[0];
    for (int k = 1; k < D; k++) s = s + w[k] * w[k];
    return s;
  }
  void eos_fill(int q) {
    /* tv = v = rhov/rho; P; c  (particle.cpp:598-601) */
    for (int d = 0; d < 3; d++) v[3 * q + d] = rhov[3 * q + d] / rho[q];
    for (int d = 0; d < 3; d++) tv[3 * q + d] = v[3 * q + d];
    int s = phase[q] - 1;
    double ei = E[q] - 0.5 * rho[q] * sqnorm_head(&v[3 * q]);
    P[q] = eos_p(ei, cs.gamma[s], cs.pinf[s]);
    c[q] = std::sqrt(cs.gamma[s] * (cs.pinf[s] + P[q]) / rho[q]);
  }
  /* Set_split_ptcl (particle.cpp:575-609) */
  void set_split(int q, int p) {
    double dr[3];
    for (int d = 0; d < 3; d++) dr[d] = x[3 * q + d] - x[3 * p + d];
    phase[q] = phase[p];
    vol[q] = (D == 3) ? vol[p] / 8.0 : vol[p] / 4.0;
    mass[q] = (D == 3) ? mass[p] / 8.0 : mass[p] / 4.0;
    h[q] = h[p] / 2.0;
    for (int t = 0; t < NS; t++) sl[NS * q + t] = sl[NS * p + t];
    double r, rv[3] = {0, 0, 0}, e;
    poly_state(p, dr, r, rv, e);
    rho[q] = r;
    for (int k = 0; k < D; k++) rhov[3 * q + k] = rv[k];
    E[q] = e;
    for (int d = 0; d < 3; d++) a[3 * q + d] = a[3 * p + d];
    eos_fill(q);
    mrg_mark[q] = 0;
    mrg[q] = 0;
  }
  /* Copy_split_state (particle.cpp:667-691): v is not copied */
  void copy_split_state(int p, int q) {
    vol[p] = vol[q]; phase[p] = phase[q]; mass[p] = mass[q]; h[p] = h[q];
    for (int d = 0; d < 3; d++) x[3 * p + d] = x[3 * q + d];
    for (int t = 0; t < NS; t++) sl[NS * p + t] = sl[NS * q + t];
    rho[p] = rho[q];
    for (int k = 0; k < D; k++) rhov[3 * p + k] = rhov[3 * q + k];
    E[p] = E[q]; c[p] = c[q];
    for (int d = 0; d < 3; d++) { a[3 * p + d] = a[3 * q + d]; tv[3 * p + d] = tv[3 * q + d]; }
    P[p] = P[q];
    mrg_mark[p] = 0;
    mrg[p] = 0;
  }
  /* Set_ptcl (particle.cpp:696-722) */
  void set_ptcl(int q, int p) {
    vol[q] = vol[p]; phase[q] = phase[p]; mass[q] = mass[p]; h[q] = h[p];
    for (int t = 0; t < NS; t++) sl[NS * q + t] = sl[NS * p + t];
    rho[q] = rho[p];
    for (int k = 0; k < D; k++) rhov[3 * q + k] = rhov[3 * p + k];
    E[q] = E[p];
    for (int d = 0; d < 3; d++) a[3 * q + d] = a[3 * p + d];
    eos_fill(q);
    mrg_mark[q] = 0;
    mrg[q] = 0;
  }
  /* Set_merge_ptcl (particle.cpp:614-661), cp == this particle */
  void set_merge(int p) {
    int q = copy[p];
    double m0 = mass[p], m1 = mass[q], v0 = vol[p], v1 = vol[q];
    double c0[3], c1[3];
    for (int d = 0; d < 3; d++) { c0[d] = x[3 * p + d]; c1[d] = x[3 * q + d]; }
    double S0[NS], S1[NS];
    for (int t = 0; t < NS; t++) { S0[t] = sl[NS * p + t]; S1[t] = sl[NS * q + t]; }
    double r0 = rho[p], r1 = rho[q];
    double rv0[3], rv1[3];
    for (int d = 0; d < 3; d++) { rv0[d] = rhov[3 * p + d]; rv1[d] = rhov[3 * q + d]; }
    double e0 = E[p], e1 = E[q];
    mass[p] = m0 + m1;
    vol[p] = v0 + v1;
    double vv = vol[p];
    h[p] = root_d(vv, D) * CELL_RATIO / CUT_OFF;
    for (int d = 0; d < 3; d++) x[3 * p + d] = (c0[d] * v0 + c1[d] * v1) / vv;
    for (int t = 0; t < NS; t++) sl[NS * p + t] = (S0[t] * v0 + S1[t] * v1) / vv;
    rho[p] = (r0 * v0 + r1 * v1) / vv;
    for (int k = 0; k < D; k++) rhov[3 * p + k] = (rv0[k] * v0 + rv1[k] * v1) / vv;
    E[p] = (e0 * v0 + e1 * v1) / vv;
    eos_fill(p);
    mrg_mark[p] = 0;
    mrg[p] = 0;
  }

  /* ------------------------------------------------------------------ */
  /* cell lists (cell_list.cpp) and neighbour scans (level_infor.cpp)   */
  /* ------------------------------------------------------------------ */
  const double* ref_x(int r) const { return is_bnd(r) ? &bx[3 * bidx(r)] : &x[3 * r]; }
  void remove_from(int64_t ci, int r) {
    auto& L = clist[ci];
    L.erase(std::remove(L.begin(), L.end(), r), L.end());
  }
  static double dist_of(const double* p, const double* q) {
    /* get_distance (glbfunc.h:175-183) */
    double dd = 0.0;
    for (int d = 0; d < D; d++) { double t = p[d] - q[d]; dd += t * t; }
    return std::sqrt(dd);
  }
  /* Level_info::Refresh_neighbor_info (level_infor.cpp:153-195), flag 2 or 3 */
  void refresh_list(int p, int flag) {
    std::vector<int>& L = nbr[p];
    L.clear();
    int pos[3];
    cell_pos(&x[3 * p], pos);
    int r = (flag == 3) ? 2 : rad2;
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      int rr = (d < D) ? r : 0;
      lo[d] = std::max(pos[d] - rr, 0);
      hi[d] = std::min(pos[d] + rr, N[d] - 1);
    }
    double lim = (flag == 3) ? cs.p_sz * 2. : h[p] * CUT_OFF;
    const double* xp = &x[3 * p];
    for (int t = lo[0]; t <= hi[0]; t++)
      for (int s = lo[1]; s <= hi[1]; s++)
        for (int m = lo[2]; m <= hi[2]; m++)
          for (int q : clist[cidx(t, s, m)]) {
            double dist = dist_of(xp, ref_x(q));
            if (dist <= lim) L.push_back(q);
          }
  }
  void mark_in_update(int p) {
    mark_in[p] = 0;
    if (x[3 * p + 0] - cs.box_l[0] < root_d(vol[p], D)) mark_in[p] = 1;  /* mpm.cpp:1398-1399 */
  }

  /* ------------------------------------------------------------------ */
  /* MPM methods                                                        */
  /* ------------------------------------------------------------------ */
  /* MPM::Set_timestep (mpm.cpp:19-57) with Particle_base::Set_timestep
   * (particle.cpp:554-569); cells when iterate_num > 1, else fluid particles. */
  int set_timestep(double* odt, double* omv) override {
    double ts = 1.e20, mv = -1.e20;
    if (iterate > 1) {
      for (int64_t ci : used_list) {
        double U2 = std::sqrt(sqnorm_head(&cv[3 * ci]));
        double hh = CELL_RATIO / CUT_OFF * cs.p_sz;  /* ini_h */
        double ds = hh / CELL_RATIO * CUT_OFF;
        double c12 = amax1(cc[ci * F + 0], cc[ci * F + 1]);
        double a12 = amax1(cac[ci * F + 0], cac[ci * F + 1]);
        double t = cs.cfl * ds / (c12 + U2);
        double tmp = cs.cfl * std::sqrt(ds / a12);
        t = amin1(t, tmp);
        ts = amin1(ts, t);
        mv = amax1(mv, U2);
      }
    } else {
      for (int p : fluid) {
        double U2 = std::sqrt(sqnorm_head(&v[3 * p]));
        double ds = h[p] / CELL_RATIO * CUT_OFF;
        double c12 = amax1(c[p], 0.0);  /* particle c[1] is never set (0) */
        double a12 = 0.0;               /* particle ac[] is never set (0) */
        double t = cs.cfl * ds / (c12 + U2);
        double tmp = cs.cfl * std::sqrt(ds / a12);
        t = amin1(t, tmp);
        ts = amin1(ts, t);
        mv = amax1(mv, U2);
      }
    }
    dt = ts;
    max_v = mv;
    if (odt) *odt = ts;
    if (omv) *omv = mv;
    return PGDG_OK;
  }

  /* MPM::Used_state_update (mpm.cpp:184-263): 5-cell dilation of cells with a
   * phase present; Used_Ele_cen in lexicographic order */
  void used_state_update() override {
    std::vector<int> us(ncell, 0);
    const int Ib[3] = {5, 5, D == 3 ? 5 : 0};
    for (int64_t ci = 0; ci < ncell; ci++) {
      if (!(cph[ci * F + 0] == 1 || cph[ci * F + 1] == 1)) continue;
      int i, j, k;
      cijk(ci, i, j, k);
      for (int t = std::max(i - Ib[0], 0); t <= std::min(i + Ib[0], N[0] - 1); t++)
        for (int s = std::max(j - Ib[1], 0); s <= std::min(j + Ib[1], N[1] - 1); s++)
          for (int q = std::max(k - Ib[2], 0); q <= std::min(k + Ib[2], N[2] - 1); q++) us[cidx(t, s, q)] = 1;
    }
    cused = us;
    used_list.clear();
    for (int64_t ci = 0; ci < ncell; ci++)
      if (cused[ci]) used_list.push_back(ci);
  }

  /* Reset_cell_list_info + Map_the_particle_to_tree (mpm.cpp:65-96) */
  void bin_particles() override {
    for (auto& L : clist) L.clear();
    for (int p : fluid) clist[cell_of(&x[3 * p])].push_back(p);
    for (int64_t b = 0; b < nbnd; b++) clist[cell_of(&bx[3 * b])].push_back(bref(b));
  }

  /* MPM::Split_particle_fast (mpm.cpp:1036-1417) */
  void split_particle_fast() override {
    const int CN = (D == 3) ? 8 : 4;
    struct SplitRec { int parent; int64_t old_cell; int child[7]; std::vector<int> old_nb; };
    struct OutRec { int p; int64_t old_cell; std::vector<int> old_nb; };
    std::vector<int> new_particles;
    std::vector<SplitRec> srec;
    std::vector<int> irec;
    std::vector<OutRec> orec;
    std::unordered_set<int> outlet_set;
    /* 1. split / inlet / outlet, in particle_fluid order */
    for (int p : fluid) {
      copy[p] = -1;
      mrg_mark[p] = 0;
      double dp = root_d(vol[p], D);
      bool f1 = vol[p] > vol_max;
      bool f2 = x[3 * p] - cs.box_l[0] >= dp && mark_in[p] == 1;
      bool f3 = x[3 * p] > cs.box_r[0];
      if (f1) {
        SplitRec rec;
        rec.parent = p;
        rec.old_cell = cell_of(&x[3 * p]);
        double pref[3] = {x[3 * p] - dp / 4., x[3 * p + 1] - dp / 4., (D == 3) ? x[3 * p + 2] - dp / 4. : 0.0};
        int child[8];
        int ci = 0;
        for (int a0 = 0; a0 < 2; ++a0)
          for (int a1 = 0; a1 < 2; ++a1)
            for (int a2 = 0; a2 < (D == 3 ? 2 : 1); ++a2) {
              int q = pmalloc();
              x[3 * q + 0] = pref[0] + dp / 2. * a0;
              x[3 * q + 1] = pref[1] + dp / 2. * a1;
              x[3 * q + 2] = (D == 3) ? pref[2] + dp / 2. * a2 : 0.0;
              set_split(q, p);
              child[ci++] = q;
            }
        rec.old_nb = nbr[p];
        copy_split_state(p, child[CN - 1]);
        pfree(child[CN - 1]);
        for (int j = 0; j < CN - 1; j++) {
          rec.child[j] = child[j];
          new_particles.push_back(child[j]);
        }
        srec.push_back(std::move(rec));
      } else if (f2) {
        int q = pmalloc();
        for (int d = 0; d < 3; d++) x[3 * q + d] = x[3 * p + d];
        x[3 * q] = x[3 * p] - dp;
        set_ptcl(q, p);
        irec.push_back(q);
        new_particles.push_back(q);
      } else if (f3) {
        OutRec rec;
        rec.p = p;
        rec.old_cell = cell_of(&x[3 * p]);
        rec.old_nb = nbr[p];
        orec.push_back(std::move(rec));
      }
    }
    for (auto& r : orec) outlet_set.insert(r.p);
    /* 2. new particles -> particle_fluid */
    for (int q : new_particles) {
      seq[q] = seq_next++;
      fluid.push_back(q);
    }
    /* 3. split cell lists */
    for (auto& r : srec) {
      remove_from(r.old_cell, r.parent);
      clist[cell_of(&x[3 * r.parent])].push_back(r.parent);
      for (int j = 0; j < CN - 1; j++) clist[cell_of(&x[3 * r.child[j]])].push_back(r.child[j]);
    }
    /* 4. inlet */
    for (int q : irec) clist[cell_of(&x[3 * q])].push_back(q);
    /* 5. outlet */
    for (auto& r : orec) remove_from(r.old_cell, r.p);
    /* 6. affected particles */
    std::vector<char> aff(vol.size(), 0);
    std::vector<char> scanned(ncell, 0);
    auto add_aff = [&](int r) {
      if (r < 0) return;  /* boundary particles: their lists are never used */
      if (outlet_set.count(r)) return;
      aff[r] = 1;
    };
    auto scan5 = [&](const double* p) {
      int pos[3];
      cell_pos(p, pos);
      int lo[3], hi[3];
      for (int d = 0; d < 3; d++) {
        int rr = (d < D) ? 2 : 0;
        lo[d] = std::max(pos[d] - rr, 0);
        hi[d] = std::min(pos[d] + rr, N[d] - 1);
      }
      for (int t = lo[0]; t <= hi[0]; t++)
        for (int s = lo[1]; s <= hi[1]; s++)
          for (int m = lo[2]; m <= hi[2]; m++) {
            int64_t ci = cidx(t, s, m);
            if (scanned[ci]) continue;
            scanned[ci] = 1;
            for (int q : clist[ci]) add_aff(q);
          }
    };
    for (auto& r : srec) {
      for (int q : r.old_nb) add_aff(q);
      int sp[8];
      sp[0] = r.parent;
      for (int j = 0; j < CN - 1; j++) sp[j + 1] = r.child[j];
      for (int j = 0; j < CN; j++) {
        add_aff(sp[j]);
        scan5(&x[3 * sp[j]]);
      }
    }
    for (int q : irec) {
      add_aff(q);
      scan5(&x[3 * q]);
    }
    for (auto& r : orec)
      for (int q : r.old_nb)
        if (q != r.p) add_aff(q);
    /* 7. reset + refresh (flag 3) */
    std::vector<int> affl;
    for (size_t s = 0; s < aff.size(); s++)
      if (aff[s]) affl.push_back((int)s);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)affl.size(); i++) refresh_list(affl[i], 3);
    /* 8. drop outlet particles, recompute mark_in */
    std::vector<int> nf;
    nf.reserve(fluid.size());
    for (int p : fluid) {
      if (outlet_set.count(p)) continue;
      mark_in_update(p);
      nf.push_back(p);
    }
    fluid.swap(nf);
    /* 9. free outlet particles */
    for (auto& r : orec) pfree(r.p);
    st.n_split += (int64_t)srec.size();
    st.n_inlet += (int64_t)irec.size();
    st.n_outlet += (int64_t)orec.size();
    st.n_affected += (int64_t)affl.size();
  }

  /* MPM::Merge_particle_fast (mpm.cpp:1536-1706), one pass */
  void merge_particle_fast() override {
    /* A: nearest small same-phase neighbour */
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)fluid.size(); i++) {
      int p = fluid[i];
      copy[p] = -1;
      mrg[p] = 0;
      mrg_mark[p] = 0;
      int cp1 = -1;
      if (vol[p] < vol_min) {
        double dss = dss0;
        for (int q : nbr[p]) {
          if (q == p) continue;
          double qvol, qphase;
          const double* qx;
          if (is_bnd(q)) { qvol = bvol; qphase = PGDG_PHASE_BOUNDARY; qx = &bx[3 * bidx(q)]; }
          else { qvol = vol[q]; qphase = phase[q]; qx = &x[3 * q]; }
          double dist = 0;
          for (int d = 0; d < D; d++) { double t = x[3 * p + d] - qx[d]; dist = (d == 0) ? t * t : dist + t * t; }
          dist = std::sqrt(dist);
          if (qvol < vol_min && dist < dss && phase[p] == qphase) {
            dss = dist;
            cp1 = q;
            mrg[p] = 1;
          }
        }
      }
      copy[p] = cp1;
    }
    /* B: mutual pairs, survivor = earlier in particle_fluid */
    struct MRec { int surv, rem; int64_t scell, rcell; std::vector<int> old_nb; };
    std::vector<MRec> recs;
    for (int p : fluid) {
      if (mrg[p] != 1) continue;
      int q = copy[p];
      if (q >= 0 && copy[q] >= 0 && copy[q] == p && mrg_mark[p] == 0) {
        MRec r;
        r.surv = p;
        r.rem = q;
        r.scell = cell_of(&x[3 * p]);
        r.rcell = cell_of(&x[3 * q]);
        r.old_nb = nbr[p];
        r.old_nb.insert(r.old_nb.end(), nbr[q].begin(), nbr[q].end());
        set_merge(p);
        mrg_mark[p] = 0;
        mrg_mark[q] = 1;
        recs.push_back(std::move(r));
      }
    }
    /* C: cell lists + affected */
    std::vector<char> aff(vol.size(), 0);
    std::vector<char> scanned(ncell, 0);
    auto add_aff = [&](int r) {
      if (r < 0) return;            /* boundary particles */
      if (mrg_mark[r] == 1) return; /* removed partners (and their slots) */
      aff[r] = 1;
    };
    for (auto& r : recs) {
      for (int q : r.old_nb)
        if (q != r.surv && q != r.rem) add_aff(q);
      remove_from(r.scell, r.surv);
      remove_from(r.rcell, r.rem);
      int pos[3];
      cell_pos(&x[3 * r.surv], pos);
      clist[cidx(pos[0], pos[1], pos[2])].push_back(r.surv);
      add_aff(r.surv);
      int lo[3], hi[3];
      for (int d = 0; d < 3; d++) {
        int rr = (d < D) ? 2 : 0;
        lo[d] = std::max(pos[d] - rr, 0);
        hi[d] = std::min(pos[d] + rr, N[d] - 1);
      }
      for (int t = lo[0]; t <= hi[0]; t++)
        for (int s = lo[1]; s <= hi[1]; s++)
          for (int m = lo[2]; m <= hi[2]; m++) {
            int64_t ci = cidx(t, s, m);
            if (scanned[ci]) continue;
            scanned[ci] = 1;
            for (int q : clist[ci]) add_aff(q);
          }
    }
    /* D: refresh (flag 3) */
    std::vector<int> affl;
    for (size_t s = 0; s < aff.size(); s++)
      if (aff[s]) affl.push_back((int)s);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)affl.size(); i++) refresh_list(affl[i], 3);
    /* E: rebuild particle_fluid */
    std::vector<int> nf;
    nf.reserve(fluid.size());
    std::vector<int> removed;
    for (int p : fluid) {
      if (mrg_mark[p] == 1) { removed.push_back(p); continue; }
      mrg[p] = 0;
      mrg_mark[p] = 0;
      copy[p] = -1;
      mark_in_update(p);
      nf.push_back(p);
    }
    fluid.swap(nf);
    for (int p : removed) {
      clearup(p);  /* mrg_mark stays 1 for the freed slot */
      freel.push_back(p);
    }
    st.n_merge += (int64_t)recs.size();
    st.n_affected += (int64_t)affl.size();
  }

  /* Reset_particle_neighbor_info(4) + Refresh_neighbor_info(4)
   * (mpm.cpp:115-158, level_infor.cpp:199-215) */
  void refresh_membership() override {
    for (int p : fluid) in_ele[p] = -1;
    for (int64_t ci : used_list) {
      cnbr[ci].clear();
      for (int q : clist[ci]) {
        if (q < 0) continue;  /* phase 10 */
        if (phase[q] == PGDG_PHASE_BOUNDARY) continue;
        cnbr[ci].push_back(q);
        if (in_ele[q] < 0) in_ele[q] = (int)ci;
      }
    }
  }

  /* Reset_particle_neighbor_info(2) + Refresh_neighbor_info(2) */
  void refresh_neighbors() override {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)fluid.size(); i++) refresh_list(fluid[i], 2);
  }

  /* 3^d stencil of a cell, clipped (mpm_ini.cpp:636-649) */
  int stencil(int64_t ci, int64_t* out) const {
    int i, j, k;
    cijk(ci, i, j, k);
    int n = 0;
    for (int t = std::max(i - 1, 0); t <= std::min(i + 1, N[0] - 1); t++)
      for (int s = std::max(j - 1, 0); s <= std::min(j + 1, N[1] - 1); s++)
        for (int q = std::max(k - 1, 0); q <= std::min(k + 1, N[2] - 1); q++) out[n++] = cidx(t, s, q);
    return n;
  }

  /* MPM::MLS_P2G (mpm.cpp:274-382) */
  void mls_p2g() override {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ii = 0; ii < (int64_t)used_list.size(); ii++) {
      int64_t ci = used_list[ii];
      const double* xc = &ccen[3 * ci];
      double mass_t[F], p_avg[F][U], Cf[F][NS];
      for (int t = 0; t < F; t++) {
        mass_t[t] = 0;
        for (int u = 0; u < U; u++) p_avg[t][u] = 0;
        for (int q = 0; q < NS; q++) Cf[t][q] = 0;
      }
      int64_t st27[27];
      int nst = stencil(ci, st27);
      for (int a0 = 0; a0 < nst; a0++) {
        for (int q : cnbr[st27[a0]]) {
          double xij[3];
          for (int d = 0; d < 3; d++) xij[d] = x[3 * q + d] - xc[d];
          double dd = 0;
          for (int d = 0; d < D; d++) dd = (d == 0) ? xij[d] * xij[d] : dd + xij[d] * xij[d];
          double dist = std::sqrt(dd);
          if (dist < 1.5 * cs.p_sz) {
            double hi = cs.p_g * 1 * 3.2 / CUT_OFF;
            double ww = kernel_w(dist, hi, D) * vol[q];
            double pj[U];
            pj[0] = rho[q];
            for (int k = 0; k < D; k++) pj[1 + k] = rhov[3 * q + k];
            pj[U - 1] = E[q];
            const double* S = &sl[NS * q];
            for (int u = 0; u < U; u++) {
              double acc = 0;
              for (int b = 0; b < D; b++) acc = (b == 0) ? S[u * D + b] * (-xij[b]) : acc + S[u * D + b] * (-xij[b]);
              pj[u] += acc;
            }
            int ph = phase[q] - 1;
            if (ph >= 0 && ph < F) {
              for (int u = 0; u < U; u++) p_avg[ph][u] += pj[u] * ww;
              for (int t = 0; t < NS; t++) Cf[ph][t] += S[t] * ww;
              mass_t[ph] += ww;
            }
          }
        }
      }
      double mass_total = 0;
      for (int t = 0; t < F; t++) mass_total += mass_t[t];
      for (int s = 0; s < F; s++) {
        int64_t cs_ = ci * F + s;
        cph[cs_] = (mass_t[s] > 0) ? 1 : 0;
        calph[cs_] = mass_t[s] / (mass_total + 1e-20);
        double* co = &ccoef[cs_ * U * B];
        if (cph[cs_] == 1 && cphb[cs_] == 0) {
          for (int t = 0; t < U * B; t++) co[t] = 0;
          for (int u = 0; u < U; u++) p_avg[s][u] /= (mass_t[s] + 1e-20);
          for (int t = 0; t < NS; t++) Cf[s][t] /= (mass_t[s] + 1e-20);
          co[0 * B + 0] = crho[cs_] = p_avg[s][0];
          for (int k = 0; k < D; k++) co[(1 + k) * B + 0] = crhov[cs_ * 3 + k] = p_avg[s][1 + k];
          co[(U - 1) * B + 0] = cE[cs_] = p_avg[s][U - 1];
          for (int u = 0; u < U; u++)
            for (int b = 0; b < D; b++) co[u * B + 1 + b] = Cf[s][u * D + b];
          for (int d = 0; d < 3; d++) cv[3 * ci + d] = crhov[cs_ * 3 + d] / crho[cs_];
          double e_j = cE[cs_] - 0.5 * sqnorm_head(&crhov[cs_ * 3]) / crho[cs_];
          cP[ci] = eos_p(e_j, cs.gamma[s], cs.pinf[s]);
          std::memcpy(&ccoef0[cs_ * U * B], co, sizeof(double) * U * B);
        }
        cphb[cs_] = cph[cs_];
        if (cph[cs_] == 0) {
          for (int t = 0; t < U * B; t++) co[t] = ccoef0[cs_ * U * B + t] = 0;
          crho[cs_] = cs.ini_rho[s];
          for (int d = 0; d < 3; d++) crhov[cs_ * 3 + d] = 0;
        }
      }
    }
  }

  static double limiter_fn(double ds, int bd_fg) {
    /* Limiter (glbfunc.h:283-299) */
    double val = 1;
    if (ds > 0 && ds < 0.5) val = 2 * ds;
    else if (ds >= 0.5) val = 1;
    if (bd_fg == 1) val = (std::fabs(ds) + ds) / (std::fabs(ds) + 1);
    return val;
  }

  /* MPM::Calculate_limiter (mpm.cpp:392-738) */
  void calculate_limiter() override {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ii = 0; ii < (int64_t)used_list.size(); ii++) {
      int64_t ci = used_list[ii];
      int i, j, k;
      cijk(ci, i, j, k);
      int idx[3] = {i, j, k};
      double u_max[F][U], u_min[F][U], pi[F][U];
      for (int s = 0; s < F; s++)
        for (int u = 0; u < U; u++) { u_max[s][u] = -1e20; u_min[s][u] = 1e20; }
      double* lim = &clim[ci * F * U];
      for (int s = 0; s < F; s++) {
        for (int u = 0; u < U; u++) lim[s * U + u] = 1.;
        pi[s][0] = crho[ci * F + s];
        for (int kk = 0; kk < D; kk++) pi[s][1 + kk] = crhov[(ci * F + s) * 3 + kk];
        pi[s][U - 1] = cE[ci * F + s];
      }
      /* G_v: central differences; one-sided with the x-sides' own v and the
       * y/z-sides' wall value 0 (mpm.cpp:469-533) */
      double* G = &cgv[ci * D * D];
      for (int t = 0; t < D * D; t++) G[t] = 0.;
      int bd_fg = 0;
      const double* vc = &cv[3 * ci];
      for (int dd = 0; dd < D; dd++) {
        double pd = cs.p_size[dd];
        if (idx[dd] == N[dd] - 1) {
          for (int r = 0; r < D; r++) G[r * D + dd] = ((dd == 0 ? vc[r] : 0.0) - vc[r]) / (0.5 * pd);
          bd_fg = 1;
        } else if (idx[dd] == 0) {
          for (int r = 0; r < D; r++) G[r * D + dd] = (vc[r] - (dd == 0 ? vc[r] : 0.0)) / (0.5 * pd);
          bd_fg = 1;
        } else {
          int lo[3] = {i, j, k}, hi[3] = {i, j, k};
          lo[dd] -= 1;
          hi[dd] += 1;
          const double* vR = &cv[3 * cidx(hi[0], hi[1], hi[2])];
          const double* vL = &cv[3 * cidx(lo[0], lo[1], lo[2])];
          for (int r = 0; r < D; r++) G[r * D + dd] = (vR[r] - vL[r]) / (2 * pd);
        }
      }
      bool mirror_j = (j == N[1] - 1 || j == 0);
      bool mirror_k = (D == 3) && (k == N[2] - 1 || k == 0);
      Face fcs[NF];
      for (int f = 0; f < NF; f++) face(ci, f, fcs[f]);
      for (int f = 0; f < NF; f++) {
        const Face& fc = fcs[f];
        double pij[U], pj[U];
        if (fc.bound == 0) {
          int64_t nb = fc.nb;
          for (int s = 0; s < F; s++) {
            for (int u = 0; u < U; u++) pj[u] = 0;
            for (int s1 = 0; s1 < F; s1++) {
              if (calph[nb * F + s1] == 0) continue;
              double rhoj = crho[nb * F + s1];
              double rvj[3];
              for (int kk = 0; kk < D; kk++) rvj[kk] = crhov[(nb * F + s1) * 3 + kk];
              double Ej = cE[nb * F + s1];
              if (s1 != s) {
                double vj[3];
                for (int kk = 0; kk < D; kk++) vj[kk] = rvj[kk] / rhoj;
                double rhoe_j = Ej - 0.5 * rhoj * sqnorm_head(vj);
                double P_j = eos_p(rhoe_j, cs.gamma[s1], cs.pinf[s1]);
                rhoj = crho[ci * F + s];
                for (int kk = 0; kk < D; kk++) rvj[kk] = rhoj * vj[kk];
                Ej = eos_rhoe(P_j, cs.gamma[s], cs.pinf[s]) + 0.5 * rhoj * sqnorm_head(vj);
              }
              double tmp[U];
              tmp[0] = rhoj;
              for (int kk = 0; kk < D; kk++) tmp[1 + kk] = rvj[kk];
              tmp[U - 1] = Ej;
              for (int u = 0; u < U; u++) pj[u] += tmp[u] * calph[nb * F + s1];
            }
            for (int u = 0; u < U; u++) {
              pij[u] = pj[u] - pi[s][u];
              u_max[s][u] = amax1(u_max[s][u], pij[u]);
              u_min[s][u] = amin1(u_min[s][u], pij[u]);
            }
          }
        } else {
          for (int s = 0; s < F; s++) {
            const double* rvc = &crhov[(ci * F + s) * 3];
            pj[0] = crho[ci * F + s];
            for (int kk = 0; kk < D; kk++) pj[1 + kk] = rvc[kk];
            pj[U - 1] = cE[ci * F + s];
            if (fc.bound == PGDG_BC_INLET || fc.bound == PGDG_BC_OUTLET || fc.bound == PGDG_BC_TRANSMISSIVE)
              for (int u = 0; u < U; u++) pj[u] = pi[s][u];
            if (fc.bound != PGDG_BC_TRANSMISSIVE) {
              if (mirror_j) pj[1 + 1] = -rvc[1];
              if (mirror_k) pj[1 + 2] = -rvc[2];
            }
            for (int u = 0; u < U; u++) {
              pij[u] = pj[u] - pi[s][u];
              u_max[s][u] = amax1(u_max[s][u], pij[u]);
              u_min[s][u] = amin1(u_min[s][u], pij[u]);
            }
          }
        }
      }
      for (int s = 0; s < F; s++)
        for (int u = 0; u < U; u++) {
          u_max[s][u] = amax1(u_max[s][u], 0.);
          u_min[s][u] = amin1(u_min[s][u], 0.);
        }
      for (int f = 0; f < NF; f++) {
        const Face& fc = fcs[f];
        double dr[3];
        for (int d = 0; d < 3; d++) dr[d] = fc.cen[d] - ccen[3 * ci + d];
        if (fc.bound == 0)
          for (int d = 0; d < 3; d++) dr[d] = ccen[3 * fc.nb + d] - ccen[3 * ci + d];
        for (int s = 0; s < F; s++) {
          const double* co = &ccoef[(ci * F + s) * U * B];
          int lim_fg = bd_fg;
          if (calph[ci * F + s] != 1) lim_fg = 1;
          for (int u = 0; u < U; u++) {
            double dU = 0;
            for (int b = 0; b < D; b++) dU = (b == 0) ? co[u * B + 1 + b] * dr[b] : dU + co[u * B + 1 + b] * dr[b];
            double sd = 1;
            if (dU >= 0) {
              sd = u_max[s][u] / (dU + 1e-20);
              sd = limiter_fn(std::fabs(sd), lim_fg);
            } else if (dU < 0) {
              sd = u_min[s][u] / (dU + 1e-20);
              sd = limiter_fn(std::fabs(sd), lim_fg);
            }
            lim[s * U + u] = amin1(lim[s * U + u], sd);
          }
        }
      }
      /* positivity probe */
      const int NPR = (D == 3) ? 8 : 4;
      for (int s = 0; s < F; s++) {
        const double* co = &ccoef[(ci * F + s) * U * B];
        const double gs = cs.gamma[s], ps_ = cs.pinf[s];
        int fg = 0;
        for (int pr = 0; pr < NPR && !fg; pr++) {
          const double* dr = cs.probe[pr];
          double Ui[U];
          for (int u = 0; u < U; u++) {
            double acc = 0;
            for (int b = 0; b < D; b++) acc = (b == 0) ? co[u * B + 1 + b] * dr[b] : acc + co[u * B + 1 + b] * dr[b];
            Ui[u] = co[u * B + 0] + lim[s * U + u] * acc;
          }
          double rho_p = Ui[0], E_p = Ui[U - 1];
          double sq = Ui[1] * Ui[1];
          for (int kk = 1; kk < D; kk++) sq = sq + Ui[1 + kk] * Ui[1 + kk];
          double e_p = E_p - 0.5 * sq / rho_p;
          double P_p = eos_p(e_p, gs, ps_);
          if (P_p < -0.05 * ps_ || rho_p < 0) fg = 1;
        }
        if (fg) for (int u = 0; u < U; u++) lim[s * U + u] = 0.;
      }
    }
  }

  /* Particle_base::Grid_acceleration (particle_flow.cpp:16-405) for one
   * (cell, phase); MPM::Grid_acceleration (mpm.cpp:747-763) */
  void grid_acc_cell(int64_t ci, int ss, int64_t& ncall, int64_t& nit, int64_t& nmax) {
    int i, j, k;
    cijk(ci, i, j, k);
    const double gs = cs.gamma[ss], pis = cs.pinf[ss];
    double ps[3] = {cs.p_size[0] / 2, cs.p_size[1] / 2, cs.p_size[2] / 2};
    double* dc = &cdcoef[(ci * F + ss) * U * B];
    for (int t = 0; t < U * B; t++) dc[t] = 0;
    const double* co = &ccoef[(ci * F + ss) * U * B];
    const double* L = &clim[(ci * F + ss) * U];
    double voli = cs.p_size[0] * cs.p_size[1];
    if (D == 3) voli = voli * cs.p_size[2];
    double mij[B];
    mij[0] = 1. * voli;
    for (int d = 0; d < D; d++) mij[1 + d] = (ps[d] * ps[d] / 3.) * voli;
    const double* xc = &ccen[3 * ci];

    auto recon = [&](const double* cf, const double* Lm, const double* dr, double* Uo) {
      for (int u = 0; u < U; u++) {
        double acc = 0;
        for (int b = 0; b < D; b++) acc = (b == 0) ? cf[u * B + 1 + b] * dr[b] : acc + cf[u * B + 1 + b] * dr[b];
        Uo[u] = cf[u * B + 0] + Lm[u] * acc;
      }
    };
    auto flux = [&](const double* Uu, const double* vv, double Pp, double DF[U][D]) {
      for (int u = 0; u < U; u++)
        for (int kk = 0; kk < D; kk++) DF[u][kk] = Uu[u] * vv[kk];
      for (int kk = 0; kk < D; kk++) DF[1 + kk][kk] += Pp;
      for (int kk = 0; kk < D; kk++) DF[U - 1][kk] += vv[kk] * Pp;
    };
    /* volume integral */
    const int NG = (D == 3) ? 8 : 4;
    for (int g = 0; g < NG; g++) {
      int g1 = (D == 3) ? (g >> 2) : (g >> 1), g2 = (D == 3) ? ((g >> 1) & 1) : (g & 1), g3 = g & 1;
      double dp[3] = {Gp[g1] * ps[0], Gp[g2] * ps[1], (D == 3) ? Gp[g3] * ps[2] : 0.0};
      double gw = Gw[g1] * Gw[g2];
      if (D == 3) gw = Gw[g1] * Gw[g2] * Gw[g3];
      double Up[U];
      recon(co, L, dp, Up);
      double rho_p = Up[0];
      double vp[3];
      for (int kk = 0; kk < D; kk++) vp[kk] = Up[1 + kk] / rho_p;
      double sq = Up[1] * Up[1];
      for (int kk = 1; kk < D; kk++) sq = sq + Up[1 + kk] * Up[1 + kk];
      double e_p = Up[U - 1] - 0.5 * sq / rho_p;
      double P_p = eos_p(e_p, gs, pis);
      double DF[U][D];
      flux(Up, vp, P_p, DF);
      for (int bi = 1; bi <= D; bi++)
        for (int u = 0; u < U; u++) dc[u * B + bi] += DF[u][bi - 1] * gw * voli * 1;
    }
    /* face integral */
    Face fcs[NF];
    for (int f = 0; f < NF; f++) face(ci, f, fcs[f]);
    bool mirror_j = (j == N[1] - 1 || j == 0);
    bool mirror_k = (D == 3) && (k == N[2] - 1 || k == 0);
    const int NQ = (D == 3) ? 4 : 2;
    for (int f = 0; f < NF; f++) {
      const Face& fc = fcs[f];
      double DFij[B][U][D];
      for (int bi = 0; bi < B; bi++)
        for (int u = 0; u < U; u++)
          for (int kk = 0; kk < D; kk++) DFij[bi][u][kk] = 0;
      for (int q = 0; q < NQ; q++) {
        int g1 = (D == 3) ? (q >> 1) : q, g2 = q & 1;
        double dpv[3];
        double gw;
        if (D == 3) {
          for (int d = 0; d < 3; d++) dpv[d] = Gp[g1] * fc.t0[d] + Gp[g2] * fc.t1[d];
          gw = Gw[g1] * Gw[g2];
        } else {
          for (int d = 0; d < 3; d++) dpv[d] = Gp[g1] * fc.t0[d];
          gw = Gw[g1];
        }
        double dri[3];
        for (int d = 0; d < 3; d++) dri[d] = dpv[d] + fc.cen[d] - xc[d];
        double Ui[U];
        recon(co, L, dri, Ui);
        double rho_i = Ui[0], E_i = Ui[U - 1];
        double v_i[3];
        for (int kk = 0; kk < D; kk++) v_i[kk] = Ui[1 + kk] / rho_i;
        double sq = Ui[1] * Ui[1];
        for (int kk = 1; kk < D; kk++) sq = sq + Ui[1 + kk] * Ui[1 + kk];
        double e_i = E_i - 0.5 * sq / rho_i;
        double P_i = eos_p(e_i, gs, pis);
        double ci_ = std::sqrt(gs * (pis + P_i) / rho_i);
        double vni = 0;
        for (int kk = 0; kk < D; kk++) vni = (kk == 0) ? v_i[kk] * fc.n[kk] : vni + v_i[kk] * fc.n[kk];
        double DFi[U][D];
        flux(Ui, v_i, P_i, DFi);
        double Nb[B];
        Nb[0] = 1.;
        for (int d = 0; d < D; d++) Nb[1 + d] = dri[d];
        if (fc.bound == 0) {
          int64_t nb = fc.nb;
          for (int s1 = 0; s1 < F; s1++) {
            double aj = calph[nb * F + s1];
            if (aj == 0) continue;
            double drj[3];
            for (int d = 0; d < 3; d++) drj[d] = dpv[d] + fc.cen[d] - ccen[3 * nb + d];
            double Uj[U];
            recon(&ccoef[(nb * F + s1) * U * B], &clim[(nb * F + s1) * U], drj, Uj);
            double rho_j = Uj[0], E_j = Uj[U - 1];
            double rhov_j[3], v_j[3];
            for (int kk = 0; kk < D; kk++) { rhov_j[kk] = Uj[1 + kk]; v_j[kk] = rhov_j[kk] / rho_j; }
            double rhoe_j = E_j - 0.5 * sqnorm_head(v_j) * rho_j;
            double P_j = eos_p(rhoe_j, cs.gamma[s1], cs.pinf[s1]);
            double vnj = 0;
            for (int kk = 0; kk < D; kk++) vnj = (kk == 0) ? v_j[kk] * fc.n[kk] : vnj + v_j[kk] * fc.n[kk];
            if (ss != s1) {
              double gh[3];
              int it = 0;
              mgfm(vni, vnj, P_i, P_j, rho_i, rho_j, gs, pis, cs.gamma[s1], cs.pinf[s1], cs.mgfm_variant, -1.0, gh, &it);
              ncall++;
              nit += it;
              if (it >= 50) nmax++;
              rho_j = gh[0];
              P_j = gh[1];
              vnj = gh[2];
              for (int kk = 0; kk < D; kk++) v_j[kk] = v_i[kk] - vni * fc.n[kk] + vnj * fc.n[kk];
              for (int kk = 0; kk < D; kk++) rhov_j[kk] = rho_j * v_j[kk];
              rhoe_j = eos_rhoe(P_j, gs, pis);
              E_j = rhoe_j + 0.5 * rho_j * sqnorm_head(v_j);
            }
            double cj = std::sqrt(gs * (pis + P_j) / rho_j);
            double Ujj[U];
            Ujj[0] = rho_j;
            for (int kk = 0; kk < D; kk++) Ujj[1 + kk] = rhov_j[kk];
            Ujj[U - 1] = E_j;
            double DFj[U][D];
            flux(Ujj, v_j, P_j, DFj);
            vni = 0;
            for (int kk = 0; kk < D; kk++) vni = (kk == 0) ? v_i[kk] * fc.n[kk] : vni + v_i[kk] * fc.n[kk];
            vnj = 0;
            for (int kk = 0; kk < D; kk++) vnj = (kk == 0) ? v_j[kk] * fc.n[kk] : vnj + v_j[kk] * fc.n[kk];
            double SL = amin1((vni - ci_), (vnj - cj));
            double SR = amax1((vni + ci_), (vnj + cj));
            double S_s = ((P_j - P_i) + rho_i * vni * (SL - vni) - rho_j * vnj * (SR - vnj)) /
                         (rho_i * (SL - vni) - rho_j * (SR - vnj));
            double rho_sL = rho_i * (SL - vni) / (SL - S_s);
            double rho_sR = rho_j * (SR - vnj) / (SR - S_s);
            double UsL[U], UsR[U];
            UsL[0] = rho_sL;
            UsR[0] = rho_sR;
            for (int kk = 0; kk < D; kk++) {
              UsL[1 + kk] = rho_sL * (v_i[kk] + (S_s - vni) * fc.n[kk]);
              UsR[1 + kk] = rho_sR * (v_j[kk] + (S_s - vnj) * fc.n[kk]);
            }
            UsL[U - 1] = rho_sL * (E_i / rho_i + (S_s - vni) * (S_s + (P_i) / (rho_i * (SL - vni))));
            UsR[U - 1] = rho_sR * (E_j / rho_j + (S_s - vnj) * (S_s + (P_j) / (rho_j * (SR - vnj))));
            double DFh[U][D];
            for (int u = 0; u < U; u++)
              for (int kk = 0; kk < D; kk++) DFh[u][kk] = 0;
            if (SL > 0) {
              std::memcpy(DFh, DFi, sizeof(DFh));
            } else if (SL <= 0 && S_s >= 0) {
              for (int u = 0; u < U; u++)
                for (int kk = 0; kk < D; kk++) DFh[u][kk] = DFi[u][kk] + SL * (UsL[u] - Ui[u]) * fc.n[kk];
            } else if (S_s <= 0 && SR >= 0) {
              for (int u = 0; u < U; u++)
                for (int kk = 0; kk < D; kk++) DFh[u][kk] = DFj[u][kk] + SR * (UsR[u] - Ujj[u]) * fc.n[kk];
            } else if (SR <= 0) {
              std::memcpy(DFh, DFj, sizeof(DFh));
            }
            for (int bi = 0; bi < B; bi++)
              for (int u = 0; u < U; u++)
                for (int kk = 0; kk < D; kk++) DFij[bi][u][kk] += DFh[u][kk] * Nb[bi] * gw * aj;
          }
        } else if (fc.bound == PGDG_BC_WALL) {
          for (int bi = 0; bi < B; bi++)
            for (int kk = 0; kk < D; kk++) DFij[bi][1 + kk][kk] += P_i * Nb[bi] * gw;
        } else {
          double rho_j = rho_i;
          double v_j[3], rhov_j[3];
          for (int kk = 0; kk < D; kk++) { v_j[kk] = v_i[kk]; rhov_j[kk] = rho_j * v_j[kk]; }
          double P_j = P_i, E_j = E_i;
          if (fc.bound == PGDG_BC_INLET) {
            rho_j = cs.inlet_rho;
            for (int kk = 0; kk < D; kk++) v_j[kk] = cs.inlet_u[kk];
            for (int kk = 0; kk < D; kk++) rhov_j[kk] = rho_j * v_j[kk];
            P_j = cs.inlet_p;
            E_j = eos_rhoe(P_j, gs, pis) + 0.5 * sqnorm_head(v_j) * rho_j;
          }
          if (fc.bound != PGDG_BC_TRANSMISSIVE) {
            if (mirror_j) {
              v_j[1] = -v_i[1];
              for (int kk = 0; kk < D; kk++) rhov_j[kk] = rho_j * v_j[kk];
            }
            if (mirror_k) {
              v_j[2] = -v_i[2];
              for (int kk = 0; kk < D; kk++) rhov_j[kk] = rho_j * v_j[kk];
            }
          }
          double Uj[U];
          Uj[0] = rho_j;
          for (int kk = 0; kk < D; kk++) Uj[1 + kk] = rhov_j[kk];
          Uj[U - 1] = E_j;
          double cj = std::sqrt(gs * (pis + P_j) / rho_j);
          double vnj = 0;
          for (int kk = 0; kk < D; kk++) vnj = (kk == 0) ? v_j[kk] * fc.n[kk] : vnj + v_j[kk] * fc.n[kk];
          double DFj[U][D];
          flux(Uj, v_j, P_j, DFj);
          double SL = amin1((vni - ci_), (vnj - cj));
          double SR = amax1((vni + ci_), (vnj + cj));
          double DFh[U][D];
          for (int u = 0; u < U; u++)
            for (int kk = 0; kk < D; kk++) DFh[u][kk] = 0;
          if (SL > 0) {
            std::memcpy(DFh, DFi, sizeof(DFh));
          } else if (SL <= 0 && SR >= 0) {
            for (int u = 0; u < U; u++)
              for (int kk = 0; kk < D; kk++)
                DFh[u][kk] = (SR * DFi[u][kk] - SL * DFj[u][kk] + SL * SR * (Uj[u] - Ui[u]) * fc.n[kk]) / (SR - SL);
          } else if (SR < 0) {
            std::memcpy(DFh, DFj, sizeof(DFh));
          }
          for (int bi = 0; bi < B; bi++)
            for (int u = 0; u < U; u++)
              for (int kk = 0; kk < D; kk++) DFij[bi][u][kk] += DFh[u][kk] * Nb[bi] * gw;
        }
      }
      for (int bi = 0; bi < B; bi++)
        for (int u = 0; u < U; u++) {
          double acc = 0;
          for (int kk = 0; kk < D; kk++) acc = (kk == 0) ? -(DFij[bi][u][kk]) * fc.n[kk] : acc + -(DFij[bi][u][kk]) * fc.n[kk];
          dc[u * B + bi] += acc * fc.S;
        }
    }
    for (int s = 0; s < B; s++) {
      double inv = 1. / (mij[s] + 1e-20);
      for (int u = 0; u < U; u++) dc[u * B + s] *= inv;
    }
  }

  void grid_acceleration() override {
    int64_t ncall = 0, nit = 0, nmax = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : ncall, nit, nmax)
    for (int64_t ii = 0; ii < (int64_t)used_list.size(); ii++) {
      int64_t ci = used_list[ii];
      for (int s = 0; s < F; s++)
        if (cph[ci * F + s] == 1) grid_acc_cell(ci, s, ncall, nit, nmax);
    }
    st.mgfm_calls += ncall;
    st.mgfm_iters += nit;
    st.mgfm_maxit_hits += nmax;
  }

  /* MPM::Update_grid (mpm.cpp:768-830) */
  void update_grid(int md) override {
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)used_list.size(); ii++) {
      int64_t ci = used_list[ii];
      double rhov_a[3] = {0, 0, 0}, rho_a = 0, P_a = 0;
      for (int s = 0; s < F; s++) {
        int64_t cs_ = ci * F + s;
        cc[cs_] = 0;
        cac[cs_] = 0;
        double* co = &ccoef[cs_ * U * B];
        double* d = &cdcoef[cs_ * U * B];
        double* c0 = &ccoef0[cs_ * U * B];
        const double* L = &clim[cs_ * U];
        for (int t = 0; t < U; t++)
          for (int b = 1; b < B; b++) {
            d[t * B + b] *= std::fabs(L[t]);
            co[t * B + b] *= std::fabs(L[t]);
          }
        if (cph[cs_] == 1) {
          if (md == 0) {
            for (int t = 0; t < U * B; t++) c0[t] = co[t];
            for (int t = 0; t < U * B; t++) co[t] = co[t] + d[t] * dt;
          } else {
            for (int t = 0; t < U * B; t++) co[t] = 0.5 * (d[t] * dt + co[t] + c0[t]);
          }
          crho[cs_] = co[0];
          for (int kk = 0; kk < D; kk++) crhov[cs_ * 3 + kk] = co[(1 + kk) * B];
          cE[cs_] = co[(U - 1) * B];
          double e_j = cE[cs_] - 0.5 * sqnorm_head(&crhov[cs_ * 3]) / crho[cs_];
          cP[ci] = eos_p(e_j, cs.gamma[s], cs.pinf[s]);
          cc[cs_] = std::sqrt(cs.gamma[s] * (cs.pinf[s] + cP[ci]) / crho[cs_]);
          for (int kk = 0; kk < D; kk++) ca[3 * ci + kk] = (d[(1 + kk) * B] - d[0] * cv[3 * ci + kk]) / crho[cs_];
          cac[cs_] = std::sqrt(sqnorm_head(&ca[3 * ci]));
        }
        for (int dd = 0; dd < 3; dd++) rhov_a[dd] += crhov[cs_ * 3 + dd] * calph[cs_];
        rho_a += crho[cs_] * calph[cs_];
        P_a += cP[ci] * calph[cs_];
      }
      for (int dd = 0; dd < 3; dd++) cv[3 * ci + dd] = rhov_a[dd] / rho_a;
      cP[ci] = P_a;
    }
  }

  /* MPM::Update_particle (mpm.cpp:839-853): pass 1 Update_state_onestep
   * (particle_flow.cpp:413-477) for every particle, pass 2 Update_PST
   * (particle_flow.cpp:485-622) for every particle. */
  void update_particle(int md) override {
    int64_t nfb = 0;
#pragma omp parallel for schedule(static) reduction(+ : nfb)
    for (int64_t i = 0; i < (int64_t)fluid.size(); i++) {
      int p = fluid[i];
      int64_t ci = in_ele[p];
      int ss = phase[p] - 1;
      const double* G = &cgv[ci * D * D];
      double divu = G[0];
      for (int kk = 1; kk < D; kk++) divu = divu + G[kk * D + kk];
      double* xp = &x[3 * p];
      if (md == 0) {
        for (int d = 0; d < 3; d++) x0[3 * p + d] = xp[d];
        vol0[p] = vol[p];
        for (int d = 0; d < D; d++) xp[d] += tv[3 * p + d] * dt;
        vol[p] = (1. + divu * dt) * vol[p];
      } else {
        for (int d = 0; d < D; d++) xp[d] = 0.5 * ((x0[3 * p + d] + xp[d]) + tv[3 * p + d] * dt);
        vol[p] = 0.5 * (vol0[p] + vol[p] + divu * dt * vol[p]);
      }
      double dri[3];
      for (int d = 0; d < 3; d++) dri[d] = xp[d] - ccen[3 * ci + d];
      const double* co = &ccoef[(ci * F + ss) * U * B];
      double Ui[U];
      for (int t = 0; t < U; t++) {
        double acc = 0;
        for (int b = 0; b < D; b++) acc = (b == 0) ? co[t * B + 1 + b] * dri[b] : acc + co[t * B + 1 + b] * dri[b];
        Ui[t] = co[t * B + 0] + 1 * acc;
      }
      for (int t = 0; t < U; t++)
        for (int b = 0; b < D; b++) sl[NS * p + t * D + b] = co[t * B + 1 + b];
      rho[p] = Ui[0];
      for (int d = 0; d < 3; d++) rhov[3 * p + d] = (d < D) ? Ui[1 + d] : 0.0;
      E[p] = Ui[U - 1];
      for (int d = 0; d < 3; d++) v[3 * p + d] = rhov[3 * p + d] / rho[p];
      double ei = E[p] - 0.5 * rho[p] * sqnorm_head(&v[3 * p]);
      P[p] = eos_p(ei, cs.gamma[ss], cs.pinf[ss]);
      c[p] = std::sqrt(cs.gamma[ss] * (cs.pinf[ss] + P[p]) / rho[p]);
      if (P[p] < -0.05 * cs.pinf[ss] || rho[p] < 0) {
        for (int t = 0; t < NS; t++) sl[NS * p + t] = 0;
        rho[p] = crho[ci * F + ss];
        for (int d = 0; d < 3; d++) rhov[3 * p + d] = crhov[(ci * F + ss) * 3 + d];
        E[p] = cE[ci * F + ss];
        c[p] = cc[ci * F + ss];
        nfb++;
      }
      mass[p] = vol[p] * rho[p];
      h[p] = root_d(vol[p], D) * CELL_RATIO / CUT_OFF;
    }
    st.g2p_fallbacks += nfb;
    const double px = cs.p_sz;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)fluid.size(); i++) {
      int p = fluid[i];
      double pst[3] = {0, 0, 0}, phs[3] = {0, 0, 0};
      /* PST (particle_flow.cpp:530-581) */
      double ca_ = max_v * 5.;
      double P_b = rho[p] * ca_ * ca_;
      double hh = h[p];
      double dxk = hh / CELL_RATIO * CUT_OFF;
      double W_dp = kernel_w(dxk, hh, D);
      const double* xp = &x[3 * p];
      for (int q : nbr[p]) {
        const double* qx = ref_x(q);
        double dr[3];
        for (int d = 0; d < 3; d++) dr[d] = xp[d] - qx[d];
        double dd = dr[0] * dr[0];
        for (int d = 1; d < D; d++) dd = dd + dr[d] * dr[d];
        double dist = std::sqrt(dd);
        if (dist != 0) {
          bool bnd = is_bnd(q);
          double vol_j = bnd ? bvol : vol[q];
          double aw = kernel_dw(dist, hh, D);
          double awax[3];
          for (int d = 0; d < 3; d++) awax[d] = (d < D) ? dr[d] * aw : dr[d];
          double Wij = kernel_w(dist, hh, D);
          double rr = Wij / W_dp;
          double R = 0.2 * ((rr * rr) * (rr * rr));
          double tmp1 = -1. * P_b * (1. / rho[p]) * (1 + R);
          double rho_q = bnd ? brho : rho[q];
          double tmp2 = 1. / (rho[p] + rho_q);
          if (!bnd) {
            for (int d = 0; d < 3; d++) pst[d] += awax[d] * tmp1 * vol_j;
            if (phase[q] != phase[p]) {
              double coefs = -0.1 * tmp2 * (c[p] * c[p] * rho[p] + c[q] * c[q] * rho[q]);
              for (int d = 0; d < 3; d++) phs[d] += coefs * awax[d] * vol_j;
            }
          } else {
            const double* nn = &bn[3 * bidx(q)];
            for (int d = 0; d < 3; d++) pst[d] += nn[d] * Wij * tmp1 * vol_j;
          }
        }
      }
      /* Bound_pen (particle_flow.cpp:587-622) */
      double bp[3] = {0, 0, 0};
      int64_t ci = in_ele[p];
      for (int f = 0; f < NF; f++) {
        Face fc;
        face(ci, f, fc);
        if (fc.bound == 0) continue;
        double nn[3] = {fc.n[0], fc.n[1], fc.n[2]};
        double ds = 0;
        for (int d = 0; d < D; d++) ds = (d == 0) ? (xp[d] - fc.cen[d]) * nn[d] : ds + (xp[d] - fc.cen[d]) * nn[d];
        if (ds < 0)
          for (int d = 0; d < 3; d++) nn[d] = -1 * nn[d];
        double dis = std::fabs(ds);
        if (dis < 0.4 * cs.p_sz) {
          double sc = 0.02 / dis * (c[p] * c[p]);
          for (int d = 0; d < 3; d++) bp[d] += sc * nn[d];
        }
      }
      /* Update_PST (particle_flow.cpp:485-525) */
      double dx[3], dx1[3], dx2[3];
      for (int d = 0; d < 3; d++) {
        dx[d] = pst[d] * dt * dt / 2.;
        dx1[d] = phs[d] * dt * dt / 2.;
        dx2[d] = bp[d] * dt * dt / 2.;
      }
      double dis = std::sqrt(sqnorm_head(dx));
      double l0 = amin1(px / 10, dis) / (dis + 1e-20);
      double dis1 = std::sqrt(sqnorm_head(dx1));
      double l1 = amin1(px / 10, dis1) / (dis1 + 1e-20);
      double dis2 = std::sqrt(sqnorm_head(dx2));
      double l2 = amin1(px / 2, dis2) / (dis2 + 1e-20);
      for (int d = 0; d < 3; d++) {
        dx[d] *= l0;
        dx1[d] *= l1;
        dx2[d] *= l2;
      }
      for (int d = 0; d < 3; d++) {
        double dv = (dx[d] + dx1[d] + dx2[d]) / dt;
        if (mark_in[p] == 1) dv = 0;
        tv[3 * p + d] = v[3 * p + d] + dv;
      }
    }
  }

  /* MPM::MPM_run_simulation (mpm_ini.cpp:682-766) */
  void run_step(int64_t n) override {
    st.time += dt; /* simulated time (Solver::MPM_Solver's integral_time) */
    if (n == 1) used_state_update();
    bin_particles();
    split_particle_fast();
    for (int it = 0; it < cs.merge_iters; it++) merge_particle_fast();
    refresh_membership();
    for (int md = 0; md < 2; md++) {
      refresh_neighbors();
      if (md == 0) mls_p2g();
      calculate_limiter();
      grid_acceleration();
      update_grid(md);
      update_particle(md);
    }
  }

  /* double-double running sum (TwoSum of each addend, the errors summed beside
   * it: Neumaier's compensated summation), rounded once: the result does not
   * depend on the order of the addends (the reference reduces under TBB in no
   * fixed order) */
  struct DDs {
    double hi = 0, lo = 0;
    void add(double b) {
      const double s = hi + b, bb = s - hi;
      lo += (hi - (s - bb)) + (b - bb);
      hi = s;
    }
    double value() const { return hi + lo; }
  };
  /* conservation totals (Triple_point_2phase/mpm_ini.cpp:599-654: particle
   * mass per phase and energy, cell mass per phase and energy) */
  void totals(double* out) override {
    DDs pm[F], pe, cm[F], ce;
    for (int p : fluid) {
      pm[phase[p] - 1].add(rho[p] * vol[p]);
      pe.add(E[p] * vol[p]);
    }
    double voli = cs.p_size[0] * cs.p_size[1] * (D == 3 ? cs.p_size[2] : 1.0);
    for (int64_t ci : used_list)
      for (int s = 0; s < F; s++) {
        if (cph[ci * F + s] != 1) continue;
        cm[s].add(voli * calph[ci * F + s] * crho[ci * F + s]);
        ce.add(voli * calph[ci * F + s] * cE[ci * F + s]);
      }
    /* per phase particle masses, particle energy, per phase cell masses, cell energy */
    for (int s = 0; s < F; s++) out[s] = pm[s].value();
    out[F] = pe.value();
    for (int s = 0; s < F; s++) out[F + 1 + s] = cm[s].value();
    out[2 * F + 1] = ce.value();
  }
  /* MPM::Output_plt_file (mpm_ini.cpp:832-980): the particles as a Tecplot
   * binary (#!TDV112, one ordered zone, twelve variables stored one after the
   * other, doubles and int32) and the cells as an ASCII table written through
   * an ostream in its default format.  Test infrastructure: the reference for
   * the library's writer. */
  template <class T>
  static void put(std::ofstream& o, T v) { o.write(reinterpret_cast<const char*>(&v), sizeof(v)); }
  static void put_name(std::ofstream& o, const char* s) {
    /* each character as an int32, then a 0 */
    for (const char* c = s; *c; c++) put<int32_t>(o, (int32_t)(unsigned char)*c);
    put<int32_t>(o, 0);
  }
  int output_plt(const char* ppath, const char* cpath) override {
    if (ppath) {
      std::ofstream o(ppath, std::ios::binary);
      if (!o) return PGDG_EINVAL;
      o.write("#!TDV112", 8);
      put<int32_t>(o, 1);
      put<int32_t>(o, 0);
      put<int32_t>(o, 0);
      static const char* names[12] = {"x", "y", "z", "phase", "vx", "vy", "vol", "rho", "P", "tv", "v", "n_neighbor"};
      static const int32_t types[12] = {2, 2, 2, 3, 2, 2, 2, 2, 2, 2, 2, 3};
      put<int32_t>(o, 12);
      for (auto n : names) put_name(o, n);
      put<float>(o, 299.0f);
      put_name(o, "grid");
      put<int32_t>(o, -1);
      put<int32_t>(o, 0);
      put<double>(o, st.time);
      put<int32_t>(o, -1);
      put<int32_t>(o, 0);
      put<int32_t>(o, 0);
      put<int32_t>(o, 0);
      put<int32_t>(o, 0);
      put<int32_t>(o, (int32_t)fluid.size());
      put<int32_t>(o, 1);
      put<int32_t>(o, 1);
      put<int32_t>(o, 0);
      put<float>(o, 357.0f);
      put<float>(o, 299.0f);
      for (auto t : types) put<int32_t>(o, t);
      put<int32_t>(o, 0);
      put<int32_t>(o, 0);
      put<int32_t>(o, -1);
      for (int j = 0; j < 12; j++) {
        put<double>(o, -1.0);
        put<double>(o, 1.0);
      }
      for (int j = 0; j < 12; j++)
        for (int p : fluid) {
          const double* xp = &x[3 * p];
          auto nrm = [&](const double* a) {
            double q = a[0] * a[0];
            for (int d = 1; d < D; d++) q = q + a[d] * a[d];
            return std::sqrt(q);
          };
          switch (j) {
            case 0: put<double>(o, xp[0]); break;
            case 1: put<double>(o, xp[1]); break;
            case 2: put<double>(o, D == 3 ? xp[2] : 0.0); break;
            case 3: put<int32_t>(o, phase[p]); break;
            case 4: put<double>(o, v[3 * p]); break;
            case 5: put<double>(o, v[3 * p + 1]); break;
            case 6: put<double>(o, vol[p]); break;
            case 7: put<double>(o, rho[p]); break;
            case 8: put<double>(o, P[p]); break;
            case 9: put<double>(o, nrm(&tv[3 * p])); break;
            case 10: put<double>(o, nrm(&v[3 * p])); break;
            default: put<int32_t>(o, (int32_t)nbr[p].size()); break;
          }
        }
      if (!o) return PGDG_EINVAL;
    }
    if (cpath) {
      std::ofstream o(cpath, std::ios::trunc);
      if (!o) return PGDG_EINVAL;
      o << "VARIABLES = \"x\",\"y\",\"z\", \"v1\",\"v2\", \"v\",\"rho0\",\"rho1\",        "
           "\"E0\",\"E1\",\"Lim0\",\"Lim1\",\"st\", \"st1\", \"P\"\n";
      o << "ZONE T=" << "\"GRID 1\"," << "SOLUTIONTIME=" << st.time << "\n";
      for (int64_t ci = 0; ci < ncell; ci++) {
        const double* vc = &cv[3 * ci];
        double q = vc[0] * vc[0];
        for (int d = 1; d < D; d++) q = q + vc[d] * vc[d];
        const double* co = &ccoef[(ci * F + 0) * U * B];
        o << ccen[3 * ci] << ' ' << ccen[3 * ci + 1] << ' ' << ccen[3 * ci + 2] << ' ' << vc[0] << ' ' << vc[1] << ' '
          << std::sqrt(q) << ' ' << crho[ci * F + 0] << ' ' << crho[ci * F + 1] << ' ' << co[1 * B + 1] << ' '
          << co[1 * B + 2] << ' ' << clim[(ci * F + 0) * U] << ' ' << clim[(ci * F + 1) * U] << ' '
          << calph[ci * F + 0] << ' ' << calph[ci * F + 1] << ' ' << cP[ci] << ' ' << '\n';
      }
      if (!o) return PGDG_EINVAL;
    }
    return PGDG_OK;
  }

  /* MPM::Output_point (mpm_ini.cpp:774-824): bubble extents along the axis and
   * the phase-2 mass, over particle_fluid in order (the ends start at the
   * box's left and right x) */
  void output_point(double* out) override {
    double dw = cs.box_l[0], jet = cs.box_r[0], ups = cs.box_r[0];
    DDs mass;
    const double a = 2.5 * cs.p_sz, b = 4 * cs.p_sz;
    for (int p : fluid) {
      if (phase[p] != 2) continue;
      const double px = x[3 * p], py = x[3 * p + 1], pz = D == 3 ? x[3 * p + 2] : 0.0;
      if (py < a && pz < a) {
        if (px > dw) dw = px;
        if (px < jet) jet = px;
      } else if (py > b || pz > b) {
        if (px < ups) ups = px;
      }
      mass.add(rho[p] * vol[p]);
    }
    out[0] = dw; out[1] = jet; out[2] = ups; out[3] = mass.value(); out[4] = (double)fluid.size();
  }

  /* ------------------------------------------------------------------ */
  /* exchange                                                           */
  /* ------------------------------------------------------------------ */
  int64_t num_particles() override { return (int64_t)fluid.size(); }

  int upload_particles(const pgdg_particles* pp) override {
    for (int p : fluid) pfree(p);
    fluid.clear();
    freel.clear();
    x.clear(); x0.clear(); v.clear(); tv.clear(); a.clear(); rhov.clear();
    vol.clear(); vol0.clear(); mass.clear(); h.clear(); P.clear(); rho.clear(); E.clear(); c.clear();
    sl.clear(); phase.clear(); mark_in.clear(); mrg.clear(); mrg_mark.clear(); copy.clear(); in_ele.clear();
    seq.clear(); nbr.clear();
    uint64_t mx = 0;
    for (int64_t i = 0; i < pp->n; i++) {
      int s = pmalloc();
      for (int d = 0; d < 3; d++) {
        x[3 * s + d] = pp->coord[3 * i + d];
        v[3 * s + d] = pp->v ? pp->v[3 * i + d] : 0.0;
        tv[3 * s + d] = pp->tv ? pp->tv[3 * i + d] : 0.0;
        rhov[3 * s + d] = pp->rhov[3 * i + d];
      }
      vol[s] = pp->vol[i]; mass[s] = pp->mass[i]; h[s] = pp->h[i]; P[s] = pp->P[i];
      rho[s] = pp->rho[i]; E[s] = pp->E[i]; c[s] = pp->c[i];
      for (int t = 0; t < NS; t++) sl[NS * s + t] = pp->slope ? pp->slope[NS * i + t] : 0.0;
      phase[s] = pp->phase[i];
      mark_in[s] = pp->mark_in ? pp->mark_in[i] : 0;
      seq[s] = pp->seq ? pp->seq[i] : (uint64_t)i;
      if (seq[s] + 1 > mx) mx = seq[s] + 1;
      fluid.push_back(s);
    }
    seq_next = mx;
    return PGDG_OK;
  }

  int download_particles(pgdg_particles* pp) override {
    int64_t n = (int64_t)fluid.size();
    if (pp->n < n) { pp->n = n; return PGDG_EINVAL; }
    for (int64_t i = 0; i < n; i++) {
      int s = fluid[i];
      for (int d = 0; d < 3; d++) {
        if (pp->coord) pp->coord[3 * i + d] = x[3 * s + d];
        if (pp->v) pp->v[3 * i + d] = v[3 * s + d];
        if (pp->tv) pp->tv[3 * i + d] = tv[3 * s + d];
        if (pp->rhov) pp->rhov[3 * i + d] = rhov[3 * s + d];
      }
      if (pp->vol) pp->vol[i] = vol[s];
      if (pp->mass) pp->mass[i] = mass[s];
      if (pp->h) pp->h[i] = h[s];
      if (pp->P) pp->P[i] = P[s];
      if (pp->rho) pp->rho[i] = rho[s];
      if (pp->E) pp->E[i] = E[s];
      if (pp->c) pp->c[i] = c[s];
      if (pp->slope) for (int t = 0; t < NS; t++) pp->slope[NS * i + t] = sl[NS * s + t];
      if (pp->phase) pp->phase[i] = phase[s];
      if (pp->mark_in) pp->mark_in[i] = mark_in[s];
      if (pp->seq) pp->seq[i] = seq[s];
    }
    pp->n = n;
    return PGDG_OK;
  }

  int upload_cells(const pgdg_cells* cc_) override {
    if (cc_->n != ncell) return PGDG_EINVAL;
    for (int64_t ci = 0; ci < ncell; ci++) {
      for (int s = 0; s < F; s++) {
        int64_t q = ci * F + s;
        crho[q] = cc_->rho[q];
        for (int d = 0; d < 3; d++) crhov[q * 3 + d] = cc_->rhov[q * 3 + d];
        cE[q] = cc_->E[q]; cc[q] = cc_->c[q]; cac[q] = cc_->ac ? cc_->ac[q] : 0.0;
        calph[q] = cc_->alph[q];
        for (int t = 0; t < U * B; t++) ccoef[q * U * B + t] = cc_->coef[q * U * B + t];
        cph[q] = cc_->ph_state[q];
        cphb[q] = cc_->ph_state_b[q];
        if (cc_->lim_u) for (int u = 0; u < U; u++) clim[q * U + u] = cc_->lim_u[q * U + u];
        if (cc_->dcoef) for (int t = 0; t < U * B; t++) cdcoef[q * U * B + t] = cc_->dcoef[q * U * B + t];
      }
      for (int d = 0; d < 3; d++) cv[3 * ci + d] = cc_->v[3 * ci + d];
      cP[ci] = cc_->P[ci];
      if (cc_->g_v) for (int t = 0; t < D * D; t++) cgv[ci * D * D + t] = cc_->g_v[ci * D * D + t];
      if (cc_->used) cused[ci] = cc_->used[ci];
    }
    used_list.clear();
    for (int64_t ci = 0; ci < ncell; ci++)
      if (cused[ci]) used_list.push_back(ci);
    return PGDG_OK;
  }

  int download_cells(pgdg_cells* co) override {
    if (co->n != ncell) return PGDG_EINVAL;
    for (int64_t ci = 0; ci < ncell; ci++) {
      for (int s = 0; s < F; s++) {
        int64_t q = ci * F + s;
        if (co->rho) co->rho[q] = crho[q];
        if (co->rhov) for (int d = 0; d < 3; d++) co->rhov[q * 3 + d] = crhov[q * 3 + d];
        if (co->E) co->E[q] = cE[q];
        if (co->c) co->c[q] = cc[q];
        if (co->ac) co->ac[q] = cac[q];
        if (co->alph) co->alph[q] = calph[q];
        if (co->coef) for (int t = 0; t < U * B; t++) co->coef[q * U * B + t] = ccoef[q * U * B + t];
        if (co->dcoef) for (int t = 0; t < U * B; t++) co->dcoef[q * U * B + t] = cdcoef[q * U * B + t];
        if (co->ph_state) co->ph_state[q] = cph[q];
        if (co->ph_state_b) co->ph_state_b[q] = cphb[q];
        if (co->lim_u) for (int u = 0; u < U; u++) co->lim_u[q * U + u] = clim[q * U + u];
      }
      if (co->v) for (int d = 0; d < 3; d++) co->v[3 * ci + d] = cv[3 * ci + d];
      if (co->P) co->P[ci] = cP[ci];
      if (co->used) co->used[ci] = cused[ci];
      if (co->g_v) for (int t = 0; t < D * D; t++) co->g_v[ci * D * D + t] = cgv[ci * D * D + t];
    }
    return PGDG_OK;
  }

  std::vector<int64_t> slot_to_index() const {
    std::vector<int64_t> m(vol.size(), -1);
    for (size_t i = 0; i < fluid.size(); i++) m[fluid[i]] = (int64_t)i;
    return m;
  }
  int64_t encode(int r, const std::vector<int64_t>& m) const {
    if (is_bnd(r)) return -2 - bidx(r);
    int64_t ix = m[r];
    return ix >= 0 ? ix : -1;
  }

  int upload_lists(const int64_t* off, const int64_t* ent) override {
    for (size_t i = 0; i < fluid.size(); i++) {
      auto& L = nbr[fluid[i]];
      L.clear();
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        int64_t v_ = ent[e];
        if (v_ >= 0) L.push_back(fluid[v_]);
        else if (v_ <= -2) L.push_back(bref(-v_ - 2));
        /* -1 (dead) entries cannot be recreated and never match; dropped */
      }
    }
    return PGDG_OK;
  }
  int download_lists(int64_t* off, int64_t* ent, int64_t cap, int64_t* total) override {
    auto m = slot_to_index();
    int64_t t = 0;
    for (size_t i = 0; i < fluid.size(); i++) {
      if (off) off[i] = t;
      for (int r : nbr[fluid[i]]) {
        if (ent && t < cap) ent[t] = encode(r, m);
        t++;
      }
    }
    if (off) off[fluid.size()] = t;
    *total = t;
    return (ent && t > cap) ? PGDG_EOVERFLOW : PGDG_OK;
  }
  int download_cell_lists(int64_t* off, int64_t* ent, int64_t cap, int64_t* total) override {
    auto m = slot_to_index();
    int64_t t = 0;
    for (int64_t ci = 0; ci < ncell; ci++) {
      if (off) off[ci] = t;
      for (int r : clist[ci]) {
        if (ent && t < cap) ent[t] = encode(r, m);
        t++;
      }
    }
    if (off) off[ncell] = t;
    *total = t;
    return (ent && t > cap) ? PGDG_EOVERFLOW : PGDG_OK;
  }
};

}  // namespace

/* ---------------------------------------------------------------------- */
extern "C" {

int po_create(const pgdg_case* cs, po_ctx** out) {
  if (!cs || !out) return PGDG_EINVAL;
  if (cs->nfld != PO_NFLD) return PGDG_EINVAL; /* one material count per build */
  if (cs->dim == 2) *out = new OracleT<2>(cs);
  else if (cs->dim == 3) *out = new OracleT<3>(cs);
  else return PGDG_EINVAL;
  return PGDG_OK;
}
int po_destroy(po_ctx* ctx) { delete ctx; return PGDG_OK; }
int po_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
  return PGDG_OK;
}
int po_upload_particles(po_ctx* ctx, const pgdg_particles* p) { return ctx->upload_particles(p); }
int po_download_particles(po_ctx* ctx, pgdg_particles* p) { return ctx->download_particles(p); }
int po_num_particles(po_ctx* ctx, int64_t* n) { *n = ctx->num_particles(); return PGDG_OK; }
int po_upload_cells(po_ctx* ctx, const pgdg_cells* c) { return ctx->upload_cells(c); }
int po_download_cells(po_ctx* ctx, pgdg_cells* c) { return ctx->download_cells(c); }
int po_upload_lists(po_ctx* ctx, const int64_t* off, const int64_t* ent) { return ctx->upload_lists(off, ent); }
int po_download_lists(po_ctx* ctx, int64_t* off, int64_t* ent, int64_t cap, int64_t* total) {
  return ctx->download_lists(off, ent, cap, total);
}
int po_download_cell_lists(po_ctx* ctx, int64_t* off, int64_t* ent, int64_t cap, int64_t* total) {
  return ctx->download_cell_lists(off, ent, cap, total);
}
int po_set_dt(po_ctx* ctx, double dt) { ctx->dt = dt; return PGDG_OK; }
int po_set_iterate(po_ctx* ctx, int64_t n) { ctx->iterate = n; return PGDG_OK; }
int po_set_max_v(po_ctx* ctx, double mv) { ctx->max_v = mv; return PGDG_OK; }
int po_get_stats(po_ctx* ctx, pgdg_stats* st) {
  *st = ctx->st;
  st->n_particles = ctx->num_particles();
  st->iterate_num = ctx->iterate;
  st->dt = ctx->dt;
  st->max_v = ctx->max_v;
  return PGDG_OK;
}
int po_set_timestep(po_ctx* ctx, double* dt, double* mv) { return ctx->set_timestep(dt, mv); }
int po_output_point(po_ctx* ctx, double* out5) {
  ctx->output_point(out5);
  return PGDG_OK;
}
int po_output_plt(po_ctx* ctx, const char* particle_path, const char* cell_path) {
  return ctx->output_plt(particle_path, cell_path);
}
int po_used_state_update(po_ctx* ctx) { ctx->used_state_update(); return PGDG_OK; }
int po_bin_particles(po_ctx* ctx) { ctx->bin_particles(); return PGDG_OK; }
int po_split_particle_fast(po_ctx* ctx) { ctx->split_particle_fast(); return PGDG_OK; }
int po_merge_particle_fast(po_ctx* ctx) { ctx->merge_particle_fast(); return PGDG_OK; }
int po_refresh_membership(po_ctx* ctx) { ctx->refresh_membership(); return PGDG_OK; }
int po_refresh_neighbors(po_ctx* ctx) { ctx->refresh_neighbors(); return PGDG_OK; }
int po_mls_p2g(po_ctx* ctx) { ctx->mls_p2g(); return PGDG_OK; }
int po_calculate_limiter(po_ctx* ctx) { ctx->calculate_limiter(); return PGDG_OK; }
int po_grid_acceleration(po_ctx* ctx) { ctx->grid_acceleration(); return PGDG_OK; }
int po_update_grid(po_ctx* ctx, int md) { ctx->update_grid(md); return PGDG_OK; }
int po_update_particle(po_ctx* ctx, int md) { ctx->update_particle(md); return PGDG_OK; }
int po_run_step(po_ctx* ctx, int64_t n) { ctx->run_step(n); return PGDG_OK; }
int po_advance(po_ctx* ctx, int nsteps) {
  for (int s = 0; s < nsteps; s++) {
    ctx->set_timestep(nullptr, nullptr);
    ctx->iterate++;
    ctx->run_step(ctx->iterate);
  }
  return PGDG_OK;
}
int po_totals(po_ctx* ctx, double* out) { ctx->totals(out); return PGDG_OK; }

int po_mgfm_batched(const double* in6, const int8_t* mat2, const double* gam, const double* pinf,
                    int variant, const double* seed, double* out3, int32_t* iters, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    const double* q = in6 + 6 * i;
    int s = mat2[2 * i], s1 = mat2[2 * i + 1];
    int it = 0;
    mgfm(q[0], q[1], q[2], q[3], q[4], q[5], gam[s], pinf[s], gam[s1], pinf[s1], variant,
         seed ? seed[i] : -1.0, out3 + 3 * i, &it);
    if (iters) iters[i] = it;
  }
  return PGDG_OK;
}
double po_root_d(double x, int d) { return root_d(x, d); }

}  // extern "C"
