/*
 * capi.cu -- the C ABI of libpgdg_gpu.so (include/pgdg.h) and the host driver.
 *
 * One context owns all device buffers of one case on one GPU and one CUDA
 * stream.  The host driver restates the reference's call order:
 * Solver::MPM_Solver (solver.cpp:30-64) -> MPM::Set_timestep -> MPM_run_simulation
 * (mpm_ini.cpp:682-766).  No host synchronisation happens inside a step; dt,
 * max_v and the particle counters live on the device.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pgdg.h"
#include "pgdg_dev.cuh"
#include "plt_writer.h"

using namespace pgdg;

struct pgdg_ctx {
  virtual ~pgdg_ctx() {}
  std::string err;
  pgdg_case cs;
  int precision = PGDG_PREC_FP64;
  void* net = nullptr;   /* attached seed surrogate (pgdg_mlp) */
  int iface_queue = 0;   /* 1: interface problems solved as one batch */
  int pst_var = -1;      /* shifting-kernel variant (-1: tune at the next call) */
  int p2g_skip = 1;      /* 1: P2G skips out-of-reach neighbour cells while the bins are fresh */
  int64_t iface_cap_fixed = -1; /* >= 0: the interface queue's capacity, never grown */
  virtual int set_iface_cap(int64_t cap) = 0;
  virtual int iface_download(double*, int8_t*, int64_t, int64_t*) = 0;
  /* captured step graphs (advance): dropped when what they bake in changes */
  virtual void invalidate_graphs() = 0;
  virtual void enable_graphs(bool on) = 0;
  int64_t iterate = 0;
  cudaStream_t st = nullptr;
  virtual int upload_particles(const pgdg_particles*) = 0;
  virtual int output_point(double* out5) = 0;
  virtual int output_plt(const char* particle_path, const char* cell_path, int async) = 0;
  virtual int output_wait() = 0;
  virtual int case_build(int id, uint64_t seed) = 0;
  virtual int download_particles(pgdg_particles*) = 0;
  virtual int num_particles(int64_t*) = 0;
  virtual int upload_cells(const pgdg_cells*) = 0;
  virtual int download_cells(pgdg_cells*) = 0;
  virtual int upload_lists(const int64_t*, const int64_t*) = 0;
  virtual int download_lists(int64_t*, int64_t*, int32_t*, int64_t, int64_t*) = 0;
  virtual int download_cell_lists(int64_t*, int64_t*, int64_t, int64_t*) = 0;
  virtual int set_dt(double) = 0;
  virtual int set_max_v(double) = 0;
  virtual int stats(pgdg_stats*) = 0;
  virtual int capacity(int64_t*) = 0;
  virtual int set_timestep(double*, double*) = 0;
  virtual int used_state() = 0;
  virtual int bin() = 0;
  virtual int split() = 0;
  virtual int merge(bool chained = false) = 0;
  virtual int refresh_membership() = 0;
  virtual int refresh_neighbors() = 0;
  virtual int p2g() = 0;
  virtual int limiter() = 0;
  virtual int grid_acc() = 0;
  virtual int update_grid(int) = 0;
  virtual int update_particle(int) = 0;
  virtual int run_step(int64_t) = 0;
  virtual int prepare_step() = 0; /* host-side upkeep between steps */
  virtual int advance(int) = 0;
  virtual int totals(double*) = 0;
  virtual int check() = 0;
  /* per-method device timing with CUDA events on the context stream */
  bool prof = false;
  int64_t launches = 0;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_next = 0;
  std::vector<std::pair<std::string, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<std::string> knames;
  std::vector<double> kms;
  std::vector<int64_t> kcnt;
  cudaEvent_t ev_get() {
    if (ev_next >= ev_pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_next++];
  }
  void flush_prof() {
    if (pending.empty()) return;
    cudaStreamSynchronize(st);
    for (auto& p : pending) {
      float ms = 0;
      cudaEventElapsedTime(&ms, p.second.first, p.second.second);
      size_t k = 0;
      for (; k < knames.size(); k++)
        if (knames[k] == p.first) break;
      if (k == knames.size()) {
        knames.push_back(p.first);
        kms.push_back(0);
        kcnt.push_back(0);
      }
      kms[k] += ms;
      kcnt[k] += 1;
    }
    pending.clear();
    ev_next = 0;
  }
  template <typename Fn>
  void timed(const char* name, int nlaunch, Fn fn) {
    launches += nlaunch;
    if (!prof) {
      fn();
      return;
    }
    if (ev_next + 2 > 4096) flush_prof();
    cudaEvent_t a = ev_get(), b = ev_get();
    cudaEventRecord(a, st);
    fn();
    cudaEventRecord(b, st);
    pending.push_back({name, {a, b}});
  }
};

namespace {

#define CK(x)                                                   \
  do {                                                          \
    cudaError_t e_ = (x);                                       \
    if (e_ != cudaSuccess) {                                    \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);    \
      return PGDG_ECUDA;                                        \
    }                                                           \
  } while (0)

template <typename T>
static cudaError_t dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e == cudaSuccess) e = cudaMemset(*p, 0, n * sizeof(T));
  return e;
}

template <int D, typename R, bool EX>
struct Ctx : pgdg_ctx {
  static constexpr int U = D + 2, B = D + 1, NS = U * D;
  CaseK K{};
  DevPtrs<R> P{};
  std::vector<void*> allocs;
  int x0b = 0;          /* step-start coordinate buffer (md 1) */
  double* d_tot = nullptr;
  IfaceQ Q{};
  PartScratch part;   /* root partition of the interface batch */
  unsigned char* pst_scratch = nullptr; /* per-stage row sort of the shifting kernel */
  /* every particle lies in its bucket's cell (true from binning until the
   * particles move); P2G then skips neighbour cells beyond its cut radius */
  bool fresh_bins = false;
  bool g2p_partial = false; /* see run_step */
  double *d_gam = nullptr, *d_pinf = nullptr;
  unsigned long long* d_ncell = nullptr;
  int dev_id = 0;
  /* the last complete stage's search coordinates and lengths (the flag-2
   * lists the snapshot writer counts); unset after the particle set changes */
  int nb_xs = 0, nb_hs = 0;
  bool nb_set = false;
  /* snapshot writers: device snapshot, copy stream, pinned chunks, worker */
  double* d_odv = nullptr;
  int32_t* d_oiv = nullptr;
  double* d_odc = nullptr;
  int64_t ocap = 0;
  cudaStream_t ost = nullptr;
  cudaEvent_t oev = nullptr, ochev[2] = {nullptr, nullptr};
  unsigned char* h_och[2] = {nullptr, nullptr};
  static constexpr size_t OCHUNK = (size_t)32 << 20;
  std::thread oth;
  bool orunning = false;
  int orc = PGDG_OK;
  std::string omsg;

  template <typename T>
  cudaError_t A(T** p, size_t n) {
    cudaError_t e = dalloc(p, n);
    if (e == cudaSuccess) allocs.push_back(*p);
    return e;
  }

  ~Ctx() override {
    output_wait();
    if (d_odv) cudaFree(d_odv);
    if (d_oiv) cudaFree(d_oiv);
    if (d_odc) cudaFree(d_odc);
    for (int k = 0; k < 2; k++) {
      if (h_och[k]) cudaFreeHost(h_och[k]);
      if (ochev[k]) cudaEventDestroy(ochev[k]);
    }
    if (oev) cudaEventDestroy(oev);
    if (ost) cudaStreamDestroy(ost);
    if (st) cudaStreamSynchronize(st);
    drop_graphs();
    for (auto e : ev_pool) cudaEventDestroy(e);
    for (void* p : allocs) cudaFree(p);
    part.release();
    if (st) cudaStreamDestroy(st);
  }

  int init(const pgdg_case* c, int prec, int64_t cap) {
    cs = *c;
    precision = prec;
    CK(cudaGetDevice(&dev_id));
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    K.dim = D;
    for (int d = 0; d < 3; d++) K.N[d] = (d < D) ? cs.ncell[d] : 1;
    for (int s = 0; s < 6; s++) K.bc[s] = cs.bc[s];
    K.mgfm_variant = cs.mgfm_variant;
    K.rad2 = (int)std::ceil(CELL_RATIO / (cs.p_g / cs.p_sz));
    K.maxpc = (D == 3) ? 64 : 32;
    K.ncell = (int64_t)K.N[0] * K.N[1] * K.N[2];
    if (cap <= 0) cap = pgdg_case_num_particles(&cs) * 3 / 2 + 4096;
    K.cap = cap;
    K.arena_cap = cap * 32;
    for (int d = 0; d < 3; d++) {
      K.bl[d] = cs.box_l[d];
      K.br[d] = cs.box_r[d];
      K.ps[d] = cs.p_size[d];
    }
    K.p_g = cs.p_g;
    K.p_sz = cs.p_sz;
    for (int s = 0; s < F; s++) {
      K.gamma[s] = cs.gamma[s];
      K.pinf[s] = cs.pinf[s];
      K.ini_rho[s] = cs.ini_rho[s];
      const bool shift = sizeof(R) == 4 && cs.pinf[s] != 0.0;
      K.eshift[s] = shift ? cs.gamma[s] * cs.pinf[s] / (cs.gamma[s] - 1.0) : 0.0;
      K.pinf_eos[s] = shift ? 0.0 : cs.pinf[s];
    }
    K.inlet_rho = cs.inlet_rho;
    for (int d = 0; d < 3; d++) K.inlet_u[d] = cs.inlet_u[d];
    K.inlet_p = cs.inlet_p;
    K.cfl = cs.cfl;
    K.vol_max = powern_d(cs.p_sz, D) * 1.6;
    K.vol_min = powern_d(cs.p_sz, D) * 2. / 3.;
    K.dss0 = root_d(K.vol_min, D);
    for (int i = 0; i < 8; i++)
      for (int d = 0; d < 3; d++) K.probe[i][d] = cs.probe[i][d];
    K.bvol = powern_d(cs.p_sz, D - 1);
    K.brho = cs.ini_rho[0];

    /* particles */
    const size_t n = (size_t)cap;
    for (int b = 0; b < 3; b++) CK(A(&P.X[b], D * n));
    for (int b = 0; b < 2; b++) CK(A(&P.H[b], n));
    CK(A(&P.vol, n)); CK(A(&P.vol0, n)); CK(A(&P.mass, n)); CK(A(&P.rho, n)); CK(A(&P.E, n));
    CK(A(&P.c, n)); CK(A(&P.P, n));
    CK(A(&P.rhov, D * n)); CK(A(&P.v, D * n)); CK(A(&P.tv, D * n));
    CK(A(&P.sl, NS * n));
    CK(A(&P.rec, 4 * n)); CK(A(&P.rec2, 2 * n));
    CK(A(&P.phase, n)); CK(A(&P.mark_in, n)); CK(A(&P.seq, n));
    CK(A(&P.lcell, n)); CK(A(&P.lkey, n)); CK(A(&P.list_len, n)); CK(A(&P.list_off, n));
    CK(A(&P.target, n)); CK(A(&P.aff, n)); CK(A(&P.mflag, n)); CK(A(&P.evcode, n));
    CK(A(&P.scan, n + 1));
    CK(A(&P.scan_blk, (n + 2047) / 2048 + 2));
    CK(A(&P.arena, (size_t)K.arena_cap));
    /* cells */
    const size_t nc = (size_t)K.ncell;
    CK(A(&P.crho, F * nc)); CK(A(&P.crhov, F * D * nc)); CK(A(&P.cE, F * nc)); CK(A(&P.cc, F * nc));
    CK(A(&P.cac, F * nc)); CK(A(&P.calph, F * nc));
    CK(A(&P.ccoef, F * U * B * nc)); CK(A(&P.ccoef0, F * U * B * nc)); CK(A(&P.cdcoef, F * U * B * nc));
    CK(A(&P.clim, F * U * nc)); CK(A(&P.cgv, D * D * nc)); CK(A(&P.cv, D * nc)); CK(A(&P.cP, nc));
    CK(A(&P.cph, F * nc)); CK(A(&P.cphb, F * nc)); CK(A(&P.cused, nc)); CK(A(&P.cnew, nc));
    CK(A(&P.bucket, nc * K.maxpc)); CK(A(&P.bcnt, nc)); CK(A(&P.cflag, nc));
    CK(A(&P.dirty_q, nc)); CK(A(&P.flag_q, nc));
    P.qcap = (int64_t)nc;
    if (const size_t rsb = Launch<D, R, EX>::pst_scratch_bytes(K)) CK(A(&pst_scratch, rsb));
    CK(A(&P.cnt, 1));
    CK(A(&d_tot, Launch<D, R, EX>::totals_scratch()));
    /* interface queue: at most 2 phases x 2D faces x 4 points x 1 other phase per cell;
     * sized for a few per cent of the cells, grown on demand */
    Q.cap = std::max<int64_t>(1 << 16, K.ncell / 8);
    CK(A(&Q.in6, 6 * (size_t)Q.cap));
    CK(A(&Q.mat, 2 * (size_t)Q.cap));
    CK(A(&Q.out3, 3 * (size_t)Q.cap));
    CK(A(&Q.off, nc + 1));
    CK(A(&Q.blk, (nc + 2047) / 2048 + 2));
    CK(A(&Q.tot, 2));
    CK(A(&d_ncell, 1));
    {
      unsigned long long v = (unsigned long long)K.ncell;
      CK(cudaMemcpy(d_ncell, &v, sizeof(v), cudaMemcpyHostToDevice));
    }
    Q.d_ncell = d_ncell;
    CK(A(&d_gam, F));
    CK(A(&d_pinf, F));
    CK(cudaMemcpy(d_gam, K.gamma, sizeof(double) * F, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_pinf, K.pinf, sizeof(double) * F, cudaMemcpyHostToDevice));
    P.xb = 0;
    P.hb = 0;
    int rc = init_boundary();
    if (rc) return rc;
    return init_cells_default();
  }

  /* boundary particles on the boundary nodes (mpm_ini.cpp:555-620) */
  int init_boundary() {
    std::vector<double> bx, bn;
    const int S2 = (D == 3) ? K.N[2] : 0;
    for (int sx = 0; sx <= K.N[0]; ++sx)
      for (int sy = 0; sy <= K.N[1]; ++sy)
        for (int sz = 0; sz <= S2; ++sz) {
          bool fg = (sx == 0 || sx == K.N[0] || sy == 0 || sy == K.N[1]);
          if (D == 3) fg = fg || sz == 0 || sz == K.N[2];
          if (!fg) continue;
          double p[3] = {K.bl[0] + K.ps[0] * (sx + 0.), K.bl[1] + K.ps[1] * (sy + 0.), 0.0};
          if (D == 3) p[2] = K.bl[2] + K.ps[2] * (sz + 0.);
          double nn[3] = {0, 0, 0};
          if (sx == 0) nn[0] = -1;
          else if (sx == K.N[0]) nn[0] = 1;
          else if (sy == 0) nn[1] = -1;
          else if (sy == K.N[1]) nn[1] = 1;
          else if (D == 3 && sz == 0) nn[2] = -1;
          else if (D == 3 && sz == K.N[2]) nn[2] = 1;
          for (int d = 0; d < 3; d++) {
            bx.push_back(p[d]);
            bn.push_back(nn[d]);
          }
        }
    int64_t nb = (int64_t)bx.size() / 3;
    K.nbnd = nb;
    std::vector<R> hx(D * nb), hn(D * nb);
    std::vector<int32_t> cellof(nb);
    for (int64_t b = 0; b < nb; b++) {
      for (int d = 0; d < D; d++) {
        hx[d * nb + b] = (R)bx[3 * b + d];
        hn[d * nb + b] = (R)bn[3 * b + d];
      }
      int pos[3] = {0, 0, 0};
      for (int d = 0; d < D; d++) {
        double q = std::floor((bx[3 * b + d] - K.bl[d]) / K.ps[d]);
        pos[d] = (!(q >= 0)) ? 0 : (q >= K.N[d] - 1 ? K.N[d] - 1 : (int)q);
      }
      cellof[b] = (int32_t)(((int64_t)pos[0] * K.N[1] + pos[1]) * K.N[2] + pos[2]);
    }
    std::vector<int32_t> off(K.ncell + 1, 0), ent(nb);
    for (int64_t b = 0; b < nb; b++) off[cellof[b] + 1]++;
    for (int64_t c = 0; c < K.ncell; c++) off[c + 1] += off[c];
    std::vector<int32_t> fill(off.begin(), off.end() - 1);
    for (int64_t b = 0; b < nb; b++) ent[fill[cellof[b]]++] = (int32_t)b;
    CK(A(&P.bx, D * nb));
    CK(A(&P.bn, D * nb));
    CK(A(&P.boff, K.ncell + 1));
    CK(A(&P.bent, nb));
    CK(cudaMemcpy(P.bx, hx.data(), sizeof(R) * D * nb, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(P.bn, hn.data(), sizeof(R) * D * nb, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(P.boff, off.data(), sizeof(int32_t) * (K.ncell + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(P.bent, ent.data(), sizeof(int32_t) * std::max<int64_t>(nb, 1), cudaMemcpyHostToDevice));
    return PGDG_OK;
  }

  int init_cells_default() {
    /* cells start as MPM::Initialize_case leaves them (mpm_ini.cpp:325-338) */
    std::vector<double> rho(F * K.ncell), c(F * K.ncell);
    pgdg_cells v{};
    v.n = K.ncell;
    std::vector<double> z3(F * 3 * K.ncell, 0.0), zf(F * K.ncell, 0.0), zc(F * U * B * K.ncell, 0.0),
        zv(3 * K.ncell, 0.0), zp(K.ncell, 0.0);
    std::vector<int32_t> ph(F * K.ncell), phb(F * K.ncell), used(K.ncell);
    std::vector<double> lim(F * U * K.ncell, 1.0);
    v.rho = rho.data(); v.rhov = z3.data(); v.E = zf.data(); v.c = c.data(); v.ac = nullptr;
    v.alph = zf.data(); v.coef = zc.data(); v.v = zv.data(); v.P = zp.data();
    v.ph_state = ph.data(); v.ph_state_b = phb.data(); v.used = used.data(); v.lim_u = lim.data();
    int rc = pgdg_case_cells(&cs, &v);
    if (rc) return rc;
    rc = upload_cells(&v);
    if (rc) return rc;
    /* counters */
    DevCounters h{};
    h.dt = 0;
    h.max_v = 1e-7;
    CK(cudaMemcpy(P.cnt, &h, sizeof(h), cudaMemcpyHostToDevice));
    return PGDG_OK;
  }

  DevCounters counters() {
    DevCounters h{};
    cudaStreamSynchronize(st);
    cudaMemcpy(&h, P.cnt, sizeof(h), cudaMemcpyDeviceToHost);
    return h;
  }

  int check() override {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      err = std::string("kernel: ") + cudaGetErrorString(e);
      return PGDG_ECUDA;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      err = std::string("launch: ") + cudaGetErrorString(e);
      return PGDG_ECUDA;
    }
    DevCounters h = counters();
    if (h.err) {
      char b[160];
      snprintf(b, sizeof(b),
               "device status 0x%x (1 bucket, 2 list arena, 4 capacity, 8 missing list, 16 cell queue, "
               "64 no finite time step)",
               h.err);
      err = b;
      if (h.err & ERR_DT) return PGDG_ENONFINITE;
      return (h.err & ERR_NOLIST) ? PGDG_ESTATE : PGDG_EOVERFLOW;
    }
    return PGDG_OK;
  }

  /* ---------------- exchange ---------------- */
  /* staging buffer of the host exchange (raw host chunks; allocated on first use) */
  XferStage stage{nullptr, 0};
  int64_t* d_alive = nullptr;
  int ensure_stage() {
    if (stage.buf) return PGDG_OK;
    stage.bytes = (size_t)256 << 20;
    CK(cudaMalloc(&stage.buf, stage.bytes));
    allocs.push_back(stage.buf);
    return PGDG_OK;
  }
  /* live slots in canonical order into d_alive; returns their number */
  int alive(int64_t* n) {
    if (!d_alive) CK(A(&d_alive, (size_t)K.cap));
    alive_index(P.phase, P.scan, P.scan_blk, &P.cnt->n_slots, K.cap, d_alive, st);
    unsigned long long tot = 0;
    CK(cudaMemcpyAsync(&tot, P.scan_blk + scan_nblk_host(K.cap), sizeof(tot), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *n = (int64_t)tot;
    return PGDG_OK;
  }
  static int scan_nblk_host(int64_t cap) { return (int)((cap + 2047) / 2048); }

  /* the case's particles and cells built on the device, in place of
   * pgdg_case_particles / pgdg_case_cells and the two uploads */
  int case_build(int id, uint64_t seed) override {
    drop_graphs();
    fresh_bins = false;
    nb_set = false;
    const int64_t n = pgdg_case_num_particles(&cs);
    if (n > K.cap) {
      err = "particle count exceeds capacity";
      return PGDG_EINVAL;
    }
    CK(cudaStreamSynchronize(st));
    P.xb = 0;
    P.hb = 0;
    x0b = 0;
    CK(cudaMemsetAsync(P.phase, 0, (size_t)K.cap, st));
    const int rc = pgdg::case_build<D, R>(K, P, cs, id, seed, n, st);
    if (rc) {
      err = "case_build: the case does not match the workload";
      return rc;
    }
    CK(cudaStreamSynchronize(st));
    DevCounters hc = counters();
    hc.n_slots = n;
    hc.n_live = n;
    hc.seq_next = (unsigned long long)n;
    hc.arena_used = 0;
    hc.err = 0;
    hc.n_dirty = hc.n_flagged = 0;
    CK(cudaMemcpy(P.cnt, &hc, sizeof(hc), cudaMemcpyHostToDevice));
    return PGDG_OK;
  }

  /* ---------------- exchange ---------------- */
  int upload_particles(const pgdg_particles* pp) override {
    drop_graphs();
    fresh_bins = false;
    nb_set = false;
    int64_t n = pp->n;
    if (n > K.cap) {
      err = "particle count exceeds capacity";
      return PGDG_EINVAL;
    }
    if (!pp->coord || !pp->rhov || !pp->vol || !pp->mass || !pp->h || !pp->P || !pp->rho || !pp->E || !pp->c ||
        !pp->phase) {
      err = "upload_particles: a required array is NULL";
      return PGDG_EINVAL;
    }
    int rc = ensure_stage();
    if (rc) return rc;
    CK(cudaStreamSynchronize(st));
    P.xb = 0;
    P.hb = 0;
    x0b = 0;
    const int64_t cap = K.cap;
    const XferMap vec = xmap(D), one = xmap(1), sl = xmap(NS);
    /* phase first: the energy shift of a particle follows its phase */
    CK(cudaMemsetAsync(P.phase, 0, (size_t)cap, st));
    CK(xfer_h2d_i8(pp->phase, 1, n, one, P.phase, cap, stage, st));
    CK(xfer_h2d<R>(pp->coord, 3, n, vec, P.X[0], cap, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(pp->rhov, 3, n, vec, P.rhov, cap, nullptr, nullptr, stage, st));
    for (int d = 0; d < D; d++) {
      if (!pp->v) CK(cudaMemsetAsync(P.v + (size_t)d * cap, 0, sizeof(R) * n, st));
      if (!pp->tv) CK(cudaMemsetAsync(P.tv + (size_t)d * cap, 0, sizeof(R) * n, st));
    }
    if (pp->v) CK(xfer_h2d<R>(pp->v, 3, n, vec, P.v, cap, nullptr, nullptr, stage, st));
    if (pp->tv) CK(xfer_h2d<R>(pp->tv, 3, n, vec, P.tv, cap, nullptr, nullptr, stage, st));
    if (pp->slope) CK(xfer_h2d<R>(pp->slope, NS, n, sl, P.sl, cap, nullptr, nullptr, stage, st));
    else
      for (int t = 0; t < NS; t++) CK(cudaMemsetAsync(P.sl + (size_t)t * cap, 0, sizeof(R) * n, st));
    CK(xfer_h2d<R>(pp->vol, 1, n, one, P.vol, cap, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(pp->mass, 1, n, one, P.mass, cap, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(pp->h, 1, n, one, P.H[0], cap, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(pp->P, 1, n, one, P.P, cap, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(pp->rho, 1, n, one, P.rho, cap, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(pp->E, 1, n, one, P.E, cap, P.phase, K.eshift, stage, st));
    CK(xfer_h2d<R>(pp->c, 1, n, one, P.c, cap, nullptr, nullptr, stage, st));
    if (pp->mark_in) CK(xfer_h2d_i8(pp->mark_in, 1, n, one, P.mark_in, cap, stage, st));
    else CK(cudaMemsetAsync(P.mark_in, 0, (size_t)n, st));
    uint64_t mx = (uint64_t)n;
    if (pp->seq) {
      CK(cudaMemcpyAsync(P.seq, pp->seq, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, st));
      mx = 0;
      for (int64_t i = 0; i < n; i++) mx = std::max<uint64_t>(mx, pp->seq[i] + 1);
    } else {
      iota_u64(P.seq, n, st);
    }
    CK(cudaMemsetAsync(P.list_len, 0, sizeof(int32_t) * n, st));
    CK(cudaMemsetAsync(P.list_off, 0, sizeof(int64_t) * n, st));
    CK(cudaStreamSynchronize(st));
    DevCounters hc = counters();
    hc.n_slots = n;
    hc.n_live = n;
    hc.seq_next = mx;
    hc.arena_used = 0;
    hc.err = 0;
    hc.n_dirty = hc.n_flagged = 0;
    CK(cudaMemcpy(P.cnt, &hc, sizeof(hc), cudaMemcpyHostToDevice));
    return PGDG_OK;
  }

  /* alive slots in canonical order (host copy, for the list exchange) */
  int alive_slots(std::vector<int64_t>& slots) {
    int64_t n = 0;
    int rc = alive(&n);
    if (rc) return rc;
    slots.resize(n);
    if (n) CK(cudaMemcpy(slots.data(), d_alive, sizeof(int64_t) * n, cudaMemcpyDeviceToHost));
    return PGDG_OK;
  }

  int num_particles(int64_t* n) override {
    DevCounters hc = counters();
    *n = (int64_t)hc.n_live;
    return PGDG_OK;
  }

  int download_particles(pgdg_particles* pp) override {
    int rc = ensure_stage();
    if (rc) return rc;
    int64_t n = 0;
    rc = alive(&n);
    if (rc) return rc;
    if (pp->n < n) {
      pp->n = n;
      err = "download capacity too small";
      return PGDG_EINVAL;
    }
    const int64_t cap = K.cap;
    const int64_t* ix = d_alive;
    const XferMap vec = xmap(D), one = xmap(1), sl = xmap(NS);
    if (pp->coord) CK(xfer_d2h<R>(P.X[P.xb], cap, ix, n, vec, pp->coord, 3, nullptr, nullptr, stage, st));
    if (pp->v) CK(xfer_d2h<R>(P.v, cap, ix, n, vec, pp->v, 3, nullptr, nullptr, stage, st));
    if (pp->tv) CK(xfer_d2h<R>(P.tv, cap, ix, n, vec, pp->tv, 3, nullptr, nullptr, stage, st));
    if (pp->rhov) CK(xfer_d2h<R>(P.rhov, cap, ix, n, vec, pp->rhov, 3, nullptr, nullptr, stage, st));
    if (pp->slope) CK(xfer_d2h<R>(P.sl, cap, ix, n, sl, pp->slope, NS, nullptr, nullptr, stage, st));
    if (pp->vol) CK(xfer_d2h<R>(P.vol, cap, ix, n, one, pp->vol, 1, nullptr, nullptr, stage, st));
    if (pp->mass) CK(xfer_d2h<R>(P.mass, cap, ix, n, one, pp->mass, 1, nullptr, nullptr, stage, st));
    if (pp->h) CK(xfer_d2h<R>(P.H[P.hb], cap, ix, n, one, pp->h, 1, nullptr, nullptr, stage, st));
    if (pp->P) CK(xfer_d2h<R>(P.P, cap, ix, n, one, pp->P, 1, nullptr, nullptr, stage, st));
    if (pp->rho) CK(xfer_d2h<R>(P.rho, cap, ix, n, one, pp->rho, 1, nullptr, nullptr, stage, st));
    if (pp->E) CK(xfer_d2h<R>(P.E, cap, ix, n, one, pp->E, 1, P.phase, K.eshift, stage, st));
    if (pp->c) CK(xfer_d2h<R>(P.c, cap, ix, n, one, pp->c, 1, nullptr, nullptr, stage, st));
    if (pp->phase) CK(xfer_d2h_i8(P.phase, cap, ix, n, one, pp->phase, 1, stage, st));
    if (pp->mark_in) CK(xfer_d2h_i8(P.mark_in, cap, ix, n, one, pp->mark_in, 1, stage, st));
    if (pp->seq) CK(xfer_d2h_u64(P.seq, ix, n, pp->seq, stage, st));
    pp->n = n;
    return PGDG_OK;
  }

  /* cell arrays: host element = cell, device component-major over ncell */
  int upload_cells(const pgdg_cells* cc) override {
    drop_graphs();
    if (cc->n != K.ncell) {
      err = "cell count mismatch";
      return PGDG_EINVAL;
    }
    if (!cc->rho || !cc->rhov || !cc->E || !cc->c || !cc->alph || !cc->coef || !cc->v || !cc->P || !cc->ph_state ||
        !cc->ph_state_b) {
      err = "upload_cells: a required array is NULL";
      return PGDG_EINVAL;
    }
    int rc = ensure_stage();
    if (rc) return rc;
    const int64_t nc = K.ncell;
    int hk[XMAP_MAX];
    double sh[XMAP_MAX];
    /* per phase scalars: host [ci][s] */
    const XferMap fs = xmap(F);
    for (int s = 0; s < F; s++) sh[s] = K.eshift[s];
    const XferMap fE = xmap(F, nullptr, sh);
    /* momentum: host [ci][s][3] -> device [(s D + d)][ci] */
    for (int s = 0; s < F; s++)
      for (int d = 0; d < D; d++) hk[s * D + d] = s * 3 + d;
    const XferMap fv = xmap(F * D, hk);
    /* coefficients: host [ci][s][u][b] -> device [(s U + u) B + b][ci], energy constant shifted */
    for (int t = 0; t < F * U * B; t++) sh[t] = (t % (U * B) == (U - 1) * B) ? K.eshift[t / (U * B)] : 0.0;
    const XferMap fc = xmap(F * U * B, nullptr, sh);
    const XferMap fd = xmap(F * U * B), fl = xmap(F * U), vec = xmap(D), gv = xmap(D * D), one = xmap(1);
    CK(cudaStreamSynchronize(st));
    CK(xfer_h2d<R>(cc->rho, F, nc, fs, P.crho, nc, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(cc->rhov, 3 * F, nc, fv, P.crhov, nc, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(cc->E, F, nc, fE, P.cE, nc, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(cc->c, F, nc, fs, P.cc, nc, nullptr, nullptr, stage, st));
    if (cc->ac) CK(xfer_h2d<R>(cc->ac, F, nc, fs, P.cac, nc, nullptr, nullptr, stage, st));
    else CK(cudaMemsetAsync(P.cac, 0, sizeof(R) * F * nc, st));
    CK(xfer_h2d<R>(cc->alph, F, nc, fs, P.calph, nc, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(cc->coef, F * U * B, nc, fc, P.ccoef, nc, nullptr, nullptr, stage, st));
    if (cc->dcoef) CK(xfer_h2d<R>(cc->dcoef, F * U * B, nc, fd, P.cdcoef, nc, nullptr, nullptr, stage, st));
    else CK(cudaMemsetAsync(P.cdcoef, 0, sizeof(R) * F * U * B * nc, st));
    if (cc->lim_u) CK(xfer_h2d<R>(cc->lim_u, F * U, nc, fl, P.clim, nc, nullptr, nullptr, stage, st));
    else fill_dev<R>(P.clim, (int64_t)F * U * nc, R(1), st);
    if (cc->g_v) CK(xfer_h2d<R>(cc->g_v, D * D, nc, gv, P.cgv, nc, nullptr, nullptr, stage, st));
    else CK(cudaMemsetAsync(P.cgv, 0, sizeof(R) * D * D * nc, st));
    CK(xfer_h2d<R>(cc->v, 3, nc, vec, P.cv, nc, nullptr, nullptr, stage, st));
    CK(xfer_h2d<R>(cc->P, 1, nc, one, P.cP, nc, nullptr, nullptr, stage, st));
    CK(xfer_h2d_i8(cc->ph_state, F, nc, fs, P.cph, nc, stage, st));
    CK(xfer_h2d_i8(cc->ph_state_b, F, nc, fs, P.cphb, nc, stage, st));
    if (cc->used) CK(xfer_h2d_i8(cc->used, 1, nc, one, P.cused, nc, stage, st));
    else CK(cudaMemsetAsync(P.cused, 1, (size_t)nc, st));
    CK(cudaStreamSynchronize(st));
    return PGDG_OK;
  }

  int download_cells(pgdg_cells* co) override {
    if (co->n != K.ncell) {
      err = "cell count mismatch";
      return PGDG_EINVAL;
    }
    int rc = ensure_stage();
    if (rc) return rc;
    const int64_t nc = K.ncell;
    int hk[XMAP_MAX];
    double sh[XMAP_MAX];
    const XferMap fs = xmap(F);
    for (int s = 0; s < F; s++) sh[s] = K.eshift[s];
    const XferMap fE = xmap(F, nullptr, sh);
    for (int s = 0; s < F; s++)
      for (int d = 0; d < D; d++) hk[s * D + d] = s * 3 + d;
    const XferMap fv = xmap(F * D, hk);
    for (int t = 0; t < F * U * B; t++) sh[t] = (t % (U * B) == (U - 1) * B) ? K.eshift[t / (U * B)] : 0.0;
    const XferMap fc = xmap(F * U * B, nullptr, sh);
    const XferMap fd = xmap(F * U * B), fl = xmap(F * U), vec = xmap(D), gv = xmap(D * D), one = xmap(1);
    CK(cudaStreamSynchronize(st));
    if (co->rho) CK(xfer_d2h<R>(P.crho, nc, nullptr, nc, fs, co->rho, F, nullptr, nullptr, stage, st));
    if (co->rhov) CK(xfer_d2h<R>(P.crhov, nc, nullptr, nc, fv, co->rhov, 3 * F, nullptr, nullptr, stage, st));
    if (co->E) CK(xfer_d2h<R>(P.cE, nc, nullptr, nc, fE, co->E, F, nullptr, nullptr, stage, st));
    if (co->c) CK(xfer_d2h<R>(P.cc, nc, nullptr, nc, fs, co->c, F, nullptr, nullptr, stage, st));
    if (co->ac) CK(xfer_d2h<R>(P.cac, nc, nullptr, nc, fs, co->ac, F, nullptr, nullptr, stage, st));
    if (co->alph) CK(xfer_d2h<R>(P.calph, nc, nullptr, nc, fs, co->alph, F, nullptr, nullptr, stage, st));
    if (co->coef) CK(xfer_d2h<R>(P.ccoef, nc, nullptr, nc, fc, co->coef, F * U * B, nullptr, nullptr, stage, st));
    if (co->dcoef) CK(xfer_d2h<R>(P.cdcoef, nc, nullptr, nc, fd, co->dcoef, F * U * B, nullptr, nullptr, stage, st));
    if (co->lim_u) CK(xfer_d2h<R>(P.clim, nc, nullptr, nc, fl, co->lim_u, F * U, nullptr, nullptr, stage, st));
    if (co->g_v) CK(xfer_d2h<R>(P.cgv, nc, nullptr, nc, gv, co->g_v, D * D, nullptr, nullptr, stage, st));
    if (co->v) CK(xfer_d2h<R>(P.cv, nc, nullptr, nc, vec, co->v, 3, nullptr, nullptr, stage, st));
    if (co->P) CK(xfer_d2h<R>(P.cP, nc, nullptr, nc, one, co->P, 1, nullptr, nullptr, stage, st));
    if (co->ph_state) CK(xfer_d2h_i8(P.cph, nc, nullptr, nc, fs, co->ph_state, F, stage, st));
    if (co->ph_state_b) CK(xfer_d2h_i8(P.cphb, nc, nullptr, nc, fs, co->ph_state_b, F, stage, st));
    if (co->used) CK(xfer_d2h_i8(P.cused, nc, nullptr, nc, one, co->used, 1, stage, st));
    return PGDG_OK;
  }

  int upload_lists(const int64_t* off, const int64_t* ent) override {
    drop_graphs();
    std::vector<int64_t> slots;
    int rc = alive_slots(slots);
    if (rc) return rc;
    int64_t n = (int64_t)slots.size();
    DevCounters hc = counters();
    int64_t ns = (int64_t)hc.n_slots;
    std::vector<int32_t> len(std::max<int64_t>(ns, 1), -1), arena;
    std::vector<int64_t> lo(std::max<int64_t>(ns, 1), 0);
    for (int64_t i = 0; i < n; i++) {
      int64_t s = slots[i];
      lo[s] = (int64_t)arena.size();
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        int64_t v = ent[e];
        if (v >= 0) arena.push_back((int32_t)slots[v]);
        else if (v == -1) arena.push_back(-1);
        /* boundary entries are not kept on the device: split/merge never match them */
      }
      len[s] = (int32_t)((int64_t)arena.size() - lo[s]);
    }
    if ((int64_t)arena.size() + 16 * K.cap > K.arena_cap) {
      /* grow the list arena to hold the uploaded lists and the ones split/merge add */
      int32_t* na = nullptr;
      CK(cudaStreamSynchronize(st));
      const size_t ncap = arena.size() * 2 + (size_t)K.cap * 32;
      CK(dalloc(&na, ncap));
      for (auto& a : allocs)
        if (a == (void*)P.arena) a = na;
      cudaFree(P.arena);
      P.arena = na;
      K.arena_cap = (int64_t)ncap;
    }
    CK(cudaStreamSynchronize(st));
    if (!arena.empty()) CK(cudaMemcpy(P.arena, arena.data(), 4 * arena.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(P.list_len, len.data(), 4 * ns, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(P.list_off, lo.data(), 8 * ns, cudaMemcpyHostToDevice));
    hc.arena_used = arena.size();
    CK(cudaMemcpy(&P.cnt->arena_used, &hc.arena_used, 8, cudaMemcpyHostToDevice));
    return PGDG_OK;
  }

  int download_lists(int64_t* off, int64_t* ent, int32_t* stored, int64_t cap, int64_t* total) override {
    std::vector<int64_t> slots;
    int rc = alive_slots(slots);
    if (rc) return rc;
    DevCounters hc = counters();
    int64_t ns = (int64_t)hc.n_slots;
    std::vector<int32_t> len(std::max<int64_t>(ns, 1));
    std::vector<int64_t> lo(std::max<int64_t>(ns, 1));
    if (hc.err) {
      err = "device status reports an error; lists are incomplete";
      return PGDG_ESTATE;
    }
    const unsigned long long used = std::min<unsigned long long>(hc.arena_used, (unsigned long long)K.arena_cap);
    std::vector<int32_t> arena(std::max<unsigned long long>(used, 1ull));
    CK(cudaMemcpy(len.data(), P.list_len, 4 * ns, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(lo.data(), P.list_off, 8 * ns, cudaMemcpyDeviceToHost));
    if (used) CK(cudaMemcpy(arena.data(), P.arena, 4 * used, cudaMemcpyDeviceToHost));
    std::vector<int64_t> canon(std::max<int64_t>(ns, 1), -1);
    for (size_t i = 0; i < slots.size(); i++) canon[slots[i]] = (int64_t)i;
    int64_t t = 0;
    for (size_t i = 0; i < slots.size(); i++) {
      int64_t s = slots[i];
      if (off) off[i] = t;
      if (stored) stored[i] = len[s] >= 0 ? 1 : 0;
      for (int32_t e = 0; e < std::max(len[s], 0); e++) {
        int32_t q = arena[lo[s] + e];
        if (ent && t < cap) ent[t] = (q >= 0) ? canon[q] : -1;
        t++;
      }
    }
    if (off) off[slots.size()] = t;
    *total = t;
    return (ent && t > cap) ? PGDG_EOVERFLOW : PGDG_OK;
  }

  int download_cell_lists(int64_t* off, int64_t* ent, int64_t cap, int64_t* total) override {
    std::vector<int64_t> slots;
    int rc = alive_slots(slots);
    if (rc) return rc;
    DevCounters hc = counters();
    int64_t ns = (int64_t)hc.n_slots;
    std::vector<int32_t> bk(K.ncell * K.maxpc), cnt(K.ncell), boff(K.ncell + 1), bent(std::max<int64_t>(K.nbnd, 1));
    std::vector<uint32_t> key(std::max<int64_t>(ns, 1));
    CK(cudaMemcpy(bk.data(), P.bucket, 4 * bk.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cnt.data(), P.bcnt, 4 * cnt.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(boff.data(), P.boff, 4 * boff.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(bent.data(), P.bent, 4 * std::max<int64_t>(K.nbnd, 1), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(key.data(), P.lkey, 4 * ns, cudaMemcpyDeviceToHost));
    std::vector<int64_t> canon(std::max<int64_t>(ns, 1), -1);
    for (size_t i = 0; i < slots.size(); i++) canon[slots[i]] = (int64_t)i;
    int64_t t = 0;
    for (int64_t c = 0; c < K.ncell; c++) {
      if (off) off[c] = t;
      int m = std::min(cnt[c], K.maxpc);
      int r = 0;
      for (; r < m && key[bk[c * K.maxpc + r]] < KEY_APPEND; r++) {
        if (ent && t < cap) ent[t] = canon[bk[c * K.maxpc + r]];
        t++;
      }
      for (int e = boff[c]; e < boff[c + 1]; e++) {
        if (ent && t < cap) ent[t] = -2 - (int64_t)bent[e];
        t++;
      }
      for (; r < m; r++) {
        if (ent && t < cap) ent[t] = canon[bk[c * K.maxpc + r]];
        t++;
      }
    }
    if (off) off[K.ncell] = t;
    *total = t;
    return (ent && t > cap) ? PGDG_EOVERFLOW : PGDG_OK;
  }

  int set_dt(double dt) override {
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(&P.cnt->dt, &dt, 8, cudaMemcpyHostToDevice));
    return PGDG_OK;
  }
  int set_max_v(double mv) override {
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(&P.cnt->max_v, &mv, 8, cudaMemcpyHostToDevice));
    return PGDG_OK;
  }
  int capacity(int64_t* c) override {
    *c = K.cap;
    return PGDG_OK;
  }
  int stats(pgdg_stats* s) override {
    DevCounters h = counters();
    std::memset(s, 0, sizeof(*s));
    s->n_particles = (int64_t)h.n_live;
    s->n_split = (int64_t)h.n_split;
    s->n_inlet = (int64_t)h.n_inlet;
    s->n_outlet = (int64_t)h.n_outlet;
    s->n_merge = (int64_t)h.n_merge;
    s->n_affected = (int64_t)h.n_affected;
    s->mgfm_calls = (int64_t)h.mgfm_calls;
    s->mgfm_iters = (int64_t)h.mgfm_iters;
    s->mgfm_maxit_hits = (int64_t)h.mgfm_maxit;
    s->g2p_fallbacks = (int64_t)h.g2p_fb;
    s->list_entries = (int64_t)h.arena_used;
    s->iterate_num = iterate;
    s->dt = h.dt;
    s->max_v = h.max_v;
    s->time = h.time;
    return PGDG_OK;
  }

  /* ---------------- methods ---------------- */
  int set_timestep(double* dt, double* mv) override {
    timed("set_timestep", 3, [&] { Launch<D, R, EX>::set_timestep(K, P, iterate > 1 ? 1 : 0, st); });
    if (dt || mv) {
      DevCounters h = counters();
      if (dt) *dt = h.dt;
      if (mv) *mv = h.max_v;
    }
    return PGDG_OK;
  }
  int used_state() override {
    timed("used_state", 1, [&] { Launch<D, R, EX>::used_state(K, P, st); });
    return PGDG_OK;
  }
  int bin() override {
    timed("bin", 2, [&] { Launch<D, R, EX>::bin(K, P, st); });
    fresh_bins = true;
    nb_set = false;
    return PGDG_OK;
  }
  int split() override {
    timed("split", 14, [&] { Launch<D, R, EX>::split(K, P, st); });
    nb_set = false;
    return PGDG_OK;
  }
  int merge(bool chained = false) override {
    timed("merge", 14, [&] { Launch<D, R, EX>::merge(K, P, chained, st); });
    nb_set = false;
    return PGDG_OK;
  }
  /* flag 4: a cell's particle list is its bucket and a particle's in_ele[0]
   * is the cell holding it (lcell); both are kept current by bin/split/merge */
  int refresh_membership() override { return PGDG_OK; }
  /* flag 2: the lists are recomputed from the stage-start coordinates inside
   * the shifting kernel; nothing to do here */
  int refresh_neighbors() override { return PGDG_OK; }
  int p2g() override {
    timed("p2g", 1, [&] { Launch<D, R, EX>::p2g(K, P, fresh_bins && p2g_skip, st); });
    timed("p2g_new", 1, [&] { Launch<D, R, EX>::p2g_new(K, P, st); });
    return PGDG_OK;
  }
  int limiter() override {
    timed("limiter", 1, [&] { Launch<D, R, EX>::limiter(K, P, st); });
    return PGDG_OK;
  }
  int iface_download(double* in6, int8_t* mat2, int64_t cap, int64_t* n) override {
    flush_prof();
    CK(cudaStreamSynchronize(st));
    unsigned long long t[2] = {0, 0};
    if (iface_queue && !EX) CK(cudaMemcpy(t, Q.tot, sizeof(t), cudaMemcpyDeviceToHost));
    *n = (int64_t)t[1];
    const int64_t m = std::min<int64_t>(cap, (int64_t)t[1]);
    if (m > 0) {
      CK(cudaMemcpy(in6, Q.in6, sizeof(double) * 6 * m, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(mat2, Q.mat, 2 * m, cudaMemcpyDeviceToHost));
    }
    return PGDG_OK;
  }
  /* autotuner: time each variant of a kernel twice on the current state (the
   * kernel must only overwrite its outputs, and all variants give the same
   * results) and keep the fastest */
  template <class F>
  int tune(int nvar, F&& run) {
    if (nvar <= 1) return 0;
    cudaEvent_t a = ev_get(), b = ev_get();
    float best = 0.f;
    int bv = 0;
    for (int v = 0; v < nvar; v++) {
      run(v);
      cudaEventRecord(a, st);
      run(v);
      run(v);
      cudaEventRecord(b, st);
      if (cudaEventSynchronize(b) != cudaSuccess) return 0;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      if (v == 0 || ms < best) {
        best = ms;
        bv = v;
      }
    }
    return bv;
  }
  int grow_queue(int64_t need) {
    drop_graphs(); /* they hold the old buffers */
    CK(cudaStreamSynchronize(st));
    for (void* p : {(void*)Q.in6, (void*)Q.mat, (void*)Q.out3}) {
      for (auto& a : allocs)
        if (a == p) a = nullptr;
      cudaFree(p);
    }
    Q.cap = need;
    CK(A(&Q.in6, 6 * (size_t)Q.cap));
    CK(A(&Q.mat, 2 * (size_t)Q.cap));
    CK(A(&Q.out3, 3 * (size_t)Q.cap));
    return PGDG_OK;
  }
  /* Host-side upkeep of the interface queue, between steps: grow it to twice
   * the last stage's problem count when that passed half its capacity, and
   * hold the batch scratch for its capacity, so that steps (captured or not)
   * never allocate or read back.  A stage that still outgrows the queue is
   * solved inline by the residual. */
  int ensure_queue() {
    if (!iface_queue || EX) return PGDG_OK;
    unsigned long long t[2] = {0, 0};
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(t, Q.tot, sizeof(t), cudaMemcpyDeviceToHost));
    if (iface_cap_fixed < 0 && (int64_t)t[0] * 2 > Q.cap) {
      int rc = grow_queue((int64_t)t[0] * 2 + 4096);
      if (rc) return rc;
    }
    const int rc = mgfm_seeded_reserve(net, part, Q.cap);
    if (rc) err = "interface batch scratch: out of device memory";
    return rc;
  }
  bool capturing = false;
  int prepare_step() override { return ensure_queue(); }
  int set_iface_cap(int64_t cap) override {
    iface_cap_fixed = cap;
    if (cap >= 0 && cap != Q.cap) return grow_queue(cap > 0 ? cap : 1);
    drop_graphs();
    return PGDG_OK;
  }
  int grid_acc() override {
    if (!iface_queue || EX) {
      timed("grid_acc", 1, [&] { Launch<D, R, EX>::grid_acc(K, P, st); });
      return PGDG_OK;
    }
    /* surrogate-seeded MGFM: queue the interface problems, solve them in one
     * batch, then evaluate the residual with the queued ghost states.  The
     * batch's size stays on the device (Q.tot): nothing is read back */
    if (!capturing) {
      const int rc = mgfm_seeded_reserve(net, part, Q.cap);
      if (rc) return rc;
    }
    timed("iface_gather", 6, [&] { Launch<D, R, EX>::iface_gather(K, P, Q, st); });
    int rc = PGDG_OK;
    timed("mgfm_seeded", net ? 8 : 6, [&] {
      rc = mgfm_seeded_run(net, Q.in6, Q.mat, d_gam, d_pinf, K.mgfm_variant, Q.out3, nullptr, Q.cap,
                           &P.cnt->mgfm_calls, part, st, Q.tot + 1);
    });
    if (rc) return rc;
    timed("grid_acc", 2, [&] { Launch<D, R, EX>::grid_acc_queued(K, P, Q, st); });
    return PGDG_OK;
  }
  int update_grid(int md) override {
    timed("update_grid", 1, [&] { Launch<D, R, EX>::update_grid(K, P, md, st); });
    return PGDG_OK;
  }
  int update_particle(int md) override {
    fresh_bins = false;
    const int xs = P.xb, hs = P.hb, hn = 1 - P.hb;
    int x0, xn;
    if (md == 0) {
      x0 = xs;
      xn = (xs + 1) % 3;
      x0b = xs;
    } else {
      x0 = x0b;
      xn = 3 - xs - x0b;
      if (xn == xs || xn == x0 || xn < 0 || xn > 2) xn = (xs + 1) % 3;  /* md 1 without md 0 */
    }
    timed("g2p", 1, [&] { Launch<D, R, EX>::g2p(K, P, md, xs, x0, xn, hn, !g2p_partial, st); });
    if (!EX) timed("rowsort", 3, [&] { Launch<D, R, EX>::rowsort(K, P, xs, pst_scratch, st); });
    if (pst_var < 0)
      pst_var = tune(Launch<D, R, EX>::pst_variants(),
                     [&](int v) { Launch<D, R, EX>::pst(K, P, xs, hs, xn, hn, v, pst_scratch, st); });
    timed("pst", 1, [&] { Launch<D, R, EX>::pst(K, P, xs, hs, xn, hn, pst_var, pst_scratch, st); });
    if (md == 1) timed("store_lists", 2, [&] { Launch<D, R, EX>::store_lists(K, P, xs, hs, xn, st); });
    if (md == 1) {
      nb_xs = xs;
      nb_hs = hs;
      nb_set = true;
    }
    P.xb = xn;
    P.hb = hn;
    return PGDG_OK;
  }
  int run_step(int64_t n) override {
    timed("set_timestep", 1, [&] { Launch<D, R, EX>::add_time(P, st); }); /* simulated time += dt */
    if (n == 1) used_state();
    bin();
    split();
    for (int it = 0; it < cs.merge_iters; it++) merge(it > 0);
    refresh_membership();
    for (int md = 0; md < 2; md++) {
      refresh_neighbors();
      if (md == 0) p2g();
      limiter();
      grid_acc();
      update_grid(md);
      /* inside a step, the first stage's G2P skips the fields the second
       * stage's G2P rewrites before anything reads them */
      g2p_partial = md == 0;
      update_particle(md);
      g2p_partial = false;
    }
    return PGDG_OK;
  }
  /* ---------------- CUDA graphs of whole steps ----------------
   * A step reads nothing back on the host (the interface queue is sized on
   * the device and checked by ensure_queue() between calls), so advance()
   * captures it.  The coordinate buffers rotate with a period of three steps
   * (the buffer indices are kernel arguments), so the graph holds three steps,
   * one per rotation phase P.xb.  Steps that cannot be captured run eagerly:
   * the first two iterations (Used_state_update, and Set_timestep's rule while
   * iterate_num <= 1), any step while per-method timing is on, a step before
   * the kernel-variant tuning, and the remainder of a call below three steps. */
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    int xb_after = 0, hb_after = 0, x0b_after = 0;
    int64_t launches = 0;
  };
  StepGraph graphs[3];
  bool graphs_enabled = true;
  void invalidate_graphs() override { drop_graphs(); }
  void enable_graphs(bool on) override {
    drop_graphs();
    graphs_enabled = on;
  }
  void drop_graphs() {
    for (auto& g : graphs) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g = StepGraph{};
    }
  }
  int capture3(StepGraph& sg) {
    const int xb0 = P.xb, hb0 = P.hb, x0b0 = x0b;
    const int64_t it0 = iterate, l0 = launches;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return PGDG_ECUDA;
    capturing = true;
    for (int k = 0; k < 3; k++) {
      set_timestep(nullptr, nullptr);
      iterate++;
      run_step(iterate);
    }
    capturing = false;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    sg.xb_after = P.xb;
    sg.hb_after = P.hb;
    sg.x0b_after = x0b;
    sg.launches = launches - l0;
    P.xb = xb0;
    P.hb = hb0;
    x0b = x0b0;
    iterate = it0;
    launches = l0;
    if (e != cudaSuccess || !g) {
      cudaGetLastError();
      return PGDG_ECUDA;
    }
    e = cudaGraphInstantiate(&sg.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      sg.exec = nullptr;
      cudaGetLastError();
      return PGDG_ECUDA;
    }
    return PGDG_OK;
  }
  int advance(int nsteps) override {
    int rc = ensure_queue();
    if (rc) return rc;
    int s = 0;
    while (s < nsteps) {
      const bool graphable = graphs_enabled && !prof && iterate >= 2 && pst_var >= 0 && nsteps - s >= 3;
      if (graphable) {
        StepGraph& sg = graphs[P.xb];
        if (!sg.exec && capture3(sg) != PGDG_OK) {
          graphs_enabled = false; /* capture refused: stay eager */
          continue;
        }
        if (cudaGraphLaunch(sg.exec, st) != cudaSuccess) {
          err = "graph launch failed";
          return PGDG_ECUDA;
        }
        P.xb = sg.xb_after;
        P.hb = sg.hb_after;
        x0b = sg.x0b_after;
        /* the graph's last stage searched with the buffers its first stage wrote */
        nb_xs = 3 - P.xb - x0b;
        nb_hs = 1 - P.hb;
        nb_set = true;
        iterate += 3;
        launches += sg.launches;
        s += 3;
        continue;
      }
      set_timestep(nullptr, nullptr);
      iterate++;
      run_step(iterate);
      s++;
    }
    return PGDG_OK;
  }
  /* Output_point (mpm_ini.cpp:774-824) on the device; 5 doubles come back */
  int output_point(double* out5) override {
    Launch<D, R, EX>::probe(K, P, d_tot, d_tot, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(out5, d_tot, 5 * sizeof(double), cudaMemcpyDeviceToHost));
    return PGDG_OK;
  }
  /* ---------------- snapshot writers (Output_plt_file) ----------------
   * The live particles and the cells are packed on the context stream into a
   * snapshot that no later call touches; a host thread (or the caller, when
   * async is 0) then copies it out through two pinned chunks on a copy stream
   * while it writes the files.  The device goes on with the next steps
   * meanwhile; a further output call, output_wait() or destruction waits for
   * the writer. */
  int output_plt(const char* pp, const char* cp, int async) override {
    int rc = output_wait();
    if (rc) return rc;
    if (!pp && !cp) return PGDG_OK;
    flush_prof();
    int64_t n = 0;
    if (pp) {
      rc = alive(&n);
      if (rc) return rc;
    }
    const DevCounters hc = counters();
    if (hc.err) {
      err = "device status reports an error; no snapshot written";
      return PGDG_ESTATE;
    }
    if (pp && n > ocap) {
      if (d_odv) cudaFree(d_odv);
      if (d_oiv) cudaFree(d_oiv);
      d_odv = nullptr;
      d_oiv = nullptr;
      ocap = 0;
      CK(cudaMalloc(&d_odv, sizeof(double) * 10 * (size_t)std::max<int64_t>(n, 1)));
      CK(cudaMalloc(&d_oiv, sizeof(int32_t) * 2 * (size_t)std::max<int64_t>(n, 1)));
      ocap = n;
    }
    if (cp && !d_odc) CK(cudaMalloc(&d_odc, sizeof(double) * 12 * (size_t)K.ncell));
    if (!ost) {
      CK(cudaStreamCreateWithFlags(&ost, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&oev, cudaEventDisableTiming));
      for (int k = 0; k < 2; k++) {
        CK(cudaEventCreateWithFlags(&ochev[k], cudaEventDisableTiming));
        CK(cudaMallocHost(&h_och[k], OCHUNK));
      }
    }
    const int xs = nb_set ? nb_xs : P.xb, hs = nb_set ? nb_hs : P.hb;
    if (pp) output_pack_particles<D, R, EX>(K, P, d_alive, n, xs, hs, d_odv, d_oiv, st);
    if (cp) output_pack_cells<D, R, EX>(K, P, d_odc, st);
    CK(cudaGetLastError());
    CK(cudaEventRecord(oev, st));
    const std::string spp = pp ? pp : "", scp = cp ? cp : "";
    const double time = hc.time;
    if (async) {
      orunning = true;
      oth = std::thread([this, n, time, spp, scp] { orc = output_job(n, time, spp, scp); });
      return PGDG_OK;
    }
    rc = output_job(n, time, spp, scp);
    if (rc) err = omsg;
    return rc;
  }
  int output_wait() override {
    if (!orunning) return PGDG_OK;
    oth.join();
    orunning = false;
    const int rc = orc;
    orc = PGDG_OK;
    if (rc) err = omsg;
    return rc;
  }
  /* device range -> file through the pinned chunks (the copy of chunk k + 1
   * overlaps the write of chunk k) */
  bool copy_out(const void* src, size_t bytes, FILE* f) {
    const size_t nch = (bytes + OCHUNK - 1) / OCHUNK;
    auto issue = [&](size_t k) {
      const size_t off = k * OCHUNK, len = std::min(OCHUNK, bytes - off);
      cudaMemcpyAsync(h_och[k & 1], static_cast<const char*>(src) + off, len, cudaMemcpyDeviceToHost, ost);
      cudaEventRecord(ochev[k & 1], ost);
    };
    if (nch) issue(0);
    for (size_t k = 0; k < nch; k++) {
      if (k + 1 < nch) issue(k + 1);
      if (cudaEventSynchronize(ochev[k & 1]) != cudaSuccess) return false;
      const size_t off = k * OCHUNK, len = std::min(OCHUNK, bytes - off);
      if (std::fwrite(h_och[k & 1], 1, len, f) != len) return false;
    }
    return true;
  }
  int output_job(int64_t n, double time, const std::string& pp, const std::string& cp) {
    if (cudaSetDevice(dev_id) != cudaSuccess || cudaStreamWaitEvent(ost, oev, 0) != cudaSuccess) {
      omsg = "snapshot writer: CUDA setup failed";
      return PGDG_ECUDA;
    }
    if (!pp.empty()) {
      FILE* f = std::fopen(pp.c_str(), "wb");
      if (!f) {
        omsg = "cannot open " + pp;
        return PGDG_EINVAL;
      }
      const std::string hdr = pgdg_out::plt_header(n, time);
      bool ok = std::fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
      /* file order x y z phase vx vy vol rho P tv v n_neighbor: (int32?, index) */
      static const int kind[12] = {0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1};
      static const int idx[12] = {0, 1, 2, 0, 3, 4, 5, 6, 7, 8, 9, 1};
      for (int j = 0; j < 12 && ok; j++) {
        if (kind[j] == 0) ok = copy_out(d_odv + (size_t)idx[j] * n, sizeof(double) * (size_t)n, f);
        else ok = copy_out(d_oiv + (size_t)idx[j] * n, sizeof(int32_t) * (size_t)n, f);
      }
      if (std::fclose(f) != 0) ok = false;
      if (!ok) {
        omsg = "writing " + pp + " failed";
        return PGDG_ECUDA;
      }
    }
    if (!cp.empty()) {
      std::vector<double> cols(12 * (size_t)K.ncell);
      if (cudaMemcpyAsync(cols.data(), d_odc, sizeof(double) * cols.size(), cudaMemcpyDeviceToHost, ost) !=
              cudaSuccess ||
          cudaStreamSynchronize(ost) != cudaSuccess) {
        omsg = "snapshot writer: cell copy failed";
        return PGDG_ECUDA;
      }
      const unsigned hw = std::thread::hardware_concurrency();
      if (pgdg_out::write_cell_table(cp.c_str(), D, K.N, cs.box_l, cs.p_size, cols.data(), time,
                                     (int)std::max(1u, std::min(hw, 16u)), &omsg))
        return PGDG_EINVAL;
    }
    return PGDG_OK;
  }
  int totals(double* out) override {
    Launch<D, R, EX>::totals(K, P, d_tot, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(out, d_tot, (2 * F + 2) * sizeof(double), cudaMemcpyDeviceToHost));
    return PGDG_OK;
  }
};

}  // namespace

/* ---------------------------------------------------------------------- */
extern "C" {

int pgdg_create(const pgdg_case* cs, int precision, int64_t capacity, pgdg_ctx** out) {
  if (!cs || !out || (cs->dim != 2 && cs->dim != 3)) return PGDG_EINVAL;
  if (cs->nfld != F) {
    fprintf(stderr, "pgdg_create: the case has %d materials; this build holds %d (FldNum is fixed per build)\n",
            cs->nfld, F);
    return PGDG_EINVAL;
  }
  if (precision != PGDG_PREC_FP64 && precision != PGDG_PREC_MIXED && precision != PGDG_PREC_FP64_FMA)
    return PGDG_EINVAL;
  for (int d = 0; d < cs->dim; d++)
    if (cs->ncell[d] < 1) return PGDG_EINVAL;
  /* the shifting kernel's row sort (mixed and FP64_FMA paths) stores each
   * entry's cell offset within its row in 16 bits */
  if (precision != PGDG_PREC_FP64 && cs->ncell[cs->dim - 1] > 65535) {
    fprintf(stderr, "pgdg_create: %d cells along the last axis; the row sort of this precision holds at most 65535\n",
            cs->ncell[cs->dim - 1]);
    return PGDG_EINVAL;
  }
  int dev = 0;
  if (cudaGetDeviceCount(&dev) != cudaSuccess || dev < 1) return PGDG_ECUDA;
  pgdg_ctx* c;
  int rc;
#define PGDG_MK(DD, RR, XX)                 \
  {                                         \
    auto* x = new Ctx<DD, RR, XX>();        \
    rc = x->init(cs, precision, capacity);  \
    c = x;                                  \
  }
  if (cs->dim == 2) {
    if (precision == PGDG_PREC_FP64) PGDG_MK(2, double, true)
    else if (precision == PGDG_PREC_FP64_FMA) PGDG_MK(2, double, false)
    else PGDG_MK(2, float, false)
  } else {
#if PGDG_WITH_3D
    if (precision == PGDG_PREC_FP64) PGDG_MK(3, double, true)
    else if (precision == PGDG_PREC_FP64_FMA) PGDG_MK(3, double, false)
    else PGDG_MK(3, float, false)
#else
    fprintf(stderr, "pgdg_create: this build holds the 2D three-material instance only\n");
    return PGDG_EINVAL;
#endif
  }
#undef PGDG_MK
  if (rc) {
    fprintf(stderr, "pgdg_create: %s\n", c->err.c_str());
    delete c;
    return rc;
  }
  *out = c;
  return PGDG_OK;
}
int pgdg_destroy(pgdg_ctx* ctx) {
  delete ctx;
  return PGDG_OK;
}
const char* pgdg_last_error(pgdg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
int pgdg_capacity(pgdg_ctx* ctx, int64_t* cap) { return ctx->capacity(cap); }
int pgdg_upload_particles(pgdg_ctx* ctx, const pgdg_particles* p) { return ctx->upload_particles(p); }
int pgdg_output_point(pgdg_ctx* ctx, double* out5) {
  if (!ctx || !out5) return PGDG_EINVAL;
  return ctx->output_point(out5);
}
int pgdg_output_plt(pgdg_ctx* ctx, const char* particle_path, const char* cell_path, int async) {
  if (!ctx) return PGDG_EINVAL;
  return ctx->output_plt(particle_path, cell_path, async);
}
int pgdg_output_wait(pgdg_ctx* ctx) {
  if (!ctx) return PGDG_EINVAL;
  return ctx->output_wait();
}
int pgdg_case_build(pgdg_ctx* ctx, int config_id, uint64_t seed) {
  if (!ctx || config_id < 1 || config_id > 5) return PGDG_EINVAL;
  return ctx->case_build(config_id, seed);
}
int pgdg_download_particles(pgdg_ctx* ctx, pgdg_particles* p) { return ctx->download_particles(p); }
int pgdg_num_particles(pgdg_ctx* ctx, int64_t* n) { return ctx->num_particles(n); }
int pgdg_upload_cells(pgdg_ctx* ctx, const pgdg_cells* c) { return ctx->upload_cells(c); }
int pgdg_download_cells(pgdg_ctx* ctx, pgdg_cells* c) { return ctx->download_cells(c); }
int pgdg_upload_lists(pgdg_ctx* ctx, const int64_t* off, const int64_t* ent) { return ctx->upload_lists(off, ent); }
int pgdg_download_lists(pgdg_ctx* ctx, int64_t* off, int64_t* ent, int32_t* stored, int64_t cap, int64_t* total) {
  return ctx->download_lists(off, ent, stored, cap, total);
}
int pgdg_download_cell_lists(pgdg_ctx* ctx, int64_t* off, int64_t* ent, int64_t cap, int64_t* total) {
  return ctx->download_cell_lists(off, ent, cap, total);
}
int pgdg_set_dt(pgdg_ctx* ctx, double dt) { return ctx->set_dt(dt); }
int pgdg_set_iterate(pgdg_ctx* ctx, int64_t n) {
  ctx->iterate = n;
  return PGDG_OK;
}
int pgdg_set_max_v(pgdg_ctx* ctx, double mv) { return ctx->set_max_v(mv); }
int pgdg_get_stats(pgdg_ctx* ctx, pgdg_stats* st) { return ctx->stats(st); }
int pgdg_set_surrogate(pgdg_ctx* ctx, pgdg_mlp* net) {
  if (net && ctx->precision == PGDG_PREC_FP64) {
    ctx->err = "the seed surrogate is not used by the exact-order FP64 path";
    return PGDG_EINVAL;
  }
  ctx->net = (void*)net;
  ctx->iface_queue = net ? 1 : ctx->iface_queue;
  ctx->invalidate_graphs();
  return PGDG_OK;
}
int pgdg_set_graphs(pgdg_ctx* ctx, int on) {
  ctx->enable_graphs(on != 0);
  return PGDG_OK;
}
int pgdg_tune(pgdg_ctx* ctx, const char* kernel, int variant, int* chosen) {
  if (kernel && std::strcmp(kernel, "iface_cap") == 0 && variant >= -1) {
    const int rc = ctx->set_iface_cap(variant);
    if (chosen) *chosen = variant;
    return rc;
  }
  if (kernel && std::strcmp(kernel, "p2g_skip") == 0 && variant >= -2 && variant <= 1) {
    if (variant >= 0) ctx->p2g_skip = variant;
    if (variant >= 0) ctx->invalidate_graphs();
    if (chosen) *chosen = ctx->p2g_skip;
    return PGDG_OK;
  }
  if (!kernel || std::strcmp(kernel, "pst") != 0 || variant < -2) {
    ctx->err = "tunable kernels: pst (variant >= -2), p2g_skip (0, 1, or -2 to query), iface_cap (>= -1)";
    return PGDG_EINVAL;
  }
  if (variant >= 0) ctx->pst_var = variant;
  else if (variant == -1) ctx->pst_var = -1;
  if (variant >= -1) ctx->invalidate_graphs();
  if (chosen) *chosen = ctx->pst_var;
  return PGDG_OK;
}
int pgdg_set_iface_queue(pgdg_ctx* ctx, int on) {
  if (on && ctx->precision == PGDG_PREC_FP64) {
    ctx->err = "the exact-order FP64 path solves interface problems inline";
    return PGDG_EINVAL;
  }
  if (!on && ctx->net) {
    ctx->err = "detach the seed surrogate first";
    return PGDG_EINVAL;
  }
  ctx->iface_queue = on ? 1 : 0;
  ctx->invalidate_graphs();
  return PGDG_OK;
}
int pgdg_iface_download(pgdg_ctx* ctx, double* in6, int8_t* mat2, int64_t cap, int64_t* n) {
  if (!in6 || !mat2 || !n || cap < 0) return PGDG_EINVAL;
  return ctx->iface_download(in6, mat2, cap, n);
}
int pgdg_synchronize(pgdg_ctx* ctx) { return ctx->check(); }
int pgdg_set_timestep(pgdg_ctx* ctx, double* dt, double* mv) { return ctx->set_timestep(dt, mv); }
int pgdg_used_state_update(pgdg_ctx* ctx) { return ctx->used_state(); }
int pgdg_bin_particles(pgdg_ctx* ctx) { return ctx->bin(); }
int pgdg_split_particle_fast(pgdg_ctx* ctx) { return ctx->split(); }
int pgdg_merge_particle_fast(pgdg_ctx* ctx) { return ctx->merge(); }
int pgdg_refresh_membership(pgdg_ctx* ctx) { return ctx->refresh_membership(); }
int pgdg_refresh_neighbors(pgdg_ctx* ctx) { return ctx->refresh_neighbors(); }
int pgdg_mls_p2g(pgdg_ctx* ctx) { return ctx->p2g(); }
int pgdg_calculate_limiter(pgdg_ctx* ctx) { return ctx->limiter(); }
int pgdg_grid_acceleration(pgdg_ctx* ctx) { return ctx->grid_acc(); }
int pgdg_update_grid(pgdg_ctx* ctx, int md) { return ctx->update_grid(md); }
int pgdg_update_particle(pgdg_ctx* ctx, int md) { return ctx->update_particle(md); }
int pgdg_run_step(pgdg_ctx* ctx, int64_t n) {
  const int rc = ctx->prepare_step();
  return rc ? rc : ctx->run_step(n);
}
int pgdg_advance(pgdg_ctx* ctx, int nsteps) { return ctx->advance(nsteps); }
int pgdg_totals(pgdg_ctx* ctx, double* out6) { return ctx->totals(out6); }

int pgdg_profile(pgdg_ctx* ctx, int enable) {
  ctx->flush_prof();
  ctx->prof = enable != 0;
  if (enable) {
    ctx->knames.clear();
    ctx->kms.clear();
    ctx->kcnt.clear();
  }
  return PGDG_OK;
}
int pgdg_profile_read(pgdg_ctx* ctx, char* names, int names_cap, double* ms, int64_t* counts, int cap, int* n) {
  ctx->flush_prof();
  int k = (int)ctx->knames.size();
  *n = k;
  std::string all;
  for (int i = 0; i < k; i++) {
    if (i < cap) {
      if (ms) ms[i] = ctx->kms[i];
      if (counts) counts[i] = ctx->kcnt[i];
    }
    all += ctx->knames[i];
    all += ';';
  }
  if (names && names_cap > 0) {
    std::strncpy(names, all.c_str(), names_cap - 1);
    names[names_cap - 1] = 0;
  }
  return PGDG_OK;
}
int pgdg_launch_count(pgdg_ctx* ctx, int64_t* n) {
  *n = ctx->launches;
  return PGDG_OK;
}
int pgdg_time_advance(pgdg_ctx* ctx, int nsteps, double* ms) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaStreamSynchronize(ctx->st);
  cudaEventRecord(a, ctx->st);
  int rc = ctx->advance(nsteps);
  cudaEventRecord(b, ctx->st);
  cudaEventSynchronize(b);
  float f = 0;
  cudaEventElapsedTime(&f, a, b);
  *ms = f;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  return ctx->check();
}

}  // extern "C"
