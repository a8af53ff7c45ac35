/*
 * k_particles.cu -- particle bookkeeping kernels: binning (Map_the_particle_to_tree),
 * Split_particle_fast, Merge_particle_fast, neighbour-list refresh for split/merge
 * and the stored-list kernel.
 *
 * Compiled with -fmad=false: the FP64 arithmetic here must reproduce the CPU
 * oracle bit for bit (split/merge are bit-exact per call on identical inputs).
 *
 * Cell lists (Cell_list::particle_list, cell_list.cpp) are fixed-capacity buckets
 * kept in list order.  A list entry's order key is its slot for entries placed by
 * Map_the_particle_to_tree (particles are binned in particle_fluid order,
 * mpm.cpp:74-96) and KEY_APPEND + n for the n-th Add_particle call of the step
 * (split/merge append at the list's end, cell_list.cpp:34-37); Remove_particle
 * (cell_list.cpp:41-52) keeps the order of the rest.  Split/merge change few
 * buckets; those are marked dirty and re-sorted.
 */
#include "pgdg_dev.cuh"

namespace pgdg {

constexpr int BLK = 256;
constexpr int SCAN_TILE = 2048;     /* 256 threads x 8 */
constexpr int MAXPC_MAX = 64;

int grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  const int64_t cap = 152 * 32;     /* grid-stride beyond 32 CTAs per SM */
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

/* ------------------------------------------------------------------ */
/* exclusive scan of unsigned 64-bit values over [0, *d_n)            */
/* ------------------------------------------------------------------ */
__global__ void k_scan_tiles(unsigned long long* data, unsigned long long* blk, const unsigned long long* d_n) {
  __shared__ unsigned long long sh[BLK];
  const int64_t n = (int64_t)*d_n;
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * 8;
  unsigned long long v[8];
  unsigned long long s = 0;
  for (int k = 0; k < 8; k++) {
    int64_t i = base + k;
    v[k] = (i < n) ? data[i] : 0ull;
    s += v[k];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < BLK; off <<= 1) {
    unsigned long long t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0ull;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  unsigned long long run = sh[threadIdx.x] - s;
  for (int k = 0; k < 8; k++) {
    int64_t i = base + k;
    if (i < n) data[i] = run;
    run += v[k];
  }
  if (threadIdx.x == BLK - 1) blk[blockIdx.x] = sh[BLK - 1];
}

__global__ void k_scan_blocks(unsigned long long* blk, int nblk) {
  /* one block; blk[nblk] receives the grand total */
  __shared__ unsigned long long sh[1024];
  const int per = (nblk + 1023) / 1024;
  const int b0 = threadIdx.x * per;
  unsigned long long s = 0;
  for (int k = 0; k < per; k++)
    if (b0 + k < nblk) s += blk[b0 + k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned long long t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0ull;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  unsigned long long run = sh[threadIdx.x] - s;
  for (int k = 0; k < per; k++)
    if (b0 + k < nblk) {
      unsigned long long t = blk[b0 + k];
      blk[b0 + k] = run;
      run += t;
    }
  if (threadIdx.x == 1023) blk[nblk] = sh[1023];
}

__global__ void k_scan_add(unsigned long long* data, const unsigned long long* blk, const unsigned long long* d_n) {
  const int64_t n = (int64_t)*d_n;
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x * 8;
  unsigned long long add = blk[blockIdx.x];
  for (int k = 0; k < 8; k++) {
    int64_t i = base + k;
    if (i < n) data[i] += add;
  }
}

/* data[0..n) -> exclusive prefix; blk[nblk] = total, nblk = ceil(cap / SCAN_TILE) */
void scan_u64(unsigned long long* data, unsigned long long* blk, const unsigned long long* d_n, int64_t cap,
              cudaStream_t st) {
  int nblk = (int)((cap + SCAN_TILE - 1) / SCAN_TILE);
  k_scan_tiles<<<nblk, BLK, 0, st>>>(data, blk, d_n);
  k_scan_blocks<<<1, 1024, 0, st>>>(blk, nblk);
  k_scan_add<<<nblk, BLK, 0, st>>>(data, blk, d_n);
}
__host__ __device__ inline int scan_nblk(int64_t cap) { return (int)((cap + SCAN_TILE - 1) / SCAN_TILE); }

/* ------------------------------------------------------------------ */
/* helpers                                                            */
/* ------------------------------------------------------------------ */
#define GRID_STRIDE(i, n) for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
                               i += (int64_t)gridDim.x * blockDim.x)

template <int D, typename R>
__device__ __forceinline__ void load_x(const CaseK& K, const R* X, int64_t p, R* x) {
  for (int d = 0; d < D; d++) x[d] = X[d * K.cap + p];
}

template <int D>
__device__ __forceinline__ double dist_exact(const double* a, const double* b) {
  /* get_distance (glbfunc.h:175-183) / Eigen norm, left to right */
  double dd = 0.0;
  for (int d = 0; d < D; d++) {
    double t = dsub(a[d], b[d]);
    dd = (d == 0) ? dmul(t, t) : dadd(dd, dmul(t, t));
  }
  return dsqrt(dd);
}

template <typename R>
__device__ __forceinline__ void mark_dirty(const DevPtrs<R>& P, int64_t c) {
  unsigned int old = atomicOr(&P.cflag[c], 1u);
  if (!(old & 1u)) {
    unsigned long long qi = atomicAdd(&P.cnt->n_dirty, 1ull);
    if ((int64_t)qi < P.qcap) P.dirty_q[qi] = (int32_t)c;
    else atomicOr(&P.cnt->err, ERR_CELLQ);
  }
}

template <int D, typename R>
__device__ __forceinline__ void flag_cells(const CaseK& K, const DevPtrs<R>& P, const int* pos) {
  int lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    int r = (d < D) ? 2 : 0;
    lo[d] = max(pos[d] - r, 0);
    hi[d] = min(pos[d] + r, (d < D ? K.N[d] : 1) - 1);
  }
  for (int t = lo[0]; t <= hi[0]; t++)
    for (int s = lo[1]; s <= hi[1]; s++)
      for (int m = lo[2]; m <= hi[2]; m++) {
        int q[3] = {t, s, m};
        int64_t c = cidx<D>(K, q);
        unsigned int old = atomicOr(&P.cflag[c], 2u);
        if (!(old & 2u)) {
          unsigned long long qi = atomicAdd(&P.cnt->n_flagged, 1ull);
          if ((int64_t)qi < P.qcap) P.flag_q[qi] = (int32_t)c;
          else atomicOr(&P.cnt->err, ERR_CELLQ);
        }
      }
}

template <typename R>
__device__ __forceinline__ void bucket_append(const CaseK& K, const DevPtrs<R>& P, int64_t c, int64_t slot) {
  int pos = atomicAdd(&P.bcnt[c], 1);
  if (pos < K.maxpc) P.bucket[c * K.maxpc + pos] = (int32_t)slot;
  else atomicOr(&P.cnt->err, ERR_BUCKET);
}

/* ------------------------------------------------------------------ */
/* binning                                                            */
/* ------------------------------------------------------------------ */
template <int D, typename R>
__global__ void k_bin_scatter(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)P.cnt->n_slots;
  const R* X = P.X[P.xb];
  GRID_STRIDE(p, n) {
    if (P.phase[p] == 0) {
      P.lcell[p] = -1;
      continue;
    }
    R x[3];
    load_x<D>(K, X, p, x);
    int pos[3];
    cell_pos<D>(K, x, pos);
    int64_t c = cidx<D>(K, pos);
    P.lcell[p] = (int32_t)c;
    P.lkey[p] = (uint32_t)p;
    bucket_append(K, P, c, p);
  }
}

/* re-sort the buckets of all cells (all = 1) or of the dirty queue */
template <typename R>
__global__ void k_bucket_fix(CaseK K, DevPtrs<R> P, int all) {
  const int64_t n = all ? K.ncell : (int64_t)min(P.cnt->n_dirty, (unsigned long long)P.qcap);
  GRID_STRIDE(i, n) {
    int64_t c = all ? i : P.dirty_q[i];
    int m = min(P.bcnt[c], K.maxpc);
    unsigned long long key[MAXPC_MAX];
    int k = 0;
    int32_t* b = P.bucket + c * K.maxpc;
    for (int r = 0; r < m; r++) {
      int32_t e = b[r];
      if (P.lcell[e] == (int32_t)c) key[k++] = ((unsigned long long)P.lkey[e] << 32) | (unsigned int)e;
    }
    for (int a = 1; a < k; a++) {
      unsigned long long t = key[a];
      int j = a - 1;
      while (j >= 0 && key[j] > t) {
        key[j + 1] = key[j];
        j--;
      }
      key[j + 1] = t;
    }
    int w = 0;
    for (int a = 0; a < k; a++) {
      if (w > 0 && key[a] == key[w - 1]) continue;
      key[w++] = key[a];
    }
    for (int a = 0; a < w; a++) b[a] = (int32_t)(key[a] & 0xffffffffu);
    if (P.bcnt[c] > K.maxpc) atomicOr(&P.cnt->err, ERR_BUCKET);
    P.bcnt[c] = w;
    if (!all) P.cflag[c] &= ~1u;
  }
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::bin(const CaseK& K, const DevPtrs<R>& P, cudaStream_t st) {
  cudaMemsetAsync(P.bcnt, 0, sizeof(int32_t) * K.ncell, st);
  k_bin_scatter<D, R><<<grid_for(K.cap, BLK), BLK, 0, st>>>(K, P);
  k_bucket_fix<R><<<grid_for(K.ncell, BLK), BLK, 0, st>>>(K, P, 1);
}

/* ------------------------------------------------------------------ */
/* particle state in FP64 (exact order, mirrors the oracle)           */
/* ------------------------------------------------------------------ */
template <int D>
struct PState {
  static constexpr int U = D + 2, NS = U * D;
  double x[3], vol, mass, h, rho, rhov[3], E, c, P, tv[3], v[3];
  double sl[NS];
  int phase;
};

template <int D, typename R>
__device__ void load_state(const CaseK& K, const DevPtrs<R>& P, int64_t p, PState<D>& s) {
  constexpr int NS = PState<D>::NS;
  const R* X = P.X[P.xb];
  for (int d = 0; d < 3; d++) s.x[d] = (d < D) ? (double)X[d * K.cap + p] : 0.0;
  s.vol = (double)P.vol[p];
  s.mass = (double)P.mass[p];
  s.h = (double)P.H[P.hb][p];
  s.rho = (double)P.rho[p];
  for (int d = 0; d < 3; d++) s.rhov[d] = (d < D) ? (double)P.rhov[d * K.cap + p] : 0.0;
  s.E = (double)P.E[p];
  s.c = (double)P.c[p];
  s.P = (double)P.P[p];
  for (int d = 0; d < 3; d++) s.tv[d] = (d < D) ? (double)P.tv[d * K.cap + p] : 0.0;
  for (int d = 0; d < 3; d++) s.v[d] = (d < D) ? (double)P.v[d * K.cap + p] : 0.0;
  for (int t = 0; t < NS; t++) s.sl[t] = (double)P.sl[t * K.cap + p];
  s.phase = P.phase[p];
}

/* store; which = bitmask of groups (1 geometry, 2 fluid state, 4 v, 8 slopes) */
template <int D, typename R>
__device__ void store_state(const CaseK& K, const DevPtrs<R>& P, int64_t p, const PState<D>& s, int which) {
  constexpr int NS = PState<D>::NS;
  R* X = P.X[P.xb];
  if (which & 1) {
    for (int d = 0; d < D; d++) X[d * K.cap + p] = (R)s.x[d];
    P.vol[p] = (R)s.vol;
    P.mass[p] = (R)s.mass;
    P.H[P.hb][p] = (R)s.h;
  }
  if (which & 2) {
    P.rho[p] = (R)s.rho;
    for (int d = 0; d < D; d++) P.rhov[d * K.cap + p] = (R)s.rhov[d];
    P.E[p] = (R)s.E;
    P.c[p] = (R)s.c;
    P.P[p] = (R)s.P;
    for (int d = 0; d < D; d++) P.tv[d * K.cap + p] = (R)s.tv[d];
  }
  if (which & 4)
    for (int d = 0; d < D; d++) P.v[d * K.cap + p] = (R)s.v[d];
  if (which & 8)
    for (int t = 0; t < NS; t++) P.sl[t * K.cap + p] = (R)s.sl[t];
  P.phase[p] = (int8_t)s.phase;
}

template <int D>
__device__ __forceinline__ double sqnorm(const double* w) {
  double s = dmul(w[0], w[0]);
  for (int k = 1; k < D; k++) s = dadd(s, dmul(w[k], w[k]));
  return s;
}

/* tv = v = rhov/rho; P; c (particle.cpp:598-601) */
template <int D>
__device__ void eos_fill(const CaseK& K, PState<D>& s) {
  for (int d = 0; d < 3; d++) s.v[d] = ddiv(s.rhov[d], s.rho);
  for (int d = 0; d < 3; d++) s.tv[d] = s.v[d];
  int ph = s.phase - 1;
  double g = K.gamma[ph], pf = K.pinf[ph];
  double ei = dsub(s.E, dmul(dmul(0.5, s.rho), sqnorm<D>(s.v)));
  s.P = eos_p_x(ei, g, K.pinf_eos[ph]);
  s.c = dsqrt(ddiv(dmul(g, dadd(pf, s.P)), s.rho));
}

/* Set_split_ptcl (particle.cpp:575-609): child at x from parent s */
template <int D>
__device__ void set_split(const CaseK& K, const PState<D>& par, PState<D>& ch) {
  constexpr int U = D + 2;
  double dr[3];
  for (int d = 0; d < 3; d++) dr[d] = dsub(ch.x[d], par.x[d]);
  ch.phase = par.phase;
  ch.vol = (D == 3) ? ddiv(par.vol, 8.0) : ddiv(par.vol, 4.0);
  ch.mass = (D == 3) ? ddiv(par.mass, 8.0) : ddiv(par.mass, 4.0);
  ch.h = ddiv(par.h, 2.0);
  for (int t = 0; t < PState<D>::NS; t++) ch.sl[t] = par.sl[t];
  double acc = 0;
  for (int b = 0; b < D; b++) acc = (b == 0) ? dmul(par.sl[b], dr[b]) : dadd(acc, dmul(par.sl[b], dr[b]));
  ch.rho = dadd(par.rho, acc);
  for (int k = 0; k < 3; k++) ch.rhov[k] = 0.0;
  for (int k = 0; k < D; k++) {
    double ak = 0;
    for (int b = 0; b < D; b++)
      ak = (b == 0) ? dmul(par.sl[(1 + k) * D + b], dr[b]) : dadd(ak, dmul(par.sl[(1 + k) * D + b], dr[b]));
    ch.rhov[k] = dadd(par.rhov[k], ak);
  }
  double ae = 0;
  for (int b = 0; b < D; b++)
    ae = (b == 0) ? dmul(par.sl[(U - 1) * D + b], dr[b]) : dadd(ae, dmul(par.sl[(U - 1) * D + b], dr[b]));
  ch.E = dadd(par.E, ae);
  eos_fill<D>(K, ch);
}

/* ------------------------------------------------------------------ */
/* split                                                              */
/* ------------------------------------------------------------------ */
template <int D, typename R>
__global__ void k_split_flags(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)P.cnt->n_slots;
  const R* X = P.X[P.xb];
  GRID_STRIDE(p, n) {
    P.target[p] = -1;
    P.mflag[p] = 0;
    int8_t code = 0;
    if (P.phase[p] != 0) {
      double vol = (double)P.vol[p];
      double x0 = (double)X[p];
      bool f1 = vol > K.vol_max;
      bool f2 = false;
      if (!f1 && P.mark_in[p] == 1) {
        double dp = root_d(vol, D);
        f2 = dsub(x0, K.bl[0]) >= dp;
      }
      bool f3 = x0 > K.br[0];
      code = f1 ? 1 : (f2 ? 2 : (f3 ? 3 : 0));
      if (code == 3) atomicAdd(&P.cnt->step_new, 1ull); /* outlet count (step_new reused) */
      if (code) atomicAdd(&P.cnt->split_events, 1ull);
    }
    P.evcode[p] = code;
    P.scan[p] = (code == 1) ? (1ull << 32) : (code == 2 ? 1ull : 0ull);
  }
}

/* the split's event sweeps cover all slots, or none when no particle has an
 * event (split, inlet or outlet) this step */
template <typename R>
__global__ void k_split_begin(DevPtrs<R> P) {
  P.cnt->split_events = 0;
}
template <typename R>
__global__ void k_split_gate(DevPtrs<R> P) {
  DevCounters* c = P.cnt;
  c->split_n = c->split_events ? c->n_slots : 0ull;
}

template <int D, typename R>
__global__ void k_split_emit(CaseK K, DevPtrs<R> P) {
  constexpr int CN = (D == 3) ? 8 : 4;
  const int64_t n = (int64_t)P.cnt->split_n;
  const unsigned long long tot = P.scan_blk[scan_nblk(K.cap)];
  const int64_t nsplit = (int64_t)(tot >> 32), ninlet = (int64_t)(tot & 0xffffffffull);
  if (n + (CN - 1) * nsplit + ninlet > K.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&P.cnt->err, ERR_CAPACITY);
    return;
  }
  const unsigned long long seq0 = P.cnt->seq_next;
  GRID_STRIDE(p, n) {
    int code = P.evcode[p];
    if (code == 0) continue;
    if (code == 3) {
      /* outlet: Remove_particle from its list; the slot becomes a tombstone */
      mark_dirty(P, P.lcell[p]);
      P.lcell[p] = -1;
      P.phase[p] = 0;
      continue;
    }
    const unsigned long long sv = P.scan[p];
    const int64_t rs = (int64_t)(sv >> 32), ri = (int64_t)(sv & 0xffffffffull);
    const int64_t cbase = n + (CN - 1) * rs + ri;
    PState<D> par;
    load_state<D>(K, P, p, par);
    double dp = root_d(par.vol, D);
    if (code == 1) {
      double pref[3] = {dsub(par.x[0], ddiv(dp, 4.)), dsub(par.x[1], ddiv(dp, 4.)),
                        (D == 3) ? dsub(par.x[2], ddiv(dp, 4.)) : 0.0};
      const int64_t old_cell = P.lcell[p];
      mark_dirty(P, old_cell);
      PState<D> last;
      int ci = 0;
      for (int a0 = 0; a0 < 2; ++a0)
        for (int a1 = 0; a1 < 2; ++a1)
          for (int a2 = 0; a2 < (D == 3 ? 2 : 1); ++a2, ++ci) {
            PState<D> ch;
            ch.x[0] = dadd(pref[0], dmul(ddiv(dp, 2.), (double)a0));
            ch.x[1] = dadd(pref[1], dmul(ddiv(dp, 2.), (double)a1));
            ch.x[2] = (D == 3) ? dadd(pref[2], dmul(ddiv(dp, 2.), (double)a2)) : 0.0;
            set_split<D>(K, par, ch);
            if (ci == CN - 1) {
              last = ch;
              continue;
            }
            int64_t q = cbase + ci;
            store_state<D, R>(K, P, q, ch, 1 | 2 | 4 | 8);
            P.mark_in[q] = 0;
            P.seq[q] = seq0 + (unsigned long long)(cbase - n + ci);
            P.list_len[q] = -1;
            P.target[q] = -1;
            P.mflag[q] = 0;
            P.evcode[q] = 0;
            P.aff[q] = 1;
            int pos[3];
            cell_pos_exact<D>(K, ch.x, pos);
            int64_t c = cidx<D>(K, pos);
            P.lcell[q] = (int32_t)c;
            P.lkey[q] = KEY_APPEND + (uint32_t)(CN * rs + 1 + ci);
            bucket_append(K, P, c, q);
            mark_dirty(P, c);
            flag_cells<D>(K, P, pos);
          }
      /* Copy_split_state (particle.cpp:667-691): the parent takes the last
       * child's state except v */
      PState<D> np = last;
      for (int d = 0; d < 3; d++) np.v[d] = par.v[d];
      store_state<D, R>(K, P, p, np, 1 | 2);
      int pos[3];
      cell_pos_exact<D>(K, np.x, pos);
      int64_t c = cidx<D>(K, pos);
      P.lcell[p] = (int32_t)c;
      P.lkey[p] = KEY_APPEND + (uint32_t)(CN * rs);
      bucket_append(K, P, c, p);
      mark_dirty(P, c);
      P.aff[p] = 1;
      flag_cells<D>(K, P, pos);
    } else {
      /* inlet (f2): clone at x - dp, Set_ptcl (particle.cpp:696-722) */
      PState<D> ch = par;
      ch.x[0] = dsub(par.x[0], dp);
      eos_fill<D>(K, ch);
      int64_t q = cbase;
      store_state<D, R>(K, P, q, ch, 1 | 2 | 4 | 8);
      P.mark_in[q] = 0;
      P.seq[q] = seq0 + (unsigned long long)(cbase - n);
      P.list_len[q] = -1;
      P.target[q] = -1;
      P.mflag[q] = 0;
      P.evcode[q] = 0;
      P.aff[q] = 1;
      int pos[3];
      cell_pos_exact<D>(K, ch.x, pos);
      int64_t c = cidx<D>(K, pos);
      P.lcell[q] = (int32_t)c;
      P.lkey[q] = KEY_APPEND + (uint32_t)(CN * nsplit + ri);
      bucket_append(K, P, c, q);
      mark_dirty(P, c);
      flag_cells<D>(K, P, pos);
    }
  }
}

template <int D, typename R>
__global__ void k_split_finish(CaseK K, DevPtrs<R> P) {
  constexpr int CN = (D == 3) ? 8 : 4;
  const unsigned long long tot = P.scan_blk[scan_nblk(K.cap)];
  const unsigned long long nsplit = tot >> 32, ninlet = tot & 0xffffffffull;
  DevCounters* c = P.cnt;
  if (c->err & ERR_CAPACITY) return;
  unsigned long long nout = c->step_new;
  unsigned long long nnew = (CN - 1) * nsplit + ninlet;
  c->n_slots += nnew;
  c->seq_next += nnew;
  c->n_live = c->n_live + nnew - nout;
  c->append_next = CN * nsplit + ninlet;
  c->n_split += nsplit;
  c->n_inlet += ninlet;
  c->n_outlet += nout;
  c->step_new = 0;
}

/* old neighbours of split parents (code 1) and outlet particles (code 3) */
template <typename R>
__global__ void k_aff_oldnbr_split(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)P.cnt->split_n;
  GRID_STRIDE(p, n) {
    int code = P.evcode[p];
    if (code != 1 && code != 3) continue;
    int32_t len = P.list_len[p];
    if (len < 0) {
      atomicOr(&P.cnt->err, ERR_NOLIST);
      continue;
    }
    const int32_t* L = P.arena + P.list_off[p];
    for (int32_t e = 0; e < len; e++) {
      int32_t q = L[e];
      if (q >= 0 && P.phase[q] != 0) P.aff[q] = 1;
    }
  }
}

template <typename R>
__global__ void k_aff_cells(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)min(P.cnt->n_flagged, (unsigned long long)P.qcap);
  GRID_STRIDE(i, n) {
    int64_t c = P.flag_q[i];
    int m = min(P.bcnt[c], K.maxpc);
    for (int r = 0; r < m; r++) P.aff[P.bucket[c * K.maxpc + r]] = 1;
    P.cflag[c] &= ~2u;
  }
}

/* Refresh_neighbor_info(3) for affected particles: dist <= 2 p_sz within +-2 cells
 * (level_infor.cpp:161-188); stored fluid entries in list order */
template <int D, typename R>
__global__ void k_refresh3(CaseK K, DevPtrs<R> P, const unsigned long long* np) {
  const int64_t n = (int64_t)*np;
  const R* X = P.X[P.xb];
  const double lim = dmul(K.p_sz, 2.);
  const float lo2 = (float)(lim * lim * (1.0 - 1e-5)), hi2 = (float)(lim * lim * (1.0 + 1e-5));
  GRID_STRIDE(p, n) {
    if (!P.aff[p]) continue;
    P.aff[p] = 0;
    if (P.phase[p] == 0) continue;
    atomicAdd(&P.cnt->n_affected, 1ull);
    R xr[3];
    load_x<D>(K, X, p, xr);
    double xp[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) xp[d] = (double)xr[d];
    int pos[3];
    cell_pos_exact<D>(K, xp, pos);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      int r = (d < D) ? 2 : 0;
      lo[d] = max(pos[d] - r, 0);
      hi[d] = min(pos[d] + r, (d < D ? K.N[d] : 1) - 1);
    }
    int64_t base = 0;
    int32_t cntv = 0;
    for (int pass = 0; pass < 2; pass++) {
      if (pass == 1) {
        unsigned long long b = atomicAdd(&P.cnt->arena_used, (unsigned long long)cntv);
        if ((int64_t)(b + cntv) > K.arena_cap) {
          atomicOr(&P.cnt->err, ERR_ARENA);
          P.list_len[p] = -1;
          break;
        }
        base = (int64_t)b;
        P.list_off[p] = base;
        P.list_len[p] = cntv;
      }
      int32_t w = 0;
      for (int t = lo[0]; t <= hi[0]; t++)
        for (int s = lo[1]; s <= hi[1]; s++)
          for (int m = lo[2]; m <= hi[2]; m++) {
            int q3[3] = {t, s, m};
            int64_t c = cidx<D>(K, q3);
            int mm = min(P.bcnt[c], K.maxpc);
            const int32_t* bk = P.bucket + c * K.maxpc;
            for (int r = 0; r < mm; r++) {
              int32_t q = bk[r];
              bool in;
              if (sizeof(R) == 4) {
                float dd = 0.f;
                for (int d = 0; d < D; d++) {
                  float t2 = (float)(xr[d] - X[d * K.cap + q]);
                  dd += t2 * t2;
                }
                if (dd < lo2) in = true;
                else if (dd > hi2) in = false;
                else {
                  double xq[3] = {0, 0, 0};
                  for (int d = 0; d < D; d++) xq[d] = (double)X[d * K.cap + q];
                  in = dist_exact<D>(xp, xq) <= lim;
                }
              } else {
                double xq[3] = {0, 0, 0};
                for (int d = 0; d < D; d++) xq[d] = (double)X[d * K.cap + q];
                in = dist_exact<D>(xp, xq) <= lim;
              }
              if (in) {
                if (pass == 1) P.arena[base + w] = q;
                w++;
              }
            }
          }
      cntv = w;
    }
  }
}

/* mark_in = (x - box_l.x < vol^(1/DIM)) (mpm.cpp:1398-1399).  events (may be
 * NULL): the event count of the merge pass just run; with no merge nothing
 * mark_in depends on has changed since the last evaluation and the kernel
 * returns at once.  The FP32 path decides in FP32 when x - box_l is more than
 * 0.1% away from vol^(1/DIM) (far beyond the rounding of either side) and
 * evaluates the rest exactly, as the FP64 path does. */
template <int D, typename R>
__global__ void k_mark_in(CaseK K, DevPtrs<R> P, const unsigned long long* events) {
  if (events && *events == 0) return;
  const int64_t n = (int64_t)P.cnt->n_slots;
  const R* X = P.X[P.xb];
  const float blf = (float)K.bl[0];
  GRID_STRIDE(p, n) {
    if (P.phase[p] == 0) continue;
    if constexpr (sizeof(R) == 4) {
      const float af = (float)X[p] - blf;
      const float rf = (D == 2) ? sqrtf((float)P.vol[p]) : cbrtf((float)P.vol[p]);
      if (af > rf * 1.001f) {
        P.mark_in[p] = 0;
        continue;
      }
      if (af < rf * 0.999f) {
        P.mark_in[p] = 1;
        continue;
      }
    }
    double a = dsub((double)X[p], K.bl[0]);
    double vol = (double)P.vol[p];
    double ra = (D == 2) ? sqrt(vol) : cbrt(vol);
    int8_t m;
    if (a > ra * 1.0001) m = 0;
    else if (a < ra * 0.9999) m = 1;
    else m = (a < root_d(vol, D)) ? 1 : 0;
    P.mark_in[p] = m;
  }
}

template <typename R>
__global__ void k_reset_queues(DevPtrs<R> P) {
  P.cnt->n_dirty = 0;
  P.cnt->n_flagged = 0;
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::split(const CaseK& K, const DevPtrs<R>& P, cudaStream_t st) {
  const int g = grid_for(K.cap, BLK);
  k_split_begin<R><<<1, 1, 0, st>>>(P);
  k_split_flags<D, R><<<g, BLK, 0, st>>>(K, P);
  k_split_gate<R><<<1, 1, 0, st>>>(P);
  scan_u64(P.scan, P.scan_blk, &P.cnt->split_n, K.cap, st);
  k_aff_oldnbr_split<R><<<g, BLK, 0, st>>>(K, P);
  k_split_emit<D, R><<<g, BLK, 0, st>>>(K, P);
  k_split_finish<D, R><<<1, 1, 0, st>>>(K, P);
  k_bucket_fix<R><<<grid_for(P.qcap, BLK), BLK, 0, st>>>(K, P, 0);
  k_aff_cells<R><<<grid_for(P.qcap, BLK), BLK, 0, st>>>(K, P);
  k_refresh3<D, R><<<g, BLK, 0, st>>>(K, P, &P.cnt->n_slots);
  k_mark_in<D, R><<<g, BLK, 0, st>>>(K, P, nullptr);
  k_reset_queues<R><<<1, 1, 0, st>>>(P);
}

/* ------------------------------------------------------------------ */
/* merge (one pass of Merge_particle_fast)                            */
/* ------------------------------------------------------------------ */
/* particles a merge pass sweeps: all slots, or none when the pass follows a
 * pass of the same sequence that merged nothing (the state is then unchanged,
 * so this pass would recompute the same partners and merge nothing too) */
template <typename R>
__global__ void k_merge_begin(DevPtrs<R> P, int chained) {
  DevCounters* c = P.cnt;
  c->merge_n = (chained && c->merge_quiet) ? 0ull : c->n_slots;
}

template <int D, typename R>
__global__ void k_merge_a(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)P.cnt->merge_n;
  const R* X = P.X[P.xb];
  GRID_STRIDE(p, n) {
    P.target[p] = -1;
    P.mflag[p] = 0;
    if (P.phase[p] == 0) continue;
    double vol = (double)P.vol[p];
    if (!(vol < K.vol_min)) continue;
    int32_t len = P.list_len[p];
    if (len < 0) {
      atomicOr(&P.cnt->err, ERR_NOLIST);
      continue;
    }
    double xp[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) xp[d] = (double)X[d * K.cap + p];
    const int ph = P.phase[p];
    double dss = K.dss0;
    int32_t cp1 = -1;
    const int32_t* L = P.arena + P.list_off[p];
    for (int32_t e = 0; e < len; e++) {
      int32_t q = L[e];
      if (q < 0 || q == p) continue;
      if (P.phase[q] != ph) continue;  /* also skips tombstones (phase 0) */
      double qvol = (double)P.vol[q];
      double xq[3] = {0, 0, 0};
      for (int d = 0; d < D; d++) xq[d] = (double)X[d * K.cap + q];
      double dist = dist_exact<D>(xp, xq);
      if (qvol < K.vol_min && dist < dss) {
        dss = dist;
        cp1 = q;
      }
    }
    P.target[p] = cp1;
  }
}

template <int D, typename R>
__global__ void k_merge_b(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)P.cnt->merge_n;
  GRID_STRIDE(p, n) {
    unsigned long long s = 0;
    int32_t q = P.target[p];
    if (q >= 0 && q > p && P.target[q] == (int32_t)p) {
      P.mflag[p] = 1;
      P.mflag[q] = 2;
      s = 1;
    }
    P.scan[p] = s;
  }
}

/* Set_merge_ptcl (particle.cpp:614-661) + list fix-up (mpm.cpp:1637-1669) */
template <int D, typename R>
__global__ void k_merge_c(CaseK K, DevPtrs<R> P) {
  constexpr int NS = PState<D>::NS;
  const int64_t n = (int64_t)P.cnt->merge_n;
  const unsigned long long app = P.cnt->append_next;
  GRID_STRIDE(p, n) {
    if (P.mflag[p] != 1) continue;
    int32_t q = P.target[p];
    mark_dirty(P, P.lcell[p]);
    mark_dirty(P, P.lcell[q]);
    PState<D> a, b;
    load_state<D>(K, P, p, a);
    load_state<D>(K, P, q, b);
    PState<D> m = a;
    double v0 = a.vol, v1 = b.vol;
    m.mass = dadd(a.mass, b.mass);
    m.vol = dadd(v0, v1);
    double vv = m.vol;
    m.h = ddiv(dmul(root_d(vv, D), CELL_RATIO), CUT_OFF);
    for (int d = 0; d < 3; d++) m.x[d] = (d < D) ? ddiv(dadd(dmul(a.x[d], v0), dmul(b.x[d], v1)), vv) : 0.0;
    for (int t = 0; t < NS; t++) m.sl[t] = ddiv(dadd(dmul(a.sl[t], v0), dmul(b.sl[t], v1)), vv);
    m.rho = ddiv(dadd(dmul(a.rho, v0), dmul(b.rho, v1)), vv);
    for (int k = 0; k < D; k++) m.rhov[k] = ddiv(dadd(dmul(a.rhov[k], v0), dmul(b.rhov[k], v1)), vv);
    m.E = ddiv(dadd(dmul(a.E, v0), dmul(b.E, v1)), vv);
    eos_fill<D>(K, m);
    store_state<D, R>(K, P, p, m, 1 | 2 | 4 | 8);
    /* partner removed */
    P.phase[q] = 0;
    P.lcell[q] = -1;
    int pos[3];
    cell_pos_exact<D>(K, m.x, pos);
    int64_t c = cidx<D>(K, pos);
    P.lcell[p] = (int32_t)c;
    P.lkey[p] = KEY_APPEND + (uint32_t)(app + P.scan[p]);
    bucket_append(K, P, c, p);
    mark_dirty(P, c);
    P.aff[p] = 1;
    flag_cells<D>(K, P, pos);
  }
}

template <typename R>
__global__ void k_aff_oldnbr_merge(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)P.cnt->merge_n;
  GRID_STRIDE(p, n) {
    if (P.mflag[p] != 1) continue;
    int32_t q = P.target[p];
    for (int w = 0; w < 2; w++) {
      int64_t o = w ? q : p;
      int32_t len = P.list_len[o];
      if (len < 0) {
        atomicOr(&P.cnt->err, ERR_NOLIST);
        continue;
      }
      const int32_t* L = P.arena + P.list_off[o];
      for (int32_t e = 0; e < len; e++) {
        int32_t r = L[e];
        if (r < 0 || r == p || r == q) continue;
        if (P.mflag[r] == 2 || P.phase[r] == 0) continue;
        P.aff[r] = 1;
      }
    }
  }
}

template <int D, typename R>
__global__ void k_merge_finish(CaseK K, DevPtrs<R> P) {
  const unsigned long long ns = P.scan_blk[scan_nblk(K.cap)];
  DevCounters* c = P.cnt;
  c->append_next += ns;
  c->n_live -= ns;
  c->n_merge += ns;
  c->merge_quiet = ns == 0 ? 1ull : 0ull;
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::merge(const CaseK& K, const DevPtrs<R>& P, bool chained, cudaStream_t st) {
  const int g = grid_for(K.cap, BLK);
  k_merge_begin<R><<<1, 1, 0, st>>>(P, chained ? 1 : 0);
  k_merge_a<D, R><<<g, BLK, 0, st>>>(K, P);
  k_merge_b<D, R><<<g, BLK, 0, st>>>(K, P);
  scan_u64(P.scan, P.scan_blk, &P.cnt->merge_n, K.cap, st);
  k_aff_oldnbr_merge<R><<<g, BLK, 0, st>>>(K, P);
  k_merge_c<D, R><<<g, BLK, 0, st>>>(K, P);
  k_merge_finish<D, R><<<1, 1, 0, st>>>(K, P);
  k_bucket_fix<R><<<grid_for(P.qcap, BLK), BLK, 0, st>>>(K, P, 0);
  k_aff_cells<R><<<grid_for(P.qcap, BLK), BLK, 0, st>>>(K, P);
  k_refresh3<D, R><<<g, BLK, 0, st>>>(K, P, &P.cnt->merge_n);
  /* the pass's merge count is still the scan total */
  k_mark_in<D, R><<<g, BLK, 0, st>>>(K, P, P.scan_blk + scan_nblk(K.cap));
  k_reset_queues<R><<<1, 1, 0, st>>>(P);
}

/* ------------------------------------------------------------------ */
/* stored lists after the second stage (the lists split/merge read    */
/* next step): Refresh_neighbor_info(2) membership, dist <= 2 h, from */
/* the stage-start coordinates, kept only for particles that can      */
/* split (vol > vol_max), merge (vol < vol_min) or leave (x > box_r)  */
/* ------------------------------------------------------------------ */
template <typename R>
__global__ void k_arena_reset(DevPtrs<R> P) { P.cnt->arena_used = 0; }

template <int D, typename R>
__global__ void k_store_lists(CaseK K, DevPtrs<R> P, int xs_b, int hs_b, int xn_b) {
  const int64_t n = (int64_t)P.cnt->n_slots;
  const R* XS = P.X[xs_b];
  const R* XN = P.X[xn_b];
  const R* HS = P.H[hs_b];
  GRID_STRIDE(p, n) {
    if (P.phase[p] == 0) continue;
    double vol = (double)P.vol[p];
    bool cand = vol > K.vol_max || vol < K.vol_min || (double)XN[p] > K.br[0];
    if (!cand) {
      P.list_len[p] = -1;
      continue;
    }
    R xr[3];
    load_x<D>(K, XS, p, xr);
    double xp[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) xp[d] = (double)xr[d];
    const double lim = dmul((double)HS[p], CUT_OFF);
    const float lo2 = (float)(lim * lim * (1.0 - 1e-5)), hi2 = (float)(lim * lim * (1.0 + 1e-5));
    int pos[3];
    cell_pos<D, R>(K, xr, pos);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      int r = (d < D) ? K.rad2 : 0;
      lo[d] = max(pos[d] - r, 0);
      hi[d] = min(pos[d] + r, (d < D ? K.N[d] : 1) - 1);
    }
    int64_t base = 0;
    int32_t cntv = 0;
    for (int pass = 0; pass < 2; pass++) {
      if (pass == 1) {
        unsigned long long b = atomicAdd(&P.cnt->arena_used, (unsigned long long)cntv);
        if ((int64_t)(b + cntv) > K.arena_cap) {
          atomicOr(&P.cnt->err, ERR_ARENA);
          P.list_len[p] = -1;
          break;
        }
        base = (int64_t)b;
        P.list_off[p] = base;
        P.list_len[p] = cntv;
      }
      int32_t w = 0;
      for (int t = lo[0]; t <= hi[0]; t++)
        for (int s = lo[1]; s <= hi[1]; s++)
          for (int m = lo[2]; m <= hi[2]; m++) {
            int q3[3] = {t, s, m};
            int64_t c = cidx<D>(K, q3);
            int mm = min(P.bcnt[c], K.maxpc);
            const int32_t* bk = P.bucket + c * K.maxpc;
            for (int r = 0; r < mm; r++) {
              int32_t q = bk[r];
              bool in;
              float dd = 0.f;
              for (int d = 0; d < D; d++) {
                float t2 = (float)(xr[d] - XS[d * K.cap + q]);
                dd += t2 * t2;
              }
              if (dd < lo2) in = true;
              else if (dd > hi2) in = false;
              else {
                double xq[3] = {0, 0, 0};
                for (int d = 0; d < D; d++) xq[d] = (double)XS[d * K.cap + q];
                in = dist_exact<D>(xp, xq) <= lim;
              }
              if (in) {
                if (pass == 1) P.arena[base + w] = q;
                w++;
              }
            }
          }
      cntv = w;
    }
  }
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::store_lists(const CaseK& K, const DevPtrs<R>& P, int xs, int hs, int xn, cudaStream_t st) {
  k_arena_reset<R><<<1, 1, 0, st>>>(P);
  k_store_lists<D, R><<<grid_for(K.cap, BLK), BLK, 0, st>>>(K, P, xs, hs, xn);
}

template <typename R>
__global__ void k_reset_lists(CaseK K, DevPtrs<R> P) {
  const int64_t n = (int64_t)P.cnt->n_slots;
  GRID_STRIDE(p, n) P.list_len[p] = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) P.cnt->arena_used = 0;
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::reset_lists(const CaseK& K, const DevPtrs<R>& P, cudaStream_t st) {
  k_reset_lists<R><<<grid_for(K.cap, BLK), BLK, 0, st>>>(K, P);
}

#define PGDG_INST(D, R, EX)                                                          \
  template void Launch<D, R, EX>::bin(const CaseK&, const DevPtrs<R>&, cudaStream_t);  \
  template void Launch<D, R, EX>::split(const CaseK&, const DevPtrs<R>&, cudaStream_t); \
  template void Launch<D, R, EX>::merge(const CaseK&, const DevPtrs<R>&, bool, cudaStream_t); \
  template void Launch<D, R, EX>::store_lists(const CaseK&, const DevPtrs<R>&, int, int, int, cudaStream_t); \
  template void Launch<D, R, EX>::reset_lists(const CaseK&, const DevPtrs<R>&, cudaStream_t);
PGDG_INST(2, double, false)
#if PGDG_WITH_3D
PGDG_INST(3, double, false)
#endif
PGDG_INST(2, float, false)
#if PGDG_WITH_3D
PGDG_INST(3, float, false)
#endif
PGDG_INST(2, double, true)
#if PGDG_WITH_3D
PGDG_INST(3, double, true)
#endif

}  // namespace pgdg
