/*
 * k_grid.cu -- grid kernels of the step: Used_state_update, Set_timestep,
 * MLS_P2G, Calculate_limiter, Grid_acceleration (DG volume + face residual with
 * the MGFM ghost state), Update_grid and the conservation totals.
 *
 * One thread per cell; cell fields are component-major (field[t * ncell + ci])
 * so a warp's loads of one field are coalesced.  R is float (mixed precision) or
 * double (plain FP64 path); the MGFM Newton solve and the P2G moment sums are
 * FP64 in both.
 */
#include "pgdg_dev.cuh"

namespace pgdg {

constexpr int BLK = 256;
#define GRID_STRIDE(i, n) for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
                               i += (int64_t)gridDim.x * blockDim.x)

template <int D>
__device__ __forceinline__ void cijk(const CaseK& K, int64_t ci, int* idx) {
  idx[2] = (int)(ci % K.N[2]);
  idx[1] = (int)((ci / K.N[2]) % K.N[1]);
  idx[0] = (int)(ci / ((int64_t)K.N[1] * K.N[2]));
}
__device__ __forceinline__ int64_t cidx3(const CaseK& K, int i, int j, int k) {
  return ((int64_t)i * K.N[1] + j) * K.N[2] + k;
}
/* cell centre box_l + p_size (idx + 0.5) (mpm_ini.cpp:305-311) */
template <int D>
__device__ __forceinline__ void center(const CaseK& K, const int* idx, double* xc) {
  for (int d = 0; d < 3; d++) xc[d] = (d < D) ? K.bl[d] + K.ps[d] * (idx[d] + 0.5) : 0.0;
}

/* Cell_dg face f (mpm_ini.cpp:447-545): order yL, xR, yR, xL, zL, zR */
struct FaceK {
  int axis;       /* normal axis */
  double sgn;     /* normal = sgn e_axis */
  double cen[3], t0[3], t1[3], S;
  int bound;
  int nb[3];
};
template <int D>
__device__ __forceinline__ void face(const CaseK& K, const int* idx, const double* xc, int f, FaceK& fc) {
  const double px = K.ps[0], py = K.ps[1], pz = K.ps[2];
  for (int d = 0; d < 3; d++) { fc.cen[d] = xc[d]; fc.t0[d] = 0; fc.t1[d] = 0; fc.nb[d] = idx[d]; }
  int side;
  switch (f) {
    case 0: fc.axis = 1; fc.sgn = -1; fc.t0[0] = 0.5 * px; fc.t1[2] = 0.5 * pz; fc.cen[1] = xc[1] - 0.5 * py;
      fc.S = (D == 3) ? px * pz : px; fc.nb[1] -= 1; side = 2; break;
    case 1: fc.axis = 0; fc.sgn = 1; fc.t0[1] = 0.5 * py; fc.t1[2] = 0.5 * pz; fc.cen[0] = xc[0] + 0.5 * px;
      fc.S = (D == 3) ? py * pz : py; fc.nb[0] += 1; side = 1; break;
    case 2: fc.axis = 1; fc.sgn = 1; fc.t0[0] = -0.5 * px; fc.t1[2] = 0.5 * pz; fc.cen[1] = xc[1] + 0.5 * py;
      fc.S = (D == 3) ? px * pz : px; fc.nb[1] += 1; side = 3; break;
    case 3: fc.axis = 0; fc.sgn = -1; fc.t0[1] = -0.5 * py; fc.t1[2] = 0.5 * pz; fc.cen[0] = xc[0] - 0.5 * px;
      fc.S = (D == 3) ? py * pz : py; fc.nb[0] -= 1; side = 0; break;
    case 4: fc.axis = 2; fc.sgn = -1; fc.t0[0] = 0.5 * px; fc.t1[1] = 0.5 * py; fc.cen[2] = xc[2] - 0.5 * pz;
      fc.S = py * px; fc.nb[2] -= 1; side = 4; break;
    default: fc.axis = 2; fc.sgn = 1; fc.t0[0] = 0.5 * px; fc.t1[1] = 0.5 * py; fc.cen[2] = xc[2] + 0.5 * pz;
      fc.S = py * px; fc.nb[2] += 1; side = 5; break;
  }
  if (D == 2) fc.t1[2] = 0;
  bool inside = true;
  for (int d = 0; d < D; d++) inside = inside && fc.nb[d] >= 0 && fc.nb[d] < K.N[d];
  fc.bound = inside ? 0 : K.bc[side];
}

/* The same face in the stage type R relative to the cell centre, for the
 * non-exact paths: centre offset, tangent half-vectors and area come from the
 * half cell sizes hps (no absolute coordinates, no FP64 arithmetic); Sax[a] is
 * the area of a face normal to axis a. */
template <typename R>
struct FaceRel {
  int axis, bound, nb[3];
  R sgn, cen[3], t0[3], t1[3], S;
};
template <int D, typename R>
__device__ __forceinline__ void face_rel(const CaseK& K, const int* idx, const R* hps, const R* Sax, int f,
                                         FaceRel<R>& fc) {
  for (int d = 0; d < 3; d++) {
    fc.cen[d] = fc.t0[d] = fc.t1[d] = R(0);
    fc.nb[d] = idx[d];
  }
  int side;
  switch (f) {
    case 0: fc.axis = 1; fc.sgn = R(-1); fc.t0[0] = hps[0]; fc.t1[2] = hps[2]; fc.cen[1] = -hps[1]; fc.nb[1] -= 1; side = 2; break;
    case 1: fc.axis = 0; fc.sgn = R(1); fc.t0[1] = hps[1]; fc.t1[2] = hps[2]; fc.cen[0] = hps[0]; fc.nb[0] += 1; side = 1; break;
    case 2: fc.axis = 1; fc.sgn = R(1); fc.t0[0] = -hps[0]; fc.t1[2] = hps[2]; fc.cen[1] = hps[1]; fc.nb[1] += 1; side = 3; break;
    case 3: fc.axis = 0; fc.sgn = R(-1); fc.t0[1] = -hps[1]; fc.t1[2] = hps[2]; fc.cen[0] = -hps[0]; fc.nb[0] -= 1; side = 0; break;
    case 4: fc.axis = 2; fc.sgn = R(-1); fc.t0[0] = hps[0]; fc.t1[1] = hps[1]; fc.cen[2] = -hps[2]; fc.nb[2] -= 1; side = 4; break;
    default: fc.axis = 2; fc.sgn = R(1); fc.t0[0] = hps[0]; fc.t1[1] = hps[1]; fc.cen[2] = hps[2]; fc.nb[2] += 1; side = 5; break;
  }
  if (D == 2) fc.t1[2] = R(0);
  fc.S = Sax[fc.axis];
  bool inside = true;
  for (int d = 0; d < D; d++) inside = inside && fc.nb[d] >= 0 && fc.nb[d] < K.N[d];
  fc.bound = inside ? 0 : K.bc[side];
}
/* half cell sizes and face areas in R */
template <int D, typename R>
__device__ __forceinline__ void cell_geom(const CaseK& K, R* hps, R* Sax) {
  for (int d = 0; d < 3; d++) hps[d] = (R)(0.5 * K.ps[d]);
  if (D == 3) {
    Sax[0] = (R)(K.ps[1] * K.ps[2]);
    Sax[1] = (R)(K.ps[0] * K.ps[2]);
    Sax[2] = (R)(K.ps[1] * K.ps[0]);
  } else {
    Sax[0] = (R)K.ps[1];
    Sax[1] = (R)K.ps[0];
    Sax[2] = R(0);
  }
}

/* ------------------------------------------------------------------ */
/* Used_state_update (mpm.cpp:184-263)                                */
/* ------------------------------------------------------------------ */
template <int D, typename R, bool EX>
__global__ void k_used_mark(CaseK K, DevPtrs<R> P, int8_t* tmp) {
  const int64_t nc = K.ncell;
  GRID_STRIDE(ci, nc) {
    if (!(P.cph[ci] == 1 || P.cph[nc + ci] == 1)) continue;
    int idx[3];
    cijk<D>(K, ci, idx);
    const int Ib[3] = {5, 5, D == 3 ? 5 : 0};
    for (int t = max(idx[0] - Ib[0], 0); t <= min(idx[0] + Ib[0], K.N[0] - 1); t++)
      for (int s = max(idx[1] - Ib[1], 0); s <= min(idx[1] + Ib[1], K.N[1] - 1); s++)
        for (int q = max(idx[2] - Ib[2], 0); q <= min(idx[2] + Ib[2], K.N[2] - 1); q++) tmp[cidx3(K, t, s, q)] = 1;
  }
}
template <int D, typename R, bool EX>
void Launch<D, R, EX>::used_state(const CaseK& K, const DevPtrs<R>& P, cudaStream_t st) {
  cudaMemsetAsync(P.cused, 0, K.ncell, st);
  k_used_mark<D, R, EX><<<grid_for(K.ncell, BLK), BLK, 0, st>>>(K, P, P.cused);
}

/* ------------------------------------------------------------------ */
/* Set_timestep (mpm.cpp:19-57, particle.cpp:554-569)                 */
/* ------------------------------------------------------------------ */
template <typename T>
__device__ __forceinline__ T warp_min(T v) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <typename R, bool EX>
__global__ void k_dt_init(DevPtrs<R> P) {
  P.cnt->dt_bits = (unsigned long long)__double_as_longlong(1.e20);
  P.cnt->maxv_bits = 0ull;
}

template <int D, typename R, bool EX>
__global__ void k_dt_reduce(CaseK K, DevPtrs<R> P, int by_cells) {
  double tmin = 1.e20, vmax = 0.0;
  if (by_cells) {
    const int64_t nc = K.ncell;
    const R hh = R(CELL_RATIO / CUT_OFF * K.p_sz);
    const R ds = hh / R(CELL_RATIO) * R(CUT_OFF);
    GRID_STRIDE(ci, nc) {
      if (!P.cused[ci]) continue;
      R sq = P.cv[ci] * P.cv[ci];
      for (int k = 1; k < D; k++) sq = sq + P.cv[k * nc + ci] * P.cv[k * nc + ci];
      R U = sqrt_r<R>(sq);
      R c12 = amax1(P.cc[ci], P.cc[nc + ci]);
      R a12 = amax1(P.cac[ci], P.cac[nc + ci]);
      R t = R(K.cfl) * ds / (c12 + U);
      R tmp = R(K.cfl) * sqrt_r<R>(ds / a12);
      t = amin1(t, tmp);
      tmin = fmin(tmin, (double)t);
      vmax = fmax(vmax, (double)U);
    }
  } else {
    const int64_t n = (int64_t)P.cnt->n_slots;
    const R* H = P.H[P.hb];
    GRID_STRIDE(p, n) {
      if (P.phase[p] == 0) continue;
      R sq = P.v[p] * P.v[p];
      for (int k = 1; k < D; k++) sq = sq + P.v[k * K.cap + p] * P.v[k * K.cap + p];
      R U = sqrt_r<R>(sq);
      R ds = H[p] / R(CELL_RATIO) * R(CUT_OFF);
      R c12 = amax1(P.c[p], R(0));
      R t = R(K.cfl) * ds / (c12 + U);
      tmin = fmin(tmin, (double)t);
      vmax = fmax(vmax, (double)U);
    }
  }
  tmin = warp_min(tmin);
  vmax = warp_max(vmax);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&P.cnt->dt_bits, (unsigned long long)__double_as_longlong(tmin));
    atomicMax(&P.cnt->maxv_bits, (unsigned long long)__double_as_longlong(vmax));
  }
}

template <typename R, bool EX>
__global__ void k_dt_final(DevPtrs<R> P) {
  P.cnt->dt = __longlong_as_double((long long)P.cnt->dt_bits);
  P.cnt->max_v = __longlong_as_double((long long)P.cnt->maxv_bits);
  /* no cell or particle gave a finite step (e.g. cells uploaded with zero
   * sound speed while the iteration count selects the cell-based step) */
  if (!(P.cnt->dt < 1.e19)) atomicOr(&P.cnt->err, ERR_DT);
}

template <typename R, bool EX>
__global__ void k_add_time(DevPtrs<R> P) {
  P.cnt->time += P.cnt->dt;
}
template <int D, typename R, bool EX>
void Launch<D, R, EX>::add_time(const DevPtrs<R>& P, cudaStream_t st) {
  k_add_time<R, EX><<<1, 1, 0, st>>>(P);
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::set_timestep(const CaseK& K, const DevPtrs<R>& P, int by_cells, cudaStream_t st) {
  k_dt_init<R, EX><<<1, 1, 0, st>>>(P);
  k_dt_reduce<D, R, EX><<<grid_for(by_cells ? K.ncell : K.cap, BLK), BLK, 0, st>>>(K, P, by_cells);
  k_dt_final<R, EX><<<1, 1, 0, st>>>(P);
}

/* ------------------------------------------------------------------ */
/* MLS_P2G (mpm.cpp:274-382)                                          */
/* ------------------------------------------------------------------ */
template <int D, typename R>
__device__ __forceinline__ R kernel_w_r(R dist, R h, R C) {
  R s = dist / h;
  R val = R(0);
  if (s < R(2)) {
    R q = R(1.) - R(0.5) * s;
    val = C * (((q * q) * q) * q) * (R(1.) + R(2.) * s);
  }
  return val;
}

/* the P2G neighbourhood of cell ci (its +-1 cells), every particle in it inside
 * the cut radius, in list order: body(q, ph, xij, ww) with the particle's phase
 * index, offset from the cell centre and kernel weight times volume */
template <int D, typename R, typename F_>
__device__ __forceinline__ void p2g_scan(const CaseK& K, const DevPtrs<R>& P, const int* idx, const double* xc,
                                         const R* xcr, double Cw, int skip, F_&& body) {
  const R* X = P.X[P.xb];
  const double hi = K.p_g * 1 * 3.2 / CUT_OFF;
  const double cut = 1.5 * K.p_sz;
  const float lo2 = (float)(cut * cut * (1.0 - 1e-5)), hi2 = (float)(cut * cut * (1.0 + 1e-5));
  int lo[3], hi3[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = max(idx[d] - 1, 0);
    hi3[d] = min(idx[d] + 1, (d < D ? K.N[d] : 1) - 1);
  }
  /* skip: bit (ox | oy << 1 | oz << 2), o = offset along the axis is nonzero,
   * set for the neighbour cells that hold no contributing particle (p2g_skip) */
  for (int t = lo[0]; t <= hi3[0]; t++)
    for (int s = lo[1]; s <= hi3[1]; s++)
      for (int m = lo[2]; m <= hi3[2]; m++) {
        const int code = (t != idx[0] ? 1 : 0) | (s != idx[1] ? 2 : 0) | (m != idx[2] ? 4 : 0);
        if ((skip >> code) & 1) continue;
        int64_t cn = cidx3(K, t, s, m);
        int cntq = min(P.bcnt[cn], K.maxpc);
        const int32_t* bk = P.bucket + cn * K.maxpc;
        for (int r = 0; r < cntq; r++) {
          int32_t q = bk[r];
          int ph = P.phase[q] - 1;
          R xij[3];
          for (int d = 0; d < D; d++) xij[d] = X[d * K.cap + q] - xcr[d];
          bool in;
          double dist;
          if (sizeof(R) == 4) {
            float dd = 0.f;
            for (int d = 0; d < D; d++) dd += (float)xij[d] * (float)xij[d];
            if (dd < lo2) in = true;
            else if (dd > hi2) in = false;
            else {
              double e2 = 0;
              for (int d = 0; d < D; d++) {
                double t2 = (double)X[d * K.cap + q] - xc[d];
                e2 = (d == 0) ? t2 * t2 : e2 + t2 * t2;
              }
              in = sqrt(e2) < cut;
            }
            dist = (double)sqrtf(dd);
          } else {
            double e2 = 0;
            for (int d = 0; d < D; d++) {
              double t2 = (double)xij[d];
              e2 = (d == 0) ? t2 * t2 : e2 + t2 * t2;
            }
            dist = sqrt(e2);
            in = dist < cut;
          }
          if (!in) continue;
          R ww = kernel_w_r<D, R>((R)dist, (R)hi, (R)Cw) * P.vol[q];
          if (ph < 0 || ph >= F) continue;
          body(q, ph, xij, ww);
        }
      }
}

/* Neighbour cells P2G can skip when every particle lies in its bucket's cell
 * (right after binning; split children, inlet clones and merged particles are
 * appended to the cell of their exact position): a cell whose box, shrunk by
 * 1e-4 of a cell against rounding, stays beyond the cut radius of the centre
 * holds no particle inside it.  Bit (ox | oy << 1 | oz << 2) for the offset
 * pattern (o = nonzero offset along that axis).  Skipping them leaves the
 * order of the remaining sum unchanged. */
template <int D>
int p2g_skip(const CaseK& K) {
  const double cut = 1.5 * K.p_sz;
  int mask = 0;
  for (int code = 0; code < 8; code++) {
    if (D == 2 && (code & 4)) continue;
    double g2 = 0.0;
    for (int d = 0; d < D; d++)
      if (code & (1 << d)) {
        const double g = 0.5 * K.ps[d] * (1.0 - 1e-4);
        g2 += g * g;
      }
    if (g2 > cut * cut) mask |= 1 << code;
  }
  return mask;
}

/* per cell: the kernel-weighted mass of each phase in the neighbourhood, the
 * phase flags and volume fractions, and the reset of absent phases; the rare
 * newly present phases are flagged in cnew for k_p2g_new (a second kernel, so
 * that this one keeps a small register footprint) */
template <int D, typename R, bool EX>
__global__ void __launch_bounds__(128) k_p2g(CaseK K, DevPtrs<R> P, double Cw, int skip) {
  constexpr int U = D + 2, B = D + 1;
  const int64_t nc = K.ncell;
  GRID_STRIDE(ci, nc) {
    if (!P.cused[ci]) {
      P.cnew[ci] = 0;
      continue;
    }
    int idx[3];
    cijk<D>(K, ci, idx);
    double xc[3];
    center<D>(K, idx, xc);
    R xcr[3];
    for (int d = 0; d < 3; d++) xcr[d] = (R)xc[d];
    double mass_t[F] = {0, 0};
    p2g_scan<D, R>(K, P, idx, xc, xcr, Cw, skip, [&](int32_t, int ph, const R*, R ww) {
#pragma unroll
      for (int s = 0; s < F; s++)
        if (s == ph) mass_t[s] += (double)ww;
    });
    int newmask = 0;
    for (int s = 0; s < F; s++)
      if (mass_t[s] > 0 && P.cphb[s * nc + ci] == 0) newmask |= 1 << s;
    P.cnew[ci] = (int8_t)newmask;
    double mass_total = 0;
    for (int t = 0; t < F; t++) mass_total += mass_t[t];
    for (int ss = 0; ss < F; ss++) {
      int ph = mass_t[ss] > 0 ? 1 : 0;
      P.cph[ss * nc + ci] = (int8_t)ph;
      P.calph[ss * nc + ci] = (R)(mass_t[ss] / (mass_total + 1e-20));
      P.cphb[ss * nc + ci] = (int8_t)ph;
      if (ph == 0) {
        for (int t = 0; t < U * B; t++) {
          P.ccoef[(ss * U * B + t) * nc + ci] = R(0);
          P.ccoef0[(ss * U * B + t) * nc + ci] = R(0);
        }
        if (K.eshift[ss] != 0.0) {
          /* true energy 0, as the reference resets it */
          P.ccoef[(ss * U * B + (U - 1) * B) * nc + ci] = (R)(-K.eshift[ss]);
          P.ccoef0[(ss * U * B + (U - 1) * B) * nc + ci] = (R)(-K.eshift[ss]);
        }
        P.crho[ss * nc + ci] = (R)K.ini_rho[ss];
        for (int k = 0; k < D; k++) P.crhov[(ss * D + k) * nc + ci] = R(0);
      }
    }
  }
}

/* initialise each newly present phase of a flagged cell (mpm.cpp:345-363) from
 * the weighted averages of its particles' reconstructed states and slopes; the
 * phase's mass is summed again over the same particles in the same order, so
 * it equals k_p2g's bit for bit */
template <int D, typename R, bool EX>
__global__ void __launch_bounds__(128) k_p2g_new(CaseK K, DevPtrs<R> P, double Cw) {
  constexpr int U = D + 2, B = D + 1, NS = U * D;
  const int64_t nc = K.ncell;
  GRID_STRIDE(ci, nc) {
    const int newmask = P.cnew[ci];
    if (!newmask) continue;
    int idx[3];
    cijk<D>(K, ci, idx);
    double xc[3];
    center<D>(K, idx, xc);
    R xcr[3];
    for (int d = 0; d < 3; d++) xcr[d] = (R)xc[d];
    for (int ss = 0; ss < F; ss++) {
      if (!(newmask & (1 << ss))) continue;
      double p_avg[U], Cf[NS], mt = 0;
      for (int u = 0; u < U; u++) p_avg[u] = 0;
      for (int t = 0; t < NS; t++) Cf[t] = 0;
      p2g_scan<D, R>(K, P, idx, xc, xcr, Cw, 0, [&](int32_t q, int ph, const R* xij, R ww) {
        if (ph != ss) return;
        mt += (double)ww;
        double wwd = (double)ww;
        double pj[U];
        pj[0] = (double)P.rho[q];
        for (int k = 0; k < D; k++) pj[1 + k] = (double)P.rhov[k * K.cap + q];
        pj[U - 1] = (double)P.E[q];
        for (int u = 0; u < U; u++) {
          double acc = 0;
          for (int b = 0; b < D; b++) {
            double sv = (double)P.sl[(u * D + b) * K.cap + q];
            acc = (b == 0) ? sv * (-(double)xij[b]) : acc + sv * (-(double)xij[b]);
          }
          pj[u] += acc;
        }
        for (int u = 0; u < U; u++) p_avg[u] += pj[u] * wwd;
        for (int tt = 0; tt < NS; tt++) Cf[tt] += (double)P.sl[tt * K.cap + q] * wwd;
      });
      mt += 1e-20;
      for (int u = 0; u < U; u++) p_avg[u] /= mt;
      for (int t = 0; t < NS; t++) Cf[t] /= mt;
      for (int u = 0; u < U; u++)
        for (int b = 0; b < B; b++) P.ccoef[((ss * U + u) * B + b) * nc + ci] = R(0);
      P.ccoef[((ss * U + 0) * B + 0) * nc + ci] = (R)p_avg[0];
      P.crho[ss * nc + ci] = (R)p_avg[0];
      for (int k = 0; k < D; k++) {
        P.ccoef[((ss * U + 1 + k) * B + 0) * nc + ci] = (R)p_avg[1 + k];
        P.crhov[(ss * D + k) * nc + ci] = (R)p_avg[1 + k];
      }
      P.ccoef[((ss * U + U - 1) * B + 0) * nc + ci] = (R)p_avg[U - 1];
      P.cE[ss * nc + ci] = (R)p_avg[U - 1];
      for (int u = 0; u < U; u++)
        for (int b = 0; b < D; b++) P.ccoef[((ss * U + u) * B + 1 + b) * nc + ci] = (R)Cf[u * D + b];
      R rho = P.crho[ss * nc + ci];
      R sq = R(0);
      for (int k = 0; k < D; k++) {
        R rv = P.crhov[(ss * D + k) * nc + ci];
        P.cv[k * nc + ci] = rv / rho;
        sq = (k == 0) ? rv * rv : sq + rv * rv;
      }
      R e_j = P.cE[ss * nc + ci] - R(0.5) * sq / rho;
      P.cP[ci] = eos_p<R>(e_j, (R)K.gamma[ss], (R)K.pinf_eos[ss]);
      for (int t = 0; t < U * B; t++) P.ccoef0[(ss * U * B + t) * nc + ci] = P.ccoef[(ss * U * B + t) * nc + ci];
    }
  }
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::p2g(const CaseK& K, const DevPtrs<R>& P, bool fresh_bins, cudaStream_t st) {
  const double hi = K.p_g * 1 * 3.2 / CUT_OFF;
  double hh = (D == 2) ? hi * hi : hi * hi * hi;
  double Cw = (D == 2) ? 1.0 / PI_REF / hh * 7. / 4. : 1.0 / PI_REF / hh * 21. / 16.;
  k_p2g<D, R, EX><<<grid_for(K.ncell, 128), 128, 0, st>>>(K, P, Cw, fresh_bins ? p2g_skip<D>(K) : 0);
}

/* the newly present phases k_p2g flagged (runs after it) */
template <int D, typename R, bool EX>
void Launch<D, R, EX>::p2g_new(const CaseK& K, const DevPtrs<R>& P, cudaStream_t st) {
  const double hi = K.p_g * 1 * 3.2 / CUT_OFF;
  double hh = (D == 2) ? hi * hi : hi * hi * hi;
  double Cw = (D == 2) ? 1.0 / PI_REF / hh * 7. / 4. : 1.0 / PI_REF / hh * 21. / 16.;
  k_p2g_new<D, R, EX><<<grid_for(K.ncell, 128), 128, 0, st>>>(K, P, Cw);
}

/* ------------------------------------------------------------------ */
/* Calculate_limiter (mpm.cpp:392-738)                                */
/* ------------------------------------------------------------------ */
template <typename R>
__device__ __forceinline__ R limiter_fn(R ds, int bd_fg) {
  /* Limiter (glbfunc.h:283-299) */
  R val = R(1);
  if (ds > R(0) && ds < R(0.5)) val = R(2) * ds;
  else if (ds >= R(0.5)) val = R(1);
  if (bd_fg == 1) val = (fabs(ds) + ds) / (fabs(ds) + R(1));
  return val;
}

template <int D, typename R, bool EX>
__global__ void __launch_bounds__(128, minblocks_f32<R>(6)) k_limiter(CaseK K, DevPtrs<R> P) {
  constexpr int U = D + 2, B = D + 1, NF = 2 * D;
  const int64_t nc = K.ncell;
  R hps[3], Sax[3];
  cell_geom<D, R>(K, hps, Sax);
  /* positivity probe offsets, converted once per block */
  __shared__ R s_probe[8][3];
  if (threadIdx.x < 24) s_probe[threadIdx.x / 3][threadIdx.x % 3] = (R)K.probe[threadIdx.x / 3][threadIdx.x % 3];
  __syncthreads();
  GRID_STRIDE(ci, nc) {
    if (!P.cused[ci]) continue;
    int idx[3];
    cijk<D>(K, ci, idx);
    double xc[3];
    if constexpr (EX) center<D>(K, idx, xc);
    R u_max[F][U], u_min[F][U], pi[F][U], lim[F][U];
    for (int s = 0; s < F; s++)
      for (int u = 0; u < U; u++) {
        u_max[s][u] = R(-1e20);
        u_min[s][u] = R(1e20);
        lim[s][u] = R(1.);
      }
    for (int s = 0; s < F; s++) {
      pi[s][0] = P.crho[s * nc + ci];
      for (int k = 0; k < D; k++) pi[s][1 + k] = P.crhov[(s * D + k) * nc + ci];
      pi[s][U - 1] = P.cE[s * nc + ci];
    }
    /* G_v (mpm.cpp:469-533) */
    int bd_fg = 0;
    R vc[3];
    for (int k = 0; k < D; k++) vc[k] = P.cv[k * nc + ci];
    for (int dd = 0; dd < D; dd++) {
      R pd = (R)K.ps[dd];
      if (idx[dd] == K.N[dd] - 1) {
        for (int r = 0; r < D; r++) P.cgv[(r * D + dd) * nc + ci] = ((dd == 0 ? vc[r] : R(0)) - vc[r]) / (R(0.5) * pd);
        bd_fg = 1;
      } else if (idx[dd] == 0) {
        for (int r = 0; r < D; r++) P.cgv[(r * D + dd) * nc + ci] = (vc[r] - (dd == 0 ? vc[r] : R(0))) / (R(0.5) * pd);
        bd_fg = 1;
      } else {
        int a[3] = {idx[0], idx[1], idx[2]}, b[3] = {idx[0], idx[1], idx[2]};
        a[dd] += 1;
        b[dd] -= 1;
        int64_t cR = cidx3(K, a[0], a[1], a[2]), cL = cidx3(K, b[0], b[1], b[2]);
        for (int r = 0; r < D; r++) P.cgv[(r * D + dd) * nc + ci] = (P.cv[r * nc + cR] - P.cv[r * nc + cL]) / (R(2) * pd);
      }
    }
    const bool mirror_j = (idx[1] == K.N[1] - 1 || idx[1] == 0);
    const bool mirror_k = (D == 3) && (idx[2] == K.N[2] - 1 || idx[2] == 0);
    for (int f = 0; f < NF; f++) {
      int fcb, fnb[3];
      if constexpr (EX) {
        FaceK fc;
        face<D>(K, idx, xc, f, fc);
        fcb = fc.bound;
        for (int d = 0; d < 3; d++) fnb[d] = fc.nb[d];
      } else {
        FaceRel<R> fc;
        face_rel<D, R>(K, idx, hps, Sax, f, fc);
        fcb = fc.bound;
        for (int d = 0; d < 3; d++) fnb[d] = fc.nb[d];
      }
      struct { int bound; int nb[3]; } fc = {fcb, {fnb[0], fnb[1], fnb[2]}};
      if (fc.bound == 0) {
        int64_t nb = cidx3(K, fc.nb[0], fc.nb[1], fc.nb[2]);
        for (int s = 0; s < F; s++) {
          R pj[U];
          for (int u = 0; u < U; u++) pj[u] = R(0);
          for (int s1 = 0; s1 < F; s1++) {
            R aj = P.calph[s1 * nc + nb];
            if (aj == R(0)) continue;
            R rhoj = P.crho[s1 * nc + nb];
            R rvj[3];
            for (int k = 0; k < D; k++) rvj[k] = P.crhov[(s1 * D + k) * nc + nb];
            R Ej = P.cE[s1 * nc + nb];
            if (s1 != s) {
              R vj[3], sq = R(0);
              for (int k = 0; k < D; k++) {
                vj[k] = qdiv<R, EX>(rvj[k], rhoj);
                sq = (k == 0) ? vj[k] * vj[k] : sq + vj[k] * vj[k];
              }
              R rhoe_j = Ej - R(0.5) * rhoj * sq;
              R P_j = eos_p<R>(rhoe_j, (R)K.gamma[s1], (R)K.pinf_eos[s1]);
              rhoj = P.crho[s * nc + ci];
              for (int k = 0; k < D; k++) rvj[k] = rhoj * vj[k];
              Ej = eos_rhoe<R>(P_j, (R)K.gamma[s], (R)K.pinf_eos[s]) + R(0.5) * rhoj * sq;
            }
            pj[0] += rhoj * aj;
            for (int k = 0; k < D; k++) pj[1 + k] += rvj[k] * aj;
            pj[U - 1] += Ej * aj;
          }
          for (int u = 0; u < U; u++) {
            R d = pj[u] - pi[s][u];
            u_max[s][u] = amax1(u_max[s][u], d);
            u_min[s][u] = amin1(u_min[s][u], d);
          }
        }
      } else {
        for (int s = 0; s < F; s++) {
          R pj[U];
          pj[0] = P.crho[s * nc + ci];
          for (int k = 0; k < D; k++) pj[1 + k] = P.crhov[(s * D + k) * nc + ci];
          pj[U - 1] = P.cE[s * nc + ci];
          if (fc.bound == PGDG_BC_INLET || fc.bound == PGDG_BC_OUTLET || fc.bound == PGDG_BC_TRANSMISSIVE)
            for (int u = 0; u < U; u++) pj[u] = pi[s][u];
          if (fc.bound != PGDG_BC_TRANSMISSIVE) {
            if (mirror_j) pj[2] = -P.crhov[(s * D + 1) * nc + ci];
            if (mirror_k) pj[3] = -P.crhov[(s * D + 2) * nc + ci];
          }
          for (int u = 0; u < U; u++) {
            R d = pj[u] - pi[s][u];
            u_max[s][u] = amax1(u_max[s][u], d);
            u_min[s][u] = amin1(u_min[s][u], d);
          }
        }
      }
    }
    for (int s = 0; s < F; s++)
      for (int u = 0; u < U; u++) {
        u_max[s][u] = amax1(u_max[s][u], R(0.));
        u_min[s][u] = amin1(u_min[s][u], R(0.));
      }
    /* per phase: its coefficients are loaded once; the face limits (a minimum
     * over the faces, so the face order does not matter) and the positivity
     * probe (mpm.cpp:690-728) then read them from registers */
    const int NPR = (D == 3) ? 8 : 4;
#pragma unroll
    for (int s = 0; s < F; s++) {
      R co[U][B];
      for (int u = 0; u < U; u++)
        for (int b = 0; b < B; b++) co[u][b] = P.ccoef[((s * U + u) * B + b) * nc + ci];
      const int lim_fg = (bd_fg || P.calph[s * nc + ci] != R(1)) ? 1 : 0;
      for (int f = 0; f < NF; f++) {
        R dr[3];
        if constexpr (EX) {
          FaceK fc;
          face<D>(K, idx, xc, f, fc);
          if (fc.bound == 0) {
            double xn[3];
            center<D>(K, fc.nb, xn);
            for (int d = 0; d < D; d++) dr[d] = (R)(xn[d] - xc[d]);
          } else {
            for (int d = 0; d < D; d++) dr[d] = (R)(fc.cen[d] - xc[d]);
          }
        } else {
          FaceRel<R> fc;
          face_rel<D, R>(K, idx, hps, Sax, f, fc);
          /* neighbour centre (interior) or face centre (boundary) from the cell centre */
          for (int d = 0; d < D; d++) dr[d] = (fc.bound == 0) ? R(2) * fc.cen[d] : fc.cen[d];
        }
        for (int u = 0; u < U; u++) {
          R dU = R(0);
          for (int b = 0; b < D; b++) dU = (b == 0) ? co[u][1 + b] * dr[b] : dU + co[u][1 + b] * dr[b];
          R sd = R(1);
          if constexpr (EX) {
            if (dU >= R(0)) sd = limiter_fn<R>(fabs(qdiv<R, EX>(u_max[s][u], dU + R(1e-20))), lim_fg);
            else if (dU < R(0)) sd = limiter_fn<R>(fabs(qdiv<R, EX>(u_min[s][u], dU + R(1e-20))), lim_fg);
          } else if (dU == dU) {
            /* The ratio |u / (dU + 1e-20)|.  A negative dU equal to -1e-20 in
             * the working precision makes the denominator zero, which is far
             * likelier in FP32 (a slope of 1e-20 / dr turns up at symmetry
             * planes) and gives inf or NaN, and the boundary limiter form
             * (|ds| + ds) / (|ds| + 1) of inf is NaN.  Here a zero numerator
             * gives 0 (its value for any non-zero denominator) and the ratio is
             * capped at 1e30, where the limiter is 1 (interior) or 2 (boundary)
             * as for every ratio above about 1e8, and the minimum with lim <= 1
             * ignores it either way: the result equals the reference's wherever
             * the reference's is finite. */
            const R um = dU >= R(0) ? u_max[s][u] : u_min[s][u];
            R ds = fabs(qdiv<R, EX>(um, dU + R(1e-20)));
            if (um == R(0)) ds = R(0);
            else if (!(ds <= R(1e30))) ds = R(1e30);
            sd = limiter_fn<R>(ds, lim_fg);
          }
          lim[s][u] = amin1(lim[s][u], sd);
        }
      }
      const R gs = (R)K.gamma[s], pf = (R)K.pinf[s], pfe = (R)K.pinf_eos[s];
      int fg = 0;
      for (int pr = 0; pr < NPR && !fg; pr++) {
        R Ui[U];
        for (int u = 0; u < U; u++) {
          R acc = R(0);
          for (int b = 0; b < D; b++)
            acc = (b == 0) ? co[u][1 + b] * s_probe[pr][b] : acc + co[u][1 + b] * s_probe[pr][b];
          Ui[u] = co[u][0] + lim[s][u] * acc;
        }
        R sq = Ui[1] * Ui[1];
        for (int k = 1; k < D; k++) sq = sq + Ui[1 + k] * Ui[1 + k];
        R e_p = Ui[U - 1] - qdiv<R, EX>(R(0.5) * sq, Ui[0]);
        R P_p = eos_p<R>(e_p, gs, pfe);
        if (P_p < R(-0.05) * pf || Ui[0] < R(0)) fg = 1;
      }
      for (int u = 0; u < U; u++) P.clim[(s * U + u) * nc + ci] = fg ? R(0.) : lim[s][u];
    }
  }
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::limiter(const CaseK& K, const DevPtrs<R>& P, cudaStream_t st) {
  k_limiter<D, R, EX><<<grid_for(K.ncell, 128), 128, 0, st>>>(K, P);
}

/* ------------------------------------------------------------------ */
/* Grid_acceleration (particle_flow.cpp:16-405)                       */
/* ------------------------------------------------------------------ */
template <int D, typename R>
struct Prim {
  R U[D + 2];
  R v[3];
  R P, c, vn;
};

/* component a of a D-vector held in registers (a select chain: indexing a
 * register array with a run-time index would move the array to local memory) */
template <int D, typename R>
__device__ __forceinline__ R pick(const R* v, int a) {
  R r = v[0];
#pragma unroll
  for (int k = 1; k < D; k++)
    if (a == k) r = v[k];
  return r;
}

/* normal-column flux F[u] = DF[u][a] with DF = U v^T + P I (+ v P in the energy row) */
template <int D, typename R>
__device__ __forceinline__ void flux_col(const R* Uu, const R* v, R Pp, int a, R* Fc, R esh) {
  constexpr int U = D + 2;
  const R va = pick<D, R>(v, a);
#pragma unroll
  for (int u = 0; u < U; u++) Fc[u] = Uu[u] * va;
#pragma unroll
  for (int k = 0; k < D; k++)
    if (k == a) Fc[1 + k] += Pp;
  Fc[U - 1] += va * Pp;
  if (esh != R(0)) Fc[U - 1] += va * esh;   /* (E_true + p) v with E_true = E + esh */
}

/* MODE 0: MGFM solved inline; MODE 2: queue every interface problem (no flux
 * work); MODE 3: read the ghost states of the interface problems from the queue */
template <int D, typename R, bool EX, int MODE>
__global__ void __launch_bounds__(128, minblocks_f32<R>(MODE == 0 ? 2 : 3)) k_grid_acc(CaseK K, DevPtrs<R> P, int variant, double voli_d,
                                                 double mij1, double mij2, double mij3, IfaceQ Q) {
  constexpr int U = D + 2, B = D + 1, NF = 2 * D, NQ = (D == 3) ? 4 : 2, NG = (D == 3) ? 8 : 4;
  const int64_t nc = K.ncell;
  const double gp[2] = {-1. / sqrt(3.), 1. / sqrt(3.)};
  /* the non-exact paths take the cell geometry in R, relative to the centre */
  const R gpr[2] = {R(-1. / sqrt(3.)), R(1. / sqrt(3.))};
  R hps[3], Sax[3];
  cell_geom<D, R>(K, hps, Sax);
  const R inv[4] = {R(1. / (voli_d + 1e-20)), R(1. / (mij1 + 1e-20)), R(1. / (mij2 + 1e-20)),
                    R(1. / (mij3 + 1e-20))};
  unsigned long long ncall = 0, nit = 0, nmax = 0;
  /* with the interface queue, a stage whose problems outgrew it runs the inline
   * solve (MODE 0 launched beside MODE 3): exactly one of the two does work */
  if (Q.tot) {
    const bool over = Q.tot[0] > (unsigned long long)Q.cap;
    if ((MODE == 3 && over) || (MODE == 0 && !over)) return;
  }
  GRID_STRIDE(ci, nc) {
    if (!P.cused[ci]) continue;
    int idx[3];
    cijk<D>(K, ci, idx);
    double xc[3];
    if constexpr (EX) center<D>(K, idx, xc);
    const bool mirror_j = (idx[1] == K.N[1] - 1 || idx[1] == 0);
    const bool mirror_k = (D == 3) && (idx[2] == K.N[2] - 1 || idx[2] == 0);
    int64_t qi = 0;
    if constexpr (MODE != 0) {
      if (Q.off[ci + 1] == Q.off[ci]) {
        if constexpr (MODE == 2) continue;
      }
      qi = (int64_t)Q.off[ci];
    }
    for (int ss = 0; ss < F; ss++) {
      if (P.cph[ss * nc + ci] != 1) continue;
      const R gs = (R)K.gamma[ss], pfs = (R)K.pinf[ss], pfe = (R)K.pinf_eos[ss], esh = (R)K.eshift[ss];
      R co[U][B], L[U], dc[U][B];
      for (int u = 0; u < U; u++) {
        for (int b = 0; b < B; b++) {
          co[u][b] = P.ccoef[((ss * U + u) * B + b) * nc + ci];
          dc[u][b] = R(0);
        }
        L[u] = P.clim[(ss * U + u) * nc + ci];
      }
      /* volume integral, 2^D Gauss points */
      const R voli = (R)voli_d;
      for (int g = 0; g < (MODE == 2 ? 0 : NG); g++) {
        int g1 = (D == 3) ? (g >> 2) : (g >> 1), g2 = (D == 3) ? ((g >> 1) & 1) : (g & 1), g3 = g & 1;
        R dp[3];
        if constexpr (EX) {
          dp[0] = (R)(gp[g1] * (K.ps[0] / 2));
          dp[1] = (R)(gp[g2] * (K.ps[1] / 2));
          dp[2] = (D == 3) ? (R)(gp[g3] * (K.ps[2] / 2)) : R(0);
        } else {
          dp[0] = gpr[g1] * hps[0];
          dp[1] = gpr[g2] * hps[1];
          dp[2] = (D == 3) ? gpr[g3] * hps[2] : R(0);
        }
        const R gw = (D == 3) ? R(0.125) : R(0.25);
        R Up[U];
        for (int u = 0; u < U; u++) {
          R acc = co[u][1] * dp[0];
          for (int b = 1; b < D; b++) acc = acc + co[u][1 + b] * dp[b];
          Up[u] = co[u][0] + L[u] * acc;
        }
        R rho_p = Up[0];
        R vp[3], sq = Up[1] * Up[1];
        for (int k = 1; k < D; k++) sq = sq + Up[1 + k] * Up[1 + k];
        for (int k = 0; k < D; k++) vp[k] = qdiv<R, EX>(Up[1 + k], rho_p);
        R P_p = eos_p<R>(Up[U - 1] - qdiv<R, EX>(R(0.5) * sq, rho_p), gs, pfe);
        for (int bi = 1; bi <= D; bi++) {
          R Fc[U];
          flux_col<D, R>(Up, vp, P_p, bi - 1, Fc, esh);
          for (int u = 0; u < U; u++) dc[u][bi] += Fc[u] * gw * voli;
        }
      }
      /* face integral */
      for (int f = 0; f < NF; f++) {
        /* exact path: the reference's absolute FP64 face geometry; otherwise
         * the same face relative to the cell centre in R */
        FaceK fc;
        FaceRel<R> fr;
        if constexpr (EX) face<D>(K, idx, xc, f, fc);
        else face_rel<D, R>(K, idx, hps, Sax, f, fr);
        const int a = EX ? fc.axis : fr.axis;
        const int fbound = EX ? fc.bound : fr.bound;
        const R na = EX ? (R)fc.sgn : fr.sgn;
        R DFn[B][U];
        for (int b = 0; b < B; b++)
          for (int u = 0; u < U; u++) DFn[b][u] = R(0);
        int64_t nb = -1;
        if (fbound == 0) {
          if constexpr (EX) nb = cidx3(K, fc.nb[0], fc.nb[1], fc.nb[2]);
          else nb = cidx3(K, fr.nb[0], fr.nb[1], fr.nb[2]);
        }
        double xn[3] = {0, 0, 0};
        if constexpr (EX)
          if (nb >= 0) center<D>(K, fc.nb, xn);
        /* the FP32 path takes, on an interior face, the neighbour phases as the
         * outer loop and the quadrature points as the inner one, so that a
         * neighbour phase's coefficients are loaded once per face; the FP64
         * paths keep the reference's order (points outer, phases inner) */
        constexpr bool HOIST = !EX && sizeof(R) == 4;
        const int nso = (HOIST && fbound == 0) ? F : 1;
        for (int so = 0; so < nso; so++) {
        R ajo = R(0), cn[U][B], ln[U];
        if constexpr (HOIST) {
          if (fbound == 0) {
            ajo = P.calph[so * nc + nb];
            if (ajo == R(0)) continue;
            if (MODE == 2 && so == ss) continue;
            for (int u = 0; u < U; u++) {
              for (int b = 0; b < B; b++) cn[u][b] = P.ccoef[((so * U + u) * B + b) * nc + nb];
              ln[u] = P.clim[(so * U + u) * nc + nb];
            }
          }
        }
        for (int qd = 0; qd < NQ; qd++) {
          int g1 = (D == 3) ? (qd >> 1) : qd, g2 = qd & 1;
          double dpv[3];
          const R gw = (D == 3) ? R(0.25) : R(0.5);
          R dri[3];
          if constexpr (EX) {
            for (int d = 0; d < 3; d++) dpv[d] = (D == 3) ? gp[g1] * fc.t0[d] + gp[g2] * fc.t1[d] : gp[g1] * fc.t0[d];
            for (int d = 0; d < D; d++) dri[d] = (R)(dpv[d] + fc.cen[d] - xc[d]);
          } else {
            for (int d = 0; d < D; d++)
              dri[d] = (D == 3) ? gpr[g1] * fr.t0[d] + gpr[g2] * fr.t1[d] + fr.cen[d] : gpr[g1] * fr.t0[d] + fr.cen[d];
          }
          R Ui[U];
          for (int u = 0; u < U; u++) {
            R acc = co[u][1] * dri[0];
            for (int b = 1; b < D; b++) acc = acc + co[u][1 + b] * dri[b];
            Ui[u] = co[u][0] + L[u] * acc;
          }
          const R rho_i = Ui[0], E_i = Ui[U - 1];
          R v_i[3], sq = Ui[1] * Ui[1];
          for (int k = 1; k < D; k++) sq = sq + Ui[1 + k] * Ui[1 + k];
          for (int k = 0; k < D; k++) v_i[k] = qdiv<R, EX>(Ui[1 + k], rho_i);
          const R P_i = eos_p<R>(E_i - qdiv<R, EX>(R(0.5) * sq, rho_i), gs, pfe);
          const R c_i = sqrt_r<R>(qdiv<R, EX>(gs * (pfs + P_i), rho_i));
          const R vni = pick<D, R>(v_i, a) * na;
          R Fi[U];
          flux_col<D, R>(Ui, v_i, P_i, a, Fi, esh);
          R Nb[B];
          Nb[0] = R(1.);
          for (int d = 0; d < D; d++) Nb[1 + d] = dri[d];
          if (fbound == 0) {
            for (int s1 = HOIST ? so : 0; s1 < (HOIST ? so + 1 : F); s1++) {
              const R aj = HOIST ? ajo : P.calph[s1 * nc + nb];
              if (aj == R(0)) continue;
              if (MODE == 2 && s1 == ss) continue;
              R drj[3];
              if constexpr (EX) {
                for (int d = 0; d < D; d++) drj[d] = (R)(dpv[d] + fc.cen[d] - xn[d]);
              } else {
                /* the neighbour centre sits at 2 x the face-centre offset */
                for (int d = 0; d < D; d++) drj[d] = dri[d] - R(2) * fr.cen[d];
              }
              R Uj[U];
              if constexpr (!HOIST) {
                for (int u = 0; u < U; u++) {
                  R acc = P.ccoef[((s1 * U + u) * B + 1) * nc + nb] * drj[0];
                  for (int b = 1; b < D; b++) acc = acc + P.ccoef[((s1 * U + u) * B + 1 + b) * nc + nb] * drj[b];
                  Uj[u] = P.ccoef[((s1 * U + u) * B) * nc + nb] + P.clim[(s1 * U + u) * nc + nb] * acc;
                }
              } else {
                for (int u = 0; u < U; u++) {
                  R acc = cn[u][1] * drj[0];
                  for (int b = 1; b < D; b++) acc = acc + cn[u][1 + b] * drj[b];
                  Uj[u] = cn[u][0] + ln[u] * acc;
                }
              }
              R rho_j = Uj[0], E_j = Uj[U - 1];
              R v_j[3], rhov_j[3];
              R sqj = R(0);
              for (int k = 0; k < D; k++) {
                rhov_j[k] = Uj[1 + k];
                v_j[k] = qdiv<R, EX>(rhov_j[k], rho_j);
                sqj = (k == 0) ? v_j[k] * v_j[k] : sqj + v_j[k] * v_j[k];
              }
              R rhoe_j = E_j - R(0.5) * sqj * rho_j;
              R P_j = eos_p<R>(rhoe_j, (R)K.gamma[s1], (R)K.pinf_eos[s1]);
              R vnj = pick<D, R>(v_j, a) * na;
              if (ss != s1) {
                double gh[3];
                if constexpr (MODE == 2) {
                  const int64_t e = qi++;
                  if (e < Q.cap) {
                    double* q6 = Q.in6 + 6 * e;
                    q6[0] = (double)vni;
                    q6[1] = (double)vnj;
                    q6[2] = (double)P_i;
                    q6[3] = (double)P_j;
                    q6[4] = (double)rho_i;
                    q6[5] = (double)rho_j;
                    Q.mat[2 * e] = (int8_t)ss;
                    Q.mat[2 * e + 1] = (int8_t)s1;
                  }
                  continue;
                } else if constexpr (MODE == 3) {
                  const int64_t e = qi++;
                  gh[0] = Q.out3[3 * e];
                  gh[1] = Q.out3[3 * e + 1];
                  gh[2] = Q.out3[3 * e + 2];
                } else {
                  int it = mgfm((double)vni, (double)vnj, (double)P_i, (double)P_j, (double)rho_i, (double)rho_j,
                                K.gamma[ss], K.pinf[ss], K.gamma[s1], K.pinf[s1], variant, -1.0, gh);
                  ncall++;
                  nit += it;
                  if (it >= 50) nmax++;
                }
                rho_j = (R)gh[0];
                P_j = (R)gh[1];
                vnj = (R)gh[2];
                sqj = R(0);
                for (int k = 0; k < D; k++) {
                  v_j[k] = v_i[k] - (k == a ? vni * na : R(0)) + (k == a ? vnj * na : R(0));
                  rhov_j[k] = rho_j * v_j[k];
                  sqj = (k == 0) ? v_j[k] * v_j[k] : sqj + v_j[k] * v_j[k];
                }
                E_j = eos_rhoe<R>(P_j, gs, pfe) + R(0.5) * rho_j * sqj;
              }
              const R c_j = sqrt_r<R>(qdiv<R, EX>(gs * (pfs + P_j), rho_j));
              R Ujj[U];
              Ujj[0] = rho_j;
              for (int k = 0; k < D; k++) Ujj[1 + k] = rhov_j[k];
              Ujj[U - 1] = E_j;
              R Fj[U];
              flux_col<D, R>(Ujj, v_j, P_j, a, Fj, esh);
              const R vni2 = pick<D, R>(v_i, a) * na;
              vnj = pick<D, R>(v_j, a) * na;
              /* HLLC (particle_flow.cpp:232-272) */
              const R SL = amin1(vni2 - c_i, vnj - c_j);
              const R SR = amax1(vni2 + c_i, vnj + c_j);
              const R S_s = qdiv<R, EX>((P_j - P_i) + rho_i * vni2 * (SL - vni2) - rho_j * vnj * (SR - vnj),
                                        rho_i * (SL - vni2) - rho_j * (SR - vnj));
              R Fh[U];
              if (SL > R(0)) {
                for (int u = 0; u < U; u++) Fh[u] = Fi[u];
              } else if (SL <= R(0) && S_s >= R(0)) {
                const R rho_sL = qdiv<R, EX>(rho_i * (SL - vni2), SL - S_s);
                R UsL[U];
                UsL[0] = rho_sL;
                for (int k = 0; k < D; k++) UsL[1 + k] = rho_sL * (v_i[k] + (k == a ? (S_s - vni2) * na : R(0)));
                UsL[U - 1] = rho_sL * (qdiv<R, EX>(E_i, rho_i) + (S_s - vni2) * (S_s + qdiv<R, EX>(P_i, rho_i * (SL - vni2))));
                if (esh != R(0)) UsL[U - 1] += esh * qdiv<R, EX>(S_s - vni2, SL - S_s);   /* esh (rho_star / rho - 1) */
                for (int u = 0; u < U; u++) Fh[u] = Fi[u] + SL * (UsL[u] - Ui[u]) * na;
              } else if (S_s <= R(0) && SR >= R(0)) {
                const R rho_sR = qdiv<R, EX>(rho_j * (SR - vnj), SR - S_s);
                R UsR[U];
                UsR[0] = rho_sR;
                for (int k = 0; k < D; k++) UsR[1 + k] = rho_sR * (v_j[k] + (k == a ? (S_s - vnj) * na : R(0)));
                UsR[U - 1] = rho_sR * (qdiv<R, EX>(E_j, rho_j) + (S_s - vnj) * (S_s + qdiv<R, EX>(P_j, rho_j * (SR - vnj))));
                if (esh != R(0)) UsR[U - 1] += esh * qdiv<R, EX>(S_s - vnj, SR - S_s);
                for (int u = 0; u < U; u++) Fh[u] = Fj[u] + SR * (UsR[u] - Ujj[u]) * na;
              } else if (SR <= R(0)) {
                for (int u = 0; u < U; u++) Fh[u] = Fj[u];
              } else {
                for (int u = 0; u < U; u++) Fh[u] = R(0);
              }
              for (int b = 0; b < B; b++)
                for (int u = 0; u < U; u++) DFn[b][u] += Fh[u] * Nb[b] * gw * aj;
            }
          } else if (MODE == 2) {
          } else if (fbound == PGDG_BC_WALL) {
            for (int b = 0; b < B; b++)
#pragma unroll
              for (int k = 0; k < D; k++)
                if (k == a) DFn[b][1 + k] += P_i * Nb[b] * gw;
          } else {
            R rho_j = rho_i, P_j = P_i, E_j = E_i;
            R v_j[3], rhov_j[3];
            for (int k = 0; k < D; k++) {
              v_j[k] = v_i[k];
              rhov_j[k] = rho_j * v_j[k];
            }
            if (fbound == PGDG_BC_INLET) {
              rho_j = (R)K.inlet_rho;
              R sqj = R(0);
              for (int k = 0; k < D; k++) {
                v_j[k] = (R)K.inlet_u[k];
                rhov_j[k] = rho_j * v_j[k];
                sqj = (k == 0) ? v_j[k] * v_j[k] : sqj + v_j[k] * v_j[k];
              }
              P_j = (R)K.inlet_p;
              E_j = eos_rhoe<R>(P_j, gs, pfe) + R(0.5) * sqj * rho_j;
            }
            if (fbound != PGDG_BC_TRANSMISSIVE) {
              if (mirror_j) {
                v_j[1] = -v_i[1];
                for (int k = 0; k < D; k++) rhov_j[k] = rho_j * v_j[k];
              }
              if (mirror_k) {
                v_j[2] = -v_i[2];
                for (int k = 0; k < D; k++) rhov_j[k] = rho_j * v_j[k];
              }
            }
            R Uj[U];
            Uj[0] = rho_j;
            for (int k = 0; k < D; k++) Uj[1 + k] = rhov_j[k];
            Uj[U - 1] = E_j;
            const R c_j = sqrt_r<R>(qdiv<R, EX>(gs * (pfs + P_j), rho_j));
            const R vnj = pick<D, R>(v_j, a) * na;
            R Fj[U];
            flux_col<D, R>(Uj, v_j, P_j, a, Fj, esh);
            const R SL = amin1(vni - c_i, vnj - c_j);
            const R SR = amax1(vni + c_i, vnj + c_j);
            R Fh[U];
            if (SL > R(0)) {
              for (int u = 0; u < U; u++) Fh[u] = Fi[u];
            } else if (SL <= R(0) && SR >= R(0)) {
              for (int u = 0; u < U; u++) Fh[u] = qdiv<R, EX>(SR * Fi[u] - SL * Fj[u] + SL * SR * (Uj[u] - Ui[u]) * na, SR - SL);
            } else if (SR < R(0)) {
              for (int u = 0; u < U; u++) Fh[u] = Fj[u];
            } else {
              for (int u = 0; u < U; u++) Fh[u] = R(0);
            }
            for (int b = 0; b < B; b++)
              for (int u = 0; u < U; u++) DFn[b][u] += Fh[u] * Nb[b] * gw;
          }
        }
        }
        const R Sj = EX ? (R)fc.S : fr.S;
        for (int b = 0; b < B; b++)
          for (int u = 0; u < U; u++) dc[u][b] += (-DFn[b][u] * na) * Sj;
      }
      if constexpr (MODE == 2) continue;
      for (int u = 0; u < U; u++)
        for (int b = 0; b < B; b++) P.cdcoef[((ss * U + u) * B + b) * nc + ci] = dc[u][b] * inv[b];
    }
  }
  if (ncall) {
    atomicAdd(&P.cnt->mgfm_calls, ncall);
    atomicAdd(&P.cnt->mgfm_iters, nit);
    if (nmax) atomicAdd(&P.cnt->mgfm_maxit, nmax);
  }
}

/* interface problems of each cell: present phase x interior face x quadrature
 * point x other neighbour phase present (the MGFM calls of particle_flow.cpp:192-204) */
template <int D, typename R, bool EX>
__global__ void k_iface_count(CaseK K, DevPtrs<R> P, unsigned long long* cnt) {
  const int64_t nc = K.ncell;
  constexpr int NQ = (D == 3) ? 4 : 2;
  GRID_STRIDE(ci, nc) {
    unsigned long long n = 0;
    if (P.cused[ci]) {
      int idx[3];
      cijk<D>(K, ci, idx);
      for (int f = 0; f < 2 * D; f++) {
        const int a = (f == 0 || f == 2) ? 1 : (f == 1 || f == 3) ? 0 : 2;
        const int sg = (f == 0 || f == 3 || f == 4) ? -1 : 1;
        int nb[3] = {idx[0], idx[1], idx[2]};
        nb[a] += sg;
        if (nb[a] < 0 || nb[a] >= K.N[a]) continue;
        const int64_t cn = cidx3(K, nb[0], nb[1], nb[2]);
        for (int ss = 0; ss < F; ss++) {
          if (P.cph[ss * nc + ci] != 1) continue;
          for (int s1 = 0; s1 < F; s1++)
            if (s1 != ss && P.calph[s1 * nc + cn] != R(0)) n += NQ;
        }
      }
    }
    cnt[ci] = n;
  }
}
template <typename R, bool EX>
__global__ void k_iface_total(const unsigned long long* blk, int nblk, unsigned long long* off, int64_t nc,
                              unsigned long long* tot, int64_t cap) {
  const unsigned long long n = blk[nblk];
  off[nc] = n;
  tot[0] = n;
  tot[1] = n <= (unsigned long long)cap ? n : 0ull; /* an overflowing stage batches nothing */
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::grid_acc(const CaseK& K, const DevPtrs<R>& P, cudaStream_t st) {
  double voli = K.ps[0] * K.ps[1];
  if (D == 3) voli = voli * K.ps[2];
  double ps[3] = {K.ps[0] / 2, K.ps[1] / 2, K.ps[2] / 2};
  double m1 = (ps[0] * ps[0] / 3.) * voli, m2 = (ps[1] * ps[1] / 3.) * voli, m3 = (ps[2] * ps[2] / 3.) * voli;
  IfaceQ Q{};
  k_grid_acc<D, R, EX, 0><<<grid_for(K.ncell, 128), 128, 0, st>>>(K, P, K.mgfm_variant, voli, m1, m2, m3, Q);
}

/* count, offsets and gather of the stage's interface problems, all on the
 * device: the count is never read back; a stage with more problems than the
 * queue holds batches none of them and the residual solves it inline */
template <int D, typename R, bool EX>
void Launch<D, R, EX>::iface_gather(const CaseK& K, const DevPtrs<R>& P, IfaceQ Q, cudaStream_t st) {
  double voli = K.ps[0] * K.ps[1];
  if (D == 3) voli = voli * K.ps[2];
  k_iface_count<D, R, EX><<<grid_for(K.ncell, BLK), BLK, 0, st>>>(K, P, Q.off);
  scan_u64(Q.off, Q.blk, Q.d_ncell, K.ncell, st);
  const int nblk = (int)((K.ncell + 2047) / 2048);
  k_iface_total<R, EX><<<1, 1, 0, st>>>(Q.blk, nblk, Q.off, K.ncell, Q.tot, Q.cap);
  k_grid_acc<D, R, EX, 2><<<grid_for(K.ncell, 128), 128, 0, st>>>(K, P, K.mgfm_variant, voli, 0, 0, 0, Q);
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::grid_acc_queued(const CaseK& K, const DevPtrs<R>& P, IfaceQ Q, cudaStream_t st) {
  double voli = K.ps[0] * K.ps[1];
  if (D == 3) voli = voli * K.ps[2];
  double ps[3] = {K.ps[0] / 2, K.ps[1] / 2, K.ps[2] / 2};
  double m1 = (ps[0] * ps[0] / 3.) * voli, m2 = (ps[1] * ps[1] / 3.) * voli, m3 = (ps[2] * ps[2] / 3.) * voli;
  k_grid_acc<D, R, EX, 3><<<grid_for(K.ncell, 128), 128, 0, st>>>(K, P, K.mgfm_variant, voli, m1, m2, m3, Q);
  /* the inline solve of a stage that outgrew the queue (returns at once otherwise) */
  k_grid_acc<D, R, EX, 0><<<grid_for(K.ncell, 128), 128, 0, st>>>(K, P, K.mgfm_variant, voli, m1, m2, m3, Q);
}

/* ------------------------------------------------------------------ */
/* Update_grid (mpm.cpp:768-830)                                      */
/* ------------------------------------------------------------------ */
template <int D, typename R, bool EX>
__global__ void __launch_bounds__(256) k_update_grid(CaseK K, DevPtrs<R> P, int md) {
  constexpr int U = D + 2, B = D + 1;
  const int64_t nc = K.ncell;
  const R dt = (R)P.cnt->dt;
  GRID_STRIDE(ci, nc) {
    if (!P.cused[ci]) continue;
    R rhov_a[3] = {0, 0, 0}, rho_a = 0, P_a = 0;
    R vcur[3];
    for (int k = 0; k < D; k++) vcur[k] = P.cv[k * nc + ci];
    R Pc = P.cP[ci];
    for (int s = 0; s < F; s++) {
      R c_s = 0, ac_s = 0;
      /* restrict-qualified bases: the loads of later coefficients may run ahead
       * of the stores of earlier ones */
      R* __restrict__ cf = P.ccoef + (int64_t)(s * U * B) * nc + ci;
      R* __restrict__ dcf = P.cdcoef + (int64_t)(s * U * B) * nc + ci;
      R* __restrict__ c0f = P.ccoef0 + (int64_t)(s * U * B) * nc + ci;
      const bool present = P.cph[s * nc + ci] == 1;
      R lim[U];
#pragma unroll
      for (int u = 0; u < U; u++) lim[u] = fabs(P.clim[(s * U + u) * nc + ci]);
      R co0 = R(0), cE = R(0), d00 = R(0), crv[3] = {0, 0, 0}, drv[3] = {0, 0, 0};
#pragma unroll
      for (int t = 0; t < U * B; t++) {
        const int u = t / B, b = t % B;
        const int64_t o = (int64_t)t * nc;
        R co = cf[o], d = dcf[o];
        if (b >= 1) {
          d *= lim[u];
          co *= lim[u];
        }
        if (present) {
          if (md == 0) {
            c0f[o] = co;
            co = co + d * dt;
          } else {
            co = R(0.5) * (d * dt + co + c0f[o]);
          }
          dcf[o] = d;
          cf[o] = co;
        } else if (b >= 1) {
          dcf[o] = d;
          cf[o] = co;
        }
        if (b == 0) {
          if (u == 0) {
            co0 = co;
            d00 = d;
          } else if (u <= D) {
            crv[u - 1] = co;
            drv[u - 1] = d;
          } else {
            cE = co;
          }
        }
      }
      const R alph = P.calph[s * nc + ci];
      if (present) {
        R rho = co0;
        P.crho[s * nc + ci] = rho;
        R sq = R(0);
        for (int k = 0; k < D; k++) {
          R rv = crv[k];
          P.crhov[(s * D + k) * nc + ci] = rv;
          sq = (k == 0) ? rv * rv : sq + rv * rv;
        }
        R E = cE;
        P.cE[s * nc + ci] = E;
        Pc = eos_p<R>(E - R(0.5) * sq / rho, (R)K.gamma[s], (R)K.pinf_eos[s]);
        c_s = sqrt_r<R>((R)K.gamma[s] * ((R)K.pinf[s] + Pc) / rho);
        R asq = R(0);
        for (int k = 0; k < D; k++) {
          R ak = (drv[k] - d00 * vcur[k]) / rho;
          asq = (k == 0) ? ak * ak : asq + ak * ak;
        }
        ac_s = sqrt_r<R>(asq);
      }
      P.cc[s * nc + ci] = c_s;
      P.cac[s * nc + ci] = ac_s;
      for (int k = 0; k < D; k++) rhov_a[k] += P.crhov[(s * D + k) * nc + ci] * alph;
      rho_a += P.crho[s * nc + ci] * alph;
      P_a += Pc * alph;
    }
    for (int k = 0; k < D; k++) P.cv[k * nc + ci] = rhov_a[k] / rho_a;
    P.cP[ci] = P_a;
  }
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::update_grid(const CaseK& K, const DevPtrs<R>& P, int md, cudaStream_t st) {
  k_update_grid<D, R, EX><<<grid_for(K.ncell, BLK), BLK, 0, st>>>(K, P, md);
}

/* ------------------------------------------------------------------ */
/* conservation totals (Triple_point_2phase/mpm_ini.cpp:599-654)       */
/* ------------------------------------------------------------------ */
/* Sums in double-double (an error-free TwoSum of each addend, the errors summed
 * beside the running sum: Neumaier's compensated summation), rounded once: the
 * result agrees with the exactly rounded sum but for sums within about
 * n^2 eps^2 of a rounding boundary, whatever the order of the addends, so the
 * parallel reduction here and the oracle's serial loop give the same double.
 * (Internal linkage: this file is compiled twice, for the exact and the other
 * paths.) */
namespace {
struct DD {
  double hi, lo;
};
__device__ __forceinline__ void dd_add(DD& a, double b) {
  const double s = a.hi + b;
  const double bb = s - a.hi;
  a.lo += (a.hi - (s - bb)) + (b - bb);
  a.hi = s;
}
__device__ __forceinline__ void dd_merge(DD& a, const DD& b) {
  dd_add(a, b.hi);
  a.lo += b.lo;
}
constexpr int TOT_BLOCKS = 304, TOT_THREADS = 256;
/* totals: particle mass per phase, particle energy, cell mass per phase, cell energy */
constexpr int NTOT = 2 * F + 2;
constexpr size_t PROBE_DOUBLES = 6 * (size_t)TOT_BLOCKS; /* the bubble probe's block partials */
/* the blocks' partial sums in block order, rounded once */
__global__ void k_totals_final(const DD* part, double* out) {
  if (threadIdx.x < NTOT) {
    DD t = part[threadIdx.x];
    for (int b = 1; b < TOT_BLOCKS; b++) dd_merge(t, part[b * NTOT + threadIdx.x]);
    out[threadIdx.x] = t.hi + t.lo;
  }
}
__global__ void k_probe_final(const double* part, double* out) {
  if (threadIdx.x == 0) {
    double r[6] = {part[0], part[1], part[2], 0, 0, part[5]};
    DD m{part[3], part[4]};
    for (int b = 1; b < TOT_BLOCKS; b++) {
      r[0] = fmax(r[0], part[b * 6 + 0]);
      r[1] = fmin(r[1], part[b * 6 + 1]);
      r[2] = fmin(r[2], part[b * 6 + 2]);
      dd_merge(m, DD{part[b * 6 + 3], part[b * 6 + 4]});
      r[5] += part[b * 6 + 5];
    }
    out[0] = r[0];
    out[1] = r[1];
    out[2] = r[2];
    out[3] = m.hi + m.lo;
    out[4] = r[5];
  }
}
}  // namespace

template <int D, typename R, bool EX>
__global__ void __launch_bounds__(TOT_THREADS) k_totals(CaseK K, DevPtrs<R> P, DD* part) {
  DD acc[NTOT];
  for (int k = 0; k < NTOT; k++) acc[k] = DD{0.0, 0.0};
  const int64_t n = (int64_t)P.cnt->n_slots;
  GRID_STRIDE(p, n) {
    int ph = P.phase[p];
    if (ph == 0) continue;
    dd_add(acc[ph - 1], (double)P.rho[p] * (double)P.vol[p]);
    double e = (double)P.E[p];
    if (K.eshift[ph - 1] != 0.0) e += K.eshift[ph - 1];
    dd_add(acc[F], e * (double)P.vol[p]);
  }
  const int64_t nc = K.ncell;
  double voli = K.ps[0] * K.ps[1] * (D == 3 ? K.ps[2] : 1.0);
  GRID_STRIDE(ci, nc) {
    if (!P.cused[ci]) continue;
    for (int s = 0; s < F; s++) {
      if (P.cph[s * nc + ci] != 1) continue;
      double a = (double)P.calph[s * nc + ci];
      dd_add(acc[F + 1 + s], voli * a * (double)P.crho[s * nc + ci]);
      double e = (double)P.cE[s * nc + ci];
      if (K.eshift[s] != 0.0) e += K.eshift[s];
      dd_add(acc[2 * F + 1], voli * a * e);
    }
  }
  __shared__ DD s_w[TOT_THREADS / 32][NTOT];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int k = 0; k < NTOT; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      DD b{__shfl_down_sync(0xffffffffu, acc[k].hi, o), __shfl_down_sync(0xffffffffu, acc[k].lo, o)};
      if (lane + o < 32) dd_merge(acc[k], b);
    }
    if (lane == 0) s_w[w][k] = acc[k];
  }
  __syncthreads();
  if (threadIdx.x < NTOT) {
    DD t = s_w[0][threadIdx.x];
    for (int v = 1; v < TOT_THREADS / 32; v++) dd_merge(t, s_w[v][threadIdx.x]);
    part[blockIdx.x * NTOT + threadIdx.x] = t;
  }
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::totals(const CaseK& K, const DevPtrs<R>& P, double* d_out, cudaStream_t st) {
  /* d_out holds the 2F + 2 results followed by the blocks' partials (totals_scratch) */
  DD* part = reinterpret_cast<DD*>(d_out + NTOT + (NTOT & 1));
  k_totals<D, R, EX><<<TOT_BLOCKS, TOT_THREADS, 0, st>>>(K, P, part);
  k_totals_final<<<1, 32, 0, st>>>(part, d_out);
}
template <int D, typename R, bool EX>
size_t Launch<D, R, EX>::totals_scratch() {
  return NTOT + (NTOT & 1) + 2 * NTOT * (size_t)TOT_BLOCKS + PROBE_DOUBLES;
}

/* ------------------------------------------------------------------ */
/* bubble probe (Output_point, mpm_ini.cpp:774-824)                   */
/* ------------------------------------------------------------------ */
/* Over the phase-2 particles: the largest and smallest x of those near the
 * axis (y and z below 2.5 p_sz: the bubble's downstream end and the jet) and
 * the smallest x of those away from it (y or z above 4 p_sz: the upstream
 * end), the phase-2 mass sum rho vol, and the number of fluid particles.
 * Per-block partials, combined in block order (deterministic). */
template <int D, typename R, bool EX>
__global__ void __launch_bounds__(TOT_THREADS) k_probe(CaseK K, DevPtrs<R> P, double* part) {
  double dw = K.bl[0], jet = K.br[0], ups = K.br[0];
  DD mass{0.0, 0.0};
  unsigned long long cnt = 0;
  const R* X = P.X[P.xb];
  const double a = 2.5 * K.p_sz, b = 4 * K.p_sz;
  const int64_t n = (int64_t)P.cnt->n_slots;
  GRID_STRIDE(p, n) {
    const int ph = P.phase[p];
    if (ph == 0) continue;
    cnt++;
    if (ph != 2) continue;
    const double x = (double)X[p], y = (double)X[K.cap + p], z = D == 3 ? (double)X[2 * K.cap + p] : 0.0;
    if (y < a && z < a) {
      dw = fmax(dw, x);
      jet = fmin(jet, x);
    } else if (y > b || z > b) {
      ups = fmin(ups, x);
    }
    dd_add(mass, (double)P.rho[p] * (double)P.vol[p]);
  }
  __shared__ double s_v[TOT_THREADS / 32][6];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double c = (double)cnt;
  for (int o = 16; o > 0; o >>= 1) {
    const double dw2 = __shfl_down_sync(0xffffffffu, dw, o), jet2 = __shfl_down_sync(0xffffffffu, jet, o);
    const double ups2 = __shfl_down_sync(0xffffffffu, ups, o);
    DD m2{__shfl_down_sync(0xffffffffu, mass.hi, o), __shfl_down_sync(0xffffffffu, mass.lo, o)};
    const double c2 = __shfl_down_sync(0xffffffffu, c, o);
    if (lane + o < 32) {
      dw = fmax(dw, dw2);
      jet = fmin(jet, jet2);
      ups = fmin(ups, ups2);
      dd_merge(mass, m2);
      c += c2;
    }
  }
  if (lane == 0) {
    s_v[w][0] = dw;
    s_v[w][1] = jet;
    s_v[w][2] = ups;
    s_v[w][3] = mass.hi;
    s_v[w][4] = mass.lo;
    s_v[w][5] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[6] = {s_v[0][0], s_v[0][1], s_v[0][2], 0, 0, s_v[0][5]};
    DD m{s_v[0][3], s_v[0][4]};
    for (int v = 1; v < TOT_THREADS / 32; v++) {
      r[0] = fmax(r[0], s_v[v][0]);
      r[1] = fmin(r[1], s_v[v][1]);
      r[2] = fmin(r[2], s_v[v][2]);
      dd_merge(m, DD{s_v[v][3], s_v[v][4]});
      r[5] += s_v[v][5];
    }
    r[3] = m.hi;
    r[4] = m.lo;
    for (int k = 0; k < 6; k++) part[blockIdx.x * 6 + k] = r[k];
  }
}
template <int D, typename R, bool EX>
void Launch<D, R, EX>::probe(const CaseK& K, const DevPtrs<R>& P, double* d_scratch, double* d_out5,
                             cudaStream_t st) {
  /* d_scratch: the totals scratch; the probe's partials use its last PROBE_DOUBLES */
  double* part = d_scratch + totals_scratch() - PROBE_DOUBLES;
  k_probe<D, R, EX><<<TOT_BLOCKS, TOT_THREADS, 0, st>>>(K, P, part);
  k_probe_final<<<1, 32, 0, st>>>(part, d_out5);
}

#define PGDG_INST(D, R, EX)                                                                     \
  template void Launch<D, R, EX>::used_state(const CaseK&, const DevPtrs<R>&, cudaStream_t);       \
  template void Launch<D, R, EX>::set_timestep(const CaseK&, const DevPtrs<R>&, int, cudaStream_t); \
  template void Launch<D, R, EX>::add_time(const DevPtrs<R>&, cudaStream_t);                       \
  template void Launch<D, R, EX>::p2g(const CaseK&, const DevPtrs<R>&, bool, cudaStream_t);        \
  template void Launch<D, R, EX>::p2g_new(const CaseK&, const DevPtrs<R>&, cudaStream_t);          \
  template void Launch<D, R, EX>::limiter(const CaseK&, const DevPtrs<R>&, cudaStream_t);          \
  template void Launch<D, R, EX>::grid_acc(const CaseK&, const DevPtrs<R>&, cudaStream_t);         \
  template void Launch<D, R, EX>::iface_gather(const CaseK&, const DevPtrs<R>&, IfaceQ, cudaStream_t); \
  template void Launch<D, R, EX>::grid_acc_queued(const CaseK&, const DevPtrs<R>&, IfaceQ, cudaStream_t); \
  template void Launch<D, R, EX>::update_grid(const CaseK&, const DevPtrs<R>&, int, cudaStream_t); \
  template void Launch<D, R, EX>::totals(const CaseK&, const DevPtrs<R>&, double*, cudaStream_t);  \
  template size_t Launch<D, R, EX>::totals_scratch();                                             \
  template void Launch<D, R, EX>::probe(const CaseK&, const DevPtrs<R>&, double*, double*, cudaStream_t);
#ifdef PGDG_EXACT_TU
PGDG_INST(2, double, true)
#if PGDG_WITH_3D
PGDG_INST(3, double, true)
#endif
#else
PGDG_INST(2, double, false)
#if PGDG_WITH_3D
PGDG_INST(3, double, false)
#endif
PGDG_INST(2, float, false)
#if PGDG_WITH_3D
PGDG_INST(3, float, false)
#endif
#endif

}  // namespace pgdg
