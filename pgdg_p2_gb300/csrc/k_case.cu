/*
 * k_case.cu -- the synthetic workloads built on the device (MPM::Initialize_case,
 * mpm_ini.cpp:33-673, for the fluid particles and cells): the context's particle
 * and cell arrays are written in place, with the values the host builder
 * (case_builder.cpp) produces, so a case needs no upload of its state.
 *
 * One thread per lattice particle and per cell.  The particle mathematics is
 * case_math.h, shared with the host builder; this file is compiled without FMA
 * contraction, so the FP64 values match the host's bit for bit before they are
 * stored in the context's precision (with the energy shift the upload applies
 * on the FP32 path).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "case_math.h"
#include "pgdg_dev.cuh"

namespace pgdg {

using namespace pgdg_case_math;

struct CaseGen {
  int id, D, na[3];
  double box_l[3], p_sz, jit, vol0, h0, gam[PGDG_MAX_FLD], pinf[PGDG_MAX_FLD], ps[3], c_ini[PGDG_MAX_FLD];
  uint64_t seed;
};

template <typename R>
__global__ void k_case_particles(CaseK K, DevPtrs<R> P, CaseGen G, int64_t n) {
  const int NS = (G.D + 2) * G.D;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(p % G.na[2]);
    const int j = (int)((p / G.na[2]) % G.na[1]);
    const int i = (int)(p / ((int64_t)G.na[1] * G.na[2]));
    const PState0 s = lattice_particle(G.id, G.D, G.box_l, G.p_sz, G.jit, G.seed, p, i, j, k, G.vol0, G.h0, G.gam,
                                       G.pinf, G.ps);
    const int ph = s.phase - 1;
    for (int d = 0; d < G.D; d++) {
      P.X[0][d * K.cap + p] = (R)s.x[d];
      P.rhov[d * K.cap + p] = (R)s.rhov[d];
      P.v[d * K.cap + p] = (R)s.u[d];
      P.tv[d * K.cap + p] = R(0);
    }
    for (int t = 0; t < NS; t++) P.sl[t * K.cap + p] = R(0);
    P.vol[p] = (R)s.vol;
    P.mass[p] = (R)s.mass;
    P.H[0][p] = (R)s.h;
    P.P[p] = (R)s.P;
    P.rho[p] = (R)s.rho;
    P.E[p] = (R)(s.E - K.eshift[ph]);
    P.c[p] = (R)s.c;
    P.phase[p] = (int8_t)s.phase;
    P.mark_in[p] = 0;
    P.seq[p] = (uint64_t)p;
    P.list_len[p] = 0;
    P.list_off[p] = 0;
  }
}

/* every cell: each phase at its absent-phase density, zero momentum, energy and
 * coefficients, limiter 1, present flag 1 (mpm_ini.cpp:299-346) */
template <int D, typename R>
__global__ void k_case_cells(CaseK K, DevPtrs<R> P, CaseGen G) {
  constexpr int U = D + 2, B = D + 1;
  const int64_t nc = K.ncell;
  for (int64_t ci = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ci < nc; ci += (int64_t)gridDim.x * blockDim.x) {
    for (int s = 0; s < F; s++) {
      P.crho[s * nc + ci] = (R)K.ini_rho[s];
      for (int d = 0; d < D; d++) P.crhov[(s * D + d) * nc + ci] = R(0);
      P.cE[s * nc + ci] = (R)(0.0 - K.eshift[s]);
      P.cc[s * nc + ci] = (R)G.c_ini[s];
      P.cac[s * nc + ci] = R(0);
      P.calph[s * nc + ci] = R(0);
      for (int t = 0; t < U * B; t++) {
        P.ccoef[(s * U * B + t) * nc + ci] = (t == (U - 1) * B) ? (R)(0.0 - K.eshift[s]) : R(0);
        P.cdcoef[(s * U * B + t) * nc + ci] = R(0);
      }
      for (int u = 0; u < U; u++) P.clim[(s * U + u) * nc + ci] = R(1);
      P.cph[s * nc + ci] = 1;
      P.cphb[s * nc + ci] = 0;
    }
    for (int t = 0; t < D * D; t++) P.cgv[t * nc + ci] = R(0);
    for (int d = 0; d < D; d++) P.cv[d * nc + ci] = R(0);
    P.cP[ci] = R(0);
    P.cused[ci] = 1;
  }
}

template <int D, typename R>
int case_build(const CaseK& K, const DevPtrs<R>& P, const pgdg_case& cs, int id, uint64_t seed, int64_t n,
               cudaStream_t st) {
  CaseGen G{};
  G.id = id;
  G.D = D;
  for (int d = 0; d < 3; d++) {
    G.na[d] = d < D ? (int)std::lround((cs.box_r[d] - cs.box_l[d]) / cs.p_sz) : 1;
    G.box_l[d] = cs.box_l[d];
  }
  G.p_sz = cs.p_sz;
  G.jit = jittered(id) ? cs.p_g / 8.0 : 0.0;
  double vol0 = 1;
  for (int d = 0; d < D; d++) vol0 *= cs.p_sz;
  G.vol0 = vol0;
  G.h0 = 3.2 / 2. * cs.p_sz;
  for (int s = 0; s < F; s++) {
    G.gam[s] = cs.gamma[s];
    G.pinf[s] = cs.pinf[s];
    G.c_ini[s] = cs.c_ini[s];
  }
  post_shock(G.ps[0], G.ps[1], G.ps[2], std::sqrt(1.4 * 1.0 / 1.0));
  G.seed = seed ? seed : 20260101ull;
  const int64_t np = (int64_t)G.na[0] * G.na[1] * G.na[2];
  if (np != n) return PGDG_EINVAL;
  const int64_t gp = std::min<int64_t>((n + 255) / 256, 152 * 32), gc = std::min<int64_t>((K.ncell + 255) / 256, 152 * 32);
  k_case_particles<R><<<(int)std::max<int64_t>(gp, 1), 256, 0, st>>>(K, P, G, n);
  k_case_cells<D, R><<<(int)std::max<int64_t>(gc, 1), 256, 0, st>>>(K, P, G);
  return cudaGetLastError() == cudaSuccess ? PGDG_OK : PGDG_ECUDA;
}

template int case_build<2, float>(const CaseK&, const DevPtrs<float>&, const pgdg_case&, int, uint64_t, int64_t,
                                  cudaStream_t);
#if PGDG_WITH_3D
template int case_build<3, float>(const CaseK&, const DevPtrs<float>&, const pgdg_case&, int, uint64_t, int64_t,
                                  cudaStream_t);
#endif
template int case_build<2, double>(const CaseK&, const DevPtrs<double>&, const pgdg_case&, int, uint64_t, int64_t,
                                   cudaStream_t);
#if PGDG_WITH_3D
template int case_build<3, double>(const CaseK&, const DevPtrs<double>&, const pgdg_case&, int, uint64_t, int64_t,
                                   cudaStream_t);
#endif

}  // namespace pgdg
