/*
 * k_output.cu -- the device half of the snapshot writers (MPM::Output_plt_file,
 * mpm_ini.cpp:832-980): the live particles' twelve output variables and the
 * cells' twelve stored output columns are packed, in canonical order, into
 * snapshot buffers that the host copies out and formats while the device goes
 * on stepping.
 *
 * Particle variables (the file's order): x, y, z, phase, vx, vy, vol, rho, P,
 * |tv|, |v| (norms over the first D components, left to right), and
 * n_neighbor = the size of the particle's flag-2 neighbour list
 * (Level_info::Refresh_neighbor_info, level_infor.cpp:153-195): the fluid and
 * boundary particles binned in the cells within rad2 of the particle's cell
 * whose distance is at most 2h, the particle itself included.  The lists
 * exist only inside the shifting kernel here, so they are counted again over
 * the coordinates and smoothing lengths the last stage searched with.
 *
 * Cell columns (after the centre, which the host computes): v0, v1, |v|,
 * rho[0], rho[1], coef[0](1,1), coef[0](1,2), Lim_u[0](0), Lim_u[1](0),
 * alph[0], alph[1], P.
 *
 * Compiled twice like the grid kernels: with FMA contraction for the mixed and
 * FP64_FMA paths and without it (-DPGDG_EXACT_TU) for the exact path, whose
 * counts and norms then equal the oracle's bit for bit.
 */
#include <cuda_runtime.h>

#include "pgdg_dev.cuh"
#include "pgdg_math.cuh"

namespace pgdg {

namespace {

/* the membership test of the shifting sum (PstPart::member): distance at most
 * 2h, as the exact path and the reference write it or as a squared comparison */
template <int D, typename R, bool EX>
__device__ __forceinline__ bool within_2h(const R* xp, const R* xq, R hs, R lim2) {
  R dd = R(0);
  for (int d = 0; d < D; d++) {
    const R t = xp[d] - xq[d];
    dd = (d == 0) ? t * t : dd + t * t;
  }
  if constexpr (EX) return sqrt_r<R>(dd) <= hs * R(CUT_OFF);
  else return dd <= lim2;
}

template <int D, typename R, bool EX>
__global__ void k_pack_particles(CaseK K, DevPtrs<R> P, const int64_t* __restrict__ alive, int64_t n, int xs,
                                 int hs, double* __restrict__ dv, int32_t* __restrict__ iv) {
  const R* X = P.X[P.xb];
  const R* XS = P.X[xs];
  const R* HS = P.H[hs];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = alive[i];
    dv[0 * n + i] = (double)X[p];
    dv[1 * n + i] = (double)X[K.cap + p];
    dv[2 * n + i] = D == 3 ? (double)X[2 * K.cap + p] : 0.0;
    iv[i] = (int32_t)P.phase[p];
    double vv[3], tt[3];
    for (int d = 0; d < D; d++) {
      vv[d] = (double)P.v[d * K.cap + p];
      tt[d] = (double)P.tv[d * K.cap + p];
    }
    dv[3 * n + i] = vv[0];
    dv[4 * n + i] = vv[1];
    dv[5 * n + i] = (double)P.vol[p];
    dv[6 * n + i] = (double)P.rho[p];
    dv[7 * n + i] = (double)P.P[p];
    double qt = tt[0] * tt[0], qv = vv[0] * vv[0];
    for (int d = 1; d < D; d++) {
      qt = qt + tt[d] * tt[d];
      qv = qv + vv[d] * vv[d];
    }
    dv[8 * n + i] = sqrt(qt);
    dv[9 * n + i] = sqrt(qv);
    /* the flag-2 list size */
    R xp[3] = {R(0), R(0), R(0)};
    for (int d = 0; d < D; d++) xp[d] = XS[d * K.cap + p];
    const R h = HS[p];
    const R lim2 = (h * R(CUT_OFF)) * (h * R(CUT_OFF));
    int pos[3];
    cell_pos<D, R>(K, xp, pos);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      const int r = (d < D) ? K.rad2 : 0;
      lo[d] = max(pos[d] - r, 0);
      hi[d] = min(pos[d] + r, (d < D ? K.N[d] : 1) - 1);
    }
    int32_t cnt = 0;
    for (int t = lo[0]; t <= hi[0]; t++)
      for (int s = lo[1]; s <= hi[1]; s++)
        for (int m = lo[2]; m <= hi[2]; m++) {
          const int64_t c = ((int64_t)t * K.N[1] + s) * K.N[2] + m;
          const int nb = min(P.bcnt[c], K.maxpc);
          for (int r = 0; r < nb; r++) {
            const int32_t q = P.bucket[c * K.maxpc + r];
            R xq[3];
            for (int d = 0; d < D; d++) xq[d] = XS[d * K.cap + q];
            cnt += within_2h<D, R, EX>(xp, xq, h, lim2) ? 1 : 0;
          }
          for (int e = P.boff[c]; e < P.boff[c + 1]; e++) {
            const int32_t b = P.bent[e];
            R xq[3];
            for (int d = 0; d < D; d++) xq[d] = P.bx[d * K.nbnd + b];
            cnt += within_2h<D, R, EX>(xp, xq, h, lim2) ? 1 : 0;
          }
        }
    iv[n + i] = cnt;
  }
}

template <int D, typename R>
__global__ void k_pack_cells(CaseK K, DevPtrs<R> P, double* __restrict__ dc) {
  constexpr int U = D + 2, B = D + 1;
  const int64_t nc = K.ncell;
  for (int64_t ci = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ci < nc; ci += (int64_t)gridDim.x * blockDim.x) {
    double* o = dc + 12 * ci;
    double v[3];
    for (int d = 0; d < D; d++) v[d] = (double)P.cv[d * nc + ci];
    double q = v[0] * v[0];
    for (int d = 1; d < D; d++) q = q + v[d] * v[d];
    o[0] = v[0];
    o[1] = v[1];
    o[2] = sqrt(q);
    o[3] = (double)P.crho[0 * nc + ci];
    o[4] = (double)P.crho[1 * nc + ci];
    o[5] = (double)P.ccoef[((0 * U + 1) * B + 1) * nc + ci];
    o[6] = (double)P.ccoef[((0 * U + 1) * B + 2) * nc + ci];
    o[7] = (double)P.clim[(0 * U + 0) * nc + ci];
    o[8] = (double)P.clim[(1 * U + 0) * nc + ci];
    o[9] = (double)P.calph[0 * nc + ci];
    o[10] = (double)P.calph[1 * nc + ci];
    o[11] = (double)P.cP[ci];
  }
}

}  // namespace

template <int D, typename R, bool EX>
void output_pack_particles(const CaseK& K, const DevPtrs<R>& P, const int64_t* alive, int64_t n, int xs, int hs,
                           double* dv, int32_t* iv, cudaStream_t st) {
  if (n <= 0) return;
  k_pack_particles<D, R, EX><<<grid_for(n, 128), 128, 0, st>>>(K, P, alive, n, xs, hs, dv, iv);
}

template <int D, typename R, bool EX>
void output_pack_cells(const CaseK& K, const DevPtrs<R>& P, double* dc, cudaStream_t st) {
  k_pack_cells<D, R><<<grid_for(K.ncell, 256), 256, 0, st>>>(K, P, dc);
}

#define PGDG_OUT_INST(D, R, EX)                                                                            \
  template void output_pack_particles<D, R, EX>(const CaseK&, const DevPtrs<R>&, const int64_t*, int64_t, int, \
                                                int, double*, int32_t*, cudaStream_t);                        \
  template void output_pack_cells<D, R, EX>(const CaseK&, const DevPtrs<R>&, double*, cudaStream_t);
#ifdef PGDG_EXACT_TU
PGDG_OUT_INST(2, double, true)
#if PGDG_WITH_3D
PGDG_OUT_INST(3, double, true)
#endif
#else
PGDG_OUT_INST(2, double, false)
#if PGDG_WITH_3D
PGDG_OUT_INST(3, double, false)
#endif
PGDG_OUT_INST(2, float, false)
#if PGDG_WITH_3D
PGDG_OUT_INST(3, float, false)
#endif
#endif

}  // namespace pgdg
