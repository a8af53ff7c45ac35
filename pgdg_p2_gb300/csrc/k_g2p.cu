/*
 * k_g2p.cu -- Update_particle (mpm.cpp:839-853): grid-to-particle update
 * (Update_state_onestep, particle_flow.cpp:413-477) and particle shifting
 * (Update_PST / PST / Bound_pen, particle_flow.cpp:485-622).
 *
 * Two passes: every particle's G2P update completes before any particle's
 * shifting sum reads its neighbours (the reference runs both in one racy loop).
 * The shifting sum runs over the neighbour list of Refresh_neighbor_info(2)
 * (level_infor.cpp:153-195) -- particles within 2h at the stage-start positions --
 * which is recomputed on the fly from the stage-start coordinate buffer instead
 * of being stored.
 */
#include "pgdg_dev.cuh"

namespace pgdg {

constexpr int BLK = 256;
#define GRID_STRIDE(i, n) for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
                               i += (int64_t)gridDim.x * blockDim.x)

template <int D, typename R>
__device__ __forceinline__ R hroot(R vol);
template <>
__device__ __forceinline__ double hroot<2, double>(double vol) { return root_d(vol, 2) * CELL_RATIO / CUT_OFF; }
template <>
__device__ __forceinline__ double hroot<3, double>(double vol) { return root_d(vol, 3) * CELL_RATIO / CUT_OFF; }
template <>
__device__ __forceinline__ float hroot<2, float>(float vol) { return sqrtf(vol) * 3.2f / 2.f; }
template <>
__device__ __forceinline__ float hroot<3, float>(float vol) { return cbrtf(vol) * 3.2f / 2.f; }

template <int D, typename R, bool EX>
__global__ void __launch_bounds__(128) k_g2p(CaseK K, DevPtrs<R> P, int md, int xs, int x0b, int xn, int hn) {
  constexpr int U = D + 2, B = D + 1;
  const int64_t n = (int64_t)P.cnt->n_slots;
  const int64_t nc = K.ncell;
  const R dt = (R)P.cnt->dt;
  const R* XS = P.X[xs];
  const R* X0 = P.X[x0b];
  R* XN = P.X[xn];
  R* HN = P.H[hn];
  unsigned long long nfb = 0;
  GRID_STRIDE(p, n) {
    const int ph = P.phase[p];
    if (ph == 0) continue;
    const int ss = ph - 1;
    const int64_t ci = P.lcell[p];
    R divu = P.cgv[ci];
    for (int k = 1; k < D; k++) divu = divu + P.cgv[(k * D + k) * nc + ci];
    R x[3];
    R vol = P.vol[p];
    if (md == 0) {
      for (int d = 0; d < D; d++) x[d] = XS[d * K.cap + p] + P.tv[d * K.cap + p] * dt;
      P.vol0[p] = vol;
      vol = (R(1.) + divu * dt) * vol;
    } else {
      for (int d = 0; d < D; d++)
        x[d] = R(0.5) * ((X0[d * K.cap + p] + XS[d * K.cap + p]) + P.tv[d * K.cap + p] * dt);
      vol = R(0.5) * (P.vol0[p] + vol + divu * dt * vol);
    }
    int idx[3];
    idx[2] = (int)(ci % K.N[2]);
    idx[1] = (int)((ci / K.N[2]) % K.N[1]);
    idx[0] = (int)(ci / ((int64_t)K.N[1] * K.N[2]));
    R dri[3];
    for (int d = 0; d < D; d++) dri[d] = x[d] - (R(K.bl[d]) + R(K.ps[d]) * R(idx[d] + 0.5));
    R Ui[U];
    for (int t = 0; t < U; t++) {
      R acc = P.ccoef[((ss * U + t) * B + 1) * nc + ci] * dri[0];
      for (int b = 1; b < D; b++) acc = acc + P.ccoef[((ss * U + t) * B + 1 + b) * nc + ci] * dri[b];
      Ui[t] = P.ccoef[((ss * U + t) * B) * nc + ci] + acc;
    }
    R rho = Ui[0], E = Ui[U - 1];
    R rhov[3], v[3], sq = R(0);
    for (int k = 0; k < D; k++) {
      rhov[k] = Ui[1 + k];
      v[k] = rhov[k] / rho;
      sq = (k == 0) ? v[k] * v[k] : sq + v[k] * v[k];
    }
    const R g = (R)K.gamma[ss], pf = (R)K.pinf[ss];
    R Pp = eos_p<R>(E - R(0.5) * rho * sq, g, pf);
    R c = rsqrt_<R>(g * (pf + Pp) / rho);
    bool fb = (Pp < R(-0.05) * pf || rho < R(0));
    for (int t = 0; t < U; t++)
      for (int b = 0; b < D; b++)
        P.sl[(t * D + b) * K.cap + p] = fb ? R(0) : P.ccoef[((ss * U + t) * B + 1 + b) * nc + ci];
    if (fb) {
      rho = P.crho[ss * nc + ci];
      for (int k = 0; k < D; k++) rhov[k] = P.crhov[(ss * D + k) * nc + ci];
      E = P.cE[ss * nc + ci];
      c = P.cc[ss * nc + ci];
      nfb++;
    }
    for (int d = 0; d < D; d++) {
      XN[d * K.cap + p] = x[d];
      P.rhov[d * K.cap + p] = rhov[d];
      P.v[d * K.cap + p] = v[d];
    }
    P.vol[p] = vol;
    P.rho[p] = rho;
    P.E[p] = E;
    P.P[p] = Pp;
    P.c[p] = c;
    P.mass[p] = vol * rho;
    HN[p] = hroot<D, R>(vol);
  }
  if (nfb) atomicAdd(&P.cnt->g2p_fb, nfb);
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::g2p(const CaseK& K, const DevPtrs<R>& P, int md, int xs, int x0, int xn, int hn, cudaStream_t st) {
  k_g2p<D, R, EX><<<grid_for(K.cap, 128), 128, 0, st>>>(K, P, md, xs, x0, xn, hn);
}

/* ------------------------------------------------------------------ */
/* particle shifting                                                  */
/* ------------------------------------------------------------------ */
template <int D, typename R>
struct PstAcc {
  R pst[3], phs[3];
};

template <int D, typename R, bool EX>
__global__ void __launch_bounds__(128) k_pst(CaseK K, DevPtrs<R> P, int xs, int hs, int xn, int hn) {
  const int64_t n = (int64_t)P.cnt->n_slots;
  const R dt = (R)P.cnt->dt;
  const R max_v = (R)P.cnt->max_v;
  const R* XS = P.X[xs];
  const R* XN = P.X[xn];
  const R* HS = P.H[hs];
  const R* HN = P.H[hn];
  const R cdim = (D == 2) ? R(1.0 / PI_REF) : R(1.0 / PI_REF);
  GRID_STRIDE(p, n) {
    const int ph = P.phase[p];
    if (ph == 0) continue;
    R xsp[3], xnp[3];
    for (int d = 0; d < D; d++) {
      xsp[d] = XS[d * K.cap + p];
      xnp[d] = XN[d * K.cap + p];
    }
    const R hs_p = HS[p], hh = HN[p];
    const R lim2 = (hs_p * R(CUT_OFF)) * (hs_p * R(CUT_OFF));
    const R rho_p = P.rho[p], c_p = P.c[p];
    const R ca = max_v * R(5.);
    const R P_b = rho_p * ca * ca;
    const R hd = (D == 2) ? hh * hh : hh * hh * hh;
    const R C = (D == 2) ? cdim / hd * R(7. / 4.) : cdim / hd * R(21. / 16.);
    const R dxk = hh / R(CELL_RATIO) * R(CUT_OFF);
    R W_dp;
    {
      R s = dxk / hh;
      R q = R(1.) - R(0.5) * s;
      W_dp = (s < R(2)) ? C * (((q * q) * q) * q) * (R(1.) + R(2.) * s) : R(0);
    }
    const R tmp1c = -R(1.) * P_b * (R(1.) / rho_p);
    const R crho_p = c_p * c_p * rho_p;
    R pst[3] = {0, 0, 0}, phs[3] = {0, 0, 0};
    /* scan centre: cell of the stage-start position */
    int pos[3];
    cell_pos<D, R>(K, xsp, pos);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      int r = (d < D) ? K.rad2 : 0;
      lo[d] = max(pos[d] - r, 0);
      hi[d] = min(pos[d] + r, (d < D ? K.N[d] : 1) - 1);
    }
    auto pair = [&](const R* xsq, const R* xnq, R volq, R rhoq, R cq, int phq, const R* nq) {
      R dd = R(0);
      for (int d = 0; d < D; d++) {
        R t = xsp[d] - xsq[d];
        dd = (d == 0) ? t * t : dd + t * t;
      }
      if constexpr (EX) {
        if (!(rsqrt_<R>(dd) <= hs_p * R(CUT_OFF))) return;  /* get_distance <= h*CUT_OFF */
      } else {
        if (!(dd <= lim2)) return;
      }
      R dr[3];
      R d2 = R(0);
      for (int d = 0; d < D; d++) {
        dr[d] = xnp[d] - xnq[d];
        d2 = (d == 0) ? dr[d] * dr[d] : d2 + dr[d] * dr[d];
      }
      R dist = rsqrt_<R>(d2);
      if (dist == R(0)) return;
      R s = dist / hh;
      if (!(s < R(2))) {
        /* beyond the kernel support: W and dW vanish, but the boundary/interface
         * terms still see tmp1 = -P_b/rho (contributions are zero) */
        return;
      }
      R q = R(1.) - R(0.5) * s;
      R q3 = (q * q) * q;
      R Wij = C * (q3 * q) * (R(1.) + R(2.) * s);
      R aw = R(-5.) * C * q3 * s / hh / dist;
      R rr = Wij / W_dp;
      R Rr = R(0.2) * ((rr * rr) * (rr * rr));
      R tmp1 = tmp1c * (R(1) + Rr);
      if (phq != PGDG_PHASE_BOUNDARY) {
        for (int d = 0; d < D; d++) pst[d] += dr[d] * aw * tmp1 * volq;
        if (phq != ph) {
          R tmp2 = R(1.) / (rho_p + rhoq);
          R cs = R(-0.1) * tmp2 * (crho_p + cq * cq * rhoq);
          for (int d = 0; d < D; d++) phs[d] += cs * (dr[d] * aw) * volq;
        }
      } else {
        for (int d = 0; d < D; d++) pst[d] += nq[d] * Wij * tmp1 * volq;
      }
    };
    for (int t = lo[0]; t <= hi[0]; t++)
      for (int s = lo[1]; s <= hi[1]; s++)
        for (int m = lo[2]; m <= hi[2]; m++) {
          const int64_t c = ((int64_t)t * K.N[1] + s) * K.N[2] + m;
          const int cnt = min(P.bcnt[c], K.maxpc);
          const int32_t* bk = P.bucket + c * K.maxpc;
          int r = 0;
          /* Cell_list order: binned fluid particles, boundary particles, then appended ones */
          for (int pass = 0; pass < 3; pass++) {
            if (pass == 1) {
              for (int e = P.boff[c]; e < P.boff[c + 1]; e++) {
                int32_t b = P.bent[e];
                R xb[3], nb[3];
                for (int d = 0; d < D; d++) {
                  xb[d] = P.bx[d * K.nbnd + b];
                  nb[d] = P.bn[d * K.nbnd + b];
                }
                pair(xb, xb, (R)K.bvol, (R)K.brho, R(0), PGDG_PHASE_BOUNDARY, nb);
              }
              continue;
            }
            for (; r < cnt; r++) {
              int32_t q = bk[r];
              if (pass == 0 && P.lkey[q] >= KEY_APPEND) break;
              R xsq[3], xnq[3];
              for (int d = 0; d < D; d++) {
                xsq[d] = XS[d * K.cap + q];
                xnq[d] = XN[d * K.cap + q];
              }
              pair(xsq, xnq, P.vol[q], P.rho[q], P.c[q], P.phase[q], nullptr);
            }
          }
        }
    /* Bound_pen (particle_flow.cpp:587-622) on the faces of the particle's cell */
    R bp[3] = {0, 0, 0};
    {
      const int64_t ci = P.lcell[p];
      int idx[3];
      idx[2] = (int)(ci % K.N[2]);
      idx[1] = (int)((ci / K.N[2]) % K.N[1]);
      idx[0] = (int)(ci / ((int64_t)K.N[1] * K.N[2]));
      const int fax[6] = {1, 0, 1, 0, 2, 2};
      const int fsg[6] = {-1, 1, 1, -1, -1, 1};
      const int fside[6] = {2, 1, 3, 0, 4, 5};
      for (int f = 0; f < 2 * D; f++) {
        int a = fax[f];
        int nbi = idx[a] + fsg[f];
        if (nbi >= 0 && nbi < K.N[a]) continue;
        if (K.bc[fside[f]] == 0) continue;
        R cen = (R)(K.bl[a] + K.ps[a] * (idx[a] + 0.5) + fsg[f] * 0.5 * K.ps[a]);
        R nn = (R)fsg[f];
        R ds = (xnp[a] - cen) * nn;
        if (ds < R(0)) nn = -nn;
        R dis = fabs(ds);
        if (dis < R(0.4) * (R)K.p_sz) bp[a] += R(0.02) / dis * (c_p * c_p) * nn;
      }
    }
    /* Update_PST (particle_flow.cpp:485-525) */
    const R px = (R)K.p_sz;
    R dx[3], dx1[3], dx2[3];
    R s0 = 0, s1 = 0, s2 = 0;
    for (int d = 0; d < D; d++) {
      dx[d] = pst[d] * dt * dt / R(2.);
      dx1[d] = phs[d] * dt * dt / R(2.);
      dx2[d] = bp[d] * dt * dt / R(2.);
      s0 = (d == 0) ? dx[d] * dx[d] : s0 + dx[d] * dx[d];
      s1 = (d == 0) ? dx1[d] * dx1[d] : s1 + dx1[d] * dx1[d];
      s2 = (d == 0) ? dx2[d] * dx2[d] : s2 + dx2[d] * dx2[d];
    }
    R dis0 = rsqrt_<R>(s0), dis1 = rsqrt_<R>(s1), dis2 = rsqrt_<R>(s2);
    R l0 = amin1(px / R(10), dis0) / (dis0 + R(1e-20));
    R l1 = amin1(px / R(10), dis1) / (dis1 + R(1e-20));
    R l2 = amin1(px / R(2), dis2) / (dis2 + R(1e-20));
    const bool mk = P.mark_in[p] == 1;
    for (int d = 0; d < D; d++) {
      R dv = (dx[d] * l0 + dx1[d] * l1 + dx2[d] * l2) / dt;
      if (mk) dv = R(0);
      P.tv[d * K.cap + p] = P.v[d * K.cap + p] + dv;
    }
  }
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::pst(const CaseK& K, const DevPtrs<R>& P, int xs, int hs, int xn, int hn, cudaStream_t st) {
  k_pst<D, R, EX><<<grid_for(K.cap, 128), 128, 0, st>>>(K, P, xs, hs, xn, hn);
}

#define PGDG_INST(D, R, EX)                                                                              \
  template void Launch<D, R, EX>::g2p(const CaseK&, const DevPtrs<R>&, int, int, int, int, int, cudaStream_t); \
  template void Launch<D, R, EX>::pst(const CaseK&, const DevPtrs<R>&, int, int, int, int, cudaStream_t);
#ifdef PGDG_EXACT_TU
PGDG_INST(2, double, true)
PGDG_INST(3, double, true)
#else
PGDG_INST(2, double, false)
PGDG_INST(3, double, false)
PGDG_INST(2, float, false)
PGDG_INST(3, float, false)
#endif

}  // namespace pgdg
