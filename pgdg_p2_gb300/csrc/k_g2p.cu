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
#include <climits>
#include <type_traits>

#include "pgdg_dev.cuh"

namespace pgdg {

constexpr int BLK = 256;

/* 16- and 8-byte (FP32) or 32- and 16-byte (FP64) vector of R */
template <typename R>
struct Vec4;
template <>
struct Vec4<float> {
  using T = float4;
};
template <>
struct Vec4<double> {
  using T = double4;
};
template <typename R>
struct Vec2;
template <>
struct Vec2<float> {
  using T = float2;
};
template <>
struct Vec2<double> {
  using T = double2;
};
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
__global__ void __launch_bounds__(128, minblocks_f32<R>(8)) k_g2p(CaseK K, DevPtrs<R> P, int md, int xs, int x0b, int xn, int hn, int full) {
  constexpr int U = D + 2, B = D + 1;
  const int64_t n = (int64_t)P.cnt->n_slots;
  const int64_t nc = K.ncell;
  const R dt = (R)P.cnt->dt;
  const R* XS = P.X[xs];
  const R* X0 = P.X[x0b];
  R* XN = P.X[xn];
  R* HN = P.H[hn];
  unsigned long long nfb = 0;
  /* case constants in R, converted once per thread */
  R blr[3], psr[3], gam_r[F], pf_r[F], pfe_r[F];
  for (int d = 0; d < 3; d++) {
    blr[d] = R(K.bl[d]);
    psr[d] = R(K.ps[d]);
  }
  for (int s = 0; s < F; s++) {
    gam_r[s] = (R)K.gamma[s];
    pf_r[s] = (R)K.pinf[s];
    pfe_r[s] = (R)K.pinf_eos[s];
  }
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
    for (int d = 0; d < D; d++) dri[d] = x[d] - (blr[d] + psr[d] * ((R)idx[d] + R(0.5)));
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
    const R g = gam_r[ss], pf = pf_r[ss];
    R Pp = eos_p<R>(E - R(0.5) * rho * sq, g, pfe_r[ss]);
    R c = sqrt_r<R>(g * (pf + Pp) / rho);
    bool fb = (Pp < R(-0.05) * pf || rho < R(0));
    if (full)
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
      if (full) P.rhov[d * K.cap + p] = rhov[d];
      P.v[d * K.cap + p] = v[d];
    }
    P.vol[p] = vol;
    P.rho[p] = rho;
    if (full) {
      P.E[p] = E;
      P.P[p] = Pp;
      P.mass[p] = vol * rho;
    }
    P.c[p] = c;
    HN[p] = hroot<D, R>(vol);
    /* the shifting sum's record: position and volume, the phase in the
     * volume's sign (two phases) or, with three (2D only), in the unused z
     * slot; density and sound speed apart (read only for pairs across the
     * interface) */
    static_assert(F == 2 || D == 2, "three materials: the record's z slot carries the phase (2D)");
    typename Vec4<R>::T r4;
    r4.x = x[0];
    r4.y = x[1];
    if constexpr (F == 2) {
      r4.z = (D == 3) ? x[2] : R(0);
      r4.w = copysign(vol, ph == 2 ? R(-1) : R(1));
    } else {
      r4.z = R(ph);
      r4.w = vol;
    }
    reinterpret_cast<typename Vec4<R>::T*>(P.rec)[p] = r4;
    typename Vec2<R>::T r2;
    r2.x = rho;
    r2.y = c;
    reinterpret_cast<typename Vec2<R>::T*>(P.rec2)[p] = r2;
  }
  if (nfb) atomicAdd(&P.cnt->g2p_fb, nfb);
}

template <int D, typename R, bool EX>
void Launch<D, R, EX>::g2p(const CaseK& K, const DevPtrs<R>& P, int md, int xs, int x0, int xn, int hn, bool full,
                           cudaStream_t st) {
  k_g2p<D, R, EX><<<grid_for(K.cap, 128), 128, 0, st>>>(K, P, md, xs, x0, xn, hn, full ? 1 : 0);
}

/* ------------------------------------------------------------------ */
/* particle shifting                                                  */
/* ------------------------------------------------------------------ */
/* One CTA per brick of cells.  The CTA stages the stage-start position and slot
 * of every particle in the brick's +-rad2 neighbourhood into shared memory as one
 * 16-byte (FP32) or 32-byte (FP64) entry, with a boundary-particle flag per cell.
 *   - Mixed and FMA paths: per row of cells along the last axis, the CTA copies
 *     the contiguous range of that row's entries sorted by the last-axis
 *     coordinate (the per-stage row sort), tags each entry with its cell's
 *     offset in the row window and reduces the row's bounds in the other axes.
 *     Each thread then takes one particle: per row, a binary search finds the
 *     chord of its 2h sphere, the cell tag keeps the reference's +-rad2 window,
 *     and members are summed at once (or queued, variant 0) in sorted order.
 *   - Exact path: per-cell list offsets, the exact bounding box of each cell's
 *     entries and the reference's list order (binned entries, boundary
 *     particles, appended entries), scanned cell by cell.
 * A particle whose scan range leaves the staged box (it crossed a cell face
 * during the first stage) reads global memory instead, in the reference's list
 * order. */
template <int D>
struct Brick;
template <>
struct Brick<3> {
  static constexpr int B0 = 4, B1 = 4, B2 = 2;
};
template <>
struct Brick<2> {
  static constexpr int B0 = 8, B1 = 8, B2 = 1;
};
/* the larger brick of variant 5: twice the cells, 512 threads, a smaller
 * staged halo per particle */
template <int D>
struct BigBrick;
template <>
struct BigBrick<3> {
  static constexpr int B0 = 4, B1 = 4, B2 = 4;
};
template <>
struct BigBrick<2> {
  static constexpr int B0 = 16, B1 = 8, B2 = 1;
};
/* and the largest brick of variant 6: four times the cells, 1024 threads, one
 * block per SM */
template <int D>
struct HugeBrick;
template <>
struct HugeBrick<3> {
  static constexpr int B0 = 4, B1 = 4, B2 = 8;
};
template <>
struct HugeBrick<2> {
  static constexpr int B0 = 16, B1 = 16, B2 = 1;
};
template <int D, int VAR>
using BrickOf = typename std::conditional<VAR == 6, HugeBrick<D>,
                                          typename std::conditional<VAR == 5, BigBrick<D>, Brick<D>>::type>::type;
__host__ __device__ constexpr int pst_threads(int var) { return var == 6 ? 1024 : var == 5 ? 512 : 256; }
__host__ __device__ constexpr int pst_minblocks(int var) { return var == 3 ? 3 : var == 6 ? 1 : 2; }
__host__ __device__ constexpr bool pst_direct(int var) { return var == 2 || var == 3 || var == 5 || var == 6; }
constexpr int PST_THREADS = 256;
/* direct-sum variants test two candidates of a row per pass */
constexpr bool PST_PAIRS = true;
constexpr int PST_BUF = 64;


template <typename R>
struct RowKey;

template <int D, typename R>
struct PstSmem {
  using V4 = typename Vec4<R>::T;
  int* off;      /* nsc + 1 */
  int* mid;      /* nsc: index of the first appended entry of each staged cell */
  int* bnd;      /* nsc: cell holds boundary particles */
  R* blo;        /* D * nsc */
  R* bhi;        /* D * nsc */
  V4* ent;       /* cap: (x, y, z | slot) of each staged particle at the stage start */
  unsigned short* buf; /* PST_BUF x PST_THREADS queued member entries */
  /* mixed / FMA paths: off holds per staged row (not per cell) the offsets of
   * its entries, which are sorted by the last-axis coordinate (z in 3D, y in
   * 2D); ecell holds each entry's cell offset in the row window, rlo/rhi the
   * row's bounds in the other axes */
  unsigned char* ecell; /* cap */
  R* rlo;        /* 2 * nrow */
  R* rhi;        /* 2 * nrow */
  long long* rsrc; /* nrow: start of each staged row's range in the row-sorted entries */
  int lo[3], n[3], nsc, nrow, cap;
};

/* shared-memory layout of one brick; with sm == nullptr only the size */
template <int D, typename R, bool EX>
__host__ __device__ inline size_t pst_layout(PstSmem<D, R>* sm, unsigned char* raw, int nsc, int nrow, int cap,
                                             int qdepth) {
  using V4 = typename Vec4<R>::T;
  size_t o = 0;
  auto take = [&](size_t bytes, size_t align) {
    o = (o + align - 1) / align * align;
    const size_t r = o;
    o += bytes;
    return r;
  };
  const size_t off_o = take(sizeof(int) * (size_t)((nsc > nrow ? nsc : nrow) + 1), 16);
  const size_t bnd_o = take(sizeof(int) * (size_t)nsc, 16);
  const size_t mid_o = EX ? take(sizeof(int) * (size_t)nsc, 16) : 0;
  const size_t blo_o = EX ? take(sizeof(R) * (size_t)(2 * D * nsc), 16) : 0;
  const size_t ent_o = take(sizeof(V4) * (size_t)cap, 32);
  const size_t buf_o = take(sizeof(unsigned short) * (size_t)qdepth * PST_THREADS, 16);
  const size_t rlo_o = EX ? 0 : take(sizeof(R) * (size_t)(4 * nrow), 16);
  const size_t ec_o = EX ? 0 : take((size_t)cap, 16);
  const size_t rs_o = EX ? 0 : take(sizeof(long long) * (size_t)nrow, 16);
  if (sm) {
    sm->off = reinterpret_cast<int*>(raw + off_o);
    sm->bnd = reinterpret_cast<int*>(raw + bnd_o);
    sm->mid = EX ? reinterpret_cast<int*>(raw + mid_o) : nullptr;
    sm->blo = EX ? reinterpret_cast<R*>(raw + blo_o) : nullptr;
    sm->bhi = EX ? sm->blo + D * nsc : nullptr;
    sm->ent = reinterpret_cast<V4*>(raw + ent_o);
    sm->buf = reinterpret_cast<unsigned short*>(raw + buf_o);
    sm->rlo = EX ? nullptr : reinterpret_cast<R*>(raw + rlo_o);
    sm->rhi = EX ? nullptr : sm->rlo + 2 * nrow;
    sm->ecell = EX ? nullptr : raw + ec_o;
    sm->rsrc = EX ? nullptr : reinterpret_cast<long long*>(raw + rs_o);
  }
  return o + 128;
}
template <int D, typename R, bool EX>
__device__ inline void pst_carve(PstSmem<D, R>& sm, unsigned char* raw, int qdepth) {
  pst_layout<D, R, EX>(&sm, raw, sm.nsc, sm.nrow, sm.cap, qdepth);
}

/* per-particle constants and accumulators of the shifting sum */
template <int D, typename R, bool EX>
struct PstPart {
  R xsp[3], xnp[3];
  R hs_p, hh, lim2, rho_p, c_p, crho_p, tmp1c, C, W_dp, inv_hh, inv_wdp, aw_c, cwr, tmp1c5;
  int ph;
  R pst[3], phs[3];

  __device__ void init(const CaseK& K, R max_v) {
    const R ca = max_v * R(5.);
    const R P_b = rho_p * ca * ca;
    const R hd = (D == 2) ? hh * hh : hh * hh * hh;
    const R cdim = R(1.0 / PI_REF);
    C = (D == 2) ? cdim / hd * R(7. / 4.) : cdim / hd * R(21. / 16.);
    const R dxk = hh / R(CELL_RATIO) * R(CUT_OFF);
    R s = dxk / hh;
    R q = R(1.) - R(0.5) * s;
    W_dp = (s < R(2)) ? C * (((q * q) * q) * q) * (R(1.) + R(2.) * s) : R(0);
    tmp1c = -R(1.) * P_b * (R(1.) / rho_p);
    crho_p = c_p * c_p * rho_p;
    lim2 = (hs_p * R(CUT_OFF)) * (hs_p * R(CUT_OFF));
    inv_hh = R(1) / hh;
    inv_wdp = R(1) / W_dp;
    aw_c = R(-5.) * C * inv_hh * inv_hh; /* dW/dr / r = -5 C q^3 / h^2 */
    cwr = C * inv_wdp;
    tmp1c5 = R(0.2) * tmp1c;
    for (int d = 0; d < 3; d++) pst[d] = phs[d] = R(0);
  }

  __device__ __forceinline__ bool member(const R* xsq) const {
    R dd = R(0);
    for (int d = 0; d < D; d++) {
      R t = xsp[d] - xsq[d];
      dd = (d == 0) ? t * t : dd + t * t;
    }
    if constexpr (EX) return sqrt_r<R>(dd) <= hs_p * R(CUT_OFF); /* get_distance <= h*CUT_OFF */
    else return dd <= lim2;
  }

  /* one neighbour's contribution (particle_flow.cpp:540-575); rc2 holds the
   * neighbour's density and sound speed, read only across the interface */
  __device__ __forceinline__ void add(const R* xnq, R volq, int phq, const R* rc2, const R* nq) {
    R dr[3];
    R d2 = R(0);
    for (int d = 0; d < D; d++) {
      dr[d] = xnp[d] - xnq[d];
      d2 = (d == 0) ? dr[d] * dr[d] : d2 + dr[d] * dr[d];
    }
    if (d2 == R(0)) return;
    if constexpr (!EX) {
      /* the same terms with the particle's constant factors folded
       * (cwr = C / W_dp, tmp1c5 = 0.2 tmp1c) and the factor common to the
       * components hoisted */
      R s;
      if constexpr (sizeof(R) == 4) s = d2 * rsqrtf(d2) * inv_hh;
      else s = sqrt_r<R>(d2) * inv_hh;
      if (!(s < R(2))) return; /* W and dW vanish beyond the support */
      const R q = R(1.) - R(0.5) * s;
      const R q2 = q * q, q3 = q2 * q;
      const R w = (q2 * q2) * (R(1.) + R(2.) * s); /* W / C */
      const R rr = cwr * w;                        /* W / W_dp */
      const R rr2 = rr * rr;
      const R tmp1 = tmp1c + tmp1c5 * (rr2 * rr2); /* tmp1c (1 + 0.2 (W / W_dp)^4) */
      if (phq != PGDG_PHASE_BOUNDARY) {
        const R f = aw_c * q3 * tmp1 * volq;
        for (int d = 0; d < D; d++) pst[d] += dr[d] * f;
        if (phq != ph) {
          const R rhoq = rc2[0], cq = rc2[1];
          const R tmp2 = R(1.) / (rho_p + rhoq);
          const R cs = R(-0.1) * tmp2 * (crho_p + cq * cq * rhoq);
          const R g = cs * aw_c * q3 * volq;
          for (int d = 0; d < D; d++) phs[d] += dr[d] * g;
        }
      } else {
        const R f = C * w * tmp1 * volq;
        for (int d = 0; d < D; d++) pst[d] += nq[d] * f;
      }
      return;
    }
    /* exact path: the reference's operation order */
    R s, q, q3, Wij, aw, rr;
    {
      R dist = sqrt_r<R>(d2);
      s = dist / hh;
      if (!(s < R(2))) return; /* W and dW vanish beyond the support */
      q = R(1.) - R(0.5) * s;
      q3 = (q * q) * q;
      Wij = C * (q3 * q) * (R(1.) + R(2.) * s);
      aw = R(-5.) * C * q3 * s / hh / dist;
      rr = Wij / W_dp;
    }
    R Rr = R(0.2) * ((rr * rr) * (rr * rr));
    R tmp1 = tmp1c * (R(1) + Rr);
    if (phq != PGDG_PHASE_BOUNDARY) {
      for (int d = 0; d < D; d++) pst[d] += dr[d] * aw * tmp1 * volq;
      if (phq != ph) {
        const R rhoq = rc2[0], cq = rc2[1];
        R tmp2 = R(1.) / (rho_p + rhoq);
        R cs = R(-0.1) * tmp2 * (crho_p + cq * cq * rhoq);
        for (int d = 0; d < D; d++) phs[d] += cs * (dr[d] * aw) * volq;
      }
    } else {
      for (int d = 0; d < D; d++) pst[d] += nq[d] * Wij * tmp1 * volq;
    }
  }
};

template <int D, typename R, bool EX>
__device__ __forceinline__ void pst_boundary_cell(const CaseK& K, const DevPtrs<R>& P, int64_t c,
                                                  PstPart<D, R, EX>& pp) {
  for (int e = P.boff[c]; e < P.boff[c + 1]; e++) {
    int32_t b = P.bent[e];
    R xb[3], nb[3];
    for (int d = 0; d < D; d++) {
      xb[d] = P.bx[d * K.nbnd + b];
      nb[d] = P.bn[d * K.nbnd + b];
    }
    if (pp.member(xb)) pp.add(xb, (R)K.bvol, PGDG_PHASE_BOUNDARY, nullptr, nb);
  }
}

/* a member's contribution from the record G2P wrote: (new x, signed volume),
 * with density and sound speed in the second array */
template <typename V4>
__device__ __forceinline__ int rec_phase(const V4& r) {
  if constexpr (F == 2) return signbit(r.w) ? 2 : 1;
  else return (int)r.z;
}
template <int D, typename R, bool EX>
__device__ __forceinline__ void pst_rec_add(const DevPtrs<R>& P, int32_t q, const typename Vec4<R>::T& a,
                                            PstPart<D, R, EX>& pp) {
  R xnq[3] = {a.x, a.y, a.z};
  pp.add(xnq, fabs(a.w), rec_phase(a), P.rec2 + 2 * (int64_t)q, nullptr);
}
template <int D, typename R, bool EX>
__device__ __forceinline__ void pst_rec(const DevPtrs<R>& P, int32_t q, PstPart<D, R, EX>& pp) {
  using V4 = typename Vec4<R>::T;
  const V4 a = reinterpret_cast<const V4*>(P.rec)[q];
  pst_rec_add<D, R, EX>(P, q, a, pp);
}

template <int D, typename R, bool EX>
__device__ __forceinline__ void pst_fluid(const DevPtrs<R>& P, int32_t q, const R* xsq, PstPart<D, R, EX>& pp) {
  if (pp.member(xsq)) pst_rec<D, R, EX>(P, q, pp);
}

/* warp-wide min / max of a coordinate over the lanes of mask (as float, rounded
 * outward, through order-preserving integer keys) */
__device__ __forceinline__ int fkey(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float fkey_inv(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF); }
__device__ __forceinline__ float warp_min_lo(unsigned mask, float x) { return fkey_inv(__reduce_min_sync(mask, fkey(x))); }
__device__ __forceinline__ float warp_max_hi(unsigned mask, float x) { return fkey_inv(__reduce_max_sync(mask, fkey(x))); }
__device__ __forceinline__ float warp_min_lo(unsigned mask, double x) { return warp_min_lo(mask, __double2float_rd(x)); }
__device__ __forceinline__ float warp_max_hi(unsigned mask, double x) { return warp_max_hi(mask, __double2float_ru(x)); }

template <typename R>
__device__ __forceinline__ int slot_of(R w);
template <>
__device__ __forceinline__ int slot_of<float>(float w) { return __float_as_int(w); }
template <>
__device__ __forceinline__ int slot_of<double>(double w) { return (int)w; }
template <typename R>
__device__ __forceinline__ R slot_as(int q);
template <>
__device__ __forceinline__ float slot_as<float>(int q) { return __int_as_float(q); }
template <>
__device__ __forceinline__ double slot_as<double>(int q) { return (double)q; }

/* total order of a staged entry along its row: the row coordinate through an
 * order-preserving integer image (so NaN and -0 have a place too), ties by slot */
template <typename R>
struct RowKey;
template <>
struct RowKey<float> {
  unsigned long long k;
  __device__ __forceinline__ static RowKey of(const float4& v, int axis) {
    const float z = axis == 2 ? v.z : v.y;
    const unsigned hi = (unsigned)fkey(z) ^ 0x80000000u;
    return RowKey{((unsigned long long)hi << 32) | (unsigned)__float_as_int(v.w)};
  }
  __device__ __forceinline__ bool lt(const RowKey& o) const { return k < o.k; }
  __device__ __forceinline__ static RowKey lowest() { return RowKey{0ull}; }
  __device__ __forceinline__ static RowKey highest() { return RowKey{~0ull}; }
};
template <>
struct RowKey<double> {
  long long z;
  int s;
  __device__ __forceinline__ static RowKey of(const double4& v, int axis) {
    const long long i = __double_as_longlong(axis == 2 ? v.z : v.y);
    return RowKey{i >= 0 ? i : i ^ 0x7FFFFFFFFFFFFFFFLL, (int)v.w};
  }
  __device__ __forceinline__ bool lt(const RowKey& o) const { return z < o.z || (z == o.z && s < o.s); }
  __device__ __forceinline__ static RowKey lowest() { return RowKey{LLONG_MIN, INT_MIN}; }
  __device__ __forceinline__ static RowKey highest() { return RowKey{LLONG_MAX, INT_MAX}; }
};

constexpr int SCAN_RED = 66;

/* ---- rows of cells sorted once per stage (mixed and FMA paths) ----
 * A row is the line of cells along the last axis (z in 3D, y in 2D).  Each
 * stage, before the shifting kernel, every row's entries -- (stage-start
 * position, slot) of the particles binned in its cells -- are sorted by the
 * last-axis coordinate (ties by slot), in three passes over the cells:
 *   k_rs_cells  sorts each cell's entries (its run) and records the run's
 *               smallest and largest key;
 *   k_rs_rows   per row: offsets of the runs, prefix maxima and suffix minima
 *               of the run keys;
 *   k_rs_rank   places each entry at its rank in the row: its place in its
 *               run, corrected by the runs of the two neighbouring cells; the
 *               prefix/suffix keys confirm that no run further away
 *               interleaves, and otherwise every run of the row is counted.
 * Bricks of the shifting kernel then copy contiguous ranges of sorted rows
 * instead of sorting their halos.  Layout: fixed maxpc slots per cell, so a
 * row of NR cells owns NR * maxpc slots of each entry array. */
template <typename R>
struct RowSortBufs {
  typename Vec4<R>::T *run, *row;
  typename Vec4<R>::T* rec; /* each sorted entry's G2P record (new position, signed volume) */
  uint16_t* rk;            /* cell offset in the row of each sorted entry */
  int32_t *off, *pmin, *pmax;
  RowKey<R> *kmin, *kmax, *pmaxk, *smink;
};
template <typename R>
struct RowSorted {
  const typename Vec4<R>::T* row;
  const typename Vec4<R>::T* rec; /* the entries' G2P records, in the same order */
  const uint16_t* rk;
  const int32_t* pmin;  /* per cell: rank of its first and last entry in its row */
  const int32_t* pmax;
};
template <typename R>
__host__ __device__ inline size_t rowsort_layout(const CaseK& K, unsigned char* base, RowSortBufs<R>* B) {
  using V4 = typename Vec4<R>::T;
  const size_t ne = (size_t)K.ncell * K.maxpc, nc = (size_t)K.ncell;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    o = (o + 255) / 256 * 256;
    const size_t r = o;
    o += bytes;
    return base ? base + r : nullptr;
  };
  unsigned char* run = take(ne * sizeof(V4));
  unsigned char* row = take(ne * sizeof(V4));
  unsigned char* rec = take(ne * sizeof(V4));
  unsigned char* rk = take(ne * sizeof(uint16_t));
  unsigned char* off = take(nc * sizeof(int32_t));
  unsigned char* pmn = take(nc * sizeof(int32_t));
  unsigned char* pmx = take(nc * sizeof(int32_t));
  unsigned char* k0 = take(nc * sizeof(RowKey<R>));
  unsigned char* k1 = take(nc * sizeof(RowKey<R>));
  unsigned char* k2 = take(nc * sizeof(RowKey<R>));
  unsigned char* k3 = take(nc * sizeof(RowKey<R>));
  if (B) {
    B->run = reinterpret_cast<V4*>(run);
    B->row = reinterpret_cast<V4*>(row);
    B->rec = reinterpret_cast<V4*>(rec);
    B->rk = reinterpret_cast<uint16_t*>(rk);
    B->off = reinterpret_cast<int32_t*>(off);
    B->pmin = reinterpret_cast<int32_t*>(pmn);
    B->pmax = reinterpret_cast<int32_t*>(pmx);
    B->kmin = reinterpret_cast<RowKey<R>*>(k0);
    B->kmax = reinterpret_cast<RowKey<R>*>(k1);
    B->pmaxk = reinterpret_cast<RowKey<R>*>(k2);
    B->smink = reinterpret_cast<RowKey<R>*>(k3);
  }
  return o;
}

/* k_rs_cells sorts a cell's run in shared memory when it holds at most
 * RS_CAP entries (entry i of thread t at [i][t], so that a warp's accesses fall
 * on consecutive banks); a fuller cell sorts in place in global memory */
constexpr int RS_T = 128, RS_CAP = 16;

template <int D, typename R>
__global__ void __launch_bounds__(RS_T) k_rs_cells(CaseK K, DevPtrs<R> P, int xs, RowSortBufs<R> B) {
  using V4 = typename Vec4<R>::T;
  extern __shared__ __align__(32) unsigned char rs_raw[];
  V4* sh = reinterpret_cast<V4*>(rs_raw);
  const R* XS = P.X[xs];
  const int t = threadIdx.x;
  GRID_STRIDE(c, K.ncell) {
    const int cnt = min(P.bcnt[c], K.maxpc);
    const int64_t base = c * K.maxpc;
    auto load = [&](int r) {
      const int32_t q = P.bucket[base + r];
      V4 v;
      v.x = XS[q];
      v.y = XS[K.cap + q];
      v.z = (D == 3) ? XS[2 * K.cap + q] : R(0);
      v.w = slot_as<R>(q);
      return v;
    };
    if (cnt <= RS_CAP) {
      for (int r = 0; r < cnt; r++) {
        const V4 v = load(r);
        const RowKey<R> key = RowKey<R>::of(v, D - 1);
        int j = r - 1;
        while (j >= 0) {
          const V4 u = sh[j * RS_T + t];
          if (RowKey<R>::of(u, D - 1).lt(key)) break;
          sh[(j + 1) * RS_T + t] = u;
          j--;
        }
        sh[(j + 1) * RS_T + t] = v;
      }
      for (int r = 0; r < cnt; r++) B.run[base + r] = sh[r * RS_T + t];
      B.kmin[c] = cnt ? RowKey<R>::of(sh[t], D - 1) : RowKey<R>::highest();
      B.kmax[c] = cnt ? RowKey<R>::of(sh[(cnt - 1) * RS_T + t], D - 1) : RowKey<R>::lowest();
    } else {
      for (int r = 0; r < cnt; r++) {
        const V4 v = load(r);
        const RowKey<R> key = RowKey<R>::of(v, D - 1);
        int j = r - 1;
        while (j >= 0) {
          const V4 u = B.run[base + j];
          if (RowKey<R>::of(u, D - 1).lt(key)) break;
          B.run[base + j + 1] = u;
          j--;
        }
        B.run[base + j + 1] = v;
      }
      B.kmin[c] = RowKey<R>::of(B.run[base], D - 1);
      B.kmax[c] = RowKey<R>::of(B.run[base + cnt - 1], D - 1);
    }
  }
}

/* warp shuffles of a row key */
__device__ __forceinline__ RowKey<float> rk_shfl(const RowKey<float>& a, int src) {
  return RowKey<float>{__shfl_sync(0xffffffffu, a.k, src)};
}
__device__ __forceinline__ RowKey<double> rk_shfl(const RowKey<double>& a, int src) {
  return RowKey<double>{__shfl_sync(0xffffffffu, a.z, src), __shfl_sync(0xffffffffu, a.s, src)};
}
__device__ __forceinline__ RowKey<float> rk_shfl_up(const RowKey<float>& a, int o) {
  return RowKey<float>{__shfl_up_sync(0xffffffffu, a.k, o)};
}
__device__ __forceinline__ RowKey<double> rk_shfl_up(const RowKey<double>& a, int o) {
  return RowKey<double>{__shfl_up_sync(0xffffffffu, a.z, o), __shfl_up_sync(0xffffffffu, a.s, o)};
}
__device__ __forceinline__ RowKey<float> rk_shfl_down(const RowKey<float>& a, int o) {
  return RowKey<float>{__shfl_down_sync(0xffffffffu, a.k, o)};
}
__device__ __forceinline__ RowKey<double> rk_shfl_down(const RowKey<double>& a, int o) {
  return RowKey<double>{__shfl_down_sync(0xffffffffu, a.z, o), __shfl_down_sync(0xffffffffu, a.s, o)};
}

/* one warp per row: run offsets (a running sum), prefix maxima of the runs'
 * largest keys and suffix minima of their smallest keys, 32 cells at a time */
template <int D, typename R>
__global__ void __launch_bounds__(128) k_rs_rows(CaseK K, DevPtrs<R> P, RowSortBufs<R> B) {
  const int NR = K.N[D - 1];
  const int64_t nrows = K.ncell / NR;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t rw = w0; rw < nrows; rw += nw) {
    const int64_t c0 = rw * NR;
    int carry = 0;
    RowKey<R> mxc = RowKey<R>::lowest();
    for (int k0 = 0; k0 < NR; k0 += 32) {
      const int k = k0 + lane;
      const bool valid = k < NR;
      const int64_t c = c0 + k;
      const int cnt = valid ? min(P.bcnt[c], K.maxpc) : 0;
      int inc = cnt;
      RowKey<R> m = valid ? B.kmax[c] : RowKey<R>::lowest();
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        const RowKey<R> z = rk_shfl_up(m, o);
        if (lane >= o) {
          inc += y;
          if (m.lt(z)) m = z;
        }
      }
      if (valid) {
        B.off[c] = carry + inc - cnt;
        B.pmaxk[c] = mxc.lt(m) ? m : mxc;
        B.pmin[c] = INT_MAX;
        B.pmax[c] = -1;
      }
      carry += __shfl_sync(0xffffffffu, inc, 31);
      const RowKey<R> top = rk_shfl(m, 31);
      if (mxc.lt(top)) mxc = top;
    }
    RowKey<R> mnc = RowKey<R>::highest();
    for (int k0 = ((NR - 1) / 32) * 32; k0 >= 0; k0 -= 32) {
      const int k = k0 + lane;
      const bool valid = k < NR;
      RowKey<R> m = valid ? B.kmin[c0 + k] : RowKey<R>::highest();
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const RowKey<R> z = rk_shfl_down(m, o);
        if (lane + o < 32 && z.lt(m)) m = z;
      }
      if (valid) B.smink[c0 + k] = m.lt(mnc) ? m : mnc;
      const RowKey<R> bot = rk_shfl(m, 0);
      if (bot.lt(mnc)) mnc = bot;
    }
  }
}

/* entries of cell c's sorted run whose key is below key */
template <int D, typename R>
__device__ __forceinline__ int rs_count_less(const CaseK& K, const DevPtrs<R>& P, const RowSortBufs<R>& B, int64_t c,
                                             const RowKey<R>& key) {
  const int cnt = min(P.bcnt[c], K.maxpc);
  if (!cnt || key.lt(B.kmin[c])) return 0;
  if (B.kmax[c].lt(key)) return cnt;
  const int64_t base = c * K.maxpc;
  int lo = 0, hi = cnt;
  while (lo < hi) {
    const int md = (lo + hi) >> 1;
    if (RowKey<R>::of(B.run[base + md], D - 1).lt(key)) lo = md + 1;
    else hi = md;
  }
  return lo;
}

template <int D, typename R>
__global__ void __launch_bounds__(256) k_rs_rank(CaseK K, DevPtrs<R> P, RowSortBufs<R> B) {
  using V4 = typename Vec4<R>::T;
  const int NR = K.N[D - 1];
  GRID_STRIDE(c, K.ncell) {
    const int cnt = min(P.bcnt[c], K.maxpc);
    if (!cnt) continue;
    const int64_t rw = c / NR;
    const int k = (int)(c - rw * NR);
    const int64_t base = c * K.maxpc, RB = rw * NR * K.maxpc;
    const int off_c = B.off[c];
    for (int r = 0; r < cnt; r++) {
      const V4 v = B.run[base + r];
      const RowKey<R> key = RowKey<R>::of(v, D - 1);
      int rank = off_c + r;
      if (k >= 1) rank -= min(P.bcnt[c - 1], K.maxpc) - rs_count_less<D, R>(K, P, B, c - 1, key);
      if (k + 1 < NR) rank += rs_count_less<D, R>(K, P, B, c + 1, key);
      const bool far_ok = (k < 2 || B.pmaxk[c - 2].lt(key)) && (k + 2 >= NR || key.lt(B.smink[c + 2]));
      if (!far_ok) {
        rank = r;
        for (int j = 0; j < NR; j++)
          if (j != k) rank += rs_count_less<D, R>(K, P, B, rw * NR + j, key);
      }
      B.row[RB + rank] = v;
      B.rec[RB + rank] = reinterpret_cast<const V4*>(P.rec)[slot_of<R>(v.w)];
      B.rk[RB + rank] = (uint16_t)k;
      if (r == 0) B.pmin[c] = rank;
      if (r == cnt - 1) B.pmax[c] = rank;
    }
  }
}

/* Block-wide in-place scan of the n counts in a[1..n]: afterwards a[0] = 0 and
 * a[l + 1] is the sum of counts 0..l.  Each thread scans a contiguous chunk,
 * warps combine through shuffles and s_red (SCAN_RED ints).  Every thread of the
 * block calls it; it returns the total to all of them. */
__device__ __forceinline__ int block_scan_counts(int* a, int n, int* s_red) {
  const int nt = blockDim.x, t = threadIdx.x, lane = t & 31, w = t >> 5, nw = (nt + 31) >> 5;
  const int per = (n + nt - 1) / nt;
  const int l0 = min(t * per, n), l1 = min(l0 + per, n);
  int s = 0;
  for (int l = l0; l < l1; l++) s += a[l + 1];
  int inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) s_red[w] = inc;
  __syncthreads();
  if (w == 0) {
    const int v = lane < nw ? s_red[lane] : 0;
    int iv = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, iv, o);
      if (lane >= o) iv += y;
    }
    s_red[32 + lane] = iv - v;
    if (lane == 31) s_red[64] = iv;
  }
  __syncthreads();
  int run = s_red[32 + w] + inc - s;
  for (int l = l0; l < l1; l++) {
    run += a[l + 1];
    a[l + 1] = run;
  }
  if (t == 0) a[0] = 0;
  const int total = s_red[64];
  __syncthreads();
  return total;
}

/* Bound_pen and Update_PST of one particle from its neighbour sums */
template <int D, typename R, bool EX>
__device__ __forceinline__ void pst_finish(const CaseK& K, const DevPtrs<R>& P, int64_t p, R dt,
                                           const PstPart<D, R, EX>& pp) {
  /* Bound_pen (particle_flow.cpp:587-622) on the faces of the particle's cell */
  R bp[3] = {0, 0, 0};
  {
    const int64_t ci = P.lcell[p];
    int idx[3];
    idx[2] = (int)(ci % K.N[2]);
    idx[1] = (int)((ci / K.N[2]) % K.N[1]);
    idx[0] = (int)(ci / ((int64_t)K.N[1] * K.N[2]));
#pragma unroll
    for (int f = 0; f < 2 * D; f++) {
      const int a = (f == 0 || f == 2) ? 1 : (f == 1 || f == 3) ? 0 : 2;
      const int sg = (f == 0 || f == 3 || f == 4) ? -1 : 1;
      const int side = (f == 0) ? 2 : (f == 1) ? 1 : (f == 2) ? 3 : (f == 3) ? 0 : (f == 4) ? 4 : 5;
      int nbi = idx[a] + sg;
      if (nbi >= 0 && nbi < K.N[a]) continue;
      if (K.bc[side] == 0) continue;
      R cen = (R)(K.bl[a] + K.ps[a] * (idx[a] + 0.5) + sg * 0.5 * K.ps[a]);
      R nn = (R)sg;
      R ds = (pp.xnp[a] - cen) * nn;
      if (ds < R(0)) nn = -nn;
      R dis = fabs(ds);
      if constexpr (!EX) {
        /* a particle exactly on the wall (far likelier with FP32 coordinates):
         * the reference's 0.02 / dis is infinite there, and the capped
         * displacement of Update_PST turns it into NaN (inf x 0).  Take the
         * limit dis -> 0 from the domain side instead: a finite push away from
         * the wall, which the cap below limits to p_sz / 2 */
        if (!(dis > R(0))) {
          dis = R(1e-6) * (R)K.p_sz;
          nn = R(-sg);
        }
      }
      if (dis < R(0.4) * (R)K.p_sz) bp[a] += R(0.02) / dis * (pp.c_p * pp.c_p) * nn;
    }
  }
  /* Update_PST (particle_flow.cpp:485-525) */
  const R px = (R)K.p_sz;
  R dx[3], dx1[3], dx2[3];
  R s0 = 0, s1 = 0, s2 = 0;
  for (int d = 0; d < D; d++) {
    dx[d] = pp.pst[d] * dt * dt / R(2.);
    dx1[d] = pp.phs[d] * dt * dt / R(2.);
    dx2[d] = bp[d] * dt * dt / R(2.);
    s0 = (d == 0) ? dx[d] * dx[d] : s0 + dx[d] * dx[d];
    s1 = (d == 0) ? dx1[d] * dx1[d] : s1 + dx1[d] * dx1[d];
    s2 = (d == 0) ? dx2[d] * dx2[d] : s2 + dx2[d] * dx2[d];
  }
  R dis0 = sqrt_r<R>(s0), dis1 = sqrt_r<R>(s1), dis2 = sqrt_r<R>(s2);
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

/* one particle: neighbour sum, Bound_pen, Update_PST; sm == nullptr -> global path */
template <int D, typename R, bool EX, int VAR>
__device__ void pst_particle(const CaseK& K, const DevPtrs<R>& P, int64_t p, const R* XS, const R* XN, const R* HS,
                             const R* HN, R dt, R max_v, const PstSmem<D, R>* sm) {
  PstPart<D, R, EX> pp;
  pp.ph = P.phase[p];
  for (int d = 0; d < 3; d++) pp.xsp[d] = pp.xnp[d] = R(0);
  for (int d = 0; d < D; d++) {
    pp.xsp[d] = XS[d * K.cap + p];
    pp.xnp[d] = XN[d * K.cap + p];
  }
  pp.hs_p = HS[p];
  pp.hh = HN[p];
  pp.rho_p = P.rho[p];
  pp.c_p = P.c[p];
  pp.init(K, max_v);
  /* scan centre: cell of the stage-start position (level_infor.cpp:169-173) */
  int pos[3];
  cell_pos<D, R>(K, pp.xsp, pos);
  int lo[3], hi[3];
  bool inside = sm != nullptr;
  for (int d = 0; d < 3; d++) {
    int r = (d < D) ? K.rad2 : 0;
    lo[d] = max(pos[d] - r, 0);
    hi[d] = min(pos[d] + r, (d < D ? K.N[d] : 1) - 1);
    if (sm && (lo[d] < sm->lo[d] || hi[d] >= sm->lo[d] + sm->n[d])) inside = false;
  }
  if (inside) {
    constexpr int BUFV = PST_BUF;
    const R lim2m = pp.lim2 * R(1.0001);
    int nbuf = 0;
    /* sum the queued members in queue (= scan) order */
    auto flush = [&]() {
      using V4 = typename Vec4<R>::T;
      int i = 0;
      for (; i + 1 < nbuf; i += 2) {
        /* two records in flight before either is summed (order kept) */
        const int e0 = sm->buf[i * PST_THREADS + threadIdx.x];
        const int e1 = sm->buf[(i + 1) * PST_THREADS + threadIdx.x];
        const int32_t q0 = slot_of<R>(sm->ent[e0].w), q1 = slot_of<R>(sm->ent[e1].w);
        const V4 a0 = reinterpret_cast<const V4*>(P.rec)[q0], a1 = reinterpret_cast<const V4*>(P.rec)[q1];
        pst_rec_add<D, R, EX>(P, q0, a0, pp);
        pst_rec_add<D, R, EX>(P, q1, a1, pp);
      }
      if (i < nbuf) {
        const int e = sm->buf[i * PST_THREADS + threadIdx.x];
        pst_rec<D, R, EX>(P, slot_of<R>(sm->ent[e].w), pp);
      }
      nbuf = 0;
    };
    auto queue = [&](int e) {
      const auto v = sm->ent[e];
      R xsq[3] = {v.x, v.y, D == 3 ? v.z : R(0)};
      if (pp.member(xsq)) {
        if (nbuf == BUFV) flush();
        sm->buf[nbuf++ * PST_THREADS + threadIdx.x] = (unsigned short)e;
      }
    };
    if constexpr (!EX) {
      if constexpr (VAR != 1) {
      /* variants 0, 2 and 3, per lane: for each row of cells along the last axis (z in
       * 3D, y in 2D) whose bounds in the other axes come within 2h, only the
       * entries whose row coordinate lies within the chord of the 2h sphere are
       * tested (binary search in the sorted row); the cell tag keeps the scan
       * to the particle's +-rad2 cell window.  Variant 0 queues the members and
       * sums them in warp-wide batches; variants 2 and 3 sum each member as it
       * is found (no queue, less shared memory; 3 is launched for 3 blocks per
       * SM). */
      constexpr int RA = D - 1;
      const int clo = lo[RA] - sm->lo[RA], chi = hi[RA] - sm->lo[RA];
      const R zp = pp.xsp[RA];
      const int u1 = (D == 3) ? hi[1] : lo[1];
      for (int t = lo[0]; t <= hi[0]; t++)
        for (int u = lo[1]; u <= u1; u++) {
          const int row = (D == 3) ? (t - sm->lo[0]) * sm->n[1] + (u - sm->lo[1]) : (t - sm->lo[0]);
          R dxy = R(0);
          for (int d = 0; d < D - 1; d++) {
            R a = sm->rlo[2 * row + d] - pp.xsp[d], b = pp.xsp[d] - sm->rhi[2 * row + d];
            R w = a > b ? a : b;
            if (w > R(0)) dxy += w * w;
          }
          if (dxy <= lim2m) {
            const R w = sqrt_r<R>(lim2m - dxy); /* half chord of the 2h sphere */
            const R za = zp - w, zb = zp + w;
            int e = sm->off[row], hi_e = sm->off[row + 1];
            const int e1 = hi_e;
            while (e < hi_e) { /* first entry with coordinate >= za */
              const int m = (e + hi_e) >> 1;
              const R zm = (RA == 2) ? sm->ent[m].z : sm->ent[m].y;
              if (zm < za) e = m + 1;
              else hi_e = m;
            }
            /* a candidate: inside the chord, in the cell window, within 2h at
             * the stage start */
            auto is_member = [&](const typename Vec4<R>::T& v, int ce) {
              if ((unsigned)(ce - clo) > (unsigned)(chi - clo)) return false;
              R xsq[3] = {v.x, v.y, D == 3 ? v.z : R(0)};
              return pp.member(xsq);
            };
            auto take = [&](const typename Vec4<R>::T& v, int ei) {
              if constexpr (pst_direct(VAR)) {
                pst_rec<D, R, EX>(P, slot_of<R>(v.w), pp); /* summed at once, same order */
              } else {
                if (nbuf == BUFV) flush();
                sm->buf[nbuf++ * PST_THREADS + threadIdx.x] = (unsigned short)ei;
              }
            };
            if constexpr (PST_PAIRS && pst_direct(VAR)) {
              /* two candidates per pass (independent tests), summed in order */
              bool more = true;
              for (; more && e + 1 < e1; e += 2) {
                const auto v0 = sm->ent[e], v1 = sm->ent[e + 1];
                const R z0 = (RA == 2) ? v0.z : v0.y, z1 = (RA == 2) ? v1.z : v1.y;
                const int c0 = sm->ecell[e], c1 = sm->ecell[e + 1];
                if (z0 > zb) {
                  more = false;
                  break;
                }
                const bool m0 = is_member(v0, c0);
                const bool in1 = !(z1 > zb);
                const bool m1 = in1 && is_member(v1, c1);
                if (m0) take(v0, e);
                if (m1) take(v1, e + 1);
                more = in1;
              }
              if (more && e < e1) {
                const auto v = sm->ent[e];
                const R zv = (RA == 2) ? v.z : v.y;
                if (!(zv > zb) && is_member(v, sm->ecell[e])) take(v, e);
              }
            } else {
              for (; e < e1; e++) {
                const auto v = sm->ent[e];
                const R zv = (RA == 2) ? v.z : v.y;
                if (zv > zb) break;
                if (is_member(v, sm->ecell[e])) take(v, e);
              }
            }
          }
          if constexpr (VAR == 0)
            if (__any_sync(__activemask(), nbuf >= BUFV / 2)) flush();
        }
      } else {
      /* variant 1, warp-cooperative: the lanes walk the union of their
       * rows of cells along the last axis (z in 3D, y in 2D) together, and in
       * each row the union of their windows of the sorted row coordinate (the
       * chord of each lane's 2h sphere); every staged entry is one broadcast
       * shared-memory read that each lane tests against its own sphere and
       * +-rad2 cell window.  A lane's members are queued in the same order as
       * a per-lane scan would queue them.  Boundary particles follow in a
       * second pass (the summation order only affects rounding). */
      constexpr int RA = D - 1;
      const unsigned am = __activemask();
      const int clo = lo[RA] - sm->lo[RA], chi = hi[RA] - sm->lo[RA];
      const R zp = pp.xsp[RA];
      const int t0 = __reduce_min_sync(am, lo[0]), t1 = __reduce_max_sync(am, hi[0]);
      const int u0 = (D == 3) ? __reduce_min_sync(am, lo[1]) : 0;
      const int u1 = (D == 3) ? __reduce_max_sync(am, hi[1]) : 0;
      for (int t = t0; t <= t1; t++)
        for (int u = u0; u <= u1; u++) {
          const int row = (D == 3) ? (t - sm->lo[0]) * sm->n[1] + (u - sm->lo[1]) : (t - sm->lo[0]);
          bool need = t >= lo[0] && t <= hi[0] && (D == 2 || (u >= lo[1] && u <= hi[1]));
          R za = R(1e30), zb = R(-1e30);
          if (need) {
            R dxy = R(0);
            for (int d = 0; d < D - 1; d++) {
              R a = sm->rlo[2 * row + d] - pp.xsp[d], b = pp.xsp[d] - sm->rhi[2 * row + d];
              R w = a > b ? a : b;
              if (w > R(0)) dxy += w * w;
            }
            if (dxy <= lim2m) {
              const R w = sqrt_r<R>(lim2m - dxy); /* half chord of the 2h sphere */
              za = zp - w;
              zb = zp + w;
            } else {
              need = false;
            }
          }
          if (!__any_sync(am, need)) continue;
          const float fa = warp_min_lo(am, za), fb = warp_max_hi(am, zb);
          int e = sm->off[row], hi_e = sm->off[row + 1];
          const int e1 = hi_e;
          while (e < hi_e) { /* first entry with coordinate >= the union's lower end */
            const int m = (e + hi_e) >> 1;
            const R zm = (RA == 2) ? sm->ent[m].z : sm->ent[m].y;
            if (zm < R(fa)) e = m + 1;
            else hi_e = m;
          }
          for (; e < e1; e++) {
            const auto v = sm->ent[e];
            const R zv = (RA == 2) ? v.z : v.y;
            if (zv > R(fb)) break;
            const int ce = sm->ecell[e];
            if (need && ce >= clo && ce <= chi) {
              R xsq[3] = {v.x, v.y, D == 3 ? v.z : R(0)};
              if (pp.member(xsq)) {
                if (nbuf == BUFV) flush();
                sm->buf[nbuf++ * PST_THREADS + threadIdx.x] = (unsigned short)e;
              }
            }
          }
          if (__any_sync(am, nbuf >= BUFV / 2)) flush();
        }
      }
      flush();
      bool edge = false;
      for (int d = 0; d < D; d++) edge = edge || lo[d] == 0 || hi[d] == K.N[d] - 1;
      if (edge)
        for (int t = lo[0]; t <= hi[0]; t++)
          for (int s = lo[1]; s <= hi[1]; s++)
            for (int m = lo[2]; m <= hi[2]; m++) {
              const int l = ((t - sm->lo[0]) * sm->n[1] + (s - sm->lo[1])) * sm->n[2] + (m - sm->lo[2]);
              if (!sm->bnd[l]) continue;
              const int64_t c = ((int64_t)t * K.N[1] + s) * K.N[2] + m;
              pst_boundary_cell<D, R, EX>(K, P, c, pp);
            }
    } else {
      /* exact path: the reference's per-cell list order (binned fluid,
       * boundary particles, appended fluid) */
      for (int t = lo[0]; t <= hi[0]; t++)
        for (int s = lo[1]; s <= hi[1]; s++) {
          int l = ((t - sm->lo[0]) * sm->n[1] + (s - sm->lo[1])) * sm->n[2] + (lo[2] - sm->lo[2]);
          for (int m = lo[2]; m <= hi[2]; m++, l++) {
            const int e0 = sm->off[l], e1 = sm->off[l + 1], em = e0 + sm->mid[l];
            R md = R(0);
            for (int d = 0; d < D; d++) {
              R a = sm->blo[d * sm->nsc + l] - pp.xsp[d];
              R b = pp.xsp[d] - sm->bhi[d * sm->nsc + l];
              R g = a > b ? a : b;
              if (g > R(0)) md += g * g;
            }
            if (md <= lim2m)
              for (int e = e0; e < em; e++) queue(e);
            if (sm->bnd[l]) {
              flush();
              const int64_t c = ((int64_t)t * K.N[1] + s) * K.N[2] + m;
              pst_boundary_cell<D, R, EX>(K, P, c, pp);
            }
            if (md <= lim2m)
              for (int e = em; e < e1; e++) queue(e);
            if (__any_sync(__activemask(), nbuf >= BUFV / 2)) flush();
          }
        }
      flush();
    }
  } else {
    for (int t = lo[0]; t <= hi[0]; t++)
      for (int s = lo[1]; s <= hi[1]; s++)
        for (int m = lo[2]; m <= hi[2]; m++) {
          const int64_t c = ((int64_t)t * K.N[1] + s) * K.N[2] + m;
          const int cnt = min(P.bcnt[c], K.maxpc);
          const int32_t* bk = P.bucket + c * K.maxpc;
          int r = 0;
          for (; r < cnt; r++) {
            int32_t q = bk[r];
            if (P.lkey[q] >= KEY_APPEND) break;
            R xsq[3] = {0, 0, 0};
            for (int d = 0; d < D; d++) xsq[d] = XS[d * K.cap + q];
            pst_fluid<D, R, EX>(P, q, xsq, pp);
          }
          pst_boundary_cell<D, R, EX>(K, P, c, pp);
          for (; r < cnt; r++) {
            int32_t q = bk[r];
            R xsq[3] = {0, 0, 0};
            for (int d = 0; d < D; d++) xsq[d] = XS[d * K.cap + q];
            pst_fluid<D, R, EX>(P, q, xsq, pp);
          }
        }
  }
  pst_finish<D, R, EX>(K, P, p, dt, pp);
}

template <int D, typename R, bool EX, int VAR>
__global__ void __launch_bounds__(pst_threads(VAR), pst_minblocks(VAR)) k_pst(CaseK K, DevPtrs<R> P, int xs, int hs, int xn, int hn,
                                                    int nb0, int nb1, int cap, RowSorted<R> RS) {
  using BK = BrickOf<D, VAR>;
  using V4 = typename Vec4<R>::T;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const R dt = (R)P.cnt->dt;
  const R max_v = (R)P.cnt->max_v;
  const R* XS = P.X[xs];
  const R* XN = P.X[xn];
  const R* HS = P.H[hs];
  const R* HN = P.H[hn];
  const int b = blockIdx.x;
  int c0[3];
  /* blockIdx = (i_b * nb1 + j_b) * nb0 + k_b */
  c0[0] = (b / (nb0 * nb1)) * BK::B0;
  c0[1] = ((b / nb0) % nb1) * BK::B1;
  c0[2] = (D == 3) ? (b % nb0) * BK::B2 : 0;
  const int bdim[3] = {BK::B0, BK::B1, D == 3 ? BK::B2 : 1};
  PstSmem<D, R> sm;
  for (int d = 0; d < 3; d++) {
    int r = (d < D) ? K.rad2 : 0;
    int Nd = (d < D) ? K.N[d] : 1;
    int lo = max(c0[d] - r, 0);
    int hi = min(c0[d] + bdim[d] - 1 + r, Nd - 1);
    sm.lo[d] = lo;
    sm.n[d] = hi - lo + 1;
  }
  sm.nsc = sm.n[0] * sm.n[1] * sm.n[2];
  sm.cap = cap;
  sm.nrow = (D == 3) ? sm.n[0] * sm.n[1] : sm.n[0];
  pst_carve<D, R, EX>(sm, smem_raw, (!EX && pst_direct(VAR)) ? 0 : PST_BUF);
  __shared__ int s_red[SCAN_RED];
  int s_total;
  if constexpr (EX) {
    for (int l = threadIdx.x; l < sm.nsc; l += blockDim.x) {
      int t = l / (sm.n[1] * sm.n[2]), s = (l / sm.n[2]) % sm.n[1], m = l % sm.n[2];
      int64_t c = ((int64_t)(sm.lo[0] + t) * K.N[1] + (sm.lo[1] + s)) * K.N[2] + (sm.lo[2] + m);
      int cnt = min(P.bcnt[c], K.maxpc);
      sm.off[l + 1] = cnt;
      sm.mid[l] = cnt;
      sm.bnd[l] = P.boff[c + 1] > P.boff[c] ? 1 : 0;
    }
    __syncthreads();
    s_total = block_scan_counts(sm.off, sm.nsc, s_red);
  } else {
    /* boundary-particle flag of each staged cell, and per staged row the range
     * of the stage's row-sorted entries that holds every entry of the row's
     * window cells (entries of other cells of the row can lie inside the range
     * where they drifted across a window end; their tag excludes them) */
    for (int l = threadIdx.x; l < sm.nsc; l += blockDim.x) {
      int t = l / (sm.n[1] * sm.n[2]), s = (l / sm.n[2]) % sm.n[1], m = l % sm.n[2];
      int64_t c = ((int64_t)(sm.lo[0] + t) * K.N[1] + (sm.lo[1] + s)) * K.N[2] + (sm.lo[2] + m);
      sm.bnd[l] = P.boff[c + 1] > P.boff[c] ? 1 : 0;
    }
    constexpr int RA = D - 1;
    const int NR = K.N[RA];
    for (int row = threadIdx.x; row < sm.nrow; row += blockDim.x) {
      const int64_t gr = (D == 3) ? (int64_t)(sm.lo[0] + row / sm.n[1]) * K.N[1] + (sm.lo[1] + row % sm.n[1])
                                  : (int64_t)(sm.lo[0] + row);
      int first = INT_MAX, last = -1;
      for (int k = 0; k < sm.n[RA]; k++) {
        const int64_t c = gr * NR + sm.lo[RA] + k;
        first = min(first, RS.pmin[c]);
        last = max(last, RS.pmax[c]);
      }
      sm.off[row + 1] = last >= first ? last - first + 1 : 0;
      sm.rsrc[row] = gr * NR * K.maxpc + (last >= first ? first : 0);
    }
    __syncthreads();
    s_total = block_scan_counts(sm.off, sm.nrow, s_red);
  }
  const bool use_sm = s_total <= cap;
  if (use_sm) {
    if constexpr (EX) {
      /* slots: one thread per staged cell copies its list into the entry
       * slots and finds the first appended entry (the reference's list order
       * puts the appended split children after the boundary particles) */
      for (int l = threadIdx.x; l < sm.nsc; l += blockDim.x) {
        const int t = l / (sm.n[1] * sm.n[2]), s = (l / sm.n[2]) % sm.n[1], m = l % sm.n[2];
        const int64_t c = ((int64_t)(sm.lo[0] + t) * K.N[1] + (sm.lo[1] + s)) * K.N[2] + (sm.lo[2] + m);
        const int32_t* bk = P.bucket + c * K.maxpc;
        const int e0 = sm.off[l], cnt = sm.off[l + 1] - e0;
        bool app = false;
        for (int r = 0; r < cnt; r++) {
          const int32_t q = bk[r];
          sm.ent[e0 + r].w = slot_as<R>(q);
          if (!app && P.lkey[q] >= KEY_APPEND) {
            sm.mid[l] = r;
            app = true;
          }
        }
      }
      __syncthreads();
      /* stage-start coordinates: one thread per entry */
      for (int e = threadIdx.x; e < s_total; e += blockDim.x) {
        V4 v = sm.ent[e];
        const int32_t q = slot_of<R>(v.w);
        v.x = XS[q];
        v.y = XS[K.cap + q];
        v.z = (D == 3) ? XS[2 * K.cap + q] : R(0);
        sm.ent[e] = v;
      }
      __syncthreads();
      /* per cell: the exact bounding box of its entries */
      for (int l = threadIdx.x; l < sm.nsc; l += blockDim.x) {
        R mn[3] = {R(1e30), R(1e30), R(1e30)}, mx[3] = {R(-1e30), R(-1e30), R(-1e30)};
        for (int e = sm.off[l]; e < sm.off[l + 1]; e++) {
          const V4 v = sm.ent[e];
          const R xv[3] = {v.x, v.y, v.z};
          for (int d = 0; d < D; d++) {
            mn[d] = xv[d] < mn[d] ? xv[d] : mn[d];
            mx[d] = xv[d] > mx[d] ? xv[d] : mx[d];
          }
        }
        for (int d = 0; d < D; d++) {
          sm.blo[d * sm.nsc + l] = mn[d];
          sm.bhi[d * sm.nsc + l] = mx[d];
        }
      }
      __syncthreads();
    } else {
      /* one warp per staged row copies its range (coalesced), tags each entry
       * with its cell's offset in the row window (255 outside the window) and
       * reduces the row's bounds in the other axes */
      constexpr int RA = D - 1;
      const int lane = threadIdx.x & 31;
      for (int row = threadIdx.x >> 5; row < sm.nrow; row += blockDim.x >> 5) {
        const int e0 = sm.off[row], len = sm.off[row + 1] - e0;
        const int64_t src = sm.rsrc[row];
        R mn[2] = {R(1e30), R(1e30)}, mx[2] = {R(-1e30), R(-1e30)};
        for (int i = lane; i < len; i += 32) {
          const V4 v = RS.row[src + i];
          const int kk = (int)RS.rk[src + i] - sm.lo[RA];
          sm.ent[e0 + i] = v;
          sm.ecell[e0 + i] = (unsigned char)((kk >= 0 && kk < sm.n[RA]) ? kk : 255);
          const R xv[2] = {v.x, v.y};
          for (int d = 0; d < D - 1; d++) {
            mn[d] = xv[d] < mn[d] ? xv[d] : mn[d];
            mx[d] = xv[d] > mx[d] ? xv[d] : mx[d];
          }
        }
        for (int d = 0; d < D - 1; d++) {
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const R a = __shfl_xor_sync(0xffffffffu, mn[d], o), b = __shfl_xor_sync(0xffffffffu, mx[d], o);
            mn[d] = a < mn[d] ? a : mn[d];
            mx[d] = b > mx[d] ? b : mx[d];
          }
        }
        if (lane < D - 1) {
          sm.rlo[2 * row + lane] = lane == 0 ? mn[0] : mn[1];
          sm.rhi[2 * row + lane] = lane == 0 ? mx[0] : mx[1];
        }
      }
      __syncthreads();
    }
  }
  /* the brick's own particles */
  const int nbc = bdim[0] * bdim[1] * bdim[2];
  __shared__ int s_boff[BK::B0 * BK::B1 * BK::B2 + 1];
  __shared__ int s_bcell[BK::B0 * BK::B1 * BK::B2];
  for (int q = threadIdx.x; q < nbc; q += blockDim.x) {
    int dt0 = q / (bdim[1] * bdim[2]), dt1 = (q / bdim[2]) % bdim[1], dt2 = q % bdim[2];
    int ci = c0[0] + dt0, cj = c0[1] + dt1, ck = c0[2] + dt2;
    int cnt = 0;
    int64_t c = -1;
    if (ci < K.N[0] && cj < K.N[1] && ck < K.N[2]) {
      c = ((int64_t)ci * K.N[1] + cj) * K.N[2] + ck;
      cnt = min(P.bcnt[c], K.maxpc);
    }
    s_bcell[q] = (int)c;
    s_boff[q + 1] = cnt;
  }
  __syncthreads();
  const int npart = block_scan_counts(s_boff, nbc, s_red);
  for (int i = threadIdx.x; i < npart; i += blockDim.x) {
    int q = 0, qh = nbc - 1; /* the brick cell holding particle i */
    while (q < qh) {
      const int md = (q + qh + 1) >> 1;
      if (s_boff[md] <= i) q = md;
      else qh = md - 1;
    }
    const int64_t c = s_bcell[q];
    const int32_t p = P.bucket[c * K.maxpc + (i - s_boff[q])];
    pst_particle<D, R, EX, VAR>(K, P, p, XS, XN, HS, HN, dt, max_v, use_sm ? &sm : nullptr);
  }
}

template <int D, typename R, bool EX, int VAR>
static void pst_launch(const CaseK& K, const DevPtrs<R>& P, int xs, int hs, int xn, int hn, const RowSorted<R>& RS,
                       cudaStream_t st) {
  using BK = BrickOf<D, VAR>;
  const int nb0 = (D == 3) ? (K.N[2] + BK::B2 - 1) / BK::B2 : 1;
  const int nb1 = (K.N[1] + BK::B1 - 1) / BK::B1;
  const int nbx = (K.N[0] + BK::B0 - 1) / BK::B0;
  const int r = K.rad2;
  const int nsc = (BK::B0 + 2 * r) * (BK::B1 + 2 * r) * (D == 3 ? BK::B2 + 2 * r : 1);
  const int ppc = (D == 3) ? 8 : 4;
  const int nrow = (D == 3) ? (BK::B0 + 2 * r) * (BK::B1 + 2 * r) : (BK::B0 + 2 * r);
  const int qdepth = (!EX && pst_direct(VAR)) ? 0 : PST_BUF;
  /* staging headroom over the nominal count (split children); variant 3 keeps
   * it at 1/8 so three blocks fit in an SM's shared memory */
  int cap = (!EX && (VAR == 3 || VAR >= 5)) ? nsc * ppc * 9 / 8 : nsc * ppc * 5 / 4;
  if (cap > 65535) cap = 65535;
  size_t bytes = pst_layout<D, R, EX>(nullptr, nullptr, nsc, nrow, cap, qdepth);
  while (bytes > 220 * 1024 && cap > 256) {
    cap = cap * 3 / 4;
    bytes = pst_layout<D, R, EX>(nullptr, nullptr, nsc, nrow, cap, qdepth);
  }
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_pst<D, R, EX, VAR>, cudaFuncAttributeMaxDynamicSharedMemorySize, 224 * 1024);
    attr_set = true;
  }
  k_pst<D, R, EX, VAR><<<nbx * nb1 * nb0, pst_threads(VAR), bytes, st>>>(K, P, xs, hs, xn, hn, nb0, nb1, cap, RS);
}

/* ---- the shifting kernel, second form (variants 6 and 7) ----
 * The same bricks, row-sorted staging and chord search as the direct variants,
 * with three changes:
 *   - members' G2P records are read in row order: the row sort places each
 *     entry's record beside it (variant 6 reads them from there through L1,
 *     variant 7 stages them in shared memory too: one block per SM with room
 *     for 12 particles per cell);
 *   - a brick whose cells hold more particles than its staging room (the
 *     compressed fluid behind a shock) scans the same sorted rows from global
 *     memory instead of falling back to the per-cell scan;
 *   - on the FP32 path, candidates are tested and their pair terms evaluated
 *     two at a time with packed arithmetic (FADD2/FMUL2/FFMA2: one instruction
 *     for both); a non-member's term is masked to zero, which keeps the lanes
 *     of a warp in step.
 * The members, each term's arithmetic and the order of the sum are those of
 * the direct variants. */
template <int D, typename R, bool SREC, bool GL>
__device__ __forceinline__ void pst2_rows(const CaseK& K, const DevPtrs<R>& P, const RowSorted<R>& RS,
                                          const int* s_off, const long long* s_rsrc, const R* s_rlo,
                                          const R* s_rhi, const typename Vec4<R>::T* s_ent,
                                          const typename Vec4<R>::T* s_rec, const unsigned char* s_tag,
                                          const int* slo, const int* sn, const int* lo, const int* hi,
                                          PstPart<D, R, false>& pp) {
  using V4 = typename Vec4<R>::T;
  constexpr int RA = D - 1;
  const int clo = lo[RA] - slo[RA], chi = hi[RA] - slo[RA];
  const R zp = pp.xsp[RA];
  const R lim2m = pp.lim2 * R(1.0001);
  const int u1 = (D == 3) ? hi[1] : lo[1];
  for (int t = lo[0]; t <= hi[0]; t++)
    for (int u = lo[1]; u <= u1; u++) {
      const int row = (D == 3) ? (t - slo[0]) * sn[1] + (u - slo[1]) : (t - slo[0]);
      R dxy = R(0);
      for (int d = 0; d < D - 1; d++) {
        R a = s_rlo[2 * row + d] - pp.xsp[d], b = pp.xsp[d] - s_rhi[2 * row + d];
        R w = a > b ? a : b;
        if (w > R(0)) dxy += w * w;
      }
      if (!(dxy <= lim2m)) continue;
      const R hw = sqrt_r<R>(lim2m - dxy); /* half chord of the 2h sphere */
      const R za = zp - hw, zb = zp + hw;
      const int eb = s_off[row], ee = s_off[row + 1];
      const long long dl = s_rsrc[row] - eb;
      auto ENT = [&](int e) -> V4 { return GL ? RS.row[e + dl] : s_ent[e]; };
      auto REC = [&](int e) -> V4 { return (SREC && !GL) ? s_rec[e] : RS.rec[e + dl]; };
      auto TAG = [&](int e) -> int {
        if constexpr (GL) return (int)RS.rk[e + dl] - slo[RA];
        else return (int)s_tag[e];
      };
      auto ZOF = [&](const V4& v) -> R { return RA == 2 ? v.z : v.y; };
      int e = eb, hi_e = ee;
      while (e < hi_e) { /* first entry with coordinate >= za */
        const int m = (e + hi_e) >> 1;
        if (ZOF(ENT(m)) < za) e = m + 1;
        else hi_e = m;
      }
      for (; e < ee; e += 2) {
        const bool hasb = e + 1 < ee;
        const V4 va = ENT(e), vb = ENT(hasb ? e + 1 : e);
        if (ZOF(va) > zb) break;
        const bool inb = hasb && !(ZOF(vb) > zb);
        const int ta = TAG(e), tb = TAG(hasb ? e + 1 : e);
        bool ma = (unsigned)(ta - clo) <= (unsigned)(chi - clo);
        bool mb = inb && (unsigned)(tb - clo) <= (unsigned)(chi - clo);
        /* within 2h at the stage start (the direct variants' test, both entries at once) */
        R ddA, ddB;
        if constexpr (sizeof(R) == 4) {
          float2 dx = __fadd2_rn(make_float2(pp.xsp[0], pp.xsp[0]), make_float2(-va.x, -vb.x));
          float2 dd = __fmul2_rn(dx, dx);
          float2 dy = __fadd2_rn(make_float2(pp.xsp[1], pp.xsp[1]), make_float2(-va.y, -vb.y));
          dd = __ffma2_rn(dy, dy, dd);
          if constexpr (D == 3) {
            float2 dz = __fadd2_rn(make_float2(pp.xsp[2], pp.xsp[2]), make_float2(-va.z, -vb.z));
            dd = __ffma2_rn(dz, dz, dd);
          }
          ddA = dd.x;
          ddB = dd.y;
        } else {
          R xa[3] = {va.x, va.y, va.z}, xb[3] = {vb.x, vb.y, vb.z};
          ddA = ddB = R(0);
          for (int d = 0; d < D; d++) {
            R t0 = pp.xsp[d] - xa[d], t1 = pp.xsp[d] - xb[d];
            ddA = (d == 0) ? t0 * t0 : ddA + t0 * t0;
            ddB = (d == 0) ? t1 * t1 : ddB + t1 * t1;
          }
        }
        ma = ma && ddA <= pp.lim2;
        mb = mb && ddB <= pp.lim2;
        if (ma || mb) {
          const V4 ra = REC(e), rb = REC(hasb ? e + 1 : e);
          if constexpr (sizeof(R) == 4) {
            const float2 drx = __fadd2_rn(make_float2(pp.xnp[0], pp.xnp[0]), make_float2(-ra.x, -rb.x));
            const float2 dry = __fadd2_rn(make_float2(pp.xnp[1], pp.xnp[1]), make_float2(-ra.y, -rb.y));
            float2 drz = make_float2(0.f, 0.f);
            float2 d2 = __fmul2_rn(drx, drx);
            d2 = __ffma2_rn(dry, dry, d2);
            if constexpr (D == 3) {
              drz = __fadd2_rn(make_float2(pp.xnp[2], pp.xnp[2]), make_float2(-ra.z, -rb.z));
              d2 = __ffma2_rn(drz, drz, d2);
            }
            /* a coincident pair contributes nothing (the reference skips it) */
            const bool ka = ma && d2.x > 0.f, kb = mb && d2.y > 0.f;
            const float2 rq = make_float2(ka ? rsqrtf(d2.x) : 0.f, kb ? rsqrtf(d2.y) : 0.f);
            float2 sv = __fmul2_rn(__fmul2_rn(d2, rq), make_float2(pp.inv_hh, pp.inv_hh));
            /* beyond the support (s >= 2) W and its gradient vanish: q = 0 there */
            sv.x = fminf(sv.x, 2.f);
            sv.y = fminf(sv.y, 2.f);
            const float2 q = __ffma2_rn(sv, make_float2(-0.5f, -0.5f), make_float2(1.f, 1.f));
            const float2 q2 = __fmul2_rn(q, q), q3 = __fmul2_rn(q2, q);
            /* the direct variants' arithmetic, operation for operation:
             * w = q^4 (1 + 2s), rr = cwr w, tmp1 = tmp1c + tmp1c5 rr^4,
             * f = aw_c q^3 tmp1 vol */
            const float2 w = __fmul2_rn(__fmul2_rn(q2, q2), __ffma2_rn(sv, make_float2(2.f, 2.f), make_float2(1.f, 1.f)));
            const float2 rr = __fmul2_rn(make_float2(pp.cwr, pp.cwr), w);
            const float2 rr2 = __fmul2_rn(rr, rr);
            const float2 t1 = __ffma2_rn(make_float2(pp.tmp1c5, pp.tmp1c5), __fmul2_rn(rr2, rr2),
                                         make_float2(pp.tmp1c, pp.tmp1c));
            const float2 vm = make_float2(ka ? fabsf(ra.w) : 0.f, kb ? fabsf(rb.w) : 0.f);
            const float2 f = __fmul2_rn(__fmul2_rn(__fmul2_rn(make_float2(pp.aw_c, pp.aw_c), q3), t1), vm);
            /* summed in candidate order, as the direct variants do */
            if (ka) {
              pp.pst[0] = fmaf(drx.x, f.x, pp.pst[0]);
              pp.pst[1] = fmaf(dry.x, f.x, pp.pst[1]);
              if constexpr (D == 3) pp.pst[2] = fmaf(drz.x, f.x, pp.pst[2]);
            }
            if (kb) {
              pp.pst[0] = fmaf(drx.y, f.y, pp.pst[0]);
              pp.pst[1] = fmaf(dry.y, f.y, pp.pst[1]);
              if constexpr (D == 3) pp.pst[2] = fmaf(drz.y, f.y, pp.pst[2]);
            }
            /* across the interface: the sharpening term (rare) */
            const bool xa = ka && rec_phase(ra) != pp.ph, xb = kb && rec_phase(rb) != pp.ph;
            if (xa || xb) {
              for (int k = 0; k < 2; k++) {
                if (!(k == 0 ? xa : xb)) continue;
                const int32_t qs = slot_of<R>(k == 0 ? va.w : vb.w);
                const R* rc2 = P.rec2 + 2 * (int64_t)qs;
                const R rhoq = rc2[0], cq = rc2[1];
                const R tmp2 = R(1.) / (pp.rho_p + rhoq);
                const R cs = R(-0.1) * tmp2 * (pp.crho_p + cq * cq * rhoq);
                const R g = cs * pp.aw_c * (k == 0 ? q3.x : q3.y) * (k == 0 ? vm.x : vm.y);
                pp.phs[0] += (k == 0 ? drx.x : drx.y) * g;
                pp.phs[1] += (k == 0 ? dry.x : dry.y) * g;
                if constexpr (D == 3) pp.phs[2] += (k == 0 ? drz.x : drz.y) * g;
              }
            }
          } else {
            if (ma) {
              R xnq[3] = {ra.x, ra.y, ra.z};
              pp.add(xnq, fabs(ra.w), rec_phase(ra), P.rec2 + 2 * (int64_t)slot_of<R>(va.w), nullptr);
            }
            if (mb) {
              R xnq[3] = {rb.x, rb.y, rb.z};
              pp.add(xnq, fabs(rb.w), rec_phase(rb), P.rec2 + 2 * (int64_t)slot_of<R>(vb.w), nullptr);
            }
          }
        }
        if (!inb) break;
      }
    }
}

template <int D, typename R, bool SREC>
__global__ void __launch_bounds__(512, SREC ? 1 : 2) k_pst2(CaseK K, DevPtrs<R> P, int xs, int hs, int xn, int hn,
                                                            int nb0, int nb1, int cap, RowSorted<R> RS) {
  using BK = BigBrick<D>;
  using V4 = typename Vec4<R>::T;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const R dt = (R)P.cnt->dt;
  const R max_v = (R)P.cnt->max_v;
  const R* XS = P.X[xs];
  const R* XN = P.X[xn];
  const R* HS = P.H[hs];
  const R* HN = P.H[hn];
  const int b = blockIdx.x;
  int c0[3];
  c0[0] = (b / (nb0 * nb1)) * BK::B0;
  c0[1] = ((b / nb0) % nb1) * BK::B1;
  c0[2] = (D == 3) ? (b % nb0) * BK::B2 : 0;
  const int bdim[3] = {BK::B0, BK::B1, D == 3 ? BK::B2 : 1};
  int slo[3], sn[3];
  for (int d = 0; d < 3; d++) {
    const int r = (d < D) ? K.rad2 : 0;
    const int Nd = (d < D) ? K.N[d] : 1;
    slo[d] = max(c0[d] - r, 0);
    sn[d] = min(c0[d] + bdim[d] - 1 + r, Nd - 1) - slo[d] + 1;
  }
  const int nsc = sn[0] * sn[1] * sn[2];
  const int nrow = (D == 3) ? sn[0] * sn[1] : sn[0];
  constexpr int RA = D - 1;
  /* shared layout: off[nrow+1] | rsrc[nrow] | rlo[2 nrow] | rhi[2 nrow] | bnd[nsc] | ent[cap] | rec[cap] | tag[cap] */
  size_t o = 0;
  auto take = [&](size_t bytes, size_t al) {
    o = (o + al - 1) / al * al;
    const size_t r0 = o;
    o += bytes;
    return smem_raw + r0;
  };
  int* s_off = reinterpret_cast<int*>(take(sizeof(int) * (nrow + 1), 16));
  long long* s_rsrc = reinterpret_cast<long long*>(take(sizeof(long long) * nrow, 16));
  R* s_rlo = reinterpret_cast<R*>(take(sizeof(R) * 2 * nrow, 16));
  R* s_rhi = reinterpret_cast<R*>(take(sizeof(R) * 2 * nrow, 16));
  int* s_bnd = reinterpret_cast<int*>(take(sizeof(int) * nsc, 16));
  V4* s_ent = reinterpret_cast<V4*>(take(sizeof(V4) * cap, 32));
  V4* s_rec = SREC ? reinterpret_cast<V4*>(take(sizeof(V4) * cap, 32)) : nullptr;
  unsigned char* s_tag = take(cap, 16);
  __shared__ int s_red[SCAN_RED];
  for (int l = threadIdx.x; l < nsc; l += blockDim.x) {
    const int t = l / (sn[1] * sn[2]), s = (l / sn[2]) % sn[1], m = l % sn[2];
    const int64_t c = ((int64_t)(slo[0] + t) * K.N[1] + (slo[1] + s)) * K.N[2] + (slo[2] + m);
    s_bnd[l] = P.boff[c + 1] > P.boff[c] ? 1 : 0;
  }
  const int NR = K.N[RA];
  for (int row = threadIdx.x; row < nrow; row += blockDim.x) {
    const int64_t gr = (D == 3) ? (int64_t)(slo[0] + row / sn[1]) * K.N[1] + (slo[1] + row % sn[1])
                                : (int64_t)(slo[0] + row);
    int first = INT_MAX, last = -1;
    for (int k = 0; k < sn[RA]; k++) {
      const int64_t c = gr * NR + slo[RA] + k;
      first = min(first, RS.pmin[c]);
      last = max(last, RS.pmax[c]);
    }
    s_off[row + 1] = last >= first ? last - first + 1 : 0;
    s_rsrc[row] = gr * NR * K.maxpc + (last >= first ? first : 0);
  }
  __syncthreads();
  const int s_total = block_scan_counts(s_off, nrow, s_red);
  const bool use_sm = s_total <= cap;
  /* one warp per row: the row's bounds in the other axes (always), and the
   * copy of its range with each entry's window tag (when it fits) */
  {
    const int lane = threadIdx.x & 31;
    for (int row = threadIdx.x >> 5; row < nrow; row += blockDim.x >> 5) {
      const int e0 = s_off[row], len = s_off[row + 1] - e0;
      const int64_t src = s_rsrc[row];
      R mn[2] = {R(1e30), R(1e30)}, mx[2] = {R(-1e30), R(-1e30)};
      for (int i = lane; i < len; i += 32) {
        const V4 v = RS.row[src + i];
        if (use_sm) {
          const int kk = (int)RS.rk[src + i] - slo[RA];
          s_ent[e0 + i] = v;
          s_tag[e0 + i] = (unsigned char)((kk >= 0 && kk < sn[RA]) ? kk : 255);
          if constexpr (SREC) s_rec[e0 + i] = RS.rec[src + i];
        }
        const R xv[2] = {v.x, v.y};
        for (int d = 0; d < D - 1; d++) {
          mn[d] = xv[d] < mn[d] ? xv[d] : mn[d];
          mx[d] = xv[d] > mx[d] ? xv[d] : mx[d];
        }
      }
      for (int d = 0; d < D - 1; d++) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const R a = __shfl_xor_sync(0xffffffffu, mn[d], off), bb = __shfl_xor_sync(0xffffffffu, mx[d], off);
          mn[d] = a < mn[d] ? a : mn[d];
          mx[d] = bb > mx[d] ? bb : mx[d];
        }
      }
      if (lane < D - 1) {
        s_rlo[2 * row + lane] = lane == 0 ? mn[0] : mn[1];
        s_rhi[2 * row + lane] = lane == 0 ? mx[0] : mx[1];
      }
    }
  }
  __syncthreads();
  /* the brick's own particles, one per thread */
  const int nbc = bdim[0] * bdim[1] * bdim[2];
  __shared__ int s_boff[BK::B0 * BK::B1 * BK::B2 + 1];
  __shared__ int s_bcell[BK::B0 * BK::B1 * BK::B2];
  for (int q = threadIdx.x; q < nbc; q += blockDim.x) {
    const int d0 = q / (bdim[1] * bdim[2]), d1 = (q / bdim[2]) % bdim[1], d2 = q % bdim[2];
    const int ci = c0[0] + d0, cj = c0[1] + d1, ck = c0[2] + d2;
    int cnt = 0;
    int64_t c = -1;
    if (ci < K.N[0] && cj < K.N[1] && ck < K.N[2]) {
      c = ((int64_t)ci * K.N[1] + cj) * K.N[2] + ck;
      cnt = min(P.bcnt[c], K.maxpc);
    }
    s_bcell[q] = (int)c;
    s_boff[q + 1] = cnt;
  }
  __syncthreads();
  const int npart = block_scan_counts(s_boff, nbc, s_red);
  for (int i = threadIdx.x; i < npart; i += blockDim.x) {
    int q = 0, qh = nbc - 1;
    while (q < qh) {
      const int md = (q + qh + 1) >> 1;
      if (s_boff[md] <= i) q = md;
      else qh = md - 1;
    }
    const int64_t c = s_bcell[q];
    const int32_t p = P.bucket[c * K.maxpc + (i - s_boff[q])];
    PstPart<D, R, false> pp;
    pp.ph = P.phase[p];
    for (int d = 0; d < 3; d++) pp.xsp[d] = pp.xnp[d] = R(0);
    for (int d = 0; d < D; d++) {
      pp.xsp[d] = XS[d * K.cap + p];
      pp.xnp[d] = XN[d * K.cap + p];
    }
    pp.hs_p = HS[p];
    pp.hh = HN[p];
    pp.rho_p = P.rho[p];
    pp.c_p = P.c[p];
    pp.init(K, max_v);
    int pos[3], lo[3], hi[3];
    cell_pos<D, R>(K, pp.xsp, pos);
    bool inside = true;
    for (int d = 0; d < 3; d++) {
      const int r = (d < D) ? K.rad2 : 0;
      lo[d] = max(pos[d] - r, 0);
      hi[d] = min(pos[d] + r, (d < D ? K.N[d] : 1) - 1);
      if (lo[d] < slo[d] || hi[d] >= slo[d] + sn[d]) inside = false;
    }
    if (!inside) {
      /* drifted out of the staged box: the per-cell scan in the reference's order */
      pst_particle<D, R, false, 0>(K, P, p, XS, XN, HS, HN, dt, max_v, nullptr);
      continue;
    }
    if (use_sm)
      pst2_rows<D, R, SREC, false>(K, P, RS, s_off, s_rsrc, s_rlo, s_rhi, s_ent, s_rec, s_tag, slo, sn, lo, hi, pp);
    else
      pst2_rows<D, R, SREC, true>(K, P, RS, s_off, s_rsrc, s_rlo, s_rhi, s_ent, s_rec, s_tag, slo, sn, lo, hi, pp);
    bool edge = false;
    for (int d = 0; d < D; d++) edge = edge || lo[d] == 0 || hi[d] == K.N[d] - 1;
    if (edge)
      for (int t = lo[0]; t <= hi[0]; t++)
        for (int s = lo[1]; s <= hi[1]; s++)
          for (int m = lo[2]; m <= hi[2]; m++) {
            const int l = ((t - slo[0]) * sn[1] + (s - slo[1])) * sn[2] + (m - slo[2]);
            if (!s_bnd[l]) continue;
            const int64_t cc = ((int64_t)t * K.N[1] + s) * K.N[2] + m;
            pst_boundary_cell<D, R, false>(K, P, cc, pp);
          }
    pst_finish<D, R, false>(K, P, p, dt, pp);
  }
}

template <int D, typename R, bool SREC>
static void pst2_launch(const CaseK& K, const DevPtrs<R>& P, int xs, int hs, int xn, int hn, const RowSorted<R>& RS,
                        cudaStream_t st) {
  using BK = BigBrick<D>;
  using V4 = typename Vec4<R>::T;
  const int nb0 = (D == 3) ? (K.N[2] + BK::B2 - 1) / BK::B2 : 1;
  const int nb1 = (K.N[1] + BK::B1 - 1) / BK::B1;
  const int nbx = (K.N[0] + BK::B0 - 1) / BK::B0;
  const int r = K.rad2;
  const int nsc = (BK::B0 + 2 * r) * (BK::B1 + 2 * r) * (D == 3 ? BK::B2 + 2 * r : 1);
  const int nrow = (D == 3) ? (BK::B0 + 2 * r) * (BK::B1 + 2 * r) : (BK::B0 + 2 * r);
  const int ppc = (D == 3) ? 8 : 4;
  /* staging room per staged cell: 9 particles (variant 6: two blocks per SM),
   * 12 (variant 7: the fluid compressed behind a shock still fits) */
  int cap = SREC ? nsc * ppc * 3 / 2 : nsc * ppc * 9 / 8;
  auto bytes_for = [&](int cp) {
    size_t o = 0;
    auto take = [&](size_t bb, size_t al) { o = (o + al - 1) / al * al + bb; };
    take(sizeof(int) * (nrow + 1), 16);
    take(sizeof(long long) * nrow, 16);
    take(sizeof(R) * 2 * nrow, 16);
    take(sizeof(R) * 2 * nrow, 16);
    take(sizeof(int) * nsc, 16);
    take(sizeof(V4) * cp, 32);
    if (SREC) take(sizeof(V4) * cp, 32);
    take(cp, 16);
    return o + 64;
  };
  const size_t limit = SREC ? 210 * 1024 : 100 * 1024;
  while (bytes_for(cap) > limit && cap > 256) cap = cap * 7 / 8;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_pst2<D, R, SREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr_set = true;
  }
  k_pst2<D, R, SREC><<<nbx * nb1 * nb0, 512, bytes_for(cap), st>>>(K, P, xs, hs, xn, hn, nb0, nb1, cap, RS);
}

/* variants of the shifting kernel (the same members; results equal to rounding,
 * since variant 1 sums boundary particles in a second pass; the context's
 * autotuner times them on its own state and keeps the fastest): 0 per-lane row scan with
 * queued members, 1 warp-cooperative row scan, 2 per-lane scan summing members
 * at once, 3 the same for 3 blocks per SM, 4 direct sums over bricks of twice
 * the cells with 512 threads, 5 over bricks of four times the cells with 1024
 * threads, 6 and 7 the second form (row-ordered records, global-row scan of
 * over-full bricks, packed pair arithmetic; 7 stages the records too).  The
 * exact path has one. */
template <int D, typename R, bool EX>
int Launch<D, R, EX>::pst_variants() {
  return EX ? 1 : 8;
}

/* device scratch of the per-stage row sort (0 on the exact path) */
template <int D, typename R, bool EX>
size_t Launch<D, R, EX>::pst_scratch_bytes(const CaseK& K) {
  return EX ? 0 : rowsort_layout<R>(K, nullptr, nullptr);
}

/* the per-stage row sort of the mixed and FMA paths (three launches; nothing
 * on the exact path) */
template <int D, typename R, bool EX>
void Launch<D, R, EX>::rowsort(const CaseK& K, const DevPtrs<R>& P, int xs, void* scratch, cudaStream_t st) {
  if constexpr (!EX) {
    RowSortBufs<R> B;
    rowsort_layout<R>(K, static_cast<unsigned char*>(scratch), &B);
    const int64_t nrows = K.ncell / K.N[D - 1];
    const size_t shb = sizeof(typename Vec4<R>::T) * RS_CAP * RS_T;
    static bool attr_set = false;
    if (!attr_set) {
      cudaFuncSetAttribute(k_rs_cells<D, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shb);
      attr_set = true;
    }
    k_rs_cells<D, R><<<grid_for(K.ncell, RS_T), RS_T, shb, st>>>(K, P, xs, B);
    k_rs_rows<D, R><<<grid_for(nrows * 32, 128), 128, 0, st>>>(K, P, B);
    k_rs_rank<D, R><<<grid_for(K.ncell, 256), 256, 0, st>>>(K, P, B);
  }
}

/* the shifting kernel (one launch); on the mixed and FMA paths it reads the
 * rows sorted by rowsort() for the same stage */
template <int D, typename R, bool EX>
void Launch<D, R, EX>::pst(const CaseK& K, const DevPtrs<R>& P, int xs, int hs, int xn, int hn, int var,
                           void* scratch, cudaStream_t st) {
  if constexpr (EX) {
    pst_launch<D, R, EX, 0>(K, P, xs, hs, xn, hn, RowSorted<R>{}, st);
  } else {
    RowSortBufs<R> B;
    rowsort_layout<R>(K, static_cast<unsigned char*>(scratch), &B);
    const RowSorted<R> RS{B.row, B.rec, B.rk, B.pmin, B.pmax};
    if (var == 1) pst_launch<D, R, EX, 1>(K, P, xs, hs, xn, hn, RS, st);
    else if (var == 2) pst_launch<D, R, EX, 2>(K, P, xs, hs, xn, hn, RS, st);
    else if (var == 3) pst_launch<D, R, EX, 3>(K, P, xs, hs, xn, hn, RS, st);
    else if (var == 4) pst_launch<D, R, EX, 5>(K, P, xs, hs, xn, hn, RS, st);
    else if (var == 5) pst_launch<D, R, EX, 6>(K, P, xs, hs, xn, hn, RS, st);
    else if (var == 6) pst2_launch<D, R, false>(K, P, xs, hs, xn, hn, RS, st);
    else if (var == 7) pst2_launch<D, R, true>(K, P, xs, hs, xn, hn, RS, st);
    else pst_launch<D, R, EX, 0>(K, P, xs, hs, xn, hn, RS, st);
  }
}

#define PGDG_INST(D, R, EX)                                                                              \
  template void Launch<D, R, EX>::g2p(const CaseK&, const DevPtrs<R>&, int, int, int, int, int, bool,     \
                                      cudaStream_t);                                                       \
  template void Launch<D, R, EX>::pst(const CaseK&, const DevPtrs<R>&, int, int, int, int, int, void*,        \
                                      cudaStream_t);                                                       \
  template size_t Launch<D, R, EX>::pst_scratch_bytes(const CaseK&);                                       \
  template void Launch<D, R, EX>::rowsort(const CaseK&, const DevPtrs<R>&, int, void*, cudaStream_t);        \
  template int Launch<D, R, EX>::pst_variants();
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
