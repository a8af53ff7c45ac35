/*
 * k_mlp.cu -- the MGFM seed surrogate: a 12-64-64-64-2 tanh MLP that predicts the
 * star pressure and velocity of the two-material Riemann problem solved by
 * MPM::MGFM (mpm.cpp:882-926), used as the Newton starting guess in place of the
 * reference's max(p_l, p_r) (mpm.cpp:893).  The pressure output is a log
 * correction to a closed-form two-shock baseline (mgfm_baseline below); the
 * velocity output is trained with a small weight and does not enter the seed.  The plain Newton solve stays the
 * fallback and the final check: a seeded solve that does not reach |f| <= tol within
 * the iteration cap is redone from the plain seed, and a problem without a
 * positive root (f(1e-8) < 0) goes straight to the plain solve.
 *
 * Everything here is project code: feature construction, forward pass (BF16
 * weights, FP32 accumulation), backward pass and Adam, all on the device.
 *
 * Parameter layout (FP32 master copy, n = 9282):
 *   W1[64][12] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[2][64] b4[2]
 * followed by the fixed feature/target normalisation (NORM = 28 floats):
 *   mean_x[12] std_x[12] mean_y[2] std_y[2]
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/pgdg.h"
#include "pgdg_dev.cuh"

namespace pgdg {

constexpr int NI = 12, NH = 64, NO = 2;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NI, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH * NH, OFF_W4 = OFF_B3 + NH, OFF_B4 = OFF_W4 + NO * NH,
              NPARAM = OFF_B4 + NO;
constexpr int NNORM = 2 * NI + 2 * NO;

/* ------------------------------------------------------------------ */
/* features of one Riemann problem                                    */
/* ------------------------------------------------------------------ */
/* Closed-form baseline p_b of the star pressure: the acoustic estimate
 * p_ac = (Z_r p_l + Z_l p_r + Z_l Z_r (u_l - u_r)) / (Z_l + Z_r), Z = sqrt(gamma (p + p_inf) rho),
 * then one linearised step of the two-shock relation with the shock speeds W
 * (mpm.cpp:908, glbfunc.h:314-337) frozen at max(p_ac, 1e-8).  For weak waves
 * the error is far below the Newton tolerance; the network corrects strong ones. */
__host__ __device__ inline double mgfm_baseline(double ul, double ur, double pl, double pr, double rl, double rr,
                                                double gl, double il, double gr, double ir) {
  const double Zl = sqrt(gl * (pl + il) * rl), Zr = sqrt(gr * (pr + ir) * rr);
  double p0 = (Zr * pl + Zl * pr + Zl * Zr * (ul - ur)) / (Zl + Zr);
  if (!(p0 > 1e-8)) p0 = 1e-8;
  const double Wl = sqrt(0.5 * rl * ((gl + 1.) * p0 + (gl - 1.) * pl + 2. * gl * il));
  const double Wr = sqrt(0.5 * rr * ((gr + 1.) * p0 + (gr - 1.) * pr + 2. * gr * ir));
  double pt = (pl / Wl + pr / Wr + (ul - ur)) / (1. / Wl + 1. / Wr);
  if (!(pt > 1e-8)) pt = 1e-8;
  return pt;
}

/* Scale-free description of a problem (FP32 transcendentals; the baseline in
 * FP64):
 *   x0,x1  log((p + p_inf)/P0) left/right, P0 the larger effective pressure
 *   x2     log(rho_l / rho_r)
 *   x3     (u_l - u_r) / a0, a0 = sqrt(P0 / sqrt(rho_l rho_r)), clamped to +-20
 *   x4     log(p_b / p_l)          x11  log(p_b / p_r)
 *   x5,x6  gamma left/right        x7,x8  p_inf / P0 left/right
 *   x9,x10 log(p / P0) left/right
 * The network's first output y predicts log(p* / p_b) / sc with the strength
 * scale sc = s^2 / (1 + s^2), s = |x4| + |x11|: the correction vanishes for
 * weak waves, where the baseline is already far inside the Newton tolerance. */
__host__ __device__ inline void mgfm_features(const double* q, double gl, double il, double gr, double ir, float* x,
                                              double* pb_out, float* sc_out) {
  double ul = q[0], ur = q[1], pl = q[2], pr = q[3], rl = q[4], rr = q[5];
  if (pl < 1e-10) pl = 1e-10;
  if (pr < 1e-10) pr = 1e-10;
  if (rl < 1e-10) rl = 1e-10;
  if (rr < 1e-10) rr = 1e-10;
  const double Pl = pl + il, Pr = pr + ir;
  const double P0 = Pl > Pr ? Pl : Pr;
  const float a0 = sqrtf((float)P0 / sqrtf((float)rl * (float)rr));
  const float du = (float)(ul - ur) / a0;
  const double pb = mgfm_baseline(ul, ur, pl, pr, rl, rr, gl, il, gr, ir);
  const float lbl = logf((float)(pb / pl)), lbr = logf((float)(pb / pr));
  const float sv = fabsf(lbl) + fabsf(lbr);
  x[0] = logf((float)(Pl / P0));
  x[1] = logf((float)(Pr / P0));
  x[2] = logf((float)(rl / rr));
  x[3] = du > 20.f ? 20.f : (du < -20.f ? -20.f : du);
  x[4] = lbl;
  x[5] = (float)gl;
  x[6] = (float)gr;
  x[7] = (float)(il / P0);
  x[8] = (float)(ir / P0);
  x[9] = logf((float)(pl / P0 + 1e-30));
  x[10] = logf((float)(pr / P0 + 1e-30));
  x[11] = lbr;
  *pb_out = pb;
  *sc_out = sv * sv / (1.f + sv * sv);
}

__global__ void k_features(const double* in6, const int8_t* mat2, const double* gam, const double* pinf, float* X,
                           int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int s = mat2[2 * i], s1 = mat2[2 * i + 1];
    double pb;
    float sc, x[NI];
    mgfm_features(in6 + 6 * i, gam[s], pinf[s], gam[s1], pinf[s1], x, &pb, &sc);
    for (int k = 0; k < NI; k++) X[i * NI + k] = x[k];
  }
}

/* ------------------------------------------------------------------ */
/* forward pass: one thread per sample, weights (BF16-rounded) in smem */
/* ------------------------------------------------------------------ */
template <bool BF16>
__device__ __forceinline__ float wq(float w) {
  if (BF16) return __bfloat162float(__float2bfloat16_rn(w));
  return w;
}

/* stage the parameters in shared memory, weights rounded to BF16 when asked */
template <bool BF16>
__device__ __forceinline__ void load_params(const float* __restrict__ params, float* w) {
  for (int k = threadIdx.x; k < NPARAM; k += blockDim.x) {
    bool isb = (k >= OFF_B1 && k < OFF_W2) || (k >= OFF_B2 && k < OFF_W3) || (k >= OFF_B3 && k < OFF_W4) || k >= OFF_B4;
    w[k] = isb ? params[k] : wq<BF16>(params[k]);
  }
  for (int k = threadIdx.x; k < NNORM; k += blockDim.x) w[NPARAM + k] = params[NPARAM + k];
  __syncthreads();
}

/* one sample through the network (normalised input xn); the loops are fully
 * unrolled so the activations stay in registers; A1..A3 (optional) receive the
 * hidden activations for the backward pass */
template <int NOUT>
__device__ __forceinline__ void mlp_eval(const float* w, const float* xn, float* y, float* A1, float* A2, float* A3,
                                         int64_t i) {
  float h[NH], g[NH];
#pragma unroll
  for (int j = 0; j < NH; j++) {
    float a = w[OFF_B1 + j];
#pragma unroll
    for (int k = 0; k < NI; k++) a = fmaf(w[OFF_W1 + j * NI + k], xn[k], a);
    h[j] = tanhf(a);
  }
  if (A1)
#pragma unroll
    for (int j = 0; j < NH; j++) A1[i * NH + j] = h[j];
#pragma unroll
  for (int j = 0; j < NH; j++) {
    float a = w[OFF_B2 + j];
#pragma unroll
    for (int k = 0; k < NH; k++) a = fmaf(w[OFF_W2 + j * NH + k], h[k], a);
    g[j] = tanhf(a);
  }
  if (A2)
#pragma unroll
    for (int j = 0; j < NH; j++) A2[i * NH + j] = g[j];
#pragma unroll
  for (int j = 0; j < NH; j++) {
    float a = w[OFF_B3 + j];
#pragma unroll
    for (int k = 0; k < NH; k++) a = fmaf(w[OFF_W3 + j * NH + k], g[k], a);
    h[j] = tanhf(a);
  }
  if (A3)
#pragma unroll
    for (int j = 0; j < NH; j++) A3[i * NH + j] = h[j];
#pragma unroll
  for (int o = 0; o < NOUT; o++) {
    float a = w[OFF_B4 + o];
#pragma unroll
    for (int k = 0; k < NH; k++) a = fmaf(w[OFF_W4 + o * NH + k], h[k], a);
    y[o] = a;
  }
}

/* Y[n][2] (normalised outputs) from raw features X; optionally store hidden
 * activations for the backward pass (A1,A2,A3 [n][64]) */
template <bool BF16>
__global__ void __launch_bounds__(128) k_mlp_forward(const float* __restrict__ params, const float* __restrict__ X,
                                                     float* __restrict__ Y, float* A1, float* A2, float* A3,
                                                     int64_t n, const unsigned long long* __restrict__ dn) {
  if (dn && (int64_t)*dn < n) n = (int64_t)*dn; /* live count of a batch sized for capacity */
  __shared__ __align__(16) float w[NPARAM + NNORM];
  load_params<BF16>(params, w);
  const float* mx = w + NPARAM;
  const float* sx = mx + NI;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float xn[NI], y[NO];
#pragma unroll
    for (int k = 0; k < NI; k++) xn[k] = (X[i * NI + k] - mx[k]) / sx[k];
    mlp_eval<NO>(w, xn, y, A1, A2, A3, i);
    Y[i * NO + 0] = y[0];
    Y[i * NO + 1] = y[1];
  }
}

/* ------------------------------------------------------------------ */
/* backward pass                                                      */
/* ------------------------------------------------------------------ */
/* dZ4 = 2 (Y - T_norm) / n ; loss partial sums */
__global__ void k_out_grad(const float* Y, const float* T, const float* params, float* dZ, double* loss, int64_t n) {
  const float* my = params + NPARAM + 2 * NI;
  const float* sy = my + NO;
  double acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int o = 0; o < NO; o++) {
      float t = (T[i * NO + o] - my[o]) / sy[o];
      float d = Y[i * NO + o] - t;
      dZ[i * NO + o] = 2.f * d / (float)(n * NO);
      acc += (double)d * d;
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

/* dA[n][K] = dZ[n][J] W[J][K]; then dZ_prev = dA * (1 - A^2)  (tanh) */
template <bool BF16>
__global__ void k_back_act(const float* dZ, const float* params, int woff, int J, int K, const float* A, float* dZp,
                           int64_t n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * K; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = t / K;
    int k = (int)(t % K);
    float s = 0;
    for (int j = 0; j < J; j++) s = fmaf(dZ[i * J + j], wq<BF16>(params[woff + j * K + k]), s);
    float a = A[i * K + k];
    dZp[t] = s * (1.f - a * a);
  }
}

/* gW[J][K] = sum_i dZ[i][J] Ain[i][K] ; gb[J] = sum_i dZ[i][J]; one block per (j) row,
 * threads over k and the batch */
__global__ void k_wgrad(const float* dZ, const float* Ain, int J, int K, float* gW, float* gb, int64_t n) {
  const int j = blockIdx.x;
  extern __shared__ float red[];
  for (int k = threadIdx.y; k < K + 1; k += blockDim.y) {
    float s = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      float a = (k < K) ? Ain[i * K + k] : 1.f;
      s = fmaf(dZ[i * J + j], a, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) red[k] = s;
  }
  __syncthreads();
  for (int k = threadIdx.y * blockDim.x + threadIdx.x; k < K + 1; k += blockDim.x * blockDim.y) {
    if (k < K) gW[j * K + k] = red[k];
    else gb[j] = red[k];
  }
}

/* normalised input features for the first layer's weight gradient */
__global__ void k_norm_x(const float* X, const float* params, float* Xn, int64_t n) {
  const float* mx = params + NPARAM;
  const float* sx = mx + NI;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * NI; t += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(t % NI);
    Xn[t] = (X[t] - mx[k]) / sx[k];
  }
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, int np, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np; k += gridDim.x * blockDim.x) {
    float gk = g[k];
    float mk = b1 * m[k] + (1 - b1) * gk;
    float vk = b2 * v[k] + (1 - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
  }
}

/* ------------------------------------------------------------------ */
/* seeded MGFM                                                        */
/* ------------------------------------------------------------------ */
/* f(p) of the two-shock relation at p (mpm.cpp:908) */
__device__ __forceinline__ double mgfm_f(double ul, double ur, double pl, double pr, double rhol, double rhor,
                                         double gl, double pinfl, double gr, double pinfr, double p) {
  double Wl = wl_cal(rhol, pl, p, gl, pinfl);
  double Wr = wl_cal(rhor, pr, p, gr, pinfr);
  return ul - ur - (p - pl) / Wl - (p - pr) / Wr;
}

/* the seed from the baseline, the strength scale and the network output; an
 * output far outside the training range that overflows the exponential gives
 * -1, the plain seed */
__device__ __forceinline__ double seed_value(double pb, float sc, float y0, float my0, float sy0) {
  const double ps = pb * (double)expf(sc * (y0 * sy0 + my0));
  if (!isfinite(ps)) return -1.0;
  return ps > 1e-8 ? ps : 1e-8;
}

/* Seeds of a batch: features, network and seed p_b exp(sc y) in one pass per
 * problem; -1 (plain solve) for a problem without a positive root, f(1e-8) < 0,
 * evaluated with the clamps of the MGFM variant (mpm.cpp:886-893). */
template <bool BF16>
__global__ void __launch_bounds__(128) k_seed(const float* __restrict__ params, const double* __restrict__ in6,
                                              const int8_t* __restrict__ mat2, const double* __restrict__ gam,
                                              const double* __restrict__ pinf, int variant, double* __restrict__ seed,
                                              int64_t n) {
  __shared__ __align__(16) float w[NPARAM + NNORM];
  load_params<BF16>(params, w);
  const float* mx = w + NPARAM;
  const float* sx = mx + NI;
  const float my0 = w[NPARAM + 2 * NI], sy0 = w[NPARAM + 2 * NI + NO];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* q = in6 + 6 * i;
    const int s = mat2[2 * i], s1 = mat2[2 * i + 1];
    const double gl = gam[s], il = pinf[s], gr = gam[s1], ir = pinf[s1];
    double pl = q[2], pr = q[3], rl = q[4], rr = q[5];
    if (variant == 0) {
      pl = amax1(pl, 1e-10);
      pr = amax1(pr, 1e-10);
      rl = amax1(rl, 1e-10);
      rr = amax1(rr, 1e-10);
    } else {
      if (pl < 0) pl = 0;
      if (pr < 0) pr = 0;
    }
    if (mgfm_f(q[0], q[1], pl, pr, rl, rr, gl, il, gr, ir, 1e-8) < 0) {
      seed[i] = -1.0;
      continue;
    }
    double pb;
    float sc, xn[NI], y[1];
    mgfm_features(q, gl, il, gr, ir, xn, &pb, &sc);
#pragma unroll
    for (int k = 0; k < NI; k++) xn[k] = (xn[k] - mx[k]) / sx[k];
    mlp_eval<1>(w, xn, y, nullptr, nullptr, nullptr, i);
    seed[i] = seed_value(pb, sc, y[0], my0, sy0);
  }
}

/* first half of the split seed path: features, baseline and strength scale
 * of each problem (pb < 0 marks a problem without a positive root) */
__global__ void k_seed_features(const double* __restrict__ in6, const int8_t* __restrict__ mat2,
                                const double* __restrict__ gam, const double* __restrict__ pinf, int variant,
                                float* __restrict__ X, double* __restrict__ pb_out, float* __restrict__ sc_out,
                                int64_t n, const unsigned long long* __restrict__ dn) {
  if (dn && (int64_t)*dn < n) n = (int64_t)*dn;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* q = in6 + 6 * i;
    const int s = mat2[2 * i], s1 = mat2[2 * i + 1];
    const double gl = gam[s], il = pinf[s], gr = gam[s1], ir = pinf[s1];
    double pl = q[2], pr = q[3], rl = q[4], rr = q[5];
    if (variant == 0) {
      pl = amax1(pl, 1e-10);
      pr = amax1(pr, 1e-10);
      rl = amax1(rl, 1e-10);
      rr = amax1(rr, 1e-10);
    } else {
      if (pl < 0) pl = 0;
      if (pr < 0) pr = 0;
    }
    if (mgfm_f(q[0], q[1], pl, pr, rl, rr, gl, il, gr, ir, 1e-8) < 0) {
      pb_out[i] = -1.0;
      continue;
    }
    double pb;
    float sc, x[NI];
    mgfm_features(q, gl, il, gr, ir, x, &pb, &sc);
    for (int k = 0; k < NI; k++) X[i * NI + k] = x[k];
    pb_out[i] = pb;
    sc_out[i] = sc;
  }
}

/* partition of a batch by the existence of a positive root: a problem without
 * one runs the plain Newton solve down to the 1e-8 floor (about 30 iterations)
 * while a seeded one converges in two or three, so the two kinds are solved in
 * separate warps.  flag[i] = 1 for a problem with a root (pb > 0 when the seed
 * path computed it, else f(1e-8) >= 0 evaluated here). */
__global__ void k_root_flag(const double* __restrict__ in6, const int8_t* __restrict__ mat2,
                            const double* __restrict__ gam, const double* __restrict__ pinf, int variant,
                            const double* __restrict__ pb, unsigned long long* __restrict__ flag, int64_t n,
                            const unsigned long long* __restrict__ dn) {
  if (dn && (int64_t)*dn < n) n = (int64_t)*dn;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    bool root;
    if (pb) {
      root = pb[i] > 0;
    } else {
      const double* q = in6 + 6 * i;
      const int s = mat2[2 * i], s1 = mat2[2 * i + 1];
      double pl = q[2], pr = q[3], rl = q[4], rr = q[5];
      if (variant == 0) {
        pl = amax1(pl, 1e-10);
        pr = amax1(pr, 1e-10);
        rl = amax1(rl, 1e-10);
        rr = amax1(rr, 1e-10);
      } else {
        if (pl < 0) pl = 0;
        if (pr < 0) pr = 0;
      }
      root = !(mgfm_f(q[0], q[1], pl, pr, rl, rr, gam[s], pinf[s], gam[s1], pinf[s1], 1e-8) < 0);
    }
    flag[i] = root ? 1ull : 0ull;
  }
}
/* order: problems with a root first, then the others, each in input order;
 * pos is the exclusive prefix of the flags, nroot_p their total */
__global__ void k_root_perm(const unsigned long long* __restrict__ pos, const unsigned long long* __restrict__ nroot_p,
                            int32_t* __restrict__ perm, int64_t n, const unsigned long long* __restrict__ dn) {
  if (dn && (int64_t)*dn < n) n = (int64_t)*dn;
  const int64_t nroot = (int64_t)*nroot_p;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = (int64_t)pos[i];
    const bool root = (i + 1 < n ? (int64_t)pos[i + 1] : nroot) > p;
    perm[root ? p : nroot + (i - p)] = (int32_t)i;
  }
}

/* Newton from the seed (or the plain seed when seed is NULL or the entry is
 * negative); a seeded solve that has not converged at the cap is redone from
 * the plain seed, and its iterations are counted together */
__global__ void k_mgfm_seeded(const double* __restrict__ in6, const int8_t* __restrict__ mat2,
                              const double* __restrict__ gam, const double* __restrict__ pinf, int variant,
                              const double* __restrict__ seed, double* __restrict__ out3, int32_t* __restrict__ iters,
                              int64_t n, unsigned long long* stats, const float* __restrict__ Y,
                              const float* __restrict__ sc, const float* __restrict__ params,
                              const int32_t* __restrict__ perm, const int* __restrict__ yerr,
                              const unsigned long long* __restrict__ dn) {
  if (dn && (int64_t)*dn < n) n = (int64_t)*dn;
  unsigned long long nit = 0, nmax = 0, ncall = 0;
  /* a tensor-core forward pass that gave up leaves Y unset: every problem then
   * starts from the plain seed (the reference's), so results stay valid */
  if (yerr && *yerr) Y = nullptr;
  const float my0 = params ? params[NPARAM + 2 * NI] : 0.f, sy0 = params ? params[NPARAM + 2 * NI + NO] : 1.f;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? (int64_t)perm[j] : j;
    const double* q = in6 + 6 * i;
    int s = mat2[2 * i], s1 = mat2[2 * i + 1];
    double o[3];
    int it = 0;
    /* seed: given, or (split path) formed from the baseline in seed[], the
     * scale and the network output */
    double sd = seed ? seed[i] : -1.0;
    if (Y && sd > 0) sd = seed_value(sd, sc[i], Y[i * NO], my0, sy0);
    else if (seed && !Y && yerr) sd = -1.0;
    bool done = false;
    if (sd > 0) {
      it = mgfm(q[0], q[1], q[2], q[3], q[4], q[5], gam[s], pinf[s], gam[s1], pinf[s1], variant, sd, o);
      /* a seeded solve is kept only when it converged to finite values (a
       * non-finite iterate fails the tolerance test and would leave the loop
       * early); otherwise the problem is solved again from the plain seed */
      done = it < 50 && isfinite(o[0]) && isfinite(o[1]) && isfinite(o[2]);
    }
    if (!done) it += mgfm(q[0], q[1], q[2], q[3], q[4], q[5], gam[s], pinf[s], gam[s1], pinf[s1], variant, -1.0, o);
    out3[3 * i + 0] = o[0];
    out3[3 * i + 1] = o[1];
    out3[3 * i + 2] = o[2];
    if (iters) iters[i] = it;
    ncall++;
    nit += it;
    if (it >= 50) nmax++;
  }
  if (stats && ncall) {
    atomicAdd(&stats[0], ncall);
    atomicAdd(&stats[1], nit);
    if (nmax) atomicAdd(&stats[2], nmax);
  }
}

}  // namespace pgdg

/* ---------------------------------------------------------------------- */
/* host side                                                              */
/* ---------------------------------------------------------------------- */
using namespace pgdg;

struct pgdg_mlp {
  int bf16 = 1;
  int tc = 0;           /* forward passes on the tensor cores (BF16 activations) */
  int* d_tcerr = nullptr;
  float* d_params = nullptr; /* NPARAM + NNORM */
  float *d_m = nullptr, *d_v = nullptr, *d_g = nullptr;
  int64_t step = 0;
  /* scratch for training / batched calls */
  float *X = nullptr, *Xn = nullptr, *Y = nullptr, *A1 = nullptr, *A2 = nullptr, *A3 = nullptr, *dZ4 = nullptr,
        *dZ3 = nullptr, *dZ2 = nullptr, *dZ1 = nullptr;
  double* d_loss = nullptr;
  int64_t cap = 0;
  PartScratch part;         /* root partition of batched solves */
  double* seeds = nullptr; /* per-problem seeds (or baselines) of batched solves */
  float* sc = nullptr;     /* per-problem strength scale of the split seed path */
  float *Xb = nullptr, *Yb = nullptr; /* features and network outputs of batched solves */
  int64_t seeds_cap = 0;
  int reserve_seeds(int64_t n) {
    if (n <= seeds_cap) return PGDG_OK;
    void** bufs[] = {(void**)&seeds, (void**)&sc, (void**)&Xb, (void**)&Yb};
    const size_t w[] = {sizeof(double), sizeof(float), sizeof(float) * NI, sizeof(float) * NO};
    seeds_cap = 0;
    for (int k = 0; k < 4; k++) {
      if (*bufs[k]) cudaFree(*bufs[k]);
      *bufs[k] = nullptr;
      if (cudaMalloc(bufs[k], w[k] * (size_t)n) != cudaSuccess) return PGDG_ENOMEM;
    }
    seeds_cap = n;
    return PGDG_OK;
  }
  int reserve(int64_t n) {
    if (n <= cap) return PGDG_OK;
    float** bufs[] = {&X, &Xn, &Y, &A1, &A2, &A3, &dZ4, &dZ3, &dZ2, &dZ1};
    const int64_t w[] = {NI, NI, NO, NH, NH, NH, NO, NH, NH, NH};
    for (int k = 0; k < 10; k++) {
      if (*bufs[k]) cudaFree(*bufs[k]);
      if (cudaMalloc((void**)bufs[k], sizeof(float) * w[k] * n) != cudaSuccess) return PGDG_ENOMEM;
    }
    cap = n;
    return PGDG_OK;
  }
  ~pgdg_mlp() {
    float* bufs[] = {d_params, d_m, d_v, d_g, X, Xn, Y, A1, A2, A3, dZ4, dZ3, dZ2, dZ1};
    for (float* b : bufs)
      if (b) cudaFree(b);
    if (d_loss) cudaFree(d_loss);
    if (seeds) cudaFree(seeds);
    if (sc) cudaFree(sc);
    if (Xb) cudaFree(Xb);
    if (Yb) cudaFree(Yb);
    if (d_tcerr) cudaFree(d_tcerr);
    part.release();
  }
};

namespace {
inline int g_for(int64_t n, int b) {
  int64_t g = (n + b - 1) / b;
  if (g > 152 * 16) g = 152 * 16;
  return g < 1 ? 1 : (int)g;
}
void forward(pgdg_mlp* m, const float* X, float* Y, float* A1, float* A2, float* A3, int64_t n, cudaStream_t st,
             const unsigned long long* dn = nullptr) {
  if (m->tc && !A1) {
    /* the flag reports this forward pass only */
    cudaMemsetAsync(m->d_tcerr, 0, sizeof(int), st);
    mlp_tc_forward(m->d_params, X, Y, n, m->d_tcerr, st, dn);
    return;
  }
  if (m->bf16) k_mlp_forward<true><<<g_for(n, 128), 128, 0, st>>>(m->d_params, X, Y, A1, A2, A3, n, dn);
  else k_mlp_forward<false><<<g_for(n, 128), 128, 0, st>>>(m->d_params, X, Y, A1, A2, A3, n, dn);
}
void seed_launch(pgdg_mlp* m, const double* in6, const int8_t* mat2, const double* gam, const double* pinf,
                 int variant, double* seed, int64_t n, cudaStream_t st) {
  if (m->bf16) k_seed<true><<<g_for(n, 128), 128, 0, st>>>(m->d_params, in6, mat2, gam, pinf, variant, seed, n);
  else k_seed<false><<<g_for(n, 128), 128, 0, st>>>(m->d_params, in6, mat2, gam, pinf, variant, seed, n);
}
/* gradient of the mean squared error of the normalised outputs into m->d_g */
void gradients(pgdg_mlp* m, const float* X, const float* T, int64_t n, cudaStream_t st) {
  forward(m, X, m->Y, m->A1, m->A2, m->A3, n, st);
  cudaMemsetAsync(m->d_loss, 0, sizeof(double), st);
  k_out_grad<<<g_for(n, 256), 256, 0, st>>>(m->Y, T, m->d_params, m->dZ4, m->d_loss, n);
  const float* P = m->d_params;
  dim3 wb(32, 8);
  auto back = [&](const float* dZ, int woff, int J, int K, const float* A, float* dZp) {
    if (m->bf16) k_back_act<true><<<g_for(n * K, 256), 256, 0, st>>>(dZ, P, woff, J, K, A, dZp, n);
    else k_back_act<false><<<g_for(n * K, 256), 256, 0, st>>>(dZ, P, woff, J, K, A, dZp, n);
  };
  k_wgrad<<<NO, wb, sizeof(float) * (NH + 1), st>>>(m->dZ4, m->A3, NO, NH, m->d_g + OFF_W4, m->d_g + OFF_B4, n);
  back(m->dZ4, OFF_W4, NO, NH, m->A3, m->dZ3);
  k_wgrad<<<NH, wb, sizeof(float) * (NH + 1), st>>>(m->dZ3, m->A2, NH, NH, m->d_g + OFF_W3, m->d_g + OFF_B3, n);
  back(m->dZ3, OFF_W3, NH, NH, m->A2, m->dZ2);
  k_wgrad<<<NH, wb, sizeof(float) * (NH + 1), st>>>(m->dZ2, m->A1, NH, NH, m->d_g + OFF_W2, m->d_g + OFF_B2, n);
  back(m->dZ2, OFF_W2, NH, NH, m->A1, m->dZ1);
  k_norm_x<<<g_for(n * NI, 256), 256, 0, st>>>(X, P, m->Xn, n);
  k_wgrad<<<NH, wb, sizeof(float) * (NI + 1), st>>>(m->dZ1, m->Xn, NH, NI, m->d_g + OFF_W1, m->d_g + OFF_B1, n);
}
}  // namespace

extern "C" {

int pgdg_surrogate_create(int bf16, pgdg_mlp** out) {
  int dev = 0;
  if (cudaGetDeviceCount(&dev) != cudaSuccess || dev < 1) return PGDG_ECUDA;
  if (bf16 < 0 || bf16 > 2) return PGDG_EINVAL;
  pgdg_mlp* m = new pgdg_mlp();
  m->bf16 = bf16 ? 1 : 0;
  m->tc = bf16 == 2 ? 1 : 0;
  if (cudaMalloc((void**)&m->d_tcerr, sizeof(int)) != cudaSuccess) {
    delete m;
    return PGDG_ENOMEM;
  }
  cudaMemset(m->d_tcerr, 0, sizeof(int));
  const size_t np = NPARAM + NNORM;
  if (cudaMalloc((void**)&m->d_params, sizeof(float) * np) != cudaSuccess ||
      cudaMalloc((void**)&m->d_m, sizeof(float) * NPARAM) != cudaSuccess ||
      cudaMalloc((void**)&m->d_v, sizeof(float) * NPARAM) != cudaSuccess ||
      cudaMalloc((void**)&m->d_g, sizeof(float) * NPARAM) != cudaSuccess ||
      cudaMalloc((void**)&m->d_loss, sizeof(double)) != cudaSuccess) {
    delete m;
    return PGDG_ENOMEM;
  }
  cudaMemset(m->d_params, 0, sizeof(float) * np);
  cudaMemset(m->d_m, 0, sizeof(float) * NPARAM);
  cudaMemset(m->d_v, 0, sizeof(float) * NPARAM);
  *out = m;
  return PGDG_OK;
}
int pgdg_surrogate_destroy(pgdg_mlp* m) {
  delete m;
  return PGDG_OK;
}
int pgdg_surrogate_num_params(void) { return NPARAM + NNORM; }
/* host arrays of NPARAM + NNORM floats */
int pgdg_surrogate_set_params(pgdg_mlp* m, const float* params) {
  return cudaMemcpy(m->d_params, params, sizeof(float) * (NPARAM + NNORM), cudaMemcpyHostToDevice) == cudaSuccess
             ? PGDG_OK : PGDG_ECUDA;
}
int pgdg_surrogate_get_params(pgdg_mlp* m, float* params) {
  return cudaMemcpy(params, m->d_params, sizeof(float) * (NPARAM + NNORM), cudaMemcpyDeviceToHost) == cudaSuccess
             ? PGDG_OK : PGDG_ECUDA;
}
/* device pointers: in6 [n][6], mat2 [n][2], gam/pinf [nmat] -> X [n][12] */
int pgdg_surrogate_features(const double* in6, const int8_t* mat2, const double* gam, const double* pinf,
                            float* X, int64_t n) {
  if (n <= 0) return PGDG_OK;
  k_features<<<g_for(n, 256), 256>>>(in6, mat2, gam, pinf, X, n);
  return cudaGetLastError() == cudaSuccess ? PGDG_OK : PGDG_ECUDA;
}
/* device pointers: X [n][12] raw features -> Y [n][2] normalised outputs */
int pgdg_surrogate_forward(pgdg_mlp* m, const float* X, float* Y, int64_t n) {
  if (n <= 0) return PGDG_OK;
  forward(m, X, Y, nullptr, nullptr, nullptr, n, 0);
  if (cudaGetLastError() != cudaSuccess) return PGDG_ECUDA;
  if (m->tc) {
    int e = 0;
    if (cudaMemcpy(&e, m->d_tcerr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return PGDG_ECUDA;
    if (e) return PGDG_ETIMEOUT;
  }
  return PGDG_OK;
}
/* gradient of the loss 1/(2n) sum |Y - normalise(T)|^2 ... returned to the host
 * (NPARAM floats) together with the loss */
int pgdg_surrogate_gradients(pgdg_mlp* m, const float* X, const float* T, int64_t n, float* grad_host,
                             double* loss) {
  int rc = m->reserve(n);
  if (rc) return rc;
  gradients(m, X, T, n, 0);
  double l = 0;
  if (cudaMemcpy(&l, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return PGDG_ECUDA;
  if (loss) *loss = l / (double)(n * NO);
  if (grad_host && cudaMemcpy(grad_host, m->d_g, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost) != cudaSuccess)
    return PGDG_ECUDA;
  return PGDG_OK;
}
/* one Adam step on a batch (device pointers) */
int pgdg_surrogate_train_step(pgdg_mlp* m, const float* X, const float* T, int64_t n, float lr, double* loss) {
  int rc = m->reserve(n);
  if (rc) return rc;
  gradients(m, X, T, n, 0);
  m->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
  k_adam<<<g_for(NPARAM, 256), 256>>>(m->d_params, m->d_g, m->d_m, m->d_v, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
  if (loss) {
    double l = 0;
    cudaMemcpy(&l, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost);
    *loss = l / (double)(n * NO);
  }
  return cudaGetLastError() == cudaSuccess ? PGDG_OK : PGDG_ECUDA;
}

/* batched MGFM (mpm.cpp:882-926) on device buffers; net == NULL: the reference's
 * plain seed; otherwise the surrogate seed with the plain solve as fallback */
int pgdg_mgfm_batched(const pgdg_mlp* net, const double* in6, const int8_t* mat2, const double* gam,
                      const double* pinf, int nmat, int variant, double* out3, int32_t* iters, int64_t n) {
  if (n < 0 || !in6 || !mat2 || !gam || !pinf || !out3 || nmat < 1) return PGDG_EINVAL;
  if (n == 0) return PGDG_OK;
  /* partition scratch: the network's, or (plain seed) a per-device cache used
   * under a lock; calls run on the default stream */
  if (net) return mgfm_seeded_run((void*)net, in6, mat2, gam, pinf, variant, out3, iters, n, nullptr,
                                  const_cast<pgdg_mlp*>(net)->part, 0, nullptr);
  static PartScratch cache[64];
  static std::mutex mu;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PGDG_ECUDA;
  std::lock_guard<std::mutex> lk(mu);
  return mgfm_seeded_run(nullptr, in6, mat2, gam, pinf, variant, out3, iters, n, nullptr, cache[dev], 0, nullptr);
}

/* Seeds of pgdg_mgfm_batched_noalloc: a file-scope device array, so the call
 * itself never allocates (see the declaration for which callers need that).
 * Its address is looked up once per device. */
static __device__ __align__(256) double g_noalloc_seeds[PGDG_MGFM_NOALLOC_MAX];

int pgdg_mgfm_batched_noalloc(const pgdg_mlp* net, const double* in6, const int8_t* mat2, const double* gam,
                              const double* pinf, int nmat, int variant, double* out3, int32_t* iters, int64_t n) {
  if (n < 0 || !in6 || !mat2 || !gam || !pinf || !out3 || nmat < 1) return PGDG_EINVAL;
  if (n > PGDG_MGFM_NOALLOC_MAX) return PGDG_EOVERFLOW;
  if (net && net->tc) return PGDG_EINVAL; /* its seeds come from the SIMT network only */
  if (n == 0) return PGDG_OK;
  const double* sd = nullptr;
  if (net) {
    constexpr int MAXDEV = 64;
    static double* seeds_of[MAXDEV] = {};
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV) return PGDG_ECUDA;
    double* seeds = nullptr;
    {
      std::lock_guard<std::mutex> lk(mu);
      if (!seeds_of[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_seeds) != cudaSuccess || !p) return PGDG_ECUDA;
        seeds_of[dev] = static_cast<double*>(p);
      }
      seeds = seeds_of[dev];
    }
    seed_launch(const_cast<pgdg_mlp*>(net), in6, mat2, gam, pinf, variant, seeds, n, 0);
    sd = seeds;
  }
  k_mgfm_seeded<<<g_for(n, 256), 256>>>(in6, mat2, gam, pinf, variant, sd, out3, iters, n, nullptr, nullptr, nullptr,
                                        nullptr, nullptr, nullptr, nullptr);
  return cudaGetLastError() == cudaSuccess ? PGDG_OK : PGDG_ECUDA;
}

}  // extern "C"

namespace pgdg {
int PartScratch::reserve(int64_t n) {
  if (n <= cap) return PGDG_OK;
  if (pos) cudaFree(pos);
  if (blk) cudaFree(blk);
  if (perm) cudaFree(perm);
  if (dn) cudaFree(dn);
  pos = blk = dn = nullptr;
  perm = nullptr;
  cap = 0;
  if (cudaMalloc((void**)&pos, sizeof(unsigned long long) * (size_t)(n + 1)) != cudaSuccess ||
      cudaMalloc((void**)&blk, sizeof(unsigned long long) * (size_t)(n / 2048 + 2)) != cudaSuccess ||
      cudaMalloc((void**)&perm, sizeof(int32_t) * (size_t)n) != cudaSuccess ||
      cudaMalloc((void**)&dn, sizeof(unsigned long long)) != cudaSuccess)
    return PGDG_ENOMEM;
  cap = n;
  return PGDG_OK;
}
void PartScratch::release() {
  if (pos) cudaFree(pos);
  if (blk) cudaFree(blk);
  if (perm) cudaFree(perm);
  if (dn) cudaFree(dn);
  pos = blk = dn = nullptr;
  perm = nullptr;
  cap = 0;
}

int mgfm_seeded_reserve(void* netv, PartScratch& ps, int64_t n) {
  int rc = ps.reserve(n);
  if (rc == PGDG_OK && netv) rc = static_cast<pgdg_mlp*>(netv)->reserve_seeds(n);
  return rc;
}

int mgfm_seeded_run(void* netv, const double* in6, const int8_t* mat2, const double* gam, const double* pinf,
                    int variant, double* out3, int32_t* iters, int64_t n, unsigned long long* stats,
                    PartScratch& ps, cudaStream_t st, const unsigned long long* dn) {
  if (n <= 0) return PGDG_OK;
  if (n > INT32_MAX) return PGDG_EINVAL;
  pgdg_mlp* m = static_cast<pgdg_mlp*>(netv);
  int rc = ps.reserve(n);
  if (rc) return rc;
  const double* sd = nullptr;
  if (m) {
    /* split seed path: features and baseline, the network, then Newton with the
     * seed formed per problem (same arithmetic as the fused k_seed) */
    rc = m->reserve_seeds(n);
    if (rc) return rc;
    k_seed_features<<<g_for(n, 256), 256, 0, st>>>(in6, mat2, gam, pinf, variant, m->Xb, m->seeds, m->sc, n, dn);
    forward(m, m->Xb, m->Yb, nullptr, nullptr, nullptr, n, st, dn);
    sd = m->seeds;
  }
  /* problems with a root first: warps of converging problems are not held up
   * by the long floor descent of problems without one (results per problem
   * are unchanged) */
  if (!dn) {
    const unsigned long long nn = (unsigned long long)n;
    cudaMemcpyAsync(ps.dn, &nn, sizeof(nn), cudaMemcpyHostToDevice, st);
  }
  k_root_flag<<<g_for(n, 256), 256, 0, st>>>(in6, mat2, gam, pinf, variant, sd, ps.pos, n, dn);
  scan_u64(ps.pos, ps.blk, dn ? dn : ps.dn, n, st);
  k_root_perm<<<g_for(n, 256), 256, 0, st>>>(ps.pos, ps.blk + (n + 2047) / 2048, ps.perm, n, dn);
  k_mgfm_seeded<<<g_for(n, 256), 256, 0, st>>>(in6, mat2, gam, pinf, variant, sd, out3, iters, n, stats,
                                               m ? m->Yb : nullptr, m ? m->sc : nullptr, m ? m->d_params : nullptr,
                                               ps.perm, m && m->tc ? m->d_tcerr : nullptr, dn);
  return cudaGetLastError() == cudaSuccess ? PGDG_OK : PGDG_ECUDA;
}
}  // namespace pgdg
