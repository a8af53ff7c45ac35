/*
 * k_mgfm.cu -- batched MGFM interface Riemann solve (MPM::MGFM, mpm.cpp:882-926)
 * over independent two-material problems, FP64.  One thread per problem; the
 * Newton iteration is the reference's (two-shock Hugoniot, analytic Jacobian,
 * step capped at 0.6 p*, at most 50 iterations).
 */
#include "../../include/pgdg.h"
#include "pgdg_dev.cuh"

namespace pgdg {

__global__ void k_mgfm_batched(const double* __restrict__ in6, const int8_t* __restrict__ mat2,
                               const double* __restrict__ gam, const double* __restrict__ pinf, int variant,
                               const double* __restrict__ seed, double* __restrict__ out3,
                               int32_t* __restrict__ iters, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* q = in6 + 6 * i;
    int s = mat2[2 * i], s1 = mat2[2 * i + 1];
    double o[3];
    int it = mgfm(q[0], q[1], q[2], q[3], q[4], q[5], gam[s], pinf[s], gam[s1], pinf[s1], variant,
                  seed ? seed[i] : -1.0, o);
    out3[3 * i + 0] = o[0];
    out3[3 * i + 1] = o[1];
    out3[3 * i + 2] = o[2];
    if (iters) iters[i] = it;
  }
}

void mgfm_batched_launch(const double* in6, const int8_t* mat2, const double* gam, const double* pinf, int variant,
                         const double* seed, double* out3, int32_t* iters, int64_t n, cudaStream_t st) {
  int g = grid_for(n, 256);
  k_mgfm_batched<<<g, 256, 0, st>>>(in6, mat2, gam, pinf, variant, seed, out3, iters, n);
}

}  // namespace pgdg

