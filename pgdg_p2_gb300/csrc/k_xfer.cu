/*
 * k_xfer.cu -- layout conversion between the host arrays of the C ABI and the
 * device state, done on the device so the host only moves raw bytes.
 *
 * Host arrays are element-major (pgdg_particles / pgdg_cells: FP64 values and
 * int32 flags, element i's components contiguous); the device state is
 * component-major in the stage type R (field[k * stride + i]) with int8 flags.
 * A chunk of host values is copied as-is into a device staging buffer and one
 * kernel converts it: component k of the device field is host component
 * map.hk[k] of the element, less map.sh[k] (the FP32 path's per-phase energy
 * shift) and less a per-element group shift (a particle's energy by its
 * phase).  Downloads run the same maps backwards, gathering live particle
 * slots through an index list, so the host receives the canonical order.
 */
#include "pgdg_dev.cuh"

namespace pgdg {

namespace {
constexpr int XB = 256;
inline int xgrid(int64_t n) {
  int64_t g = (n + XB - 1) / XB;
  if (g > 152 * 32) g = 152 * 32;
  return g < 1 ? 1 : (int)g;
}

/* the per-group shifts of a transfer (a particle's energy by its phase, one
 * group per material), passed by value */
struct GroupShift {
  double g[F];
  __device__ __forceinline__ double of(int grp1) const {
    const int k = grp1 - 1;
    return (k >= 0 && k < F) ? g[k] : 0.0;
  }
};
inline GroupShift group_shift(const double* gsh) {
  GroupShift s{};
  for (int k = 0; k < F; k++) s.g[k] = gsh ? gsh[k] : 0.0;
  return s;
}

template <typename R>
__global__ void k_h2d(const double* __restrict__ h, int hstride, int64_t i0, int64_t m, XferMap km,
                      R* __restrict__ d, int64_t dstride, const int8_t* __restrict__ grp, GroupShift gsh) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const double gs = grp ? gsh.of(grp[i0 + i]) : 0.0;
    for (int k = 0; k < km.n; k++) {
      double x = h[i * hstride + km.hk[k]];
      if (km.sh[k] != 0.0) x -= km.sh[k];
      if (gs != 0.0) x -= gs;
      d[k * dstride + i0 + i] = (R)x;
    }
  }
}

template <typename R>
__global__ void k_d2h(const R* __restrict__ d, int64_t dstride, const int64_t* __restrict__ idx, int64_t i0,
                      int64_t m, XferMap km, double* __restrict__ h, int hstride, const int8_t* __restrict__ grp,
                      GroupShift gsh) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t src = idx ? idx[i0 + i] : i0 + i;
    const double gs = grp ? gsh.of(grp[src]) : 0.0;
    for (int k = 0; k < km.n; k++) {
      double x = (double)d[k * dstride + src];
      if (km.sh[k] != 0.0) x += km.sh[k];
      if (gs != 0.0) x += gs;
      h[i * hstride + km.hk[k]] = x;
    }
  }
}

__global__ void k_h2d_i8(const int32_t* __restrict__ h, int hstride, int64_t i0, int64_t m, XferMap km,
                         int8_t* __restrict__ d, int64_t dstride) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    for (int k = 0; k < km.n; k++) d[k * dstride + i0 + i] = (int8_t)h[i * hstride + km.hk[k]];
}

__global__ void k_d2h_i8(const int8_t* __restrict__ d, int64_t dstride, const int64_t* __restrict__ idx, int64_t i0,
                         int64_t m, XferMap km, int32_t* __restrict__ h, int hstride) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t src = idx ? idx[i0 + i] : i0 + i;
    for (int k = 0; k < km.n; k++) h[i * hstride + km.hk[k]] = d[k * dstride + src];
  }
}

__global__ void k_gather_u64(const uint64_t* __restrict__ d, const int64_t* __restrict__ idx, int64_t i0, int64_t m,
                             uint64_t* __restrict__ h) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    h[i] = d[idx ? idx[i0 + i] : i0 + i];
}

__global__ void k_iota_u64(uint64_t* d, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (uint64_t)i;
}

template <typename R>
__global__ void k_fill(R* d, int64_t n, R v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) d[i] = v;
}

__global__ void k_alive_flag(const int8_t* __restrict__ phase, unsigned long long* __restrict__ f,
                             const unsigned long long* __restrict__ d_n) {
  const int64_t n = (int64_t)*d_n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    f[i] = phase[i] != 0 ? 1ull : 0ull;
}

__global__ void k_alive_index(const int8_t* __restrict__ phase, const unsigned long long* __restrict__ pos,
                              const unsigned long long* __restrict__ d_n, int64_t* __restrict__ idx) {
  const int64_t n = (int64_t)*d_n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (phase[i] != 0) idx[pos[i]] = i;
}
}  // namespace

XferMap xmap(int n, const int* hk, const double* sh) {
  XferMap m{};
  m.n = n;
  for (int k = 0; k < n && k < XMAP_MAX; k++) {
    m.hk[k] = hk ? hk[k] : k;
    m.sh[k] = sh ? sh[k] : 0.0;
  }
  return m;
}

template <typename R>
cudaError_t xfer_h2d(const double* host, int hstride, int64_t n, const XferMap& km, R* dev, int64_t dstride,
                     const int8_t* grp, const double* gsh, XferStage& sg, cudaStream_t st) {
  const int64_t per = (int64_t)(sg.bytes / (sizeof(double) * (size_t)hstride));
  const GroupShift gs = group_shift(gsh);
  for (int64_t i0 = 0; i0 < n; i0 += per) {
    const int64_t m = n - i0 < per ? n - i0 : per;
    cudaError_t e = cudaMemcpyAsync(sg.buf, host + i0 * hstride, sizeof(double) * (size_t)(m * hstride),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    k_h2d<R><<<xgrid(m), XB, 0, st>>>(static_cast<const double*>(sg.buf), hstride, i0, m, km, dev, dstride, grp, gs);
  }
  return cudaGetLastError();
}

template <typename R>
cudaError_t xfer_d2h(const R* dev, int64_t dstride, const int64_t* idx, int64_t n, const XferMap& km, double* host,
                     int hstride, const int8_t* grp, const double* gsh, XferStage& sg, cudaStream_t st) {
  const int64_t per = (int64_t)(sg.bytes / (sizeof(double) * (size_t)hstride));
  const GroupShift gs = group_shift(gsh);
  for (int64_t i0 = 0; i0 < n; i0 += per) {
    const int64_t m = n - i0 < per ? n - i0 : per;
    cudaError_t e = cudaMemsetAsync(sg.buf, 0, sizeof(double) * (size_t)(m * hstride), st);
    if (e != cudaSuccess) return e;
    k_d2h<R><<<xgrid(m), XB, 0, st>>>(dev, dstride, idx, i0, m, km, static_cast<double*>(sg.buf), hstride, grp, gs);
    e = cudaMemcpyAsync(host + i0 * hstride, sg.buf, sizeof(double) * (size_t)(m * hstride), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t xfer_h2d_i8(const int32_t* host, int hstride, int64_t n, const XferMap& km, int8_t* dev, int64_t dstride,
                        XferStage& sg, cudaStream_t st) {
  const int64_t per = (int64_t)(sg.bytes / (sizeof(int32_t) * (size_t)hstride));
  for (int64_t i0 = 0; i0 < n; i0 += per) {
    const int64_t m = n - i0 < per ? n - i0 : per;
    cudaError_t e = cudaMemcpyAsync(sg.buf, host + i0 * hstride, sizeof(int32_t) * (size_t)(m * hstride),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    k_h2d_i8<<<xgrid(m), XB, 0, st>>>(static_cast<const int32_t*>(sg.buf), hstride, i0, m, km, dev, dstride);
  }
  return cudaGetLastError();
}

cudaError_t xfer_d2h_i8(const int8_t* dev, int64_t dstride, const int64_t* idx, int64_t n, const XferMap& km,
                        int32_t* host, int hstride, XferStage& sg, cudaStream_t st) {
  const int64_t per = (int64_t)(sg.bytes / (sizeof(int32_t) * (size_t)hstride));
  for (int64_t i0 = 0; i0 < n; i0 += per) {
    const int64_t m = n - i0 < per ? n - i0 : per;
    k_d2h_i8<<<xgrid(m), XB, 0, st>>>(dev, dstride, idx, i0, m, km, static_cast<int32_t*>(sg.buf), hstride);
    cudaError_t e = cudaMemcpyAsync(host + i0 * hstride, sg.buf, sizeof(int32_t) * (size_t)(m * hstride),
                                    cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t xfer_d2h_u64(const uint64_t* dev, const int64_t* idx, int64_t n, uint64_t* host, XferStage& sg,
                         cudaStream_t st) {
  const int64_t per = (int64_t)(sg.bytes / sizeof(uint64_t));
  for (int64_t i0 = 0; i0 < n; i0 += per) {
    const int64_t m = n - i0 < per ? n - i0 : per;
    k_gather_u64<<<xgrid(m), XB, 0, st>>>(dev, idx, i0, m, static_cast<uint64_t*>(sg.buf));
    cudaError_t e = cudaMemcpyAsync(host + i0, sg.buf, sizeof(uint64_t) * (size_t)m, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

void iota_u64(uint64_t* d, int64_t n, cudaStream_t st) {
  if (n > 0) k_iota_u64<<<xgrid(n), XB, 0, st>>>(d, n);
}

template <typename R>
void fill_dev(R* d, int64_t n, R v, cudaStream_t st) {
  if (n > 0) k_fill<R><<<xgrid(n), XB, 0, st>>>(d, n, v);
}

/* live slots in canonical order: idx[j] = j-th slot with phase != 0; the
 * count is the scan total (blk[nblk]) */
void alive_index(const int8_t* phase, unsigned long long* scan, unsigned long long* blk,
                 const unsigned long long* d_n, int64_t cap, int64_t* idx, cudaStream_t st) {
  k_alive_flag<<<xgrid(cap), XB, 0, st>>>(phase, scan, d_n);
  scan_u64(scan, blk, d_n, cap, st);
  k_alive_index<<<xgrid(cap), XB, 0, st>>>(phase, scan, d_n, idx);
}

#define PGDG_XFER_INST(R)                                                                                        \
  template cudaError_t xfer_h2d<R>(const double*, int, int64_t, const XferMap&, R*, int64_t, const int8_t*,   \
                                   const double*, XferStage&, cudaStream_t);                                   \
  template cudaError_t xfer_d2h<R>(const R*, int64_t, const int64_t*, int64_t, const XferMap&, double*, int,  \
                                   const int8_t*, const double*, XferStage&, cudaStream_t);                    \
  template void fill_dev<R>(R*, int64_t, R, cudaStream_t);
PGDG_XFER_INST(float)
PGDG_XFER_INST(double)

}  // namespace pgdg
