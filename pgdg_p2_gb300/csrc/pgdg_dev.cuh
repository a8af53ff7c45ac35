/*
 * pgdg_dev.cuh -- device state of one context and the launch interface between
 * the host driver (capi.cu) and the kernel translation units.
 *
 * Layout in HBM (structure of arrays, component-major so that a warp reading
 * one field of consecutive particles or cells is coalesced):
 *   particles  field[t * cap + slot]   slots in canonical (particle_fluid) order;
 *              new particles are appended, removed ones become tombstones
 *              (phase 0) until compaction
 *   cells      field[t * ncell + ci]   ci = (i * NY + j) * NZ + k
 *   buckets    bucket[ci * maxpc + r]  the Cell_list of every cell (fluid slots
 *              in list order) with count bcnt[ci]
 */
#ifndef PGDG_DEV_CUH
#define PGDG_DEV_CUH

#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/pgdg_types.h"
#include "pgdg_math.cuh"

/* FldNum (glbparam.h:41): the number of materials is a compile-time constant,
 * as in the reference, which builds one binary per material count.  The
 * default build holds two materials (every 2D and 3D workload); a build with
 * -DPGDG_NFLD=3 holds the 2D three-material instance (Triple_point_3phase). */
#ifndef PGDG_NFLD
#define PGDG_NFLD 2
#endif
#if PGDG_NFLD == 2
#define PGDG_WITH_3D 1
#else
#define PGDG_WITH_3D 0
#endif

namespace pgdg {

constexpr int F = PGDG_NFLD;
/* list-order keys (Cell_list order): base entries are ordered by slot,
 * appended entries (Add_particle during split/merge) by an append counter */
constexpr uint32_t KEY_APPEND = 0x80000000u;

/* error bits */
enum : uint32_t {
  ERR_BUCKET = 1u << 0,    /* a cell bucket overflowed */
  ERR_ARENA = 1u << 1,     /* neighbour-list arena overflowed */
  ERR_CAPACITY = 1u << 2,  /* particle slot capacity exceeded */
  ERR_NOLIST = 1u << 3,    /* split/merge needed a list the device did not keep */
  ERR_CELLQ = 1u << 4,     /* flagged-cell queue overflowed */
  ERR_QUEUE = 1u << 5,     /* interface queue overflowed */
  ERR_DT = 1u << 6,        /* no finite CFL time step */
};

struct DevCounters {
  unsigned long long n_slots;     /* slots in use (live + tombstones) */
  unsigned long long n_live;
  unsigned long long seq_next;
  unsigned long long append_next; /* Add_particle counter within a step */
  unsigned long long arena_used;
  unsigned long long n_dirty, n_flagged;
  unsigned long long n_split, n_inlet, n_outlet, n_merge, n_affected;
  unsigned long long step_split, step_new, step_surv;
  unsigned long long mgfm_calls, mgfm_iters, mgfm_maxit, g2p_fb;
  unsigned long long dt_bits, maxv_bits; /* atomic min/max scratch */
  unsigned long long queue_n;
  unsigned long long merge_n;     /* slots the current merge pass sweeps */
  unsigned long long merge_quiet; /* the last merge pass merged nothing */
  unsigned long long split_events; /* particles with a split, inlet or outlet event */
  unsigned long long split_n;      /* slots the split's event sweeps cover */
  unsigned int err;
  unsigned int pad;
  double dt, max_v;
  double time;                    /* simulated time: sum of the steps' dt */
};

/* case constants handed to kernels by value */
struct CaseK {
  int dim;
  int N[3];
  int bc[6];
  int mgfm_variant;
  int rad2;          /* flag-2 scan radius in cells (level_infor.cpp:155) */
  int maxpc;
  int64_t ncell;
  int64_t cap;
  int64_t nbnd;
  int64_t arena_cap;
  double bl[3], br[3], ps[3];
  double p_g, p_sz;
  double gamma[F], pinf[F], ini_rho[F];
  /* energy shift of the FP32 path: stored E = E_true - eshift[s] with
   * eshift = gamma p_inf / (gamma - 1), so the EOS reads p = (gamma-1)(E - rho v^2/2)
   * without the cancellation against gamma p_inf (pinf_eos = 0); both are 0 and
   * pinf on the FP64 paths, which store E unshifted */
  double eshift[F], pinf_eos[F];
  double inlet_rho, inlet_u[3], inlet_p;
  double cfl;
  double vol_max, vol_min, dss0;
  double probe[8][3];
  double bvol, brho;
};

/* device pointers; R is the storage/arithmetic type of the stage fields */
template <typename R>
struct DevPtrs {
  /* particles */
  R* X[3];          /* rotating coordinate buffers, each D*cap */
  R* H[2];          /* ping-pong smoothing length */
  R *vol, *vol0, *mass, *rho, *E, *c, *P;
  R *rhov, *v, *tv; /* D*cap */
  R* sl;            /* U*D*cap: coef[0] columns 1..D */
  R* rec;           /* 4*cap: per-particle record of the shifting sum, written
                     * by G2P: new x[3] and the volume signed by the phase */
  R* rec2;          /* 2*cap: density and sound speed of the same particle */
  int8_t* phase;    /* 0 = tombstone */
  int8_t* mark_in;
  uint64_t* seq;
  int32_t* lcell;   /* Cell_list the slot is in (-1 none) */
  uint32_t* lkey;   /* order inside that list */
  int32_t* list_len;/* stored neighbour list (-1: not kept) */
  int64_t* list_off;
  int32_t* target;  /* merge partner (copy_p[0]) */
  uint8_t* aff;     /* affected (needs a fresh flag-3 list) */
  uint8_t* mflag;   /* merge role: 1 survivor, 2 removed */
  int8_t* evcode;   /* split event code */
  unsigned long long* scan;  /* cap+1 prefix buffer */
  unsigned long long* scan_blk;
  int32_t* arena;
  /* boundary particles */
  R *bx, *bn;       /* D*nbnd */
  int32_t *boff, *bent;  /* per-cell CSR of boundary particles */
  /* cells */
  R *crho, *crhov, *cE, *cc, *cac, *calph;  /* F, F*D, F, F, F, F */
  R *ccoef, *ccoef0, *cdcoef;                /* F*U*B */
  R *clim;                                   /* F*U */
  R *cgv;                                    /* D*D */
  R *cv;                                     /* D */
  R* cP;
  int8_t *cph, *cphb, *cused;                /* F, F, 1 */
  int8_t* cnew;                              /* P2G: mask of newly present phases */
  int32_t *bucket, *bcnt;
  uint32_t* cflag;  /* bit0 dirty bucket, bit1 flagged (affected neighbourhood) */
  int32_t *dirty_q, *flag_q;
  int64_t qcap;     /* capacity of dirty_q / flag_q */
  DevCounters* cnt;
  int xb;           /* index of the current coordinate buffer */
  int hb;           /* index of the current h buffer */
};

/* queue of interface Riemann problems of one stage (mixed path with the seed
 * surrogate): off = exclusive per-cell offsets (ncell + 1) */
struct IfaceQ {
  double* in6;
  int8_t* mat;
  double* out3;
  unsigned long long* off;
  unsigned long long* blk;
  const unsigned long long* d_ncell;
  /* [0] the stage's interface problems, [1] those the batch solves: [0], or 0
   * when [0] exceeds cap (the residual then solves the stage inline) */
  unsigned long long* tot;
  int64_t cap;
};

/* ---------------- cell ids ---------------- */
template <int D>
__device__ __forceinline__ int64_t cidx(const CaseK& K, const int* pos) {
  return ((int64_t)pos[0] * K.N[1] + (D > 1 ? pos[1] : 0)) * K.N[2] + (D > 2 ? pos[2] : 0);
}

/* get_cell_id (glbfunc.h:161-173) in FP64 */
template <int D>
__device__ void cell_pos_exact(const CaseK& K, const double* x, int* pos) {
  pos[0] = pos[1] = pos[2] = 0;
  for (int d = 0; d < D; d++) {
    double q = floor(ddiv(dsub(x[d], K.bl[d]), K.ps[d]));
    int ip;
    if (!(q >= 0)) ip = 0;
    else if (q >= K.N[d] - 1) ip = K.N[d] - 1;
    else ip = (int)q;
    pos[d] = ip;
  }
}

/* the same cell id from stored coordinates; in FP32 storage a float quotient
 * decides unless it lies within a relative 1e-6 of an integer */
template <int D, typename R>
__device__ void cell_pos(const CaseK& K, const R* xr, int* pos) {
  if (sizeof(R) == 4) {
    bool ok = true;
    pos[0] = pos[1] = pos[2] = 0;
    for (int d = 0; d < D; d++) {
      float qf = ((float)xr[d] - (float)K.bl[d]) / (float)K.ps[d];
      float fl = floorf(qf);
      float fr = qf - fl;
      float m = 1e-6f * (fabsf(qf) + 16.f);
      if (!(fr >= m && fr <= 1.f - m)) ok = false;
      int ip;
      if (!(fl >= 0.f)) ip = 0;
      else if (fl >= (float)(K.N[d] - 1)) ip = K.N[d] - 1;
      else ip = (int)fl;
      pos[d] = ip;
    }
    if (ok) return;
  }
  double xd[3] = {0, 0, 0};
  for (int d = 0; d < D; d++) xd[d] = (double)xr[d];
  cell_pos_exact<D>(K, xd, pos);
}

/* ---------------- host-side launch interface ---------------- */
/* EX = true: exact-order FP64 build (no FMA contraction), bit-identical to the oracle */
template <int D, typename R, bool EX>
struct Launch {
  /* k_particles.cu */
  static void bin(const CaseK&, const DevPtrs<R>&, cudaStream_t);
  static void split(const CaseK&, const DevPtrs<R>&, cudaStream_t);
  /* chained: the pass follows another of the same sequence (it is skipped
   * on the device when that one merged nothing) */
  static void merge(const CaseK&, const DevPtrs<R>&, bool chained, cudaStream_t);
  static void store_lists(const CaseK&, const DevPtrs<R>&, int xs, int hs, int xn, cudaStream_t);
  static void reset_lists(const CaseK&, const DevPtrs<R>&, cudaStream_t);
  /* k_grid.cu */
  static void used_state(const CaseK&, const DevPtrs<R>&, cudaStream_t);
  static void set_timestep(const CaseK&, const DevPtrs<R>&, int by_cells, cudaStream_t);
  static void add_time(const DevPtrs<R>&, cudaStream_t);
  /* fresh_bins: every particle lies in its bucket's cell (right after
   * binning), so neighbour cells beyond the cut radius can be skipped */
  static void p2g(const CaseK&, const DevPtrs<R>&, bool fresh_bins, cudaStream_t);
  static void p2g_new(const CaseK&, const DevPtrs<R>&, cudaStream_t);
  static void limiter(const CaseK&, const DevPtrs<R>&, cudaStream_t);
  static void grid_acc(const CaseK&, const DevPtrs<R>&, cudaStream_t);
  /* queued variant: returns the number of interface problems (negative: over capacity) */
  static void iface_gather(const CaseK&, const DevPtrs<R>&, IfaceQ, cudaStream_t);
  static void grid_acc_queued(const CaseK&, const DevPtrs<R>&, IfaceQ, cudaStream_t);
  static void update_grid(const CaseK&, const DevPtrs<R>&, int md, cudaStream_t);
  /* 2F + 2 totals into d_out: particle mass per phase, particle energy, cell
   * mass per phase, cell energy */
  static void totals(const CaseK&, const DevPtrs<R>&, double* d_out, cudaStream_t);
  static size_t totals_scratch(); /* doubles d_out must hold */
  /* bubble probe (downstream end, jet, upstream end, phase-2 mass, fluid
   * count) into d_out5, with the totals scratch for its partials */
  static void probe(const CaseK&, const DevPtrs<R>&, double* d_scratch, double* d_out5, cudaStream_t);
  /* k_g2p.cu */
  /* xs/hs: stage-start coordinate/h buffers, x0: step-start coordinates (md 1),
   * xn/hn: buffers receiving the new coordinates/h */
  /* full = false: skip the slopes, energy, pressure, momentum and mass, which
   * nothing reads before the next G2P of the same step rewrites them */
  static void g2p(const CaseK&, const DevPtrs<R>&, int md, int xs, int x0, int xn, int hn, bool full,
                  cudaStream_t);
  /* shifting: scratch holds pst_scratch_bytes(K) bytes of device memory */
  static void pst(const CaseK&, const DevPtrs<R>&, int xs, int hs, int xn, int hn, int var, void* scratch,
                  cudaStream_t);
  static size_t pst_scratch_bytes(const CaseK&);
  /* per-stage row sort the shifting kernel of the same stage reads (mixed and
   * FMA paths; no launch on the exact path) */
  static void rowsort(const CaseK&, const DevPtrs<R>&, int xs, void* scratch, cudaStream_t);
  static int pst_variants();
};

/* ---------------- host <-> device layout conversion (k_xfer.cu) ---------------- */
constexpr int XMAP_MAX = 48;
/* device component k <- host component hk[k] (minus sh[k] on upload, plus on download) */
struct XferMap {
  int n;
  int hk[XMAP_MAX];
  double sh[XMAP_MAX];
};
XferMap xmap(int n, const int* hk = nullptr, const double* sh = nullptr);
/* device staging buffer for raw host chunks */
struct XferStage {
  void* buf;
  size_t bytes;
};
template <typename R>
cudaError_t xfer_h2d(const double* host, int hstride, int64_t n, const XferMap& km, R* dev, int64_t dstride,
                     const int8_t* grp, const double* gsh, XferStage& sg, cudaStream_t st);
template <typename R>
cudaError_t xfer_d2h(const R* dev, int64_t dstride, const int64_t* idx, int64_t n, const XferMap& km, double* host,
                     int hstride, const int8_t* grp, const double* gsh, XferStage& sg, cudaStream_t st);
cudaError_t xfer_h2d_i8(const int32_t* host, int hstride, int64_t n, const XferMap& km, int8_t* dev, int64_t dstride,
                        XferStage& sg, cudaStream_t st);
cudaError_t xfer_d2h_i8(const int8_t* dev, int64_t dstride, const int64_t* idx, int64_t n, const XferMap& km,
                        int32_t* host, int hstride, XferStage& sg, cudaStream_t st);
cudaError_t xfer_d2h_u64(const uint64_t* dev, const int64_t* idx, int64_t n, uint64_t* host, XferStage& sg,
                         cudaStream_t st);
void iota_u64(uint64_t* d, int64_t n, cudaStream_t st);
template <typename R>
void fill_dev(R* d, int64_t n, R v, cudaStream_t st);
void alive_index(const int8_t* phase, unsigned long long* scan, unsigned long long* blk,
                 const unsigned long long* d_n, int64_t cap, int64_t* idx, cudaStream_t st);

/* forward pass of the seed surrogate on the tensor cores (k_mlp_tc.cu); with
 * dn, a batch launched for n entries whose live count *dn (<= n) is known on
 * the device only */
int mlp_tc_forward(const float* params, const float* X, float* Y, int64_t n, int* err, cudaStream_t st,
                   const unsigned long long* dn = nullptr);

/* scratch of the root partition of a batch (prefix, block sums, order, count) */
struct PartScratch {
  unsigned long long *pos = nullptr, *blk = nullptr, *dn = nullptr;
  int32_t* perm = nullptr;
  int64_t cap = 0;
  int reserve(int64_t n);
  void release();
};
/* seeded batched MGFM over device buffers (k_mlp.cu); stats += (calls,
 * iterations, cap hits).  Launches are sized for n; with dn the batch's live
 * count is *dn (clamped to n), read on the device, so the call reads nothing
 * back on the host and can be captured in a graph once its scratch holds n */
int mgfm_seeded_run(void* net, const double* in6, const int8_t* mat2, const double* gam, const double* pinf,
                    int variant, double* out3, int32_t* iters, int64_t n, unsigned long long* stats,
                    PartScratch& ps, cudaStream_t st, const unsigned long long* dn);
/* allocate the scratch a batch of n needs (partition and, with a network, seeds
 * and features) ahead of a capture, so the captured call allocates nothing */
int mgfm_seeded_reserve(void* net, PartScratch& ps, int64_t n);

/* the synthetic workload id built in place on the device (k_case.cu): n
 * lattice particles and every cell, as the host builder makes them */
template <int D, typename R>
int case_build(const CaseK& K, const DevPtrs<R>& P, const pgdg_case& cs, int id, uint64_t seed, int64_t n,
               cudaStream_t st);

/* snapshot packing of Output_plt_file (k_output.cu): the n live particles of
 * alive[] into dv (10 x n doubles: x y z vx vy vol rho P |tv| |v|) and iv
 * (2 x n int32: phase, flag-2 list size over coordinates X[xs] and lengths
 * H[hs]); the cells into dc (12 doubles per cell) */
template <int D, typename R, bool EX>
void output_pack_particles(const CaseK& K, const DevPtrs<R>& P, const int64_t* alive, int64_t n, int xs, int hs,
                           double* dv, int32_t* iv, cudaStream_t st);
template <int D, typename R, bool EX>
void output_pack_cells(const CaseK& K, const DevPtrs<R>& P, double* dc, cudaStream_t st);

/* minimum resident 128-thread blocks per SM asked of the FP32 instantiations of
 * the per-cell and per-particle kernels (a register cap that trades a few
 * registers for more warps in flight; these kernels are latency-bound); the
 * FP64 instantiations keep the compiler's own register count */
template <typename R>
__host__ __device__ constexpr int minblocks_f32(int n) {
  return sizeof(R) == 4 ? n : 1;
}

/* shared helpers used by several translation units */
int grid_for(int64_t n, int block);
void scan_u64(unsigned long long* data, unsigned long long* blk, const unsigned long long* d_n, int64_t cap,
              cudaStream_t st);

}  // namespace pgdg
#endif
