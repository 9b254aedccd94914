// Diagnostics of evaluation.py on the GPU: per-cell sums over SIPs in
// ascending ID order, bit for bit the reference's loops.  The SIPs are
// binned (histogram, scan, scatter, ID order) into the caller's workspace;
// one thread folds one cell's slots in order.  Compiled with -fmad=false:
// every product is rounded before it is added, as in the reference.
#include <cuda_runtime.h>

#include "lacmo_internal.cuh"

namespace lacmo {

// x^n for an integer n >= 0 by repeated squaring (Numba's integer power)
__device__ __forceinline__ double diag_ipow(double x, int64_t n) {
  double r = 1.0;
  while (n != 0) {
    if (n & 1) r *= x;
    n >>= 1;
    x *= x;
  }
  return r;
}

// kind 0: sum m_w xi, then * (1E-18 * mass_dry_inv)  (evaluation.py:93-133)
// kind 1: sum xi, then * mass_dry_inv                 (evaluation.py:136-174)
// kind 2: sum xi R^order (xi for order 0), then / V0  (evaluation.py:1392-1445)
// Masked SIPs removed at the ground (cell -1 - i) add to cell (i, nz - 1),
// where the reference's index -1 lands; they follow that cell's others.
struct DiagArgs {
  int kind;
  int64_t order;
  const double *a, *b;   // kinds 0/1: m_w, xi; kind 2: R_p, xi
  const uint8_t* mask;   // kinds 0/1 (kind 2: the active SIPs)
  const double* mdi;     // mass_dry_inv [nx][nz]
  double V0;
  const int32_t *cell, *start, *perm;
  int64_t n, nx, nz;
  double* out;
};

__device__ __forceinline__ double diag_term(const DiagArgs& d, int64_t k) {
  if (d.kind == 0) return d.a[k] * d.b[k];
  if (d.kind == 1) return d.b[k];
  return d.order == 0 ? d.b[k] : d.b[k] * diag_ipow(d.a[k], d.order);
}

__global__ void k_diag_fold(const DiagArgs d) {
  const int64_t C = d.nx * d.nz;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int32_t s = d.start[c]; s < d.start[c + 1]; ++s) {
      const int32_t k = d.perm[s];
      if (d.kind != 2 && !d.mask[k]) continue;
      acc += diag_term(d, k);
    }
    d.out[c] = acc;
  }
}

// masked removed SIPs, one warp in ascending ID order (kinds 0/1)
__global__ void k_diag_removed(const DiagArgs d) {
  const int lane = threadIdx.x;
  for (int64_t base = 0; base < d.n; base += 32) {
    const int64_t k = base + lane;
    const bool take = k < d.n && d.cell[k] < 0 && d.mask[k];
    unsigned bal = __ballot_sync(0xffffffffu, take);
    if (lane == 0) {
      while (bal) {
        const int64_t q = base + __ffs(bal) - 1;
        const int64_t i = -1 - (int64_t)d.cell[q];
        d.out[i * d.nz + d.nz - 1] += diag_term(d, q);
        bal &= bal - 1;
      }
    }
    __syncwarp();
  }
}

__global__ void k_diag_scale(const DiagArgs d) {
  const int64_t C = d.nx * d.nz;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x) {
    if (d.kind == 0) d.out[c] *= 1.0E-18 * d.mdi[c];
    else if (d.kind == 1) d.out[c] *= d.mdi[c];
    else d.out[c] = d.out[c] / d.V0;
  }
}

static int diag_run(DiagArgs d, void* ws, size_t bytes, cudaStream_t s) {
  Ws w;
  if (!ws_carve(ws, bytes, d.n, d.nx, d.nz, &w)) return LACMO_ERR_WORKSPACE;
  const int64_t C = d.nx * d.nz;
  if (cudaMemsetAsync(w.counts, 0, 4 * (size_t)C, s) != cudaSuccess ||
      cudaMemsetAsync(w.rm_count, 0, 4, s) != cudaSuccess)
    return LACMO_ERR_CUDA;
  lacmo_sips_t sp = {};
  sp.n = d.n; sp.cell = (int32_t*)d.cell;
  lacmo_grid_t g = {};
  g.nx = d.nx; g.nz = d.nz;
  const Bt B = single(sp, g, w, 0);
  if (launch_histogram(B, s) != cudaSuccess || launch_bin(B, s) != cudaSuccess)
    return LACMO_ERR_CUDA;
  d.start = w.start; d.perm = w.perm;
  const int threads = 128;
  const int blocks = (int)((C + threads - 1) / threads);
  k_diag_fold<<<blocks, threads, 0, s>>>(d); note_launches(1);
  if (d.kind != 2) { k_diag_removed<<<1, 32, 0, s>>>(d); note_launches(1); }
  k_diag_scale<<<blocks, threads, 0, s>>>(d); note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

}  // namespace lacmo

using namespace lacmo;

extern "C" int lacmo_update_cell_sum(int kind, const double* m_w, const double* xi,
                                     const int32_t* cell, const uint8_t* mask,
                                     const double* mass_dry_inv, int64_t n, int64_t nx,
                                     int64_t nz, double* out, void* ws, size_t bytes,
                                     void* stream) {
  if ((kind != 0 && kind != 1) || n <= 0 || n >= 0x7fffffff || nx <= 0 || nz <= 0 || !xi ||
      !cell || !mask || !mass_dry_inv || !out || (kind == 0 && !m_w))
    return LACMO_ERR_ARG;
  DiagArgs d = {};
  d.kind = kind; d.a = m_w; d.b = xi; d.mask = mask; d.mdi = mass_dry_inv;
  d.cell = cell; d.n = n; d.nx = nx; d.nz = nz; d.out = out;
  return diag_run(d, ws, bytes, (cudaStream_t)stream);
}

extern "C" int lacmo_compute_moment_R_grid(int64_t order, const double* R_p, const double* xi,
                                           double V0, const int32_t* cell, int64_t n,
                                           int64_t nx, int64_t nz, double* out, void* ws,
                                           size_t bytes, void* stream) {
  if (order < 0 || n <= 0 || n >= 0x7fffffff || nx <= 0 || nz <= 0 || !R_p || !xi || !cell ||
      !out)
    return LACMO_ERR_ARG;
  DiagArgs d = {};
  d.kind = 2; d.order = order; d.a = R_p; d.b = xi; d.V0 = V0;
  d.cell = cell; d.n = n; d.nx = nx; d.nz = nz; d.out = out;
  return diag_run(d, ws, bytes, (cudaStream_t)stream);
}
