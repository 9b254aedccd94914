// Diagnostics of evaluation.py on the GPU: per-cell sums over SIPs in
// ascending ID order, bit for bit the reference's loops.  The SIPs are
// binned (histogram, scan, scatter, ID order) into the caller's workspace;
// one thread folds one cell's slots in order.  Compiled with -fmad=false:
// every product is rounded before it is added, as in the reference.
#include <cuda_runtime.h>

#include "lacmo_internal.cuh"
#include "lacmo_physics.cuh"

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

// microphysics.py:208-266: radius (condensation path: cbrt), solute mass
// fraction and density per SIP
__global__ void k_R_p_w_s_rho_p(int sol, int64_t n, const double* __restrict__ m_w,
                                const double* __restrict__ m_s, const double* __restrict__ T_p,
                                double* R_p, double* w_s, double* rho_p) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double m_p = m_w[k] + m_s[k];
    const double w = m_s[k] / m_p;
    const double rho = sol == SOL_AS ? density_water(T_p[k]) * poly_rho_AS(w)
                                     : density_NaCl_solution(w, T_p[k]);
    R_p[k] = radius_from_mass(m_p, rho);
    if (w_s) w_s[k] = w;
    if (rho_p) rho_p[k] = rho;
  }
}
// microphysics.py:83-100 with one density for every mass
__global__ void k_radius_from_mass(int64_t n, const double* __restrict__ m, double rho,
                                   double* R) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    R[k] = radius_from_mass(m[k], rho);
}
// numpy.histogram with weights: bins [e_b, e_b+1), the last one closed;
// values outside [e_0, e_nb] and NaN count nowhere.  The bin comes from a
// binary search of the ascending edges; the weights add up with FP64
// atomics (any order).
__global__ void k_histogram_weighted(const double* __restrict__ x, const double* __restrict__ w,
                                     int64_t n, const double* __restrict__ e, int64_t nb,
                                     double* out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[k];
    if (!(v >= e[0] && v <= e[nb])) continue;
    int64_t lo = 0, hi = nb;   // the last edge <= v, among e[0 .. nb - 1]
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (e[mid] <= v) lo = mid; else hi = mid;
    }
    atomicAdd(out + lo, w ? w[k] : 1.0);
  }
}

static int diag_blocks(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

}  // namespace lacmo

using namespace lacmo;

extern "C" int lacmo_compute_R_p_w_s_rho_p(int solute, int64_t n, const double* m_w,
                                           const double* m_s, const double* T_p, double* R_p,
                                           double* w_s, double* rho_p, void* stream) {
  if ((solute != 0 && solute != 1) || n < 0 || !m_w || !m_s || !T_p || !R_p)
    return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  k_R_p_w_s_rho_p<<<diag_blocks(n), 256, 0, (cudaStream_t)stream>>>(solute, n, m_w, m_s, T_p,
                                                                    R_p, w_s, rho_p);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

extern "C" int lacmo_radius_from_mass(int64_t n, const double* m, double rho, double* R,
                                      void* stream) {
  if (n < 0 || !m || !R) return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  k_radius_from_mass<<<diag_blocks(n), 256, 0, (cudaStream_t)stream>>>(n, m, rho, R);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

extern "C" int lacmo_histogram_weighted(const double* x, const double* w, int64_t n,
                                        const double* edges, int64_t nbins, double* out,
                                        void* stream) {
  if (n < 0 || nbins < 1 || !x || !edges || !out) return LACMO_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(out, 0, (size_t)nbins * sizeof(double), s) != cudaSuccess)
    return LACMO_ERR_CUDA;
  if (n == 0) return LACMO_OK;
  k_histogram_weighted<<<diag_blocks(n), 256, 0, s>>>(x, w, n, edges, nbins, out);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

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
