// Particle, grid and cell-binning kernels of the SIP hot path (FP64).
//
// k_particles fuses one whole particle sub-step of the reference
// (integration.py:944-1091): T_p from the cell, radius / mass fraction /
// density, the implicit Newton condensation (integration.py:728-940), the
// implicit drag update with the staggered bilinear wind interpolation
// (integration.py:632-719, grid.py:257-323), the Euler position update with
// periodic x, capped z and ground removal (integration.py:552-630) and the
// cell re-index (integration.py:509-550).  It reads each SIP attribute once
// and writes it once; grid data come from small L2-resident arrays.
//
// Order-dependent sums the reference accumulates in ascending SIP ID (the
// per-cell condensed mass delta_m_l, integration.py:916-936, and
// water_removed, integration.py:620-628) are formed here in the same order:
// k_cell_update folds each cell's dm*xi over the cell's SIPs sorted by ID, and
// the removal list is sorted by ID before it is folded.  Results are therefore
// deterministic and, given identical per-SIP values, equal to the reference's.
#include <cuda_runtime.h>

#include <atomic>

#include "lacmo_internal.cuh"
#include "lacmo_physics.cuh"

namespace lacmo {

static inline int nblocks(int64_t n, int t, int cap = 152 * 32) {
  int64_t b = (n + t - 1) / t;
  if (b < 1) b = 1;
  return (int)(b < cap ? b : cap);
}

// ---------------------------------------------------------------------------
__global__ void k_cells_import(const int64_t* __restrict__ cells, const uint8_t* __restrict__ act,
                               int32_t* __restrict__ cell, int64_t n, int64_t nz) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = cells[k], j = cells[n + k];
    cell[k] = act[k] ? (int32_t)(i * nz + j) : (int32_t)(-1 - i);
  }
}

__global__ void k_cells_export(const int32_t* __restrict__ cell, const double* __restrict__ pos,
                               double* __restrict__ rel, int64_t* __restrict__ cells,
                               uint8_t* __restrict__ act, int64_t n, int64_t nz, double x_min,
                               double z_min, double dx, double dz) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = cell[k];
    if (c >= 0) {
      int64_t i = c / nz, j = c - (c / nz) * nz;
      cells[k] = i; cells[n + k] = j; act[k] = 1;
      rel[k] = (pos[k] - x_min) / dx - (double)i;
      rel[n + k] = (pos[n + k] - z_min) / dz - (double)j;
    } else {
      cells[k] = -1 - (int64_t)c; cells[n + k] = -1; act[k] = 0;
    }
  }
}

// per-cell terms of the mass rate for the next sub-step; their FP32 copies in
// the cell records (cell_records) feed the mixed-precision kernel without
// double->float conversions there
__device__ __forceinline__ void write_aux(const double* gsf, const double* gmp, double* aux,
                                          int64_t c, int64_t C) {
  CellAmb a = make_cell_amb(gsf[c], gsf[C + c], gsf[6 * C + c], gsf[7 * C + c], gmp[2 * C + c],
                            gmp[c], gmp[C + c]);
  aux[c] = a.sigw; aux[C + c] = a.rhow; aux[2 * C + c] = a.lap0; aux[3 * C + c] = a.lbp0;
  aux[4 * C + c] = a.c1; aux[5 * C + c] = a.c2;
  float4* af = cell_records(aux, C) + CELL_REC * c;
  af[0] = make_float4((float)a.T, (float)(a.S - 1.0), (float)a.sigw, (float)a.rhow);
  af[1] = make_float4((float)a.lap0, (float)a.lbp0, (float)a.c1, (float)a.c2);
  af[2] = make_float4((float)gmp[5 * C + c], (float)gmp[6 * C + c], 0.0f, 0.0f);
}

__global__ void k_cell_aux(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  const int64_t C = mb.g.nx * mb.g.nz;
  const double *gsf = mb.g.scalar_fields, *gmp = mb.g.mat_prop;
  double* aux = mb.w.aux;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x)
    write_aux(gsf, gmp, aux, c, C);
}

// ---------------------------------------------------------------------------
// binning: histogram (arrival rank) -> scan -> scatter -> order by ID
__global__ void k_histogram(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  const int32_t* __restrict__ cell = mb.sp.cell;
  const int64_t n = mb.sp.n;
  int32_t *counts = mb.w.counts, *rank = mb.w.rank;
  const int64_t C = mb.g.nx * mb.g.nz;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = cell[k];
    if (c < 0) continue;
    if (c < C) rank[k] = atomicAdd(counts + c, 1);
    else atomicOr(mb.w.flags, LACMO_FLAG_CELL_RANGE);   // left out of the binning
  }
}

// Single block: folds the sorted ground-removal list into water_removed, then
// the exclusive scans of the SIP counts (slots) and pair counts (draws).
__global__ void __launch_bounds__(1024) k_scan(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  int32_t *counts = mb.w.counts, *start = mb.w.start, *rm_count = mb.w.rm_count,
          *rm_id = mb.w.rm_id;
  int64_t *draw_off = mb.w.draw_off, *total_pairs = mb.w.total_pairs;
  double *rm_val = mb.w.rm_val, *water_removed = mb.sp.water_removed;
  const int64_t C = mb.g.nx * mb.g.nz;
  __shared__ int64_t s_slot[1024];
  __shared__ int64_t s_pair[1024];
  __shared__ int32_t s_id[2048];
  __shared__ double s_val[2048];
  const int t = threadIdx.x;
  // ---- ground removals, ascending ID (integration.py:620-628) ----
  int nrm = *rm_count;
  if (nrm > 0 && nrm <= 2048) {
    int P = 1;
    while (P < nrm) P <<= 1;
    for (int q = t; q < P; q += blockDim.x) {
      s_id[q] = q < nrm ? rm_id[q] : 0x7fffffff;
      s_val[q] = q < nrm ? rm_val[q] : 0.0;
    }
    __syncthreads();
    for (int kk = 2; kk <= P; kk <<= 1) {
      for (int jj = kk >> 1; jj > 0; jj >>= 1) {
        for (int q = t; q < P; q += blockDim.x) {
          int p2 = q ^ jj;
          if (p2 > q) {
            bool up = ((q & kk) == 0);
            int a = s_id[q], b = s_id[p2];
            if ((a > b) == up) {
              s_id[q] = b; s_id[p2] = a;
              double v = s_val[q]; s_val[q] = s_val[p2]; s_val[p2] = v;
            }
          }
        }
        __syncthreads();
      }
    }
    if (t == 0) {
      double wr = water_removed[0];
      for (int q = 0; q < nrm; ++q) wr += s_val[q];
      water_removed[0] = wr;
    }
    __syncthreads();
  } else if (nrm > 2048) {
    // rare: repeated extraction of the smallest remaining ID
    if (t == 0) {
      double wr = water_removed[0];
      int32_t last = -1;
      for (int r = 0; r < nrm; ++r) {
        int32_t best = 0x7fffffff; int bq = -1;
        for (int q = 0; q < nrm; ++q)
          if (rm_id[q] > last && rm_id[q] < best) { best = rm_id[q]; bq = q; }
        wr += rm_val[bq];
        last = best;
      }
      water_removed[0] = wr;
    }
    __syncthreads();
  }
  if (t == 0) *rm_count = 0;
  // ---- scans ----
  int64_t chunk = (C + blockDim.x - 1) / blockDim.x;
  int64_t b0 = t * chunk, b1 = b0 + chunk < C ? b0 + chunk : C;
  int64_t ss = 0, sp = 0;
  for (int64_t c = b0; c < b1; ++c) {
    int64_t m = counts[c];
    ss += m; sp += m * (m - 1) / 2;
  }
  s_slot[t] = ss; s_pair[t] = sp;
  __syncthreads();
  for (int off = 1; off < (int)blockDim.x; off <<= 1) {
    int64_t a = t >= off ? s_slot[t - off] : 0, b = t >= off ? s_pair[t - off] : 0;
    __syncthreads();
    s_slot[t] += a; s_pair[t] += b;
    __syncthreads();
  }
  int64_t os = s_slot[t] - ss, op = s_pair[t] - sp;
  for (int64_t c = b0; c < b1; ++c) {
    int64_t m = counts[c];
    start[c] = (int32_t)os; draw_off[c] = op;
    os += m; op += m * (m - 1) / 2;
    counts[c] = 0;
  }
  if (t == blockDim.x - 1) { start[C] = (int32_t)os; draw_off[C] = op; *total_pairs = op; }
  // ---- collision work order: cells by descending SIP count (a counting
  // sort on min(count, 1023); the order inside a size class is arbitrary) ----
  __shared__ int32_t s_hist[1024];
  int32_t* order = mb.w.cell_order;
  s_hist[t] = 0;
  __syncthreads();
  for (int64_t c = b0; c < b1; ++c) {
    const int32_t m = start[c + 1] - start[c];
    atomicAdd(&s_hist[1023 - (m < 1023 ? m : 1023)], 1);
  }
  __syncthreads();
  const int32_t hv = s_hist[t];
  s_slot[t] = hv;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int64_t add = t >= off ? s_slot[t - off] : 0;
    __syncthreads();
    s_slot[t] += add;
    __syncthreads();
  }
  s_hist[t] = (int32_t)(s_slot[t] - hv);
  __syncthreads();
  for (int64_t c = b0; c < b1; ++c) {
    const int32_t m = start[c + 1] - start[c];
    order[atomicAdd(&s_hist[1023 - (m < 1023 ? m : 1023)], 1)] = (int32_t)c;
  }
}

__global__ void k_scatter(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  const int32_t* __restrict__ cell = mb.sp.cell;
  const int32_t* __restrict__ rank = mb.w.rank;
  const int32_t* __restrict__ start = mb.w.start;
  int32_t* perm = mb.w.perm;
  const int64_t n = mb.sp.n, C = mb.g.nx * mb.g.nz;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = cell[k];
    if (c >= 0 && c < C) perm[start[c] + rank[k]] = (int32_t)k;
  }
}

// Bitonic sort of 32 * PER keys held by a warp, key[u] = element lane * PER + u,
// ascending: compare-exchange stages of distance j >= PER between lanes
// (shuffles), of smaller distance within a lane's registers.
template <int PER>
__device__ __forceinline__ void warp_bitonic(int32_t (&key)[PER], int lane) {
  constexpr int N = 32 * PER;
#pragma unroll
  for (int k = 2; k <= N; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= PER) {
#pragma unroll
        for (int u = 0; u < PER; ++u) {
          const int e = lane * PER + u;
          const int32_t other = __shfl_xor_sync(0xffffffffu, key[u], j / PER);
          const bool take_min = ((e & k) == 0) == ((e & j) == 0);
          key[u] = take_min ? min(key[u], other) : max(key[u], other);
        }
      } else {
#pragma unroll
        for (int u = 0; u < PER; ++u) {
          if (u & j) continue;
          const bool up = ((lane * PER + u) & k) == 0;
          const int32_t x = key[u], y = key[u ^ j];
          key[u] = up ? min(x, y) : max(x, y);
          key[u ^ j] = up ? max(x, y) : min(x, y);
        }
      }
    }
  }
}
// the L <= 32 * PER slots of one cell sorted by SIP ID in the warp's registers
template <int PER>
__device__ __forceinline__ void sort_cell_ids(int32_t* perm, int32_t b, int L, int lane) {
  int32_t key[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int e = lane * PER + u;
    key[u] = e < L ? perm[b + e] : 0x7fffffff;
  }
  warp_bitonic<PER>(key, lane);
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int e = lane * PER + u;
    if (e < L) perm[b + e] = key[u];
  }
}

// Number of keys of the sorted run a[0..len) that are below x (IDs are
// unique, so keys of the other run never tie with x).
__device__ __forceinline__ int32_t count_below(const int32_t* a, int32_t len, int32_t x) {
  int32_t lo = 0, hi = len;
  while (lo < hi) {
    const int32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// one warp per cell: order the cell's slots by ascending SIP ID.  Up to 256
// slots: a bitonic sort in registers.  Larger cells: runs of 256 sorted in
// registers, then merged pairwise, each key placed at its rank in the merged
// run (its index in its own run plus a binary search in the other), ping-pong
// between perm and the rank array (free after the scatter); O(L log L).
constexpr int ORDER_SMEM = 256;
__global__ void __launch_bounds__(256) k_order(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  const int32_t* __restrict__ start = mb.w.start;
  int32_t *perm = mb.w.perm, *scratch = mb.w.rank;
  const int64_t C = mb.g.nx * mb.g.nz;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t c = blockIdx.x * 8LL + wid; c < C; c += (int64_t)gridDim.x * 8) {
    const int32_t b = start[c], L = start[c + 1] - b;
    if (L <= 1) continue;
    if (L <= ORDER_SMEM) {
      if (L <= 64) sort_cell_ids<2>(perm, b, L, lane);
      else if (L <= 128) sort_cell_ids<4>(perm, b, L, lane);
      else sort_cell_ids<8>(perm, b, L, lane);
      __syncwarp();
      continue;
    }
    for (int32_t r0 = 0; r0 < L; r0 += ORDER_SMEM) {
      const int32_t len = L - r0 < ORDER_SMEM ? L - r0 : ORDER_SMEM;
      sort_cell_ids<8>(perm, b + r0, len, lane);
    }
    __syncwarp();
    int32_t* src = perm + b;
    int32_t* dst = scratch + b;
    for (int32_t width = ORDER_SMEM; width < L; width <<= 1) {
      for (int32_t lo = 0; lo < L; lo += 2 * width) {
        const int32_t mid = lo + width < L ? lo + width : L;
        const int32_t hi = lo + 2 * width < L ? lo + 2 * width : L;
        const int32_t *A = src + lo, *Bv = src + mid;
        const int32_t la = mid - lo, lb = hi - mid;
        for (int32_t q = lane; q < la; q += 32) dst[lo + q + count_below(Bv, lb, A[q])] = A[q];
        for (int32_t q = lane; q < lb; q += 32) dst[lo + q + count_below(A, la, Bv[q])] = Bv[q];
      }
      __syncwarp();
      int32_t* t = src; src = dst; dst = t;
    }
    if (src != perm + b)
      for (int32_t q = lane; q < L; q += 32) perm[b + q] = src[q];
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
struct PArgs {
  double *pos, *vel, *m_w, *rel, *T_p;
  const double *m_s, *xi;
  int32_t* cell;
  const double *gsf, *gmp, *aux, *gv;
  int64_t n, nx, nz;
  double x_min, x_max, z_min, z_cap, dx, dz;
  double dt_sub, dt_pos, g_set;
  int no_iter, sol, write_Tp;
  double* dmxi;
  int32_t *counts, *rank, *rm_count, *rm_id;
  double* rm_val;
  // mixed precision: SIPs whose Newton repeats in FP64 (k_newton_fallback),
  // queued in scratch that mixed sub-steps leave unused
  int32_t *fb_count, *fb_done, *fb_id, *fb_c;
  double* fb_mw;
  uint32_t* flags;
  // mixed precision
  double* acc;                  // [C] per-cell sums of dm * xi, int64 units of 2^-4 fg
  int hist;                     // count SIPs per new cell for a following binning
  unsigned long long* nfb;      // SIPs whose Newton fell back to FP64
  const float4* crec;           // [C][CELL_REC] FP32 cell records (cell_records)
  double inv_dx, inv_dz;
  float inv_dxf, inv_dzf, dt_subf, dtg_f, dt_posf;
  float x_minf, x_maxf, z_minf, z_capf;
  double* water_removed;
};

// per-call scalars of a particle sub-step (common to all members)
struct PCall {
  double dt_sub, dt_pos, g_set;
  int no_iter, sol, write_Tp, hist;
  float dt_subf, dtg_f, dt_posf;
};
struct PK {
  MRef m;
  PCall c;
};

__device__ __forceinline__ PArgs make_pargs(const Member& mb, const PCall& c) {
  PArgs a;
  const lacmo_sips_t& sp = mb.sp;
  const lacmo_grid_t& g = mb.g;
  const Ws& w = mb.w;
  a.pos = sp.pos; a.vel = sp.vel; a.m_w = sp.m_w; a.rel = sp.rel_pos; a.T_p = sp.T_p;
  a.m_s = sp.m_s; a.xi = sp.xi; a.cell = sp.cell;
  a.gsf = g.scalar_fields; a.gmp = g.mat_prop; a.aux = w.aux; a.gv = g.velocity;
  a.n = sp.n; a.nx = g.nx; a.nz = g.nz;
  a.x_min = g.x_min; a.x_max = g.x_max; a.z_min = g.z_min; a.z_cap = mb.z_cap;
  a.dx = g.dx; a.dz = g.dz;
  a.dt_sub = c.dt_sub; a.dt_pos = c.dt_pos; a.g_set = c.g_set;
  a.no_iter = c.no_iter; a.sol = c.sol; a.write_Tp = c.write_Tp;
  a.dmxi = w.dmxi; a.counts = w.counts; a.rank = w.rank; a.rm_count = w.rm_count;
  a.rm_id = w.rm_id; a.rm_val = w.rm_val; a.flags = w.flags;
  a.fb_count = w.fb_count; a.fb_done = w.fb_done; a.fb_id = w.rm_id; a.fb_c = w.colk;
  a.fb_mw = w.rm_val;
  a.acc = w.div; a.hist = c.hist; a.nfb = w.nfb;
  a.crec = cell_records(w.aux, g.nx * g.nz);
  a.inv_dx = mb.inv_dx; a.inv_dz = mb.inv_dz;
  a.inv_dxf = mb.inv_dxf; a.inv_dzf = mb.inv_dzf;
  a.dt_subf = c.dt_subf; a.dtg_f = c.dtg_f; a.dt_posf = c.dt_posf;
  a.x_minf = mb.x_minf; a.x_maxf = mb.x_maxf; a.z_minf = mb.z_minf; a.z_capf = mb.z_capf;
  a.water_removed = sp.water_removed;
  return a;
}


// The wind corners the FP32 interpolation of grid.py:257-323 can read in cell
// (i, j), in float4 3..5 of the cell's record (float4 6 holds i, j and
// whether j is the bottom or top row): U[a][b] = u at (i + a,
// j - 1 + b), a < 2, b < 3, and V[a][b] = w at (i - 1 + a, j + b), a < 3,
// b < 2, as (U00 U01 U02 U10) (U11 U12 V00 V01) (V10 V11 V20 V21); indices
// below zero wrap like the reference's (the periodic column i = -1 is column
// nx; row j - 1 = -1 is never read).
__global__ void k_wind_table(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  const double* in = mb.g.velocity;
  const int64_t nx = mb.g.nx, nz = mb.g.nz, C = nx * nz;
  float4* rec = cell_records(mb.w.aux, C);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = c / nz, j = c - i * nz;
    auto at = [&](int comp, int64_t ii, int64_t jj) {
      if (ii < 0) ii += nx + 1;
      if (jj < 0) jj += nz + 1;
      return (float)in[((int64_t)comp * (nx + 1) + ii) * (nz + 1) + jj];
    };
    float4* out = rec + CELL_REC * c;
    out[3] = make_float4(at(0, i, j - 1), at(0, i, j), at(0, i, j + 1), at(0, i + 1, j - 1));
    out[4] = make_float4(at(0, i + 1, j), at(0, i + 1, j + 1), at(1, i - 1, j), at(1, i - 1, j + 1));
    out[5] = make_float4(at(1, i, j), at(1, i, j + 1), at(1, i + 1, j), at(1, i + 1, j + 1));
    out[6] = make_float4((float)i, (float)j, j == 0 ? 1.0f : 0.0f, j == nz - 1 ? 1.0f : 0.0f);
  }
}

// grid.py:257-323 in FP32 from a cell's wind corners (k_wind_table); wx, wy
// are the position in the cell in units of the cell size, jlo / jhi mark the
// bottom and top rows of cells
__device__ __forceinline__ void interp_wind(const float4 w0, const float4 w1, const float4 w2,
                                            bool jlo, bool jhi, float wx, float wy, float& u,
                                            float& v) {
  if ((jlo && wy <= 0.5f) || (jhi && wy >= 0.5f)) {
    u = wx * w1.x + (1 - wx) * w0.y;
  } else if (wy > 0.5f) {
    const float b = wy - 0.5f;
    u = wx * (b * w1.y + (1 - b) * w1.x) + (1 - wx) * (b * w0.z + (1 - b) * w0.y);
  } else {
    const float b = wy + 0.5f;
    u = wx * (b * w1.x + (1 - b) * w0.w) + (1 - wx) * (b * w0.y + (1 - b) * w0.x);
  }
  if (wx > 0.5f) {
    const float a = wx - 0.5f;
    v = a * (wy * w2.w + (1 - wy) * w2.z) + (1 - a) * (wy * w2.y + (1 - wy) * w2.x);
  } else {
    const float a = wx + 0.5f;
    v = a * (wy * w2.y + (1 - wy) * w2.x) + (1 - a) * (wy * w1.w + (1 - wy) * w1.z);
  }
}

template <bool PHYS>
__global__ void __launch_bounds__(128) k_particles(const __grid_constant__ PK x) {
  __shared__ PArgs s_a;
  if (threadIdx.x == 0) s_a = make_pargs(x.m.get(), x.c);
  __syncthreads();
  const PArgs& a = s_a;
  const int64_t C = a.nx * a.nz;
  const GridVel gv{a.gv, a.nx, a.nz};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = a.cell[k];
    const bool active = c >= 0;
    const int64_t i = active ? (int64_t)c / a.nz : (int64_t)(-1 - c);
    const int64_t j = active ? (int64_t)c - i * a.nz : -1;
    double x = a.pos[k], z = a.pos[a.n + k];
    double u = a.vel[k], w = a.vel[a.n + k];
    double mw = a.m_w[k];
    double xik = 0.0;
    double rel_x = 0.0, rel_z = 0.0;
    if (PHYS) {
      const double T_p = __ldg(a.gsf + i * a.nz + (active ? j : a.nz - 1));
      if (a.write_Tp) a.T_p[k] = T_p;
      if (active) {
        CellAmb amb;
        amb.T = T_p; amb.p = __ldg(a.gsf + C + c); amb.S = __ldg(a.gsf + 6 * C + c);
        amb.e_s = __ldg(a.gsf + 7 * C + c); amb.K = __ldg(a.gmp + c); amb.D_v = __ldg(a.gmp + C + c);
        amb.L_v = __ldg(a.gmp + 2 * C + c);
        amb.sigw = __ldg(a.aux + c); amb.rhow = __ldg(a.aux + C + c);
        amb.lap0 = __ldg(a.aux + 2 * C + c); amb.lbp0 = __ldg(a.aux + 3 * C + c);
        amb.c1 = __ldg(a.aux + 4 * C + c); amb.c2 = __ldg(a.aux + 5 * C + c);
        const double ms = a.m_s[k];
        xik = a.xi[k];
        // integration.py:1044 compute_R_p_w_s_rho_p, :916-936 Newton
        double m_p = mw + ms;
        double w_s = ms / m_p;
        double rho = (a.sol == SOL_AS) ? density_AS_solution_rw(w_s, amb.rhow)
                                       : density_NaCl_solution(w_s, T_p);
        double R = radius_from_mass(m_p, rho);
        double sig = (a.sol == SOL_AS) ? surface_tension_AS_sw(w_s, amb.sigw)
                                       : surface_tension_NaCl_sw(w_s, amb.sigw);
        double dm = newton_full(a.sol, a.dt_sub, a.no_iter, mw, ms, w_s, R, T_p, rho, sig, amb,
                                nullptr);
        mw += dm;
        a.dmxi[k] = dm * xik;
        // integration.py:1075 radius of ammonium sulfate whatever the solute
        m_p = mw + ms;
        w_s = ms / m_p;
        rho = density_AS_solution_rw(w_s, amb.rhow);
        R = radius_from_mass(m_p, rho);
        // integration.py:699-718
        rel_x = (x - a.x_min) / a.dx - (double)i;
        rel_z = (z - a.z_min) / a.dz - (double)j;
        double uf, wf;
        gv.interp(i, j, rel_x, rel_z, uf, wf);
        const double mu_f = __ldg(a.gmp + 5 * C + c), rho_f = __ldg(a.gmp + 6 * C + c);
        const double d0 = uf - u, d1 = wf - w;
        const double vel_dev = sqrt(d0 * d0 + d1 * d1);
        const double Re_p = 2.0E-6 * rho_f * R * vel_dev / mu_f;
        double k_dt = 4.5E12 * a.dt_sub * mu_f / (rho * R * R);
        if (Re_p > 0.5) {
          if (Re_p < 1000.0) k_dt *= (1 + 0.15 * pow(Re_p, 0.687));
          else k_dt *= 0.0183333333333 * Re_p;
        }
        u = (u + k_dt * uf) / (1.0 + k_dt);
        w = (w + k_dt * wf - a.dt_sub * a.g_set) / (1.0 + k_dt);
      }
    } else if (active) {
      xik = a.xi[k];
      rel_x = (x - a.x_min) / a.dx - (double)i;
      rel_z = (z - a.z_min) / a.dz - (double)j;
    }
    // integration.py:552-630
    x += a.dt_pos * u;
    z += a.dt_pos * w;
    x = py_mod(x, a.x_max);
    z = np_min(z, a.z_cap);
    int32_t newc = c;
    if (active) {
      if (z <= a.z_min) {
        z = a.z_min - 0.01 * a.dz;
        u = 0.0; w = 0.0;
        const int slot = atomicAdd(a.rm_count, 1);
        a.rm_id[slot] = (int32_t)k;
        a.rm_val[slot] = xik * mw;
        // the re-index of this call leaves the old relative position divided
        // by the cell size (integration.py:548-549)
        a.rel[k] = rel_x / a.dx - (double)i;
        a.rel[a.n + k] = rel_z / a.dz - (-1.0);
        newc = (int32_t)(-1 - i);
      } else {
        int64_t ci = (int64_t)floor(x / a.dx), cj = (int64_t)floor(z / a.dz);
        if (ci >= a.nx || ci < 0 || cj >= a.nz || cj < 0) {
          atomicOr(a.flags, LACMO_FLAG_CELL_CLAMPED);
          ci = ci < 0 ? 0 : (ci >= a.nx ? a.nx - 1 : ci);
          cj = cj < 0 ? 0 : (cj >= a.nz ? a.nz - 1 : cj);
        }
        newc = (int32_t)(ci * a.nz + cj);
        a.rank[k] = atomicAdd(a.counts + newc, 1);
      }
    } else {
      a.rel[k] = a.rel[k] / a.dx - (double)i;
      a.rel[a.n + k] = a.rel[a.n + k] / a.dz - (-1.0);
    }
    a.pos[k] = x; a.pos[a.n + k] = z;
    a.vel[k] = u; a.vel[a.n + k] = w;
    if (PHYS && active) a.m_w[k] = mw;
    a.cell[k] = newc;
  }
}

// ---------------------------------------------------------------------------
// integration.py:402-484 for one cell (and update_material_properties :359)
__device__ __forceinline__ void grid_cell_update(double* gsf, double* gmp, int64_t c, int64_t C,
                                                 double p_ref, double p_ref_inv, double dTh,
                                                 double drv, double dml, double V) {
  double Th = gsf[2 * C + c];
  const double rho_d = gsf[3 * C + c];
  double r_v = gsf[4 * C + c];
  const double mdi = gsf[8 * C + c];
  const double L_v = gmp[2 * C + c];
  Th += dTh;
  r_v += drv - dml * mdi;
  const double ToT = pow(p_ref_inv * LC_R_D * rho_d * Th, LC_KAPPA_FACTOR2);
  Th += ToT * (L_v * dml) / (LC_C_PD * rho_d * V * (1.0 + r_v * LC_HEAT_FACTOR_R_V));
  const double pdr = pow(rho_d * Th * LC_R_D * p_ref_inv, LC_KAPPA_FACTOR);
  const double T = Th * pow(pdr, LC_KAPPA_AIR_DRY);
  const double p = pdr * p_ref * (1 + r_v / LC_EPSILON_GC);
  const double e_s = 2.53E11 * exp(-5420.0 / T);
  const double S = rho_d * r_v * T * LC_R_V / e_s;
  gsf[c] = T; gsf[C + c] = p; gsf[2 * C + c] = Th; gsf[4 * C + c] = r_v;
  gsf[6 * C + c] = S; gsf[7 * C + c] = e_s;
  gmp[c] = 4.1868E-3 * (5.69 + 0.017 * (T - 273.15));
  gmp[C + c] = 4.01218E-5 * pow(T, 1.94) / p;
  gmp[2 * C + c] = 1.0E3 * (2500.82 - 2.358 * (T - 273.0));
  gmp[3 * C + c] = surface_tension_water(T);
  gmp[4 * C + c] = LC_C_PD * (1 + 0.897 * r_v);
  gmp[5 * C + c] = 1.458E-6 * pow(T, 1.5) / (T + 110.4);
  gmp[6 * C + c] = rho_d * (1.0 + r_v);
}

// one thread per cell: delta_m_l as the ascending-ID fold of dm*xi over the
// cell's SIPs (integration.py:916-936), then the grid update of the cell and
// its mass-rate terms for the next sub-step; all lanes carry FP64 work
__global__ void __launch_bounds__(32) k_cell_update(const __grid_constant__ MRef mr,
                                                     int grid_update) {
  const Member& mb = mr.get();
  const int32_t* __restrict__ start = mb.w.start;
  const int32_t* __restrict__ perm = mb.w.perm;
  const double* __restrict__ dmxi = mb.w.dmxi;
  double *delta_m_l = mb.g.delta_m_l, *gsf = mb.g.scalar_fields, *gmp = mb.g.mat_prop,
         *aux = mb.w.aux;
  const double *dTh = mb.w.dTh, *drv = mb.w.drv;
  const int64_t C = mb.g.nx * mb.g.nz;
  const double p_ref = mb.g.p_ref, p_ref_inv = mb.g.p_ref_inv, V = mb.g.volume_cell;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int32_t b = start[c], e = start[c + 1];
    double acc = 0.0;
#pragma unroll 8
    for (int32_t k = b; k < e; ++k) acc += __ldg(dmxi + __ldg(perm + k));
    const double dml = acc * 1.0E-18;
    delta_m_l[c] = dml;
    if (grid_update) {
      grid_cell_update(gsf, gmp, c, C, p_ref, p_ref_inv, dTh[c], drv[c], dml, V);
      write_aux(gsf, gmp, aux, c, C);
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed precision particle sub-step.  GB300 issues FP64 arithmetic, FP64
// compares and double<->float conversions on a pipe that is 64x narrower than
// the FP32 one, so this kernel keeps the FP64 pipe for the three state
// updates x += dx, z += dz, m_w += dm and does everything else in FP32 or in
// integer units:
//  * double -> float rounding (to nearest even) and float -> double are done
//    on the IEEE bit patterns with integer instructions (d2f_int / f2d_int);
//  * comparisons of non-negative doubles compare their bit patterns;
//  * the new cell index comes from the FP32 position with a certified margin
//    (1e-4 of a cell) around cell edges, inside which FP64 decides;
//  * the per-cell sums of dm * xi are exact integer sums (acc_add), which L2
//    executes, independent of their order.
// The Newton condensation and the drag update run in FP32 (lacmo_physics.cuh)
// with the FP64 Newton for SIPs near the critical radius.  water_removed takes
// the SIPs reaching the ground with FP64 atomics, in arbitrary order (the
// removal list of the FP64 path holds the FP64 Newton queue here).
// Rare FP64 paths stay out of line (__noinline__) so that the common path
// issues no FP64 instruction, not even predicated off.
// removed SIP: only the relative position keeps its per-call division
__device__ __noinline__ void mixed_inactive_rel(double* rel, int64_t n, double dx, double dz,
                                                int64_t k, int i) {
  rel[k] = rel[k] / dx - (double)i;
  rel[n + k] = rel[n + k] / dz - (-1.0);
}
// near the critical radius: FP64 residual and Newton step
struct NewtonFP64 {
  const double *gsf, *gmp, *aux;
  int64_t C;
  double dt_sub;
  int sol, no_iter;
  unsigned long long* nfb;
};
__device__ __noinline__ double mixed_newton_fp64(NewtonFP64 a, int32_t c, double mw, double ms) {
  const int64_t C = a.C;
  const double T_p = __ldg(a.gsf + c);   // the cell temperature
  CellAmb amb;
  amb.T = T_p; amb.p = __ldg(a.gsf + C + c); amb.S = __ldg(a.gsf + 6 * C + c);
  amb.e_s = __ldg(a.gsf + 7 * C + c); amb.K = __ldg(a.gmp + c);
  amb.D_v = __ldg(a.gmp + C + c); amb.L_v = __ldg(a.gmp + 2 * C + c);
  amb.sigw = __ldg(a.aux + c); amb.rhow = __ldg(a.aux + C + c);
  amb.lap0 = __ldg(a.aux + 2 * C + c); amb.lbp0 = __ldg(a.aux + 3 * C + c);
  amb.c1 = __ldg(a.aux + 4 * C + c); amb.c2 = __ldg(a.aux + 5 * C + c);
  const double m_p = mw + ms;
  const double w_s = ms / m_p;
  const double rho64 = (a.sol == SOL_AS) ? density_AS_solution_rw(w_s, amb.rhow)
                                         : density_NaCl_solution(w_s, T_p);
  const double R64 = radius_from_mass(m_p, rho64);
  const double sig64 = (a.sol == SOL_AS) ? surface_tension_AS_sw(w_s, amb.sigw)
                                         : surface_tension_NaCl_sw(w_s, amb.sigw);
  atomicAdd(a.nfb, 1ull);
  return newton_full(a.sol, a.dt_sub, a.no_iter, mw, ms, w_s, R64, T_p, rho64, sig64, amb,
                     nullptr);
}
// the FP64 position update near or past a boundary: periodic x
// (integration.py:577-583), capped z (:585-589), and whether the SIP reached
// the ground (:606); bit 0 of the result: below z_min
struct EdgeIn { double x, z, dx, dz, x_max, z_cap, z_min; int wrap, cap; };
__device__ __noinline__ int mixed_edges(EdgeIn e, double* xo, double* zo) {
  double x = e.x, z = e.z;
  if (e.wrap) x = py_mod(x, e.x_max);
  if (e.cap) z = np_min(z, e.z_cap);
  *xo = x; *zo = z;
  return z <= e.z_min ? 1 : 0;
}
__device__ __noinline__ int mixed_floor_div(double x, double d) { return (int)floor(x / d); }
// SIP reaching the ground (integration.py:606-630)
struct GroundGeo {
  double* rel;
  double* water_removed;
  int64_t n;
  double x_min, z_min, dx, dz;
};
__device__ __noinline__ double mixed_remove(GroundGeo a, int64_t k, int i, int j, double x0,
                                            double z0, double xik, double mw) {
  atomicAdd(a.water_removed, xik * mw);   // FP64, any order
  const double rel_x = (x0 - a.x_min) / a.dx - (double)i;
  const double rel_z = (z0 - a.z_min) / a.dz - (double)j;
  a.rel[k] = rel_x / a.dx - (double)i;
  a.rel[a.n + k] = rel_z / a.dz - (-1.0);
  return a.z_min - 0.01 * a.dz;
}

// ---- bulk copies into shared memory (cp.async.bulk + mbarrier) ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared, completion counted in bytes on the mbarrier; the SIP
// state streams through once per sub-step (L2 evict-first policy) so that
// the per-cell records the kernel gathers stay in L2
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1], %2, [%3], %4;\n" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];\n" ::"l"(p));
}
// Mixed precision: the per-cell sums of dm * xi (FP32 products) are exact
// integer sums in units of 2^-4 fg, so their order does not matter and a
// step gives the same bits run to run and batched or not.  v 2^4 rounded to
// the nearest integer (halves away from zero) from the FP32 bits, without a
// conversion instruction; |v| up to 2^58 fg (a cell's per-sub-step total
// stays below 2^59 / 2^4 fg = 36 kg); beyond, the value is clamped and
// LACMO_FLAG_ACC_RANGE raised.
constexpr double ACC_UNIT = 0.0625;   // fg per integer unit
__device__ __forceinline__ long long fix_of(float v, uint32_t* flags) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  if (e == 0) return 0;   // zero or below 2^-126
  const uint64_t m = (uint64_t)((b & 0x7fffffu) | 0x800000u);
  const int sh = e - 146;   // v 2^4 = m 2^(e - 150 + 4)
  uint64_t mag;
  if (sh >= 35 || e == 0xff) {
    atomicOr(flags, LACMO_FLAG_ACC_RANGE);
    mag = 1ull << 58;
  } else if (sh >= 0) {
    mag = m << sh;
  } else if (sh > -26) {
    mag = (m + (1ull << (-sh - 1))) >> (-sh);
  } else {
    mag = 0;
  }
  return (b >> 31) ? -(long long)mag : (long long)mag;
}
__device__ __forceinline__ void acc_add(double* acc, int64_t c, float v, uint32_t* flags) {
  atomicAdd((unsigned long long*)(acc + c), (unsigned long long)fix_of(v, flags));
}

// an mbarrier wait never spins without bound: after this many polls (each
// try_wait suspends the thread for a while) the kernel gives up and raises
// LACMO_FLAG_SYNC_TIMEOUT
constexpr uint32_t MBAR_POLL_LIMIT = 1u << 22;

// Tiles of PM_TILE consecutive SIPs move HBM -> shared memory as bulk copies,
// one per attribute, issued by one thread two tiles ahead (three stages).
// Each attribute's slot has room for a window that starts at the 16-byte
// boundary below the tile's first element (the rows z and w start 8 bytes off
// a boundary when n is odd).  When a tile's data lands, every thread
// prefetches the cell record of its SIP in that tile into L1, one tile
// before it is used.  Tiles a bulk copy cannot take (the last ones of a
// member, or arrays not 16-byte aligned) are loaded by the threads.
#ifndef LACMO_PM_THREADS
#define LACMO_PM_THREADS 128
#endif
constexpr int PM_THREADS = LACMO_PM_THREADS;
constexpr int PM_TILE = PM_THREADS;
constexpr int PM_STAGES = 3;
enum { PF_X, PF_Z, PF_U, PF_W, PF_MW, PF_MS, PF_XI, PF_N };
struct PmStage {
  double f[PF_N][PM_TILE + 2];
  int32_t c[PM_TILE + 4];
};

template <bool PHYS>
struct PmTiles {
  // the rows z and w (second rows of pos and vel) start 8 bytes off a 16-byte
  // boundary when n is odd: their slots then hold the window from 8 bytes
  // below the tile's first element, and the data starts at slot index zoff
  int zoff;
  bool bulk;   // arrays aligned for bulk copies
  __device__ __forceinline__ void init(const PArgs& a) {
    uintptr_t al = (uintptr_t)a.pos | (uintptr_t)a.vel | (uintptr_t)a.cell;
    if (PHYS) al |= (uintptr_t)a.m_w | (uintptr_t)a.m_s | (uintptr_t)a.xi;
    bulk = al % 16 == 0;
    zoff = bulk ? (int)(a.n & 1) : 0;
  }
  // tile k0 by bulk copy: aligned arrays, and every window inside its array
  // (the window of a second row reaches 8 bytes past the tile's end)
  __device__ __forceinline__ bool by_bulk(const PArgs& a, int64_t k0) const {
    return bulk && k0 + PM_TILE + 2 <= a.n;
  }
  __device__ __forceinline__ void issue(const PArgs& a, int64_t k0, PmStage& s, uint64_t* bar,
                                        uint64_t pol) const {
    const uint32_t zb = PM_TILE * 8 + 16 * zoff;   // bytes of a second-row window
    mbar_expect_tx(bar, PM_TILE * 4 + (PHYS ? 5 : 2) * PM_TILE * 8 + 2 * zb);
    bulk_g2s(&s.f[PF_X][0], a.pos + k0, PM_TILE * 8, bar, pol);
    bulk_g2s(&s.f[PF_Z][0], a.pos + a.n + k0 - zoff, zb, bar, pol);
    bulk_g2s(&s.f[PF_U][0], a.vel + k0, PM_TILE * 8, bar, pol);
    bulk_g2s(&s.f[PF_W][0], a.vel + a.n + k0 - zoff, zb, bar, pol);
    if (PHYS) {
      bulk_g2s(&s.f[PF_MW][0], a.m_w + k0, PM_TILE * 8, bar, pol);
      bulk_g2s(&s.f[PF_MS][0], a.m_s + k0, PM_TILE * 8, bar, pol);
      bulk_g2s(&s.f[PF_XI][0], a.xi + k0, PM_TILE * 8, bar, pol);
    }
    bulk_g2s(&s.c[0], a.cell + k0, PM_TILE * 4, bar, pol);
  }
  // the slot of thread t's SIP in the stage
  __device__ __forceinline__ double get(const PmStage& s, int f, int t) const {
    return s.f[f][(f == PF_Z || f == PF_W) ? zoff + t : t];
  }
  // the threads' own loads of a tile (same slots)
  __device__ __forceinline__ void load(const PArgs& a, int64_t k, PmStage& s, int t) const {
    if (k >= a.n) return;
    s.f[PF_X][t] = __ldcs(a.pos + k);
    s.f[PF_Z][zoff + t] = __ldcs(a.pos + a.n + k);
    s.f[PF_U][t] = __ldcs(a.vel + k);
    s.f[PF_W][zoff + t] = __ldcs(a.vel + a.n + k);
    if (PHYS) {
      s.f[PF_MW][t] = __ldcs(a.m_w + k);
      s.f[PF_MS][t] = __ldcs(a.m_s + k);
      s.f[PF_XI][t] = __ldcs(a.xi + k);
    }
    s.c[t] = __ldcs(a.cell + k);
  }
};

// MINB: resident blocks per SM the register budget is set for (the
// TUNE_PARTICLE_BLOCKS knob picks the instance)
template <bool PHYS, int MINB>
__global__ void __launch_bounds__(PM_THREADS, MINB) k_particles_mixed(const __grid_constant__ PK x) {
  // the member's arguments, once per block in shared memory: threads read
  // them on use instead of holding some 60 registers of pointers and sizes
  __shared__ PArgs s_a;
  extern __shared__ __align__(128) unsigned char pm_smem[];
  PmStage* st = (PmStage*)pm_smem;
  __shared__ __align__(8) uint64_t s_bar[PM_STAGES];
  const int t = threadIdx.x;
  if (t == 0) {
    s_a = make_pargs(x.m.get(), x.c);
    for (int q = 0; q < PM_STAGES; ++q) mbar_init(&s_bar[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncthreads();
  const PArgs& a = s_a;
  const int C = (int)(a.nx * a.nz);
  const int nz = (int)a.nz;
  PmTiles<PHYS> tl;
  tl.init(a);
  // SIP indices fit in 32 bits (n < 2^31)
  const int ntiles = (int)((a.n + PM_TILE - 1) / PM_TILE);
  const int G = gridDim.x;
  const int first = blockIdx.x;
  const int my_tiles = first < ntiles ? (ntiles - first + G - 1) / G : 0;
  // prologue: tiles 0 and 1 of this block in flight
  if (t == 0) {
    const uint64_t pol = l2_evict_first_policy();
    for (int i = 0; i < 2 && i < my_tiles; ++i) {
      const int k0 = (first + i * G) * PM_TILE;
      if (tl.by_bulk(a, k0)) tl.issue(a, k0, st[i], &s_bar[i], pol);
    }
  }
  bool tout = false;   // an mbarrier wait of this thread ran out of polls
  int i = 0;
  for (; i < my_tiles; ++i) {
    const int k0 = (first + i * G) * PM_TILE;
    const int sg = i % PM_STAGES;
    // every thread is done with tile i - 1's stage; all stop together when a
    // wait ran out
    if (i > 0 && __syncthreads_or(tout)) break;
    if (t == 0 && i + 2 < my_tiles) {
      const int k2 = (first + (i + 2) * G) * PM_TILE;
      const int s2 = (i + 2) % PM_STAGES;
      if (tl.by_bulk(a, k2)) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        tl.issue(a, k2, st[s2], &s_bar[s2], l2_evict_first_policy());
      }
    }
    // this tile's data (the first tile's, else waited for one tile ago), and
    // the next tile's: its cell records go to L1 now
    for (int w = (i == 0 ? 0 : 1); w <= 1; ++w) {
      const int iw = i + w;
      if (iw >= my_tiles) break;
      const int kw = (first + iw * G) * PM_TILE;
      if (!tl.by_bulk(a, kw)) continue;
      const int sw = iw % PM_STAGES;
      const uint32_t parity = (uint32_t)((iw / PM_STAGES) & 1);
      uint32_t polls = 0;
      while (!mbar_try_wait(&s_bar[sw], parity)) {
        if (++polls >= MBAR_POLL_LIMIT) { tout = true; break; }
      }
      if (PHYS && w == 1 && !tout) {
        const int32_t cn = st[sw].c[t];
        if (cn >= 0) prefetch_l1(a.crec + CELL_REC * (int64_t)cn);
      }
    }
    if (tout) continue;   // this tile's data cannot be trusted
    PmStage& S = st[sg];
    const int k = k0 + t;
    if (!tl.by_bulk(a, k0)) tl.load(a, k, S, t);
    if (k >= a.n) continue;
    const int32_t c = S.c[t];
    if (c < 0) {
      const int i_ = -1 - c;
      if (a.write_Tp) a.T_p[k] = __ldg(a.gsf + (int64_t)i_ * nz + nz - 1);
      mixed_inactive_rel(a.rel, a.n, a.dx, a.dz, k, i_);
      continue;
    }
    if (a.write_Tp) a.T_p[k] = __ldg(a.gsf + c);
    float un, wn2, d = 0.0f, xf, zf;
    int fb_slot = -1;   // queue slot of a SIP whose Newton repeats in FP64
    const float4* rec = a.crec + CELL_REC * (int64_t)c;
    if (PHYS) {
      const float4 q0 = __ldg(rec), q1 = __ldg(rec + 1);
      CellAmbF af;
      af.T = q0.x; af.S_m1 = q0.y; af.sigw = q0.z; af.rhow = q0.w;
      af.lap0 = q1.x; af.lbp0 = q1.y; af.c1 = q1.z; af.c2 = q1.w;
      const float msf = d2f_int(tl.get(S, PF_MS, t)), mwf = d2f_int(tl.get(S, PF_MW, t));
      const float mpf = mwf + msf;
      const float wsf = msf * f_rcp(mpf);
      const float rho = (a.sol == SOL_AS)
                            ? af.rhow * ((((float)LC_PAR_RHO_AS_0 * wsf + (float)LC_PAR_RHO_AS_1) *
                                              wsf + (float)LC_PAR_RHO_AS_2) * wsf +
                                         (float)LC_PAR_RHO_AS_3)
                            : (float)LC_PAR_SOL_DENS_NACL_0 + (float)LC_PAR_SOL_DENS_NACL_1 * wsf +
                                  (float)LC_PAR_SOL_DENS_NACL_2 * af.T +
                                  (float)LC_PAR_SOL_DENS_NACL_3 * wsf * wsf +
                                  (float)LC_PAR_SOL_DENS_NACL_4 * wsf * af.T +
                                  (float)LC_PAR_SOL_DENS_NACL_5 * af.T * af.T;
      const float R = f_cbrt((float)LC_FOUR_PI_OVER_THREE_INV * mpf * f_rcp(rho));
      const float sig = af.sigw * (1.0f + (a.sol == SOL_AS ? (float)LC_PAR_SIGMA_AS
                                                            : (float)LC_PAR_SIGMA_NACL) *
                                               wsf * f_rcp(1.f - wsf));
      // efflorescence floor m_s (1/0.78 - 1) as an increment, in FP32
      const float d_effl = msf * (float)(LC_W_S_MAX_AS_INV - 1.0) - mwf;
      const bool ok = newton_mixed_f(a.sol, a.dt_subf, a.no_iter, mwf, msf, wsf, R, af.T, rho,
                                     sig, af, d_effl, &d);
      if (ok) {
        // per-cell exact sum of dm * xi (executed by L2)
        acc_add(a.acc, c, d * d2f_int(tl.get(S, PF_XI, t)), a.flags);
      } else {
        // near the critical radius the Newton repeats in FP64, in full warps
        // in k_newton_fallback: queue the SIP with its mass before the
        // sub-step; drag and motion go on with the FP32 increment
        fb_slot = atomicAdd(a.fb_count, 1);
        a.fb_id[fb_slot] = (int32_t)k;
        a.fb_c[fb_slot] = c;
        a.fb_mw[fb_slot] = tl.get(S, PF_MW, t);
      }
      // drag (integration.py:699-718) in FP32 with the ammonium-sulfate radius
      const float mpn = (mwf + d) + msf;
      const float wn = msf * f_rcp(mpn);
      const float rhon = af.rhow * ((((float)LC_PAR_RHO_AS_0 * wn + (float)LC_PAR_RHO_AS_1) * wn +
                                     (float)LC_PAR_RHO_AS_2) * wn + (float)LC_PAR_RHO_AS_3);
      const float Rn = f_cbrt((float)LC_FOUR_PI_OVER_THREE_INV * mpn * f_rcp(rhon));
      const float4 cij = __ldg(rec + 6);   // (i, j, j == 0, j == nz - 1)
      xf = d2f_int(tl.get(S, PF_X, t));
      zf = d2f_int(tl.get(S, PF_Z, t));
      const float rxf = (xf - a.x_minf) * a.inv_dxf - cij.x;
      const float rzf = (zf - a.z_minf) * a.inv_dzf - cij.y;
      float uf, wf;
      interp_wind(__ldg(rec + 3), __ldg(rec + 4), __ldg(rec + 5), cij.z != 0.0f, cij.w != 0.0f,
                  rxf, rzf, uf, wf);
      const float2 q2 = __ldg((const float2*)(rec + 2));
      const float mu_f = q2.x, rho_f = q2.y;
      const float uo = d2f_int(tl.get(S, PF_U, t)), wo = d2f_int(tl.get(S, PF_W, t));
      const float d0 = uf - uo, d1 = wf - wo;
      const float vel_dev = f_sqrt(d0 * d0 + d1 * d1);
      const float inv_mu = f_rcp(mu_f);
      const float Re_p = 2.0E-6f * rho_f * Rn * vel_dev * inv_mu;
      float k_dt = 4.5E12f * a.dt_subf * mu_f * f_rcp(rhon * Rn * Rn);
      if (Re_p > 0.5f) {
        if (Re_p < 1000.0f) k_dt *= (1.f + 0.15f * f_pow(Re_p, 0.687f));
        else k_dt *= 0.0183333333333f * Re_p;
      }
      const float inv = f_rcp(1.0f + k_dt);
      un = (uo + k_dt * uf) * inv;
      wn2 = (wo + k_dt * wf - a.dtg_f) * inv;
    } else {
      // the half-step move of integration.py:1474-1481: positions only
      un = d2f_int(tl.get(S, PF_U, t));
      wn2 = d2f_int(tl.get(S, PF_W, t));
      xf = d2f_int(tl.get(S, PF_X, t));
      zf = d2f_int(tl.get(S, PF_Z, t));
    }
    // position (integration.py:552-630)
    const double x0 = tl.get(S, PF_X, t), z0 = tl.get(S, PF_Z, t);
    const float xf0 = xf, zf0 = zf;
    const float dxf = a.dt_posf * un, dzf = a.dt_posf * wn2;
    double xn = x0 + f2d_int(dxf);
    double zn = z0 + f2d_int(dzf);
    const float xnf = xf0 + dxf, znf = zf0 + dzf;
    double u = f2d_int(un), w = f2d_int(wn2);
    // periodic x / capped z / ground: exact FP64 only when near or past a
    // boundary
    const int wrap = !(xnf > 1e-3f && xnf < a.x_maxf - 1e-3f);
    const int cap = !(znf < a.z_capf - 1e-3f);
    const int low = !(znf > a.z_minf + 1e-3f);
    int edge = 0;
    if (wrap | cap | low)
      edge = mixed_edges(EdgeIn{xn, zn, a.dx, a.dz, a.x_max, a.z_cap, a.z_min, wrap, cap}, &xn,
                         &zn);
    int32_t newc;
    bool removed = false;
    if (low && (edge & 1)) {
      const int i_ = c / nz, j_ = c - i_ * nz;
      const double xik = PHYS ? tl.get(S, PF_XI, t) : a.xi[k];
      double mw = PHYS ? tl.get(S, PF_MW, t) + f2d_int(d) : a.m_w[k];
      if (PHYS && fb_slot >= 0) {
        // a queued SIP leaving the domain: its FP64 Newton here, for the
        // water it takes along
        const double mw0 = tl.get(S, PF_MW, t);
        const double dm = mixed_newton_fp64(NewtonFP64{a.gsf, a.gmp, a.aux, (int64_t)C, a.dt_sub,
                                                       a.sol, a.no_iter, a.nfb},
                                            c, mw0, tl.get(S, PF_MS, t));
        mw = mw0 + dm;
        acc_add(a.acc, c, d2f_int(dm) * d2f_int(xik), a.flags);
        a.fb_id[fb_slot] = -1;
      }
      if (PHYS) __stcs(a.m_w + k, mw);
      zn = mixed_remove(GroundGeo{a.rel, a.water_removed, a.n, a.x_min, a.z_min, a.dx, a.dz}, k,
                        i_, j_, x0, z0, xik, mw);
      u = 0.0; w = 0.0;
      removed = true;
      newc = (int32_t)(-1 - i_);
    } else {
      // the new cell from the FP32 position, FP64 when within 1e-4 of an edge
      const float px = wrap ? d2f_int(xn) : xnf, pz = cap ? d2f_int(zn) : znf;
      const float qx = px * a.inv_dxf, qz = pz * a.inv_dzf;
      int ci = __float2int_rd(qx), cj = __float2int_rd(qz);
      const float fx = qx - floorf(qx), fz = qz - floorf(qz);
      if (!(fx > 1e-4f && fx < 0.9999f)) ci = mixed_floor_div(xn, a.dx);
      if (!(fz > 1e-4f && fz < 0.9999f)) cj = mixed_floor_div(zn, a.dz);
      if (ci >= a.nx || ci < 0 || cj >= nz || cj < 0) {
        atomicOr(a.flags, LACMO_FLAG_CELL_CLAMPED);
        ci = ci < 0 ? 0 : (ci >= a.nx ? (int)a.nx - 1 : ci);
        cj = cj < 0 ? 0 : (cj >= nz ? nz - 1 : cj);
      }
      newc = (int32_t)(ci * nz + cj);
      if (a.hist) a.rank[k] = atomicAdd(a.counts + newc, 1);
      if (PHYS) __stcs(a.m_w + k, tl.get(S, PF_MW, t) + f2d_int(d));
    }
    // streaming stores (evict first)
    __stcs(a.pos + k, xn); __stcs(a.pos + a.n + k, zn);
    if (PHYS || removed) { __stcs(a.vel + k, u); __stcs(a.vel + a.n + k, w); }
    __stcs(a.cell + k, newc);
  }
  if (__syncthreads_or(tout)) {
    // a wait ran out: flag it, and wait (again bounded) for the copies this
    // block may still have in flight before the block's shared memory goes
    if (t == 0) {
      atomicOr(a.flags, LACMO_FLAG_SYNC_TIMEOUT);
      for (int j = i; j < i + 2 && j < my_tiles; ++j) {
        if (!tl.by_bulk(a, (first + j * G) * PM_TILE)) continue;
        const int sj = (int)(j % PM_STAGES);
        for (uint32_t p = 0; p < MBAR_POLL_LIMIT; ++p)
          if (mbar_try_wait(&s_bar[sj], (uint32_t)((j / PM_STAGES) & 1))) break;
      }
    }
  }
}
constexpr size_t PM_SMEM = (size_t)PM_STAGES * sizeof(PmStage);

// The FP64 Newton of the SIPs a mixed sub-step queued (near the critical
// radius), one SIP per thread: the mass and the per-cell sum as the inline
// FP64 path gives them; the last block empties the queue.
__global__ void __launch_bounds__(128) k_newton_fallback(const __grid_constant__ PK x) {
  __shared__ PArgs s_a;
  if (threadIdx.x == 0) s_a = make_pargs(x.m.get(), x.c);
  __syncthreads();
  const PArgs& a = s_a;
  const int cnt = *(volatile int32_t*)a.fb_count;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += gridDim.x * blockDim.x) {
    const int32_t k = a.fb_id[q];
    if (k < 0) continue;   // handled where it left the domain
    const int32_t c = a.fb_c[q];
    const double mw0 = a.fb_mw[q];
    const double dm = mixed_newton_fp64(NewtonFP64{a.gsf, a.gmp, a.aux, a.nx * a.nz, a.dt_sub,
                                                   a.sol, a.no_iter, a.nfb},
                                        c, mw0, a.m_s[k]);
    a.m_w[k] = mw0 + dm;
    acc_add(a.acc, c, d2f_int(dm) * d2f_int(a.xi[k]), a.flags);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(a.fb_done, 1) == (int)gridDim.x - 1) {
      *a.fb_count = 0;
      *a.fb_done = 0;
    }
  }
}

// Mixed precision: the grid update of one cell (integration.py:402-484,
// update_material_properties :359-400) in FP64 with exp/log in place of pow,
// pow(x, y) = exp(y log x) to a few 1e-15 relative, and the chained powers of
// the Exner function folded into one log; then the per-cell Newton terms
// (FP64 and the FP32 table) from the same values.
__device__ __forceinline__ void grid_cell_update_mixed(double* gsf, double* gmp, double* aux,
                                                       int64_t c, int64_t C, double p_ref,
                                                       double p_ref_inv, double dTh, double drv,
                                                       double dml, double V) {
  double Th = gsf[2 * C + c];
  const double rho_d = gsf[3 * C + c];
  double r_v = gsf[4 * C + c];
  const double mdi = gsf[8 * C + c];
  const double L_v0 = gmp[2 * C + c];
  Th += dTh;
  r_v += drv - dml * mdi;
  const double ToT = exp(LC_KAPPA_FACTOR2 * log(p_ref_inv * LC_R_D * rho_d * Th));
  Th += ToT * (L_v0 * dml) / (LC_C_PD * rho_d * V * (1.0 + r_v * LC_HEAT_FACTOR_R_V));
  const double L2 = log(rho_d * Th * LC_R_D * p_ref_inv);
  const double pdr = exp(LC_KAPPA_FACTOR * L2);
  const double T = Th * exp((LC_KAPPA_FACTOR * LC_KAPPA_AIR_DRY) * L2);
  const double p = pdr * p_ref * (1 + r_v / LC_EPSILON_GC);
  const double e_s = 2.53E11 * exp(-5420.0 / T);
  const double S = rho_d * r_v * T * LC_R_V / e_s;
  const double K = 4.1868E-3 * (5.69 + 0.017 * (T - 273.15));
  const double D_v = 4.01218E-5 * exp(1.94 * log(T)) / p;
  const double L_v = 1.0E3 * (2500.82 - 2.358 * (T - 273.0));
  const double tau = 1 - T / 647.096;
  const double sigw = 0.2358 * exp(1.256 * log(tau)) * (1 - 0.625 * tau);
  const double mu = 1.458E-6 * T * sqrt(T) / (T + 110.4);
  const double rho_f = rho_d * (1.0 + r_v);
  gsf[c] = T; gsf[C + c] = p; gsf[2 * C + c] = Th; gsf[4 * C + c] = r_v;
  gsf[6 * C + c] = S; gsf[7 * C + c] = e_s;
  gmp[c] = K; gmp[C + c] = D_v; gmp[2 * C + c] = L_v; gmp[3 * C + c] = sigw;
  gmp[4 * C + c] = LC_C_PD * (1 + 0.897 * r_v); gmp[5 * C + c] = mu; gmp[6 * C + c] = rho_f;
  // the terms of make_cell_amb (lacmo_physics.cuh) from the values above
  const double rhow = density_water(T);
  const double lap0 = (LC_C_ALPHA_1 + LC_C_ALPHA_2 * (T - LC_T_ALPHA_0)) * K / p;
  const double lbp0 = LC_C_BETA_1 * (1.0 + LC_C_BETA_2 * (T - LC_T_ALPHA_0)) * D_v;
  const double c1 = L_v * L_v / (LC_R_V * K * T * T);
  const double c2 = LC_R_V * T / (D_v * e_s);
  aux[c] = sigw; aux[C + c] = rhow; aux[2 * C + c] = lap0; aux[3 * C + c] = lbp0;
  aux[4 * C + c] = c1; aux[5 * C + c] = c2;
  float4* af = cell_records(aux, C) + CELL_REC * c;
  af[0] = make_float4((float)T, (float)(S - 1.0), (float)sigw, (float)rhow);
  af[1] = make_float4((float)lap0, (float)lbp0, (float)c1, (float)c2);
  af[2] = make_float4((float)mu, (float)rho_f, 0.0f, 0.0f);
}

// mixed precision: the grid sub-step from the per-cell exact sums (then zeroed)
__global__ void k_grid_acc(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  double *acc = mb.w.div, *delta_m_l = mb.g.delta_m_l, *gsf = mb.g.scalar_fields,
         *gmp = mb.g.mat_prop, *aux = mb.w.aux;
  const double *dTh = mb.w.dTh, *drv = mb.w.drv;
  const int64_t C = mb.g.nx * mb.g.nz;
  const double p_ref = mb.g.p_ref, p_ref_inv = mb.g.p_ref_inv, V = mb.g.volume_cell;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x) {
    long long* acc_i = (long long*)acc;
    const double dml = (double)acc_i[c] * ACC_UNIT * 1.0E-18;
    acc_i[c] = 0;
    delta_m_l[c] = dml;
    grid_cell_update_mixed(gsf, gmp, aux, c, C, p_ref, p_ref_inv, dTh[c], drv[c], dml, V);
  }
}

__global__ void k_grid_only(double* gsf, double* gmp, double* aux, const double* dTh,
                            const double* drv, const double* dml, int64_t C, double p_ref,
                            double p_ref_inv, double V) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x) {
    grid_cell_update(gsf, gmp, c, C, p_ref, p_ref_inv, dTh[c], drv[c], dml[c], V);
    if (aux) write_aux(gsf, gmp, aux, c, C);
  }
}

// grid.py:370-412 (ascending-ID fold per cell)
__global__ void __launch_bounds__(256) k_r_l(const __grid_constant__ MRef mr) {
  const Member& mb = mr.get();
  const int32_t* __restrict__ start = mb.w.start;
  const int32_t* __restrict__ perm = mb.w.perm;
  const double* __restrict__ m_w = mb.sp.m_w;
  const double* __restrict__ xi = mb.sp.xi;
  double* gsf = mb.g.scalar_fields;
  const int64_t C = mb.g.nx * mb.g.nz;
  const int lane = threadIdx.x & 31;
  for (int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; c < C;
       c += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t b = start[c], e = start[c + 1];
    double acc = 0.0;
    for (int32_t base = b; base < e; base += 32) {
      const int32_t idx = base + lane;
      double v = 0.0;
      if (idx < e) { int32_t id = perm[idx]; v = m_w[id] * xi[id]; }
      const int m = (e - base) < 32 ? (e - base) : 32;
      for (int q = 0; q < m; ++q) acc += __shfl_sync(0xffffffffu, v, q);
    }
    if (lane == 0) gsf[5 * C + c] = acc * (1.0E-18 * gsf[8 * C + c]);
  }
}

// ---------------------------------------------------------------------------
// integration.py:80-148 limiter and face flux (Hundsdorfer et al. 1995)
__device__ __forceinline__ double limiter_arg(double a0, double a1, double a2) {
  const double r = (fabs(a1 - a2) > 1.0E-8 * fabs(a0 - a1)) ? (a0 - a1) / (a1 - a2)
                                                             : (a0 - a1) * 1.0E8 * np_sign(a1 - a2);
  const double K = (1.0 + 2.0 * r) * LC_ONE_THIRD;
  return np_max(0.0, fmin(2.0 * r, fmin(K, 2.0)));
}
__device__ __forceinline__ double face_flux(double u, double am2, double am1, double a0,
                                            double ap1) {
  const double lp = limiter_arg(a0, am1, am2);
  const double f_pos = am1 + 0.5 * lp * (am1 - am2);
  const double ln = limiter_arg(am1, a0, ap1);
  const double f_neg = a0 + 0.5 * ln * (a0 - ap1);
  return (u >= 0.0) ? u * f_pos : u * f_neg;
}
__device__ __forceinline__ int64_t bc_idx(int64_t i, int64_t N, int bc) {
  if (bc == 0) { i %= N; return i < 0 ? i + N : i; }
  return i < 0 ? 0 : (i > N - 1 ? N - 1 : i);
}
// integration.py:150-287, divergence of field * flux in cell (i, j)
__device__ double divergence_cell(const double* f, const double* flux, int64_t nx, int64_t nz,
                                  int64_t i, int64_t j, double dx, double dz, int bcx, int bcz) {
  double Fx[2], Fz[2];
  for (int s = 0; s < 2; ++s) {
    const int64_t fi = i + s;  // face index
    double u = flux[fi * (nz + 1) + j];
    Fx[s] = face_flux(u, f[bc_idx(fi - 2, nx, bcx) * nz + j], f[bc_idx(fi - 1, nx, bcx) * nz + j],
                      f[bc_idx(fi, nx, bcx) * nz + j], f[bc_idx(fi + 1, nx, bcx) * nz + j]);
    if (bcx == 1 && (fi == 0 || fi == nx)) Fx[s] = 0.0;
    const int64_t fj = j + s;
    double w = flux[(nx + 1) * (nz + 1) + i * (nz + 1) + fj];
    Fz[s] = face_flux(w, f[i * nz + bc_idx(fj - 2, nz, bcz)], f[i * nz + bc_idx(fj - 1, nz, bcz)],
                      f[i * nz + bc_idx(fj, nz, bcz)], f[i * nz + bc_idx(fj + 1, nz, bcz)]);
    if (bcz == 1 && (fj == 0 || fj == nz)) Fz[s] = 0.0;
  }
  return (Fx[1] - Fx[0]) / dx + (Fz[1] - Fz[0]) / dz;
}

__global__ void k_divergence(const double* f, const double* flux, int64_t nx, int64_t nz, double dx,
                             double dz, int bcx, int bcz, double* out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nx * nz;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = c / nz, j = c - i * nz;
    out[c] = divergence_cell(f, flux, nx, nz, i, j, dx, dz, bcx, bcz);
  }
}

// integration.py:325-354; the column sum runs over x in order like NumPy's
// axis-0 reduction of a C-ordered array
__global__ void k_relaxation(const double* f, int64_t nx, int64_t nz, const double* prof,
                             const double* trel, double dt, double* out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nz;
       j += (int64_t)gridDim.x * blockDim.x) {
    double s = f[j];
    for (int64_t i = 1; i < nx; ++i) s += f[i * nz + j];
    out[j] = dt * (prof[j] - s / (double)nx) / trel[j];
  }
}

// both relaxation terms of a sub-step in one launch: r_v into out[0:nz],
// Theta into out[nz:2nz] (integration.py:325-354)
__global__ void k_relaxation2(const __grid_constant__ MRef mr, const double* prof_rv,
                              const double* prof_th, const double* trel, double dt) {
  const Member& mb = mr.get();
  const double* gsf = mb.g.scalar_fields;
  const int64_t nx = mb.g.nx, nz = mb.g.nz;
  double* out = mb.w.relax;
  if (mb.prof_rv) { prof_rv = mb.prof_rv; prof_th = mb.prof_th; trel = mb.t_relax; }
  const int64_t C = nx * nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 2 * nz;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t < nz ? t : t - nz;
    const double* f = gsf + (t < nz ? 4 : 2) * C;
    const double* prof = t < nz ? prof_rv : prof_th;
    double s = f[j];
#pragma unroll 8
    for (int64_t i = 1; i < nx; ++i) s += f[i * nz + j];
    out[t] = dt * (prof[j] - s / (double)nx) / trel[j];
  }
}

// integration.py:1483-1508 (factor 1) and 1536-1561 (factor 2, minus the
// previous increment): advective + relaxation increments per sub-step
__global__ void k_advection(const __grid_constant__ MRef mr, double dt_sub, int relax_on,
                            int second) {
  const Member& mb = mr.get();
  const double *gsf = mb.g.scalar_fields, *flux = mb.g.mass_flux_air_dry, *relax = mb.w.relax;
  const int64_t nx = mb.g.nx, nz = mb.g.nz;
  const double dx = mb.g.dx, dz = mb.g.dz;
  double *dTh = mb.w.dTh, *drv = mb.w.drv;
  const int64_t C = nx * nz;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = c / nz, j = c - i * nz;
    const double rdi = gsf[9 * C + c];
    const double drv_div = divergence_cell(gsf + 4 * C, flux, nx, nz, i, j, dx, dz, 0, 1);
    const double dth_div = divergence_cell(gsf + 2 * C, flux, nx, nz, i, j, dx, dz, 0, 1);
    double a, b;
    if (!second) {
      a = -dt_sub * drv_div * rdi;
      b = -dt_sub * dth_div * rdi;
      if (relax_on) { a += relax[j]; b += relax[nz + j]; }
    } else {
      a = -2.0 * dt_sub * drv_div * rdi - drv[c];
      b = -2.0 * dt_sub * dth_div * rdi - dTh[c];
      if (relax_on) { a += 2. * relax[j]; b += 2. * relax[nz + j]; }
    }
    drv[c] = a; dTh[c] = b;
  }
}

// ---------------------------------------------------------------------------
// elementwise microphysics (unit parity entry points)
__global__ void k_mass_rate(int sol, int64_t n, InPtrs in, double* g, double* dg) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    CellAmb a = make_cell_amb(in.p[6][k], in.p[7][k], in.p[8][k], in.p[9][k], in.p[10][k], in.p[11][k], in.p[12][k]);
    a.sigw = surface_tension_water(in.p[4][k]);
    a.rhow = density_water(in.p[4][k]);
    mass_rate_and_derivative(sol, in.p[0][k], in.p[1][k], in.p[2][k], in.p[3][k], in.p[4][k], in.p[5][k],
                             in.p[13][k], a, g[k], dg[k]);
  }
}
__global__ void k_newton(int sol, int64_t n, double dt_sub, int no_iter, InPtrs in, double* dm,
                         double* g0) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    CellAmb a = make_cell_amb(in.p[6][k], in.p[7][k], in.p[8][k], in.p[9][k], in.p[10][k], in.p[11][k], in.p[12][k]);
    a.sigw = surface_tension_water(in.p[4][k]);
    a.rhow = density_water(in.p[4][k]);
    dm[k] = newton_full(sol, dt_sub, no_iter, in.p[0][k], in.p[1][k], in.p[2][k], in.p[3][k], in.p[4][k],
                        in.p[5][k], in.p[13][k], a, g0 + k);
  }
}
__global__ void k_interp(const int32_t* cell, const double* rel, const double* gvp, int64_t n,
                         int64_t nx, int64_t nz, double* out) {
  const GridVel gv{gvp, nx, nz};
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int32_t c = cell[k];
    double u = 0.0, v = 0.0;
    if (c >= 0) {
      int64_t i = c / nz, j = c - (c / nz) * nz;
      gv.interp(i, j, rel[k], rel[n + k], u, v);
    }
    out[k] = u; out[n + k] = v;
  }
}

// ---------------------------------------------------------------------------
cudaError_t launch_cells_import(const int64_t* cells, const uint8_t* act, int32_t* cell, int64_t n,
                                int64_t nx, int64_t nz, cudaStream_t s) {
  (void)nx;
  k_cells_import<<<nblocks(n, 256), 256, 0, s>>>(cells, act, cell, n, nz); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_cells_export(const int32_t* cell, const double* pos, double* rel, int64_t* cells,
                                uint8_t* act, int64_t n, int64_t nx, int64_t nz, double x_min,
                                double z_min, double dx, double dz, cudaStream_t s) {
  (void)nx;
  k_cells_export<<<nblocks(n, 256), 256, 0, s>>>(cell, pos, rel, cells, act, n, nz, x_min, z_min,
                                                 dx, dz); note_launches(1);
  return cudaGetLastError();
}
static inline dim3 grid2(int64_t per_member, int t, int M, int cap = 152 * 32) {
  return dim3((unsigned)nblocks(per_member, t, cap), (unsigned)M);
}
static PCall pcall(const lacmo_params_t& p, double dt_sub, double dt_pos, bool write_Tp,
                   bool hist) {
  PCall c;
  c.dt_sub = dt_sub; c.dt_pos = dt_pos; c.g_set = p.g_set;
  c.no_iter = p.no_iter_impl_mass; c.sol = p.solute; c.write_Tp = write_Tp ? 1 : 0;
  c.hist = hist ? 1 : 0;
  c.dt_subf = (float)dt_sub; c.dtg_f = (float)(dt_sub * p.g_set); c.dt_posf = (float)dt_pos;
  return c;
}
cudaError_t launch_cell_aux(const Bt& B, cudaStream_t s) {
  k_cell_aux<<<grid2(B.nx * B.nz, 32, B.M), 32, 0, s>>>(B.ref()); note_launches(1);
  // the wind part of the cell records too, for sub-steps run before a full step
  k_wind_table<<<grid2(B.nx * B.nz, 256, B.M), 256, 0, s>>>(B.ref()); note_launches(1);
  return cudaGetLastError();
}
__global__ void k_set_i64(int64_t* p, int64_t v) { *p = v; }
cudaError_t launch_set_i64(int64_t* p, int64_t v, cudaStream_t s) {
  k_set_i64<<<1, 1, 0, s>>>(p, v); note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_histogram(const Bt& B, cudaStream_t s) {
  k_histogram<<<grid2(B.n_max, 256, B.M), 256, 0, s>>>(B.ref()); note_launches(1);
  return cudaGetLastError();
}
// the ground removals folded into water_removed without binning (k_scan over
// counts left at zero: the binning it writes is empty until the next one)
cudaError_t launch_fold_removals(const Bt& B, cudaStream_t s) {
  k_scan<<<dim3(1, B.M), 1024, 0, s>>>(B.ref()); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_bin(const Bt& B, cudaStream_t s) {
  const int64_t C = B.nx * B.nz;
  k_scan<<<dim3(1, B.M), 1024, 0, s>>>(B.ref()); note_launches(1);
  k_scatter<<<grid2(B.n_max, 256, B.M), 256, 0, s>>>(B.ref()); note_launches(1);
  k_order<<<grid2(C * 32, 256, B.M, 152 * tune_value(TUNE_ORDER_CTAS)), 256, 0, s>>>(B.ref());
  note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_particles(const Bt& B, const lacmo_params_t& p, double dt_sub,
                             double dt_sub_pos, bool write_Tp, cudaStream_t s) {
  PK x{B.ref(), pcall(p, dt_sub, dt_sub_pos, write_Tp, true)};
  k_particles<true><<<grid2(B.n_max, 128, B.M, 152 * 16), 128, 0, s>>>(x); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_move(const Bt& B, double dt_pos, cudaStream_t s) {
  lacmo_params_t p = {};
  PK x{B.ref(), pcall(p, 0.0, dt_pos, false, true)};
  k_particles<false><<<grid2(B.n_max, 128, B.M, 152 * 16), 128, 0, s>>>(x); note_launches(1);
  return cudaGetLastError();
}
// Resident-sized grid for the pipelined mixed kernel: each thread walks many
// SIPs so the one-ahead staging hides the loads of all but the first.
template <bool PHYS, int MINB>
static cudaError_t mixed_launch(const Bt& B, const PK& x, cudaStream_t s) {
  static std::atomic<int> cached[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int res = dev < 64 ? cached[dev].load() : 0;
  if (res <= 0) {
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_particles_mixed<PHYS, MINB>,
                                                      PM_THREADS, PM_SMEM);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    res = per_sm * sms > 0 ? per_sm * sms : 1;
    if (dev < 64) cached[dev].store(res);
  }
  // resident-sized grid: each warp walks many tiles through the staging
  // pipeline; small states take one block per tile (more blocks in flight
  // hide the latency better)
  int64_t bx = res / B.M;
  const int64_t need = (B.n_max + PM_THREADS - 1) / PM_THREADS;
  if (bx * PM_THREADS * 8 > B.n_max) bx = need < 152 * 16 ? need : 152 * 16;
  if (bx > need) bx = need;
  if (bx < 1) bx = 1;
  k_particles_mixed<PHYS, MINB><<<dim3((unsigned)bx, (unsigned)B.M), PM_THREADS, PM_SMEM, s>>>(x);
  note_launches(1);
  return cudaGetLastError();
}
template <bool PHYS>
static cudaError_t mixed_launch_tuned(const Bt& B, const PK& x, cudaStream_t s) {
  switch (tune_value(TUNE_PARTICLE_BLOCKS)) {
    case 5: return mixed_launch<PHYS, 5>(B, x, s);
    case 8: return mixed_launch<PHYS, 8>(B, x, s);
    default: return mixed_launch<PHYS, 6>(B, x, s);
  }
}
cudaError_t launch_particles_mixed(const Bt& B, const lacmo_params_t& p, double dt_sub,
                                   double dt_sub_pos, bool write_Tp, bool hist, cudaStream_t s) {
  PK x{B.ref(), pcall(p, dt_sub, dt_sub_pos, write_Tp, hist)};
  cudaError_t e = mixed_launch_tuned<true>(B, x, s);
  if (e != cudaSuccess) return e;
  k_newton_fallback<<<dim3(64, B.M), 128, 0, s>>>(x); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_move_mixed(const Bt& B, double dt_pos, cudaStream_t s) {
  lacmo_params_t p = {};
  PK x{B.ref(), pcall(p, 0.0, dt_pos, false, true)};
  return mixed_launch<false, 6>(B, x, s);
}
cudaError_t launch_wind_float(const Bt& B, cudaStream_t s) {
  k_wind_table<<<grid2(B.nx * B.nz, 256, B.M), 256, 0, s>>>(B.ref()); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_grid_acc(const Bt& B, cudaStream_t s) {
  k_grid_acc<<<grid2(B.nx * B.nz, 32, B.M), 32, 0, s>>>(B.ref()); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_cell_update(const Bt& B, bool grid_update, cudaStream_t s) {
  k_cell_update<<<grid2(B.nx * B.nz, 32, B.M), 32, 0, s>>>(B.ref(), grid_update ? 1 : 0); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_grid_only(const lacmo_grid_t& g, const double* dTh, const double* drv,
                             const double* dml, double* aux, cudaStream_t s) {
  int64_t C = g.nx * g.nz;
  k_grid_only<<<nblocks(C, 32), 32, 0, s>>>(g.scalar_fields, g.mat_prop, aux, dTh, drv, dml, C,
                                              g.p_ref, g.p_ref_inv, g.volume_cell); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_advection(const Bt& B, const lacmo_params_t& p, bool second, cudaStream_t s) {
  const bool relax_on = p.act_relaxation && p.init_profile_r_v && p.init_profile_Theta &&
                        p.relaxation_time_profile;
  if (relax_on) {
    k_relaxation2<<<grid2(2 * B.nz, 32, B.M), 32, 0, s>>>(B.ref(), p.init_profile_r_v,
                                                           p.init_profile_Theta,
                                                           p.relaxation_time_profile, p.dt_sub); note_launches(1);
  }
  k_advection<<<grid2(B.nx * B.nz, 32, B.M), 32, 0, s>>>(B.ref(), p.dt_sub, relax_on ? 1 : 0,
                                                          second ? 1 : 0); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_divergence(const double* f, const double* flux, int64_t nx, int64_t nz,
                              double dx, double dz, int bcx, int bcz, double* out, cudaStream_t s) {
  k_divergence<<<nblocks(nx * nz, 128), 128, 0, s>>>(f, flux, nx, nz, dx, dz, bcx, bcz, out); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_relaxation(const double* f, int64_t nx, int64_t nz, const double* prof,
                              const double* trel, double dt, double* out, cudaStream_t s) {
  k_relaxation<<<nblocks(nz, 128), 128, 0, s>>>(f, nx, nz, prof, trel, dt, out); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_r_l_binned(const Bt& B, cudaStream_t s) {
  k_r_l<<<grid2(B.nx * B.nz * 32, 256, B.M, 152 * 16), 256, 0, s>>>(B.ref()); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_mass_rate(int sol, int64_t n, const InPtrs& in, double* g, double* dg,
                             cudaStream_t s) {
  k_mass_rate<<<nblocks(n, 128), 128, 0, s>>>(sol, n, in, g, dg); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_newton(int sol, int64_t n, double dt_sub, int no_iter, const InPtrs& in,
                          double* dm, double* g0, cudaStream_t s) {
  k_newton<<<nblocks(n, 128), 128, 0, s>>>(sol, n, dt_sub, no_iter, in, dm, g0); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_interp(const int32_t* cell, const double* rel, const double* gv, int64_t n,
                          int64_t nx, int64_t nz, double* out, cudaStream_t s) {
  k_interp<<<nblocks(n, 128), 128, 0, s>>>(cell, rel, gv, n, nx, nz, out); note_launches(1);
  return cudaGetLastError();
}

}  // namespace lacmo
