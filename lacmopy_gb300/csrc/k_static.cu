// All-cells collision step that allocates nothing: its scratch memory is a
// fixed-size array in this library's own device memory instead of a
// caller-provided workspace.
//
// Some callers cannot allocate device memory when they want to run a
// collision step: code that runs inside another framework's memory pool or
// under a strict memory budget, plugin hosts that forbid cudaMalloc after
// start-up, or a stream that is being recorded.  For them this variant keeps
// its scratch (cell counts and offsets, the (cell, ID) order, the radius /
// kernel-bin fallback for big cells) in the file-scope array below.  The
// array is part of the library image: every GPU that loads the library holds
// it until the process exits.  Each call clears what must start at zero.
// Every call uses the same array, so calls whose work overlaps on the GPU
// (different streams, or different host threads on one device) race and
// must be serialised by the caller.
#include <cuda_runtime.h>

#include "lacmo_internal.cuh"

namespace lacmo {

// capacities of the scratch array
constexpr int64_t STATIC_MAX_SIPS = LACMO_NOALLOC_MAX_SIPS;
constexpr int64_t STATIC_MAX_CELLS = LACMO_NOALLOC_MAX_CELLS;

constexpr size_t a256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t st_off_counts = 0;
constexpr size_t st_off_start = a256(st_off_counts + 4 * STATIC_MAX_CELLS);
constexpr size_t st_off_draw = a256(st_off_start + 4 * (STATIC_MAX_CELLS + 1));
constexpr size_t st_off_perm = a256(st_off_draw + 8 * (STATIC_MAX_CELLS + 1));
constexpr size_t st_off_rank = a256(st_off_perm + 4 * STATIC_MAX_SIPS);
constexpr size_t st_off_colR = a256(st_off_rank + 4 * STATIC_MAX_SIPS);
constexpr size_t st_off_colrho = a256(st_off_colR + 8 * STATIC_MAX_SIPS);
constexpr size_t st_off_colk = a256(st_off_colrho + 8 * STATIC_MAX_SIPS);
constexpr size_t st_off_order = a256(st_off_colk + 4 * STATIC_MAX_SIPS);
constexpr size_t st_off_gcopy = a256(st_off_order + 4 * STATIC_MAX_CELLS);
constexpr size_t st_off_gstats = a256(st_off_gcopy + 24 * STATIC_MAX_SIPS);
constexpr size_t st_off_Ef = a256(st_off_gstats + 32 * (STATIC_MAX_SIPS / 32 + STATIC_MAX_CELLS + 1));
constexpr size_t st_off_scalars =
    a256(st_off_Ef + 4 * (size_t)LACMO_MAX_KERNEL_BINS * (LACMO_MAX_KERNEL_BINS + 1));
constexpr size_t STATIC_BYTES = st_off_scalars + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[STATIC_BYTES];

// The device address of the array.  In host code the symbol name is only a
// host-side stand-in, so the address is looked up with the caller's device
// current.  The lookup runs on every call (it is not a stream operation):
// a cached address would go stale after cudaDeviceReset or after the primary
// context is released and created again, when the module is loaded anew.
// The first lookup on a device loads the module there, which is why the
// first call should come before any stream capture.
static cudaError_t scratch_address(void** out) {
  return cudaGetSymbolAddress(out, g_noalloc_scratch);
}

// zero the cell counters and the scalars; set the collision-step counter
__global__ void k_static_clear(int32_t* counts, int64_t C, uint32_t* flags, int32_t* rm_count,
                               int64_t* cursor, int64_t* col_step, int64_t* total,
                               int32_t* cell_ctr, int64_t step) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
       c += (int64_t)gridDim.x * blockDim.x)
    counts[c] = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *flags = 0; *rm_count = 0; *cursor = 0; *col_step = step; *total = 0; *cell_ctr = 0;
  }
}

}  // namespace lacmo

using namespace lacmo;

extern "C" int lacmo_collision_step_cells_noalloc(double* xi, double* m_w, double* m_s,
                                                  const double* vel, const double* grid_T,
                                                  const int32_t* cell, int64_t n, int64_t nx,
                                                  int64_t nz, const lacmo_params_t* prm,
                                                  const lacmo_draws_t* draws, uint64_t step,
                                                  int64_t* no_cols, void* stream) {
  if (!xi || !m_w || !m_s || !vel || !grid_T || !cell || !prm || !draws || !no_cols || n <= 0 ||
      nx <= 0 || nz <= 0)
    return LACMO_ERR_ARG;
  if (prm->solute != 0 && prm->solute != 1) return LACMO_ERR_ARG;
  if (prm->E_col_grid && prm->no_kernel_bins <= 0) return LACMO_ERR_ARG;
  // nx and nz are bounded before they are multiplied (no int64 overflow)
  if (n > STATIC_MAX_SIPS || nx > STATIC_MAX_CELLS || nz > STATIC_MAX_CELLS ||
      nx * nz > STATIC_MAX_CELLS)
    return LACMO_ERR_CAPACITY;
  void* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return LACMO_ERR_CUDA;
  char* b = (char*)base;
  Ws w = {};
  w.counts = (int32_t*)(b + st_off_counts);
  w.start = (int32_t*)(b + st_off_start);
  w.draw_off = (int64_t*)(b + st_off_draw);
  w.perm = (int32_t*)(b + st_off_perm);
  w.rank = (int32_t*)(b + st_off_rank);
  w.colR = (double*)(b + st_off_colR);
  w.colrho = (double*)(b + st_off_colrho);
  w.colk = (int32_t*)(b + st_off_colk);
  w.cell_order = (int32_t*)(b + st_off_order);
  w.gcopy = (float*)(b + st_off_gcopy);
  w.gstats = (float*)(b + st_off_gstats);
  w.Ef = (float*)(b + st_off_Ef);
  char* sc = b + st_off_scalars;
  w.flags = (uint32_t*)sc;
  w.rm_count = (int32_t*)(sc + 4);
  w.cursor = (int64_t*)(sc + 8);
  w.col_step = (int64_t*)(sc + 16);
  w.total_pairs = (int64_t*)(sc + 24);
  w.cell_ctr = (int32_t*)(sc + 40);
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t C = nx * nz;
  // the entry points below read only these members of the SIP and grid state
  lacmo_sips_t sp = {};
  sp.n = n; sp.vel = (double*)vel; sp.m_w = m_w; sp.m_s = m_s; sp.xi = xi;
  sp.cell = (int32_t*)cell; sp.no_cols = no_cols;
  lacmo_grid_t g = {};
  g.nx = nx; g.nz = nz; g.scalar_fields = (double*)grid_T;
  int blocks = (int)((C + 255) / 256 < 1024 ? (C + 255) / 256 : 1024);
  k_static_clear<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(w.counts, C, w.flags, w.rm_count,
                                                         w.cursor, w.col_step, w.total_pairs,
                                                         w.cell_ctr, (int64_t)step);
  note_launches(1);
  if (cudaGetLastError() != cudaSuccess) return LACMO_ERR_CUDA;
  const Bt B = single(sp, g, w, draws->seed);
  if (launch_histogram(B, s) != cudaSuccess) return LACMO_ERR_CUDA;
  if (launch_bin(B, s) != cudaSuccess) return LACMO_ERR_CUDA;
  if (launch_collide_cells(B, *prm, *draws, s) != cudaSuccess) return LACMO_ERR_CUDA;
  return LACMO_OK;
}

extern "C" int lacmo_noalloc_status(uint32_t* flags, int64_t* pairs, void* stream) {
  if (!flags && !pairs) return LACMO_ERR_ARG;
  void* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return LACMO_ERR_CUDA;
  const char* sc = (const char*)base + st_off_scalars;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t f = 0;
  int64_t p = 0;
  if (cudaMemcpyAsync(&f, sc, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&p, sc + 24, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return LACMO_ERR_CUDA;
  if (flags) *flags = f;
  if (pairs) *pairs = p;
  return LACMO_OK;
}
