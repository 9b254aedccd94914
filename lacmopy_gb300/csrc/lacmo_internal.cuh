// Internal definitions shared by the kernels and the C ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lacmo_gb300.h"

namespace lacmo {

// Workspace layout: one caller-owned device buffer carved into these arrays.
// C = nx * nz cells, n SIPs.
struct Ws {
  int32_t* counts;     // [C]   SIPs per cell for the next binning (zeroed by the scan)
  int32_t* start;      // [C+1] first slot of each cell in perm
  int64_t* draw_off;   // [C+1] first pair draw of each cell, relative to the cursor
  int32_t* perm;       // [n]   SIP IDs sorted by (cell, ID)
  int32_t* rank;       // [n]   arrival slot of each SIP inside its cell
  double* dmxi;        // [n]   dm * xi of the last condensation sub-step
  int32_t* rm_id;      // [n]   SIPs removed at the ground in the last sub-step
  double* rm_val;      // [n]   their xi * m_w
  double* aux;         // [6][C] per-cell terms: sigma_w, rho_w, l_alpha, l_beta, c1, c2,
                       // then the mixed path's FP32 table [C][12]
  double* dTh;         // [C]   Delta Theta (advection + relaxation) per sub-step
  double* drv;         // [C]   Delta r_v per sub-step
  double* div;         // [C]   divergence scratch
  double* relax;       // [2][nz] relaxation terms (r_v, Theta)
  double* colR;        // [n]   collision scratch for cells above the shared-memory size
  double* colrho;      // [n]
  int32_t* colk;       // [n]
  // scalars
  uint32_t* flags;
  int32_t* rm_count;
  int64_t* cursor;     // injected-draw cursor
  int64_t* col_step;   // collision-step counter (Philox)
  int64_t* total_pairs;
  unsigned long long* nfb;   // mixed precision: Newton repeats in FP64
  float* Ef;                 // [LACMO_MAX_KERNEL_BINS^2] FP32 copy of the efficiency table,
                             // then [LACMO_MAX_KERNEL_BINS] row maxima
  int32_t* cell_order;       // [C]   cells by descending SIP count (collision work order)
  int32_t* cell_ctr;         // next entry of cell_order a collision warp takes
  int32_t *fb_count, *fb_done;   // mixed precision: FP64 Newton queue length, blocks done
  float* gcopy;              // [6][n] collision FP32 copies of cells above the shared-memory size
  float* gstats;             // [n/32 + C + 1][8] block statistics of those cells (thinned draws)
};

// The FP32 per-cell records of the mixed-precision particle kernel, after the
// six FP64 per-cell terms in the aux array: 8 float4 (one 128-byte line) per
// cell, cell-major: [0..2] the Newton and drag terms (write_aux), [3..5] the
// wind corners (k_wind_table).
__host__ __device__ inline size_t cell_records_offset(int64_t C) {
  return (size_t)((6 * C + 15) / 16) * 16;   // in doubles, 128-byte aligned
}
__host__ __device__ inline float4* cell_records(double* aux, int64_t C) {
  return (float4*)(aux + cell_records_offset(C));
}
constexpr int CELL_REC = 8;   // float4 per cell record


// launch-shape knobs of lacmo_tune_* (process-wide; read at launch, so a
// CUDA graph keeps the shapes it was captured with)
enum { TUNE_PARTICLE_BLOCKS = 0, TUNE_COLLISION_BLOCKS = 1, TUNE_ORDER_CTAS = 2, TUNE_KNOBS = 3 };
int tune_value(int knob);

size_t ws_bytes(int64_t n, int64_t nx, int64_t nz);
bool ws_carve(void* base, size_t bytes, int64_t n, int64_t nx, int64_t nz, Ws* ws);
// process-wide count of kernels this library has launched (lacmo_kernel_launches)
void note_launches(int k);

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): one block of 128 random
// bits per (key, counter).  A collision pair of rank k draws from block
// (k >> 1, c1): its uniform has the 53 bits (x0 >> 5, x1 >> 6) for even k
// and (x2 >> 5, x3 >> 6) for odd k, so one block serves two pairs.
struct PhiloxBlock { uint32_t x0, x1, x2, x3; };
__device__ __forceinline__ PhiloxBlock philox_block(uint64_t key, uint64_t c0, uint64_t c1) {
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  uint32_t x0 = (uint32_t)c0, x1 = (uint32_t)(c0 >> 32), x2 = (uint32_t)c1, x3 = (uint32_t)(c1 >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
    uint32_t y0 = hi1 ^ x1 ^ k0, y1 = lo1, y2 = hi0 ^ x3 ^ k1, y3 = lo0;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return PhiloxBlock{x0, x1, x2, x3};
}
__device__ __forceinline__ uint64_t philox_half53(const PhiloxBlock& b, bool odd) {
  const uint32_t a = odd ? b.x2 : b.x0, c = odd ? b.x3 : b.x1;
  return (uint64_t)(a >> 5) * 67108864ull + (uint64_t)(c >> 6);
}
// the 53 bits of pair rank k, and its uniform in [0, 1)
__device__ __forceinline__ uint64_t philox_bits53(uint64_t key, uint64_t k, uint64_t c1) {
  return philox_half53(philox_block(key, k >> 1, c1), (k & 1) != 0);
}
__device__ __forceinline__ double philox_uniform(uint64_t key, uint64_t k, uint64_t c1) {
  return (double)philox_bits53(key, k, c1) * (1.0 / 9007199254740992.0);
}

// One ensemble member as the kernels see it: its SIP and grid state, its
// workspace slice, its Philox key and derived geometry constants (computed on
// the host, so kernels convert nothing).  A batch keeps a table of members in
// device memory and its kernels index it by blockIdx.y; a single member is
// passed by value in the kernel parameters.  All members share nx and nz.
struct Member {
  lacmo_sips_t sp;
  lacmo_grid_t g;
  Ws w;
  uint64_t seed;
  const double *prof_rv, *prof_th, *t_relax;   // member's relaxation profiles (null: common)
  double z_cap, inv_dx, inv_dz;
  float x_minf, x_maxf, z_minf, z_capf, inv_dxf, inv_dzf;
};
Member make_member(const lacmo_sips_t& sp, const lacmo_grid_t& g, const Ws& w, uint64_t seed);

// kernel-side handle: the table or the single member
struct MRef {
  const Member* dev;
  Member one;
  __device__ __forceinline__ const Member& get() const { return dev ? dev[blockIdx.y] : one; }
};

// launch context of M members (M == 1: dev is null and one holds the member)
struct Bt {
  int M;
  const Member* dev;
  Member one;
  int64_t n_max;   // largest member SIP count
  int64_t nx, nz;  // common grid shape
  MRef ref() const { return MRef{dev, one}; }
};
Bt single(const lacmo_sips_t& sp, const lacmo_grid_t& g, const Ws& w, uint64_t seed);

// ---- launches (k_particles.cu) ----
cudaError_t launch_cells_import(const int64_t* cells, const uint8_t* act, int32_t* cell, int64_t n,
                                int64_t nx, int64_t nz, cudaStream_t s);
cudaError_t launch_cells_export(const int32_t* cell, const double* pos, double* rel_pos,
                                int64_t* cells, uint8_t* act, int64_t n, int64_t nx, int64_t nz,
                                double x_min, double z_min, double dx, double dz, cudaStream_t s);
cudaError_t launch_cell_aux(const Bt& B, cudaStream_t s);
// *p = v, stream-ordered (one thread)
cudaError_t launch_set_i64(int64_t* p, int64_t v, cudaStream_t s);
cudaError_t launch_histogram(const Bt& B, cudaStream_t s);
cudaError_t launch_bin(const Bt& B, cudaStream_t s);
cudaError_t launch_fold_removals(const Bt& B, cudaStream_t s);
cudaError_t launch_particles(const Bt& B, const lacmo_params_t& p, double dt_sub,
                             double dt_sub_pos, bool write_Tp, cudaStream_t s);
cudaError_t launch_move(const Bt& B, double dt_pos, cudaStream_t s);
cudaError_t launch_particles_mixed(const Bt& B, const lacmo_params_t& p, double dt_sub,
                                   double dt_sub_pos, bool write_Tp, bool hist, cudaStream_t s);
cudaError_t launch_move_mixed(const Bt& B, double dt_pos, cudaStream_t s);
cudaError_t launch_grid_acc(const Bt& B, cudaStream_t s);
cudaError_t launch_wind_float(const Bt& B, cudaStream_t s);
cudaError_t launch_cell_update(const Bt& B, bool grid_update, cudaStream_t s);
cudaError_t launch_grid_only(const lacmo_grid_t& g, const double* dTh, const double* drv,
                             const double* dml, double* aux, cudaStream_t s);
cudaError_t launch_advection(const Bt& B, const lacmo_params_t& p, bool second, cudaStream_t s);
cudaError_t launch_divergence(const double* f, const double* flux, int64_t nx, int64_t nz,
                              double dx, double dz, int bcx, int bcz, double* out, cudaStream_t s);
cudaError_t launch_relaxation(const double* f, int64_t nx, int64_t nz, const double* prof,
                              const double* trel, double dt, double* out, cudaStream_t s);
cudaError_t launch_r_l_binned(const Bt& B, cudaStream_t s);
// inputs of the elementwise microphysics kernels, in the order of
// lacmo_mass_rate_and_derivative's array arguments
struct InPtrs { const double* p[14]; };
cudaError_t launch_mass_rate(int sol, int64_t n, const InPtrs& in, double* g, double* dg,
                             cudaStream_t s);
cudaError_t launch_newton(int sol, int64_t n, double dt_sub, int no_iter, const InPtrs& in,
                          double* dm, double* g0, cudaStream_t s);
cudaError_t launch_interp(const int32_t* cell, const double* rel, const double* gv, int64_t n,
                          int64_t nx, int64_t nz, double* out, cudaStream_t s);

// ---- launches (k_collision.cu) ----
// draws: injected buffer (single member only) or null for Philox keyed by
// each member's seed
cudaError_t launch_collide_cells(const Bt& B, const lacmo_params_t& p, const lacmo_draws_t& d,
                                 cudaStream_t s);
cudaError_t launch_golovin(double* xis, double* m, int64_t n, double dtdv, int64_t* no_cols,
                           const double* rnd, uint64_t seed, uint64_t step, cudaStream_t s);
cudaError_t launch_kgrid_box(double* xis, double* m, int64_t n, double dtdv, const double* K,
                             int64_t nb, double lo, double bl, int64_t* no_cols, const double* rnd,
                             uint64_t seed, uint64_t step, cudaStream_t s);
cudaError_t launch_ecol_box(double* xis, double* m, double* R, const double* vel,
                            const double* rho, int64_t n, double dtdv, const double* E, int64_t nb,
                            double lo, double bl, int64_t* no_cols, const double* rnd,
                            uint64_t seed, uint64_t step, cudaStream_t s);
cudaError_t launch_beard(double* vel, const double* R, int64_t n, cudaStream_t s);
cudaError_t launch_radius_bin(const double* m, const double* rho, int64_t n, double lo, double bl,
                              int64_t nb, double* R, int64_t* k, cudaStream_t s);

}  // namespace lacmo
