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
  double* aux;         // [6][C] per-cell terms: sigma_w, rho_w, l_alpha, l_beta, c1, c2
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
  float* gvf;                // [2][nx+1][nz+1] FP32 copy of the wind (mixed precision)
};

size_t ws_bytes(int64_t n, int64_t nx, int64_t nz);
bool ws_carve(void* base, size_t bytes, int64_t n, int64_t nx, int64_t nz, Ws* ws);
// process-wide count of kernels this library has launched (lacmo_kernel_launches)
void note_launches(int k);

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), returns a uniform double
// in [0, 1) with 53 random bits.
__device__ __forceinline__ double philox_uniform(uint64_t key, uint64_t c0, uint64_t c1) {
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
  uint64_t a = x0 >> 5, b = x1 >> 6;
  return (double)(a * 67108864ull + b) * (1.0 / 9007199254740992.0);
}

// The 53 random bits of the same generator (philox_uniform = bits * 2^-53).
__device__ __forceinline__ uint64_t philox_bits53(uint64_t key, uint64_t c0, uint64_t c1) {
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
  return (uint64_t)(x0 >> 5) * 67108864ull + (uint64_t)(x1 >> 6);
}

// ---- launches (k_particles.cu) ----
cudaError_t launch_cells_import(const int64_t* cells, const uint8_t* act, int32_t* cell, int64_t n,
                                int64_t nx, int64_t nz, cudaStream_t s);
cudaError_t launch_cells_export(const int32_t* cell, const double* pos, double* rel_pos,
                                int64_t* cells, uint8_t* act, int64_t n, int64_t nx, int64_t nz,
                                double x_min, double z_min, double dx, double dz, cudaStream_t s);
cudaError_t launch_cell_aux(const lacmo_grid_t& g, const Ws& w, cudaStream_t s);
cudaError_t launch_histogram(const int32_t* cell, int64_t n, const Ws& w, cudaStream_t s);
cudaError_t launch_bin(const lacmo_sips_t& sp, int64_t C, const Ws& w, cudaStream_t s);
cudaError_t launch_particles(const lacmo_sips_t& sp, const lacmo_grid_t& g, const lacmo_params_t& p,
                             double dt_sub, double dt_sub_pos, bool write_Tp, const Ws& w,
                             cudaStream_t s);
cudaError_t launch_particles_mixed(const lacmo_sips_t& sp, const lacmo_grid_t& g,
                                   const lacmo_params_t& p, double dt_sub, double dt_sub_pos,
                                   bool write_Tp, bool hist, const Ws& w, cudaStream_t s);
cudaError_t launch_grid_acc(const lacmo_grid_t& g, const Ws& w, cudaStream_t s);
cudaError_t launch_wind_float(const lacmo_grid_t& g, const Ws& w, cudaStream_t s);
cudaError_t launch_cell_update(const lacmo_sips_t& sp, const lacmo_grid_t& g, const Ws& w,
                               const double* dTh, const double* drv, bool grid_update,
                               cudaStream_t s);
cudaError_t launch_grid_only(const lacmo_grid_t& g, const double* dTh, const double* drv,
                             const double* dml, double* aux, cudaStream_t s);
cudaError_t launch_advection(const lacmo_grid_t& g, const lacmo_params_t& p, const Ws& w,
                             double factor, bool subtract_prev, cudaStream_t s);
cudaError_t launch_divergence(const double* f, const double* flux, int64_t nx, int64_t nz,
                              double dx, double dz, int bcx, int bcz, double* out, cudaStream_t s);
cudaError_t launch_relaxation(const double* f, int64_t nx, int64_t nz, const double* prof,
                              const double* trel, double dt, double* out, cudaStream_t s);
cudaError_t launch_r_l_binned(const lacmo_sips_t& sp, const lacmo_grid_t& g, const Ws& w,
                              cudaStream_t s);
cudaError_t launch_move(const lacmo_sips_t& sp, const lacmo_grid_t& g, double dt_pos, const Ws& w,
                        cudaStream_t s);
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
cudaError_t launch_collide_cells(const lacmo_sips_t& sp, const lacmo_grid_t& g,
                                 const lacmo_params_t& p, const lacmo_draws_t& d, const Ws& w,
                                 cudaStream_t s);
cudaError_t launch_col_advance(const Ws& w, cudaStream_t s);
cudaError_t launch_golovin(double* xis, double* m, int64_t n, double dtdv, int64_t* no_cols,
                           const double* rnd, uint64_t seed, uint64_t step, cudaStream_t s);
cudaError_t launch_ecol_box(double* xis, double* m, double* R, const double* vel,
                            const double* rho, int64_t n, double dtdv, const double* E, int64_t nb,
                            double lo, double bl, int64_t* no_cols, const double* rnd,
                            uint64_t seed, uint64_t step, cudaStream_t s);
cudaError_t launch_beard(double* vel, const double* R, int64_t n, cudaStream_t s);
cudaError_t launch_radius_bin(const double* m, const double* rho, int64_t n, double lo, double bl,
                              int64_t nb, double* R, int64_t* k, cudaStream_t s);

}  // namespace lacmo
