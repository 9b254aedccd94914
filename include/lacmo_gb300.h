/*
 * lacmo_gb300 — C ABI of the GB300 (sm_103a) super-droplet (SIP) hot path.
 *
 * Drop-in boundary for LacmoPy's per-timestep step functions.  Every entry
 * point takes raw DEVICE pointers, sizes and a CUDA stream (as void*), never
 * synchronises unless stated, and returns an int status (LACMO_OK = 0).  The
 * caller owns all memory; scratch ("workspace") memory is also passed in by
 * the caller, sized by lacmo_workspace_bytes().  Arrays keep the reference's
 * layout (row-major NumPy): particle arrays are indexed by SIP ID, pos/vel/
 * rel_pos are [2][n], grid fields are [fields][nx][nz], staggered velocity
 * and mass flux are [2][nx+1][nz+1].  The one internal format is the cell
 * index: int32 cell[n] = i*nz + j for active SIPs and -1-i for SIPs removed at
 * the ground (the reference keeps cells[2][n] int64 plus active_ids[n];
 * lacmo_cells_import/export convert).
 *
 * Reference file:line citations are relative to the LacmoPy source tree.
 */
#ifndef LACMO_GB300_H
#define LACMO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LACMO_ABI_VERSION 1
/* tables up to this many kernel bins get an FP32 copy for the pair screen */
#define LACMO_MAX_KERNEL_BINS 512

/* status codes (negative: error, nothing or part of the work done) */
#define LACMO_OK 0
#define LACMO_ERR_ARG (-1)          /* bad size, null pointer, bad option    */
#define LACMO_ERR_CUDA (-2)         /* a CUDA runtime call failed            */
#define LACMO_ERR_DRAWS (-3)        /* injected draw buffer too short        */
#define LACMO_ERR_WORKSPACE (-4)    /* workspace too small                   */
#define LACMO_ERR_CAPACITY (-5)     /* size above a fixed capacity           */
/* device-side condition flags, read with lacmo_read_flags() */
#define LACMO_FLAG_DRAWS_SHORT 0x1u     /* a collision step skipped: draws   */
#define LACMO_FLAG_CELL_CLAMPED 0x2u    /* x == x_max after the periodic wrap */
#define LACMO_FLAG_NONFINITE 0x4u       /* NaN/inf met in a SIP mass         */
#define LACMO_FLAG_CELL_TOO_BIG 0x8u    /* a cell above 65535 SIPs was not collided */
#define LACMO_FLAG_CELL_RANGE 0x10u     /* a SIP's cell index >= nx*nz: left out of
                                           the binning (not collided)           */
#define LACMO_FLAG_SYNC_TIMEOUT 0x20u   /* a kernel's bounded wait on its own
                                           copies ran out; its work is incomplete */
#define LACMO_FLAG_ACC_RANGE 0x40u      /* mixed precision: a SIP's dm * xi beyond
                                           2^58 fg in a cell sum (clamped)      */

#define LACMO_SOLUTE_AS 0
#define LACMO_SOLUTE_NACL 1

/* SIP state, device pointers; arrays indexed by SIP ID 0..n-1. */
typedef struct {
  int64_t n;
  double* pos;            /* [2][n] x, z (m)                                 */
  double* vel;            /* [2][n] u, w (m/s)                               */
  double* rel_pos;        /* [2][n] relative cell position                   */
  double* m_w;            /* [n] water mass (1e-18 kg)                       */
  double* m_s;            /* [n] solute mass (1e-18 kg)                      */
  double* xi;             /* [n] multiplicity                                */
  double* T_p;            /* [n] particle temperature (K)                    */
  int32_t* cell;          /* [n] see header comment                          */
  double* water_removed;  /* [1] water mass removed at the ground            */
  int64_t* no_cols;       /* [2] collision counters (single, multiple)       */
} lacmo_sips_t;

/* Grid state, device pointers. */
typedef struct {
  int64_t nx, nz;
  double* scalar_fields;          /* [10][nx][nz] T,p,Theta,rho_d,r_v,r_l,S,e_s,1/m_d,1/rho_d */
  double* mat_prop;               /* [7][nx][nz]  K,D_v,L_v,sigma_w,c_p,mu,rho_f              */
  const double* velocity;         /* [2][nx+1][nz+1]                                          */
  const double* mass_flux_air_dry;/* [2][nx+1][nz+1]                                          */
  double* delta_m_l;              /* [nx][nz] condensed mass of the last sub-step (kg)        */
  double x_min, x_max, z_min, z_max, dx, dz;
  double volume_cell, p_ref, p_ref_inv;
} lacmo_grid_t;

/* Step parameters (integration.py:1298-1313 argument list). */
typedef struct {
  double dt, dt_sub, dt_sub_half, dt_col_over_dV, g_set;
  int32_t scale_dt_cond, no_col_per_adv, act_collisions, act_relaxation;
  int32_t no_iter_impl_mass, solute;
  const double* init_profile_r_v;         /* [nz] or NULL                    */
  const double* init_profile_Theta;       /* [nz] or NULL                    */
  const double* relaxation_time_profile;  /* [nz] or NULL                    */
  const double* E_col_grid;               /* [nb][nb], NULL: constant E      */
  double E_col_const;
  int64_t no_kernel_bins;
  double R_kernel_low_log, bin_factor_R_log;
  int32_t precision;     /* LACMO_PRECISION_FP64 or LACMO_PRECISION_MIXED     */
  int32_t thin_draws;    /* Philox draws only: 0 one draw per pair; 1 the
                            thinned draws (the same iid uniforms, one draw per
                            low-probability segment of up to 32 pairs;
                            lacmo_thin.h; needs E_col_grid with at most
                            LACMO_MAX_KERNEL_BINS bins, else per pair)         */
} lacmo_params_t;

/* Arithmetic of lacmo_integrate_adv_step.  FP64: the reference's FP64 path
 * (per-cell sums in SIP-ID order).  MIXED: the Newton condensation and the
 * drag update in FP32, with the Newton repeated in FP64 for SIPs near the
 * critical radius of activation; state, positions, per-cell condensed-mass
 * sums (into Theta / r_v), multiplicities and the collision step stay FP64;
 * the per-cell sums of dm * xi are exact integer sums (units of 2^-4 fg), so
 * their order does not matter and the state after a step is the same run to
 * run; only water_removed adds the SIPs reaching the ground with FP64
 * atomics (any order). */
#define LACMO_PRECISION_FP64 0
#define LACMO_PRECISION_MIXED 1

/* Uniform draws for the all-or-nothing collisions.  With draws != NULL the
 * steps consume the buffer in the reference's order (cells x-outer, z-inner;
 * pairs i<j lexicographic, SIPs by ascending ID) from a device-side cursor
 * that starts at 0 when the workspace is reset; this reproduces the
 * reference's np.random.rand stream when the buffer holds it.  With
 * draws == NULL each pair draws from Philox4x32-10 keyed by seed and
 * counted by (collision step, cell, pair rank). */
typedef struct {
  const double* draws;
  int64_t n_draws;
  uint64_t seed;
} lacmo_draws_t;

/* ---- library, workspace, status ------------------------------------------ */
int lacmo_abi_version(void);
/* Number of CUDA kernels this library has launched in this process. */
uint64_t lacmo_kernel_launches(void);
const char* lacmo_error_string(int status);
/* Bytes of device scratch the entry points below need for n SIPs and an
 * nx x nz grid (no allocation happens inside the library). */
size_t lacmo_workspace_bytes(int64_t n, int64_t nx, int64_t nz);
/* Zero the workspace: draw cursor, collision-step counter, flags. */
int lacmo_workspace_reset(void* ws, size_t ws_bytes, int64_t n, int64_t nx, int64_t nz,
                          void* stream);
/* Number of SIP sub-steps whose Newton ran in FP64 in mixed precision
 * (near-critical SIPs) since the workspace was reset (synchronises). */
int lacmo_read_fallbacks(const void* ws, int64_t n, int64_t nx, int64_t nz, uint64_t* count,
                         void* stream);
/* The Philox collision-step counter of a workspace: the counter word of the
 * draws (collision step, cell) that the next collision step uses.  Each
 * collision step advances it by one.  lacmo_workspace_reset sets it to 0; a
 * caller that rebuilds a workspace for every call (like a drop-in step
 * function called once per time step) carries it from one call to the next,
 * so that each call draws fresh uniforms as the reference's np.random.rand
 * does (collision/all_or_nothing.py:545).  _get synchronises the stream. */
int lacmo_get_collision_step(const void* ws, int64_t n, int64_t nx, int64_t nz, int64_t* step,
                             void* stream);
int lacmo_set_collision_step(void* ws, int64_t n, int64_t nx, int64_t nz, int64_t step,
                             void* stream);
/* Copy the device-side flags to *flags (synchronises the stream). */
int lacmo_read_flags(const void* ws, int64_t n, int64_t nx, int64_t nz, uint32_t* flags,
                     void* stream);

/* ---- launch shapes (autotuning) ----------------------------------------------
 * Knobs of the launch shapes of the hot kernels, process-wide: each knob takes
 * one of a fixed list of options (lacmo_tune_options writes them, the default
 * first, and returns their count); kernels read the knobs when they are
 * launched, so a CUDA graph keeps the shapes it was captured with.  The
 * results do not depend on the knobs (FP64 bit for bit), only the speed.
 * The reference runs on the CPU and has no counterpart; its per-seed process
 * launch (run_lacmo.sh) is what a batch replaces. */
#define LACMO_TUNE_PARTICLE_BLOCKS 0   /* mixed particle kernel, blocks per SM */
#define LACMO_TUNE_COLLISION_BLOCKS 1  /* collision kernels, blocks per SM     */
#define LACMO_TUNE_ORDER_CTAS 2        /* cell ordering, blocks per SM         */
int lacmo_tune_options(int knob, int* values, int max_values);
int lacmo_tune_set(int knob, int value);   /* LACMO_ERR_ARG for a value not listed */
int lacmo_tune_get(int knob);

/* ---- layout conversion ------------------------------------------------------ */
/* cells[2][n] int64 + active_ids[n] (uint8) -> cell[n] (file_handling.py
 * state layout; integration.py:509-550 cell convention). */
int lacmo_cells_import(const int64_t* cells, const uint8_t* active_ids, int32_t* cell,
                       int64_t n, int64_t nx, int64_t nz, void* stream);
/* cell[n] -> cells[2][n] int64 + active_ids[n]; fills rel_pos of active SIPs
 * from pos (integration.py:509-550) so the reference's rel_pos is complete. */
int lacmo_cells_export(const int32_t* cell, const double* pos, double* rel_pos,
                       int64_t* cells, uint8_t* active_ids, int64_t n, int64_t nx, int64_t nz,
                       double x_min, double z_min, double dx, double dz, void* stream);

/* ---- time integration --------------------------------------------------------- */
/* Prepare derived per-cell data and the cell binning from the current state.
 * Call after importing a state or changing it outside these entry points. */
int lacmo_prepare(const lacmo_sips_t* sips, const lacmo_grid_t* grid, const lacmo_params_t* prm,
                  void* ws, size_t ws_bytes, void* stream);
/* One advection step dt: replaces integration.py:1298 integrate_adv_step_np
 * (with integrate_subloop_n_steps_np :1095, propagate_particles_subloop_step
 * :944, propagate_grid_subloop_step :402, compute_divergence_upwind :150,
 * compute_relaxation_term :325 and the all-cells collision step
 * collision/all_or_nothing.py:754).  Requires lacmo_prepare() once before. */
int lacmo_integrate_adv_step(const lacmo_sips_t* sips, const lacmo_grid_t* grid,
                             const lacmo_params_t* prm, const lacmo_draws_t* draws, void* ws,
                             size_t ws_bytes, void* stream);
/* A CUDA graph of n_steps consecutive lacmo_integrate_adv_step calls with
 * fixed arguments, captured on `stream` (not the legacy default stream);
 * lacmo_plan_launch replays it.  All step-to-step state (SIPs, grid, draw
 * cursor, Philox step counter) lives in device memory, so replays continue
 * the time integration.  Not for host-side draw generation. */
typedef struct lacmo_plan lacmo_plan;
int lacmo_plan_create(const lacmo_sips_t* sips, const lacmo_grid_t* grid, const lacmo_params_t* prm,
                      const lacmo_draws_t* draws, void* ws, size_t ws_bytes, int n_steps,
                      void* stream, lacmo_plan** plan);
int lacmo_plan_launch(lacmo_plan* plan, void* stream);
int lacmo_plan_destroy(lacmo_plan* plan);
/* Kernel launches one replay of the plan performs (-1 on error). */
int64_t lacmo_plan_kernel_nodes(const lacmo_plan* plan);

/* One call of integrate_adv_step_np (integration.py:1298-1313) on host
 * arrays, in place, with the device buffers the caller keeps between calls:
 * copies the host arrays in (the `in` list), imports the cells (lacmo_cells_
 * import), clears the workspace, prepares (lacmo_prepare), sets the Philox
 * collision-step counter to col_step (when >= 0), advances one step (the
 * captured plan when given, else lacmo_integrate_adv_step), exports the
 * cells (lacmo_cells_export into cells_out / active_out), copies the `out`
 * list back to the host, stores the counter after the step in *col_step_out
 * (when given) and synchronises `stream`.  Host memory may be pageable.
 * copy_mode: LACMO_COPY_AUTO takes LACMO_COPY_KERNEL where the device reads
 * and writes pageable host memory directly (cudaDevAttrPageableMemoryAccess:
 * a Grace host's coherent NVLink-C2C link), else LACMO_COPY_ENGINE;
 * LACMO_COPY_ENGINE issues one cudaMemcpyAsync per entry; LACMO_COPY_KERNEL
 * moves every entry of a list in one kernel launch, asynchronously to the
 * host (LACMO_ERR_ARG where the device cannot).  The sips/grid/params/draws
 * structures name the device buffers. */
#define LACMO_COPY_AUTO 0
#define LACMO_COPY_ENGINE 1
#define LACMO_COPY_KERNEL 2
typedef struct {
  void* dst;
  const void* src;
  int64_t bytes;
} lacmo_copy_t;
typedef struct {
  const lacmo_copy_t* in;   /* host -> device, before the step */
  int32_t n_in;
  const lacmo_copy_t* out;  /* device -> host, after it         */
  int32_t n_out;
  const lacmo_sips_t* sips;
  const lacmo_grid_t* grid;
  const lacmo_params_t* prm;
  const lacmo_draws_t* draws;
  void* ws;
  size_t ws_bytes;
  const int64_t* cells_in;  /* device [2][n]: the reference's cells      */
  const uint8_t* active_in; /* device [n]: its active_ids as bytes       */
  int64_t* cells_out;       /* device [2][n], written by the export      */
  uint8_t* active_out;      /* device [n]                                */
  lacmo_plan* plan;         /* a plan of this state (one step), or NULL  */
  int64_t col_step;         /* collision-step counter to start from; -1: 0 after the clear */
  int64_t* col_step_out;    /* host: the counter after the step, or NULL */
  int32_t copy_mode;        /* LACMO_COPY_*                              */
} lacmo_dropin_t;
int lacmo_dropin_adv_step(const lacmo_dropin_t* call, void* stream);

/* Batched ensemble: M independent model states (members) advanced together,
 * each kernel launch covering all members (blockIdx.y = member).  The
 * reference runs one simulation per process (integration.py:1790-2066
 * simulate_interval / simulate); a batch is M such simulations with the same
 * parameters, grid shape and time step, different SIP counts and states, and
 * Philox collision draws keyed by each member's seed.  The caller owns the
 * member arrays and one workspace of lacmo_batch_workspace_bytes() bytes;
 * lacmo_batch_create zeroes it, uploads the member table (synchronously) and
 * returns a handle that refers to the caller's memory.  prms (optional, M
 * entries) supplies each member's relaxation profiles (integration.py:
 * 325-354 relaxes towards the member's own initial profiles); every other
 * parameter comes from the lacmo_params_t of the stepping calls. */
typedef struct lacmo_batch lacmo_batch;
size_t lacmo_batch_workspace_bytes(int M, const int64_t* n, int64_t nx, int64_t nz);
int lacmo_batch_create(int M, const lacmo_sips_t* sips, const lacmo_grid_t* grids,
                       const lacmo_params_t* prms, const uint64_t* seeds, void* ws,
                       size_t ws_bytes, lacmo_batch** batch);
/* lacmo_prepare for every member */
int lacmo_batch_prepare(lacmo_batch* batch, const lacmo_params_t* prm, void* stream);
/* one advection step of every member (lacmo_integrate_adv_step, Philox draws) */
int lacmo_batch_adv_step(lacmo_batch* batch, const lacmo_params_t* prm, void* stream);
/* A mixed-precision batch step does not bin its SIPs after its last sub-step
 * (the next step bins after its half-step move; water_removed is complete
 * all the same), so between steps a member's binning is empty; lacmo_batch_rebin bins every member's SIPs by their
 * current cells, for entry points that read a member's binning between steps
 * (lacmo_update_grid_r_l with lacmo_batch_member_workspace). */
int lacmo_batch_rebin(lacmo_batch* batch, void* stream);
/* a CUDA graph of n_steps batch advection steps (see lacmo_plan_create) */
int lacmo_batch_plan_create(lacmo_batch* batch, const lacmo_params_t* prm, int n_steps,
                            void* stream, lacmo_plan** plan);
/* one particle sub-step kernel of every member alone (no grid update, no
 * binning): for timing the fused particle pass; leaves the step incomplete */
int lacmo_batch_particles_only(lacmo_batch* batch, const lacmo_params_t* prm, void* stream);
/* member m's workspace slice, for lacmo_read_flags / lacmo_read_fallbacks */
int lacmo_batch_member_workspace(const lacmo_batch* batch, int m, void** ws, size_t* ws_bytes);
int lacmo_batch_destroy(lacmo_batch* batch);
/* Phases of lacmo_integrate_adv_step, for callers that run the collision
 * steps themselves (e.g. to draw each step's uniforms from a host generator
 * exactly as the reference does):
 * _begin: x_{n+1/2}, re-index and the first-half advective + relaxation
 *   increments kept in the workspace (integration.py:1474-1508);
 * _second_half: the second-half increments (integration.py:1536-1561);
 * _substep: one particle + grid sub-step with those increments; positions
 *   move by dt_sub_pos, T_p is written when write_T_p != 0
 *   (integration.py:1265-1281, 1593-1610). */
int lacmo_adv_step_begin(const lacmo_sips_t* sips, const lacmo_grid_t* grid,
                         const lacmo_params_t* prm, void* ws, size_t ws_bytes, void* stream);
int lacmo_adv_step_second_half(const lacmo_sips_t* sips, const lacmo_grid_t* grid,
                               const lacmo_params_t* prm, void* ws, size_t ws_bytes,
                               void* stream);
int lacmo_adv_substep(const lacmo_sips_t* sips, const lacmo_grid_t* grid,
                      const lacmo_params_t* prm, double dt_sub_pos, int write_T_p, void* ws,
                      size_t ws_bytes, void* stream);
/* The two halves of a particle sub-step, for callers that time or schedule
 * them separately: the fused per-SIP kernel (condensation, drag, position,
 * re-index; it also counts SIPs per new cell), and the cell binning that
 * folds the ground-removal list into water_removed and sorts the SIPs by
 * (cell, ID).  lacmo_bin must follow lacmo_particles_only before any other
 * entry point uses the binning. */
int lacmo_particles_only(const lacmo_sips_t* sips, const lacmo_grid_t* grid,
                         const lacmo_params_t* prm, double dt_sub, double dt_sub_pos, void* ws,
                         size_t ws_bytes, void* stream);
int lacmo_bin(const lacmo_sips_t* sips, const lacmo_grid_t* grid, void* ws, size_t ws_bytes,
              void* stream);
/* One particle sub-step: replaces integration.py:944
 * propagate_particles_subloop_step_np (T_p, Newton condensation with the
 * per-cell delta_m_l, drag, position, ground removal, cell re-index). */
int lacmo_propagate_particles_subloop_step(const lacmo_sips_t* sips, const lacmo_grid_t* grid,
                                           const lacmo_params_t* prm, double dt_sub,
                                           double dt_sub_pos, void* ws, size_t ws_bytes,
                                           void* stream);
/* One grid sub-step: replaces integration.py:402 propagate_grid_subloop_step_np
 * (and update_material_properties :359). */
int lacmo_propagate_grid_subloop_step(const lacmo_grid_t* grid, const double* delta_Theta_ad,
                                      const double* delta_r_v_ad, const double* delta_m_l,
                                      void* stream);
/* Replaces integration.py:150 compute_divergence_upwind_np; bc 0 periodic,
 * 1 solid.  out[nx][nz]. */
int lacmo_divergence_upwind(const double* field, const double* flux, int64_t nx, int64_t nz,
                            double dx, double dz, int bc_x, int bc_z, double* out, void* stream);
/* Replaces integration.py:325 compute_relaxation_term. out[nz]. */
int lacmo_relaxation_term(const double* field, int64_t nx, int64_t nz, const double* profile0,
                          const double* t_relax, double dt, double* out, void* stream);
/* Replaces grid.py:370 update_grid_r_l_np (uses the current cell binning). */
int lacmo_update_grid_r_l(const lacmo_sips_t* sips, const lacmo_grid_t* grid, void* ws,
                          size_t ws_bytes, void* stream);

/* ---- diagnostics ---------------------------------------------------------------- */
/* Per-cell sums over the SIPs in ascending ID order, bit for bit the
 * reference's loops.  cell: the int32 cell index of lacmo_cells_import (a SIP
 * removed at the ground, -1 - i, counts in cell (i, nz - 1) where the
 * reference's row index -1 lands).  ws: a workspace of
 * lacmo_workspace_bytes(n, nx, nz), whose cell binning the call replaces.
 * out[nx][nz].
 * kind 0 replaces evaluation.py:93 update_mixing_ratio (sum m_w xi over the
 * masked SIPs, times 1E-18 mass_dry_inv); kind 1 replaces evaluation.py:136
 * update_number_concentration_per_dry_mass (sum xi, times mass_dry_inv). */
int lacmo_update_cell_sum(int kind, const double* m_w, const double* xi, const int32_t* cell,
                          const uint8_t* mask, const double* mass_dry_inv, int64_t n, int64_t nx,
                          int64_t nz, double* out, void* ws, size_t ws_bytes, void* stream);
/* Replaces evaluation.py:1393 compute_moment_R_grid: sum over the active SIPs
 * of xi R_p^order (R_p^order by repeated squaring, as Numba's integer
 * power), divided by V0. */
int lacmo_compute_moment_R_grid(int64_t order, const double* R_p, const double* xi, double V0,
                                const int32_t* cell, int64_t n, int64_t nx, int64_t nz,
                                double* out, void* ws, size_t ws_bytes, void* stream);

/* Replaces microphysics.py:208-266 compute_R_p_w_s_rho_p (AS or NaCl): radius
 * (um), solute mass fraction and density (kg/m^3) per SIP; w_s and rho_p may
 * be null. */
int lacmo_compute_R_p_w_s_rho_p(int solute, int64_t n, const double* m_w, const double* m_s,
                                const double* T_p, double* R_p, double* w_s, double* rho_p,
                                void* stream);
/* Replaces microphysics.py:83-100 compute_radius_from_mass for one density
 * (e.g. dry radii from solute masses). */
int lacmo_radius_from_mass(int64_t n, const double* m, double rho, double* R, void* stream);
/* Weighted histogram with numpy.histogram's bins (evaluation.py:1172-1390
 * size spectra): edges [nbins + 1] ascending, bins [e_b, e_b+1) with the last
 * one closed; w null counts 1 per value; out [nbins] is overwritten. */
int lacmo_histogram_weighted(const double* x, const double* w, int64_t n, const double* edges,
                             int64_t nbins, double* out, void* stream);

/* ---- initialisation (init.py:439-1236) ------------------------------------------
 * SinSIP mass ensembles (generation_SIP_ensemble.py:147-384) of n_seg
 * (level, cell, mode) segments at once: segment s of mode seg_mode[s] takes
 * its bins' uniforms from rnd + rnd_off[s] (l_max draws, then l_max more
 * with the weak threshold, weak != 0), mode_par = [mu_m_log][sigma_m_log]
 * [bin factor][m_low] (n_modes each) then sqrt(2 pi); the kept bins go to the
 * front of masses / weights [n_seg][lmax_cap], their number to count[n_seg]. */
int lacmo_sinsip_generate(const double* rnd, const int64_t* rnd_off, const int32_t* seg_mode,
                          int64_t n_seg, int n_modes, const double* mode_par,
                          const int32_t* l_max, double eta, int weak, int64_t lmax_cap,
                          double* masses, double* weights, int32_t* count, void* stream);
/* The kept bins of every segment concatenated from off[s] (exclusive sums of
 * count), multiplicities = weights * seg_scale[s] (real particles per cell). */
int lacmo_sinsip_gather(const double* masses, const double* weights, const int32_t* count,
                        const int64_t* off, int64_t n_seg, int64_t lmax_cap,
                        const double* seg_scale, double* m_out, double* xi_out, int64_t n_out,
                        void* stream);
/* Replaces microphysics.py:686-785 compute_initial_mass_fraction_solute_m_s
 * (AS or NaCl, scipy fminbound / brentq per SIP): the solute mass fraction in
 * equilibrium with S_amb at T_amb, the activation maximum where S_amb is
 * above it, w_s_max where S_amb is below the efflorescence saturation. */
int lacmo_init_mass_fraction(int solute, int64_t n, const double* m_s, double S_amb,
                             double T_amb, double volume_to_radius, double w_s_max,
                             double solubility, double* w_s, void* stream);
/* One saturation-adjustment iteration of a level (init.py:887-960): the
 * implicit Newton condensation step dt (no_iter evaluations) of every SIP at
 * the level's T and p and its cell's capped S and e_s; the SIPs of cell c are
 * off[c] .. off[c + 1] - 1 (clipped to the n_sips of m_w, m_s, xi); m_w is
 * updated; dml_cell / mwxi_cell [cells] receive the cell sums of dm * xi and
 * m_w * xi (1e-18 kg). */
int lacmo_saturation_adjust_level(int solute, int64_t cells, const int64_t* off, int64_t n_sips,
                                  double* m_w, const double* m_s, const double* xi,
                                  const double* S_cap,
                                  const double* e_s, double T, double p, double L_v, double K,
                                  double D_v, double dt, int no_iter, double* dml_cell,
                                  double* mwxi_cell, void* stream);

/* ---- collisions ------------------------------------------------------------------ */
/* All cells of the 2-D grid: replaces collision/all_or_nothing.py:754
 * collision_step_Ecol_grid_R_all_cells_2D_multicomp_np (and :498 / :637 per
 * cell).  Uses the binning of the last lacmo_prepare / sub-step.  Injected
 * draws are read from the start of the buffer (it must hold the count from
 * lacmo_collision_pair_count). */
int lacmo_collision_step_cells(const lacmo_sips_t* sips, const lacmo_grid_t* grid,
                               const lacmo_params_t* prm, const lacmo_draws_t* draws, void* ws,
                               size_t ws_bytes, void* stream);
/* All-cells collision step that allocates nothing.  This entry point has no
 * counterpart in the reference; it exists for callers that cannot allocate
 * device memory at the time they collide (code inside another framework's
 * memory pool or under a fixed memory budget, plugin hosts that forbid
 * cudaMalloc after start-up).  It does the work of lacmo_collision_step_cells
 * from the SIP cell indices alone (binning included), with its scratch in a
 * fixed array inside the library (about 28 MB of device memory, held by every
 * GPU that loads the library until the process exits) instead of a
 * workspace.  The caller still passes all inputs and outputs: xi, m_w, m_s
 * are updated in place, vel is [2][n], grid_T is the [nx][nz] temperature,
 * cell is the int32 cell index of lacmo_cells_import.  Limits:
 * n <= LACMO_NOALLOC_MAX_SIPS and nx*nz <= LACMO_NOALLOC_MAX_CELLS, else
 * LACMO_ERR_CAPACITY.  Injected draws are read from the start of the buffer;
 * Philox draws use `step` as the collision-step counter.  The first call on a
 * device loads the library's module there when it looks up the array's
 * device address (every call looks it up, with the caller's device current),
 * so make that first call before any stream capture.  All calls share the one
 * array and each call clears what must start at zero: calls whose work
 * overlaps on the GPU race and must be serialised.  SIPs whose cell index is
 * >= nx*nz are left out of the step (LACMO_FLAG_CELL_RANGE).  The step's
 * condition flags and pair count stay in the array until the next call:
 * read them with lacmo_noalloc_status.  A step whose injected buffer holds
 * fewer draws than the step's pair count is skipped as a whole (the state is
 * unchanged, LACMO_FLAG_DRAWS_SHORT), and the pair count it reports sizes the
 * buffer for the repeated call. */
#define LACMO_NOALLOC_MAX_SIPS 524288
#define LACMO_NOALLOC_MAX_CELLS 16384
int lacmo_collision_step_cells_noalloc(double* xi, double* m_w, double* m_s, const double* vel,
                                       const double* grid_T, const int32_t* cell, int64_t n,
                                       int64_t nx, int64_t nz, const lacmo_params_t* prm,
                                       const lacmo_draws_t* draws, uint64_t step,
                                       int64_t* no_cols, void* stream);
/* Condition flags (LACMO_FLAG_*) and pair count of the last
 * lacmo_collision_step_cells_noalloc call on the current device, read from
 * the library's fixed array into host memory (synchronises the stream; either
 * pointer may be null).  This reader has no counterpart in the reference. */
int lacmo_noalloc_status(uint32_t* flags, int64_t* pairs, void* stream);
/* Number of pair draws the next all-cells collision step consumes
 * (synchronises the stream; used to size an injected draw buffer). */
int lacmo_collision_pair_count(const void* ws, int64_t n, int64_t nx, int64_t nz,
                               int64_t* pairs, void* stream);
/* Box model, Golovin kernel: replaces collision/all_or_nothing.py:109
 * collision_step_Golovin_np.  rnd: n(n-1)/2 draws or NULL for Philox
 * (seed, step).  n <= LACMO_BOX_MAX_SIPS. */
#define LACMO_BOX_MAX_SIPS 8192
#define LACMO_ECOL_BOX_MAX_SIPS 4096
int lacmo_collision_step_golovin(double* xis, double* masses, int64_t n, double dt_over_dV,
                                 int64_t* no_cols, const double* rnd, uint64_t seed,
                                 uint64_t step, void* stream);
/* Box model, kernel K(m1, m2) tabulated on a logarithmic mass grid
 * (kernel_grid[nb][nb]; bin int((log m - m_low_log) / bin_factor_m_log + 0.5)
 * clamped): replaces collision/all_or_nothing.py:392
 * collision_step_kernel_grid_m_np.  n <= LACMO_BOX_MAX_SIPS. */
int lacmo_collision_step_kernel_grid_m(double* xis, double* masses, int64_t n, double dt_over_dV,
                                       const double* kernel_grid, int64_t no_kernel_bins,
                                       double m_kernel_low_log, double bin_factor_m_log,
                                       int64_t* no_cols, const double* rnd, uint64_t seed,
                                       uint64_t step, void* stream);
/* Box model, E_col(R1, R2) table and 1-D velocities: replaces
 * collision/all_or_nothing.py:269 collision_step_Ecol_grid_R_np. */
int lacmo_collision_step_ecol_grid_r_box(double* xis, double* masses, double* radii,
                                         const double* vel, const double* mass_densities,
                                         int64_t n, double dt_over_dV, const double* E_col_grid,
                                         int64_t no_kernel_bins, double R_kernel_low_log,
                                         double bin_factor_R_log, int64_t* no_cols,
                                         const double* rnd, uint64_t seed, uint64_t step,
                                         void* stream);
/* Beard terminal velocity: replaces collision/kernel.py:193 update_velocity_Beard. */
int lacmo_update_velocity_beard(double* vel, const double* R, int64_t n, void* stream);

/* ---- elementwise microphysics (unit-level parity) ------------------------------------ */
/* microphysics.py:1359 / :1239 compute_mass_rate_and_derivative_{AS,NaCl}_np */
int lacmo_mass_rate_and_derivative(int solute, int64_t n, const double* m_w, const double* m_s,
                                   const double* w_s, const double* R_p, const double* T_p,
                                   const double* rho_p, const double* T_amb, const double* p_amb,
                                   const double* S_amb, const double* e_s_amb, const double* L_v,
                                   const double* K, const double* D_v, const double* sigma_p,
                                   double* gamma, double* dgamma_dm, void* stream);
/* integration.py:728 compute_dml_and_gamma_impl_Newton_full_np */
int lacmo_newton_full(int solute, int64_t n, double dt_sub, int no_iter, const double* m_w,
                      const double* m_s, const double* w_s, const double* R_p, const double* T_p,
                      const double* rho_p, const double* T_amb, const double* p_amb,
                      const double* S_amb, const double* e_s_amb, const double* L_v,
                      const double* K, const double* D_v, const double* sigma_p, double* dm,
                      double* gamma0, void* stream);
/* grid.py:257 interpolate_velocity_from_cell_bilinear (cells as cell[n]) */
int lacmo_interpolate_velocity(const int32_t* cell, const double* rel_pos, const double* grid_vel,
                               int64_t n, int64_t nx, int64_t nz, double* out, void* stream);
/* Correctly-rounded radius and kernel bin of the collision path
 * (microphysics.py:83-100, collision/all_or_nothing.py:35-67). */
int lacmo_radius_and_bin(const double* m, const double* rho, int64_t n, double R_kernel_low_log,
                         double bin_factor_R_log, int64_t no_kernel_bins, double* R,
                         int64_t* bin, void* stream);

/* Event log of the all-cells collision steps of single states (not batches),
 * for the adjoint's replay of collisions as recorded events.  While set,
 * every such step appends one 32-byte record per collection to events[]:
 * int32 imin, imax (the SIPs of smaller and larger multiplicity), int32 kind
 * (0 ordinary collection, 1 equal-multiplicity split, 2 multiple collection),
 * int32 0, double a, b (kind 1: the multiplicities of imin and imax before;
 * kind 2: a = p_crit).  *count (device) counts the records, also those past
 * capacity, which are not written; a cell's records appear in its sequential
 * order.  events = null switches the log off.  Process-wide. */
int lacmo_collision_event_log(void* events, int64_t capacity, unsigned long long* count);

/* ---- adjoint of the condensation sub-steps (k_adjoint.cu) ----
 * The differentiated model: the SIPs' cells per sub-step and their
 * multiplicities are recorded events (SIP motion, ground removal and cell
 * re-indexing of integration.py:509-719 enter only through the piecewise
 * constant cell index, whose derivative is zero); each sub-step runs the
 * condensation step of integration.py:840-940 for every SIP with cell >= 0,
 * then updates Theta and r_v of the cells as integration.py:402-438 does, the
 * ambient terms following from Theta and r_v.  Hygroscopicity kappa scales the
 * ammonium-sulfate water activity, a_w = 1 + (kappa / 0.6)(a_w_AS(w_s) - 1);
 * kappa = 0.6 is the reference.
 * Arrays are device pointers: m_w, m_s, xi [n]; cell [n_sub][n] with row
 * stride cell_stride (0: the same cells every sub-step); Theta, r_v, rho_d,
 * mass_dry_inv [C]; dTh, drv [C] the increments every sub-step adds (null =
 * 0); dml [C] scratch.  no_iter > 0: the condensation step is the time step's
 * own map of no_iter damped Newton evaluations (integration.py:786-836),
 * differentiated exactly; no_iter = 0: the implicit Euler step solved to
 * convergence, differentiated through the implicit-function theorem.
 * lacmo_adj_forward advances n_sub sub-steps in place and, when tape_m
 * ([n_sub + 1][n]) and tape_c ([n_sub][2][C]) are given, records the states
 * for lacmo_adj_backward.  lacmo_adj_backward turns the adjoints of the final
 * state (lam_m [n], lam_Th, lam_rv [C]) into those of the initial state,
 * accumulating d/d m_s into grad_ms [n], d/d kappa into grad_kappa [1] and,
 * when lam_inc ([2][C]) is given, the adjoints of (dTh, drv) into lam_inc;
 * lam_dml [C] is scratch. */
int lacmo_adj_forward(int64_t n, int64_t C, double* m_w, const double* m_s, const double* xi,
                      const int32_t* cell, int64_t cell_stride, double* Th, double* r_v,
                      const double* rho_d, const double* mass_dry_inv, const double* dTh,
                      const double* drv, double* dml, double dt_sub, double kappa, double p_ref,
                      double V, int n_sub, int no_iter, double* tape_m, double* tape_c,
                      void* stream);
int lacmo_adj_backward(int64_t n, int64_t C, const double* m_s, const double* xi,
                       const int32_t* cell, int64_t cell_stride, const double* rho_d,
                       const double* mass_dry_inv, const double* dTh, const double* drv,
                       double* dml, double dt_sub, double kappa, double p_ref, double V,
                       int n_sub, int no_iter, const double* tape_m, const double* tape_c,
                       double* lam_m, double* lam_Th, double* lam_rv, double* lam_dml,
                       double* grad_ms, double* grad_kappa, double* lam_inc, void* stream);
/* The increments a half advection step adds every sub-step (integration.py:
 * 1483-1508 for second = 0; 1536-1561 for second = 1, where inc_Th, inc_rv
 * hold the first half's increments on entry): the upwind divergence of the
 * Hundsdorfer et al. (1995) scheme of Theta and r_v with the mass flux
 * ([2][nx+1][nz+1], x periodic, z solid) times rho_dry_inv, and, when t_relax
 * [nz] is given, the relaxation to the profiles prof_Th, prof_rv [nz].
 * lacmo_adj_increments_vjp adds factor * J^T lam_inc ([2][C]) to lam_Th,
 * lam_rv, J the Jacobian of the first-half increments at (Theta, r_v), and
 * factor * lam_inc . (advective increments) / flux_scale to grad_s [1], the
 * derivative by a common factor of the mass flux when flux is flux_scale
 * times the unscaled one. */
int lacmo_adj_increments(const double* Th, const double* r_v, const double* rho_dry_inv,
                         const double* flux, int64_t nx, int64_t nz, double dx, double dz,
                         double dt_sub, const double* prof_Th, const double* prof_rv,
                         const double* t_relax, int second, double* inc_Th, double* inc_rv,
                         void* stream);
int lacmo_adj_increments_vjp(const double* Th, const double* r_v, const double* rho_dry_inv,
                             const double* flux, int64_t nx, int64_t nz, double dx, double dz,
                             double dt_sub, const double* prof_Th, const double* prof_rv,
                             const double* t_relax, double factor, double flux_scale,
                             const double* lam_inc, double* lam_Th, double* lam_rv,
                             double* grad_s, void* stream);
/* Collisions as recorded events (records of lacmo_collision_event_log,
 * grouped: the records of group g are events[off[g] .. off[g + 1] - 1] in
 * their sequential order, groups independent, e.g. one per cell).
 * lacmo_adj_collisions_forward replays them on m_w, m_s, xi as the collision
 * step applies them (collision/all_or_nothing.py:577-633, kind 2 with the
 * recorded p_crit); lacmo_adj_collisions_backward maps the adjoints of m_w
 * and m_s after the events to those before (the transposed linear maps, in
 * reverse order; p_crit and the split's multiplicities held fixed). */
int lacmo_adj_collisions_forward(const void* events, const int64_t* off, int64_t n_groups,
                                 double* m_w, double* m_s, double* xi, void* stream);
int lacmo_adj_collisions_backward(const void* events, const int64_t* off, int64_t n_groups,
                                  double* lam_w, double* lam_s, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LACMO_GB300_H */
