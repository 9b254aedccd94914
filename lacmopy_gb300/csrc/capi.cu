// extern "C" entry points: argument checks, workspace carving and the
// launch sequence of one advection step (integration.py:1298-1611).
#include <cuda_runtime.h>
#include <string.h>

#include <atomic>
#include <vector>

#include "lacmo_internal.cuh"

namespace lacmo {

static std::atomic<uint64_t> g_launches{0};
void note_launches(int k) { g_launches.fetch_add((uint64_t)k, std::memory_order_relaxed); }

// Launch-shape knobs (process-wide): the options each knob may take, the
// first listed is the default.
static const int k_tune_options[TUNE_KNOBS][4] = {
    {6, 5, 8, 0},    // mixed particle kernel: resident blocks per SM (register budget)
    {3, 2, 4, 0},    // collision kernels: resident blocks per SM
    {16, 8, 4, 0},   // cell ordering: blocks per SM
};
static std::atomic<int> g_tune[TUNE_KNOBS] = {{6}, {3}, {16}};
int tune_value(int knob) { return g_tune[knob].load(std::memory_order_relaxed); }

static inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

struct WsPlan {
  size_t off[32];
  size_t total;
};

static WsPlan ws_plan(int64_t n, int64_t nx, int64_t nz) {
  const size_t C = (size_t)(nx * nz), N = (size_t)(n > 0 ? n : 1);
  const size_t sizes[] = {
      4 * C,           // counts
      4 * (C + 1),     // start
      8 * (C + 1),     // draw_off
      4 * N,           // perm
      4 * N,           // rank
      8 * N,           // dmxi
      4 * N,           // rm_id
      8 * N,           // rm_val
      8 * cell_records_offset((int64_t)C) + 16 * CELL_REC * C,  // aux: 6 doubles, records
      8 * C,           // dTh
      8 * C,           // drv
      8 * C,           // div
      8 * 2 * (size_t)nz,  // relax
      8 * N,           // colR
      8 * N,           // colrho
      4 * N,           // colk
      64,              // scalars
      0,               // (unused)
      4 * (size_t)LACMO_MAX_KERNEL_BINS * (LACMO_MAX_KERNEL_BINS + 1),  // Ef, row maxima
      4 * C,           // cell_order
      24 * N,          // gcopy
      32 * (N / 32 + C + 1),  // gstats
  };
  WsPlan p;
  size_t o = 0;
  for (size_t k = 0; k < sizeof(sizes) / sizeof(sizes[0]); ++k) {
    p.off[k] = o;
    o += al(sizes[k]);
  }
  p.total = o;
  return p;
}

size_t ws_bytes(int64_t n, int64_t nx, int64_t nz) { return ws_plan(n, nx, nz).total; }

bool ws_carve(void* base, size_t bytes, int64_t n, int64_t nx, int64_t nz, Ws* w) {
  WsPlan p = ws_plan(n, nx, nz);
  if (!base || bytes < p.total) return false;
  char* b = (char*)base;
  w->counts = (int32_t*)(b + p.off[0]);
  w->start = (int32_t*)(b + p.off[1]);
  w->draw_off = (int64_t*)(b + p.off[2]);
  w->perm = (int32_t*)(b + p.off[3]);
  w->rank = (int32_t*)(b + p.off[4]);
  w->dmxi = (double*)(b + p.off[5]);
  w->rm_id = (int32_t*)(b + p.off[6]);
  w->rm_val = (double*)(b + p.off[7]);
  w->aux = (double*)(b + p.off[8]);
  w->dTh = (double*)(b + p.off[9]);
  w->drv = (double*)(b + p.off[10]);
  w->div = (double*)(b + p.off[11]);
  w->relax = (double*)(b + p.off[12]);
  w->colR = (double*)(b + p.off[13]);
  w->colrho = (double*)(b + p.off[14]);
  w->colk = (int32_t*)(b + p.off[15]);
  char* sc = b + p.off[16];
  w->flags = (uint32_t*)sc;
  w->rm_count = (int32_t*)(sc + 4);
  w->cursor = (int64_t*)(sc + 8);
  w->col_step = (int64_t*)(sc + 16);
  w->total_pairs = (int64_t*)(sc + 24);
  w->nfb = (unsigned long long*)(sc + 32);
  w->Ef = (float*)(b + p.off[18]);
  w->cell_order = (int32_t*)(b + p.off[19]);
  w->cell_ctr = (int32_t*)(sc + 40);
  w->fb_count = (int32_t*)(sc + 44);
  w->fb_done = (int32_t*)(sc + 48);
  w->gcopy = (float*)(b + p.off[20]);
  w->gstats = (float*)(b + p.off[21]);
  return true;
}

static bool sips_ok(const lacmo_sips_t* s) {
  return s && s->n > 0 && s->n < (int64_t)0x7fffffff && s->pos && s->vel && s->rel_pos && s->m_w &&
         s->m_s && s->xi && s->T_p && s->cell && s->water_removed && s->no_cols;
}
static bool grid_ok(const lacmo_grid_t* g) {
  return g && g->nx > 0 && g->nz > 0 && g->nx * g->nz < (int64_t)0x7fffffff && g->scalar_fields &&
         g->mat_prop && g->velocity && g->mass_flux_air_dry && g->delta_m_l && g->dx > 0 &&
         g->dz > 0;
}
static bool prm_ok(const lacmo_params_t* p) {
  return p && p->no_iter_impl_mass >= 1 && (p->solute == 0 || p->solute == 1) &&
         (p->precision == LACMO_PRECISION_FP64 || p->precision == LACMO_PRECISION_MIXED) &&
         p->scale_dt_cond >= 1 && p->no_col_per_adv >= 1 &&
         (p->E_col_grid == nullptr || p->no_kernel_bins > 0);
}

#define LCHK(x)                                   \
  do {                                            \
    if ((x) != cudaSuccess) return LACMO_ERR_CUDA; \
  } while (0)

Member make_member(const lacmo_sips_t& sp, const lacmo_grid_t& g, const Ws& w, uint64_t seed) {
  Member m;
  memset(&m, 0, sizeof(m));
  m.sp = sp; m.g = g; m.w = w; m.seed = seed;
  m.z_cap = g.z_max * 0.999999;
  m.inv_dx = 1.0 / g.dx; m.inv_dz = 1.0 / g.dz;
  m.x_minf = (float)g.x_min; m.x_maxf = (float)g.x_max; m.z_minf = (float)g.z_min;
  m.z_capf = (float)m.z_cap; m.inv_dxf = (float)m.inv_dx; m.inv_dzf = (float)m.inv_dz;
  return m;
}

Bt single(const lacmo_sips_t& sp, const lacmo_grid_t& g, const Ws& w, uint64_t seed) {
  Bt B;
  B.M = 1; B.dev = nullptr; B.one = make_member(sp, g, w, seed);
  B.n_max = sp.n; B.nx = g.nx; B.nz = g.nz;
  return B;
}

// integration.py:1095-1294
static int subloop(const Bt& B, const lacmo_params_t& p, const lacmo_draws_t& d, int no_cond,
                   int no_col, cudaStream_t s) {
  const bool col = p.act_collisions != 0;
  if (col && no_col == 1) LCHK(launch_collide_cells(B, p, d, s));
  for (int k = 0; k < no_cond; ++k) {
    if (col && no_col > 1) LCHK(launch_collide_cells(B, p, d, s));
    LCHK(launch_particles(B, p, p.dt_sub, p.dt_sub, false, s));
    LCHK(launch_cell_update(B, true, s));
    LCHK(launch_bin(B, s));
  }
  if (col && no_col > no_cond) LCHK(launch_collide_cells(B, p, d, s));
  return LACMO_OK;
}

// Mixed precision sub-loop: the particle sub-steps skip the cell binning
// unless a collision step follows before the next position update.
static int subloop_mixed(const Bt& B, const lacmo_params_t& p, const lacmo_draws_t& d, int no_cond,
                         int no_col, bool bin_at_end, cudaStream_t s) {
  const bool col = p.act_collisions != 0;
  if (col && no_col == 1) LCHK(launch_collide_cells(B, p, d, s));
  for (int k = 0; k < no_cond; ++k) {
    if (col && no_col > 1) LCHK(launch_collide_cells(B, p, d, s));
    const bool bin = (col && no_col > 1) || (k == no_cond - 1 && bin_at_end);
    LCHK(launch_particles_mixed(B, p, p.dt_sub, p.dt_sub, false, bin, s));
    LCHK(launch_grid_acc(B, s));
    if (bin) LCHK(launch_bin(B, s));
  }
  if (col && no_col > no_cond) LCHK(launch_collide_cells(B, p, d, s));
  return LACMO_OK;
}

// keep_binning: bin the SIPs after the step's last sub-step (single states,
// whose entry points between steps read the binning); otherwise (mixed
// batches) the binning is left empty (launch_fold_removals: the scan over
// zero counts): the next step bins after its half-step move anyway, and the
// batch's between-step entry points rebin first (lacmo_batch_rebin)
static int adv_step_mixed(const Bt& B, const lacmo_params_t& p, const lacmo_draws_t& d,
                          cudaStream_t s, bool keep_binning) {
  LCHK(launch_wind_float(B, s));
  LCHK(launch_move_mixed(B, p.dt_sub_half, s));
  LCHK(launch_bin(B, s));
  LCHK(launch_advection(B, p, false, s));
  const int nc1 = p.no_col_per_adv == 1 ? 0 : (p.no_col_per_adv == 2 ? 1 : p.scale_dt_cond);
  const int nc2 = (p.no_col_per_adv == 1 || p.no_col_per_adv == 2) ? 1 : p.scale_dt_cond;
  int rc = subloop_mixed(B, p, d, p.scale_dt_cond, nc1, p.act_collisions && nc2 >= 1, s);
  if (rc) return rc;
  LCHK(launch_advection(B, p, true, s));
  rc = subloop_mixed(B, p, d, p.scale_dt_cond - 1, nc2, false, s);
  if (rc) return rc;
  // last sub-step; the binning afterwards keeps it valid for the entry points
  // that use it between advection steps
  LCHK(launch_particles_mixed(B, p, p.dt_sub, p.dt_sub_half, true, keep_binning, s));
  LCHK(launch_grid_acc(B, s));
  LCHK(keep_binning ? launch_bin(B, s) : launch_fold_removals(B, s));
  return LACMO_OK;
}

static int adv_step(const Bt& B, const lacmo_params_t& p, const lacmo_draws_t& d, cudaStream_t s,
                    bool keep_binning = true) {
  if (p.precision == LACMO_PRECISION_MIXED) return adv_step_mixed(B, p, d, s, keep_binning);
  // b) x_{n+1/2} (integration.py:1474-1481)
  LCHK(launch_move(B, p.dt_sub_half, s));
  LCHK(launch_bin(B, s));
  // c) advective increments (+ relaxation)
  LCHK(launch_advection(B, p, false, s));
  int no_col = p.no_col_per_adv == 1 ? 0 : (p.no_col_per_adv == 2 ? 1 : p.scale_dt_cond);
  int rc = subloop(B, p, d, p.scale_dt_cond, no_col, s);
  if (rc) return rc;
  // e) second-half increments
  LCHK(launch_advection(B, p, true, s));
  no_col = (p.no_col_per_adv == 1 || p.no_col_per_adv == 2) ? 1 : p.scale_dt_cond;
  rc = subloop(B, p, d, p.scale_dt_cond - 1, no_col, s);
  if (rc) return rc;
  // last sub-step: positions move by dt_sub/2 (integration.py:1593-1610)
  LCHK(launch_particles(B, p, p.dt_sub, p.dt_sub_half, true, s));
  LCHK(launch_cell_update(B, true, s));
  LCHK(launch_bin(B, s));   // the FP64 path counts cells in every sub-step
  return LACMO_OK;
}

// capture n_steps advection steps of B into an executable graph
static int capture_plan(const Bt& B, const lacmo_params_t& p, const lacmo_draws_t& d, int n_steps,
                        cudaStream_t s, cudaGraph_t* graph_out, cudaGraphExec_t* exec_out,
                        bool keep_binning = true) {
  if (s == nullptr) return LACMO_ERR_ARG;  // the legacy default stream cannot be captured
  LCHK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = LACMO_OK;
  for (int k = 0; k < n_steps && rc == LACMO_OK; ++k) rc = adv_step(B, p, d, s, keep_binning);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (rc != LACMO_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return rc != LACMO_OK ? rc : LACMO_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
    cudaGraphDestroy(graph);
    return LACMO_ERR_CUDA;
  }
  *graph_out = graph;
  *exec_out = exec;
  return LACMO_OK;
}

}  // namespace lacmo

using namespace lacmo;

extern "C" {

int lacmo_abi_version(void) { return LACMO_ABI_VERSION; }

int lacmo_tune_options(int knob, int* values, int max_values) {
  if (knob < 0 || knob >= TUNE_KNOBS) return LACMO_ERR_ARG;
  int n = 0;
  while (n < 4 && k_tune_options[knob][n] > 0) {
    if (values && n < max_values) values[n] = k_tune_options[knob][n];
    ++n;
  }
  return n;
}

int lacmo_tune_set(int knob, int value) {
  if (knob < 0 || knob >= TUNE_KNOBS) return LACMO_ERR_ARG;
  for (int q = 0; q < 4 && k_tune_options[knob][q] > 0; ++q)
    if (k_tune_options[knob][q] == value) {
      g_tune[knob].store(value, std::memory_order_relaxed);
      return LACMO_OK;
    }
  return LACMO_ERR_ARG;
}

int lacmo_tune_get(int knob) {
  if (knob < 0 || knob >= TUNE_KNOBS) return LACMO_ERR_ARG;
  return tune_value(knob);
}

uint64_t lacmo_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int lacmo_particles_only(const lacmo_sips_t* sp, const lacmo_grid_t* g, const lacmo_params_t* p,
                         double dt_sub, double dt_sub_pos, void* ws, size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  LCHK(launch_particles(single(*sp, *g, w, 0), *p, dt_sub, dt_sub_pos, true,
                        (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_bin(const lacmo_sips_t* sp, const lacmo_grid_t* g, void* ws, size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  LCHK(launch_bin(single(*sp, *g, w, 0), (cudaStream_t)stream));
  return LACMO_OK;
}

const char* lacmo_error_string(int status) {
  switch (status) {
    case LACMO_OK: return "ok";
    case LACMO_ERR_ARG: return "invalid argument";
    case LACMO_ERR_CUDA: return "CUDA runtime error";
    case LACMO_ERR_DRAWS: return "injected draw buffer too short";
    case LACMO_ERR_WORKSPACE: return "workspace missing or too small";
    case LACMO_ERR_CAPACITY: return "size above the fixed capacity";
    default: return "unknown status";
  }
}

size_t lacmo_workspace_bytes(int64_t n, int64_t nx, int64_t nz) {
  if (n < 0 || nx <= 0 || nz <= 0) return 0;
  return ws_bytes(n, nx, nz);
}

int lacmo_workspace_reset(void* ws, size_t bytes, int64_t n, int64_t nx, int64_t nz, void* stream) {
  Ws w;
  if (!ws_carve(ws, bytes, n, nx, nz, &w)) return LACMO_ERR_WORKSPACE;
  LCHK(cudaMemsetAsync(ws, 0, ws_bytes(n, nx, nz), (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_read_fallbacks(const void* ws, int64_t n, int64_t nx, int64_t nz, uint64_t* count,
                         void* stream) {
  Ws w;
  if (!count || !ws_carve((void*)ws, ws_bytes(n, nx, nz), n, nx, nz, &w)) return LACMO_ERR_ARG;
  LCHK(cudaMemcpyAsync(count, w.nfb, 8, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  LCHK(cudaStreamSynchronize((cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_get_collision_step(const void* ws, int64_t n, int64_t nx, int64_t nz, int64_t* step,
                             void* stream) {
  Ws w;
  if (!step || !ws_carve((void*)ws, ws_bytes(n, nx, nz), n, nx, nz, &w)) return LACMO_ERR_ARG;
  LCHK(cudaMemcpyAsync(step, w.col_step, 8, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  LCHK(cudaStreamSynchronize((cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_set_collision_step(void* ws, int64_t n, int64_t nx, int64_t nz, int64_t step,
                             void* stream) {
  Ws w;
  if (step < 0 || !ws_carve(ws, ws_bytes(n, nx, nz), n, nx, nz, &w)) return LACMO_ERR_ARG;
  LCHK(launch_set_i64(w.col_step, step, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_read_flags(const void* ws, int64_t n, int64_t nx, int64_t nz, uint32_t* flags,
                     void* stream) {
  Ws w;
  if (!flags || !ws_carve((void*)ws, ws_bytes(n, nx, nz), n, nx, nz, &w)) return LACMO_ERR_ARG;
  LCHK(cudaMemcpyAsync(flags, w.flags, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  LCHK(cudaStreamSynchronize((cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_cells_import(const int64_t* cells, const uint8_t* act, int32_t* cell, int64_t n,
                       int64_t nx, int64_t nz, void* stream) {
  if (!cells || !act || !cell || n <= 0 || nx <= 0 || nz <= 0) return LACMO_ERR_ARG;
  LCHK(launch_cells_import(cells, act, cell, n, nx, nz, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_cells_export(const int32_t* cell, const double* pos, double* rel_pos, int64_t* cells,
                       uint8_t* act, int64_t n, int64_t nx, int64_t nz, double x_min, double z_min,
                       double dx, double dz, void* stream) {
  if (!cell || !pos || !rel_pos || !cells || !act || n <= 0 || nx <= 0 || nz <= 0)
    return LACMO_ERR_ARG;
  LCHK(launch_cells_export(cell, pos, rel_pos, cells, act, n, nx, nz, x_min, z_min, dx, dz,
                           (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_prepare(const lacmo_sips_t* sp, const lacmo_grid_t* g, const lacmo_params_t* p, void* ws,
                  size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const Bt B = single(*sp, *g, w, 0);
  LCHK(launch_cell_aux(B, s));
  LCHK(launch_histogram(B, s));
  LCHK(launch_bin(B, s));
  return LACMO_OK;
}

int lacmo_integrate_adv_step(const lacmo_sips_t* sp, const lacmo_grid_t* g,
                             const lacmo_params_t* p, const lacmo_draws_t* d, void* ws,
                             size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p) || !d) return LACMO_ERR_ARG;
  if (d->draws && d->n_draws < 0) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  return adv_step(single(*sp, *g, w, d->seed), *p, *d, (cudaStream_t)stream);
}

int lacmo_adv_step_begin(const lacmo_sips_t* sp, const lacmo_grid_t* g, const lacmo_params_t* p,
                         void* ws, size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const Bt B = single(*sp, *g, w, 0);
  LCHK(launch_move(B, p->dt_sub_half, s));
  LCHK(launch_bin(B, s));
  LCHK(launch_advection(B, *p, false, s));
  return LACMO_OK;
}

int lacmo_adv_step_second_half(const lacmo_sips_t* sp, const lacmo_grid_t* g,
                               const lacmo_params_t* p, void* ws, size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  LCHK(launch_advection(single(*sp, *g, w, 0), *p, true, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_adv_substep(const lacmo_sips_t* sp, const lacmo_grid_t* g, const lacmo_params_t* p,
                      double dt_sub_pos, int write_T_p, void* ws, size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const Bt B = single(*sp, *g, w, 0);
  LCHK(launch_particles(B, *p, p->dt_sub, dt_sub_pos, write_T_p != 0, s));
  LCHK(launch_cell_update(B, true, s));
  LCHK(launch_bin(B, s));
  return LACMO_OK;
}

struct lacmo_plan {
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

int lacmo_plan_create(const lacmo_sips_t* sp, const lacmo_grid_t* g, const lacmo_params_t* p,
                      const lacmo_draws_t* d, void* ws, size_t bytes, int n_steps, void* stream,
                      lacmo_plan** out) {
  if (!out || n_steps < 1) return LACMO_ERR_ARG;
  *out = nullptr;
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p) || !d) return LACMO_ERR_ARG;
  if (d->draws && d->n_draws < 0) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const int rc = capture_plan(single(*sp, *g, w, d->seed), *p, *d, n_steps, (cudaStream_t)stream,
                              &graph, &exec);
  if (rc != LACMO_OK) return rc;
  lacmo_plan* pl = new lacmo_plan{graph, exec};
  *out = pl;
  return LACMO_OK;
}

int lacmo_plan_launch(lacmo_plan* pl, void* stream) {
  if (!pl) return LACMO_ERR_ARG;
  LCHK(cudaGraphLaunch(pl->exec, (cudaStream_t)stream));
  return LACMO_OK;
}

int64_t lacmo_plan_kernel_nodes(const lacmo_plan* pl) {
  if (!pl || !pl->graph) return -1;
  size_t n = 0;
  if (cudaGraphGetNodes(pl->graph, nullptr, &n) != cudaSuccess) return -1;
  if (n == 0) return 0;
  cudaGraphNode_t* nodes = new cudaGraphNode_t[n];
  int64_t k = 0;
  if (cudaGraphGetNodes(pl->graph, nodes, &n) == cudaSuccess) {
    for (size_t i = 0; i < n; ++i) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
  } else {
    k = -1;
  }
  delete[] nodes;
  return k;
}

int lacmo_plan_destroy(lacmo_plan* pl) {
  if (!pl) return LACMO_OK;
  if (pl->exec) cudaGraphExecDestroy(pl->exec);
  if (pl->graph) cudaGraphDestroy(pl->graph);
  delete pl;
  return LACMO_OK;
}

// Host <-> device copies by the SMs, for devices that access pageable host
// memory directly: one launch moves every entry of a list (blockIdx.y =
// entry), 16-byte words where both ends are 16-byte aligned, else 8-byte
// words where 8-byte aligned, and the remaining bytes one by one.
constexpr int XFER_MAX = 40;
struct Xfer {
  int32_t n;
  const char* src[XFER_MAX];
  char* dst[XFER_MAX];
  int64_t bytes[XFER_MAX];
};
__global__ void __launch_bounds__(256) k_xfer(const __grid_constant__ Xfer x) {
  const int e = blockIdx.y;
  if (e >= x.n) return;
  const char* src = x.src[e];
  char* dst = x.dst[e];
  const int64_t nb = x.bytes[e];
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const uintptr_t al = (uintptr_t)src | (uintptr_t)dst;
  int64_t done = 0;
  if (al % 16 == 0) {
    const int64_t nv = nb / 16;
    for (int64_t i = t; i < nv; i += stride) ((int4*)dst)[i] = ((const int4*)src)[i];
    done = nv * 16;
  } else if (al % 8 == 0) {
    const int64_t nv = nb / 8;
    for (int64_t i = t; i < nv; i += stride) ((long long*)dst)[i] = ((const long long*)src)[i];
    done = nv * 8;
  }
  for (int64_t i = done + t; i < nb; i += stride) dst[i] = src[i];
}

// the device reads and writes pageable host memory (cached per device)
static bool pageable_access() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return false;
  int v = dev < 64 ? cached[dev].load() : 0;
  if (v == 0) {
    int a = 0;
    if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) a = 0;
    v = a == 1 ? 1 : -1;
    if (dev < 64) cached[dev].store(v);
  }
  return v == 1;
}

// the entries of a copy list with bytes > 0, by the SMs (launches of up to
// XFER_MAX entries) or one cudaMemcpyAsync each
static cudaError_t copy_list(const lacmo_copy_t* l, int32_t n, bool by_kernel,
                             cudaMemcpyKind kind, cudaStream_t s) {
  if (!by_kernel) {
    for (int32_t i = 0; i < n; ++i)
      if (l[i].bytes) {
        const cudaError_t e = cudaMemcpyAsync(l[i].dst, l[i].src, (size_t)l[i].bytes, kind, s);
        if (e != cudaSuccess) return e;
      }
    return cudaSuccess;
  }
  Xfer x;
  x.n = 0;
  int64_t largest = 0;
  for (int32_t i = 0; i <= n; ++i) {
    if (i == n || x.n == XFER_MAX) {
      if (x.n) {
        const int64_t blocks = (largest / 16 + 255) / 256;
        const unsigned gx = (unsigned)(blocks < 1 ? 1 : (blocks > 304 ? 304 : blocks));
        k_xfer<<<dim3(gx, (unsigned)x.n), 256, 0, s>>>(x);
        note_launches(1);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
      }
      x.n = 0;
      largest = 0;
      if (i == n) break;
    }
    if (!l[i].bytes) continue;
    x.src[x.n] = (const char*)l[i].src;
    x.dst[x.n] = (char*)l[i].dst;
    x.bytes[x.n] = l[i].bytes;
    largest = l[i].bytes > largest ? l[i].bytes : largest;
    ++x.n;
  }
  return cudaSuccess;
}

// the stream work of lacmo_dropin_adv_step, without the final synchronisation
static int dropin_sequence(const lacmo_dropin_t& c, const Ws& w, bool by_kernel, cudaStream_t s) {
  const lacmo_sips_t& sp = *c.sips;
  const lacmo_grid_t& g = *c.grid;
  LCHK(copy_list(c.in, c.n_in, by_kernel, cudaMemcpyHostToDevice, s));
  LCHK(launch_cells_import(c.cells_in, c.active_in, sp.cell, sp.n, g.nx, g.nz, s));
  LCHK(cudaMemsetAsync(c.ws, 0, ws_bytes(sp.n, g.nx, g.nz), s));
  const Bt B = single(sp, g, w, c.draws->seed);
  LCHK(launch_cell_aux(B, s));
  LCHK(launch_histogram(B, s));
  LCHK(launch_bin(B, s));
  if (c.col_step >= 0) LCHK(launch_set_i64(w.col_step, c.col_step, s));
  if (c.plan) {
    LCHK(cudaGraphLaunch(c.plan->exec, s));
  } else {
    const int rc = adv_step(B, *c.prm, *c.draws, s);
    if (rc != LACMO_OK) return rc;
  }
  LCHK(launch_cells_export(sp.cell, sp.pos, sp.rel_pos, c.cells_out, c.active_out, sp.n, g.nx,
                           g.nz, g.x_min, g.z_min, g.dx, g.dz, s));
  if (c.col_step_out)
    LCHK(cudaMemcpyAsync(c.col_step_out, w.col_step, 8, cudaMemcpyDeviceToHost, s));
  LCHK(copy_list(c.out, c.n_out, by_kernel, cudaMemcpyDeviceToHost, s));
  return LACMO_OK;
}

int lacmo_dropin_adv_step(const lacmo_dropin_t* c, void* stream) {
  if (!c || !sips_ok(c->sips) || !grid_ok(c->grid) || !prm_ok(c->prm) || !c->draws ||
      !c->cells_in || !c->active_in || !c->cells_out || !c->active_out || c->n_in < 0 ||
      c->n_out < 0 || (c->n_in && !c->in) || (c->n_out && !c->out))
    return LACMO_ERR_ARG;
  if (c->draws->draws && c->draws->n_draws < 0) return LACMO_ERR_ARG;
  const lacmo_sips_t& sp = *c->sips;
  const lacmo_grid_t& g = *c->grid;
  Ws w;
  if (!ws_carve(c->ws, c->ws_bytes, sp.n, g.nx, g.nz, &w)) return LACMO_ERR_WORKSPACE;
  for (int32_t i = 0; i < c->n_in + c->n_out; ++i) {
    const lacmo_copy_t& e = i < c->n_in ? c->in[i] : c->out[i - c->n_in];
    if (e.bytes < 0 || (e.bytes && (!e.dst || !e.src))) return LACMO_ERR_ARG;
  }
  if (c->copy_mode < LACMO_COPY_AUTO || c->copy_mode > LACMO_COPY_KERNEL) return LACMO_ERR_ARG;
  const bool direct = pageable_access();
  if (c->copy_mode == LACMO_COPY_KERNEL && !direct) return LACMO_ERR_ARG;
  const bool by_kernel = c->copy_mode == LACMO_COPY_KERNEL ||
                         (c->copy_mode == LACMO_COPY_AUTO && direct);
  cudaStream_t s = (cudaStream_t)stream;
  const int rc = dropin_sequence(*c, w, by_kernel, s);
  // copies into the caller's host arrays may be in flight when a step of the
  // sequence failed: none outlives the call
  const cudaError_t e = cudaStreamSynchronize(s);
  if (rc != LACMO_OK) return rc;
  return e == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

struct lacmo_batch {
  Bt B;
  std::vector<Member> members;
  std::vector<size_t> ws_off, ws_len;
  char* ws;
};

static size_t batch_table_bytes(int M) { return al((size_t)M * sizeof(Member)); }

size_t lacmo_batch_workspace_bytes(int M, const int64_t* n, int64_t nx, int64_t nz) {
  if (M < 1 || !n || nx <= 0 || nz <= 0) return 0;
  size_t t = batch_table_bytes(M);
  for (int m = 0; m < M; ++m) {
    if (n[m] <= 0) return 0;
    t += al(ws_bytes(n[m], nx, nz));
  }
  return t;
}

int lacmo_batch_create(int M, const lacmo_sips_t* sips, const lacmo_grid_t* grids,
                       const lacmo_params_t* prms, const uint64_t* seeds, void* ws, size_t bytes,
                       lacmo_batch** out) {
  if (!out || M < 1 || M > 65535 || !sips || !grids || !seeds || !ws) return LACMO_ERR_ARG;
  *out = nullptr;
  for (int m = 0; m < M; ++m) {
    if (!sips_ok(&sips[m]) || !grid_ok(&grids[m])) return LACMO_ERR_ARG;
    if (prms && !prm_ok(&prms[m])) return LACMO_ERR_ARG;
    if (grids[m].nx != grids[0].nx || grids[m].nz != grids[0].nz) return LACMO_ERR_ARG;
  }
  const int64_t nx = grids[0].nx, nz = grids[0].nz;
  std::vector<int64_t> ns((size_t)M);
  for (int m = 0; m < M; ++m) ns[(size_t)m] = sips[m].n;
  const size_t need = lacmo_batch_workspace_bytes(M, ns.data(), nx, nz);
  if (need == 0 || bytes < need) return LACMO_ERR_WORKSPACE;
  lacmo_batch* b = new lacmo_batch;
  b->ws = (char*)ws;
  b->members.resize((size_t)M);
  size_t off = batch_table_bytes(M);
  int64_t n_max = 0;
  for (int m = 0; m < M; ++m) {
    const size_t len = ws_bytes(sips[m].n, nx, nz);
    Ws w;
    ws_carve(b->ws + off, len, sips[m].n, nx, nz, &w);
    Member& mb = b->members[(size_t)m];
    mb = make_member(sips[m], grids[m], w, seeds[m]);
    if (prms && prms[m].init_profile_r_v && prms[m].init_profile_Theta &&
        prms[m].relaxation_time_profile) {
      mb.prof_rv = prms[m].init_profile_r_v;
      mb.prof_th = prms[m].init_profile_Theta;
      mb.t_relax = prms[m].relaxation_time_profile;
    }
    b->ws_off.push_back(off);
    b->ws_len.push_back(len);
    off += al(len);
    if (sips[m].n > n_max) n_max = sips[m].n;
  }
  if (cudaMemset(ws, 0, need) != cudaSuccess ||
      cudaMemcpy(ws, b->members.data(), (size_t)M * sizeof(Member), cudaMemcpyHostToDevice) !=
          cudaSuccess) {
    delete b;
    return LACMO_ERR_CUDA;
  }
  b->B.M = M;
  b->B.dev = (const Member*)ws;
  b->B.one = b->members[0];
  b->B.n_max = n_max;
  b->B.nx = nx;
  b->B.nz = nz;
  *out = b;
  return LACMO_OK;
}

int lacmo_batch_prepare(lacmo_batch* b, const lacmo_params_t* p, void* stream) {
  if (!b || !prm_ok(p)) return LACMO_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  LCHK(launch_cell_aux(b->B, s));
  LCHK(launch_histogram(b->B, s));
  LCHK(launch_bin(b->B, s));
  return LACMO_OK;
}

int lacmo_batch_adv_step(lacmo_batch* b, const lacmo_params_t* p, void* stream) {
  if (!b || !prm_ok(p)) return LACMO_ERR_ARG;
  const lacmo_draws_t d = {nullptr, 0, 0};
  return adv_step(b->B, *p, d, (cudaStream_t)stream, false);
}

int lacmo_batch_rebin(lacmo_batch* b, void* stream) {
  if (!b) return LACMO_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  LCHK(launch_histogram(b->B, s));
  LCHK(launch_bin(b->B, s));
  return LACMO_OK;
}

int lacmo_batch_plan_create(lacmo_batch* b, const lacmo_params_t* p, int n_steps, void* stream,
                            lacmo_plan** out) {
  if (!out || n_steps < 1) return LACMO_ERR_ARG;
  *out = nullptr;
  if (!b || !prm_ok(p)) return LACMO_ERR_ARG;
  const lacmo_draws_t d = {nullptr, 0, 0};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const int rc = capture_plan(b->B, *p, d, n_steps, (cudaStream_t)stream, &graph, &exec, false);
  if (rc != LACMO_OK) return rc;
  *out = new lacmo_plan{graph, exec};
  return LACMO_OK;
}

int lacmo_batch_particles_only(lacmo_batch* b, const lacmo_params_t* p, void* stream) {
  if (!b || !prm_ok(p)) return LACMO_ERR_ARG;
  if (p->precision == LACMO_PRECISION_MIXED)
    LCHK(launch_particles_mixed(b->B, *p, p->dt_sub, p->dt_sub, false, false, (cudaStream_t)stream));
  else
    LCHK(launch_particles(b->B, *p, p->dt_sub, p->dt_sub, false, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_batch_member_workspace(const lacmo_batch* b, int m, void** ws, size_t* bytes) {
  if (!b || m < 0 || m >= b->B.M || !ws || !bytes) return LACMO_ERR_ARG;
  *ws = b->ws + b->ws_off[(size_t)m];
  *bytes = b->ws_len[(size_t)m];
  return LACMO_OK;
}

int lacmo_batch_destroy(lacmo_batch* b) {
  delete b;
  return LACMO_OK;
}

int lacmo_propagate_particles_subloop_step(const lacmo_sips_t* sp, const lacmo_grid_t* g,
                                           const lacmo_params_t* p, double dt_sub,
                                           double dt_sub_pos, void* ws, size_t bytes,
                                           void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  const Bt B = single(*sp, *g, w, 0);
  LCHK(launch_cell_aux(B, s));
  LCHK(launch_particles(B, *p, dt_sub, dt_sub_pos, true, s));
  LCHK(launch_cell_update(B, false, s));
  LCHK(launch_bin(B, s));
  return LACMO_OK;
}

int lacmo_propagate_grid_subloop_step(const lacmo_grid_t* g, const double* dTh, const double* drv,
                                      const double* dml, void* stream) {
  if (!grid_ok(g) || !dTh || !drv || !dml) return LACMO_ERR_ARG;
  LCHK(launch_grid_only(*g, dTh, drv, dml, nullptr, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_divergence_upwind(const double* f, const double* flux, int64_t nx, int64_t nz, double dx,
                            double dz, int bcx, int bcz, double* out, void* stream) {
  if (!f || !flux || !out || nx <= 0 || nz <= 0 || (bcx != 0 && bcx != 1) ||
      (bcz != 0 && bcz != 1))
    return LACMO_ERR_ARG;
  LCHK(launch_divergence(f, flux, nx, nz, dx, dz, bcx, bcz, out, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_relaxation_term(const double* f, int64_t nx, int64_t nz, const double* prof,
                          const double* trel, double dt, double* out, void* stream) {
  if (!f || !prof || !trel || !out || nx <= 0 || nz <= 0) return LACMO_ERR_ARG;
  LCHK(launch_relaxation(f, nx, nz, prof, trel, dt, out, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_update_grid_r_l(const lacmo_sips_t* sp, const lacmo_grid_t* g, void* ws, size_t bytes,
                          void* stream) {
  if (!sips_ok(sp) || !grid_ok(g)) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  LCHK(launch_r_l_binned(single(*sp, *g, w, 0), (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_collision_step_cells(const lacmo_sips_t* sp, const lacmo_grid_t* g,
                               const lacmo_params_t* p, const lacmo_draws_t* d, void* ws,
                               size_t bytes, void* stream) {
  if (!sips_ok(sp) || !grid_ok(g) || !prm_ok(p) || !d) return LACMO_ERR_ARG;
  Ws w;
  if (!ws_carve(ws, bytes, sp->n, g->nx, g->nz, &w)) return LACMO_ERR_WORKSPACE;
  if (d->draws) LCHK(cudaMemsetAsync(w.cursor, 0, 8, (cudaStream_t)stream));
  LCHK(launch_collide_cells(single(*sp, *g, w, d->seed), *p, *d, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_collision_pair_count(const void* ws, int64_t n, int64_t nx, int64_t nz, int64_t* pairs,
                               void* stream) {
  Ws w;
  if (!pairs || !ws_carve((void*)ws, ws_bytes(n, nx, nz), n, nx, nz, &w)) return LACMO_ERR_ARG;
  LCHK(cudaMemcpyAsync(pairs, w.total_pairs, 8, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  LCHK(cudaStreamSynchronize((cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_collision_step_golovin(double* xis, double* masses, int64_t n, double dtdv,
                                 int64_t* no_cols, const double* rnd, uint64_t seed, uint64_t step,
                                 void* stream) {
  if (!xis || !masses || !no_cols || n < 0) return LACMO_ERR_ARG;
  if (n > LACMO_BOX_MAX_SIPS) return LACMO_ERR_CAPACITY;
  if (n < 2) return LACMO_OK;
  LCHK(launch_golovin(xis, masses, n, dtdv, no_cols, rnd, seed, step, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_collision_step_kernel_grid_m(double* xis, double* masses, int64_t n, double dtdv,
                                       const double* kernel_grid, int64_t nb, double m_low_log,
                                       double bin_factor_m_log, int64_t* no_cols,
                                       const double* rnd, uint64_t seed, uint64_t step,
                                       void* stream) {
  if (!xis || !masses || !kernel_grid || nb <= 0 || !no_cols || n < 0) return LACMO_ERR_ARG;
  if (n > LACMO_BOX_MAX_SIPS) return LACMO_ERR_CAPACITY;
  if (n < 2) return LACMO_OK;
  LCHK(launch_kgrid_box(xis, masses, n, dtdv, kernel_grid, nb, m_low_log, bin_factor_m_log,
                        no_cols, rnd, seed, step, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_collision_step_ecol_grid_r_box(double* xis, double* masses, double* radii,
                                         const double* vel, const double* rho, int64_t n,
                                         double dtdv, const double* E, int64_t nb, double lo,
                                         double bl, int64_t* no_cols, const double* rnd,
                                         uint64_t seed, uint64_t step, void* stream) {
  if (!xis || !masses || !radii || !vel || !rho || !E || nb <= 0 || !no_cols || n < 0)
    return LACMO_ERR_ARG;
  if (n > LACMO_ECOL_BOX_MAX_SIPS) return LACMO_ERR_CAPACITY;
  if (n < 1) return LACMO_OK;
  LCHK(launch_ecol_box(xis, masses, radii, vel, rho, n, dtdv, E, nb, lo, bl, no_cols, rnd, seed,
                       step, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_update_velocity_beard(double* vel, const double* R, int64_t n, void* stream) {
  if (!vel || !R || n < 0) return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  LCHK(launch_beard(vel, R, n, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_mass_rate_and_derivative(int sol, int64_t n, const double* m_w, const double* m_s,
                                   const double* w_s, const double* R_p, const double* T_p,
                                   const double* rho_p, const double* T_amb, const double* p_amb,
                                   const double* S_amb, const double* e_s_amb, const double* L_v,
                                   const double* K, const double* D_v, const double* sigma_p,
                                   double* gamma, double* dgamma, void* stream) {
  InPtrs in = {{m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v, K, D_v, sigma_p}};
  for (int k = 0; k < 14; ++k)
    if (!in.p[k]) return LACMO_ERR_ARG;
  if (!gamma || !dgamma || n < 0 || (sol != 0 && sol != 1)) return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  LCHK(launch_mass_rate(sol, n, in, gamma, dgamma, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_newton_full(int sol, int64_t n, double dt_sub, int no_iter, const double* m_w,
                      const double* m_s, const double* w_s, const double* R_p, const double* T_p,
                      const double* rho_p, const double* T_amb, const double* p_amb,
                      const double* S_amb, const double* e_s_amb, const double* L_v,
                      const double* K, const double* D_v, const double* sigma_p, double* dm,
                      double* gamma0, void* stream) {
  InPtrs in = {{m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v, K, D_v, sigma_p}};
  for (int k = 0; k < 14; ++k)
    if (!in.p[k]) return LACMO_ERR_ARG;
  if (!dm || !gamma0 || n < 0 || no_iter < 1 || (sol != 0 && sol != 1)) return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  LCHK(launch_newton(sol, n, dt_sub, no_iter, in, dm, gamma0, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_interpolate_velocity(const int32_t* cell, const double* rel, const double* gv, int64_t n,
                               int64_t nx, int64_t nz, double* out, void* stream) {
  if (!cell || !rel || !gv || !out || n < 0 || nx <= 0 || nz <= 0) return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  LCHK(launch_interp(cell, rel, gv, n, nx, nz, out, (cudaStream_t)stream));
  return LACMO_OK;
}

int lacmo_radius_and_bin(const double* m, const double* rho, int64_t n, double lo, double bl,
                         int64_t nb, double* R, int64_t* bin, void* stream) {
  if (!m || !rho || !R || n < 0 || (bin && nb <= 0)) return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  LCHK(launch_radius_bin(m, rho, n, lo, bl, nb, R, bin, (cudaStream_t)stream));
  return LACMO_OK;
}

}  // extern "C"
