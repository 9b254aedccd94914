// Hand-written adjoint of the condensation sub-steps with their cell heat and
// vapour feedback (integration.py:840-940 with the Newton of :728-836 and the
// grid update of :402-484), for gradients of liquid water with respect to
// per-SIP solute mass and hygroscopicity.
//
// Differentiated model ("condensation model"): SIPs keep their cells and
// multiplicities (positions, advection and collisions are recorded events held
// fixed); every sub-step of length dt_sub solves the implicit Euler step
// m - m_w - dt_sub gamma(m) = 0 of each SIP to convergence (the damped Newton
// of the reference, iterated until the step falls below 1e-15 relative),
// floored at the efflorescence mass, and then updates Theta and r_v of each
// cell from the condensed mass, with all ambient terms (T, p, S, e_s, K, D_v,
// L_v, sigma_w, rho_w) functions of the cell's Theta and r_v.
// Hygroscopicity: the ammonium-sulfate water activity a_w(w_s) (material_
// properties.py:429-436) becomes 1 + (kappa / 0.6) (a_w(w_s) - 1), so kappa =
// 0.6 reproduces the reference.
//
// Reverse sweep per sub-step: the implicit-function theorem through the root,
// dm/dx = dt (dgamma/dx) / (1 - dt dgamma/dm) for x = m_w, m_s, kappa, Theta,
// r_v (dm/dm_w = 1 / (1 - dt dgamma/dm)), or dm/dm_s = 1/0.78 - 1 on the
// floor; the local partials come from forward-mode dual numbers through the
// same formulas; the cell update's Jacobian likewise.  Sums over a cell's
// SIPs use atomics (FP64).
#include <cuda_runtime.h>

#include "lacmo_internal.cuh"
#include "lacmo_physics.cuh"

namespace lacmo {
namespace adj {

// ---- dual numbers: value and N partial derivatives ----
template <int N>
struct Dual {
  double v;
  double d[N];
};
template <int N>
__device__ __forceinline__ Dual<N> cst(double v) {
  Dual<N> r; r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> var(double v, int k) {
  Dual<N> r = cst<N>(v); r.d[k] = 1.0; return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, double b) { return a + cst<N>(b); }
template <int N>
__device__ __forceinline__ Dual<N> operator+(double a, const Dual<N>& b) { return cst<N>(a) + b; }
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, double b) { return a - cst<N>(b); }
template <int N>
__device__ __forceinline__ Dual<N> operator-(double a, const Dual<N>& b) { return cst<N>(a) - b; }
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) { return a * (1.0 / b); }
template <int N>
__device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) { return cst<N>(a) / b; }
template <int N>
__device__ __forceinline__ Dual<N> chain(const Dual<N>& a, double f, double df) {
  Dual<N> r; r.v = f;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = df * a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dexp(const Dual<N>& a) { const double e = exp(a.v); return chain(a, e, e); }
template <int N>
__device__ __forceinline__ Dual<N> dlog(const Dual<N>& a) { return chain(a, log(a.v), 1.0 / a.v); }
template <int N>
__device__ __forceinline__ Dual<N> dpow(const Dual<N>& a, double y) {
  const double p = pow(a.v, y);
  return chain(a, p, y * p / a.v);
}
template <int N>
__device__ __forceinline__ Dual<N> dcbrt(const Dual<N>& a) {
  const double c = cbrt(a.v);
  return chain(a, c, c / (3.0 * a.v));
}
__device__ __forceinline__ double dexp(double a) { return exp(a); }
__device__ __forceinline__ double dlog(double a) { return log(a); }
__device__ __forceinline__ double dpow(double a, double y) { return pow(a, y); }
__device__ __forceinline__ double dcbrt(double a) { return cbrt(a); }
__device__ __forceinline__ double val(double a) { return a; }
template <int N>
__device__ __forceinline__ double val(const Dual<N>& a) { return a.v; }

// ---- cell ambient from Theta and r_v (integration.py:402-484, 359-400) ----
struct GridConst {
  double p_ref, p_ref_inv, V;
};
template <class S>
struct Amb {
  S T, p, Sat, e_s, K, D_v, L_v, sigw, rhow, lap0, lbp0, c1, c2;
};
template <class S>
__device__ __forceinline__ Amb<S> ambient(const S& Th, const S& r_v, double rho_d,
                                          const GridConst& g) {
  Amb<S> a;
  const S pdr = dpow(rho_d * Th * (LC_R_D * g.p_ref_inv), LC_KAPPA_FACTOR);
  a.T = Th * dpow(pdr, LC_KAPPA_AIR_DRY);
  a.p = pdr * g.p_ref * (1.0 + r_v / LC_EPSILON_GC);
  a.e_s = 2.53E11 * dexp(-5420.0 / a.T);
  a.Sat = rho_d * r_v * a.T * LC_R_V / a.e_s;
  a.K = 4.1868E-3 * (5.69 + 0.017 * (a.T - 273.15));
  a.D_v = 4.01218E-5 * dpow(a.T, 1.94) / a.p;
  a.L_v = 1.0E3 * (2500.82 - 2.358 * (a.T - 273.0));
  const S tau = 1.0 - a.T / 647.096;
  a.sigw = 0.2358 * dpow(tau, 1.256) * (1.0 - 0.625 * tau);
  const S dT = a.T - LC_PAR_WATER_DENS_2;
  a.rhow = LC_PAR_WATER_DENS_0 + LC_PAR_WATER_DENS_1 * (dT * dT);
  a.lap0 = (LC_C_ALPHA_1 + LC_C_ALPHA_2 * (a.T - LC_T_ALPHA_0)) * a.K / a.p;
  a.lbp0 = LC_C_BETA_1 * (1.0 + LC_C_BETA_2 * (a.T - LC_T_ALPHA_0)) * a.D_v;
  a.c1 = a.L_v * a.L_v / (LC_R_V * a.K * a.T * a.T);
  a.c2 = LC_R_V * a.T / (a.D_v * a.e_s);
  return a;
}

// ---- mass rate of an ammonium-sulfate SIP (microphysics.py:1359-1469) with
// the kappa scaling; gamma in fg/s and (for S = double) dgamma/dm_w ----
template <class S>
__device__ __forceinline__ S mass_rate(double m, const S& m_s, const S& ks, const Amb<S>& a,
                                       double* dg_out) {
  const S m_p = m + m_s;
  const S w_s = m_s / m_p;
  S pr = LC_PAR_RHO_AS_0 * w_s + LC_PAR_RHO_AS_1;
  pr = pr * w_s + LC_PAR_RHO_AS_2;
  pr = pr * w_s + LC_PAR_RHO_AS_3;
  const S rho_p = a.rhow * pr;
  const S R_p = dcbrt(LC_FOUR_PI_OVER_THREE_INV * m_p / rho_p);
  const S sigma_p = a.sigw * (1.0 + LC_PAR_SIGMA_AS * w_s / (1.0 - w_s));
  const S l_a = 1.0E-6 * (R_p + a.lap0);
  const S l_b = 1.0E-6 * (R_p + a.lbp0);
  const S m_p_inv_SI = 1.0E18 / m_p;
  const S wfac = w_s / ((1.0 - w_s) * (1.0 - w_s));
  S pd = LC_PAR_RHO_DERIV_AS_0 * w_s + LC_PAR_RHO_DERIV_AS_1;
  pd = pd * w_s + LC_PAR_RHO_DERIV_AS_2;
  const S drho_dm_over_rho = -1.0 * a.rhow * m_p_inv_SI / rho_p * w_s * pd;
  S aw = LC_PAR_WAT_ACT_AS_0 * w_s + LC_PAR_WAT_ACT_AS_1;
  aw = aw * w_s + LC_PAR_WAT_ACT_AS_2;
  aw = aw * w_s + LC_PAR_WAT_ACT_AS_3;
  const S aw_m1 = ks * (aw * w_s);                    // a_w - 1, scaled by kappa / 0.6
  const S a_w = 1.0 + aw_m1;
  S da = LC_PAR_WAT_ACT_DERIV_AS_0 * w_s + LC_PAR_WAT_ACT_DERIV_AS_1;
  da = da * w_s + LC_PAR_WAT_ACT_DERIV_AS_2;
  da = da * w_s + LC_PAR_WAT_ACT_DERIV_AS_3;
  const S da_w_dm = -1.0 * ks * m_p_inv_SI * w_s * da;
  const S dsigma_dm = -LC_PAR_SIGMA_AS * a.sigw * m_p_inv_SI * wfac;
  const S dR_dm_over_R = LC_ONE_THIRD * (m_p_inv_SI - drho_dm_over_rho);
  const S dR_dm = 1.0E-6 * dR_dm_over_R * R_p;
  const S eps_k = 2.0E6 * sigma_p / (LC_R_V * a.T * rho_p * R_p);
  const S kel = dexp(eps_k);
  const S S_eq = a_w * kel;
  const S f3 = 1.0 / (l_a * S_eq * a.c1 + l_b * a.c2);
  const S f1f3 = LC_FOUR_PI * R_p * R_p * f3;
  const S f2 = a.Sat - S_eq;
  if (dg_out) {
    const double dSeq = val(da_w_dm) * val(kel) +
                        val(S_eq) * val(eps_k) *
                            (val(dsigma_dm) / val(sigma_p) - val(drho_dm_over_rho) -
                             val(dR_dm_over_R));
    const double dg1 = (dSeq * val(l_a) + val(S_eq) * val(dR_dm)) * val(a.c1) +
                       val(dR_dm) * val(a.c2);
    *dg_out = 1.0E-12 * val(f1f3) *
              (val(f2) * (2.0 * val(dR_dm_over_R) - val(f3) * dg1) - dSeq);
  }
  return 1.0E6 * f1f3 * f2;
}

// the implicit Euler step solved to convergence; returns the new mass and
// whether it sits on the efflorescence floor
__device__ __forceinline__ double solve_step(double m_w, double m_s, double ks,
                                             const Amb<double>& a, double dt, bool* floored) {
  const double m_eff = m_s * (LC_W_S_MAX_AS_INV - 1.0);
  double dg;
  double g = mass_rate<double>(m_w, m_s, ks, a, &dg);
  double x = dt * dg;
  double m = m_w + dt * g * ((x < 0.9) ? 1.0 / (1.0 - x) : 10.0);
  if (!(m >= m_eff)) m = m_eff;
  for (int it = 0; it < 40; ++it) {
    g = mass_rate<double>(m, m_s, ks, a, &dg);
    x = dt * dg;
    double mn = m + (dt * g + m_w - m) * ((x < 0.9) ? 1.0 / (1.0 - x) : 10.0);
    if (!(mn >= m_eff)) mn = m_eff;
    const double step = fabs(mn - m);
    m = mn;
    if (step <= 1e-15 * fabs(m)) break;
  }
  *floored = !(m > m_eff);
  return m;
}

// cell update (integration.py:402-438): Theta and r_v after the sub-step
template <class S>
__device__ __forceinline__ void cell_update(const S& Th, const S& r_v, const S& dml, double rho_d,
                                            double mdi, double dTh, double drv,
                                            const GridConst& g, S* Th_out, S* rv_out) {
  const Amb<S> a = ambient<S>(Th, r_v, rho_d, g);   // L_v before the update
  const S Th1 = Th + dTh;
  const S rv1 = r_v + drv - dml * mdi;
  const S ToT = dpow(g.p_ref_inv * LC_R_D * rho_d * Th1, LC_KAPPA_FACTOR2);
  *Th_out = Th1 + ToT * (a.L_v * dml) / (LC_C_PD * rho_d * g.V * (1.0 + rv1 * LC_HEAT_FACTOR_R_V));
  *rv_out = rv1;
}

struct Args {
  int64_t n, C;
  double* m_w;          // [n] in/out
  const double* m_s;    // [n]
  const double* xi;     // [n]
  const int32_t* cell;  // [n] (negative: not condensing)
  double* Th;           // [C] in/out
  double* r_v;          // [C] in/out
  const double* rho_d;  // [C]
  const double* mdi;    // [C] mass_dry_inv
  const double* dTh;    // [C] per sub-step forcing, or null
  const double* drv;    // [C]
  double* dml;          // [C] scratch
  double dt, ks;
  GridConst g;
};

__global__ void k_fwd_sips(Args a, double* tape_m) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double mw = a.m_w[k];
    if (tape_m) tape_m[k] = mw;
    const int32_t c = a.cell[k];
    if (c < 0) continue;
    const Amb<double> am = ambient<double>(a.Th[c], a.r_v[c], a.rho_d[c], a.g);
    bool fl;
    const double m = solve_step(mw, a.m_s[k], a.ks, am, a.dt, &fl);
    a.m_w[k] = m;
    atomicAdd(a.dml + c, (m - mw) * a.xi[k]);
  }
}

__global__ void k_fwd_cells(Args a, double* tape_c) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.C;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double Th = a.Th[c], rv = a.r_v[c];
    if (tape_c) { tape_c[c] = Th; tape_c[a.C + c] = rv; }
    const double dml = a.dml[c] * 1.0E-18;
    a.dml[c] = 0.0;
    double Th2, rv2;
    cell_update<double>(Th, rv, dml, a.rho_d[c], a.mdi[c], a.dTh ? a.dTh[c] : 0.0,
                        a.drv ? a.drv[c] : 0.0, a.g, &Th2, &rv2);
    a.Th[c] = Th2;
    a.r_v[c] = rv2;
  }
}

// reverse of one sub-step.  In: lam_m [n], lam_Th, lam_rv [C] (adjoints of the
// state after the sub-step), tape_m (m_w before), tape_c (Theta, r_v before),
// m_after [n] (m_w after).  Out: the same adjoints for the state before;
// grad_ms [n] and grad_ks [1] accumulate.
__global__ void k_bwd_cells(Args a, const double* tape_c, const double* m_before,
                            const double* m_after, double* lam_Th, double* lam_rv,
                            double* lam_dml) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.C;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double Th = tape_c[c], rv = tape_c[a.C + c];
    const double dml = a.dml[c] * 1.0E-18;   // recomputed forward sum of this sub-step
    Dual<3> Th2, rv2;
    cell_update<Dual<3>>(var<3>(Th, 0), var<3>(rv, 1), var<3>(dml, 2), a.rho_d[c], a.mdi[c],
                         a.dTh ? a.dTh[c] : 0.0, a.drv ? a.drv[c] : 0.0, a.g, &Th2, &rv2);
    const double lT = lam_Th[c], lr = lam_rv[c];
    lam_Th[c] = lT * Th2.d[0] + lr * rv2.d[0];
    lam_rv[c] = lT * Th2.d[1] + lr * rv2.d[1];
    lam_dml[c] = (lT * Th2.d[2] + lr * rv2.d[2]) * 1.0E-18;   // per fg of dm*xi
    a.dml[c] = 0.0;
  }
}

__global__ void k_bwd_sum_dml(Args a, const double* m_before, const double* m_after) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = a.cell[k];
    if (c >= 0) atomicAdd(a.dml + c, (m_after[k] - m_before[k]) * a.xi[k]);
  }
}

__global__ void k_bwd_sips(Args a, const double* tape_c, const double* m_before,
                           const double* m_after, double* lam_m, const double* lam_dml,
                           double* lam_Th_pre, double* lam_rv_pre, double* grad_ms,
                           double* grad_ks) {
  double gk = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = a.cell[k];
    if (c < 0) continue;   // not condensing: m_w passes through
    const double xi = a.xi[k];
    const double m = m_after[k];
    const double ms = a.m_s[k];
    // total adjoint of the new mass: the state after, and the cell sum
    const double lm = lam_m[k] + lam_dml[c] * xi;
    const double m_eff = ms * (LC_W_S_MAX_AS_INV - 1.0);
    if (!(m > m_eff)) {
      grad_ms[k] += lm * (LC_W_S_MAX_AS_INV - 1.0);
      lam_m[k] = -lam_dml[c] * xi;
      continue;
    }
    const double Th = tape_c[c], rv = tape_c[a.C + c];
    const Amb<Dual<4>> am = ambient<Dual<4>>(var<4>(Th, 2), var<4>(rv, 3), a.rho_d[c], a.g);
    double dg;
    {
      const Amb<double> a0 = ambient<double>(Th, rv, a.rho_d[c], a.g);
      mass_rate<double>(m, ms, a.ks, a0, &dg);
    }
    const Dual<4> gam = mass_rate<Dual<4>>(m, var<4>(ms, 0), var<4>(a.ks, 1), am, nullptr);
    const double inv = 1.0 / (1.0 - a.dt * dg);
    const double t = lm * a.dt * inv;
    grad_ms[k] += t * gam.d[0];
    gk += t * gam.d[1] * (1.0 / 0.6);   // ks = kappa / 0.6
    atomicAdd(lam_Th_pre + c, t * gam.d[2]);
    atomicAdd(lam_rv_pre + c, t * gam.d[3]);
    lam_m[k] = lm * inv - lam_dml[c] * xi;
  }
  if (gk != 0.0) atomicAdd(grad_ks, gk);
}

static inline int nb(int64_t n, int t) {
  int64_t b = (n + t - 1) / t;
  return (int)(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}

}  // namespace adj
}  // namespace lacmo

using namespace lacmo;
using namespace lacmo::adj;

static Args make_args(int64_t n, int64_t C, double* m_w, const double* m_s, const double* xi,
                      const int32_t* cell, double* Th, double* r_v, const double* rho_d,
                      const double* mdi, const double* dTh, const double* drv, double* dml,
                      double dt, double kappa, double p_ref, double V) {
  Args a;
  a.n = n; a.C = C; a.m_w = m_w; a.m_s = m_s; a.xi = xi; a.cell = cell; a.Th = Th; a.r_v = r_v;
  a.rho_d = rho_d; a.mdi = mdi; a.dTh = dTh; a.drv = drv; a.dml = dml; a.dt = dt;
  a.ks = kappa / 0.6;
  a.g.p_ref = p_ref; a.g.p_ref_inv = 1.0 / p_ref; a.g.V = V;
  return a;
}

extern "C" {

int lacmo_adj_forward(int64_t n, int64_t C, double* m_w, const double* m_s, const double* xi,
                      const int32_t* cell, double* Th, double* r_v, const double* rho_d,
                      const double* mdi, const double* dTh, const double* drv, double* dml,
                      double dt_sub, double kappa, double p_ref, double V, int n_sub,
                      double* tape_m, double* tape_c, void* stream) {
  if (n <= 0 || C <= 0 || !m_w || !m_s || !xi || !cell || !Th || !r_v || !rho_d || !mdi || !dml ||
      n_sub < 0 || !(kappa > 0.0) || !(p_ref > 0.0))
    return LACMO_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Args a = make_args(n, C, m_w, m_s, xi, cell, Th, r_v, rho_d, mdi, dTh, drv, dml, dt_sub, kappa,
                     p_ref, V);
  if (cudaMemsetAsync(dml, 0, 8 * C, s) != cudaSuccess) return LACMO_ERR_CUDA;
  for (int k = 0; k < n_sub; ++k) {
    k_fwd_sips<<<nb(n, 128), 128, 0, s>>>(a, tape_m ? tape_m + (size_t)k * n : nullptr);
    k_fwd_cells<<<nb(C, 64), 64, 0, s>>>(a, tape_c ? tape_c + (size_t)k * 2 * C : nullptr);
    note_launches(2);
  }
  if (tape_m) {   // the state after the last sub-step closes the tape
    if (cudaMemcpyAsync(tape_m + (size_t)n_sub * n, m_w, 8 * n, cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
      return LACMO_ERR_CUDA;
  }
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

int lacmo_adj_backward(int64_t n, int64_t C, const double* m_s, const double* xi,
                       const int32_t* cell, const double* rho_d, const double* mdi,
                       const double* dTh, const double* drv, double* dml, double dt_sub,
                       double kappa, double p_ref, double V, int n_sub, const double* tape_m,
                       const double* tape_c, double* lam_m, double* lam_Th, double* lam_rv,
                       double* lam_dml, double* grad_ms, double* grad_kappa, void* stream) {
  if (n <= 0 || C <= 0 || !m_s || !xi || !cell || !rho_d || !mdi || !dml || n_sub < 0 ||
      !tape_m || !tape_c || !lam_m || !lam_Th || !lam_rv || !lam_dml || !grad_ms || !grad_kappa ||
      !(kappa > 0.0))
    return LACMO_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Args a = make_args(n, C, nullptr, m_s, xi, cell, nullptr, nullptr, rho_d, mdi, dTh, drv, dml,
                     dt_sub, kappa, p_ref, V);
  if (cudaMemsetAsync(dml, 0, 8 * C, s) != cudaSuccess) return LACMO_ERR_CUDA;
  double* gks = grad_kappa;
  for (int k = n_sub - 1; k >= 0; --k) {
    const double* mb = tape_m + (size_t)k * n;
    const double* ma = tape_m + (size_t)(k + 1) * n;
    const double* tc = tape_c + (size_t)k * 2 * C;
    k_bwd_sum_dml<<<nb(n, 128), 128, 0, s>>>(a, mb, ma);
    k_bwd_cells<<<nb(C, 64), 64, 0, s>>>(a, tc, mb, ma, lam_Th, lam_rv, lam_dml);
    k_bwd_sips<<<nb(n, 128), 128, 0, s>>>(a, tc, mb, ma, lam_m, lam_dml, lam_Th, lam_rv, grad_ms,
                                          gks);
    note_launches(3);
  }
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

}  // extern "C"
