// Hand-written adjoint of the condensation sub-steps with their cell heat and
// vapour feedback and the grid advection of Theta and r_v (integration.py:
// 840-940 with the Newton of :728-836, the grid update of :402-484 and the
// advective increments of :80-287, 1483-1508, 1536-1561), for gradients of
// liquid water and surface rain with respect to per-SIP solute mass,
// hygroscopicity and the strength of the prescribed mass flux.
//
// Differentiated model: the SIPs' cells per sub-step and their multiplicities
// are recorded events (positions, ground removal and collisions are held
// fixed; SIP motion reaches condensation only through the piecewise constant
// cell index); every sub-step runs the condensation step of each SIP, either
// the time step's own map of no_iter damped Newton evaluations (the product's
// map, differentiated exactly with forward-mode duals through every
// evaluation, second derivatives included) or the implicit Euler step solved
// to convergence (implicit-function theorem), and then updates Theta and r_v
// of each cell from the condensed mass and the half step's advective (+
// relaxation) increments, with all ambient terms (T, p, S, e_s, K, D_v, L_v,
// sigma_w, rho_w) functions of the cell's Theta and r_v.  The reference sets a
// SIP's temperature to its cell's at the start of every sub-step
// (integration.py:1059-1060), so T_p is the ambient T here.
// Hygroscopicity: the ammonium-sulfate water activity a_w(w_s) (material_
// properties.py:429-436) becomes 1 + (kappa / 0.6) (a_w(w_s) - 1), so kappa =
// 0.6 reproduces the reference.
//
// Reverse sweep per sub-step: the local partials come from forward-mode dual
// numbers through the same formulas; the cell update's Jacobian likewise; the
// increments' Jacobian from duals through the limited face fluxes.  Sums over
// a cell's SIPs use atomics (FP64).
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
// a constant of scalar type S
template <class S>
struct Const {
  static __device__ __forceinline__ S of(double v) { return v; }
};
template <int N>
struct Const<Dual<N>> {
  static __device__ __forceinline__ Dual<N> of(double v) { return cst<N>(v); }
};

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
template <class S, class M>
__device__ __forceinline__ S mass_rate(const M& m, const S& m_s, const S& ks, const Amb<S>& a,
                                       S* dg_out) {
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
  if (dg_out) {   // dgamma/dm_w in the arithmetic of S (second derivatives for duals)
    const S dSeq = da_w_dm * kel + S_eq * eps_k * (dsigma_dm / sigma_p - drho_dm_over_rho -
                                                   dR_dm_over_R);
    const S dg1 = (dSeq * l_a + S_eq * dR_dm) * a.c1 + dR_dm * a.c2;
    *dg_out = 1.0E-12 * f1f3 * (f2 * (2.0 * dR_dm_over_R - f3 * dg1) - dSeq);
  }
  return 1.0E6 * f1f3 * f2;
}

// the implicit Euler step solved to convergence; returns the new mass and
// whether it sits on the efflorescence floor
// (no_iter > 0: exactly no_iter evaluations, the map of integration.py:728-836
// the time step uses; 0: to convergence)
__device__ __forceinline__ double solve_step(double m_w, double m_s, double ks,
                                             const Amb<double>& a, double dt, int no_iter,
                                             bool* floored) {
  const double m_eff = m_s * (LC_W_S_MAX_AS_INV - 1.0);
  double dg;
  double g = mass_rate<double>(m_w, m_s, ks, a, &dg);
  double x = dt * dg;
  double m = m_w + dt * g * ((x < 0.9) ? 1.0 / (1.0 - x) : 10.0);
  if (!(m >= m_eff)) m = m_eff;
  const int iters = no_iter > 0 ? no_iter - 1 : 40;
  for (int it = 0; it < iters; ++it) {
    g = mass_rate<double>(m, m_s, ks, a, &dg);
    x = dt * dg;
    double mn = m + (dt * g + m_w - m) * ((x < 0.9) ? 1.0 / (1.0 - x) : 10.0);
    if (!(mn >= m_eff)) mn = m_eff;
    const double step = fabs(mn - m);
    m = mn;
    if (no_iter == 0 && step <= 1e-15 * fabs(m)) break;
  }
  *floored = !(m > m_eff);
  return m;
}

// the time step's own map (integration.py:786-836): no_iter evaluations of the
// damped Newton, each floored at the efflorescence mass, in the arithmetic of
// S (duals: the exact derivative of the map, branches taken as evaluated)
template <class S>
__device__ __forceinline__ S newton_map(const S& m_w, const S& m_s, const S& ks, const Amb<S>& a,
                                        double dt, int no_iter) {
  const S m_eff = m_s * (LC_W_S_MAX_AS_INV - 1.0);
  S dg;
  S g = mass_rate<S>(m_w, m_s, ks, a, &dg);
  S x = dt * dg;
  S m = m_w + dt * g * ((val(x) < 0.9) ? 1.0 / (1.0 - x) : Const<S>::of(10.0));
  if (!(val(m) >= val(m_eff))) m = m_eff;
  for (int it = 0; it < no_iter - 1; ++it) {
    g = mass_rate<S>(m, m_s, ks, a, &dg);
    x = dt * dg;
    m = m + (dt * g + m_w - m) * ((val(x) < 0.9) ? 1.0 / (1.0 - x) : Const<S>::of(10.0));
    if (!(val(m) >= val(m_eff))) m = m_eff;
  }
  return m;
}

// cell update (integration.py:402-438): Theta and r_v after the sub-step
template <class S, class F>
__device__ __forceinline__ void cell_update(const S& Th, const S& r_v, const S& dml, double rho_d,
                                            double mdi, const F& dTh, const F& drv,
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
  const int32_t* cell;  // [n] this sub-step's cells (negative: not condensing)
  double* Th;           // [C] in/out
  double* r_v;          // [C] in/out
  const double* rho_d;  // [C]
  const double* mdi;    // [C] mass_dry_inv
  const double* dTh;    // [C] per sub-step forcing, or null
  const double* drv;    // [C]
  double* dml;          // [C] scratch
  double dt, ks;
  GridConst g;
  int no_iter;          // 0: implicit step to convergence, else the step's map
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
    const double m = solve_step(mw, a.m_s[k], a.ks, am, a.dt, a.no_iter, &fl);
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
    cell_update<double, double>(Th, rv, dml, a.rho_d[c], a.mdi[c], a.dTh ? a.dTh[c] : 0.0,
                                a.drv ? a.drv[c] : 0.0, a.g, &Th2, &rv2);
    a.Th[c] = Th2;
    a.r_v[c] = rv2;
  }
}

// reverse of one sub-step.  In: lam_m [n], lam_Th, lam_rv [C] (adjoints of the
// state after the sub-step), tape_m (m_w before), tape_c (Theta, r_v before),
// m_after [n] (m_w after).  Out: the same adjoints for the state before;
// grad_ms [n] and grad_ks [1] accumulate.
// lam_inc (optional, [2][C]) accumulates the adjoints of the increments
// (dTh, drv), which every sub-step of a half step shares
__global__ void k_bwd_cells(Args a, const double* tape_c, const double* m_before,
                            const double* m_after, double* lam_Th, double* lam_rv,
                            double* lam_dml, double* lam_inc) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.C;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double Th = tape_c[c], rv = tape_c[a.C + c];
    const double dml = a.dml[c] * 1.0E-18;   // recomputed forward sum of this sub-step
    const double fT = a.dTh ? a.dTh[c] : 0.0, fr = a.drv ? a.drv[c] : 0.0;
    Dual<5> Th2, rv2;
    cell_update<Dual<5>, Dual<5>>(var<5>(Th, 0), var<5>(rv, 1), var<5>(dml, 2), a.rho_d[c],
                                  a.mdi[c], var<5>(fT, 3), var<5>(fr, 4), a.g, &Th2, &rv2);
    const double lT = lam_Th[c], lr = lam_rv[c];
    lam_Th[c] = lT * Th2.d[0] + lr * rv2.d[0];
    lam_rv[c] = lT * Th2.d[1] + lr * rv2.d[1];
    lam_dml[c] = (lT * Th2.d[2] + lr * rv2.d[2]) * 1.0E-18;   // per fg of dm*xi
    if (lam_inc) {
      lam_inc[c] += lT * Th2.d[3] + lr * rv2.d[3];
      lam_inc[a.C + c] += lT * Th2.d[4] + lr * rv2.d[4];
    }
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
    if (a.no_iter > 0) {   // the time step's map, differentiated exactly
      const double Th = tape_c[c], rv = tape_c[a.C + c];
      const Amb<Dual<5>> am = ambient<Dual<5>>(var<5>(Th, 3), var<5>(rv, 4), a.rho_d[c], a.g);
      const Dual<5> mn = newton_map<Dual<5>>(var<5>(m_before[k], 0), var<5>(ms, 1),
                                             var<5>(a.ks, 2), am, a.dt, a.no_iter);
      grad_ms[k] += lm * mn.d[1];
      gk += lm * mn.d[2] * (1.0 / 0.6);
      atomicAdd(lam_Th_pre + c, lm * mn.d[3]);
      atomicAdd(lam_rv_pre + c, lm * mn.d[4]);
      lam_m[k] = lm * mn.d[0] - lam_dml[c] * xi;
      continue;
    }
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

// ---- advective increments of Theta and r_v (integration.py:80-287 with the
// sub-step increments of :1483-1508 and :1536-1561) in the arithmetic of S ----
__device__ __forceinline__ double dfmin(double x, double y) { return fmin(x, y); }
template <int N>
__device__ __forceinline__ Dual<N> dfmin(const Dual<N>& x, const Dual<N>& y) {
  if (isnan(x.v)) return y;   // C fmin: a NaN operand is ignored
  if (isnan(y.v)) return x;
  return (y.v < x.v) ? y : x;
}
__device__ __forceinline__ double dmax0(double z) { return np_max(0.0, z); }
template <int N>
__device__ __forceinline__ Dual<N> dmax0(const Dual<N>& z) {   // np.maximum(0, z)
  return (0.0 >= z.v) ? cst<N>(0.0) : z;
}
// integration.py:113-148 limiter of the Hundsdorfer et al. (1995) scheme
template <class S>
__device__ __forceinline__ S limiter_of(const S& a0, const S& a1, const S& a2) {
  const S r = (fabs(val(a1) - val(a2)) > 1.0E-8 * fabs(val(a0) - val(a1)))
                  ? (a0 - a1) / (a1 - a2)
                  : (a0 - a1) * 1.0E8 * np_sign(val(a1) - val(a2));
  const S K = (1.0 + 2.0 * r) * LC_ONE_THIRD;
  return dmax0(dfmin(2.0 * r, dfmin(K, Const<S>::of(2.0))));
}
// flux through the face left of stencil value a0 (integration.py:204-228)
template <class S>
__device__ __forceinline__ S face_flux_of(double u, const S& am2, const S& am1, const S& a0,
                                          const S& ap1) {
  if (u >= 0.0) return u * (am1 + 0.5 * limiter_of(a0, am1, am2) * (am1 - am2));
  return u * (a0 + 0.5 * limiter_of(am1, a0, ap1) * (a0 - ap1));
}
__device__ __forceinline__ int64_t wrap_idx(int64_t i, int64_t N, int bc) {
  if (bc == 0) { i %= N; return i < 0 ? i + N : i; }
  return i < 0 ? 0 : (i > N - 1 ? N - 1 : i);
}
// the four face fluxes of cell (i, j) (x: periodic, z: solid walls) and the
// flat indices of their stencils
struct Stencil {
  double u[4];
  int64_t idx[4][4];
  bool zero[4];
};
__device__ __forceinline__ Stencil stencil_of(const double* flux, int64_t nx, int64_t nz,
                                              int64_t i, int64_t j) {
  Stencil st;
  for (int s = 0; s < 2; ++s) {
    const int64_t fi = i + s, fj = j + s;
    st.u[s] = flux[fi * (nz + 1) + j];
    st.zero[s] = false;
    st.u[2 + s] = flux[(nx + 1) * (nz + 1) + i * (nz + 1) + fj];
    st.zero[2 + s] = (fj == 0 || fj == nz);
    for (int t = 0; t < 4; ++t) {
      st.idx[s][t] = wrap_idx(fi - 2 + t, nx, 0) * nz + j;
      st.idx[2 + s][t] = i * nz + wrap_idx(fj - 2 + t, nz, 1);
    }
  }
  return st;
}

struct IncArgs {
  const double* f[2];     // Theta, r_v [C]
  const double* rdi;      // rho_dry_inv [C]
  const double* flux;     // mass flux at the faces [2][nx+1][nz+1]
  const double* trel;     // relaxation time [nz] or null (no relaxation)
  const double* prof[2];  // initial profiles of Theta and r_v [nz]
  int64_t nx, nz;
  double dx, dz, dt;
};

// increments of a half step: second = 0: inc = -dt div rdi + relax;
// second = 1: inc = -2 dt div rdi - inc_prev + 2 relax (inc holds inc_prev)
__global__ void k_increments(IncArgs a, int second, double* inc_Th, double* inc_rv) {
  const int64_t C = a.nx * a.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 2 * C;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int fld = t < C ? 0 : 1;
    const int64_t c = t - fld * C, i = c / a.nz, j = c - i * a.nz;
    const double* f = a.f[fld];
    const Stencil st = stencil_of(a.flux, a.nx, a.nz, i, j);
    double F[4];
    for (int q = 0; q < 4; ++q)
      F[q] = st.zero[q] ? 0.0
                        : face_flux_of<double>(st.u[q], f[st.idx[q][0]], f[st.idx[q][1]],
                                               f[st.idx[q][2]], f[st.idx[q][3]]);
    const double div = (F[1] - F[0]) / a.dx + (F[3] - F[2]) / a.dz;
    double relax = 0.0;
    if (a.trel) {   // integration.py:325-354, column sum in x order
      double sum = f[j];
      for (int64_t ii = 1; ii < a.nx; ++ii) sum += f[ii * a.nz + j];
      relax = a.dt * (a.prof[fld][j] - sum / (double)a.nx) / a.trel[j];
    }
    double* out = fld == 0 ? inc_Th : inc_rv;
    double v;
    if (!second) {
      v = -a.dt * div * a.rdi[c];
      if (a.trel) v += relax;
    } else {
      v = -2.0 * a.dt * div * a.rdi[c] - out[c];
      if (a.trel) v += 2. * relax;
    }
    out[c] = v;
  }
}

// vector-Jacobian product of factor * (advective + relaxation increment):
// lam_f += factor J^T lam_inc for both fields; grad_s += factor lam_inc .
// (advective increment) / flux_scale, the derivative by a common factor s of
// the mass flux (the flux passed is s times the unscaled one)
__global__ void k_increments_vjp(IncArgs a, double factor, double flux_scale,
                                 const double* lam_inc, double* lam_Th, double* lam_rv,
                                 double* grad_s) {
  const int64_t C = a.nx * a.nz;
  double gs = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 2 * C;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int fld = t < C ? 0 : 1;
    const int64_t c = t - fld * C, i = c / a.nz, j = c - i * a.nz;
    const double* f = a.f[fld];
    double* lam_f = fld == 0 ? lam_Th : lam_rv;
    const double li = lam_inc[fld * C + c];
    if (li == 0.0) continue;
    const Stencil st = stencil_of(a.flux, a.nx, a.nz, i, j);
    const double ld = factor * li * (-a.dt * a.rdi[c]);   // adjoint of div(c)
    double div = 0.0;
    for (int q = 0; q < 4; ++q) {
      if (st.zero[q]) continue;
      const Dual<4> F = face_flux_of<Dual<4>>(st.u[q], var<4>(f[st.idx[q][0]], 0),
                                              var<4>(f[st.idx[q][1]], 1),
                                              var<4>(f[st.idx[q][2]], 2),
                                              var<4>(f[st.idx[q][3]], 3));
      const double w = (q & 1 ? 1.0 : -1.0) / (q < 2 ? a.dx : a.dz);
      div += w * F.v;
      for (int m = 0; m < 4; ++m)
        if (F.d[m] != 0.0) atomicAdd(lam_f + st.idx[q][m], ld * w * F.d[m]);
    }
    gs += factor * li * (-a.dt * div * a.rdi[c]) / flux_scale;
    if (a.trel) {   // relax_j depends on the column mean of field j
      const double lr = -factor * li * a.dt / (a.trel[j] * (double)a.nx);
      for (int64_t ii = 0; ii < a.nx; ++ii) atomicAdd(lam_f + ii * a.nz + j, lr);
    }
  }
  if (gs != 0.0) atomicAdd(grad_s, gs);
}

// ---- collisions as recorded events (collision/all_or_nothing.py:577-633) ----
struct EvRec {
  int32_t imin, imax, kind, pad;
  double a, b;
};

// one thread per group, the group's records in order, in the collision
// step's own operation order
__global__ void k_ev_forward(const EvRec* ev, const int64_t* off, int64_t G, double* MW,
                             double* MS, double* XI) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G;
       g += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t q = off[g]; q < off[g + 1]; ++q) {
      const EvRec r = ev[q];
      const int32_t imin = r.imin, imax = r.imax;
      if (r.kind == 2) {
        const double p = r.a;
        const double xi_col = p * XI[imin];
        MW[imin] = MW[imin] + p * MW[imax];
        MS[imin] = MS[imin] + p * MS[imax];
        XI[imax] -= xi_col;
      } else if (r.kind == 1) {
        const double xi_min = XI[imin], xi_max = XI[imax];
        const double xi_ges = xi_min + xi_max;
        MW[imin] = 2.0 * (xi_min * MW[imin] + xi_max * MW[imax]) / xi_ges;
        MS[imin] = 2.0 * (xi_min * MS[imin] + xi_max * MS[imax]) / xi_ges;
        MW[imax] = MW[imin];
        MS[imax] = MS[imin];
        XI[imax] = 0.5 * 0.7 * xi_ges;
        XI[imin] = 0.5 * xi_ges - XI[imax];
      } else {
        MW[imin] += MW[imax];
        MS[imin] += MS[imax];
        XI[imax] -= XI[imin];
      }
    }
  }
}

// the transposed maps, records in reverse order
__global__ void k_ev_backward(const EvRec* ev, const int64_t* off, int64_t G, double* LW,
                              double* LS) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G;
       g += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t q = off[g + 1] - 1; q >= off[g]; --q) {
      const EvRec r = ev[q];
      const int32_t imin = r.imin, imax = r.imax;
      if (r.kind == 1) {   // both take 2 (xi_min m_min + xi_max m_max) / xi_ges
        const double xi_ges = r.a + r.b;
        const double cmin = 2.0 * r.a / xi_ges, cmax = 2.0 * r.b / xi_ges;
        const double sw = LW[imin] + LW[imax], ss = LS[imin] + LS[imax];
        LW[imin] = cmin * sw; LW[imax] = cmax * sw;
        LS[imin] = cmin * ss; LS[imax] = cmax * ss;
      } else {   // m_min += f m_max, f = p_crit (kind 2) or 1
        const double f = r.kind == 2 ? r.a : 1.0;
        LW[imax] += f * LW[imin];
        LS[imax] += f * LS[imin];
      }
    }
  }
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
                      double dt, double kappa, double p_ref, double V, int no_iter) {
  Args a;
  a.no_iter = no_iter;
  a.n = n; a.C = C; a.m_w = m_w; a.m_s = m_s; a.xi = xi; a.cell = cell; a.Th = Th; a.r_v = r_v;
  a.rho_d = rho_d; a.mdi = mdi; a.dTh = dTh; a.drv = drv; a.dml = dml; a.dt = dt;
  a.ks = kappa / 0.6;
  a.g.p_ref = p_ref; a.g.p_ref_inv = 1.0 / p_ref; a.g.V = V;
  return a;
}

extern "C" {

int lacmo_adj_forward(int64_t n, int64_t C, double* m_w, const double* m_s, const double* xi,
                      const int32_t* cell, int64_t cell_stride, double* Th, double* r_v,
                      const double* rho_d, const double* mdi, const double* dTh,
                      const double* drv, double* dml, double dt_sub, double kappa, double p_ref,
                      double V, int n_sub, int no_iter, double* tape_m, double* tape_c,
                      void* stream) {
  if (n <= 0 || C <= 0 || !m_w || !m_s || !xi || !cell || !Th || !r_v || !rho_d || !mdi || !dml ||
      n_sub < 0 || cell_stride < 0 || no_iter < 0 || !(kappa > 0.0) || !(p_ref > 0.0))
    return LACMO_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Args a = make_args(n, C, m_w, m_s, xi, cell, Th, r_v, rho_d, mdi, dTh, drv, dml, dt_sub, kappa,
                     p_ref, V, no_iter);
  if (cudaMemsetAsync(dml, 0, 8 * C, s) != cudaSuccess) return LACMO_ERR_CUDA;
  for (int k = 0; k < n_sub; ++k) {
    a.cell = cell + (size_t)k * cell_stride;
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
                       const int32_t* cell, int64_t cell_stride, const double* rho_d,
                       const double* mdi, const double* dTh, const double* drv, double* dml,
                       double dt_sub, double kappa, double p_ref, double V, int n_sub,
                       int no_iter, const double* tape_m, const double* tape_c, double* lam_m,
                       double* lam_Th, double* lam_rv, double* lam_dml, double* grad_ms,
                       double* grad_kappa, double* lam_inc, void* stream) {
  if (n <= 0 || C <= 0 || !m_s || !xi || !cell || !rho_d || !mdi || !dml || n_sub < 0 ||
      cell_stride < 0 || no_iter < 0 || !tape_m || !tape_c || !lam_m || !lam_Th || !lam_rv ||
      !lam_dml || !grad_ms || !grad_kappa || !(kappa > 0.0))
    return LACMO_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Args a = make_args(n, C, nullptr, m_s, xi, cell, nullptr, nullptr, rho_d, mdi, dTh, drv, dml,
                     dt_sub, kappa, p_ref, V, no_iter);
  if (cudaMemsetAsync(dml, 0, 8 * C, s) != cudaSuccess) return LACMO_ERR_CUDA;
  for (int k = n_sub - 1; k >= 0; --k) {
    a.cell = cell + (size_t)k * cell_stride;
    const double* mb = tape_m + (size_t)k * n;
    const double* ma = tape_m + (size_t)(k + 1) * n;
    const double* tc = tape_c + (size_t)k * 2 * C;
    k_bwd_sum_dml<<<nb(n, 128), 128, 0, s>>>(a, mb, ma);
    k_bwd_cells<<<nb(C, 64), 64, 0, s>>>(a, tc, mb, ma, lam_Th, lam_rv, lam_dml, lam_inc);
    k_bwd_sips<<<nb(n, 128), 128, 0, s>>>(a, tc, mb, ma, lam_m, lam_dml, lam_Th, lam_rv, grad_ms,
                                          grad_kappa);
    note_launches(3);
  }
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

static bool inc_args(IncArgs* a, const double* Th, const double* r_v, const double* rdi,
                     const double* flux, int64_t nx, int64_t nz, double dx, double dz,
                     double dt_sub, const double* prof_Th, const double* prof_rv,
                     const double* t_relax) {
  if (!Th || !r_v || !rdi || !flux || nx <= 0 || nz <= 0 || !(dx > 0.0) || !(dz > 0.0))
    return false;
  if (t_relax && (!prof_Th || !prof_rv)) return false;
  a->f[0] = Th; a->f[1] = r_v; a->rdi = rdi; a->flux = flux; a->trel = t_relax;
  a->prof[0] = prof_Th; a->prof[1] = prof_rv;
  a->nx = nx; a->nz = nz; a->dx = dx; a->dz = dz; a->dt = dt_sub;
  return true;
}

int lacmo_adj_increments(const double* Th, const double* r_v, const double* rho_dry_inv,
                         const double* flux, int64_t nx, int64_t nz, double dx, double dz,
                         double dt_sub, const double* prof_Th, const double* prof_rv,
                         const double* t_relax, int second, double* inc_Th, double* inc_rv,
                         void* stream) {
  IncArgs a;
  if (!inc_args(&a, Th, r_v, rho_dry_inv, flux, nx, nz, dx, dz, dt_sub, prof_Th, prof_rv,
                t_relax) || !inc_Th || !inc_rv)
    return LACMO_ERR_ARG;
  k_increments<<<nb(2 * nx * nz, 128), 128, 0, (cudaStream_t)stream>>>(a, second ? 1 : 0,
                                                                       inc_Th, inc_rv);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

int lacmo_adj_increments_vjp(const double* Th, const double* r_v, const double* rho_dry_inv,
                             const double* flux, int64_t nx, int64_t nz, double dx, double dz,
                             double dt_sub, const double* prof_Th, const double* prof_rv,
                             const double* t_relax, double factor, double flux_scale,
                             const double* lam_inc, double* lam_Th, double* lam_rv,
                             double* grad_s, void* stream) {
  IncArgs a;
  if (!inc_args(&a, Th, r_v, rho_dry_inv, flux, nx, nz, dx, dz, dt_sub, prof_Th, prof_rv,
                t_relax) || !lam_inc || !lam_Th || !lam_rv || !grad_s || !(flux_scale > 0.0))
    return LACMO_ERR_ARG;
  k_increments_vjp<<<nb(2 * nx * nz, 128), 128, 0, (cudaStream_t)stream>>>(
      a, factor, flux_scale, lam_inc, lam_Th, lam_rv, grad_s);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

int lacmo_adj_collisions_forward(const void* events, const int64_t* off, int64_t n_groups,
                                 double* m_w, double* m_s, double* xi, void* stream) {
  if (n_groups < 0 || (n_groups > 0 && (!events || !off || !m_w || !m_s || !xi)))
    return LACMO_ERR_ARG;
  if (n_groups == 0) return LACMO_OK;
  k_ev_forward<<<nb(n_groups, 128), 128, 0, (cudaStream_t)stream>>>(
      (const EvRec*)events, off, n_groups, m_w, m_s, xi);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

int lacmo_adj_collisions_backward(const void* events, const int64_t* off, int64_t n_groups,
                                  double* lam_w, double* lam_s, void* stream) {
  if (n_groups < 0 || (n_groups > 0 && (!events || !off || !lam_w || !lam_s)))
    return LACMO_ERR_ARG;
  if (n_groups == 0) return LACMO_OK;
  k_ev_backward<<<nb(n_groups, 128), 128, 0, (cudaStream_t)stream>>>(
      (const EvRec*)events, off, n_groups, lam_w, lam_s);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

}  // extern "C"
