// Device-side FP64 physics of the SIP hot path.
//
// Each function restates the reference formula with the reference's operation
// order (cited per function).  Quantities that depend only on the grid cell
// (surface tension and density of water at T, the linearised Fukuta size
// corrections, the c1/c2 terms of the mass-rate denominator) are evaluated
// once per cell per sub-step in CellAmb instead of once per SIP and Newton
// iteration; they are the same expressions on the same inputs, so the values
// are unchanged.  The radius (m / rho)^(1/3) uses cbrt here (the condensation
// path is compared to the oracle within 1e-10 relative); the bit-exact
// collision path uses the correctly-rounded pow of lacmo_crmath.h instead.
#pragma once
#include <stdint.h>

#include "lacmo_constants.h"

#define LACMO_DEV __device__ __forceinline__

namespace lacmo {

enum { SOL_AS = 0, SOL_NACL = 1 };

struct CellAmb {
  double T, p, S, e_s, L_v, K, D_v;   // grid scalar fields / material properties
  double sigw, rhow;                  // sigma_w(T), rho_w(T)
  double lap0, lbp0;                  // l_alpha(T,p,K), l_beta(T,D_v) (um)
  double c1, c2;                      // mass-rate denominator factors
};

// numpy.maximum / minimum semantics (NaN propagates)
LACMO_DEV double np_max(double a, double b) { return (a >= b || isnan(a)) ? a : b; }
LACMO_DEV double np_min(double a, double b) { return (a <= b || isnan(a)) ? a : b; }
LACMO_DEV double np_sign(double x) { return isnan(x) ? x : (x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0)); }
// Python float modulo (sign of the divisor)
LACMO_DEV double py_mod(double a, double b) {
  // one wrap at most, the common case: the same value fmod gives (b > 0;
  // a - b and a + b are exact or the same single rounding as fmod + b)
  if (b > 0.0) {
    if (a > 0.0 && a < b) return a;
    if (a >= b && a < 2.0 * b) return a - b;
    if (a < 0.0 && a > -b) return a + b;
  }
  double m = fmod(a, b);
  if (m != 0.0) { if ((b < 0) != (m < 0)) m += b; }
  else m = copysign(0.0, b);
  return m;
}

// material_properties.py:31-50
LACMO_DEV double density_water(double T) {
  double d = T - LC_PAR_WATER_DENS_2;
  return LC_PAR_WATER_DENS_0 + LC_PAR_WATER_DENS_1 * (d * d);
}
// material_properties.py:56-85
LACMO_DEV double density_NaCl_solution(double w, double T) {
  return LC_PAR_SOL_DENS_NACL_0 + LC_PAR_SOL_DENS_NACL_1 * w + LC_PAR_SOL_DENS_NACL_2 * T +
         LC_PAR_SOL_DENS_NACL_3 * w * w + LC_PAR_SOL_DENS_NACL_4 * w * T +
         LC_PAR_SOL_DENS_NACL_5 * T * T;
}
// algebra.py:10-34 with the AS density coefficients (material_properties.py:87-115)
LACMO_DEV double poly_rho_AS(double w) {
  double r = LC_PAR_RHO_AS_0 * w + LC_PAR_RHO_AS_1;
  r = r * w + LC_PAR_RHO_AS_2;
  return r * w + LC_PAR_RHO_AS_3;
}
LACMO_DEV double density_AS_solution_rw(double w, double rhow) { return rhow * poly_rho_AS(w); }
// material_properties.py:224-244
LACMO_DEV double surface_tension_water(double T) {
  double tau = 1 - T / 647.096;
  return 0.2358 * pow(tau, 1.256) * (1 - 0.625 * tau);
}
// material_properties.py:346-366 / 272-293 with sigma_w(T) given
LACMO_DEV double surface_tension_AS_sw(double w, double sigw) {
  return sigw * (1.0 + LC_PAR_SIGMA_AS * w / (1. - w));
}
LACMO_DEV double surface_tension_NaCl_sw(double w, double sigw) {
  return sigw * (1.0 + LC_PAR_SIGMA_NACL * w / (1. - w));
}
// microphysics.py:83-100 (condensation path: cbrt, see file comment)
LACMO_DEV double radius_from_mass(double m, double rho) {
  return cbrt(LC_FOUR_PI_OVER_THREE_INV * m / rho);
}

// Cell-constant terms, microphysics.py:989-1017, 1026-1051, 1454-1455
LACMO_DEV CellAmb make_cell_amb(double T, double p, double S, double e_s, double L_v, double K,
                                double D_v) {
  CellAmb a;
  a.T = T; a.p = p; a.S = S; a.e_s = e_s; a.L_v = L_v; a.K = K; a.D_v = D_v;
  a.sigw = surface_tension_water(T);
  a.rhow = density_water(T);
  a.lap0 = (LC_C_ALPHA_1 + LC_C_ALPHA_2 * (T - LC_T_ALPHA_0)) * K / p;
  a.lbp0 = LC_C_BETA_1 * (1.0 + LC_C_BETA_2 * (T - LC_T_ALPHA_0)) * D_v;
  a.c1 = L_v * L_v / (LC_R_V * K * T * T);
  a.c2 = LC_R_V * T / (D_v * e_s);
  return a;
}

// microphysics.py:1359-1469 (AS) and :1239-1353 (NaCl).  T_p equals the cell
// temperature on the particle path, so rho_w(T_p) and sigma_w(T_p) come from
// the cell terms.
LACMO_DEV void mass_rate_and_derivative(int sol, double m_w, double m_s, double w_s, double R_p,
                                        double T_p, double rho_p, double sigma_p,
                                        const CellAmb& a, double& g, double& dg) {
  const double l_alpha_plus_R_p = 1.0E-6 * (R_p + a.lap0);
  const double l_beta_plus_R_p = 1.0E-6 * (R_p + a.lbp0);
  const double m_p_inv_SI = 1.0E18 / (m_w + m_s);
  double drho_dm_over_rho, a_w, da_w_dm, dsigma_dm;
  const double wfac = w_s / ((1. - w_s) * (1. - w_s));
  if (sol == SOL_AS) {
    double pd = LC_PAR_RHO_DERIV_AS_0 * w_s + LC_PAR_RHO_DERIV_AS_1;
    pd = pd * w_s + LC_PAR_RHO_DERIV_AS_2;
    drho_dm_over_rho = -a.rhow * m_p_inv_SI / rho_p * w_s * pd;
    double aw = LC_PAR_WAT_ACT_AS_0 * w_s + LC_PAR_WAT_ACT_AS_1;
    aw = aw * w_s + LC_PAR_WAT_ACT_AS_2; aw = aw * w_s + LC_PAR_WAT_ACT_AS_3;
    a_w = aw * w_s + LC_PAR_WAT_ACT_AS_4;
    double da = LC_PAR_WAT_ACT_DERIV_AS_0 * w_s + LC_PAR_WAT_ACT_DERIV_AS_1;
    da = da * w_s + LC_PAR_WAT_ACT_DERIV_AS_2;
    da = da * w_s + LC_PAR_WAT_ACT_DERIV_AS_3;
    da_w_dm = -m_p_inv_SI * w_s * da;
    dsigma_dm = -LC_PAR_SIGMA_AS * a.sigw * m_p_inv_SI * wfac;
  } else {
    drho_dm_over_rho = -w_s * m_p_inv_SI / rho_p *
                       (LC_PAR_SOL_DENS_NACL_1 + 2.0 * LC_PAR_SOL_DENS_NACL_3 * w_s +
                        LC_PAR_SOL_DENS_NACL_4 * T_p);
    double aw = LC_PAR_WAT_ACT_NACL_0 * w_s + LC_PAR_WAT_ACT_NACL_1;
    aw = aw * w_s + LC_PAR_WAT_ACT_NACL_2; aw = aw * w_s + LC_PAR_WAT_ACT_NACL_3;
    a_w = aw * w_s + LC_PAR_WAT_ACT_NACL_4;
    double da = LC_PAR_WAT_ACT_DERIV_NACL_0 * w_s + LC_PAR_WAT_ACT_DERIV_NACL_1;
    da = da * w_s + LC_PAR_WAT_ACT_DERIV_NACL_2;
    da = da * w_s + LC_PAR_WAT_ACT_DERIV_NACL_3;
    da_w_dm = -m_p_inv_SI * w_s * da;
    dsigma_dm = -LC_PAR_SIGMA_NACL * a.sigw * m_p_inv_SI * wfac;
  }
  const double dR_p_dm_over_R_p = LC_ONE_THIRD * (m_p_inv_SI - drho_dm_over_rho);
  const double dR_p_dm = 1.0E-6 * dR_p_dm_over_R_p * R_p;
  const double eps_k = 2.0E6 * sigma_p / (LC_R_V * T_p * rho_p * R_p);
  const double kelvin_term = exp(eps_k);
  const double S_eq = a_w * kelvin_term;
  const double dSeq_dm =
      da_w_dm * kelvin_term + S_eq * eps_k * (dsigma_dm / sigma_p - drho_dm_over_rho - dR_p_dm_over_R_p);
  const double f3 = 1.0 / ((l_alpha_plus_R_p) * S_eq * a.c1 + (l_beta_plus_R_p) * a.c2);
  const double f1f3 = LC_FOUR_PI * R_p * R_p * f3;
  const double dg1_dm = (dSeq_dm * (l_alpha_plus_R_p) + S_eq * dR_p_dm) * a.c1 + dR_p_dm * a.c2;
  const double f2 = a.S - S_eq;
  g = 1.0E6 * f1f3 * f2;
  dg = 1.0E-12 * f1f3 * (f2 * (2.0 * dR_p_dm_over_R_p - f3 * dg1_dm) - dSeq_dm);
}

// integration.py:728-836.  Efflorescence floor, density and surface tension
// inside the iterations are those of ammonium sulfate for either solute, as in
// the reference.
LACMO_DEV double newton_full(int sol, double dt_sub, int no_iter, double m_w, double m_s,
                             double w_s, double R_p, double T_p, double rho_p, double sigma_p,
                             const CellAmb& a, double* gamma0_out) {
  const double m_w_effl = m_s * (LC_W_S_MAX_AS_INV - 1.0);
  double gamma0, dgdm;
  mass_rate_and_derivative(sol, m_w, m_s, w_s, R_p, T_p, rho_p, sigma_p, a, gamma0, dgdm);
  double x = dt_sub * dgdm;
  double denom_inv = (x < 0.9) ? 1.0 / (1.0 - x) : 10.0;
  double mass_new = np_max(m_w_effl, m_w + dt_sub * gamma0 * denom_inv);
  for (int it = 0; it < no_iter - 1; ++it) {
    const double m_p = mass_new + m_s;
    const double w = m_s / m_p;
    const double rho = density_AS_solution_rw(w, a.rhow);
    const double R = radius_from_mass(m_p, rho);
    const double sig = surface_tension_AS_sw(w, a.sigw);
    double g;
    mass_rate_and_derivative(sol, mass_new, m_s, w, R, T_p, rho, sig, a, g, dgdm);
    x = dt_sub * dgdm;
    denom_inv = (x < 0.9) ? 1.0 / (1.0 - x) : 10.0;
    mass_new += (dt_sub * g + m_w - mass_new) * denom_inv;
    mass_new = np_max(m_w_effl, mass_new);
  }
  if (gamma0_out) *gamma0_out = gamma0;
  return mass_new - m_w;
}

// ---------------------------------------------------------------------------
// Mixed precision: the same Fukuta-Walter mass rate, derivative and implicit
// ---------------------------------------------------------------------------
// FP32 building blocks of the mixed-precision path, on the hardware's special
// function unit (the .approx.ftz forms of rcp, lg2, ex2 and rsqrt, written as
// inline PTX so that no range fix-ups are issued; every argument here is a
// normal float: masses, densities, radii, speeds and Reynolds numbers).  Each
// stays far inside the path's FP32 budget:
//  f_rcp(b): relative error below 2^-23;
//  f_cbrt(x): 2^(log2(x)/3) (relative error near 1e-6), then one Newton step
//    on y^3 = x, which squares it: within a few ulp for x > 0;
//  f_expm1(e): Taylor series to e^8 for |e| <= 0.5 (truncation below 1e-8
//    relative); 2^(e log2 e) - 1 beyond, where there is no cancellation;
//  f_pow(x, y) = 2^(y log2 x) for x > 0 (relative error near 1e-6 for the
//    drag's Reynolds factor, whose exponent is 0.687);
//  f_sqrt(v) = v rsqrt(v) for v > 0 (relative error below 2^-22), 0 else.
LACMO_DEV float f_rcp(float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return r;
}
LACMO_DEV float f_div(float a, float b) { return a * f_rcp(b); }
LACMO_DEV float f_lg2(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
LACMO_DEV float f_ex2(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
LACMO_DEV float f_sqrt(float v) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return v > 0.0f ? v * r : 0.0f;
}
LACMO_DEV float f_cbrt(float x) {
  const float y = f_ex2(f_lg2(x) * (1.0f / 3.0f));
  return (2.0f / 3.0f) * y + (1.0f / 3.0f) * x * f_rcp(y * y);
}
LACMO_DEV float f_expm1(float e) {
  float p = 2.4801587e-05f;                 // 1/8!
  p = p * e + 1.9841270e-04f;               // 1/7!
  p = p * e + 1.3888889e-03f;               // 1/6!
  p = p * e + 8.3333333e-03f;               // 1/5!
  p = p * e + 4.1666667e-02f;               // 1/4!
  p = p * e + 1.6666667e-01f;               // 1/3!
  p = p * e + 0.5f;
  p = p * e + 1.0f;
  return fabsf(e) <= 0.5f ? p * e : f_ex2(e * 1.4426950408889634f) - 1.0f;
}
LACMO_DEV float f_pow(float x, float y) { return f_ex2(y * f_lg2(x)); }

// Conversions between FP64 and FP32 with integer operations: GB300 runs
// FP64 arithmetic and double<->float conversions on a narrow pipe, and the
// mixed kernel converts about a dozen values per SIP.  Branch-free (no call
// on any path, so no register spills around one).
//  d2f_int: for finite x within the FP32 range (positions, velocities,
//    masses, multiplicities), the FP32 value rounded half away from zero on
//    the magnitude (within 1 ulp of the correctly rounded value; the FP32
//    copies only feed approximations with certified margins); below the FP32
//    normal range a signed zero.  A NaN or huge x gives some finite value:
//    the FP32 results then only feed increments that are added to the FP64
//    state, which carries the NaN on.
//  f2d_int: exact for normal floats and zero; FP32 subnormals give a signed
//    zero, infinities and NaNs stay what they are.
LACMO_DEV float d2f_int(double x) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const uint32_t ax = hi & 0x7fffffffu, sign = hi & 0x80000000u;
  // (ax << 3 | lo >> 29) holds the low 9 exponent bits over 23 mantissa bits
  const uint32_t f = ((__funnelshift_l(lo, ax, 3) - (384u << 23)) + ((lo >> 28) & 1u)) | sign;
  return __uint_as_float(ax < (897u << 20) ? sign : f);
}
LACMO_DEV double f2d_int(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t a = b & 0x7fffffffu, sign = b & 0x80000000u;
  const uint32_t hi = ((a >> 3) + (896u << 20)) | sign | (a >= 0x7f800000u ? 0x7ff00000u : 0u);
  const bool tiny = a < 0x00800000u;
  return __hiloint2double((int)(tiny ? sign : hi), (int)(tiny ? 0u : b << 29));
}

// Newton in FP32.  The residual f2 = S_amb - S_eq is formed from the two
// deviations from saturation, S_amb - 1 (exact in FP64, rounded once) and
// S_eq - 1 = (a_w - 1) + a_w (exp(eps_k) - 1) with a_w - 1 from the water-
// activity polynomial without its constant term and expm1, so it carries no
// cancellation; the Newton iterates on the increment dm = m_new - m_w, and the
// new mass m_w + dm is formed in FP64 by the caller.
struct CellAmbF {
  float T, S_m1, sigw, rhow, lap0, lbp0, c1, c2;
};

LACMO_DEV void mass_rate_and_derivative_f(int sol, float m_w, float m_s, float w_s, float R_p,
                                          float rho_p, float sigma_p, float T_p, float rhow_p,
                                          const CellAmbF& a, float& g, float& dg, float& f2o) {
  const float l_alpha_plus_R_p = 1.0E-6f * (R_p + a.lap0);
  const float l_beta_plus_R_p = 1.0E-6f * (R_p + a.lbp0);
  const float m_p_inv_SI = 1.0E18f * f_rcp(m_w + m_s);
  const float inv_1mw = f_rcp(1.f - w_s);
  const float wfac = w_s * inv_1mw * inv_1mw;
  const float inv_rho = f_rcp(rho_p);
  float drho_dm_over_rho, aw_m1, da_w_dm, dsigma_dm;
  if (sol == SOL_AS) {
    const float pd = ((float)LC_PAR_RHO_DERIV_AS_0 * w_s + (float)LC_PAR_RHO_DERIV_AS_1) * w_s +
                     (float)LC_PAR_RHO_DERIV_AS_2;
    drho_dm_over_rho = -rhow_p * m_p_inv_SI * inv_rho * w_s * pd;
    aw_m1 = w_s * ((((float)LC_PAR_WAT_ACT_AS_0 * w_s + (float)LC_PAR_WAT_ACT_AS_1) * w_s +
                    (float)LC_PAR_WAT_ACT_AS_2) * w_s + (float)LC_PAR_WAT_ACT_AS_3);
    const float da = (((float)LC_PAR_WAT_ACT_DERIV_AS_0 * w_s + (float)LC_PAR_WAT_ACT_DERIV_AS_1) *
                          w_s + (float)LC_PAR_WAT_ACT_DERIV_AS_2) * w_s +
                     (float)LC_PAR_WAT_ACT_DERIV_AS_3;
    da_w_dm = -m_p_inv_SI * w_s * da;
    dsigma_dm = -(float)LC_PAR_SIGMA_AS * a.sigw * m_p_inv_SI * wfac;
  } else {
    drho_dm_over_rho = -w_s * m_p_inv_SI * inv_rho *
                       ((float)LC_PAR_SOL_DENS_NACL_1 + 2.0f * (float)LC_PAR_SOL_DENS_NACL_3 * w_s +
                        (float)LC_PAR_SOL_DENS_NACL_4 * T_p);
    aw_m1 = w_s * ((((float)LC_PAR_WAT_ACT_NACL_0 * w_s + (float)LC_PAR_WAT_ACT_NACL_1) * w_s +
                    (float)LC_PAR_WAT_ACT_NACL_2) * w_s + (float)LC_PAR_WAT_ACT_NACL_3);
    const float da = (((float)LC_PAR_WAT_ACT_DERIV_NACL_0 * w_s +
                       (float)LC_PAR_WAT_ACT_DERIV_NACL_1) * w_s +
                      (float)LC_PAR_WAT_ACT_DERIV_NACL_2) * w_s +
                     (float)LC_PAR_WAT_ACT_DERIV_NACL_3;
    da_w_dm = -m_p_inv_SI * w_s * da;
    dsigma_dm = -(float)LC_PAR_SIGMA_NACL * a.sigw * m_p_inv_SI * wfac;
  }
  const float dR_p_dm_over_R_p = (1.0f / 3.0f) * (m_p_inv_SI - drho_dm_over_rho);
  const float dR_p_dm = 1.0E-6f * dR_p_dm_over_R_p * R_p;
  const float eps_k = 2.0E6f * sigma_p * inv_rho * f_rcp((float)LC_R_V * T_p * R_p);
  const float em1 = f_expm1(eps_k);
  const float kelvin_term = 1.0f + em1;
  const float Seq_m1 = aw_m1 + (1.0f + aw_m1) * em1;
  const float S_eq = 1.0f + Seq_m1;
  const float dSeq_dm = da_w_dm * kelvin_term +
                        S_eq * eps_k *
                            (dsigma_dm * f_rcp(sigma_p) - drho_dm_over_rho - dR_p_dm_over_R_p);
  const float f3 = f_rcp(l_alpha_plus_R_p * S_eq * a.c1 + l_beta_plus_R_p * a.c2);
  const float f1f3 = (float)LC_FOUR_PI * R_p * R_p * f3;
  const float dg1_dm = (dSeq_dm * l_alpha_plus_R_p + S_eq * dR_p_dm) * a.c1 + dR_p_dm * a.c2;
  const float f2 = a.S_m1 - Seq_m1;
  g = 1.0E6f * f1f3 * f2;
  dg = 1.0E-12f * f1f3 * (f2 * (2.0f * dR_p_dm_over_R_p - f3 * dg1_dm) - dSeq_dm);
  f2o = f2;
}

// The FP32 Newton of integration.py:728-836 on the increment d = m_new - m_w
// (m_w32 = m_w rounded), with the ammonium-sulfate density and surface
// tension inside the iterations as the reference hard-wires them.  Returns
// false when a residual came near the critical radius (|f2| < 1e-6 with
// |dt gamma'| < 0.5), where the caller repeats the solve in FP64.
LACMO_DEV bool newton_mixed_f(int sol, float dt_sub, int no_iter, float m_w32, float m_s,
                              float w_s, float R_p, float T_p, float rho_p, float sigma_p,
                              const CellAmbF& a, float d_effl, float* d_out) {
  float g, dg, f2;
  mass_rate_and_derivative_f(sol, m_w32, m_s, w_s, R_p, rho_p, sigma_p, T_p, a.rhow, a, g, dg, f2);
  float x = dt_sub * dg;
  bool near_crit = (fabsf(f2) < 1.0e-6f) && (fabsf(x) < 0.5f);
  float denom_inv = (x < 0.9f) ? f_rcp(1.0f - x) : 10.0f;
  const float d0 = dt_sub * g * denom_inv;
  float d = (d0 != d0) ? d0 : fmaxf(d_effl, d0);
  for (int it = 0; it < no_iter - 1; ++it) {
    const float mass = m_w32 + d;
    const float m_p = mass + m_s;
    const float w = m_s * f_rcp(m_p);
    const float pr = (((float)LC_PAR_RHO_AS_0 * w + (float)LC_PAR_RHO_AS_1) * w +
                      (float)LC_PAR_RHO_AS_2) * w + (float)LC_PAR_RHO_AS_3;
    const float rho = a.rhow * pr;
    const float R = f_cbrt((float)LC_FOUR_PI_OVER_THREE_INV * m_p * f_rcp(rho));
    const float sig = a.sigw * (1.0f + (float)LC_PAR_SIGMA_AS * w * f_rcp(1.f - w));
    mass_rate_and_derivative_f(sol, mass, m_s, w, R, rho, sig, T_p, a.rhow, a, g, dg, f2);
    x = dt_sub * dg;
    near_crit = near_crit || ((fabsf(f2) < 1.0e-6f) && (fabsf(x) < 0.5f));
    denom_inv = (x < 0.9f) ? f_rcp(1.0f - x) : 10.0f;
    d += (dt_sub * g - d) * denom_inv;
    d = (d != d) ? d : fmaxf(d_effl, d);
  }
  *d_out = d;
  return !near_crit;
}

// grid.py:195-323: staggered bilinear interpolation; index -1 wraps onto the
// last column of the (nx+1)-wide staggered arrays, as NumPy indexing does.
struct GridVel {
  const double* gv;
  int64_t nx, nz;
  LACMO_DEV double at(int c, int64_t i, int64_t j) const {
    if (i < 0) i += nx + 1;
    if (j < 0) j += nz + 1;
    return __ldg(gv + ((int64_t)c * (nx + 1) + i) * (nz + 1) + j);
  }
  LACMO_DEV double bilin(int c, int64_t i, int64_t j, double a, double b) const {
    return a * (b * at(c, i + 1, j + 1) + (1 - b) * at(c, i + 1, j)) +
           (1 - a) * (b * at(c, i, j + 1) + (1 - b) * at(c, i, j));
  }
  LACMO_DEV void interp(int64_t i, int64_t j, double wx, double wy, double& u, double& v) const {
    if ((j == 0 && wy <= 0.5) || (j == nz - 1 && wy >= 0.5)) {
      u = wx * at(0, i + 1, j) + (1 - wx) * at(0, i, j);
    } else if (wy > 0.5) {
      u = bilin(0, i, j, wx, wy - 0.5);
    } else {
      u = bilin(0, i, j - 1, wx, wy + 0.5);
    }
    if (wx > 0.5) v = bilin(1, i, j, wx - 0.5, wy);
    else v = bilin(1, i - 1, j, wx + 0.5, wy);
  }
};

}  // namespace lacmo
