/*
 * CPU oracle for the LacmoPy per-timestep super-droplet (SIP) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates the reference algorithm in
 * plain C so that the CUDA path can be checked against it (tests/, the smoke
 * check and the CPU-baseline leg of bench.py).  It is never linked into the
 * product library.
 *
 * Every function follows the reference's floating-point operation order
 * (built with -ffp-contract=off; no FMA contraction, IEEE double), citing the
 * reference file:line it restates.  Build variants (see oracle/Makefile):
 *   ORC_SQUARE_POW   : x**2 evaluates as pow(x, 2.0) like CPython does when the
 *                      reference runs with Numba stubbed out; otherwise x*x as
 *                      Numba compiles it.  Used to pin the oracle bit-for-bit
 *                      against the golden fixtures made by the reference.
 *   ORC_CRMATH       : the collision path's radius pow(x, 1/3) and kernel-bin
 *                      log are correctly rounded (the oracle's own binary128
 *                      evaluation, rounded once), instead of glibc libm.
 *                      Collision outputs of the GPU, whose math is correctly
 *                      rounded, equal this variant bit for bit.
 * Sums that the reference accumulates sequentially in SIP-ID order
 * (delta_m_l per cell, water_removed) are accumulated in that order here too,
 * also when OpenMP runs the per-SIP work in parallel.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../lacmopy_gb300/csrc/lacmo_constants.h"

#ifdef ORC_CRMATH
/* Correctly rounded log and pow for the collision path, the oracle's own:
   evaluated in IEEE binary128 (113-bit significand; __float128 with
   libquadmath on x86-64, long double on AArch64 Linux) and rounded once to
   double.  The binary128 result is within a few of its ulps (2^-112
   relative) of the exact value, so the rounding is the correct one unless the
   exact value lies within about 2^-100 of a midpoint of two doubles, which
   *hard reports. */
#include <float.h>
#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 orc_quad;
#define ORC_QLOG(x) logq(x)
#define ORC_QPOW(x, y) powq(x, y)
#define ORC_QFABS(x) fabsq(x)
#elif defined(__aarch64__) && LDBL_MANT_DIG == 113
typedef long double orc_quad;
#define ORC_QLOG(x) logl(x)
#define ORC_QPOW(x, y) powl(x, y)
#define ORC_QFABS(x) fabsl(x)
#else
#error "the correctly rounded oracle variant needs binary128 arithmetic"
#endif
static double orc_round_quad(orc_quad v, int* hard) {
  const double d = (double)v;
  if (hard) *hard = 0;
  if (hard && isfinite(d) && d != 0.0) {
    const double up = nextafter(d, INFINITY), dn = nextafter(d, -INFINITY);
    const orc_quad mid_up = ((orc_quad)d + (orc_quad)up) / 2, mid_dn = ((orc_quad)d + (orc_quad)dn) / 2;
    const orc_quad tol = ORC_QFABS(v) * (orc_quad)0x1p-100;
    if (ORC_QFABS(v - mid_up) <= tol || ORC_QFABS(v - mid_dn) <= tol) *hard = 1;
  }
  return d;
}
static double orc_cr_log(double x, int* hard) { return orc_round_quad(ORC_QLOG((orc_quad)x), hard); }
static double orc_cr_pow(double x, double y, int* hard) {
  return orc_round_quad(ORC_QPOW((orc_quad)x, (orc_quad)y), hard);
}
#define COL_POW13(x) orc_cr_pow(x, LC_ONE_THIRD, NULL)
#define COL_LOG(x) orc_cr_log(x, NULL)
#else
#define COL_POW13(x) pow(x, LC_ONE_THIRD)
#define COL_LOG(x) log(x)
#endif

#ifdef ORC_SQUARE_POW
#define SQ(x) pow((x), 2.0)
#define POW4(x) pow((x), 4.0)
#else
static inline double sq_(double x) { return x * x; }
static inline double pow4_(double x) { double a = x * x; return a * a; }
#define SQ(x) sq_(x)
#define POW4(x) pow4_(x)
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

enum { SOL_AS = 0, SOL_NACL = 1 };

/* numpy.maximum / numpy.minimum: NaN propagates */
static inline double np_max(double a, double b) { return (a >= b || isnan(a)) ? a : b; }
static inline double np_min(double a, double b) { return (a <= b || isnan(a)) ? a : b; }
static inline double np_sign(double x) { return isnan(x) ? x : (x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0)); }
/* Python float modulo: result has the sign of the divisor */
static inline double py_mod(double a, double b) {
  double m = fmod(a, b);
  if (m != 0.0) { if ((b < 0) != (m < 0)) m += b; }
  else m = copysign(0.0, b);
  return m;
}
/* float -> int64 as compiled code on x86-64 does it (cvttsd2si): truncation
   toward zero, and INT64_MIN for NaN or out-of-range values */
static inline int64_t trunc_i64(double x) {
  if (!(x > -9.2233720368547758e18 && x < 9.2233720368547758e18)) return INT64_MIN;
  return (int64_t)x;
}

/* algebra.py:10-34 */
static inline double poly4(const double* p, double x) {   /* 4 coefficients */
  double r = p[0] * x + p[1];
  r = r * x + p[2];
  r = r * x + p[3];
  return r;
}
static inline double poly5(const double* p, double x) {
  double r = p[0] * x + p[1];
  r = r * x + p[2]; r = r * x + p[3]; r = r * x + p[4];
  return r;
}
static inline double poly3(const double* p, double x) {
  double r = p[0] * x + p[1];
  r = r * x + p[2];
  return r;
}

static const double PAR_RHO_AS[4] = {LC_PAR_RHO_AS_0, LC_PAR_RHO_AS_1, LC_PAR_RHO_AS_2, LC_PAR_RHO_AS_3};
static const double PAR_RHO_DERIV_AS[3] = {LC_PAR_RHO_DERIV_AS_0, LC_PAR_RHO_DERIV_AS_1, LC_PAR_RHO_DERIV_AS_2};
static const double PAR_WAT_ACT_AS[5] = {LC_PAR_WAT_ACT_AS_0, LC_PAR_WAT_ACT_AS_1, LC_PAR_WAT_ACT_AS_2, LC_PAR_WAT_ACT_AS_3, LC_PAR_WAT_ACT_AS_4};
static const double PAR_WAT_ACT_DERIV_AS[4] = {LC_PAR_WAT_ACT_DERIV_AS_0, LC_PAR_WAT_ACT_DERIV_AS_1, LC_PAR_WAT_ACT_DERIV_AS_2, LC_PAR_WAT_ACT_DERIV_AS_3};
static const double PAR_WAT_ACT_NACL[5] = {LC_PAR_WAT_ACT_NACL_0, LC_PAR_WAT_ACT_NACL_1, LC_PAR_WAT_ACT_NACL_2, LC_PAR_WAT_ACT_NACL_3, LC_PAR_WAT_ACT_NACL_4};
static const double PAR_WAT_ACT_DERIV_NACL[4] = {LC_PAR_WAT_ACT_DERIV_NACL_0, LC_PAR_WAT_ACT_DERIV_NACL_1, LC_PAR_WAT_ACT_DERIV_NACL_2, LC_PAR_WAT_ACT_DERIV_NACL_3};

/* material_properties.py:31-50 */
static inline double density_water(double T) {
  return LC_PAR_WATER_DENS_0 + LC_PAR_WATER_DENS_1 * SQ(T - LC_PAR_WATER_DENS_2);
}
/* material_properties.py:56-85 */
static inline double density_NaCl_solution(double w, double T) {
  return LC_PAR_SOL_DENS_NACL_0 + LC_PAR_SOL_DENS_NACL_1 * w + LC_PAR_SOL_DENS_NACL_2 * T
       + LC_PAR_SOL_DENS_NACL_3 * w * w + LC_PAR_SOL_DENS_NACL_4 * w * T
       + LC_PAR_SOL_DENS_NACL_5 * T * T;
}
/* material_properties.py:89-115 */
static inline double density_AS_solution(double w, double T) {
  return density_water(T) * poly4(PAR_RHO_AS, w);
}
/* material_properties.py:224-244 */
static inline double surface_tension_water(double T) {
  double tau = 1 - T / 647.096;
  return 0.2358 * pow(tau, 1.256) * (1 - 0.625 * tau);
}
/* material_properties.py:272-293 */
static inline double surface_tension_NaCl(double w, double T) {
  return surface_tension_water(T) * (1.0 + LC_PAR_SIGMA_NACL * w / (1. - w));
}
/* material_properties.py:346-366 */
static inline double surface_tension_AS(double w, double T) {
  return surface_tension_water(T) * (1.0 + LC_PAR_SIGMA_AS * w / (1. - w));
}
/* microphysics.py:83-100 (Numba / glibc pow) */
static inline double radius_from_mass(double m, double rho) {
  return pow(LC_FOUR_PI_OVER_THREE_INV * m / rho, LC_ONE_THIRD);
}
/* the same on the collision path, with the selectable pow */
static inline double radius_from_mass_col(double m, double rho) {
  return COL_POW13(LC_FOUR_PI_OVER_THREE_INV * m / rho);
}
/* microphysics.py:179-266 */
static inline void R_ws_rho(int sol, double m_w, double m_s, double T, double* R, double* ws, double* rho) {
  double m_p = m_w + m_s;
  double w = m_s / m_p;
  double r = (sol == SOL_AS) ? density_AS_solution(w, T) : density_NaCl_solution(w, T);
  *ws = w; *rho = r; *R = radius_from_mass(m_p, r);
}
/* microphysics.py:989-1017, 1026-1051 */
static inline double l_alpha_lin(double T, double p, double K) {
  return (LC_C_ALPHA_1 + LC_C_ALPHA_2 * (T - LC_T_ALPHA_0)) * K / p;
}
static inline double l_beta_lin(double T, double D_v) {
  return LC_C_BETA_1 * (1.0 + LC_C_BETA_2 * (T - LC_T_ALPHA_0)) * D_v;
}

/* microphysics.py:1359-1469 (AS) and 1239-1353 (NaCl): Fukuta-Walter mass
   rate gamma (fg/s) and its analytic derivative d gamma / d m_w (1/s) */
static void mass_rate_and_derivative(int sol, double m_w, double m_s, double w_s, double R_p,
                                     double T_p, double rho_p, double T_amb, double p_amb,
                                     double S_amb, double e_s_amb, double L_v, double K,
                                     double D_v, double sigma_p, double* g, double* dg) {
  double l_alpha_plus_R_p = 1.0E-6 * (R_p + l_alpha_lin(T_amb, p_amb, K));
  double l_beta_plus_R_p = 1.0E-6 * (R_p + l_beta_lin(T_amb, D_v));
  double m_p_inv_SI = 1.0E18 / (m_w + m_s);
  double drho_dm_over_rho, a_w, da_w_dm, dsigma_dm;
  if (sol == SOL_AS) {
    drho_dm_over_rho = -density_water(T_p) * m_p_inv_SI / rho_p * w_s * poly3(PAR_RHO_DERIV_AS, w_s);
  } else {
    drho_dm_over_rho = -w_s * m_p_inv_SI / rho_p
                       * (LC_PAR_SOL_DENS_NACL_1 + 2.0 * LC_PAR_SOL_DENS_NACL_3 * w_s
                          + LC_PAR_SOL_DENS_NACL_4 * T_p);
  }
  double dR_p_dm_over_R_p = LC_ONE_THIRD * (m_p_inv_SI - drho_dm_over_rho);
  double dR_p_dm = 1.0E-6 * dR_p_dm_over_R_p * R_p;
  double eps_k = 2.0E6 * sigma_p / (LC_R_V * T_p * rho_p * R_p);
  double kelvin_term = exp(eps_k);
  if (sol == SOL_AS) {
    a_w = poly5(PAR_WAT_ACT_AS, w_s);
    da_w_dm = -m_p_inv_SI * w_s * poly4(PAR_WAT_ACT_DERIV_AS, w_s);
    dsigma_dm = -LC_PAR_SIGMA_AS * surface_tension_water(T_p) * m_p_inv_SI * (w_s / ((1. - w_s) * (1. - w_s)));
  } else {
    a_w = poly5(PAR_WAT_ACT_NACL, w_s);
    da_w_dm = -m_p_inv_SI * w_s * poly4(PAR_WAT_ACT_DERIV_NACL, w_s);
    dsigma_dm = -LC_PAR_SIGMA_NACL * surface_tension_water(T_p) * m_p_inv_SI * (w_s / ((1. - w_s) * (1. - w_s)));
  }
  double S_eq = a_w * kelvin_term;
  double dSeq_dm = da_w_dm * kelvin_term
                   + S_eq * eps_k * (dsigma_dm / sigma_p - drho_dm_over_rho - dR_p_dm_over_R_p);
  double c1 = L_v * L_v / (LC_R_V * K * T_amb * T_amb);
  double c2 = LC_R_V * T_amb / (D_v * e_s_amb);
  double f3 = 1.0 / ((l_alpha_plus_R_p) * S_eq * c1 + (l_beta_plus_R_p) * c2);
  double f1f3 = LC_FOUR_PI * R_p * R_p * f3;
  double dg1_dm = (dSeq_dm * (l_alpha_plus_R_p) + S_eq * dR_p_dm) * c1 + dR_p_dm * c2;
  double f2 = S_amb - S_eq;
  *g = 1.0E6 * f1f3 * f2;
  *dg = 1.0E-12 * f1f3 * (f2 * (2.0 * dR_p_dm_over_R_p - f3 * dg1_dm) - dSeq_dm);
}

/* integration.py:728-836: implicit Newton for the condensed mass; the
   efflorescence floor and the in-iteration density / surface tension are
   those of ammonium sulfate whatever the solute (as in the reference) */
static void newton_full(int sol, double dt_sub, int no_iter, double m_w, double m_s, double w_s,
                        double R_p, double T_p, double rho_p, double T_amb, double p_amb,
                        double S_amb, double e_s_amb, double L_v, double K, double D_v,
                        double sigma_p, double* dm, double* gamma0_out) {
  double m_w_effl = m_s * (LC_W_S_MAX_AS_INV - 1.0);
  double gamma0, dgdm;
  mass_rate_and_derivative(sol, m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb,
                           L_v, K, D_v, sigma_p, &gamma0, &dgdm);
  double x = dt_sub * dgdm;
  double denom_inv = (x < 0.9) ? 1.0 / (1.0 - x) : 10.0;
  double mass_new = np_max(m_w_effl, m_w + dt_sub * gamma0 * denom_inv);
  for (int it = 0; it < no_iter - 1; ++it) {
    double m_p = mass_new + m_s;
    double w = m_s / m_p;
    double rho = density_AS_solution(w, T_p);
    double R = radius_from_mass(m_p, rho);
    double sig = surface_tension_AS(w, T_p);
    double g;
    mass_rate_and_derivative(sol, mass_new, m_s, w, R, T_p, rho, T_amb, p_amb, S_amb, e_s_amb,
                             L_v, K, D_v, sig, &g, &dgdm);
    x = dt_sub * dgdm;
    denom_inv = (x < 0.9) ? 1.0 / (1.0 - x) : 10.0;
    mass_new += (dt_sub * g + m_w - mass_new) * denom_inv;
    mass_new = np_max(m_w_effl, mass_new);
  }
  *dm = mass_new - m_w;
  *gamma0_out = gamma0;
}

ORC_EXPORT void orc_mass_rate_and_derivative(int sol, int64_t n, const double* m_w, const double* m_s,
    const double* w_s, const double* R_p, const double* T_p, const double* rho_p,
    const double* T_amb, const double* p_amb, const double* S_amb, const double* e_s_amb,
    const double* L_v, const double* K, const double* D_v, const double* sigma_p,
    double* g, double* dg) {
  for (int64_t i = 0; i < n; ++i)
    mass_rate_and_derivative(sol, m_w[i], m_s[i], w_s[i], R_p[i], T_p[i], rho_p[i], T_amb[i],
                             p_amb[i], S_amb[i], e_s_amb[i], L_v[i], K[i], D_v[i], sigma_p[i],
                             &g[i], &dg[i]);
}

ORC_EXPORT void orc_newton_full(int sol, int64_t n, double dt_sub, int no_iter, const double* m_w,
    const double* m_s, const double* w_s, const double* R_p, const double* T_p, const double* rho_p,
    const double* T_amb, const double* p_amb, const double* S_amb, const double* e_s_amb,
    const double* L_v, const double* K, const double* D_v, const double* sigma_p,
    double* dm, double* g0) {
  for (int64_t i = 0; i < n; ++i)
    newton_full(sol, dt_sub, no_iter, m_w[i], m_s[i], w_s[i], R_p[i], T_p[i], rho_p[i], T_amb[i],
                p_amb[i], S_amb[i], e_s_amb[i], L_v[i], K[i], D_v[i], sigma_p[i], &dm[i], &g0[i]);
}

ORC_EXPORT void orc_R_ws_rho(int sol, int64_t n, const double* m_w, const double* m_s,
                             const double* T_p, double* R, double* ws, double* rho) {
  for (int64_t i = 0; i < n; ++i) R_ws_rho(sol, m_w[i], m_s[i], T_p[i], &R[i], &ws[i], &rho[i]);
}

ORC_EXPORT void orc_surface_tension(int sol, int64_t n, const double* w_s, const double* T_p, double* out) {
  for (int64_t i = 0; i < n; ++i)
    out[i] = (sol == SOL_AS) ? surface_tension_AS(w_s[i], T_p[i]) : surface_tension_NaCl(w_s[i], T_p[i]);
}

/* ---------------------------------------------------------------------- */
/* grid.py:195-323: staggered bilinear velocity interpolation.  Index -1
   (cell 0, left half) wraps onto the last column of the (Nx+1)-wide array.
   For inactive SIPs (j < 0) the reference keeps the previous SIP's (u, v);
   the value is never used, and here (u, v) carries over the same way.     */
#define GV(c, i, j) gv[((int64_t)(c) * (Nx + 1) + (i)) * (Nz + 1) + (j)]
static inline int64_t wrapx(int64_t i, int64_t Nx) { return i < 0 ? i + Nx + 1 : i; }
static inline int64_t wrapz(int64_t j, int64_t Nz) { return j < 0 ? j + Nz + 1 : j; }
static inline double bilin(const double* gv, int c, int64_t Nx, int64_t Nz, int64_t i, int64_t j, double a, double b) {
  int64_t i0 = wrapx(i, Nx), i1 = wrapx(i + 1, Nx), j0 = wrapz(j, Nz), j1 = wrapz(j + 1, Nz);
  return a * (b * GV(c, i1, j1) + (1 - b) * GV(c, i1, j0)) + (1 - a) * (b * GV(c, i0, j1) + (1 - b) * GV(c, i0, j0));
}
ORC_EXPORT void orc_interpolate_velocity(const int64_t* cells, const double* rel_pos, const double* gv,
                                         int64_t Nx, int64_t Nz, int64_t n, double* out) {
  double u = 0., v = 0.;
  for (int64_t k = 0; k < n; ++k) {
    int64_t i = cells[k], j = cells[n + k];
    double wx = rel_pos[k], wy = rel_pos[n + k];
    if (j >= 0) {
      if ((j == 0 && wy <= 0.5) || (j == Nz - 1 && wy >= 0.5)) {
        u = wx * GV(0, wrapx(i + 1, Nx), j) + (1 - wx) * GV(0, wrapx(i, Nx), j);
      } else {
        if (wy > 0.5) u = bilin(gv, 0, Nx, Nz, i, j, wx, wy - 0.5);
        else u = bilin(gv, 0, Nx, Nz, i, j - 1, wx, wy + 0.5);
      }
      if (wx > 0.5) v = bilin(gv, 1, Nx, Nz, i, j, wx - 0.5, wy);
      else v = bilin(gv, 1, Nx, Nz, i - 1, j, wx + 0.5, wy);
    }
    out[k] = u; out[n + k] = v;
  }
}

/* ---------------------------------------------------------------------- */
/* collision/kernel.py:107-167: Beard (1976) terminal velocity, R in um */
static const double P1_BEARD[7] = {-0.327815e-5, 0.855176e-4, -0.578878e-3, -0.987059e-3,
                                   -0.153193e-2, 0.992696, -0.318657e1};
static const double P2_BEARD[6] = {0.238449e-2, -0.542819e-1, 0.475294, -0.204914e1,
                                   0.523778e1, -0.500015e1};
static double polyn(const double* p, int n, double x) {
  double r = p[0] * x + p[1];
  for (int k = 2; k < n; ++k) r = r * x + p[k];
  return r;
}
static double terminal_velocity_Beard(double R) {
  const double rho_w = 1.0E3, rho_a = 1.225, visc = 1.818E-5, sigma = 73.0E-3;
  const double R_0 = 10.0, R_1 = 535.0, R_max = 3500.0, g = 9.80665;
  const double drho = rho_w - rho_a;
  double v;
  if (R < R_0) {
    double l0 = 6.62E-2;
    double C1 = drho * g / (4.5 * visc);
    double C_sc = 1.0 + 1.257 * l0 / R;
    v = C1 * C_sc * R * R * 1.0E-12;
  } else if (R < R_1) {
    double N_Da = 32.0E-18 * R * R * R * rho_a * drho * g / (3.0 * visc * visc);
    double Y = log(N_Da);
    Y = polyn(P1_BEARD, 7, Y);
    double l0 = 6.62E-2;
    double C_sc = 1.0 + 1.257 * l0 / R;
    v = visc * C_sc * exp(Y) / (rho_a * R * 2.0E-6);
  } else if (R < R_max) {
    double N_Bo = 16.0E-12 * R * R * drho * g / (3.0 * sigma);
    double N_P16 = pow(sigma * sigma * sigma * rho_a * rho_a / (POW4(visc) * drho * g), 1.0 / 6.0);
    double Y = log(N_Bo * N_P16);
    Y = polyn(P2_BEARD, 6, Y);
    v = visc * N_P16 * exp(Y) / (rho_a * R * 2.0E-6);
  } else v = 9.04929248;
  return v;
}
/* collision/kernel.py:193-210 */
ORC_EXPORT void orc_update_velocity_Beard(double* vel, const double* R, int64_t n) {
  for (int64_t i = 0; i < n; ++i) vel[i] = terminal_velocity_Beard(R[i]);
}

/* Philox4x32-10 (Salmon et al., SC'11) uniform double with 53 random bits;
   the same generator and counter layout as the GPU kernels use when no draw
   buffer is given: key = seed; pair rank k reads block (k >> 1, collision
   step << 32 | cell) and takes (x0 >> 5, x1 >> 6) for even k, (x2 >> 5,
   x3 >> 6) for odd k. */
static uint32_t mulhi32(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
static double philox_uniform(uint64_t key, uint64_t k, uint64_t c1) {
  const uint64_t c0 = k >> 1;
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  uint32_t x0 = (uint32_t)c0, x1 = (uint32_t)(c0 >> 32), x2 = (uint32_t)c1, x3 = (uint32_t)(c1 >> 32);
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = mulhi32(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
    uint32_t hi1 = mulhi32(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
    uint32_t y0 = hi1 ^ x1 ^ k0, y1 = lo1, y2 = hi0 ^ x3 ^ k1, y3 = lo0;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  uint64_t a = (k & 1) ? (x2 >> 5) : (x0 >> 5), b = (k & 1) ? (x3 >> 6) : (x1 >> 6);
  return (double)(a * 67108864ull + b) * (1.0 / 9007199254740992.0);
}

/* ---- thinned Philox draws (the draw definition of the GPU collision step,
   restated here from its description) ----
   The SIP slots of a cell form blocks of ORC_THIN_L; the pairs (i, j) of row
   i with j in block b form a segment, taken in lexicographic order.  The
   unprocessed part of a segment (pairs (i, j .. jend-1), part counter sub)
   is bounded by Q >= p_crit of all its pairs from FP32 copies of SIP i and
   the block's statistics.  Q >= ORC_THIN_TAU or no valid bound: per-pair
   draws for the rest of the segment.  Otherwise q = 2^-e >= Q, m remaining
   pairs: one uniform decides whether some draw of the part falls below q
   (probability H(e, m) = 1 - (1 - q)^m); if none does the segment is done;
   else the first such pair h is drawn from its conditional law (pair g of r
   remaining is first with probability P(e, r) = q / H(e, r)), its draw is
   q u, and the pairs after h form part sub + 1.  The bound uses IEEE single
   +, -, * and comparisons only, in a fixed order.  Uniforms: Philox4x32-10
   of key = seed, counter (2^62 | chunk << 20 | sub << 8 | j, c1), the 53
   bits (x0 >> 5) 2^26 + (x1 >> 6). */
#define ORC_THIN_L 32
#define ORC_THIN_E_MIN 2
#define ORC_THIN_E_MAX 127
#define ORC_THIN_NE (ORC_THIN_E_MAX - ORC_THIN_E_MIN + 1)
#define ORC_THIN_TAU 0x1p-6f

static uint32_t th_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float th_float(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static float th_max(float a, float b) { return a > b ? a : b; }
static float th_min(float a, float b) { return a < b ? a : b; }
static float th_abs(float a) { return a < 0.0f ? -a : a; }

/* FP32 cube root: exponent-thirding first guess, three Newton steps */
static float th_cbrtf(float x) {
  float y = th_float(th_bits(x) / 3u + 0x2a5137a0u);
  for (int it = 0; it < 3; ++it) y = (y + y + x / (y * y)) / 3.0f;
  return y;
}

typedef struct {
  float xmax, Rmax, umin, umax, wmin, wmax;
  int ok;
} th_block_t;

static void th_block_stats(const float* x, const float* R, const float* u, const float* w,
                           int64_t lo, int64_t hi, th_block_t* s) {
  s->xmax = 0.0f;
  s->Rmax = 0.0f;
  s->umin = INFINITY; s->wmin = INFINITY;
  s->umax = -INFINITY; s->wmax = -INFINITY;
  s->ok = 1;
  for (int64_t q = lo; q < hi; ++q) {
    if (!(x[q] > 0.0f) || isnan(R[q]) || isnan(u[q]) || isnan(w[q])) s->ok = 0;
    s->xmax = th_max(s->xmax, x[q]);
    s->Rmax = th_max(s->Rmax, R[q]);
    s->umin = th_min(s->umin, u[q]);
    s->umax = th_max(s->umax, u[q]);
    s->wmin = th_min(s->wmin, w[q]);
    s->wmax = th_max(s->wmax, w[q]);
  }
}

/* Q >= p_crit of SIP a against every SIP of the block: the largest
   multiplicity, the sum of radii squared, the largest velocity difference and
   the row's largest efficiency, each at least the pair's own, with slack for
   the FP32 copies (velocities 2^-21 sum |u|, |w|; roundings 2^-14 relative,
   1e-36 absolute); negative: no valid bound */
static float th_bound(float xa, float Ra, float ua, float wa, const th_block_t* s, float er,
                      float dtdv) {
  if (!s->ok || !(xa > 0.0f) || isnan(Ra) || isnan(ua) || isnan(wa)) return -1.0f;
  const float du = th_max(ua - s->umin, s->umax - ua);
  const float dw = th_max(wa - s->wmin, s->wmax - wa);
  const float um = th_max(th_abs(s->umin), th_abs(s->umax));
  const float wm = th_max(th_abs(s->wmin), th_abs(s->wmax));
  const float slack = 0x1p-21f * (((th_abs(ua) + um) + th_abs(wa)) + wm);
  const float rs = Ra + s->Rmax;
  const float core = ((((th_max(xa, s->xmax) * dtdv) * 3.14159265e-12f) * rs) * rs) * er;
  if (!(core >= 1e-30f)) return isnan(core) ? -1.0f : 1e-27f;
  const float pb = ((core * ((du + dw) + slack)) * (1.0f + 0x1p-14f)) + 1e-36f;
  return isnan(pb) ? -1.0f : pb;
}

/* e of the smallest q = 2^-e >= Q, clamped to the table */
static int th_exponent(float Q) {
  int E;
  const float f = frexpf(Q, &E);   /* Q = f 2^E, f in [0.5, 1) */
  int e = (f == 0.5f) ? 1 - E : -E;
  if (e < ORC_THIN_E_MIN) e = ORC_THIN_E_MIN;
  if (e > ORC_THIN_E_MAX) e = ORC_THIN_E_MAX;
  return e;
}

static void philox_block(uint64_t key, uint64_t c0, uint64_t c1, uint32_t* out);
static uint64_t th_u53(uint64_t key, uint64_t chunk, uint32_t sub, uint32_t j, uint64_t c1) {
  uint32_t x[4];
  philox_block(key, (1ull << 62) | (chunk << 20) | ((uint64_t)sub << 8) | (uint64_t)j, c1, x);
  return ((uint64_t)(x[0] >> 5) << 26) + (uint64_t)(x[1] >> 6);
}

/* H(e, m), P(e, r) rounded to nearest double from their exact rational
   values, and the 53-bit thresholds ceil(2^53 H), ceil(2^53 P): u < H <=>
   u53 < ceil(2^53 H) for u = u53 2^-53.  Computed once with a small
   fixed-size big-integer type. */
#define BN_LIMBS 144   /* 4608 bits >= 127 * 32 + 2 * 64 */
typedef struct { uint32_t w[BN_LIMBS]; int n; } bn_t;   /* n: limbs in use */
static void bn_set(bn_t* a, uint64_t v) {
  memset(a->w, 0, sizeof a->w);
  a->w[0] = (uint32_t)v; a->w[1] = (uint32_t)(v >> 32);
  a->n = 2;
}
static void bn_norm(bn_t* a) { while (a->n > 1 && a->w[a->n - 1] == 0) --a->n; }
static void bn_shl(bn_t* a, int s) {
  const int L = s / 32, b = s % 32;
  int n = a->n + L + 1;
  if (n > BN_LIMBS) n = BN_LIMBS;
  for (int i = n - 1; i >= 0; --i) {
    uint64_t v = 0;
    if (i - L >= 0) v = (uint64_t)a->w[i - L] << b;
    if (b && i - L - 1 >= 0) v |= a->w[i - L - 1] >> (32 - b);
    a->w[i] = (uint32_t)v;
  }
  a->n = n;
  bn_norm(a);
}
static void bn_sub(bn_t* a, const bn_t* b) {   /* a -= b, a >= b */
  int64_t br = 0;
  for (int i = 0; i < a->n; ++i) {
    int64_t v = (int64_t)a->w[i] - (i < b->n ? (int64_t)b->w[i] : 0) - br;
    br = v < 0;
    a->w[i] = (uint32_t)(v + (br << 32));
  }
  bn_norm(a);
}
static void bn_mul_u64(bn_t* r, const bn_t* a, uint64_t m) {   /* r = a m */
  const uint64_t ml = (uint32_t)m, mh = m >> 32;
  memset(r->w, 0, sizeof r->w);
  uint64_t carry = 0;
  int n = a->n + 2 < BN_LIMBS ? a->n + 2 : BN_LIMBS;
  for (int i = 0; i < n; ++i) {   /* low half */
    uint64_t v = (i < a->n ? (uint64_t)a->w[i] * ml : 0) + carry;
    r->w[i] = (uint32_t)v; carry = v >> 32;
  }
  carry = 0;
  for (int i = 0; i + 1 < n; ++i) {   /* high half, one limb up */
    uint64_t v = (i < a->n ? (uint64_t)a->w[i] * mh : 0) + r->w[i + 1] + carry;
    r->w[i + 1] = (uint32_t)v; carry = v >> 32;
  }
  r->n = n;
  bn_norm(r);
}
static int bn_cmp(const bn_t* a, const bn_t* b) {
  const int n = a->n > b->n ? a->n : b->n;
  for (int i = n - 1; i >= 0; --i) {
    const uint32_t x = i < a->n ? a->w[i] : 0, y = i < b->n ? b->w[i] : 0;
    if (x != y) return x < y ? -1 : 1;
  }
  return 0;
}
static int bn_bitlen(const bn_t* a) {
  for (int i = a->n - 1; i >= 0; --i)
    if (a->w[i]) { int b = 32; while (!(a->w[i] >> (b - 1))) --b; return 32 * i + b; }
  return 0;
}
/* the double nearest num / den (ties to even), 0 < num / den <= 1 */
static double bn_ratio(const bn_t* num, const bn_t* den) {
  const int s = 63 - (bn_bitlen(num) - bn_bitlen(den));   /* quotient in [2^62, 2^64) */
  bn_t ns = *num, t;
  bn_shl(&ns, s);
  uint64_t lo = 1ull << 61, hi = ~0ull;   /* largest Q with Q den <= ns */
  while (lo < hi) {
    const uint64_t mid = lo + ((hi - lo) >> 1) + ((hi - lo) & 1);
    bn_mul_u64(&t, den, mid);
    if (bn_cmp(&t, &ns) <= 0) lo = mid; else hi = mid - 1;
  }
  bn_mul_u64(&t, den, lo);
  const int exact = bn_cmp(&t, &ns) == 0;
  int bl = 64;
  while (!(lo >> (bl - 1))) --bl;
  const int sh = bl - 53;
  uint64_t M = lo >> sh;
  const uint64_t rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (!exact || (M & 1)))) ++M;
  return ldexp((double)M, sh - s);
}
static double th_H[ORC_THIN_NE][ORC_THIN_L], th_P[ORC_THIN_NE][ORC_THIN_L];
static uint64_t th_HT[ORC_THIN_NE][ORC_THIN_L], th_PT[ORC_THIN_NE][ORC_THIN_L];
__attribute__((constructor)) static void th_tables(void) {
  for (int e = ORC_THIN_E_MIN; e <= ORC_THIN_E_MAX; ++e) {
    bn_t A, t, den, num, n2;
    bn_set(&A, 1);   /* (2^e - 1)^m */
    for (int m = 1; m <= ORC_THIN_L; ++m) {
      t = A;
      bn_shl(&A, e);
      bn_sub(&A, &t);
      bn_set(&den, 1);
      bn_shl(&den, e * m);
      num = den;
      bn_sub(&num, &A);   /* 2^(em) H = 2^(em) - (2^e - 1)^m */
      bn_set(&n2, 1);
      bn_shl(&n2, e * (m - 1));   /* P = q / H = 2^(e(m-1)) / (2^(em) H) */
      const int k = e - ORC_THIN_E_MIN;
      th_H[k][m - 1] = bn_ratio(&num, &den);
      th_P[k][m - 1] = bn_ratio(&n2, &num);
      th_HT[k][m - 1] = (uint64_t)ceil(ldexp(th_H[k][m - 1], 53));
      th_PT[k][m - 1] = (uint64_t)ceil(ldexp(th_P[k][m - 1], 53));
    }
  }
}
/* ---- diagnostics (evaluation.py) ------------------------------------------
   Per-cell sums over SIPs in ascending ID order, as the reference's loops
   over id_list[mask] (id_list = 0 .. N-1).  A removed SIP has cells[1] = -1,
   which the reference's indexing wraps to the top row nz - 1. */
static inline int64_t diag_cell(const int64_t* cells, int64_t N, int64_t Nz, int64_t id) {
  int64_t j = cells[N + id];
  if (j < 0) j += Nz;
  return cells[id] * Nz + j;
}
/* x**n for an integer n >= 0: CPython's pow(x, n) in the _py variant, else
   Numba's exponentiation by squaring */
static inline double diag_ipow(double x, int64_t n) {
#ifdef ORC_SQUARE_POW
  return pow(x, (double)n);
#else
  double r = 1.0;
  while (n != 0) {
    if (n & 1) r *= x;
    n >>= 1;
    x *= x;
  }
  return r;
#endif
}
/* evaluation.py:93-133 (kind 0: m_w xi, 1E-18 / m_dry) and :136-174 (kind 1:
   xi, 1 / m_dry) */
ORC_EXPORT void orc_update_cell_sum(int kind, double* out, const double* m_w, const double* xi,
                                    const int64_t* cells, int64_t N, int64_t Nx, int64_t Nz,
                                    const double* mass_dry_inv, const uint8_t* mask) {
  for (int64_t c = 0; c < Nx * Nz; ++c) out[c] = 0.0;
  for (int64_t id = 0; id < N; ++id) {
    if (!mask[id]) continue;
    const int64_t c = diag_cell(cells, N, Nz, id);
    out[c] += kind == 0 ? m_w[id] * xi[id] : xi[id];
  }
  for (int64_t c = 0; c < Nx * Nz; ++c)
    out[c] *= kind == 0 ? 1.0E-18 * mass_dry_inv[c] : mass_dry_inv[c];
}
/* evaluation.py:1392-1445: the n-th radius moment per cell, active SIPs */
ORC_EXPORT void orc_compute_moment_R_grid(int64_t n, const double* R_p, const double* xi,
                                          double V0, const int64_t* cells,
                                          const uint8_t* active, int64_t N, int64_t Nx,
                                          int64_t Nz, double* out) {
  for (int64_t c = 0; c < Nx * Nz; ++c) out[c] = 0.0;
  for (int64_t id = 0; id < N; ++id) {
    if (!active[id]) continue;
    const int64_t c = diag_cell(cells, N, Nz, id);
    if (n == 0) out[c] += xi[id];
    else out[c] += xi[id] * diag_ipow(R_p[id], n);
  }
  for (int64_t c = 0; c < Nx * Nz; ++c) out[c] = out[c] / V0;
}

/* the segment bound of the thinned draws for SIP a against the block of
   slots [lo, hi) of the FP32 copies (certification tests) */
ORC_EXPORT float orc_segment_bound(const float* x, const float* R, const float* u, const float* w,
                                   int64_t a, int64_t lo, int64_t hi, float er, float dtdv_f) {
  th_block_t st;
  th_block_stats(x, R, u, w, lo, hi, &st);
  return th_bound(x[a], R[a], u[a], w[a], &st, er, dtdv_f);
}
/* the FP32 cube root of the thinned draws (accuracy tests) */
ORC_EXPORT void orc_lt_cbrtf(const float* x, int64_t n, float* out) {
  for (int64_t k = 0; k < n; ++k) out[k] = th_cbrtf(x[k]);
}
/* the thinned draws' probability tables and thresholds [126][32] each */
ORC_EXPORT void orc_thin_tables(double* H, double* P, uint64_t* HT, uint64_t* PT) {
  memcpy(H, th_H, sizeof th_H); memcpy(P, th_P, sizeof th_P);
  memcpy(HT, th_HT, sizeof th_HT); memcpy(PT, th_PT, sizeof th_PT);
}
/* the raw Philox4x32-10 block, for known-answer tests */
static void philox_block(uint64_t key, uint64_t c0, uint64_t c1, uint32_t* out) {
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  uint32_t x0 = (uint32_t)c0, x1 = (uint32_t)(c0 >> 32), x2 = (uint32_t)c1, x3 = (uint32_t)(c1 >> 32);
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = mulhi32(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
    uint32_t hi1 = mulhi32(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
    uint32_t y0 = hi1 ^ x1 ^ k0, y1 = lo1, y2 = hi0 ^ x3 ^ k1, y3 = lo0;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}
ORC_EXPORT void orc_philox_block(uint64_t key, uint64_t c0, uint64_t c1, uint32_t* out) {
  philox_block(key, c0, c1, out);
}
ORC_EXPORT void orc_philox_uniform(uint64_t key, const uint64_t* c0, const uint64_t* c1, int64_t n,
                                   double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = philox_uniform(key, c0[i], c1[i]);
}

/* collision/all_or_nothing.py:35-67 */
static inline int64_t kernel_index(double x, double lo, double bl, int64_t nb) {
  int64_t ind = trunc_i64((COL_LOG(x) - lo) / bl + 0.5);
  if (ind < 0) ind = 0;
  else if (ind > nb - 1) ind = nb - 1;
  return ind;
}
ORC_EXPORT void orc_kernel_index(const double* x, int64_t n, double lo, double bl, int64_t nb, int64_t* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = kernel_index(x[i], lo, bl, nb);
}
ORC_EXPORT void orc_radius_from_mass_col(const double* m, const double* rho, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = radius_from_mass_col(m[i], rho[i]);
}

/* collision/all_or_nothing.py:109-185: Golovin box step, all pairs i < j */
/* collision/all_or_nothing.py:392-491: box model with the kernel K(m1, m2)
   tabulated on a logarithmic mass grid; draws rnd[n(n-1)/2] in pair order */
ORC_EXPORT void orc_collision_step_kernel_grid_m(double* xis, double* masses, int64_t n,
                                                 double dt_over_dV, const double* K, int64_t nb,
                                                 double lo, double bl, int64_t* no_cols,
                                                 const double* rnd) {
  int64_t* ind = (int64_t*)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  for (int64_t q = 0; q < n; ++q) ind[q] = kernel_index(masses[q], lo, bl, nb);
  int64_t cnt = 0;
  for (int64_t i = 0; i < n - 1; ++i) {
    for (int64_t j = i + 1; j < n; ++j) {
      int64_t imin, imax;
      if (xis[i] <= xis[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
      const double xi_min = xis[imin], xi_max = xis[imax];
      const double m_min = masses[imin], m_max = masses[imax];
      const double p_crit = xi_max * K[ind[i] * nb + ind[j]] * dt_over_dV;
      if (p_crit > 1.0) {
        const double xi_col = p_crit * xi_min;
        masses[imin] = (xi_min * m_min + xi_col * m_max) / xi_min;
        xis[imax] -= xi_col;
        ind[imin] = kernel_index(masses[imin], lo, bl, nb);
        no_cols[1] += 1;
      } else if (p_crit > rnd[cnt]) {
        no_cols[0] += 1;
        const double xi_rel_dev = (xi_max - xi_min) / xi_max;
        if (xi_rel_dev < 1.0E-5) {
          const double xi_ges = xi_min + xi_max;
          masses[imin] = 2.0 * (xi_min * m_min + xi_max * m_max) / xi_ges;
          masses[imax] = masses[imin];
          xis[imax] = 0.5 * 0.7 * xi_ges;
          xis[imin] = 0.5 * xi_ges - xis[imax];
          ind[imin] = kernel_index(masses[imin], lo, bl, nb);
          ind[imax] = ind[imin];
        } else {
          masses[imin] += m_max;
          xis[imax] -= xi_min;
          ind[imin] = kernel_index(masses[imin], lo, bl, nb);
        }
      }
      ++cnt;
    }
  }
  free(ind);
}

ORC_EXPORT void orc_collision_step_Golovin(double* xis, double* masses, int64_t n,
                                           double dt_over_dV, int64_t* no_cols, const double* rnd) {
  int64_t cnt = 0;
  for (int64_t i = 0; i < n - 1; ++i) {
    for (int64_t j = i + 1; j < n; ++j) {
      int64_t imin, imax;
      if (xis[i] <= xis[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
      double xi_min = xis[imin], xi_max = xis[imax];
      double m_min = masses[imin], m_max = masses[imax];
      double p_crit = xi_max * ((m_min + m_max) * 1.5E-18) * dt_over_dV;
      if (p_crit > 1.0) {
        no_cols[1] += 1;
        double xi_col = p_crit * xi_min;
        masses[imin] = (xi_min * m_min + xi_col * m_max) / xi_min;
        xis[imax] -= xi_col;
      } else if (p_crit > rnd[cnt]) {
        no_cols[0] += 1;
        double xi_rel_dev = (xi_max - xi_min) / xi_max;
        if (xi_rel_dev < 1.0E-5) {
          double xi_ges = xi_min + xi_max;
          masses[imin] = 2.0 * (xi_min * m_min + xi_max * m_max) / xi_ges;
          masses[imax] = masses[imin];
          xis[imax] = 0.5 * 0.7 * xi_ges;
          xis[imin] = 0.5 * xi_ges - xis[imax];
        } else {
          masses[imin] += m_max;
          xis[imax] -= xi_min;
        }
      }
      cnt += 1;
    }
  }
}

/* collision/all_or_nothing.py:269-390: box step with E_col(R1, R2) table and
   1-D (terminal) velocities */
ORC_EXPORT void orc_collision_step_Ecol_grid_R(double* xis, double* masses, double* radii,
    const double* vel, const double* rho, int64_t n, double dt_over_dV, const double* E, int64_t nb,
    double lo, double bl, int64_t* no_cols, const double* rnd) {
  int64_t* k = (int64_t*)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; ++i) k[i] = kernel_index(radii[i], lo, bl, nb);
  int64_t cnt = 0;
  for (int64_t i = 0; i < n - 1; ++i) {
    for (int64_t j = i + 1; j < n; ++j) {
      int64_t imin, imax;
      if (xis[i] <= xis[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
      double xi_min = xis[imin], xi_max = xis[imax];
      double m_min = masses[imin], m_max = masses[imax];
      double s = radii[i] + radii[j];
      double p_crit = xi_max * dt_over_dV * (LC_PI * s * s * E[k[i] * nb + k[j]] * fabs(vel[i] - vel[j]) * 1.0E-12);
      if (p_crit > 1.0) {
        double xi_col = p_crit * xi_min;
        masses[imin] = (xi_min * m_min + xi_col * m_max) / xi_min;
        radii[imin] = radius_from_mass_col(masses[imin], rho[imin]);
        xis[imax] -= xi_col;
        k[imin] = kernel_index(radii[imin], lo, bl, nb);
        no_cols[1] += 1;
      } else if (p_crit > rnd[cnt]) {
        no_cols[0] += 1;
        double xi_rel_dev = (xi_max - xi_min) / xi_max;
        if (xi_rel_dev < 1.0E-5) {
          double xi_ges = xi_min + xi_max;
          masses[imin] = 2.0 * (xi_min * m_min + xi_max * m_max) / xi_ges;
          masses[imax] = masses[imin];
          radii[imin] = radius_from_mass_col(masses[imin], rho[imin]);
          radii[imax] = radii[imin];
          xis[imax] = 0.5 * 0.7 * xi_ges;
          xis[imin] = 0.5 * xi_ges - xis[imax];
          k[imin] = kernel_index(radii[imin], lo, bl, nb);
          k[imax] = k[imin];
        } else {
          masses[imin] += m_max;
          radii[imin] = radius_from_mass_col(masses[imin], rho[imin]);
          xis[imax] -= xi_min;
          k[imin] = kernel_index(radii[imin], lo, bl, nb);
        }
      }
      cnt += 1;
    }
  }
  free(k);
}

/* collision/all_or_nothing.py:498-635 (E table) and :637-751 (constant E):
   one cell, two-component masses, 2-D velocities.  E == NULL selects the
   constant efficiency E_const. */
static void collide_cell_2d(double* xis, double* m_w, double* m_s, double* radii,
                            const double* v0, const double* v1, const double* rho, int64_t n,
                            double dt_over_dV, const double* E, double E_const, int64_t nb,
                            double lo, double bl, int64_t* no_cols, const double* rnd,
                            int64_t* kbuf, uint64_t seed, uint64_t pc1) {
  if (E) for (int64_t i = 0; i < n; ++i) kbuf[i] = kernel_index(radii[i], lo, bl, nb);
  int64_t cnt = 0;
  for (int64_t i = 0; i < n - 1; ++i) {
    for (int64_t j = i + 1; j < n; ++j) {
      int64_t imin, imax;
      if (xis[i] <= xis[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
      double xi_min = xis[imin], xi_max = xis[imax];
      double m_w_min = m_w[imin], m_w_max = m_w[imax];
      double m_s_min = m_s[imin], m_s_max = m_s[imax];
      double s = radii[i] + radii[j];
      double e = E ? E[kbuf[i] * nb + kbuf[j]] : E_const;
      double dv = sqrt(SQ(v0[i] - v0[j]) + SQ(v1[i] - v1[j]));
      double p_crit = xi_max * dt_over_dV * (LC_PI * s * s * e * dv * 1.0E-12);
      if (p_crit > 1.0) {
        double xi_col = p_crit * xi_min;
        m_w[imin] = m_w_min + p_crit * m_w_max;
        m_s[imin] = m_s_min + p_crit * m_s_max;
        radii[imin] = radius_from_mass_col((m_w[imin] + m_s[imin]), rho[imin]);
        xis[imax] -= xi_col;
        if (E) kbuf[imin] = kernel_index(radii[imin], lo, bl, nb);
        no_cols[1] += 1;
      } else if (p_crit > (rnd ? rnd[cnt] : philox_uniform(seed, (uint64_t)cnt, pc1))) {
        no_cols[0] += 1;
        double xi_rel_dev = (xi_max - xi_min) / xi_max;
        if (xi_rel_dev < 1.0E-5) {
          double xi_ges = xi_min + xi_max;
          m_w[imin] = 2.0 * (xi_min * m_w_min + xi_max * m_w_max) / xi_ges;
          m_s[imin] = 2.0 * (xi_min * m_s_min + xi_max * m_s_max) / xi_ges;
          m_w[imax] = m_w[imin];
          m_s[imax] = m_s[imin];
          radii[imin] = radius_from_mass_col((m_w[imin] + m_s[imin]), rho[imin]);
          radii[imax] = radii[imin];
          xis[imax] = 0.5 * 0.7 * xi_ges;
          xis[imin] = 0.5 * xi_ges - xis[imax];
          if (E) { kbuf[imin] = kernel_index(radii[imin], lo, bl, nb); kbuf[imax] = kbuf[imin]; }
        } else {
          m_w[imin] += m_w_max;
          m_s[imin] += m_s_max;
          radii[imin] = radius_from_mass_col((m_w[imin] + m_s[imin]), rho[imin]);
          xis[imax] -= xi_min;
          if (E) kbuf[imin] = kernel_index(radii[imin], lo, bl, nb);
        }
      }
      cnt += 1;
    }
  }
}

/* the FP32 radius of a SIP whose masses a collection changed: from the
   rounded mass sum and the rounded step-start density */
static float th_radius_f(double m_w, double m_s, double rho) {
  return th_cbrtf((float)LC_FOUR_PI_OVER_THREE_INV * (float)(m_w + m_s) / (float)rho);
}

/* One pair (i, j) with draw r (collision/all_or_nothing.py:553-633), as in
   collide_cell_2d.  When xf is given the FP32 copies (xi, R) of the changed
   SIPs are refreshed the way the GPU refreshes its shared copies: an
   equal-multiplicity split rounds the new exact radius, the other
   collections recompute R in FP32 (th_radius_f). */
static void process_pair_2d(int64_t i, int64_t j, double r, double* xis, double* m_w,
                            double* m_s, double* radii, const double* v0, const double* v1,
                            const double* rho, double dt_over_dV, const double* E,
                            double E_const, int64_t nb, double lo, double bl, int64_t* no_cols,
                            int64_t* kbuf, float* xf, float* Rf) {
  int64_t imin, imax;
  if (xis[i] <= xis[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
  double xi_min = xis[imin], xi_max = xis[imax];
  double m_w_min = m_w[imin], m_w_max = m_w[imax];
  double m_s_min = m_s[imin], m_s_max = m_s[imax];
  double s = radii[i] + radii[j];
  double e = E ? E[kbuf[i] * nb + kbuf[j]] : E_const;
  double dv = sqrt(SQ(v0[i] - v0[j]) + SQ(v1[i] - v1[j]));
  double p_crit = xi_max * dt_over_dV * (LC_PI * s * s * e * dv * 1.0E-12);
  if (p_crit > 1.0) {
    double xi_col = p_crit * xi_min;
    m_w[imin] = m_w_min + p_crit * m_w_max;
    m_s[imin] = m_s_min + p_crit * m_s_max;
    radii[imin] = radius_from_mass_col((m_w[imin] + m_s[imin]), rho[imin]);
    xis[imax] -= xi_col;
    if (E) kbuf[imin] = kernel_index(radii[imin], lo, bl, nb);
    no_cols[1] += 1;
    if (xf) { xf[imax] = (float)xis[imax]; Rf[imin] = th_radius_f(m_w[imin], m_s[imin], rho[imin]); }
  } else if (p_crit > r) {
    no_cols[0] += 1;
    double xi_rel_dev = (xi_max - xi_min) / xi_max;
    if (xi_rel_dev < 1.0E-5) {
      double xi_ges = xi_min + xi_max;
      m_w[imin] = 2.0 * (xi_min * m_w_min + xi_max * m_w_max) / xi_ges;
      m_s[imin] = 2.0 * (xi_min * m_s_min + xi_max * m_s_max) / xi_ges;
      m_w[imax] = m_w[imin];
      m_s[imax] = m_s[imin];
      radii[imin] = radius_from_mass_col((m_w[imin] + m_s[imin]), rho[imin]);
      radii[imax] = radii[imin];
      xis[imax] = 0.5 * 0.7 * xi_ges;
      xis[imin] = 0.5 * xi_ges - xis[imax];
      if (E) { kbuf[imin] = kernel_index(radii[imin], lo, bl, nb); kbuf[imax] = kbuf[imin]; }
      if (xf) {
        xf[imin] = (float)xis[imin]; xf[imax] = (float)xis[imax];
        Rf[imin] = (float)radii[imin]; Rf[imax] = Rf[imin];
      }
    } else {
      m_w[imin] += m_w_max;
      m_s[imin] += m_s_max;
      radii[imin] = radius_from_mass_col((m_w[imin] + m_s[imin]), rho[imin]);
      xis[imax] -= xi_min;
      if (E) kbuf[imin] = kernel_index(radii[imin], lo, bl, nb);
      if (xf) { xf[imax] = (float)xis[imax]; Rf[imin] = th_radius_f(m_w[imin], m_s[imin], rho[imin]); }
    }
  }
}

/* The thinned Philox draws for one cell: the sequential definition the GPU
   kernel parallelises (segments of row i over blocks of ORC_THIN_L slots).
   FP32 copies follow the GPU: xi, u, w rounded from the doubles; R from the
   FP32 mass and density at the cell temperature Tc, refreshed after each
   change as process_pair_2d says.  erow[k] is the largest FP32 efficiency of
   row k of the table. */
static void collide_cell_2d_thin(double* xis, double* m_w, double* m_s, double* radii,
                                 const double* v0, const double* v1, const double* rho, int64_t n,
                                 double dt_over_dV, const double* E, double E_const, int64_t nb,
                                 double lo, double bl, int64_t* no_cols, int64_t* kbuf,
                                 uint64_t seed, uint64_t pc1, double Tc, int sol, float* xf,
                                 float* Rf, float* uf, float* wf, const float* erow) {
  if (E) for (int64_t i = 0; i < n; ++i) kbuf[i] = kernel_index(radii[i], lo, bl, nb);
  const float Tf = (float)Tc;
  const float rhow_f = (float)LC_PAR_WATER_DENS_0 +
                       (float)LC_PAR_WATER_DENS_1 * ((Tf - (float)LC_PAR_WATER_DENS_2) *
                                                      (Tf - (float)LC_PAR_WATER_DENS_2));
  const float c43 = (float)LC_FOUR_PI_OVER_THREE_INV;
  for (int64_t q = 0; q < n; ++q) {
    const float mwf = (float)m_w[q], msf = (float)m_s[q];
    const float mpf = mwf + msf;
    const float wsf = msf / mpf;
    const float rh = (sol == SOL_AS)
                         ? rhow_f * ((((float)LC_PAR_RHO_AS_0 * wsf + (float)LC_PAR_RHO_AS_1) *
                                          wsf + (float)LC_PAR_RHO_AS_2) * wsf +
                                     (float)LC_PAR_RHO_AS_3)
                         : (float)LC_PAR_SOL_DENS_NACL_0 + (float)LC_PAR_SOL_DENS_NACL_1 * wsf +
                               (float)LC_PAR_SOL_DENS_NACL_2 * Tf +
                               (float)LC_PAR_SOL_DENS_NACL_3 * wsf * wsf +
                               (float)LC_PAR_SOL_DENS_NACL_4 * wsf * Tf +
                               (float)LC_PAR_SOL_DENS_NACL_5 * Tf * Tf;
    Rf[q] = th_cbrtf(c43 * mpf / rh);
    xf[q] = (float)xis[q];
    uf[q] = (float)v0[q];
    wf[q] = (float)v1[q];
  }
  const float dtdv_f = (float)dt_over_dV;
  const float Ec_f = (float)E_const;
  const int64_t L = ORC_THIN_L;
  const int64_t B = (n + L - 1) / L;
  for (int64_t i = 0; i + 1 < n; ++i) {
    for (int64_t b = (i + 1) / L; b < B; ++b) {
      const int64_t blo = b * L, bhi = (b + 1) * L < n ? (b + 1) * L : n;
      int64_t j = blo > i + 1 ? blo : i + 1;
      const uint64_t chunk = (uint64_t)(i * n - i * (i + 1) / 2 + (j - i - 1));   /* rank of (i, j) */
      uint32_t sub = 0;
      while (j < bhi) {
        th_block_t st;
        th_block_stats(xf, Rf, uf, wf, blo, bhi, &st);
        const float er = E ? erow[kbuf[i]] : Ec_f;
        const float Q = th_bound(xf[i], Rf[i], uf[i], wf[i], &st, er, dtdv_f);
        if (!(Q >= 0.0f && Q < ORC_THIN_TAU)) {
          /* per-pair draws for the rest of the segment */
          for (; j < bhi; ++j) {
            const int64_t rk = i * n - i * (i + 1) / 2 + (j - i - 1);
            process_pair_2d(i, j, philox_uniform(seed, (uint64_t)rk, pc1), xis, m_w, m_s, radii,
                            v0, v1, rho, dt_over_dV, E, E_const, nb, lo, bl, no_cols, kbuf, xf, Rf);
          }
          break;
        }
        const int m = (int)(bhi - j);
        const int e = th_exponent(Q);
        if (th_u53(seed, chunk, sub, 0u, pc1) >= th_HT[e - ORC_THIN_E_MIN][m - 1])
          break;   /* no draw of the part falls below q */
        uint32_t jd = 1;
        int g = 0;
        for (; g < m - 1; ++g)
          if (th_u53(seed, chunk, sub, jd++, pc1) < th_PT[e - ORC_THIN_E_MIN][m - g - 1])
            break;
        const double r = ldexp((double)th_u53(seed, chunk, sub, jd, pc1) *
                                   (1.0 / 9007199254740992.0), -e);
        process_pair_2d(i, j + g, r, xis, m_w, m_s, radii, v0, v1, rho, dt_over_dV, E, E_const, nb,
                        lo, bl, no_cols, kbuf, xf, Rf);
        j += g + 1;
        ++sub;
      }
    }
  }
}

/* collision/all_or_nothing.py:754-846: every cell, x-outer / z-inner, SIPs of
   a cell in ascending ID; the radius uses the cell temperature and the
   solute's density.  Draws are consumed in that order from rnd[*rnd_pos..].
   Returns 0, or -1 if rnd holds too few draws (nothing is changed then). */
static int collision_all_cells(double* xis, double* m_w, double* m_s,
    const double* vel, const double* T, const int64_t* cells, int64_t N, int64_t Nx, int64_t Nz,
    double dt_over_dV, const double* E, double E_const, int64_t nb, double lo, double bl,
    int64_t* no_cols, int sol, const double* rnd, int64_t rnd_len, int64_t* rnd_pos,
    uint64_t seed, int64_t* col_step, int thin) {
  int64_t C = Nx * Nz;
  int64_t* start = (int64_t*)calloc(C + 1, sizeof(int64_t));
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (N > 0 ? N : 1));
  int64_t* draw0 = (int64_t*)malloc(sizeof(int64_t) * (C + 1));
  for (int64_t k = 0; k < N; ++k) {
    int64_t i = cells[k], j = cells[N + k];
    if (i >= 0 && i < Nx && j >= 0 && j < Nz) start[i * Nz + j + 1] += 1;
  }
  for (int64_t c = 0; c < C; ++c) start[c + 1] += start[c];
  draw0[0] = rnd_pos ? *rnd_pos : 0;
  for (int64_t c = 0; c < C; ++c) {
    int64_t nc = start[c + 1] - start[c];
    draw0[c + 1] = draw0[c] + nc * (nc - 1) / 2;
  }
  if (rnd && draw0[C] > rnd_len) { free(start); free(order); free(draw0); return -1; }
  const uint64_t cstep = col_step ? (uint64_t)*col_step : 0;
  float* erow = NULL;
  if (thin && E) {
    erow = (float*)malloc(sizeof(float) * (nb > 0 ? nb : 1));
    for (int64_t k = 0; k < nb; ++k) {
      float mx = (float)E[k * nb];
      for (int64_t q = 1; q < nb; ++q) mx = th_max(mx, (float)E[k * nb + q]);
      erow[k] = mx;
    }
  }
  {
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (C > 0 ? C : 1));
    memcpy(fill, start, sizeof(int64_t) * C);
    for (int64_t k = 0; k < N; ++k) {
      int64_t i = cells[k], j = cells[N + k];
      if (i >= 0 && i < Nx && j >= 0 && j < Nz) order[fill[i * Nz + j]++] = k;
    }
    free(fill);
  }
  int64_t nc0 = 0, nc1 = 0;
#pragma omp parallel reduction(+ : nc0, nc1)
  {
    int64_t cap = 0;
    double *xb = NULL, *wb = NULL, *sb = NULL, *Rb = NULL, *v0 = NULL, *v1 = NULL, *rb = NULL;
    int64_t* kb = NULL;
    float *fx = NULL, *fR = NULL, *fu = NULL, *fw = NULL;
#pragma omp for schedule(dynamic, 16)
    for (int64_t c = 0; c < C; ++c) {
      int64_t n = start[c + 1] - start[c];
      if (n == 0) continue;
      if (n > cap) {
        cap = n;
        xb = realloc(xb, 8 * n); wb = realloc(wb, 8 * n); sb = realloc(sb, 8 * n);
        Rb = realloc(Rb, 8 * n); v0 = realloc(v0, 8 * n); v1 = realloc(v1, 8 * n);
        rb = realloc(rb, 8 * n); kb = realloc(kb, 8 * n);
        fx = realloc(fx, 4 * n); fR = realloc(fR, 4 * n); fu = realloc(fu, 4 * n);
        fw = realloc(fw, 4 * n);
      }
      const int64_t* ids = order + start[c];
      double Tc = T[c];
      for (int64_t q = 0; q < n; ++q) {
        int64_t id = ids[q];
        xb[q] = xis[id]; wb[q] = m_w[id]; sb[q] = m_s[id];
        v0[q] = vel[id]; v1[q] = vel[N + id];
        double m_p = wb[q] + sb[q];
        double w = sb[q] / m_p;
        double r = (sol == SOL_AS) ? density_AS_solution(w, Tc) : density_NaCl_solution(w, Tc);
        rb[q] = r;
        Rb[q] = radius_from_mass_col(m_p, r);
      }
      int64_t cnt[2] = {0, 0};
      if (thin && !rnd)
        collide_cell_2d_thin(xb, wb, sb, Rb, v0, v1, rb, n, dt_over_dV, E, E_const, nb, lo, bl,
                             cnt, kb, seed, (cstep << 32) | (uint64_t)c, Tc, sol, fx, fR, fu, fw,
                             erow);
      else
        collide_cell_2d(xb, wb, sb, Rb, v0, v1, rb, n, dt_over_dV, E, E_const, nb, lo, bl, cnt,
                        rnd ? rnd + draw0[c] : NULL, kb, seed, (cstep << 32) | (uint64_t)c);
      nc0 += cnt[0]; nc1 += cnt[1];
      for (int64_t q = 0; q < n; ++q) {
        int64_t id = ids[q];
        xis[id] = xb[q]; m_w[id] = wb[q]; m_s[id] = sb[q];
      }
    }
    free(xb); free(wb); free(sb); free(Rb); free(v0); free(v1); free(rb); free(kb);
    free(fx); free(fR); free(fu); free(fw);
  }
  no_cols[0] += nc0; no_cols[1] += nc1;
  if (rnd) *rnd_pos = draw0[C];
  if (col_step) *col_step += 1;
  free(start); free(order); free(draw0); free(erow);
  return 0;
}

ORC_EXPORT int orc_collision_step_all_cells_2d(double* xis, double* m_w, double* m_s,
    const double* vel, const double* T, const int64_t* cells, int64_t N, int64_t Nx, int64_t Nz,
    double dt_over_dV, const double* E, double E_const, int64_t nb, double lo, double bl,
    int64_t* no_cols, int sol, const double* rnd, int64_t rnd_len, int64_t* rnd_pos) {
  return collision_all_cells(xis, m_w, m_s, vel, T, cells, N, Nx, Nz, dt_over_dV, E, E_const, nb,
                             lo, bl, no_cols, sol, rnd, rnd_len, rnd_pos, 0, NULL, 0);
}

/* the same with Philox draws (key seed, collision-step counter *col_step) */
ORC_EXPORT int orc_collision_step_all_cells_2d_philox(double* xis, double* m_w, double* m_s,
    const double* vel, const double* T, const int64_t* cells, int64_t N, int64_t Nx, int64_t Nz,
    double dt_over_dV, const double* E, double E_const, int64_t nb, double lo, double bl,
    int64_t* no_cols, int sol, uint64_t seed, int64_t* col_step, int thin) {
  return collision_all_cells(xis, m_w, m_s, vel, T, cells, N, Nx, Nz, dt_over_dV, E, E_const, nb,
                             lo, bl, no_cols, sol, NULL, 0, NULL, seed, col_step, thin);
}

/* total number of pair draws the next all-cells step consumes */
ORC_EXPORT int64_t orc_collision_pair_count(const int64_t* cells, int64_t N, int64_t Nx, int64_t Nz) {
  int64_t C = Nx * Nz;
  int64_t* cnt = (int64_t*)calloc(C > 0 ? C : 1, sizeof(int64_t));
  for (int64_t k = 0; k < N; ++k) {
    int64_t i = cells[k], j = cells[N + k];
    if (i >= 0 && i < Nx && j >= 0 && j < Nz) cnt[i * Nz + j] += 1;
  }
  int64_t tot = 0;
  for (int64_t c = 0; c < C; ++c) tot += cnt[c] * (cnt[c] - 1) / 2;
  free(cnt);
  return tot;
}

/* ---------------------------------------------------------------------- */
/* integration.py:489-507 */
static void update_T_p(const double* Tg, const int64_t* cells, double* T_p, int64_t N, int64_t Nz) {
  for (int64_t k = 0; k < N; ++k) {
    int64_t j = cells[N + k];
    if (j < 0) j += Nz;
    T_p[k] = Tg[cells[k] * Nz + j];
  }
}

/* integration.py:509-550 */
static void update_cells_and_rel_pos(const double* pos, int64_t* cells, double* rel_pos,
                                     const uint8_t* active, const double* ranges,
                                     const double* steps, int64_t N) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < N; ++k) {
    if (active[k]) {
      double x = pos[k], y = pos[N + k];
      rel_pos[k] = x - ranges[0];
      rel_pos[N + k] = y - ranges[2];
      cells[k] = (int64_t)floor(x / steps[0]);
      cells[N + k] = (int64_t)floor(y / steps[1]);
    }
    rel_pos[k] = rel_pos[k] / steps[0] - (double)cells[k];
    rel_pos[N + k] = rel_pos[N + k] / steps[1] - (double)cells[N + k];
  }
}

/* integration.py:552-630 */
static void update_pos_from_vel_BC_PS(const double* m_w, double* pos, double* vel, const double* xi,
                                      int64_t* cells, double* water_removed, uint8_t* active,
                                      const double* ranges, const double* steps, double dt,
                                      int64_t N) {
  double z_min = ranges[2];
  double x_max = ranges[1];
  double z_cap = ranges[3] * 0.999999;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < N; ++k) {
    pos[k] += dt * vel[k];
    pos[N + k] += dt * vel[N + k];
    pos[k] = py_mod(pos[k], x_max);
    pos[N + k] = np_min(pos[N + k], z_cap);
  }
  for (int64_t k = 0; k < N; ++k) {       /* ascending ID: ordered sum */
    if (active[k] && pos[N + k] <= z_min) {
      pos[N + k] = z_min - 0.01 * steps[1];
      vel[k] = 0.0;
      vel[N + k] = 0.0;
      active[k] = 0;
      water_removed[0] += xi[k] * m_w[k];
      cells[N + k] = -1;
    }
  }
}

typedef struct {
  const double *gsf, *gmp, *gv;
  int64_t Nx, Nz;
  const double *ranges, *steps;
  double *pos, *vel, *rel_pos, *m_w;
  const double *m_s, *xi;
  int64_t* cells;
  double* water_removed;
  uint8_t* active;
  double* T_p;
  int sol;
  double* delta_m_l;
  int64_t N;
} orc_particles_t;

/* integration.py:944-1091: one particle sub-step (condensation, drag,
   position, cell re-index) */
static void particles_substep(orc_particles_t* s, double dt_sub, double dt_sub_pos, int no_iter, double g_set) {
  const int64_t N = s->N, Nx = s->Nx, Nz = s->Nz, C = Nx * Nz;
  const double* Tg = s->gsf;
  const double* pg = s->gsf + 1 * C;
  const double* Sg = s->gsf + 6 * C;
  const double* esg = s->gsf + 7 * C;
  const double* Kg = s->gmp;
  const double* Dg = s->gmp + 1 * C;
  const double* Lg = s->gmp + 2 * C;
  const double* mug = s->gmp + 5 * C;
  const double* rhofg = s->gmp + 6 * C;
  update_T_p(Tg, s->cells, s->T_p, N, Nz);
  double* dmxi = (double*)malloc(sizeof(double) * (N > 0 ? N : 1));
  double* velf = (double*)malloc(sizeof(double) * 2 * (N > 0 ? N : 1));
  /* condensation (integration.py:840-940); the per-cell sum runs afterwards */
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t k = 0; k < N; ++k) {
    double R, w, rho;
    R_ws_rho(s->sol, s->m_w[k], s->m_s[k], s->T_p[k], &R, &w, &rho);
    if (!s->active[k]) continue;
    int64_t c = s->cells[k] * Nz + s->cells[N + k];
    double sig = (s->sol == SOL_AS) ? surface_tension_AS(w, s->T_p[k]) : surface_tension_NaCl(w, s->T_p[k]);
    double dm, g0;
    newton_full(s->sol, dt_sub, no_iter, s->m_w[k], s->m_s[k], w, R, s->T_p[k], rho, Tg[c], pg[c],
                Sg[c], esg[c], Lg[c], Kg[c], Dg[c], sig, &dm, &g0);
    s->m_w[k] += dm;
    dmxi[k] = dm * s->xi[k];
  }
  for (int64_t c = 0; c < C; ++c) s->delta_m_l[c] = 0.0;
  for (int64_t k = 0; k < N; ++k)
    if (s->active[k]) s->delta_m_l[s->cells[k] * Nz + s->cells[N + k]] += dmxi[k];
  for (int64_t c = 0; c < C; ++c) s->delta_m_l[c] *= 1.0E-18;
  /* velocity (integration.py:632-719) with the ammonium-sulfate radius */
  orc_interpolate_velocity(s->cells, s->rel_pos, s->gv, Nx, Nz, N, velf);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < N; ++k) {
    if (!s->active[k]) continue;
    double R, w, rho;
    R_ws_rho(SOL_AS, s->m_w[k], s->m_s[k], s->T_p[k], &R, &w, &rho);
    int64_t c = s->cells[k] * Nz + s->cells[N + k];
    double mu_f = mug[c], rho_f = rhofg[c];
    double d0 = velf[k] - s->vel[k], d1 = velf[N + k] - s->vel[N + k];
    double vel_dev = sqrt(d0 * d0 + d1 * d1);
    double Re_p = 2.0E-6 * rho_f * R * vel_dev / mu_f;
    double k_dt = 4.5E12 * dt_sub * mu_f / (rho * R * R);
    if (Re_p > 0.5) {
      if (Re_p < 1000.0) k_dt *= (1 + 0.15 * pow(Re_p, 0.687));
      else k_dt *= 0.0183333333333 * Re_p;
    }
    s->vel[k] = (s->vel[k] + k_dt * velf[k]) / (1.0 + k_dt);
    s->vel[N + k] = (s->vel[N + k] + k_dt * velf[N + k] - dt_sub * g_set) / (1.0 + k_dt);
  }
  free(dmxi);
  free(velf);
  update_pos_from_vel_BC_PS(s->m_w, s->pos, s->vel, s->xi, s->cells, s->water_removed, s->active,
                            s->ranges, s->steps, dt_sub_pos, N);
  update_cells_and_rel_pos(s->pos, s->cells, s->rel_pos, s->active, s->ranges, s->steps, N);
}

ORC_EXPORT void orc_propagate_particles_subloop_step(const double* gsf, const double* gmp, const double* gv,
    int64_t Nx, int64_t Nz, const double* ranges, const double* steps, double* pos, double* vel,
    int64_t* cells, double* rel_pos, double* m_w, const double* m_s, const double* xi,
    double* water_removed, uint8_t* active, double* T_p, int sol, double* delta_m_l, int64_t N,
    double dt_sub, double dt_sub_pos, int no_iter, double g_set) {
  orc_particles_t s = {gsf, gmp, gv, Nx, Nz, ranges, steps, pos, vel, rel_pos, m_w, m_s, xi,
                       cells, water_removed, active, T_p, sol, delta_m_l, N};
  particles_substep(&s, dt_sub, dt_sub_pos, no_iter, g_set);
}

/* integration.py:359-400 */
static void update_material_properties(double* gsf, double* gmp, int64_t C) {
  for (int64_t c = 0; c < C; ++c) {
    double T = gsf[c], p = gsf[C + c], rho_d = gsf[3 * C + c], r_v = gsf[4 * C + c];
    gmp[c] = 4.1868E-3 * (5.69 + 0.017 * (T - 273.15));
    gmp[C + c] = 4.01218E-5 * pow(T, 1.94) / p;
    gmp[2 * C + c] = 1.0E3 * (2500.82 - 2.358 * (T - 273.0));
    gmp[3 * C + c] = surface_tension_water(T);
    gmp[4 * C + c] = LC_C_PD * (1 + 0.897 * r_v);
    gmp[5 * C + c] = 1.458E-6 * pow(T, 1.5) / (T + 110.4);
    gmp[6 * C + c] = rho_d * (1.0 + r_v);
  }
}

/* integration.py:402-484 */
ORC_EXPORT void orc_propagate_grid_subloop_step(double* gsf, double* gmp, int64_t Nx, int64_t Nz,
    double p_ref, double p_ref_inv, const double* dTheta, const double* dr_v, const double* dml,
    double V) {
  int64_t C = Nx * Nz;
  for (int64_t c = 0; c < C; ++c) {
    double* T = gsf + c; double* p = gsf + C + c; double* Th = gsf + 2 * C + c;
    double rho_d = gsf[3 * C + c]; double* r_v = gsf + 4 * C + c;
    double* S = gsf + 6 * C + c; double* e_s = gsf + 7 * C + c; double mdi = gsf[8 * C + c];
    double L_v = gmp[2 * C + c];
    *Th += dTheta[c];
    *r_v += dr_v[c] - dml[c] * mdi;
    double ToT = pow(p_ref_inv * LC_R_D * rho_d * *Th, LC_KAPPA_FACTOR2);
    *Th += ToT * (L_v * dml[c]) / (LC_C_PD * rho_d * V * (1.0 + *r_v * LC_HEAT_FACTOR_R_V));
    double pdr = pow(rho_d * *Th * LC_R_D * p_ref_inv, LC_KAPPA_FACTOR);
    *T = *Th * pow(pdr, LC_KAPPA_AIR_DRY);
    *p = pdr * p_ref * (1 + *r_v / LC_EPSILON_GC);
    *e_s = 2.53E11 * exp(-5420.0 / *T);
    *S = rho_d * *r_v * *T * LC_R_V / *e_s;
  }
  update_material_properties(gsf, gmp, C);
}

/* integration.py:80-111 */
static inline double limiter(double r) {
  double K = (1.0 + 2.0 * r) * LC_ONE_THIRD;
  return np_max(0.0, fmin(2.0 * r, fmin(K, 2.0)));
}
/* integration.py:113-148 */
static inline double limiter_arg(double a0, double a1, double a2) {
  double r = (fabs(a1 - a2) > 1.0E-8 * fabs(a0 - a1)) ? (a0 - a1) / (a1 - a2)
                                                       : (a0 - a1) * 1.0E8 * np_sign(a1 - a2);
  return limiter(r);
}
/* flux through the face with upwind cells a1 (u >= 0) and a0 (u < 0):
   integration.py:214-240 */
static inline double face_flux(double u, double am2, double am1, double a0, double ap1) {
  double lp = limiter_arg(a0, am1, am2);
  double f_pos = am1 + 0.5 * lp * (am1 - am2);
  double ln = limiter_arg(am1, a0, ap1);
  double f_neg = a0 + 0.5 * ln * (a0 - ap1);
  return (u >= 0.0) ? u * f_pos : u * f_neg;
}
/* integration.py:150-287: 3rd-order limited upwind divergence of
   field * flux; bc 0 = periodic, 1 = solid (zero flux at the walls) */
ORC_EXPORT void orc_divergence_upwind(const double* f, const double* flux, int64_t Nx, int64_t Nz,
                                      const double* steps, int bcx, int bcz, double* out) {
#define FI(i, j) f[(i) * Nz + (j)]
  /* x-direction faces i = 0..Nx for each column j */
  double* Fx = (double*)malloc(sizeof(double) * (Nx + 1) * Nz);
  double* Fz = (double*)malloc(sizeof(double) * Nx * (Nz + 1));
  for (int64_t i = 0; i <= Nx; ++i) {
    for (int64_t j = 0; j < Nz; ++j) {
      int64_t im2, im1, i0, ip1;
      if (bcx == 0) {
        im2 = ((i - 2) % Nx + Nx) % Nx; im1 = ((i - 1) % Nx + Nx) % Nx;
        i0 = i % Nx; ip1 = (i + 1) % Nx;
      } else {
        im2 = i - 2 < 0 ? 0 : i - 2; im1 = i - 1 < 0 ? 0 : i - 1;
        i0 = i > Nx - 1 ? Nx - 1 : i; ip1 = i + 1 > Nx - 1 ? Nx - 1 : i + 1;
      }
      double u = flux[i * (Nz + 1) + j];
      Fx[i * Nz + j] = face_flux(u, FI(im2, j), FI(im1, j), FI(i0, j), FI(ip1, j));
    }
  }
  if (bcx == 1) for (int64_t j = 0; j < Nz; ++j) { Fx[j] = 0.0; Fx[Nx * Nz + j] = 0.0; }
  for (int64_t i = 0; i < Nx; ++i) {
    for (int64_t j = 0; j <= Nz; ++j) {
      int64_t jm2, jm1, j0, jp1;
      if (bcz == 0) {
        jm2 = ((j - 2) % Nz + Nz) % Nz; jm1 = ((j - 1) % Nz + Nz) % Nz;
        j0 = j % Nz; jp1 = (j + 1) % Nz;
      } else {
        jm2 = j - 2 < 0 ? 0 : j - 2; jm1 = j - 1 < 0 ? 0 : j - 1;
        j0 = j > Nz - 1 ? Nz - 1 : j; jp1 = j + 1 > Nz - 1 ? Nz - 1 : j + 1;
      }
      double w = flux[(Nx + 1) * (Nz + 1) + i * (Nz + 1) + j];
      Fz[i * (Nz + 1) + j] = face_flux(w, FI(i, jm2), FI(i, jm1), FI(i, j0), FI(i, jp1));
    }
    if (bcz == 1) { Fz[i * (Nz + 1)] = 0.0; Fz[i * (Nz + 1) + Nz] = 0.0; }
  }
  for (int64_t i = 0; i < Nx; ++i)
    for (int64_t j = 0; j < Nz; ++j)
      out[i * Nz + j] = (Fx[(i + 1) * Nz + j] - Fx[i * Nz + j]) / steps[0]
                        + (Fz[i * (Nz + 1) + j + 1] - Fz[i * (Nz + 1) + j]) / steps[1];
  free(Fx); free(Fz);
#undef FI
}

/* integration.py:325-354: column-mean relaxation, summed over x in order */
ORC_EXPORT void orc_relaxation_term(const double* f, int64_t Nx, int64_t Nz, const double* profile,
                                    const double* t_relax, double dt, double* out) {
  for (int64_t j = 0; j < Nz; ++j) {
    double s = f[j];
    for (int64_t i = 1; i < Nx; ++i) s += f[i * Nz + j];
    out[j] = dt * (profile[j] - s / (double)Nx) / t_relax[j];
  }
}

/* grid.py:370-412 */
ORC_EXPORT void orc_update_grid_r_l(const double* m_w, const double* xi, const int64_t* cells,
                                    double* r_l, const double* mdi, const uint8_t* active,
                                    int64_t N, int64_t Nx, int64_t Nz) {
  int64_t C = Nx * Nz;
  for (int64_t c = 0; c < C; ++c) r_l[c] = 0.0;
  for (int64_t k = 0; k < N; ++k)
    if (active[k]) r_l[cells[k] * Nz + cells[N + k]] += m_w[k] * xi[k];
  for (int64_t c = 0; c < C; ++c) r_l[c] *= 1.0E-18 * mdi[c];
}

typedef struct {
  double *gsf, *gmp;
  const double *gv, *flux;
  double p_ref, p_ref_inv;
  int64_t Nx, Nz;
  const double *ranges, *steps;
  double V;
  double *pos, *vel;
  int64_t* cells;
  double *rel_pos, *m_w, *m_s, *xi;
  int sol;
  double* water_removed;
  uint8_t* active;
  double *T_p, *delta_m_l;
  double dt, dt_sub, dt_sub_half, dt_col_over_dV;
  int scale_dt_cond, no_col_per_adv, act_collisions, act_relaxation;
  const double *prof_r_v, *prof_Theta, *t_relax;
  int no_iter;
  double g_set;
  const double* E;
  double E_const;
  int64_t nb;
  double lo, bl;
  int64_t* no_cols;
  const double* rnd;
  int64_t rnd_len;
  int64_t* rnd_pos;
  int64_t N;
  uint64_t seed;
  int64_t* col_step;
  int thin;
} orc_adv_t;

static int collide_all(orc_adv_t* a) {
  return collision_all_cells(a->xi, a->m_w, a->m_s, a->vel, a->gsf, a->cells, a->N, a->Nx, a->Nz,
                             a->dt_col_over_dV, a->E, a->E_const, a->nb, a->lo, a->bl, a->no_cols,
                             a->sol, a->rnd, a->rnd_len, a->rnd_pos, a->seed, a->col_step,
                             a->thin);
}

/* integration.py:1095-1294 */
static int subloop(orc_adv_t* a, const double* dTh, const double* drv, int no_cond, int no_col) {
  orc_particles_t s = {a->gsf, a->gmp, a->gv, a->Nx, a->Nz, a->ranges, a->steps, a->pos, a->vel,
                       a->rel_pos, a->m_w, a->m_s, a->xi, a->cells, a->water_removed, a->active,
                       a->T_p, a->sol, a->delta_m_l, a->N};
  if (a->act_collisions && no_col == 1) if (collide_all(a)) return -1;
  for (int n = 0; n < no_cond; ++n) {
    if (a->act_collisions && no_col > 1) if (collide_all(a)) return -1;
    particles_substep(&s, a->dt_sub, a->dt_sub, a->no_iter, a->g_set);
    orc_propagate_grid_subloop_step(a->gsf, a->gmp, a->Nx, a->Nz, a->p_ref, a->p_ref_inv, dTh, drv,
                                    a->delta_m_l, a->V);
  }
  if (a->act_collisions && no_col > no_cond) if (collide_all(a)) return -1;
  return 0;
}

/* integration.py:1298-1611: one advection step dt */
static int adv_step(orc_adv_t* a) {
  const int64_t Nx = a->Nx, Nz = a->Nz, C = Nx * Nz;
  double* dTh = (double*)malloc(sizeof(double) * C);
  double* drv = (double*)malloc(sizeof(double) * C);
  double* div = (double*)malloc(sizeof(double) * C);
  double* rel = (double*)malloc(sizeof(double) * Nz);
  const double* rdi = a->gsf + 9 * C;
  int rc = 0;
  update_pos_from_vel_BC_PS(a->m_w, a->pos, a->vel, a->xi, a->cells, a->water_removed, a->active,
                            a->ranges, a->steps, a->dt_sub_half, a->N);
  update_cells_and_rel_pos(a->pos, a->cells, a->rel_pos, a->active, a->ranges, a->steps, a->N);
  orc_divergence_upwind(a->gsf + 4 * C, a->flux, Nx, Nz, a->steps, 0, 1, div);
  for (int64_t c = 0; c < C; ++c) drv[c] = -a->dt_sub * div[c] * rdi[c];
  orc_divergence_upwind(a->gsf + 2 * C, a->flux, Nx, Nz, a->steps, 0, 1, div);
  for (int64_t c = 0; c < C; ++c) dTh[c] = -a->dt_sub * div[c] * rdi[c];
  if (a->act_relaxation) {
    orc_relaxation_term(a->gsf + 4 * C, Nx, Nz, a->prof_r_v, a->t_relax, a->dt_sub, rel);
    for (int64_t c = 0; c < C; ++c) drv[c] += rel[c % Nz];
    orc_relaxation_term(a->gsf + 2 * C, Nx, Nz, a->prof_Theta, a->t_relax, a->dt_sub, rel);
    for (int64_t c = 0; c < C; ++c) dTh[c] += rel[c % Nz];
  }
  int no_col = (a->no_col_per_adv == 1) ? 0 : (a->no_col_per_adv == 2 ? 1 : a->scale_dt_cond);
  rc = subloop(a, dTh, drv, a->scale_dt_cond, no_col);
  if (rc) goto done;
  orc_divergence_upwind(a->gsf + 4 * C, a->flux, Nx, Nz, a->steps, 0, 1, div);
  for (int64_t c = 0; c < C; ++c) drv[c] = -2.0 * a->dt_sub * div[c] * rdi[c] - drv[c];
  orc_divergence_upwind(a->gsf + 2 * C, a->flux, Nx, Nz, a->steps, 0, 1, div);
  for (int64_t c = 0; c < C; ++c) dTh[c] = -2.0 * a->dt_sub * div[c] * rdi[c] - dTh[c];
  if (a->act_relaxation) {
    orc_relaxation_term(a->gsf + 4 * C, Nx, Nz, a->prof_r_v, a->t_relax, a->dt_sub, rel);
    for (int64_t c = 0; c < C; ++c) drv[c] += 2. * rel[c % Nz];
    orc_relaxation_term(a->gsf + 2 * C, Nx, Nz, a->prof_Theta, a->t_relax, a->dt_sub, rel);
    for (int64_t c = 0; c < C; ++c) dTh[c] += 2. * rel[c % Nz];
  }
  no_col = (a->no_col_per_adv == 1 || a->no_col_per_adv == 2) ? 1 : a->scale_dt_cond;
  rc = subloop(a, dTh, drv, a->scale_dt_cond - 1, no_col);
  if (rc) goto done;
  {
    orc_particles_t s = {a->gsf, a->gmp, a->gv, a->Nx, a->Nz, a->ranges, a->steps, a->pos, a->vel,
                         a->rel_pos, a->m_w, a->m_s, a->xi, a->cells, a->water_removed, a->active,
                         a->T_p, a->sol, a->delta_m_l, a->N};
    particles_substep(&s, a->dt_sub, a->dt_sub_half, a->no_iter, a->g_set);
    orc_propagate_grid_subloop_step(a->gsf, a->gmp, Nx, Nz, a->p_ref, a->p_ref_inv, dTh, drv,
                                    a->delta_m_l, a->V);
  }
done:
  free(dTh); free(drv); free(div); free(rel);
  return rc;
}

ORC_EXPORT int orc_integrate_adv_step(double* gsf, double* gmp, const double* gv, const double* flux,
    double p_ref, double p_ref_inv, int64_t Nx, int64_t Nz, const double* ranges,
    const double* steps, double V, double* pos, double* vel, int64_t* cells, double* rel_pos,
    double* m_w, double* m_s, double* xi, int sol, double* water_removed, uint8_t* active,
    double* T_p, double* delta_m_l, double dt, double dt_sub, double dt_sub_half,
    double dt_col_over_dV, int scale_dt_cond, int no_col_per_adv, int act_collisions,
    int act_relaxation, const double* prof_r_v, const double* prof_Theta, const double* t_relax,
    int no_iter, double g_set, const double* E, double E_const, int64_t nb, double lo, double bl,
    int64_t* no_cols, const double* rnd, int64_t rnd_len, int64_t* rnd_pos, int64_t N,
    uint64_t seed, int64_t* col_step, int thin) {
  orc_adv_t a = {gsf, gmp, gv, flux, p_ref, p_ref_inv, Nx, Nz, ranges, steps, V, pos, vel, cells,
                 rel_pos, m_w, m_s, xi, sol, water_removed, active, T_p, delta_m_l, dt, dt_sub,
                 dt_sub_half, dt_col_over_dV, scale_dt_cond, no_col_per_adv, act_collisions,
                 act_relaxation, prof_r_v, prof_Theta, t_relax, no_iter, g_set, E, E_const, nb, lo,
                 bl, no_cols, rnd, rnd_len, rnd_pos, N, seed, col_step, thin};
  return adv_step(&a);
}

ORC_EXPORT void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
ORC_EXPORT int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

#ifdef ORC_CRMATH
/* the correctly rounded routines, for their own tests */
ORC_EXPORT void orc_cr_pow_array(const double* x, const double* y, int64_t n, double* out, int* hard) {
  for (int64_t i = 0; i < n; ++i) out[i] = orc_cr_pow(x[i], y[i], &hard[i]);
}
ORC_EXPORT void orc_cr_log_array(const double* x, int64_t n, double* out, int* hard) {
  for (int64_t i = 0; i < n; ++i) out[i] = orc_cr_log(x[i], &hard[i]);
}
#endif
