// Initialisation of the 2-D case on the GPU (init.py:439-1236 with
// generation_SIP_ensemble.py:147-384 and microphysics.py:570-785):
//  - SinSIP mass ensembles of every (level, cell, mode) at once, one thread
//    per ensemble: the bins' sampled masses and lognormal weights in the
//    reference's sequential order, the weight threshold, then compaction;
//  - the equilibrium solute mass fraction of every SIP of a level: the
//    activation maximum of the Koehler curve by Brent's bounded minimisation
//    and the root of S_eq(w_s) - S_amb by a bracketed bisection (the
//    reference calls scipy's fminbound and brentq per SIP);
//  - one saturation-adjustment iteration of a level: the implicit Newton
//    condensation of every SIP (the step's own newton_full) and the per-cell
//    sums of dm * xi and m_w * xi, one warp per cell.
// The host drives the level loop (lacmopy_gb300/init.py).
#include <cuda_runtime.h>

#include "lacmo_internal.cuh"
#include "lacmo_physics.cuh"

namespace lacmo {

// distributions.py:71-96 (the square as a product, as x**2 evaluates)
__device__ __forceinline__ double pdf_lognormal(double x, double mu_log, double sigma_log,
                                                double two_pi_sqrt) {
  const double u = (log(x) - mu_log) / sigma_log;
  return exp(-0.5 * (u * u)) / (x * two_pi_sqrt * sigma_log);
}

struct SinSIPArgs {
  const double* rnd;        // the draws, segment by segment
  const int64_t* rnd_off;   // [S] first draw of each segment
  const int32_t* seg_mode;  // [S]
  const double *mu_m_log, *sigma_m_log, *bin_factor, *m_low;   // [modes]
  const int32_t* l_max;     // [modes]
  double eta;
  const double* two_pi_sqrt;   // device: mode_par[4 n_modes]
  int weak;                 // weak threshold: a second draw per bin
  int64_t S, lmax_cap;
  double *masses, *weights; // [S][lmax_cap], the kept bins first
  int32_t* count;           // [S]
};

// generation_SIP_ensemble.py:147-265 for one (level, cell, mode)
__global__ void k_sinsip(const SinSIPArgs a) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.S;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int k = a.seg_mode[s];
    const int L = a.l_max[k];
    const double* r = a.rnd + a.rnd_off[s];
    const double* r2 = r + L;
    double* M = a.masses + s * a.lmax_cap;
    double* W = a.weights + s * a.lmax_cap;
    double m_left = a.m_low[k], wmax = 0.0;
    for (int b = 0; b < L; ++b) {
      const double m_right = m_left * a.bin_factor[k];
      const double width = m_right - m_left;
      const double mu = m_left + r[b] * width;
      const double w = pdf_lognormal(mu, a.mu_m_log[k], a.sigma_m_log[k], *a.two_pi_sqrt) * width;
      M[b] = mu;
      W[b] = w;
      wmax = (b == 0 || w > wmax) ? w : wmax;
      m_left = m_right;
    }
    const double crit = wmax * a.eta;
    int n = 0;
    for (int b = 0; b < L; ++b) {
      double w = W[b];
      if (w < crit) {
        if (a.weak && r2[b] < w / crit) w = crit;
        else continue;
      }
      M[n] = M[b];
      W[n] = w;
      ++n;
    }
    a.count[s] = n;
  }
}

// the kept bins of every segment, concatenated (off: exclusive sums of
// count); a segment whose range leaves [0, n_out) is skipped
__global__ void k_sinsip_gather(const double* masses, const double* weights, const int32_t* count,
                                const int64_t* off, int64_t S, int64_t lmax_cap,
                                const double* seg_scale, double* m_out, double* xi_out,
                                int64_t n_out) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < S;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int32_t n = count[s];
    if (n < 0 || n > lmax_cap || off[s] < 0 || off[s] + n > n_out) continue;
    for (int b = 0; b < n; ++b) {
      m_out[off[s] + b] = masses[s * lmax_cap + b];
      xi_out[off[s] + b] = weights[s * lmax_cap + b] * seg_scale[s];
    }
  }
}

// microphysics.py:400-445 Kelvin term from the mass fraction, and the
// equilibrium saturation S_eq(w_s) = a_w(w_s) * Kelvin (microphysics.py:
// 531-610), at the ambient temperature T
struct Koehler {
  int sol;
  double T, m_s, rhow, sigw, vol_to_R;
  __device__ double seq(double w) const {
    const double rho = sol == SOL_AS ? rhow * poly_rho_AS(w) : density_NaCl_solution(w, T);
    const double sig = sol == SOL_AS ? surface_tension_AS_sw(w, sigw)
                                     : surface_tension_NaCl_sw(w, sigw);
    double aw;
    if (sol == SOL_AS) {
      aw = LC_PAR_WAT_ACT_AS_0 * w + LC_PAR_WAT_ACT_AS_1;
      aw = aw * w + LC_PAR_WAT_ACT_AS_2;
      aw = aw * w + LC_PAR_WAT_ACT_AS_3;
      aw = aw * w + LC_PAR_WAT_ACT_AS_4;
    } else {
      aw = LC_PAR_WAT_ACT_NACL_0 * w + LC_PAR_WAT_ACT_NACL_1;
      aw = aw * w + LC_PAR_WAT_ACT_NACL_2;
      aw = aw * w + LC_PAR_WAT_ACT_NACL_3;
      aw = aw * w + LC_PAR_WAT_ACT_NACL_4;
    }
    const double kel = exp(2.0 * sig * 1.0E6 * pow(w / m_s, LC_ONE_THIRD) /
                           (LC_R_V * T * pow(rho, 0.66666667) * vol_to_R));
    return aw * kel;
  }
};

// The largest S_eq on [lo, hi] by Brent's bounded minimisation of -S_eq
// (golden sections with parabolic steps; R. P. Brent, Algorithms for
// Minimization without Derivatives, 1973, ch. 5), absolute tolerance xtol.
__device__ double koehler_argmax(const Koehler& K, double lo, double hi, double xtol,
                                 int max_iter) {
  const double g = 0.5 * (3.0 - sqrt(5.0));
  double a = lo, b = hi;
  double v = a + g * (b - a), w = v, x = v;
  double fx = -K.seq(x), fv = fx, fw = fx;
  double d = 0.0, e = 0.0;
  for (int it = 0; it < max_iter; ++it) {
    const double m = 0.5 * (a + b);
    const double tol = 1.4901161193847656e-08 * fabs(x) + xtol / 3.0;
    const double t2 = 2.0 * tol;
    if (fabs(x - m) <= t2 - 0.5 * (b - a)) break;
    bool golden = true;
    if (fabs(e) > tol) {
      double r = (x - w) * (fx - fv);
      double q = (x - v) * (fx - fw);
      double p = (x - v) * q - (x - w) * r;
      q = 2.0 * (q - r);
      if (q > 0.0) p = -p;
      q = fabs(q);
      const double et = e;
      e = d;
      if (fabs(p) < fabs(0.5 * q * et) && p > q * (a - x) && p < q * (b - x)) {
        d = p / q;
        const double u = x + d;
        if (u - a < t2 || b - u < t2) d = x < m ? tol : -tol;
        golden = false;
      }
    }
    if (golden) {
      e = (x < m ? b : a) - x;
      d = g * e;
    }
    const double u = fabs(d) >= tol ? x + d : (d > 0.0 ? x + tol : x - tol);
    const double fu = -K.seq(u);
    if (fu <= fx) {
      if (u < x) b = x; else a = x;
      v = w; fv = fw; w = x; fw = fx; x = u; fx = fu;
    } else {
      if (u < x) a = u; else b = u;
      if (fu <= fw || w == x) { v = w; fv = fw; w = u; fw = fu; }
      else if (fu <= fv || v == x || v == w) { v = u; fv = fu; }
    }
  }
  return x;
}

// microphysics.py:686-785: the initial solute mass fraction of every SIP in
// equilibrium with the ambient saturation S (capped at the activation
// maximum; w_s_max where S is below the efflorescence saturation)
__global__ void k_init_mass_fraction(int sol, int64_t n, const double* m_s, double S, double T,
                                     double vol_to_R, double w_max, double solub, double* w_s) {
  const double rhow = density_water(T), sigw = surface_tension_water(T);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const Koehler K{sol, T, m_s[k], rhow, sigw, vol_to_R};
    if (S <= K.seq(w_max)) { w_s[k] = w_max; continue; }
    double w_act = koehler_argmax(K, 1E-8, w_max, 1.0E-12, 500);
    if (!(w_act > 0.0)) w_act = solub;
    w_act *= 1.000001;
    const double S_act = K.seq(w_act);
    if (S > S_act) { w_s[k] = w_act; continue; }
    // S_eq falls from S_act at w_act to S_eq(w_max) < S: bisection to the
    // last bit
    double lo = w_act, hi = w_max;
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      if (K.seq(mid) - S > 0.0) lo = mid; else hi = mid;
    }
    const double flo = fabs(K.seq(lo) - S), fhi = fabs(K.seq(hi) - S);
    w_s[k] = flo <= fhi ? lo : hi;
  }
}

// init.py:887-960: one implicit Newton condensation step of every SIP of a
// level at the level's T, p and per-cell S (capped) and e_s; one warp per
// cell (SIPs of a cell are contiguous: off[c] .. off[c + 1]); writes m_w and
// the cell sums of dm * xi and m_w * xi
__global__ void k_sat_adjust(int sol, int64_t cells, const int64_t* off, int64_t n_sips,
                             double* m_w, const double* m_s, const double* xi, const double* S2,
                             const double* e_s, double T, double p, double L_v, double K,
                             double D_v, double dt, int no_iter, double* dml_cell,
                             double* mwxi_cell) {
  const int lane = threadIdx.x & 31;
  const int64_t c = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= cells) return;
  const CellAmb amb = make_cell_amb(T, p, S2[c], e_s[c], L_v, K, D_v);
  double sd = 0.0, sm = 0.0;
  // the cell's SIPs, clipped to [0, n_sips)
  const int64_t k0 = off[c] < 0 ? 0 : off[c];
  const int64_t k1 = off[c + 1] > n_sips ? n_sips : off[c + 1];
  for (int64_t k = k0 + lane; k < k1; k += 32) {
    const double mw = m_w[k], ms = m_s[k];
    const double m_p = mw + ms;
    const double w = ms / m_p;
    const double rho = sol == SOL_AS ? amb.rhow * poly_rho_AS(w) : density_NaCl_solution(w, T);
    const double R = radius_from_mass(m_p, rho);
    // the water's surface tension, as init.py:906 passes it
    const double dm = newton_full(sol, dt, no_iter, mw, ms, w, R, T, rho, amb.sigw, amb, nullptr);
    const double mn = mw + dm;
    m_w[k] = mn;
    sd += dm * xi[k];
    sm += mn * xi[k];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sd += __shfl_down_sync(0xffffffffu, sd, o);
    sm += __shfl_down_sync(0xffffffffu, sm, o);
  }
  if (lane == 0) { dml_cell[c] = sd; mwxi_cell[c] = sm; }
}

static int nblk(int64_t n, int t) {
  int64_t b = (n + t - 1) / t;
  return (int)(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

}  // namespace lacmo

using namespace lacmo;

extern "C" int lacmo_sinsip_generate(const double* rnd, const int64_t* rnd_off,
                                     const int32_t* seg_mode, int64_t n_seg, int n_modes,
                                     const double* mode_par, const int32_t* l_max, double eta,
                                     int weak, int64_t lmax_cap, double* masses, double* weights,
                                     int32_t* count, void* stream) {
  if (!rnd || !rnd_off || !seg_mode || n_seg < 0 || n_modes < 1 || !mode_par || !l_max ||
      lmax_cap < 1 || !masses || !weights || !count)
    return LACMO_ERR_ARG;
  if (n_seg == 0) return LACMO_OK;
  SinSIPArgs a;
  a.rnd = rnd; a.rnd_off = rnd_off; a.seg_mode = seg_mode;
  a.mu_m_log = mode_par; a.sigma_m_log = mode_par + n_modes;
  a.bin_factor = mode_par + 2 * n_modes; a.m_low = mode_par + 3 * n_modes;
  a.l_max = l_max; a.eta = eta; a.two_pi_sqrt = mode_par + 4 * n_modes;
  a.weak = weak; a.S = n_seg; a.lmax_cap = lmax_cap;
  a.masses = masses; a.weights = weights; a.count = count;
  k_sinsip<<<nblk(n_seg, 128), 128, 0, (cudaStream_t)stream>>>(a);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

extern "C" int lacmo_sinsip_gather(const double* masses, const double* weights,
                                   const int32_t* count, const int64_t* off, int64_t n_seg,
                                   int64_t lmax_cap, const double* seg_scale, double* m_out,
                                   double* xi_out, int64_t n_out, void* stream) {
  if (!masses || !weights || !count || !off || n_seg < 0 || lmax_cap < 1 || !seg_scale ||
      !m_out || !xi_out || n_out < 0)
    return LACMO_ERR_ARG;
  if (n_seg == 0) return LACMO_OK;
  k_sinsip_gather<<<nblk(n_seg, 128), 128, 0, (cudaStream_t)stream>>>(
      masses, weights, count, off, n_seg, lmax_cap, seg_scale, m_out, xi_out, n_out);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

extern "C" int lacmo_init_mass_fraction(int solute, int64_t n, const double* m_s, double S_amb,
                                        double T_amb, double volume_to_radius, double w_s_max,
                                        double solubility, double* w_s, void* stream) {
  if ((solute != 0 && solute != 1) || n < 0 || !m_s || !w_s) return LACMO_ERR_ARG;
  if (n == 0) return LACMO_OK;
  k_init_mass_fraction<<<nblk(n, 128), 128, 0, (cudaStream_t)stream>>>(
      solute, n, m_s, S_amb, T_amb, volume_to_radius, w_s_max, solubility, w_s);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}

extern "C" int lacmo_saturation_adjust_level(int solute, int64_t cells, const int64_t* off,
                                             int64_t n_sips, double* m_w, const double* m_s,
                                             const double* xi,
                                             const double* S_cap, const double* e_s, double T,
                                             double p, double L_v, double K, double D_v,
                                             double dt, int no_iter, double* dml_cell,
                                             double* mwxi_cell, void* stream) {
  if ((solute != 0 && solute != 1) || cells < 1 || !off || n_sips < 0 || !m_w || !m_s || !xi ||
      !S_cap || !e_s || no_iter < 1 || !dml_cell || !mwxi_cell)
    return LACMO_ERR_ARG;
  const int64_t blocks = (cells + 3) / 4;
  k_sat_adjust<<<(unsigned)blocks, 128, 0, (cudaStream_t)stream>>>(
      solute, cells, off, n_sips, m_w, m_s, xi, S_cap, e_s, T, p, L_v, K, D_v, dt, no_iter,
      dml_cell, mwxi_cell);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? LACMO_OK : LACMO_ERR_CUDA;
}
