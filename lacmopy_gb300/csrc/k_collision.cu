// All-or-nothing (AON) collision kernels, bit-exact with the reference.
//
// The reference visits the pairs (i, j), i < j, of a cell in lexicographic
// order and each pair may update SIPs i and j (collision/all_or_nothing.py:
// 553-633).  Two pairs that share no SIP commute exactly, and every pair that
// shares a SIP with (i, j) and comes earlier lexicographically has a smaller
// index sum i + j, every later one a larger sum.  So processing the
// anti-diagonals s = i + j = 1 .. 2n-3 in order, the pairs of one diagonal in
// parallel, gives the sequential result bit for bit: 2n-3 barrier steps of at
// most n/2 independent pairs.  The collision counters are integer sums.
//
// Bit-exactness also needs the reference's floating-point operation order
// (this file is compiled with -fmad=false, so no a*b+c is fused) and the same
// pow/log values: the radius (3/(4 pi) m/rho)^(1/3) and the kernel bin
// int((log R - a)/b + 0.5) use the correctly-rounded routines of
// lacmo_crmath.h.  Draws come either from an injected buffer in the
// reference's consumption order or from Philox4x32-10.
#include <cuda_runtime.h>

#include <atomic>

#include "lacmo_crmath.h"
#include "lacmo_internal.cuh"
#include "lacmo_physics.cuh"
#include "lacmo_thin.h"

namespace lacmo {

// x^(1/3 rounded to double) correctly rounded, fast path.  With c = double(1/3)
// = 1/3 - d, d = 2^-54/3, the value is cbrt(x) * exp(-d ln x).  y = cbrt(x)
// (faithful) is refined by one Newton step whose residual x - y^3 is formed in
// double-double, and exp(-d ln x) = 1 - d L + (d L)^2/2 to far below 2^-100.
// So z = y + t with t computed to ~2^-100 |y|.  The rounded sum y + t is the
// correctly-rounded result unless y + t lies within 2^-85 |y| of a rounding
// midpoint; then (or for non-normal x) the full routine decides.  The margin
// is wider than the full routine's own uncertainty, so both always agree.
__device__ __forceinline__ double cr_pow13_dd(double x) {
  if (!(x >= 0x1p-1000 && x <= 0x1p1000)) return lacmo_cr_pow(x, LC_ONE_THIRD);
  const double y = cbrt(x);
  const lacmo_dd y2 = lacmo_two_prod(y, y);
  const lacmo_dd y3 = lacmo_dd_mul_d(y2, y);
  const double r = (x - y3.hi) - y3.lo;           // x - y3.hi is exact (Sterbenz)
  const double corr = r / (3.0 * y2.hi);
  const double dL = 0x1.5555555555555p-56 * log(x);  // d * ln x, d = 2^-54 / 3
  const double t = corr - y * dL + y * (0.5 * dL * dL);
  const double s = y + t;
  const double e = (y - s) + t;                   // y + t = s + e exactly
  const uint64_t b = lacmo_as_u64(s);
  const int64_t ex = (int64_t)((b >> 52) & 0x7ff);
  double half_ulp = lacmo_as_f64((uint64_t)(ex - 53) << 52);
  if (e < 0.0 && (b & 0x000fffffffffffffULL) == 0) half_ulp *= 0.5;
  if (fabs(fabs(e) - half_ulp) <= 0x1p-85 * s) return lacmo_cr_pow(x, LC_ONE_THIRD);
  return s;
}

// The same value with most of the FP64 work moved to FP32 (GB300's FP64 pipe
// is narrow, and the collision events run on single lanes).  For x in
// [2^-40, 2^40] (every radius from 1 nm to 1 cm in micrometres):
//  - y: the FP32 cube root (a few ulp) refined by two Newton steps
//    y += (x - y^3) / (3 y^2), the residual in FP64 and the quotient in FP32:
//    the error goes 2^-21 -> 2^-43 -> within about an ulp (FP64 rounding of
//    the residual);
//  - t = r / (3 y^2) - y d ln x with r = x - y^3 in double-double as above,
//    both terms in FP32: |r / (3 y^2)| < 2^-50 y and |y d ln x| < 2^-46 y,
//    each within 2^-22 relative, their sum within 2^-24 of the larger, and the
//    neglected (d ln x)^2 / 2 below 2^-92: t is within 2^-67 y of its value;
//  - a flushed FP32 residual (|r| < 2^-126) changes t by less than
//    2^-126 / (3 x) <= 2^-86 y.
// s = y + t is then the correctly-rounded result unless it lies within
// 2^-62 s of a rounding midpoint (about one call in 500), where cr_pow13_dd
// decides.
__device__ __forceinline__ double cr_pow13(double x) {
  if (!(x >= 0x1p-40 && x <= 0x1p40)) return cr_pow13_dd(x);
  const float xf = d2f_int(x);
  double y = f2d_int(f_cbrt(xf));
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const float yf = d2f_int(y);
    const double r0 = x - (y * y) * y;
    y = y + f2d_int(d2f_int(r0) * f_rcp(3.0f * yf * yf));
  }
  const lacmo_dd y2 = lacmo_two_prod(y, y);
  const lacmo_dd y3 = lacmo_dd_mul_d(y2, y);
  const double r = (x - y3.hi) - y3.lo;
  const float yf = d2f_int(y);
  const float tf = d2f_int(r) * f_rcp(3.0f * yf * yf) -
                   yf * (0x1.555556p-56f * (f_lg2(xf) * 0.693147181f));
  const double t = f2d_int(tf);
  const double s = y + t;
  const double e = (y - s) + t;
  const uint64_t b = lacmo_as_u64(s);
  const int64_t ex = (int64_t)((b >> 52) & 0x7ff);
  double half_ulp = lacmo_as_f64((uint64_t)(ex - 53) << 52);
  if (e < 0.0 && (b & 0x000fffffffffffffULL) == 0) half_ulp *= 0.5;
  if (fabs(fabs(e) - half_ulp) <= 0x1p-62 * s) return cr_pow13_dd(x);
  return s;
}

__device__ __forceinline__ double col_radius(double m, double rho) {
  return cr_pow13(LC_FOUR_PI_OVER_THREE_INV * m / rho);
}
// collision/all_or_nothing.py:35-67; float -> int as x86-64 compiled code
// does it (NaN / out of range -> INT64_MIN -> bin 0).  The bin of the
// correctly-rounded log: with the hardware log the index value is within
// 1e-12 of it, so unless it lies within 1e-9 of an integer the truncation is
// the same; near a bin edge the correctly-rounded log decides.
__device__ __forceinline__ int32_t col_bin(double R, double lo, double bl, int64_t nb) {
  double v = (log(R) - lo) / bl + 0.5;
  const double fl = floor(v);
  if (!(v - fl > 1e-9 && (fl + 1.0) - v > 1e-9 && fabs(v) < 1e15))
    v = (lacmo_cr_log(R) - lo) / bl + 0.5;
  int64_t ind = (v > -9.2233720368547758e18 && v < 9.2233720368547758e18) ? (int64_t)v : INT64_MIN;
  if (ind < 0) ind = 0;
  else if (ind > nb - 1) ind = nb - 1;
  return (int32_t)ind;
}
// The same bin from an FP32 bin position first: lo_f, inv_bl_f are lo and 1/bl
// rounded to FP32 and margin bounds the error of the FP32 position (it is
// derived for radii within 1e-6; R is rounded to within 2^-24 here).  A
// position farther than margin from every bin edge gives the bin of the exact
// position; closer ones take col_bin.
__device__ __forceinline__ int32_t col_bin_f(double R, double lo, double bl, int64_t nb,
                                             float lo_f, float inv_bl_f, float margin) {
  const float Rf = d2f_int(R);
  const float v = (f_lg2(Rf) * 0.693147181f - lo_f) * inv_bl_f + 0.5f;
  const float fl = floorf(v);
  if (v - fl > margin && (fl + 1.0f) - v > margin && v > -1e6f && v < 1e6f && Rf > 1e-30f &&
      Rf < 1e30f) {
    int32_t kb = __float2int_rz(fl);
    return kb < 0 ? 0 : (kb > nb - 1 ? (int32_t)nb - 1 : kb);
  }
  return col_bin(R, lo, bl, nb);
}
__device__ __forceinline__ int64_t pair_rank(int64_t i, int64_t j, int64_t n) {
  return i * n - i * (i + 1) / 2 + (j - i - 1);
}

// ---------------------------------------------------------------------------
// 2-D cells: one warp per cell (collision/all_or_nothing.py:498-635, 637-751,
// 754-846).  SIP state of cells with up to CELL_SMEM SIPs lives in shared
// memory; larger cells use per-SIP global scratch.
constexpr int CELL_SMEM = 256;
constexpr int CELL_WARPS = 8;

// one collection of the sequential order, as a log record for the adjoint's
// replay (recorded events): kind 0 ordinary, 1 equal-xi split (a, b: xi of
// imin and imax before), 2 multiple collection (a: p_crit)
struct EvRec {
  int32_t imin, imax, kind, pad;
  double a, b;
};

struct CellArgs {
  EvRec* log;                       // event log (single states), or null
  int64_t log_cap;
  unsigned long long* log_count;
  double *xi, *m_w, *m_s;
  const double* vel;
  const double* T;
  const int32_t *start, *perm;
  const int64_t* draw_off;
  int64_t n, C;
  double dtdv;
  const double* E;
  double E_const;
  int64_t nb;
  double lo, bl;
  int sol;
  const double* draws;
  int64_t n_draws;
  uint64_t seed;
  const int64_t *cursor, *col_step, *total_pairs;
  int64_t* no_cols;
  uint32_t* flags;
  double *gR, *grho;   // per SIP: exact radius and density, or the step-start m_p, m_s
  int32_t* gk;         // per SIP: exact kernel bin, or -1 while gR/grho hold m_p, m_s
  float dtdv_f, lo_f, inv_bl_f, E_const_f;   // FP32 copies for the screen
  float bin_margin;    // distance from a bin edge below which the FP32 bin is not trusted
  const float* Ef;     // FP32 efficiency table, or null (then E is read and rounded)
  const int32_t* cell_order;   // cells, largest first
  int32_t* cell_ctr;           // next cell_order entry to take
  float* gcopy;                // [6][n] FP32 copies by slot, for cells above CELL_SMEM
  float4* gstats;              // block statistics of cells above CELL_SMEM (thinned draws)
  const float* erow;           // largest FP32 efficiency of each table row (thinned draws)
  int thin;                    // thinned Philox draws (lacmo_thin.h)
};

// the parameters a collision step shares across members
struct CellCommon {
  EvRec* log;
  int64_t log_cap;
  unsigned long long* log_count;
  double dtdv;
  const double* E;
  double E_const;
  int64_t nb;
  double lo, bl;
  int sol;
  const double* draws;
  int64_t n_draws;
  float dtdv_f, lo_f, inv_bl_f, E_const_f, bin_margin;
  const float* Ef;
  const float* erow;
  int thin;
};
struct CK {
  MRef m;
  CellCommon cc;
};
__device__ __forceinline__ void make_cellargs(CellArgs& a, const Member& mb, const CellCommon& cc) {
  a.log = cc.log; a.log_cap = cc.log_cap; a.log_count = cc.log_count;
  a.xi = mb.sp.xi; a.m_w = mb.sp.m_w; a.m_s = mb.sp.m_s; a.vel = mb.sp.vel;
  a.T = mb.g.scalar_fields;
  a.start = mb.w.start; a.perm = mb.w.perm; a.draw_off = mb.w.draw_off;
  a.n = mb.sp.n; a.C = mb.g.nx * mb.g.nz;
  a.dtdv = cc.dtdv; a.E = cc.E; a.E_const = cc.E_const; a.nb = cc.nb; a.lo = cc.lo; a.bl = cc.bl;
  a.sol = cc.sol; a.draws = cc.draws; a.n_draws = cc.n_draws; a.seed = mb.seed;
  a.cursor = mb.w.cursor; a.col_step = mb.w.col_step; a.total_pairs = mb.w.total_pairs;
  a.no_cols = mb.sp.no_cols; a.flags = mb.w.flags;
  a.gR = mb.w.colR; a.grho = mb.w.colrho; a.gk = mb.w.colk;
  a.dtdv_f = cc.dtdv_f; a.lo_f = cc.lo_f; a.inv_bl_f = cc.inv_bl_f; a.E_const_f = cc.E_const_f;
  a.bin_margin = cc.bin_margin;
  a.Ef = cc.Ef;
  a.cell_order = mb.w.cell_order; a.cell_ctr = mb.w.cell_ctr;
  a.gcopy = mb.w.gcopy;
  a.gstats = (float4*)mb.w.gstats;
  a.erow = cc.erow;
  a.thin = cc.thin;
}

// integer-unit conversions (GB300 runs FP64 conversions on its narrow FP64
// pipe): round to nearest even, and truncation toward zero for r >= 0
__device__ __noinline__ float d2f_rn_slow(double x) { return (float)x; }
__device__ __forceinline__ float d2f_rn(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e - 897u > 253u) return d2f_rn_slow(x);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const uint64_t m = b & 0x000fffffffffffffull;
  const uint32_t fm = (uint32_t)(m >> 29), rem = (uint32_t)m & 0x1fffffffu;
  uint32_t fb = sign | ((e - 896u) << 23) | fm;
  fb += (rem > 0x10000000u) || (rem == 0x10000000u && (fm & 1u));
  return __int_as_float((int)fb);
}
// round to nearest even with zero/subnormal results flushed to zero and
// overflow (and NaN) to infinity: integer instructions only (screen inputs,
// where a flushed value makes the pair undecided or stays inside the bounds)
__device__ __forceinline__ float d2f_flush(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  if (e < 897u) return __int_as_float((int)sign);
  if (e > 1150u) return __int_as_float((int)(sign | 0x7f800000u));
  const uint64_t m = b & 0x000fffffffffffffull;
  const uint32_t fm = (uint32_t)(m >> 29), rem = (uint32_t)m & 0x1fffffffu;
  uint32_t fb = sign | ((e - 896u) << 23) | fm;
  fb += (rem > 0x10000000u) || (rem == 0x10000000u && (fm & 1u));
  return __int_as_float((int)fb);
}
__device__ __forceinline__ float d2f_down_pos(double r) {  // r in [0, 1)
  const uint64_t b = (uint64_t)__double_as_longlong(r);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e < 897u) return 0.0f;
  return __int_as_float((int)(((e - 896u) << 23) | (uint32_t)((b >> 29) & 0x7fffffu)));
}

// Exact per-SIP collision data (collision/all_or_nothing.py:812-826), kept
// in gR / grho / gk and computed on first need.  The density belongs to the
// step-start masses and the cell temperature (the reference keeps it for the
// whole step); the radius and its kernel bin follow from the current masses
// and that density, which the reference recomputes after every collection
// (all_or_nothing.py:596-633).  A radius only matters when an exact
// evaluation reads it, so after a collection it is recomputed lazily:
//   gk = GK_NONE:  nothing computed; gR, grho hold the step-start m_p, m_s
//   gk = GK_STALE: grho holds the density; gR, gk are out of date
//   gk >= 0:       gR, gk are the exact radius and bin of the current masses
constexpr int32_t GK_NONE = -1, GK_STALE = -2;
__device__ __forceinline__ double density_of(const CellArgs& a, double m_p, double ms, double Tc) {
  const double w_s = ms / m_p;
  return (a.sol == SOL_AS) ? density_water(Tc) * poly_rho_AS(w_s)
                           : density_NaCl_solution(w_s, Tc);
}
__device__ __noinline__ void compute_density(const CellArgs& a, int32_t id, double Tc) {
  a.grho[id] = density_of(a, a.gR[id], a.grho[id], Tc);
  a.gk[id] = GK_STALE;
}
__device__ __forceinline__ void ensure_density(const CellArgs& a, int32_t id, double Tc) {
  if (a.gk[id] == GK_NONE) compute_density(a, id, Tc);
}
__device__ __noinline__ void compute_exact(const CellArgs& a, int32_t id, double Tc, bool use_E) {
  if (a.gk[id] == GK_NONE) a.grho[id] = density_of(a, a.gR[id], a.grho[id], Tc);
  const double R = col_radius(a.m_w[id] + a.m_s[id], a.grho[id]);
  a.gR[id] = R;
  a.gk[id] = use_E ? col_bin_f(R, a.lo, a.bl, a.nb, a.lo_f, a.inv_bl_f, a.bin_margin) : 0;
}
// the exact kernel bin of SIP id from its current masses, stored nowhere
__device__ __noinline__ int32_t exact_bin_of(const CellArgs& a, int32_t id, double Tc) {
  const double m_p = a.m_w[id] + a.m_s[id];
  return col_bin(col_radius(m_p, density_of(a, m_p, a.m_s[id], Tc)), a.lo, a.bl, a.nb);
}
__device__ __forceinline__ void ensure_exact(const CellArgs& a, int32_t id, double Tc, bool use_E) {
  if (a.gk[id] < 0) compute_exact(a, id, Tc, use_E);
}

// FP32 copies of a cell's SIPs: v = (xi, R, u, w) per SIP, the kernel bin
// and the SIP ID; in a warp's shared-memory slice, or in the cell's slots of
// the global scratch for cells above the shared-memory size
struct CellSmem {
  float4* v;
  int32_t *sk, *sid;
  float4* st;   // thinned draws: statistics of block b at st[2b], st[2b + 1]
};

// SIP id's masses changed in a collection: its exact radius and bin become
// stale, and its FP32 copies at slot l follow now from the FP32 masses and
// the step-start density (the radius within the screen's 1e-6, as at the
// cell's load; a bin near an edge is computed exactly, as there).
__device__ __noinline__ void masses_changed(const CellArgs& a, const CellSmem* S, int32_t id,
                                            int l, double Tc, bool use_E) {
  a.gk[id] = GK_STALE;
  if (!S) return;
  const float Rf = lt_cbrtf((float)LC_FOUR_PI_OVER_THREE_INV * d2f_rn(a.m_w[id] + a.m_s[id]) /
                            d2f_rn(a.grho[id]));
  int32_t kb = 0;
  if (use_E) {
    const float v = (__logf(Rf) - a.lo_f) * a.inv_bl_f + 0.5f;
    const float fl = floorf(v);
    if (v - fl > a.bin_margin && (fl + 1.0f) - v > a.bin_margin && v > -1e6f && v < 1e6f &&
        Rf > 0.f) {
      kb = __float2int_rz(fl);
      kb = kb < 0 ? 0 : (kb > a.nb - 1 ? (int32_t)a.nb - 1 : kb);
    } else {
      compute_exact(a, id, Tc, use_E);
      kb = a.gk[id];
    }
  }
  S->v[l].y = Rf;
  S->sk[l] = kb;
}

// append a collection to the event log; a cell's events come from one warp
// in its sequential order, one at a time, so their slots increase in that
// order (slots past the capacity are counted, not written)
__device__ __noinline__ void log_event(const CellArgs& a, int32_t imin, int32_t imax, int kind,
                                       double x, double y) {
  const unsigned long long slot = atomicAdd(a.log_count, 1ull);
  if (slot < (unsigned long long)a.log_cap) {
    EvRec r;
    r.imin = imin; r.imax = imax; r.kind = kind; r.pad = 0; r.a = x; r.b = y;
    a.log[slot] = r;
  }
}

// One ordinary collection (p_crit <= 1 and p_crit > r) of the pair imin/imax
// (collision/all_or_nothing.py:607-633) on the global arrays; the density of
// imin must be known.  S (may be null) receives the FP32 copies at local
// slots lmin/lmax.
__device__ __forceinline__ void collect_once(const CellArgs& a, const CellSmem* S, int32_t imin,
                                             int32_t imax, int lmin, int lmax, double Tc,
                                             bool use_E) {
  double *XI = a.xi, *MW = a.m_w, *MS = a.m_s, *RR = a.gR;
  const double* RHO = a.grho;
  const double xi_min = XI[imin], xi_max = XI[imax];
  const double m_w_min = MW[imin], m_w_max = MW[imax];
  const double m_s_min = MS[imin], m_s_max = MS[imax];
  const double xi_rel_dev = (xi_max - xi_min) / xi_max;
  if (xi_rel_dev < 1.0E-5) {
    if (a.log) log_event(a, imin, imax, 1, xi_min, xi_max);
    // both radii follow from imin's density (all_or_nothing.py:615-624):
    // computed now, not left stale
    ensure_density(a, imax, Tc);
    const double xi_ges = xi_min + xi_max;
    MW[imin] = 2.0 * (xi_min * m_w_min + xi_max * m_w_max) / xi_ges;
    MS[imin] = 2.0 * (xi_min * m_s_min + xi_max * m_s_max) / xi_ges;
    MW[imax] = MW[imin];
    MS[imax] = MS[imin];
    RR[imin] = col_radius((MW[imin] + MS[imin]), RHO[imin]);
    RR[imax] = RR[imin];
    XI[imax] = 0.5 * 0.7 * xi_ges;
    XI[imin] = 0.5 * xi_ges - XI[imax];
    a.gk[imin] = use_E ? col_bin_f(RR[imin], a.lo, a.bl, a.nb, a.lo_f, a.inv_bl_f, a.bin_margin)
                       : 0;
    a.gk[imax] = a.gk[imin];
    if (S) {
      S->v[lmin].x = d2f_rn(XI[imin]); S->v[lmax].x = d2f_rn(XI[imax]);
      S->v[lmin].y = d2f_rn(RR[imin]); S->v[lmax].y = S->v[lmin].y;
      S->sk[lmin] = a.gk[imin]; S->sk[lmax] = a.gk[imax];
    }
  } else {
    if (a.log) log_event(a, imin, imax, 0, 0.0, 0.0);
    MW[imin] += m_w_max;
    MS[imin] += m_s_max;
    XI[imax] -= xi_min;
    masses_changed(a, S, imin, lmin, Tc, use_E);
    if (S) S->v[lmax].x = d2f_rn(XI[imax]);
  }
}

// Exact FP64 evaluation of the pair ii/jj (collision/all_or_nothing.py:
// 553-633) in the reference's operation order, on the global arrays.  Returns
// 0 (no collision), 1 (one collection) or 2 (multiple collection).  Sm holds
// the warp's shared-memory slice, or null (cells above its size).
__device__ __noinline__ int exact_pair(const CellArgs& a, CellSmem Sm, int32_t ii, int32_t jj,
                                       int li, int lj, double Tc, bool use_E, double r) {
  const CellSmem* S = &Sm;
  ensure_exact(a, ii, Tc, use_E);
  ensure_exact(a, jj, Tc, use_E);
  double *XI = a.xi, *MW = a.m_w, *MS = a.m_s, *RR = a.gR;
  const double *U = a.vel, *W = a.vel + a.n;
  int32_t imin, imax;
  int lmin, lmax;
  if (XI[ii] <= XI[jj]) { imin = ii; imax = jj; lmin = li; lmax = lj; }
  else { imin = jj; imax = ii; lmin = lj; lmax = li; }
  const double xi_min = XI[imin], xi_max = XI[imax];
  const double Rs = RR[ii] + RR[jj];
  const double e = use_E ? __ldg(a.E + (int64_t)a.gk[ii] * a.nb + a.gk[jj]) : a.E_const;
  const double du = U[ii] - U[jj], dw = W[ii] - W[jj];
  const double dv = sqrt(du * du + dw * dw);
  const double p_crit = xi_max * a.dtdv * (LC_PI * Rs * Rs * e * dv * 1.0E-12);
  if (p_crit > 1.0) {
    if (a.log) log_event(a, imin, imax, 2, p_crit, 0.0);
    const double xi_col = p_crit * xi_min;
    MW[imin] = MW[imin] + p_crit * MW[imax];
    MS[imin] = MS[imin] + p_crit * MS[imax];
    XI[imax] -= xi_col;
    masses_changed(a, S, imin, lmin, Tc, use_E);
    if (S) S->v[lmax].x = d2f_rn(XI[imax]);
    return 2;
  }
  if (!(p_crit > r)) return 0;
  collect_once(a, S, imin, imax, lmin, lmax, Tc, use_E);
  return 1;
}

// A pair the FP32 bounds place certainly in an ordinary collection.
__device__ __noinline__ void certain_collection(const CellArgs& a, CellSmem S, int i, int j,
                                                double Tc, bool use_E) {
  const int32_t ii = S.sid[i], jj = S.sid[j];
  const bool lo_i = a.xi[ii] <= a.xi[jj];
  const int32_t imin = lo_i ? ii : jj, imax = lo_i ? jj : ii;
  ensure_density(a, imin, Tc);
  collect_once(a, &S, imin, imax, lo_i ? i : j, lo_i ? j : i, Tc, use_E);
}

__device__ __noinline__ double philox_from_bits(uint64_t k53) {
  return (double)k53 * (1.0 / 9007199254740992.0);
}

// FP32 screen of the pair (i, j): 0 = certainly no collision, 1 = certainly
// one ordinary collection (0 < p_crit <= 1 and p_crit > r), 2 = undecided
// (the exact FP64 evaluation decides).  Two-sided bounds of p_crit: the FP32
// radii are within 1e-6 (relative) of the exact ones, every other FP32
// operation and conversion within 2^-24, the velocity difference carries an
// absolute slack for its cancellation, and the bounds are widened by 2^-14
// relative (and 1e-36 absolute); |du| + |dw| in place of the Euclidean norm
// gives a looser upper bound that decides most skips alone.  Non-positive
// multiplicities (left by multiple collections) are undecided.  [r_lo, r_hi]
// brackets the draw.
__device__ __forceinline__ int screen_pair(const CellArgs& a, bool use_E, float4 vi, int32_t ki,
                                           float4 vj, int32_t kj, float r_lo, float r_hi) {
  const float du = vi.z - vj.z, dw = vi.w - vj.w;
  const float adu = fabsf(du), adw = fabsf(dw);
  const float slack = 0x1p-21f * (fabsf(vi.z) + fabsf(vj.z) + fabsf(vi.w) + fabsf(vj.w));
  const float rs = vi.y + vj.y;
  float ef = a.E_const_f;
  if (use_E) {
    const int64_t ke = (int64_t)ki * a.nb + kj;
    ef = a.Ef ? __ldg(a.Ef + ke) : d2f_flush(__ldg(a.E + ke));
  }
  const float core = ((fmaxf(vi.x, vj.x) * a.dtdv_f) * (float)(LC_PI * 1.0E-12)) * rs * rs * ef;
  const bool sane = vi.x > 0.0f && vj.x > 0.0f && core >= 1e-30f;
  // common case first: |du| + |dw| >= |(du, dw)| gives an upper bound without
  // the square root, enough to skip the pair when the draw is above it
  const float p_l1 = core * ((adu + adw) + slack) * (1.0f + 0x1p-14f) + 1e-36f;
  if (sane && p_l1 < 1.0f && p_l1 < r_lo) return 0;
  const float dvm = sqrtf(du * du + dw * dw);
  const float p_hi = core * (dvm + slack) * (1.0f + 0x1p-14f) + 1e-36f;
  const float p_lo = core * fmaxf(dvm - slack, 0.0f) * (1.0f - 0x1p-14f);
  const bool ok = sane && p_hi < 1.0f;
  if (ok && p_hi < r_lo) return 0;
  if (ok && p_lo > r_hi) return 1;
  return 2;
}
// draw intervals: Philox bits (exact: r - r_lo < 2^-24) or an injected draw
// (an injected draw outside [0, 1) gives an empty interval: undecided)
__device__ __forceinline__ void philox_interval(uint64_t k53, float& r_lo, float& r_hi) {
  r_lo = (float)(uint32_t)(k53 >> 29) * 0x1p-24f;
  r_hi = r_lo + 0x1p-24f;
}
__device__ __forceinline__ void injected_interval(double r, float& r_lo, float& r_hi) {
  const uint64_t rb = (uint64_t)__double_as_longlong(r);
  const bool in01 = rb < 0x3ff0000000000000ull;
  r_lo = in01 ? d2f_down_pos(r) : 2.0f;
  r_hi = in01 ? r_lo + 0x1p-24f : -1.0f;
}

// the exact data of a cell's SIPs, computed lazily from the step-start masses
__device__ __forceinline__ void init_exact_scratch(const CellArgs& a, const CellSmem& S, int n,
                                                   int lane) {
  for (int q = lane; q < n; q += 32) {
    const int32_t id = S.sid[q];
    a.gR[id] = a.m_w[id] + a.m_s[id];
    a.grho[id] = a.m_s[id];
    a.gk[id] = -1;
  }
  __syncwarp();
}

// one pair with draw r: the screen on the FP32 copies, else the exact
// evaluation; returns 0 (no change) or the outcome counters it adds
__device__ __forceinline__ void decide_pair(const CellArgs& a, const CellSmem& S, bool use_E,
                                            int i, int j, double r, float r_lo, float r_hi,
                                            double Tc, int64_t& c0, int64_t& c1) {
  const int sc = screen_pair(a, use_E, S.v[i], S.sk[i], S.v[j], S.sk[j], r_lo, r_hi);
  if (sc == 0) return;
  if (sc == 1) {
    certain_collection(a, S, i, j, Tc, use_E);
    c0 += 1;
    return;
  }
  const int o = exact_pair(a, S, S.sid[i], S.sid[j], i, j, Tc, use_E, r);
  c0 += o == 1;
  c1 += o == 2;
}

// order-preserving keys of non-NaN floats (for warp min/max reductions)
__device__ __forceinline__ uint32_t ord_key(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord_val(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// statistics (lt_block_stats) of block b, slots [32 b, min(32 b + 32, n)),
// from the FP32 copies, warp-cooperative: st[2b] = (xmax, Rmax, umin, umax),
// st[2b + 1] = (wmin, wmax, ok, 0)
__device__ __forceinline__ void block_stats(const CellSmem& S, int n, int b, int lane) {
  constexpr unsigned FULL = 0xffffffffu;
  const int q = (b << 5) + lane;
  const bool in = q < n;
  const float4 v = in ? S.v[q] : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  const bool bad = in && !(v.x > 0.0f && v.y == v.y && v.z == v.z && v.w == v.w);
  const int ok = __ballot_sync(FULL, bad) == 0u;
  const uint32_t xk = __reduce_max_sync(FULL, in ? ord_key(v.x) : 0u);
  const uint32_t Rk = __reduce_max_sync(FULL, in ? ord_key(v.y) : 0u);
  const uint32_t ulo = __reduce_min_sync(FULL, in ? ord_key(v.z) : 0xffffffffu);
  const uint32_t uhi = __reduce_max_sync(FULL, in ? ord_key(v.z) : 0u);
  const uint32_t wlo = __reduce_min_sync(FULL, in ? ord_key(v.w) : 0xffffffffu);
  const uint32_t whi = __reduce_max_sync(FULL, in ? ord_key(v.w) : 0u);
  if (lane == 0) {
    S.st[2 * b] = make_float4(ord_val(xk), ord_val(Rk), ord_val(ulo), ord_val(uhi));
    S.st[2 * b + 1] = make_float4(ord_val(wlo), ord_val(whi), __int_as_float(ok), 0.0f);
  }
}

// segment (i, b) moved forward by `adv` segments (row i holds the segments
// b = (i + 1) / 32 .. B - 1); past the cell's last segment b >= B
__device__ __forceinline__ void advance_seg(int n, int B, int& i, int& b, int adv) {
  b += adv;
  while (b > B - 1 && i < n - 2) {
    ++i;
    b += ((i + 1) >> 5) - B;
  }
}

// The thinned draws of lacmo_thin.h for one cell, warp-cooperative.  A round
// takes 32 consecutive segments, one per lane (lane 0 the current part of the
// current segment): each lane bounds its segment from SIP i and the block
// statistics and, when the bound is below LACMO_THIN_TAU, draws the uniform
// that decides whether the segment holds a draw below q.  Segments with
// neither such a hit nor per-pair draws are done; the first one with either
// is then processed by the warp: per-pair draws screened in parallel, or the
// hit's first-hit draws evaluated by all lanes at once and the hit pair by
// one lane.  The statistics of the blocks it may have changed are refreshed,
// and the next round starts after it.
__device__ __forceinline__ int2 thin_cell(const CellArgs& a, const CellSmem S, int n, double Tc,
                                       bool use_E, uint64_t pc1, int lane) {
  static_assert(LACMO_THIN_L == 32, "one block of slots per warp");
  int c0 = 0, c1 = 0;   // this lane's outcome counts
  constexpr unsigned FULL = 0xffffffffu;
  const int B = (n + 31) >> 5;
  for (int b = 0; b < B; ++b) block_stats(S, n, b, lane);
  __syncwarp();
  int si = 0, sb = 0, sj = 1, ssub = 0;   // current segment, its part start and counter
  bool scratch = false;
  for (;;) {
    // lane l takes the l-th segment from (si, sb): the segments left in rows
    // si, si + 1, ... (one row per lane) summed by a warp scan, then the row
    // holding offset l found by a binary search over the sums
    int cnt = 0;
    {
      const int r = si + lane;
      if (r <= n - 2) cnt = B - (lane ? (r + 1) >> 5 : sb);
    }
    int csum = cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int v = __shfl_up_sync(FULL, csum, off);
      if (lane >= off) csum += v;
    }
    int rho = 0;   // first row k with csum_k > lane
#pragma unroll
    for (int step = 16; step; step >>= 1) {
      const int ck = __shfl_sync(FULL, csum, rho + step - 1);
      if (ck <= lane) rho += step;
    }
    const int before = __shfl_sync(FULL, csum, rho > 0 ? rho - 1 : 0);
    const bool valid = lane < __shfl_sync(FULL, csum, 31);
    const int i = si + rho;
    const int b = (rho ? (i + 1) >> 5 : sb) + lane - (rho ? before : 0);
    const int blo = b << 5;
    const int jfirst = blo > i + 1 ? blo : i + 1;
    const int j = lane ? jfirst : sj;
    const int jend = blo + 32 < n ? blo + 32 : n;
    const uint32_t sub = lane ? 0u : (uint32_t)ssub;
    bool indiv = false, hit = false;
    int e = 0;
    if (valid) {
      const float4 vi = S.v[i];
      const float4 s0 = S.st[2 * b], s1 = S.st[2 * b + 1];
      const lt_block_t st{s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, __float_as_int(s1.z)};
      const float er = use_E ? __ldg(a.erow + S.sk[i]) : a.E_const_f;
      const float Q = lt_segment_bound(vi.x, vi.y, vi.z, vi.w, &st, er, a.dtdv_f);
      indiv = !(Q >= 0.0f && Q < LACMO_THIN_TAU);
      if (!indiv) {
        e = lt_exponent(Q);
        const uint64_t u = lt_bits53(a.seed, (uint64_t)pair_rank(i, jfirst, n), sub, 0u, pc1);
        hit = u < __ldg(&LACMO_THIN_HT[e - LACMO_THIN_E_MIN][jend - j - 1]);
      }
    }
    const unsigned ev = __ballot_sync(FULL, valid && (indiv || hit));
    const bool all_valid = __ballot_sync(FULL, valid) == FULL;
    // the lane's segment, packed into three words for the event loop
    // (n <= 65535 so i, j < 2^16; B <= 2048; e < 128; sub <= 32)
    const uint32_t pk_ij = (uint32_t)i | ((uint32_t)j << 16);
    const uint32_t pk_fe = (uint32_t)jfirst | ((uint32_t)jend << 16);
    const uint32_t pk_b = ((uint32_t)b & 0x7ffu) | ((uint32_t)e << 11) | ((uint32_t)indiv << 18) |
                          (sub << 19);
    // the round's segments with an event, in order.  An event that changes
    // nothing (no collection) leaves the state, and so the bounds and hit
    // draws of the later lanes, as they were: the next event of the round is
    // processed at once.  A collection (or a hit whose segment has pairs
    // left, a new part with its own draw) ends the round; the next one
    // starts after it.
    unsigned pend = ev;
    bool restart = false, cell_done = false;
    while (pend) {
      const int L = __ffs(pend) - 1;
      pend &= pend - 1u;
      const uint32_t qij = __shfl_sync(FULL, pk_ij, L), qfe = __shfl_sync(FULL, pk_fe, L);
      const uint32_t qb = __shfl_sync(FULL, pk_b, L);
      const int ei = (int)(qij & 0xffffu), ej = (int)(qij >> 16);
      const int ejf = (int)(qfe & 0xffffu), eend = (int)(qfe >> 16);
      const int eb = (int)(qb & 0x7ffu), ee = (int)((qb >> 11) & 0x7fu);
      const bool eind = ((qb >> 18) & 1u) != 0;
      const uint32_t esub = qb >> 19;
      if (!scratch) { init_exact_scratch(a, S, n, lane); scratch = true; }
      int next_j = eend;
      bool changed = false;
      if (eind) {
        // per-pair draws of the rest of the segment (pair ej + lane per
        // lane, drawn once), screened in parallel; the candidates are
        // processed in order, and the rest is screened again only after a
        // state change
        const int q = ej + lane;
        const bool mine = q < eend;
        uint64_t k53 = 0;
        float r_lo = 0.0f, r_hi = 0.0f;
        if (mine) {
          k53 = philox_bits53(a.seed, (uint64_t)pair_rank(ei, q, n), pc1);
          philox_interval(k53, r_lo, r_hi);
        }
        unsigned todo = __ballot_sync(FULL, mine);   // pairs not processed yet
        while (todo) {
          int sc = 0;
          if ((todo >> lane) & 1u)
            sc = screen_pair(a, use_E, S.v[ei], S.sk[ei], S.v[q], S.sk[q], r_lo, r_hi);
          unsigned cand = __ballot_sync(FULL, sc != 0);
          bool col_now = false;
          while (cand) {
            const int t = __ffs(cand) - 1;
            int col = 0;
            if (lane == t) {
              if (sc == 1) {
                certain_collection(a, S, ei, q, Tc, use_E);
                c0 += 1;
                col = 1;
              } else {
                const int o = exact_pair(a, S, S.sid[ei], S.sid[q], ei, q, Tc, use_E,
                                         philox_from_bits(k53));
                c0 += o == 1;
                c1 += o == 2;
                col = o != 0;
              }
            }
            col = __shfl_sync(FULL, col, t);
            __threadfence_block();
            __syncwarp();
            todo &= ~((2u << t) - 1u);   // pairs up to t are done
            if (col) { col_now = true; break; }
            cand &= cand - 1u;   // no change: the later screens still hold
          }
          if (!col_now) break;
          changed = true;
        }
      } else {
        // the hit: first-hit draws of all lanes, then the pair with r = q u
        const int m = eend - ej;
        const uint64_t chunk = (uint64_t)pair_rank(ei, ejf, n);
        bool succ = false;
        if (lane < m - 1)
          succ = lt_bits53(a.seed, chunk, esub, (uint32_t)(1 + lane), pc1) <
                 __ldg(&LACMO_THIN_PT[ee - LACMO_THIN_E_MIN][m - lane - 1]);
        const unsigned bal = __ballot_sync(FULL, succ);
        const int g = bal ? __ffs(bal) - 1 : m - 1;
        const uint32_t jd = g < m - 1 ? (uint32_t)(g + 2) : (uint32_t)m;
        int col = 0;
        if (lane == 0) {
          const double r = ldexp((double)lt_bits53(a.seed, chunk, esub, jd, pc1) *
                                     (1.0 / 9007199254740992.0), -ee);
          // a float interval around r: truncation and the next float up
          // (below the normal range: [0, 2^-126])
          const bool normal = r >= 0x1p-126;
          const float r_lo = normal ? d2f_down_pos(r) : 0.0f;
          const float r_hi = normal ? __uint_as_float(__float_as_uint(r_lo) + 1u) : 0x1p-126f;
          int64_t d0 = 0, d1 = 0;
          decide_pair(a, S, use_E, ei, ej + g, r, r_lo, r_hi, Tc, d0, d1);
          c0 += (int)d0;
          c1 += (int)d1;
          col = (d0 | d1) != 0;
        }
        changed = __shfl_sync(FULL, col, 0) != 0;
        __threadfence_block();
        __syncwarp();
        next_j = ej + g + 1;
      }
      const bool part_left = !eind && next_j < eend;
      if (!changed && !part_left) continue;   // the round goes on
      if (changed) {
        // the statistics of the blocks the event may have changed
        block_stats(S, n, ei >> 5, lane);
        if ((ei >> 5) != eb) block_stats(S, n, eb, lane);
        __syncwarp();
      }
      si = ei; sb = eb;
      if (part_left) {
        sj = next_j;
        ssub = (int)esub + 1;
      } else {
        advance_seg(n, B, si, sb, 1);
        if (sb >= B) { cell_done = true; break; }
        sj = (sb << 5) > si + 1 ? (sb << 5) : si + 1;
        ssub = 0;
      }
      restart = true;
      break;
    }
    if (cell_done) break;
    if (restart) continue;
    // every segment of the round is done
    if (!all_valid) break;   // the cell's last segment is done
    si = (int)(__shfl_sync(FULL, pk_ij, 31) & 0xffffu);
    sb = (int)(__shfl_sync(FULL, pk_b, 31) & 0x7ffu);
    advance_seg(n, B, si, sb, 1);
    if (sb >= B) break;
    sj = (sb << 5) > si + 1 ? (sb << 5) : si + 1;
    ssub = 0;
  }
  return make_int2((int)c0, (int)c1);
}

// One warp per cell.  Shared memory holds FP32 copies of xi, R, u, w and the
// kernel bin (24 B per SIP with the SIP ID); the pairs are screened in
// parallel in lexicographic order and only the events of the sequential
// order (collections and undecided pairs) are processed one at a time.
constexpr size_t CELL_WARP_BYTES = (size_t)CELL_SMEM * (4 * 4 + 4 + 4) + (CELL_SMEM / 32) * 32;

// THIN: the thinned draws, else per-pair draws.  MINB: resident blocks per
// SM the register budget is set for (the TUNE_COLLISION_BLOCKS knob picks the
// instance; 3 by default: the thinned rounds gain more from the warps than
// they lose to spills)
template <bool THIN, int MINB>
__global__ void __launch_bounds__(CELL_WARPS * 32, MINB)
    k_collide_cells(const __grid_constant__ CK x) {
  // the member's arguments, once per block (all warps of a block belong to
  // the same member); shared memory keeps them addressable without a copy
  // per thread
  __shared__ CellArgs s_args;
  if (threadIdx.x == 0) make_cellargs(s_args, x.m.get(), x.cc);
  __syncthreads();
  const CellArgs& a = s_args;
  extern __shared__ float4 fsm[];   // 16-byte aligned warp slices
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* const wslice = (float*)((char*)fsm + (size_t)wid * CELL_WARP_BYTES);
  const int64_t cursor = a.draws ? *a.cursor : 0;
  if (a.draws && cursor + *a.total_pairs > a.n_draws) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.flags, LACMO_FLAG_DRAWS_SHORT);
    return;
  }
  const uint64_t cstep = (uint64_t)*a.col_step;
  const bool use_E = a.E != nullptr;
  const float c43 = (float)LC_FOUR_PI_OVER_THREE_INV;
  int64_t c0 = 0, c1 = 0;
  // persistent warps take the member's cells, largest first, from a counter
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(a.cell_ctr, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= a.C) break;
    const int64_t c = a.cell_order[idx];
    const int32_t b = a.start[c];
    const int n = a.start[c + 1] - b;
    if (n < 2) break;   // the remaining cells hold fewer than two SIPs
    if (n > 65535) {    // pair ranks would leave 32 bits
      if (lane == 0) atomicOr(a.flags, LACMO_FLAG_CELL_TOO_BIG);
      continue;
    }
    const double Tc = a.T[c];
    const double* rnd = a.draws ? a.draws + cursor + a.draw_off[c] : nullptr;
    const uint64_t pc1 = (cstep << 32) | (uint64_t)c;
    const int32_t* ids = a.perm + b;
    // cells above the shared-memory size keep their copies in global scratch
    const bool big = n > CELL_SMEM;
    CellSmem S;
    if (big) {
      S.v = (float4*)a.gcopy + b;
      S.sk = (int32_t*)((float4*)a.gcopy + a.n) + b;
      S.sid = S.sk + a.n;
      S.st = a.gstats + 2 * ((int64_t)(b >> 5) + c);
    } else {
      S.v = (float4*)wslice;
      S.sk = (int32_t*)(S.v + CELL_SMEM);
      S.sid = S.sk + CELL_SMEM;
      S.st = (float4*)(S.sid + CELL_SMEM);
    }
    const float Tf = d2f_rn(Tc);
    const float rhow_f = (float)LC_PAR_WATER_DENS_0 +
                         (float)LC_PAR_WATER_DENS_1 * ((Tf - (float)LC_PAR_WATER_DENS_2) *
                                                        (Tf - (float)LC_PAR_WATER_DENS_2));
    // load: FP32 copies, FP32 radius and bin (exact when near a bin edge)
    for (int q = lane; q < n; q += 32) {
      const int32_t id = ids[q];
      const float mwf = d2f_rn(a.m_w[id]), msf = d2f_rn(a.m_s[id]);
      const float mpf = mwf + msf;
      const float wsf = msf / mpf;
      const float rho = (a.sol == SOL_AS)
                            ? rhow_f * ((((float)LC_PAR_RHO_AS_0 * wsf + (float)LC_PAR_RHO_AS_1) *
                                             wsf + (float)LC_PAR_RHO_AS_2) * wsf +
                                        (float)LC_PAR_RHO_AS_3)
                            : (float)LC_PAR_SOL_DENS_NACL_0 + (float)LC_PAR_SOL_DENS_NACL_1 * wsf +
                                  (float)LC_PAR_SOL_DENS_NACL_2 * Tf +
                                  (float)LC_PAR_SOL_DENS_NACL_3 * wsf * wsf +
                                  (float)LC_PAR_SOL_DENS_NACL_4 * wsf * Tf +
                                  (float)LC_PAR_SOL_DENS_NACL_5 * Tf * Tf;
      const float Rf = lt_cbrtf(c43 * mpf / rho);
      int32_t kb = 0;
      if (use_E) {
        const float v = (__logf(Rf) - a.lo_f) * a.inv_bl_f + 0.5f;
        const float fl = floorf(v);
        if (v - fl > a.bin_margin && (fl + 1.0f) - v > a.bin_margin && v > -1e6f && v < 1e6f &&
            Rf > 0.f) {
          kb = __float2int_rz(fl);
          kb = kb < 0 ? 0 : (kb > a.nb - 1 ? (int32_t)a.nb - 1 : kb);
        } else {
          kb = exact_bin_of(a, id, Tc);
        }
      }
      S.v[q] = make_float4(d2f_rn(a.xi[id]), Rf, d2f_rn(a.vel[id]), d2f_rn(a.vel[a.n + id]));
      S.sk[q] = kb;
      S.sid[q] = id;
    }
    __syncwarp();
    const int P = (int)((int64_t)n * (n - 1) / 2);
    if constexpr (THIN) {
      const int2 tc = thin_cell(a, S, n, Tc, use_E, pc1, lane);
      c0 += tc.x;
      c1 += tc.y;
      __syncwarp();
      continue;
    }
    // Speculative sequential order.  From rank pos on, the lanes screen the
    // pairs in parallel with the current state: lane l takes the couples
    // (p0 + 2l + 64t, p0 + 2l + 64t + 1), p0 = pos rounded down to even, in
    // lexicographic order, one Philox block per couple.  The first pair p*
    // the screen does not skip is the next event of the sequential order:
    // every pair before it is skipped with the very state it would see.  The
    // lane that found p* processes it (certain collection or exact FP64
    // evaluation), then screening resumes at p* + 1.  Most cells have no
    // event at all.  A cell with many events finishes with the anti-diagonal
    // schedule from its current position.
    const int event_limit = 16 + P / 64;
    int pos = 0;           // first rank not processed yet
    int bi = 0, bj = 1;    // the pair of rank pos & ~1
    int events = 0;
    bool diagonal = false;
    for (;;) {
      int my_p = 0x7fffffff, my_i = 0, my_j = 0, my_sc = 0;
      uint64_t my_k53 = 0;
      {
        int i = bi, j = bj + 2 * lane, p = (pos & ~1) + 2 * lane;
        for (;;) {
          while (j > n - 1 && i < n - 2) { j += i + 2 - n; ++i; }
          if (j > n - 1) break;
          // the next pair in lexicographic order (absent past the last pair)
          int i2 = i, j2 = j + 1;
          if (j2 > n - 1) { i2 = i + 1; j2 = i + 2; }
          const bool has2 = i2 < n - 1;
          float rl0, rh0, rl1 = 0.f, rh1 = 0.f;
          uint64_t k0 = 0, k1 = 0;
          if (rnd) {
            injected_interval(rnd[p], rl0, rh0);
            if (has2) injected_interval(rnd[p + 1], rl1, rh1);
          } else {
            const PhiloxBlock blk = philox_block(a.seed, (uint64_t)(p >> 1), pc1);
            k0 = philox_half53(blk, false);
            k1 = philox_half53(blk, true);
            philox_interval(k0, rl0, rh0);
            philox_interval(k1, rl1, rh1);
          }
          const float4 vi = S.v[i], vj = S.v[j];
          const int32_t ki = S.sk[i], kj = S.sk[j];
          if (p >= pos) {
            const int sc = screen_pair(a, use_E, vi, ki, vj, kj, rl0, rh0);
            if (sc != 0) { my_p = p; my_i = i; my_j = j; my_sc = sc; my_k53 = k0; break; }
          }
          if (has2) {
            // the couple's second pair shares SIP i unless it starts a new row
            const bool same = i2 == i;
            const float4 vi2 = same ? vi : S.v[i2];
            const int32_t ki2 = same ? ki : S.sk[i2];
            const int sc = screen_pair(a, use_E, vi2, ki2, S.v[j2], S.sk[j2], rl1, rh1);
            if (sc != 0) { my_p = p + 1; my_i = i2; my_j = j2; my_sc = sc; my_k53 = k1; break; }
          }
          j += 64;
          p += 64;
        }
      }
      const int pstar = __reduce_min_sync(0xffffffffu, my_p);
      if (pstar == 0x7fffffff) break;   // no further event in this cell
      if (events == 0) {
        // exact data of the cell's SIPs, computed lazily from the step-start masses
        for (int q = lane; q < n; q += 32) {
          const int32_t id = S.sid[q];
          a.gR[id] = a.m_w[id] + a.m_s[id];
          a.grho[id] = a.m_s[id];
          a.gk[id] = -1;
        }
        __syncwarp();
      }
      const int L = __ffs(__ballot_sync(0xffffffffu, my_p == pstar)) - 1;
      if (lane == L) {
        if (my_sc == 1) {
          certain_collection(a, S, my_i, my_j, Tc, use_E);
          c0 += 1;
        } else {
          const int o = exact_pair(a, S, S.sid[my_i], S.sid[my_j], my_i, my_j, Tc,
                                   use_E, rnd ? rnd[pstar] : philox_from_bits(my_k53));
          c0 += o == 1;
          c1 += o == 2;
        }
      }
      __threadfence_block();
      __syncwarp();
      const int si = __shfl_sync(0xffffffffu, my_i, L), sj = __shfl_sync(0xffffffffu, my_j, L);
      pos = pstar + 1;
      if (pstar & 1) {   // rank pos is even: the successor of p*
        bi = si; bj = sj + 1;
        if (bj > n - 1) { bi = si + 1; bj = si + 2; }
      } else {           // rank pos is odd: its couple starts at p* itself
        bi = si; bj = sj;
      }
      if (pos >= P) break;
      if (++events >= event_limit) { diagonal = true; break; }
    }
    if (diagonal) {
      // anti-diagonal schedule of the pairs from rank pos on
      for (int s = 1; s <= 2 * n - 3; ++s) {
        const int ilo = s - (n - 1) > 0 ? s - (n - 1) : 0;
        const int ihi = (s - 1) >> 1;
        for (int i = ilo + lane; i <= ihi; i += 32) {
          const int j = s - i;
          const int64_t rk = pair_rank(i, j, n);
          if (rk < pos) continue;
          uint64_t k53 = 0;
          float r_lo, r_hi;
          if (rnd) {
            injected_interval(rnd[rk], r_lo, r_hi);
          } else {
            k53 = philox_bits53(a.seed, (uint64_t)rk, pc1);
            philox_interval(k53, r_lo, r_hi);
          }
          const int sc = screen_pair(a, use_E, S.v[i], S.sk[i], S.v[j], S.sk[j], r_lo, r_hi);
          if (sc == 0) continue;
          if (sc == 1) {
            certain_collection(a, S, i, j, Tc, use_E);
            c0 += 1;
            continue;
          }
          const int o = exact_pair(a, S, S.sid[i], S.sid[j], i, j, Tc, use_E,
                                   rnd ? rnd[rk] : philox_from_bits(k53));
          c0 += o == 1;
          c1 += o == 2;
        }
        __threadfence_block();
        __syncwarp();
      }
    }
    __syncwarp();
  }
  // counters (integer sums commute)
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    c0 += __shfl_down_sync(0xffffffffu, c0, off);
    c1 += __shfl_down_sync(0xffffffffu, c1, off);
  }
  if (lane == 0 && (c0 | c1)) {
    atomicAdd((unsigned long long*)a.no_cols, (unsigned long long)c0);
    atomicAdd((unsigned long long*)(a.no_cols + 1), (unsigned long long)c1);
  }
}

__global__ void k_col_advance(const __grid_constant__ MRef mr, int draws) {
  const Ws& w = mr.get().w;
  if (draws && !(*w.flags & LACMO_FLAG_DRAWS_SHORT)) *w.cursor += *w.total_pairs;
  *w.col_step += 1;
  *w.cell_ctr = 0;
}

// ---------------------------------------------------------------------------
// Box models: one CTA runs the whole single-cell step, SIP state in shared
// memory, one __syncthreads per anti-diagonal.
constexpr int BOX_THREADS = 1024;

// collision/all_or_nothing.py:109-185 (Golovin kernel, kernel.py:461-480)
__global__ void __launch_bounds__(BOX_THREADS) k_golovin(double* xis, double* masses, int n,
                                                         double dtdv, int64_t* no_cols,
                                                         const double* rnd, uint64_t seed,
                                                         uint64_t step) {
  extern __shared__ double sm[];
  double* X = sm;
  double* M = sm + n;
  for (int q = threadIdx.x; q < n; q += blockDim.x) { X[q] = xis[q]; M[q] = masses[q]; }
  __syncthreads();
  int64_t c0 = 0, c1 = 0;
  for (int s = 1; s <= 2 * n - 3; ++s) {
    const int ilo = s - (n - 1) > 0 ? s - (n - 1) : 0;
    const int ihi = (s - 1) >> 1;
    for (int i = ilo + threadIdx.x; i <= ihi; i += blockDim.x) {
      const int j = s - i;
      int imin, imax;
      if (X[i] <= X[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
      const double xi_min = X[imin], xi_max = X[imax];
      const double m_min = M[imin], m_max = M[imax];
      const double p_crit = xi_max * ((m_min + m_max) * 1.5E-18) * dtdv;
      if (p_crit > 1.0) {
        c1 += 1;
        const double xi_col = p_crit * xi_min;
        M[imin] = (xi_min * m_min + xi_col * m_max) / xi_min;
        X[imax] -= xi_col;
      } else {
        const int64_t rk = pair_rank(i, j, n);
        const double r = rnd ? rnd[rk] : philox_uniform(seed, (uint64_t)rk, step);
        if (p_crit > r) {
          c0 += 1;
          const double xi_rel_dev = (xi_max - xi_min) / xi_max;
          if (xi_rel_dev < 1.0E-5) {
            const double xi_ges = xi_min + xi_max;
            M[imin] = 2.0 * (xi_min * m_min + xi_max * m_max) / xi_ges;
            M[imax] = M[imin];
            X[imax] = 0.5 * 0.7 * xi_ges;
            X[imin] = 0.5 * xi_ges - X[imax];
          } else {
            M[imin] += m_max;
            X[imax] -= xi_min;
          }
        }
      }
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < n; q += blockDim.x) { xis[q] = X[q]; masses[q] = M[q]; }
  for (int off = 16; off > 0; off >>= 1) {
    c0 += __shfl_down_sync(0xffffffffu, c0, off);
    c1 += __shfl_down_sync(0xffffffffu, c1, off);
  }
  if ((threadIdx.x & 31) == 0 && (c0 | c1)) {
    atomicAdd((unsigned long long*)no_cols, (unsigned long long)c0);
    atomicAdd((unsigned long long*)(no_cols + 1), (unsigned long long)c1);
  }
}

// collision/all_or_nothing.py:392-491 (kernel K(m1, m2) tabulated on a
// logarithmic mass grid): p_crit = xi_max K[k_i][k_j] dt/dV, the bins of
// the collected SIP recomputed from its new mass
__global__ void __launch_bounds__(BOX_THREADS) k_kgrid_box(double* xis, double* masses, int n,
                                                           double dtdv, const double* K,
                                                           int64_t nb, double lo, double bl,
                                                           int64_t* no_cols, const double* rnd,
                                                           uint64_t seed, uint64_t step) {
  extern __shared__ double sm[];
  double* X = sm;
  double* M = sm + n;
  int32_t* B = (int32_t*)(sm + 2 * n);
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    X[q] = xis[q]; M[q] = masses[q];
    B[q] = col_bin(M[q], lo, bl, nb);
  }
  __syncthreads();
  int64_t c0 = 0, c1 = 0;
  for (int s = 1; s <= 2 * n - 3; ++s) {
    const int ilo = s - (n - 1) > 0 ? s - (n - 1) : 0;
    const int ihi = (s - 1) >> 1;
    for (int i = ilo + threadIdx.x; i <= ihi; i += blockDim.x) {
      const int j = s - i;
      int imin, imax;
      if (X[i] <= X[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
      const double xi_min = X[imin], xi_max = X[imax];
      const double m_min = M[imin], m_max = M[imax];
      const double p_crit = xi_max * K[(int64_t)B[i] * nb + B[j]] * dtdv;
      if (p_crit > 1.0) {
        c1 += 1;
        const double xi_col = p_crit * xi_min;
        M[imin] = (xi_min * m_min + xi_col * m_max) / xi_min;
        X[imax] -= xi_col;
        B[imin] = col_bin(M[imin], lo, bl, nb);
      } else {
        const int64_t rk = pair_rank(i, j, n);
        const double r = rnd ? rnd[rk] : philox_uniform(seed, (uint64_t)rk, step);
        if (p_crit > r) {
          c0 += 1;
          const double xi_rel_dev = (xi_max - xi_min) / xi_max;
          if (xi_rel_dev < 1.0E-5) {
            const double xi_ges = xi_min + xi_max;
            M[imin] = 2.0 * (xi_min * m_min + xi_max * m_max) / xi_ges;
            M[imax] = M[imin];
            X[imax] = 0.5 * 0.7 * xi_ges;
            X[imin] = 0.5 * xi_ges - X[imax];
            B[imin] = col_bin(M[imin], lo, bl, nb);
            B[imax] = B[imin];
          } else {
            M[imin] += m_max;
            X[imax] -= xi_min;
            B[imin] = col_bin(M[imin], lo, bl, nb);
          }
        }
      }
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < n; q += blockDim.x) { xis[q] = X[q]; masses[q] = M[q]; }
  for (int off = 16; off > 0; off >>= 1) {
    c0 += __shfl_down_sync(0xffffffffu, c0, off);
    c1 += __shfl_down_sync(0xffffffffu, c1, off);
  }
  if ((threadIdx.x & 31) == 0 && (c0 | c1)) {
    atomicAdd((unsigned long long*)no_cols, (unsigned long long)c0);
    atomicAdd((unsigned long long*)(no_cols + 1), (unsigned long long)c1);
  }
}

// collision/all_or_nothing.py:269-390 (E_col(R1, R2) table, 1-D velocities)
__global__ void __launch_bounds__(BOX_THREADS) k_ecol_box(double* xis, double* masses,
                                                          double* radii, const double* vel,
                                                          const double* rho, int n, double dtdv,
                                                          const double* E, int64_t nb, double lo,
                                                          double bl, int64_t* no_cols,
                                                          const double* rnd, uint64_t seed,
                                                          uint64_t step) {
  extern __shared__ double sm[];
  double* X = sm;
  double* M = sm + n;
  double* R = sm + 2 * n;
  double* Vv = sm + 3 * n;
  double* Rh = sm + 4 * n;
  int32_t* K = (int32_t*)(sm + 5 * n);
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    X[q] = xis[q]; M[q] = masses[q]; R[q] = radii[q]; Vv[q] = vel[q]; Rh[q] = rho[q];
    K[q] = col_bin(R[q], lo, bl, nb);
  }
  __syncthreads();
  int64_t c0 = 0, c1 = 0;
  for (int s = 1; s <= 2 * n - 3; ++s) {
    const int ilo = s - (n - 1) > 0 ? s - (n - 1) : 0;
    const int ihi = (s - 1) >> 1;
    for (int i = ilo + threadIdx.x; i <= ihi; i += blockDim.x) {
      const int j = s - i;
      int imin, imax;
      if (X[i] <= X[j]) { imin = i; imax = j; } else { imin = j; imax = i; }
      const double xi_min = X[imin], xi_max = X[imax];
      const double m_min = M[imin], m_max = M[imax];
      const double Rs = R[i] + R[j];
      const double p_crit = xi_max * dtdv *
                            (LC_PI * Rs * Rs * __ldg(E + (int64_t)K[i] * nb + K[j]) *
                             fabs(Vv[i] - Vv[j]) * 1.0E-12);
      if (p_crit > 1.0) {
        const double xi_col = p_crit * xi_min;
        M[imin] = (xi_min * m_min + xi_col * m_max) / xi_min;
        R[imin] = col_radius(M[imin], Rh[imin]);
        X[imax] -= xi_col;
        K[imin] = col_bin(R[imin], lo, bl, nb);
        c1 += 1;
      } else {
        const int64_t rk = pair_rank(i, j, n);
        const double r = rnd ? rnd[rk] : philox_uniform(seed, (uint64_t)rk, step);
        if (p_crit > r) {
          c0 += 1;
          const double xi_rel_dev = (xi_max - xi_min) / xi_max;
          if (xi_rel_dev < 1.0E-5) {
            const double xi_ges = xi_min + xi_max;
            M[imin] = 2.0 * (xi_min * m_min + xi_max * m_max) / xi_ges;
            M[imax] = M[imin];
            R[imin] = col_radius(M[imin], Rh[imin]);
            R[imax] = R[imin];
            X[imax] = 0.5 * 0.7 * xi_ges;
            X[imin] = 0.5 * xi_ges - X[imax];
            K[imin] = col_bin(R[imin], lo, bl, nb);
            K[imax] = K[imin];
          } else {
            M[imin] += m_max;
            R[imin] = col_radius(M[imin], Rh[imin]);
            X[imax] -= xi_min;
            K[imin] = col_bin(R[imin], lo, bl, nb);
          }
        }
      }
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < n; q += blockDim.x) { xis[q] = X[q]; masses[q] = M[q]; radii[q] = R[q]; }
  for (int off = 16; off > 0; off >>= 1) {
    c0 += __shfl_down_sync(0xffffffffu, c0, off);
    c1 += __shfl_down_sync(0xffffffffu, c1, off);
  }
  if ((threadIdx.x & 31) == 0 && (c0 | c1)) {
    atomicAdd((unsigned long long*)no_cols, (unsigned long long)c0);
    atomicAdd((unsigned long long*)(no_cols + 1), (unsigned long long)c1);
  }
}

// collision/kernel.py:107-167 Beard (1976) terminal velocity (R in um)
__device__ double beard_velocity(double R) {
  const double rho_w = 1.0E3, rho_a = 1.225, visc = 1.818E-5, sigma = 73.0E-3;
  const double g = 9.80665, drho = rho_w - rho_a;
  if (R < 10.0) {
    const double l0 = 6.62E-2;
    const double C1 = drho * g / (4.5 * visc);
    const double C_sc = 1.0 + 1.257 * l0 / R;
    return C1 * C_sc * R * R * 1.0E-12;
  } else if (R < 535.0) {
    const double N_Da = 32.0E-18 * R * R * R * rho_a * drho * g / (3.0 * visc * visc);
    double Y = log(N_Da);
    const double p1[7] = {-0.327815e-5, 0.855176e-4, -0.578878e-3, -0.987059e-3,
                          -0.153193e-2, 0.992696, -0.318657e1};
    double r = p1[0] * Y + p1[1];
    for (int k = 2; k < 7; ++k) r = r * Y + p1[k];
    const double l0 = 6.62E-2;
    const double C_sc = 1.0 + 1.257 * l0 / R;
    return visc * C_sc * exp(r) / (rho_a * R * 2.0E-6);
  } else if (R < 3500.0) {
    const double N_Bo = 16.0E-12 * R * R * drho * g / (3.0 * sigma);
    const double v4 = (visc * visc) * (visc * visc);
    const double N_P16 = pow(sigma * sigma * sigma * rho_a * rho_a / (v4 * drho * g), 1.0 / 6.0);
    const double Y = log(N_Bo * N_P16);
    const double p2[6] = {0.238449e-2, -0.542819e-1, 0.475294, -0.204914e1, 0.523778e1,
                          -0.500015e1};
    double r = p2[0] * Y + p2[1];
    for (int k = 2; k < 6; ++k) r = r * Y + p2[k];
    return visc * N_P16 * exp(r) / (rho_a * R * 2.0E-6);
  }
  return 9.04929248;
}
__global__ void k_beard(double* vel, const double* R, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    vel[k] = beard_velocity(R[k]);
}
__global__ void k_radius_bin(const double* m, const double* rho, int64_t n, double lo, double bl,
                             int64_t nb, double* R, int64_t* k) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const double r = col_radius(m[q], rho[q]);
    R[q] = r;
    if (k) k[q] = col_bin(r, lo, bl, nb);
  }
}

// ---------------------------------------------------------------------------
static inline int nblk(int64_t n, int t) {
  int64_t b = (n + t - 1) / t;
  if (b < 1) b = 1;
  return (int)(b < 152 * 32 ? b : 152 * 32);
}
static const size_t CELL_SMEM_BYTES = (size_t)CELL_WARPS * CELL_WARP_BYTES;

__global__ void k_table_to_float(const double* __restrict__ E, float* __restrict__ Ef, int64_t m) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m;
       k += (int64_t)gridDim.x * blockDim.x)
    Ef[k] = (float)E[k];
}
// largest FP32 efficiency of each row, one warp per row: the maximum of the
// row's positive values by a warp reduction; a row with a NaN, or whose
// largest value is not positive (where the sign of a zero or the place of a
// NaN decides), is taken in column order by one lane, as the oracle does
__global__ void k_table_rowmax(const double* __restrict__ E, float* __restrict__ erow, int64_t nb) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t k = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); k < nb;
       k += warps) {
    const double* row = E + k * nb;
    uint32_t mk = 0;
    bool odd = false;
    for (int64_t q = lane; q < nb; q += 32) {
      const float v = (float)__ldg(row + q);
      odd |= v != v;
      if (v > 0.0f) mk = max(mk, __float_as_uint(v));   // positive floats order as integers
    }
    mk = __reduce_max_sync(0xffffffffu, mk);
    odd = __any_sync(0xffffffffu, odd) || mk == 0;
    if (lane == 0) {
      if (odd) {
        float mx = (float)row[0];
        for (int64_t q = 1; q < nb; ++q) mx = lt_max(mx, (float)row[q]);
        erow[k] = mx;
      } else {
        erow[k] = __uint_as_float(mk);
      }
    }
  }
}

// Bound on the error of the FP32 bin position v = (__logf(Rf) - lo_f) *
// inv_bl_f + 0.5 against the exact (log R - lo) / bl + 0.5, doubled: Rf is
// within 1e-6 of R (relative), so log Rf within 1e-6; __logf within 2^-21.41
// absolute on [0.5, 2] and 3 ulp elsewhere (taken as 4 ulp of the largest
// |log R| a bin edge can have); lo_f and the subtraction round within one ulp
// of that value together; inv_bl_f, the product and the + 0.5 each within
// 2^-24 of v <= nb + 1.  Bins closer than this to an edge are taken from the
// exact FP64 path.
static float fp32_bin_margin(double lo, double bl, int64_t nb) {
  if (!(bl > 0.0) || nb <= 0) return 0.5f;
  const double lmax = fmax(fabs(lo), fabs(lo + (double)(nb + 1) * bl)) + 1.0;
  const double ulp = ldexp(1.0, (int)floor(log2(lmax)) - 23);
  const double log_err = fmax(ldexp(1.0, -21) , 4.0 * ulp);
  const double v_err = (1e-6 + log_err + ulp) / bl + 3.0 * (double)(nb + 1) * ldexp(1.0, -24);
  const double m = 2.0 * v_err;
  return (float)(m < 0.5 ? m : 0.5);
}

// persistent blocks: as many as are resident at once, split over members
template <bool THIN, int MINB>
static cudaError_t launch_cells(const Bt& B, const CK& x, cudaStream_t s) {
  static std::atomic<int> resident[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int res = dev < 64 ? resident[dev].load() : 0;
  if (res <= 0) {
    e = cudaFuncSetAttribute(k_collide_cells<THIN, MINB>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CELL_SMEM_BYTES);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_collide_cells<THIN, MINB>,
                                                      CELL_WARPS * 32, CELL_SMEM_BYTES);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    res = per_sm * sms > 0 ? per_sm * sms : 1;
    if (dev < 64) resident[dev].store(res);
  }
  const int64_t C = B.nx * B.nz;
  int64_t bx = res / B.M;
  const int64_t need = (C + CELL_WARPS - 1) / CELL_WARPS;
  if (bx > need) bx = need;
  if (bx < 1) bx = 1;
  k_collide_cells<THIN, MINB><<<dim3((unsigned)bx, (unsigned)B.M), CELL_WARPS * 32,
                                CELL_SMEM_BYTES, s>>>(x);
  note_launches(1);
  return cudaGetLastError();
}

// the event log of single-state collision steps (lacmo_collision_event_log)
static std::atomic<EvRec*> g_log{nullptr};
static std::atomic<int64_t> g_log_cap{0};
static std::atomic<unsigned long long*> g_log_count{nullptr};

cudaError_t launch_collide_cells(const Bt& B, const lacmo_params_t& p, const lacmo_draws_t& d,
                                 cudaStream_t s) {
  if (B.M > 1 && d.draws) return cudaErrorInvalidValue;   // batches draw from Philox
  CellCommon cc;
  cc.log = B.M == 1 ? g_log.load() : nullptr;
  cc.log_cap = g_log_cap.load();
  cc.log_count = g_log_count.load();
  if (!cc.log_count) cc.log = nullptr;
  cc.dtdv = p.dt_col_over_dV; cc.E = p.E_col_grid; cc.E_const = p.E_col_const;
  cc.nb = p.no_kernel_bins; cc.lo = p.R_kernel_low_log; cc.bl = p.bin_factor_R_log;
  cc.sol = p.solute; cc.draws = d.draws; cc.n_draws = d.n_draws;
  cc.dtdv_f = (float)cc.dtdv; cc.lo_f = (float)cc.lo; cc.inv_bl_f = (float)(1.0 / cc.bl);
  cc.bin_margin = fp32_bin_margin(cc.lo, cc.bl, cc.nb);
  cc.E_const_f = (float)cc.E_const;
  cc.Ef = nullptr;
  cc.erow = nullptr;
  float* Ef = B.one.w.Ef;   // member 0's slot serves the whole batch
  if (p.E_col_grid && Ef && p.no_kernel_bins <= LACMO_MAX_KERNEL_BINS) {
    const int64_t m = p.no_kernel_bins * p.no_kernel_bins;
    k_table_to_float<<<nblk(m, 256), 256, 0, s>>>(p.E_col_grid, Ef, m); note_launches(1);
    cc.Ef = Ef;
    if (p.thin_draws) {
      float* erow = Ef + (int64_t)LACMO_MAX_KERNEL_BINS * LACMO_MAX_KERNEL_BINS;
      k_table_rowmax<<<nblk(p.no_kernel_bins * 32, 128), 128, 0, s>>>(p.E_col_grid, erow,
                                                                      p.no_kernel_bins);
      note_launches(1);
      cc.erow = erow;
    }
  }
  // thinned draws need the row maxima of a tabulated efficiency
  cc.thin = (p.thin_draws != 0 && d.draws == nullptr && (!p.E_col_grid || cc.erow)) ? 1 : 0;
  CK x{B.ref(), cc};
  cudaError_t e;
  const int minb = tune_value(TUNE_COLLISION_BLOCKS);
  if (cc.thin) {
    e = minb == 2 ? launch_cells<true, 2>(B, x, s)
                  : (minb == 4 ? launch_cells<true, 4>(B, x, s) : launch_cells<true, 3>(B, x, s));
  } else {
    e = minb == 2 ? launch_cells<false, 2>(B, x, s)
                  : (minb == 4 ? launch_cells<false, 4>(B, x, s)
                               : launch_cells<false, 3>(B, x, s));
  }
  if (e != cudaSuccess) return e;
  k_col_advance<<<dim3(1, B.M), 1, 0, s>>>(B.ref(), d.draws ? 1 : 0); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_golovin(double* xis, double* m, int64_t n, double dtdv, int64_t* no_cols,
                           const double* rnd, uint64_t seed, uint64_t step, cudaStream_t s) {
  size_t sh = (size_t)n * 16;
  cudaError_t e = cudaFuncSetAttribute(k_golovin, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(LACMO_BOX_MAX_SIPS * 16));
  if (e != cudaSuccess) return e;
  k_golovin<<<1, BOX_THREADS, sh, s>>>(xis, m, (int)n, dtdv, no_cols, rnd, seed, step); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_ecol_box(double* xis, double* m, double* R, const double* vel,
                            const double* rho, int64_t n, double dtdv, const double* E, int64_t nb,
                            double lo, double bl, int64_t* no_cols, const double* rnd,
                            uint64_t seed, uint64_t step, cudaStream_t s) {
  size_t sh = (size_t)n * 44;
  cudaError_t e = cudaFuncSetAttribute(k_ecol_box, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(LACMO_ECOL_BOX_MAX_SIPS * 44));
  if (e != cudaSuccess) return e;
  k_ecol_box<<<1, BOX_THREADS, sh, s>>>(xis, m, R, vel, rho, (int)n, dtdv, E, nb, lo, bl, no_cols,
                                        rnd, seed, step); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_kgrid_box(double* xis, double* m, int64_t n, double dtdv, const double* K,
                             int64_t nb, double lo, double bl, int64_t* no_cols, const double* rnd,
                             uint64_t seed, uint64_t step, cudaStream_t s) {
  size_t sh = (size_t)n * 20;
  cudaError_t e = cudaFuncSetAttribute(k_kgrid_box, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(LACMO_BOX_MAX_SIPS * 20));
  if (e != cudaSuccess) return e;
  k_kgrid_box<<<1, BOX_THREADS, sh, s>>>(xis, m, (int)n, dtdv, K, nb, lo, bl, no_cols, rnd, seed,
                                         step); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_beard(double* vel, const double* R, int64_t n, cudaStream_t s) {
  k_beard<<<nblk(n, 128), 128, 0, s>>>(vel, R, n); note_launches(1);
  return cudaGetLastError();
}
cudaError_t launch_radius_bin(const double* m, const double* rho, int64_t n, double lo, double bl,
                              int64_t nb, double* R, int64_t* k, cudaStream_t s) {
  k_radius_bin<<<nblk(n, 128), 128, 0, s>>>(m, rho, n, lo, bl, nb, R, k); note_launches(1);
  return cudaGetLastError();
}

}  // namespace lacmo

extern "C" int lacmo_collision_event_log(void* events, int64_t capacity,
                                         unsigned long long* count) {
  if (events && (capacity < 0 || !count)) return LACMO_ERR_ARG;
  lacmo::g_log_count.store(events ? count : nullptr);
  lacmo::g_log_cap.store(events ? capacity : 0);
  lacmo::g_log.store((lacmo::EvRec*)events);
  return LACMO_OK;
}
