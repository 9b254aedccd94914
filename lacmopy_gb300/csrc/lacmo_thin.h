/* Thinned Philox draws of the all-or-nothing collision step, shared by the
 * CUDA kernel (k_collision.cu) and the oracle (plain C), which must take every
 * decision identically.
 *
 * The reference draws one uniform r_k per pair k of a cell (lexicographic
 * order) and collects when p_crit(k) > r_k.  The thinned draws define the same
 * iid uniforms partly implicitly.  The SIP slots of a cell form blocks of
 * LACMO_THIN_L; the pairs (i, j) of row i with j in block b form a segment,
 * and the segments are taken in lexicographic order.  The still unprocessed
 * part of a segment (pairs (i, j .. jend-1), part counter `sub`) is handled
 * with a certified bound Q >= p_crit of all its pairs, computed from the FP32
 * copies of SIP i and the statistics of block b (lt_segment_bound):
 *  - if Q >= LACMO_THIN_TAU or there is no valid bound, every remaining pair
 *    of the segment takes its own per-pair Philox draw, in order;
 *  - otherwise, with q = 2^-e >= Q and m remaining pairs, one uniform decides
 *    whether a draw falls below q (probability 1 - (1 - q)^m); if none does,
 *    no pair collects and the segment is done; else the first such pair h is
 *    drawn from its exact conditional distribution, its draw is r = q u
 *    (uniform below q), the pair is evaluated with r, and the pairs after h
 *    form a new part (sub + 1) bounded from the state after it.  Pairs before
 *    h have r_k >= q > p_crit and are skipped.
 * The probabilities come from exact rational tables (lacmo_thin_tables.h,
 * compared as 53-bit integers); the bound uses only IEEE single-precision +,
 * -, * and comparisons (no contraction), so device and host agree bit for bit.
 */
#ifndef LACMO_THIN_H_
#define LACMO_THIN_H_

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__) && !defined(LACMO_THIN_QUAL)
#define LACMO_THIN_QUAL static __device__ const   /* device global memory, read through L1 */
#endif
#include "lacmo_thin_tables.h"

/* segments bounded at or above this take per-pair draws */
#define LACMO_THIN_TAU 0x1p-6f

#ifdef __CUDACC__
#define LT_FN __host__ __device__ __forceinline__
#else
#define LT_FN static inline
#endif

LT_FN uint32_t lt_f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
LT_FN float lt_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
LT_FN float lt_max(float a, float b) { return a > b ? a : b; }
LT_FN float lt_min(float a, float b) { return a < b ? a : b; }
LT_FN float lt_abs(float a) { return a < 0.0f ? -a : a; }

/* cube root of x > 0 from IEEE operations only: a bit-pattern first guess
 * (within 4% relative) and three Newton steps y <- (2y + x/y^2)/3, which
 * leave it within a few ulp */
LT_FN float lt_cbrtf(float x) {
  float y = lt_u2f(lt_f2u(x) / 3u + 0x2a5137a0u);
  y = (y + y + x / (y * y)) / 3.0f;
  y = (y + y + x / (y * y)) / 3.0f;
  y = (y + y + x / (y * y)) / 3.0f;
  return y;
}

/* statistics of one block of SIP slots from the FP32 copies (x = multiplicity,
 * R = radius, u, w = velocity): maxima of x and R, ranges of u and w, and
 * ok = every SIP has x > 0 and R, u, w not NaN (otherwise the values are
 * not used) */
typedef struct {
  float xmax, Rmax, umin, umax, wmin, wmax;
  int ok;
} lt_block_t;

LT_FN void lt_block_stats(const float* x, const float* R, const float* u, const float* w, int64_t lo,
                          int64_t hi, lt_block_t* s) {
  s->xmax = 0.0f; s->Rmax = 0.0f;
  s->umin = s->wmin = lt_u2f(0x7f800000u); s->umax = s->wmax = lt_u2f(0xff800000u);
  s->ok = 1;
  for (int64_t q = lo; q < hi; ++q) {
    if (!(x[q] > 0.0f) || !(R[q] == R[q] && u[q] == u[q] && w[q] == w[q])) s->ok = 0;
    s->xmax = lt_max(s->xmax, x[q]); s->Rmax = lt_max(s->Rmax, R[q]);
    s->umin = lt_min(s->umin, u[q]); s->umax = lt_max(s->umax, u[q]);
    s->wmin = lt_min(s->wmin, w[q]); s->wmax = lt_max(s->wmax, w[q]);
  }
}

/* certified upper bound of p_crit over the pairs (a, j), j in a block with
 * statistics s, from the FP32 copies of SIP a, the largest FP32 efficiency
 * er of row bin(a) and dt/dV: every factor is at least the pair's own (the
 * operations are monotone), and the bound carries the slack of the FP32
 * radii (1e-6 relative), velocities (2^-21 sum |u|, |w|) and roundings
 * (2^-14 relative, 1e-36 absolute).  Returns a negative value when the
 * segment must take per-pair draws (non-positive multiplicity, NaN). */
LT_FN float lt_segment_bound(float xa, float Ra, float ua, float wa, const lt_block_t* s, float er,
                             float dtdv_f) {
  if (!s->ok || !(xa > 0.0f) || !(Ra == Ra && ua == ua && wa == wa)) return -1.0f;
  const float du = lt_max(ua - s->umin, s->umax - ua);
  const float dw = lt_max(wa - s->wmin, s->wmax - wa);
  const float um = lt_max(lt_abs(s->umin), lt_abs(s->umax));
  const float wm = lt_max(lt_abs(s->wmin), lt_abs(s->wmax));
  const float slack = 0x1p-21f * (((lt_abs(ua) + um) + lt_abs(wa)) + wm);
  const float rs = Ra + s->Rmax;
  const float core = ((((lt_max(xa, s->xmax) * dtdv_f) * 3.14159265e-12f) * rs) * rs) * er;
  if (!(core >= 1e-30f)) return core == core ? 1e-27f : -1.0f;
  const float pb = ((core * ((du + dw) + slack)) * (1.0f + 0x1p-14f)) + 1e-36f;
  return pb == pb ? pb : -1.0f;
}

/* q = 2^-e, the smallest power of two >= qmax (1e-36 <= qmax < LACMO_THIN_TAU) */
LT_FN int lt_exponent(float qmax) {
  const uint32_t b = lt_f2u(qmax);
  const int E = (int)((b >> 23) & 0xffu) - 127;
  int e = (b & 0x7fffffu) ? -E - 1 : -E;
  if (e < LACMO_THIN_E_MIN) e = LACMO_THIN_E_MIN;
  if (e > LACMO_THIN_E_MAX) e = LACMO_THIN_E_MAX;
  return e;
}

/* Philox4x32-10 block, words (x0, x1) as a 53-bit integer u53: the j-th
 * uniform u = u53 2^-53 of part `sub` of chunk `chunk` under counter word c1
 * (collision step << 32 | cell) */
LT_FN uint64_t lt_bits53(uint64_t key, uint64_t chunk, uint32_t sub, uint32_t j, uint64_t c1) {
  const uint64_t c0 = (1ull << 62) | (chunk << 20) | ((uint64_t)sub << 8) | (uint64_t)j;
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  uint32_t x0 = (uint32_t)c0, x1 = (uint32_t)(c0 >> 32), x2 = (uint32_t)c1, x3 = (uint32_t)(c1 >> 32);
#ifdef __CUDA_ARCH__
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
    x0 = hi1 ^ x1 ^ k0; x1 = lo1; x2 = hi0 ^ x3 ^ k1; x3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
#else
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
    const uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0, y1 = (uint32_t)p1;
    const uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1, y3 = (uint32_t)p0;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
#endif
  return (uint64_t)(x0 >> 5) * 67108864ull + (uint64_t)(x1 >> 6);
}

#endif
