/* Thinned Philox draws of the all-or-nothing collision step, shared by the
 * CUDA kernel (k_collision.cu) and the oracle (plain C), which must take every
 * decision identically.
 *
 * The reference draws one uniform r_k per pair k of a cell (lexicographic
 * order) and collects when p_crit(k) > r_k.  The thinned draws define the same
 * iid uniforms partly implicitly.  The pairs are grouped in chunks of
 * LACMO_THIN_L consecutive ranks; the still unprocessed part of a chunk
 * (ranks pos .. end-1, part counter `sub`) is handled as follows, with a
 * certified bound b_k >= p_crit(k) of each pair from the FP32 copies of the
 * current state (lt_pair_bound):
 *  - an "individual" pair (b_k >= LACMO_THIN_TAU, or no valid bound) keeps
 *    its own per-pair Philox draw;
 *  - the other ("background") pairs share q = 2^-e >= every background b_k
 *    and each "hits" when its draw falls below q: one uniform decides whether
 *    the m background pairs hold a hit (probability 1 - (1 - q)^m); if they
 *    do, the first hit h is drawn from its exact conditional distribution and
 *    its draw is r = q u (uniform below q).  A background pair before h has
 *    r_k >= q >= p_crit and is skipped.
 * The part is then walked in rank order: at the hit h the pair is evaluated
 * with r, and at an individual pair with its own draw; the walk stops after
 * h, or after an individual pair that collides, and the rest of the chunk
 * starts again as a new part (sub + 1) from the state after it; otherwise
 * the part ends with its chunk.
 * The probabilities come from exact rational tables (lacmo_thin_tables.h); the
 * bound uses only IEEE single-precision +, -, *, /, fabs and fmax (no
 * contraction), so device and host agree bit for bit.
 */
#ifndef LACMO_THIN_H_
#define LACMO_THIN_H_

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__) && !defined(LACMO_THIN_QUAL)
#define LACMO_THIN_QUAL static __device__ const   /* device global memory, read through L1 */
#endif
#include "lacmo_thin_tables.h"

/* pairs bounded at or above this keep their own draw */
#define LACMO_THIN_TAU 0x1p-12f

#ifdef __CUDACC__
#define LT_FN __host__ __device__ __forceinline__
#else
#define LT_FN static inline
#endif

LT_FN uint32_t lt_f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
LT_FN float lt_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

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

/* certified upper bound of p_crit of a pair from the FP32 copies (xi, R, u,
 * w) of its SIPs and the FP32 efficiency ef; returns a negative value when the
 * pair must use its own draw (a non-positive multiplicity, NaN) */
LT_FN float lt_pair_bound(float xa, float Ra, float ua, float wa, float xb, float Rb, float ub,
                          float wb, float ef, float dtdv_f) {
  if (!(xa > 0.0f && xb > 0.0f)) return -1.0f;
  const float du = ua - ub;
  const float dw = wa - wb;
  const float slack = 0x1p-21f * (((fabsf(ua) + fabsf(ub)) + fabsf(wa)) + fabsf(wb));
  const float rs = Ra + Rb;
  const float core = ((((xa > xb ? xa : xb) * dtdv_f) * 3.14159265e-12f) * rs) * rs * ef;
  if (!(core >= 1e-30f)) return core == core ? 1e-27f : -1.0f;
  const float pb = ((core * ((fabsf(du) + fabsf(dw)) + slack)) * (1.0f + 0x1p-14f)) + 1e-36f;
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

/* Philox4x32-10 block, words (x0, x1) as 53 bits: the j-th uniform of part
 * `sub` of chunk `chunk` under counter word c1 (collision step << 32 | cell) */
LT_FN double lt_uniform(uint64_t key, uint64_t chunk, uint32_t sub, uint32_t j, uint64_t c1) {
  const uint64_t c0 = (1ull << 62) | (chunk << 20) | ((uint64_t)sub << 8) | (uint64_t)j;
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  uint32_t x0 = (uint32_t)c0, x1 = (uint32_t)(c0 >> 32), x2 = (uint32_t)c1, x3 = (uint32_t)(c1 >> 32);
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
    const uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0, y1 = (uint32_t)p1;
    const uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1, y3 = (uint32_t)p0;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return (double)((uint64_t)(x0 >> 5) * 67108864ull + (uint64_t)(x1 >> 6)) *
         (1.0 / 9007199254740992.0);
}

#endif
