/* kdgr_math.h -- the exponential of the oracle-matching kernels (C; on the
 * host compiled with -ffp-contract=off).
 *
 * The reference kernel uses CUDA's expf inside particleResponse
 * (cudaRenderer.cu:663-680).  A CPU restatement cannot reproduce a
 * vendor-library result bit for bit, so the oracle-matching kernels use this
 * project exponential instead, and the CPU oracle restates the same method
 * in its own code (the two agree bit for bit):
 *
 *   exp(x) = 2^k * e^r,  k = floor(x*log2(e) + 1/2),
 *   r = (x - k*C1) - k*C2  with C1 = 355/512 and C2 = ln2 - C1
 *   (W. J. Cody and W. Waite, "Software Manual for the Elementary
 *   Functions", 1980: C1 has 9 significant bits, so k*C1 is exact),
 *   e^r from its Taylor series to degree 7 by Horner's rule.
 *
 * On |r| <= ln2/2 the series truncation is below r^8/8! < 6e-9 relative
 * (0.1 ulp); the maximum error against a double-precision exp over the
 * response domain, and the agreement with the oracle's copy, are checked by
 * tests/test_oracle.py.  Domain: x <= 88
 * (the renderer only evaluates x <= 0); x < -87.3 returns 0.
 *
 * KDGR_MUL/KDGR_ADD are IEEE round-to-nearest operations that the CUDA
 * compiler never fuses into an FMA (__fmul_rn/__fadd_rn); on the host they
 * are plain operators under -ffp-contract=off.
 */
#ifndef KDGR_MATH_H_
#define KDGR_MATH_H_

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define KDGR_HD __host__ __device__ __forceinline__
#else
#define KDGR_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define KDGR_MUL(a, b) __fmul_rn((a), (b))
#define KDGR_ADD(a, b) __fadd_rn((a), (b))
#define KDGR_SUB(a, b) __fsub_rn((a), (b))
#define KDGR_DIV(a, b) __fdiv_rn((a), (b))
#define KDGR_SQRT(a) __fsqrt_rn((a))
#else
#define KDGR_MUL(a, b) ((a) * (b))
#define KDGR_ADD(a, b) ((a) + (b))
#define KDGR_SUB(a, b) ((a) - (b))
#define KDGR_DIV(a, b) ((a) / (b))
#define KDGR_SQRT(a) sqrtf((a))
#endif

KDGR_HD float kdgr_bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

KDGR_HD float kdgr_expf(float x) {
  if (!(x >= -87.3f)) return (x != x) ? x : 0.0f;
  if (x > 88.0f) return kdgr_bits_to_float(0x7f800000u);
  const float kf = floorf(KDGR_ADD(KDGR_MUL(x, 1.44269504088896341f), 0.5f));
  float r = KDGR_SUB(x, KDGR_MUL(kf, 0.693359375f));
  r = KDGR_ADD(r, KDGR_MUL(kf, 2.12194440e-4f));
  float p = 1.98412698e-4f; /* 1/5040 */
  p = KDGR_ADD(KDGR_MUL(p, r), 1.38888889e-3f); /* 1/720 */
  p = KDGR_ADD(KDGR_MUL(p, r), 8.33333333e-3f); /* 1/120 */
  p = KDGR_ADD(KDGR_MUL(p, r), 4.16666667e-2f); /* 1/24 */
  p = KDGR_ADD(KDGR_MUL(p, r), 1.66666667e-1f); /* 1/6 */
  p = KDGR_ADD(KDGR_MUL(p, r), 0.5f);
  p = KDGR_ADD(KDGR_MUL(p, r), 1.0f);
  p = KDGR_ADD(KDGR_MUL(p, r), 1.0f);
  const int k = (int)kf;
  return KDGR_MUL(p, kdgr_bits_to_float((uint32_t)(k + 127) << 23));
}

#endif /* KDGR_MATH_H_ */
