/*
 * dml_rng.h - counter-based random streams shared bit-for-bit by the CUDA
 * kernels and the host code that checks them.
 *
 * The reference draws every random number from one sequential stream:
 * Numerical Recipes `ran()` (xorshift + Park-Miller) and a polar Box-Muller
 * `gasdev()` that caches its second deviate (src/dana.F90:1379-1428).  A
 * sequential stream cannot be reproduced by parallel threads, so the GPU path
 * replaces each call site with a draw from a counter-based Philox4x32-10
 * generator keyed by (seed, step, atom id, stream, sub).  The same draw is
 * obtained from the host build of this header, so a serial restatement of the
 * reference fed by these draws is an exact oracle for the device code.
 *
 * Philox4x32-10 follows Salmon, Moraes, Dror and Shaw, "Parallel random
 * numbers: as easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64 bit
 * multiplications with the published multipliers and Weyl key increments.
 *
 * Normals come from the Box-Muller transform evaluated in single precision
 * (the reference's own gasdev also rounds its radius through a real(4)
 * intermediate, dana.F90:1380-1381), returned as doubles.  `log`, `sin` and
 * `cos` are NOT taken from libm or CUDA (their results differ between host
 * and device); they are written here from textbook series:
 *   log(m) = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...),  s = (m-1)/(m+1),
 *            with m in [sqrt(1/2), sqrt(2)) after removing the binary exponent;
 *   sin, cos: Taylor series on [0, pi/4] after an exact quadrant reduction of
 *            the angle 2*pi*u (u is a multiple of 2^-24, so 4u is exact).
 * Every operation is an IEEE single add, subtract, multiply, divide or sqrt
 * in a fixed order with no fused multiply-add, so host and device agree to
 * the last bit.  Accuracy: |error| < 2e-7 relative for log, < 2e-7 absolute
 * for sin/cos (checked against libm in the CPU test suite).  The radius uses
 * a 32-bit uniform in (0,1], so the normal tail reaches 6.6 sigma.
 * Uniforms are doubles with 53 random bits.
 */
#ifndef DML_RNG_H
#define DML_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define DML_HD __host__ __device__ __forceinline__
#else
#define DML_HD static inline
#endif

/* Explicit rounding: on the device these are the round-to-nearest intrinsics
 * (never contracted into FMA); on the host the translation unit is compiled
 * with -ffp-contract=off. */
#if defined(__CUDA_ARCH__)
#define DMLF_MUL(a, b) __fmul_rn((a), (b))
#define DMLF_ADD(a, b) __fadd_rn((a), (b))
#define DMLF_SUB(a, b) __fsub_rn((a), (b))
#define DMLF_DIV(a, b) __fdiv_rn((a), (b))
#define DMLF_SQRT(a) __fsqrt_rn(a)
#define DML_MUL(a, b) __dmul_rn((a), (b))
#define DML_ADD(a, b) __dadd_rn((a), (b))
#define DML_SUB(a, b) __dsub_rn((a), (b))
#define DML_DIV(a, b) __ddiv_rn((a), (b))
#define DML_SQRT(a) __dsqrt_rn(a)
#else
#include <math.h>
#include <string.h>
#define DMLF_MUL(a, b) ((float)(a) * (float)(b))
#define DMLF_ADD(a, b) ((float)(a) + (float)(b))
#define DMLF_SUB(a, b) ((float)(a) - (float)(b))
#define DMLF_DIV(a, b) ((float)(a) / (float)(b))
#define DMLF_SQRT(a) sqrtf(a)
#define DML_MUL(a, b) ((a) * (b))
#define DML_ADD(a, b) ((a) + (b))
#define DML_SUB(a, b) ((a) - (b))
#define DML_DIV(a, b) ((a) / (b))
#define DML_SQRT(a) sqrt(a)
#endif

/* Stream identifiers: one per reference call site that draws random numbers. */
enum {
  DML_RNG_ERMAK = 1,    /* ermak_a: 2 normals per dimension (dana.F90:1006-1015) */
  DML_RNG_BROWN = 2,    /* cbrownian_hs: 1 normal per dimension (dana.F90:825-833) */
  DML_RNG_CAPTURE = 3,  /* atom_pbc capture draw at z<=0 (dana.F90:1233-1242) */
  DML_RNG_OVERLAP = 4,  /* overlap_moveback contact capture draw (dana.F90:896-898) */
  DML_RNG_GCMC = 5,     /* gcmc_run trial uniforms (dana.F90:627-686) */
  DML_RNG_GCMC_VEL = 6, /* gcmc_run Maxwell velocity normals (dana.F90:666-668) */
  DML_RNG_INIT = 7      /* initial-configuration generators (not on the step path) */
};

typedef struct {
  uint32_t w[4];
} dml_u4;

DML_HD uint32_t dml_mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

/* Philox4x32 with 10 rounds (Salmon et al. 2011, Sec. 4). */
DML_HD dml_u4 dml_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = dml_mulhi32(M0, c0), lo0 = M0 * c0;
    uint32_t hi1 = dml_mulhi32(M1, c2), lo1 = M1 * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  dml_u4 out;
  out.w[0] = c0;
  out.w[1] = c1;
  out.w[2] = c2;
  out.w[3] = c3;
  return out;
}

/* One keyed draw.  Counter = (id low, stream<<24 | sub, step low, step high ^ id high),
 * key = seed.  `sub` < 2^24 indexes several draws of one stream for one id/step. */
DML_HD dml_u4 dml_draw(uint64_t seed, int64_t step, uint64_t id, uint32_t stream, uint32_t sub) {
  uint64_t st = (uint64_t)step;
  return dml_philox4x32_10((uint32_t)id, (stream << 24) | (sub & 0xFFFFFFu), (uint32_t)st,
                           (uint32_t)(st >> 32) ^ (uint32_t)(id >> 32), (uint32_t)seed,
                           (uint32_t)(seed >> 32));
}

/* Uniform on [0,1) with 53 random bits: exact integer arithmetic in double. */
DML_HD double dml_u53(uint32_t a, uint32_t b) {
  double hi = (double)(a >> 5);           /* 27 bits */
  double lo = (double)(b >> 6);           /* 26 bits */
  double k = DML_ADD(DML_MUL(hi, 67108864.0), lo); /* < 2^53, exact */
  return DML_MUL(k, 0x1.0p-53);
}

DML_HD uint64_t dml_f64_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

DML_HD double dml_bits_f64(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

DML_HD uint32_t dml_f32_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

DML_HD float dml_bits_f32(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

/* Integer-to-float conversions written with integer operations on the
 * device, where GB300 issues conversion instructions on its narrow FP64
 * pipe (about 1/64 of the FP32 rate); the results are the conversions'
 * own (round to nearest, ties to even), so host and device still agree.
 * dml_small_i2f: exact for |e| < 2^22 (1.5 * 2^23 + e is a float whose low
 * mantissa bits are e; subtracting 1.5 * 2^23 is exact).
 * dml_u32_to_f32_rn: RN32 of a 32-bit unsigned integer. */
DML_HD float dml_small_i2f(int e) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(__int_as_float(0x4B400000 + e), 12582912.0f);
#else
  return (float)e;
#endif
}

DML_HD float dml_u32_to_f32_rn(uint32_t x) {
#if defined(__CUDA_ARCH__)
  if (x == 0u) return 0.0f;
  int n = 31 - __clz((int)x); /* position of the leading one */
  uint32_t m;
  if (n <= 23) {
    m = x << (23 - n); /* exact */
  } else {
    const int sh = n - 23; /* 1 .. 8 dropped bits */
    m = x >> sh;
    const uint32_t rem = x & ((1u << sh) - 1u), half = 1u << (sh - 1);
    if (rem > half || (rem == half && (m & 1u))) m += 1u;
    if (m == (1u << 24)) { /* carry into the next binade */
      m >>= 1;
      n += 1;
    }
  }
  return __uint_as_float(((uint32_t)(127 + n) << 23) | (m & 0x7FFFFFu));
#else
  return (float)x;
#endif
}

/* binary32 -> binary64, exact; on the device by rebiasing a normal float's
 * exponent (1023 - 127 = 896) with its 23 mantissa bits at the top of the
 * double's 52 (zero, subnormal, inf and NaN take the conversion). */
DML_HD double dml_f32_to_f64(float f) {
#if defined(__CUDA_ARCH__)
  const uint32_t b = __float_as_uint(f), e = (b >> 23) & 0xFFu;
  if (e == 0u || e == 0xFFu) return (double)f;
  const uint32_t hi = (b & 0x80000000u) | (((b & 0x7FFFFFFFu) >> 3) + (896u << 20));
  return __hiloint2double((int)hi, (int)(b << 29));
#else
  return (double)f;
#endif
}

/* Natural logarithm for normal positive x (the Box-Muller argument lies in
 * [2^-32, 1]).  Exponent split + atanh series, see the header comment. */
DML_HD float dml_logf(float x) {
  uint32_t bits = dml_f32_bits(x);
  int e = (int)((bits >> 23) & 0xFFu) - 127;
  float m = dml_bits_f32((bits & 0x007FFFFFu) | 0x3F800000u);
  if (m > 0x1.6a09e6p+0f) { /* sqrt(2) */
    m = DMLF_MUL(m, 0.5f);
    e += 1;
  }
  float f = DMLF_SUB(m, 1.0f); /* exact (Sterbenz) */
  float s = DMLF_DIV(f, DMLF_ADD(2.0f, f));
  float s2 = DMLF_MUL(s, s);
  /* r = s2/3 + s2^2/5 + ... + s2^5/11, Horner from the highest term. */
  float q = 0x1.745d18p-4f;                        /* 1/11 */
  q = DMLF_ADD(DMLF_MUL(q, s2), 0x1.c71c72p-4f);   /* 1/9 */
  q = DMLF_ADD(DMLF_MUL(q, s2), 0x1.24924ap-3f);   /* 1/7 */
  q = DMLF_ADD(DMLF_MUL(q, s2), 0x1.99999ap-3f);   /* 1/5 */
  q = DMLF_ADD(DMLF_MUL(q, s2), 0x1.555556p-2f);   /* 1/3 */
  float r = DMLF_MUL(s2, q);
  float two_s = DMLF_MUL(2.0f, s);
  float lm = DMLF_ADD(two_s, DMLF_MUL(two_s, r));
  return DMLF_ADD(DMLF_MUL(dml_small_i2f(e), 0x1.62e430p-1f), lm); /* + e ln2 */
}

/* sin and cos of theta in [0, pi/4] by Taylor series (to theta^9 / theta^10). */
DML_HD void dml_sincosf_small(float th, float* s, float* c) {
  float t2 = DMLF_MUL(th, th);
  float ps = 0x1.71de3ap-19f;                        /* +1/9! */
  ps = DMLF_ADD(DMLF_MUL(ps, t2), -0x1.a01a02p-13f); /* -1/7! */
  ps = DMLF_ADD(DMLF_MUL(ps, t2), 0x1.111112p-7f);   /* +1/5! */
  ps = DMLF_ADD(DMLF_MUL(ps, t2), -0x1.555556p-3f);  /* -1/3! */
  *s = DMLF_ADD(th, DMLF_MUL(DMLF_MUL(ps, t2), th));
  float pc = -0x1.27e4fcp-22f;                       /* -1/10! */
  pc = DMLF_ADD(DMLF_MUL(pc, t2), 0x1.a01a02p-16f);  /* +1/8! */
  pc = DMLF_ADD(DMLF_MUL(pc, t2), -0x1.6c16c2p-10f); /* -1/6! */
  pc = DMLF_ADD(DMLF_MUL(pc, t2), 0x1.555556p-5f);   /* +1/4! */
  pc = DMLF_ADD(DMLF_MUL(pc, t2), -0.5f);            /* -1/2! */
  *c = DMLF_ADD(1.0f, DMLF_MUL(pc, t2));
}

/* sin(2 pi u) and cos(2 pi u) for u = x * 2^-24, x a 24-bit integer: the
 * quadrant is floor(4u) = x >> 22 and the fraction 4u - floor(4u) =
 * (x mod 2^22) * 2^-22, both exact (no rounding or conversion instruction
 * on the device). */
DML_HD void dml_sincosf_2pi_bits(uint32_t x, float* sn, float* cs) {
  const int qi = (int)(x >> 22);
  float f = DMLF_MUL(dml_u32_to_f32_rn(x & 0x3FFFFFu), 0x1.0p-22f); /* exact, [0,1) */
  int swap = f > 0.5f;
  float g = swap ? DMLF_SUB(1.0f, f) : f; /* exact */
  float th = DMLF_MUL(g, 0x1.921fb6p+0f); /* g * pi/2, in [0, pi/4] */
  float s0, c0;
  dml_sincosf_small(th, &s0, &c0);
  float sa = swap ? c0 : s0; /* sin(f pi/2) */
  float ca = swap ? s0 : c0; /* cos(f pi/2) */
  switch (qi & 3) {
    case 0: *sn = sa; *cs = ca; break;
    case 1: *sn = ca; *cs = -sa; break;
    case 2: *sn = -sa; *cs = -ca; break;
    default: *sn = -ca; *cs = sa; break;
  }
}

/* The same for a float u in [0,1) that is a multiple of 2^-24. */
DML_HD void dml_sincosf_2pi(float u, float* sn, float* cs) {
  dml_sincosf_2pi_bits((uint32_t)DMLF_MUL(u, 0x1.0p+24f), sn, cs);
}

/* Two standard normals from two 32-bit words (Box-Muller): a uniform in
 * (0,1] from the first word, u1 = RN32(a + 1) * 2^-32 (a + 1 = 2^32 is
 * exact), and the angle 2 pi u2 from the top 24 bits of the second,
 * u2 = (b >> 8) * 2^-24. */
DML_HD void dml_normal_pair32f(uint32_t a, uint32_t b, float* n0, float* n1) {
#if defined(__CUDA_ARCH__)
  float a1 = a == 0xFFFFFFFFu ? 0x1.0p+32f : dml_u32_to_f32_rn(a + 1u);
  float u1 = __fmul_rn(a1, 0x1.0p-32f); /* (0,1] */
#else
  float u1 = (float)((uint64_t)a + 1ull) * 0x1.0p-32f;
#endif
  float r = DMLF_SQRT(DMLF_MUL(-2.0f, dml_logf(u1)));
  float s, c;
  dml_sincosf_2pi_bits(b >> 8, &s, &c);
  *n0 = DMLF_MUL(r, c);
  *n1 = DMLF_MUL(r, s);
}

DML_HD void dml_normal_pair32(uint32_t a, uint32_t b, double* n0, double* n1) {
  float f0, f1;
  dml_normal_pair32f(a, b, &f0, &f1);
  *n0 = dml_f32_to_f64(f0);
  *n1 = dml_f32_to_f64(f1);
}

/* Four standard normals from one 128-bit draw (FP32 values). */
DML_HD void dml_normal_quadf(dml_u4 w, float* n) {
  dml_normal_pair32f(w.w[0], w.w[1], &n[0], &n[1]);
  dml_normal_pair32f(w.w[2], w.w[3], &n[2], &n[3]);
}

DML_HD void dml_normal_quad(dml_u4 w, double* n) {
  dml_normal_pair32(w.w[0], w.w[1], &n[0], &n[1]);
  dml_normal_pair32(w.w[2], w.w[3], &n[2], &n[3]);
}

/* Uniform on [0,1) from the first two words of a draw. */
DML_HD double dml_uniform(dml_u4 w) { return dml_u53(w.w[0], w.w[1]); }

#endif /* DML_RNG_H */
