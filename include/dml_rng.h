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
 * Normals come from the Box-Muller transform.  `log`, `sin` and `cos` are NOT
 * taken from libm or CUDA (their results differ between host and device);
 * they are written here from textbook series:
 *   log(m) = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...),  s = (m-1)/(m+1),
 *            with m in [sqrt(1/2), sqrt(2)) after removing the binary exponent;
 *   sin, cos: Taylor series on [0, pi/4] after an exact quadrant reduction of
 *            the angle 2*pi*u (u is a multiple of 2^-53, so 4u is exact).
 * Every operation is an IEEE double add, subtract, multiply, divide or sqrt
 * in a fixed order with no fused multiply-add, so host and device agree to
 * the last bit.  Accuracy: |error| < 4e-16 relative for log, < 3e-16 absolute
 * for sin/cos (checked against libm in the CPU test suite).
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
#define DML_MUL(a, b) __dmul_rn((a), (b))
#define DML_ADD(a, b) __dadd_rn((a), (b))
#define DML_SUB(a, b) __dsub_rn((a), (b))
#define DML_DIV(a, b) __ddiv_rn((a), (b))
#define DML_SQRT(a) __dsqrt_rn(a)
#else
#include <math.h>
#include <string.h>
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

/* Natural logarithm for normal positive x (the Box-Muller argument lies in
 * [2^-53, 1]).  Exponent split + atanh series, see the header comment. */
DML_HD double dml_log(double x) {
  uint64_t bits = dml_f64_bits(x);
  int e = (int)((bits >> 52) & 0x7FF) - 1023;
  double m = dml_bits_f64((bits & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);
  if (m > 0x1.6a09e667f3bcdp+0) { /* sqrt(2) */
    m = DML_MUL(m, 0.5);
    e += 1;
  }
  double f = DML_SUB(m, 1.0);          /* exact (Sterbenz) */
  double s = DML_DIV(f, DML_ADD(2.0, f));
  double s2 = DML_MUL(s, s);
  /* r = s2/3 + s2^2/5 + ... + s2^11/23, Horner from the highest term. */
  double p = 0x1.642c8590b2164p-5;                         /* 1/23 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.8618618618618p-5);      /* 1/21 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.af286bca1af28p-5);      /* 1/19 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.e1e1e1e1e1e1ep-5);      /* 1/17 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.1111111111111p-4);      /* 1/15 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.3b13b13b13b14p-4);      /* 1/13 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.745d1745d1746p-4);      /* 1/11 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.c71c71c71c71cp-4);      /* 1/9 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.2492492492492p-3);      /* 1/7 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.999999999999ap-3);      /* 1/5 */
  p = DML_ADD(DML_MUL(p, s2), 0x1.5555555555555p-2);      /* 1/3 */
  double r = DML_MUL(s2, p);
  double two_s = DML_MUL(2.0, s);
  double lm = DML_ADD(two_s, DML_MUL(two_s, r));
  double de = (double)e;
  /* ln2 split in a high part (exact products with |e| <= 1100) and a low part. */
  return DML_ADD(DML_MUL(de, 0x1.62e42fefa39efp-1), DML_ADD(lm, DML_MUL(de, 0x1.abc9e3b39803fp-56)));
}

/* sin and cos of theta in [0, pi/4] by Taylor series (terms to theta^19 / theta^18). */
DML_HD void dml_sincos_small(double th, double* s, double* c) {
  double t2 = DML_MUL(th, th);
  double ps = -0x1.2f49b46814157p-57;                    /* -1/19! */
  ps = DML_ADD(DML_MUL(ps, t2), 0x1.952c77030ad4ap-49);  /* +1/17! */
  ps = DML_ADD(DML_MUL(ps, t2), -0x1.ae7f3e733b81fp-41); /* -1/15! */
  ps = DML_ADD(DML_MUL(ps, t2), 0x1.6124613a86d09p-33);  /* +1/13! */
  ps = DML_ADD(DML_MUL(ps, t2), -0x1.ae64567f544e4p-26); /* -1/11! */
  ps = DML_ADD(DML_MUL(ps, t2), 0x1.71de3a556c734p-19);  /* +1/9! */
  ps = DML_ADD(DML_MUL(ps, t2), -0x1.a01a01a01a01ap-13); /* -1/7! */
  ps = DML_ADD(DML_MUL(ps, t2), 0x1.1111111111111p-7);   /* +1/5! */
  ps = DML_ADD(DML_MUL(ps, t2), -0x1.5555555555555p-3);  /* -1/3! */
  *s = DML_ADD(th, DML_MUL(DML_MUL(ps, t2), th));
  double pc = 0x1.6827863b97d97p-53;                     /* +1/18! */
  pc = DML_ADD(DML_MUL(pc, t2), -0x1.ae7f3e733b81fp-45); /* -1/16! */
  pc = DML_ADD(DML_MUL(pc, t2), 0x1.93974a8c07c9dp-37);  /* +1/14! */
  pc = DML_ADD(DML_MUL(pc, t2), -0x1.1eed8eff8d898p-29); /* -1/12! */
  pc = DML_ADD(DML_MUL(pc, t2), 0x1.27e4fb7789f5cp-22);  /* +1/10! */
  pc = DML_ADD(DML_MUL(pc, t2), -0x1.a01a01a01a01ap-16); /* -1/8! */
  pc = DML_ADD(DML_MUL(pc, t2), 0x1.6c16c16c16c17p-10);  /* +1/6! */
  pc = DML_ADD(DML_MUL(pc, t2), -0x1.5555555555555p-5);  /* -1/4! */
  pc = DML_ADD(DML_MUL(pc, t2), 0x1.0p-1);               /* +1/2! */
  *c = DML_SUB(1.0, DML_MUL(pc, t2));
}

/* sin(2 pi u) and cos(2 pi u) for u in [0,1) that is a multiple of 2^-53. */
DML_HD void dml_sincos_2pi(double u, double* sn, double* cs) {
  double t4 = DML_MUL(u, 4.0); /* exact */
  double q = floor(t4);
  double f = DML_SUB(t4, q);  /* exact, [0,1) */
  int qi = (int)q;
  int swap = f > 0.5;
  double g = swap ? DML_SUB(1.0, f) : f; /* exact */
  double th = DML_MUL(g, 0x1.921fb54442d18p+0); /* g * pi/2, in [0, pi/4] */
  double s0, c0;
  dml_sincos_small(th, &s0, &c0);
  double sa = swap ? c0 : s0; /* sin(f pi/2) */
  double ca = swap ? s0 : c0; /* cos(f pi/2) */
  switch (qi & 3) {
    case 0: *sn = sa; *cs = ca; break;
    case 1: *sn = ca; *cs = -sa; break;
    case 2: *sn = -sa; *cs = -ca; break;
    default: *sn = -ca; *cs = sa; break;
  }
}

/* Two independent standard normals from one 128-bit draw (Box-Muller). */
DML_HD void dml_normal_pair(dml_u4 w, double* n0, double* n1) {
  double u1 = DML_SUB(1.0, dml_u53(w.w[0], w.w[1])); /* (0,1] */
  double u2 = dml_u53(w.w[2], w.w[3]);
  double r = DML_SQRT(DML_MUL(-2.0, dml_log(u1)));
  double s, c;
  dml_sincos_2pi(u2, &s, &c);
  *n0 = DML_MUL(r, c);
  *n1 = DML_MUL(r, s);
}

/* Uniform on [0,1) from the first two words of a draw. */
DML_HD double dml_uniform(dml_u4 w) { return dml_u53(w.w[0], w.w[1]); }

#endif /* DML_RNG_H */
