/*
 * refmath.h — FP32 evaluations of the reference's mixed float/double
 * expressions, for the per-pair inner loops where GB300's FP64 rate (about
 * 1/64 of FP32) would dominate.
 *
 * The reference's FLOAT is float, but several expressions promote to double
 * and round back once (src/kernel.cpp:4-10, glibc hypotf via
 * src/utility.cpp:16-18, the FLIP blend of src/flip3D.cpp:1095). The
 * functions below evaluate the exact value as an unevaluated float pair
 * (s, lo) with error-free transforms (Knuth TwoSum, FMA-based TwoProd) and
 * round it once. Where that rounding is ambiguous — the pair lies within
 * 2^-16 of a half-spacing from a float rounding boundary, closer than the
 * pair's own error allows to decide — they evaluate the reference's double
 * expression instead, so the result is the reference's in every case; the
 * slow branch is rare (about 4% of FLIP blends, far fewer elsewhere).
 * tests/test_refmath.py checks millions of samples against the double
 * formulas on the host.
 *
 * Compile without FMA contraction (nvcc -fmad=false, g++ -ffp-contract=off):
 * every a*b+c below that is not an explicit fmaf must round twice.
 */
#ifndef FLIP_REFMATH_H
#define FLIP_REFMATH_H

#if defined(__CUDACC__)
#define RM_FN __host__ __device__ __forceinline__
/* The double-precision fallbacks are out of line: inlined, the compiler may
 * hoist their float-to-double conversions onto the common path, and every
 * FP64 instruction costs the time of dozens of FP32 ones on this GPU. */
#define RM_COLD static __host__ __device__ __noinline__
#else
#include <cmath>
#define RM_FN static inline
#define RM_COLD static
#endif

namespace refmath {

/* ---- double expressions of the reference, taken only when the FP32
 * error-free evaluation cannot decide the rounding ---- */
RM_COLD float hypot_d(float a, float b) {
  return (float)sqrt((double)a * (double)a + (double)b * (double)b);
}
RM_COLD float sharp_d(float hh, float r2) { return (float)((double)hh / (double)r2 - 1.0); }
RM_COLD float add_d(float a, double b) { return (float)((double)a + b); }
RM_COLD float blend_d(float x, float y, double c1, double c2) {
  double a = c1 * (double)x;
  double b = c2 * (double)y;
  return (float)(a + b);
}
RM_COLD float axpy_d(float p, float v, double c) {
  double d = c * (double)v;
  return (float)((double)p + d);
}

/* s + e == a + b exactly (Knuth TwoSum). */
RM_FN void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

/* p + e == a * b exactly. */
RM_FN void two_prod(float a, float b, float &p, float &e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

RM_FN unsigned bits_of(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  unsigned u;
  __builtin_memcpy(&u, &x, sizeof u);
  return u;
#endif
}
RM_FN float from_bits(unsigned u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  __builtin_memcpy(&x, &u, sizeof x);
  return x;
#endif
}

/* r = round(s + lo) and t = (s + lo) - r exactly. True when r could be the
 * wrong neighbour: |t| is within 2^-16 of half the gap to the float on t's
 * side (the gap halves below a power of two). */
RM_FN bool near_tie(float r, float t) {
  unsigned b = bits_of(r) & 0x7fffffffu;
  if (b == 0 || b >= 0x7f800000u) return t != 0.0f;
  float ar = from_bits(b);
  float gap = from_bits(b + 1) - ar;
  bool toward_zero = (r > 0.0f) ? (t < 0.0f) : (t > 0.0f);
  if ((b & 0x7fffffu) == 0 && toward_zero && b > 0x00800000u) gap *= 0.5f;
  float half = 0.5f * gap;
  return fabsf(fabsf(t) - half) <= half * 0x1p-16f;
}

/* glibc hypotf(a, b) = (float)sqrt((double)a*a + (double)b*b), as the
 * reference's length() calls it (src/utility.cpp:16-18). */
RM_FN float hypot_ref(float a, float b) {
  float p1, e1, p2, e2, s, es;
  two_prod(a, a, p1, e1);
  two_prod(b, b, p2, e2);
  two_sum(p1, p2, s, es);
  if (s == 0.0f) return 0.0f;
  float lo = es + (e1 + e2);
  float r = sqrtf(s);
  float d = fmaf(-r, r, s) + lo;       /* (s + lo) - r*r */
  float corr = d * (0.5f / r);         /* sqrt(s + lo) - r to ~2^-24 rel */
  float out, t;
  two_sum(r, corr, out, t);
  if (near_tie(out, t)) return hypot_d(a, b);
  return out;
}

/* length(p0, p1) = hypotf(hypotf(dx, dy), dz) (src/utility.cpp:16-18). */
RM_FN float length_ref(float dx, float dy, float dz) {
  return hypot_ref(hypot_ref(dx, dy), dz);
}

/* hypot2 (src/utility.cpp:20-22): a*a + b*b + c*c, each step rounded. */
RM_FN float hypot2_ref(float a, float b, float c) {
  return a * a + b * b + c * c;
}

/* smooth_kernel (src/kernel.cpp:4-6): fmax(1.0 - r2/(h*h), 0.0) rounded
 * to float. 1 - q is exact in double for the float q involved, so a single
 * float subtraction rounds it the same way. hh = h*h in float. */
RM_FN float smooth_ref(float r2, float hh) {
  float q = r2 / hh;
  return fmaxf(1.0f - q, 0.0f);
}

/* smooth_ref with hh a power of two (rcp = 1/hh exactly): the quotient is
 * an exact scaling, so a multiply gives the division's result bit for bit. */
RM_FN float smooth_ref_pow2(float r2, float rcp) {
  float q = r2 * rcp;
  return fmaxf(1.0f - q, 0.0f);
}

/* sharp_kernel (src/kernel.cpp:8-10): fmax(hh/fmax(r2,1e-5) - 1.0, 0.0) in
 * double, rounded to float. For r2 >= hh the result is 0. r2 below 1e-5
 * (r2_floor is the smallest float above 1e-5) takes the constant branch
 * `small` = float(hh/1e-5 - 1), precomputed in double by the caller. */
RM_FN float sharp_ref(float r2, float hh, float r2_floor, float small) {
  if (!(r2 < hh)) return 0.0f;
  if (r2 < r2_floor) return small;
  float q = hh / r2;                  /* correctly rounded quotient */
  /* Near the support edge (q < 1 + 2^-8) q - 1 cancels: there hh - r2 is
   * exact (Sterbenz), so D/r2 rounds the exact value once. The reference
   * rounds hh/r2 to double first, which can move a result lying within about
   * 2^-12 ulp of a tie; those go to its double expression. */
  if (q < 1.00390625f) {
    float D = hh - r2;
    float X = D / r2;
    float R = fmaf(-X, r2, D);        /* exact remainder */
    float t = R / r2;
    float gapx = from_bits(bits_of(X) + 1) - X;
    if (fabsf(fabsf(t) - 0.5f * gapx) <= gapx * 0x1p-10f || X == 0.0f) return sharp_d(hh, r2);
    return X;
  }
  float rem = fmaf(-q, r2, hh);       /* hh - q*r2, exact */
  float t, e;
  two_sum(q, -1.0f, t, e);            /* t + e == q - 1 exactly */
  float c1 = rem / r2;                /* Q - q, to float accuracy ... */
  float rem2 = fmaf(-c1, r2, rem);    /* ... whose remainder is exact ... */
  float c = c1 + rem2 / r2;           /* ... to double-float accuracy */
  float out, r;
  two_sum(t, e + c, out, r);
  if (near_tie(out, r)) return sharp_d(hh, r2);
  return out;
}

/* (float)((double)a + (double)b_hi + (double)b_lo) for a double constant
 * split into b_hi = float(b), b_lo = float(b - b_hi): a + b rounded once. */
/* The pair's error is below 2^-46 of its largest term; when the result has
 * cancelled to under 2^-20 of that term the float path cannot decide it. */
RM_FN bool cancelled(float out, float big) {
  return fabsf(out) < fabsf(big) * 0x1p-20f;
}

RM_FN float add_fd(float a, float b_hi, float b_lo, double b) {
  float s, e, out, t;
  two_sum(a, b_hi, s, e);
  two_sum(s, e + b_lo, out, t);
  if (near_tie(out, t) || cancelled(out, fmaxf(fabsf(a), fabsf(b_hi)))) return add_d(a, b);
  return out;
}

/* (float)(c*(double)x) for a double constant c = c_hi + c_lo. */
RM_FN void mul_fd(float x, float c_hi, float c_lo, float &p, float &e) {
  two_prod(x, c_hi, p, e);
  e = fmaf(x, c_lo, e);
}

/* (float)(c1*(double)x + c2*(double)y): the FLIP blend of
 * src/flip3D.cpp:1095 with c1 = 1-ALPHA, c2 = ALPHA. */
RM_FN float blend_ref(float x, float y, float c1h, float c1l, float c2h,
                      float c2l, double c1, double c2) {
  float p1, e1, p2, e2, s, es, out, t;
  mul_fd(x, c1h, c1l, p1, e1);
  mul_fd(y, c2h, c2l, p2, e2);
  two_sum(p1, p2, s, es);
  two_sum(s, es + (e1 + e2), out, t);
  if (near_tie(out, t) || cancelled(out, fmaxf(fabsf(p1), fabsf(p2)))) return blend_d(x, y, c1, c2);
  return out;
}

/* (float)((double)p + c*(double)v): the Euler step p += DT*vel of
 * src/flip3D.cpp:884 with c = DT. */
RM_FN float axpy_fd(float p, float v, float ch, float cl, double c) {
  float m, me, s, es, out, t;
  mul_fd(v, ch, cl, m, me);
  two_sum(p, m, s, es);
  two_sum(s, es + me, out, t);
  if (near_tie(out, t) || cancelled(out, fmaxf(fabsf(p), fabsf(m)))) return axpy_d(p, v, c);
  return out;
}

} // namespace refmath

#endif
