/* Portable single-precision cos/sin for the oracle (test infrastructure).
 *
 * Why it exists: the reference's per-pixel RNG (Assets/Tracer.comp:225-234) is
 *     rand() = fract(cos(dot((coords + ++rand_salt) * 5, K1)) * 12345.6789)
 * with |argument| up to ~1e6.  One ulp of the argument there is ~0.06, and the
 * cosine is then scaled by 1.2e4 before fract(), so two cos implementations
 * that differ by one ulp give unrelated random streams.  GLSL leaves cos
 * accuracy to the driver, so the reference has no single "true" stream.  This
 * file defines the stream used by the oracle and the CUDA kernels: every step
 * below is an IEEE-754 single-precision operation (multiply, fused
 * multiply-add, round-to-integer), so any conforming host or device gives the
 * same bits.
 *
 * Method (own derivation, nothing taken from a vendor library):
 *   k = rint(x * 2/pi), r = x - k*(C1 + C2 + C3)   Cody-Waite reduction with
 *   pi/2 split into three floats, each the float nearest to what is left of
 *   pi/2 after the previous ones.  With C1 rounded to 24 bits, x - k*C1 done
 *   in one fma is exact for |x| < 2^24 (the result is a multiple of 2^-23
 *   below 2 in magnitude).  pi was computed with Machin's formula
 *   pi = 16 atan(1/5) - 4 atan(1/239) to 80 digits.
 *   cos r and sin r on |r| <= pi/4 (+ slack) by their Taylor series to r^12 and
 *   r^11 (truncation < 2e-10), coefficients 1/n! rounded to float, evaluated
 *   by Horner's rule with fma.
 *   Quadrant q = k mod 4 picks +-cos r / +-sin r.
 * Accuracy against double-precision cos/sin: a few float ulps for
 * |x| < 2^22 (checked by tests/test_oracle_rng.py).  NaN and +-inf give NaN.
 *
 * The file must be compiled with -ffp-contract=off on the host so that no
 * extra fused operation is formed.
 */
#ifndef ORACLE_RNG_TRIG_H
#define ORACLE_RNG_TRIG_H

#include <math.h>

#define ORACLE_TRIG_TWO_OVER_PI 0x1.45f306p-1f
#define ORACLE_TRIG_C1 0x1.921fb6p+0f
#define ORACLE_TRIG_C2 (-0x1.777a5cp-25f)
#define ORACLE_TRIG_C3 (-0x1.ee59dap-50f)

#define ORACLE_COS_C2 (-0x1.0p-1f)
#define ORACLE_COS_C4 0x1.555556p-5f
#define ORACLE_COS_C6 (-0x1.6c16c2p-10f)
#define ORACLE_COS_C8 0x1.a01a02p-16f
#define ORACLE_COS_C10 (-0x1.27e4fcp-22f)
#define ORACLE_COS_C12 0x1.1eed8ep-29f

#define ORACLE_SIN_S3 (-0x1.555556p-3f)
#define ORACLE_SIN_S5 0x1.111112p-7f
#define ORACLE_SIN_S7 (-0x1.a01a02p-13f)
#define ORACLE_SIN_S9 0x1.71de3ap-19f
#define ORACLE_SIN_S11 (-0x1.ae6456p-26f)

/* Reduces x to r in about [-pi/4, pi/4]; *q = quadrant in 0..3. */
static inline float oracle_trig_reduce(float x, int* q)
{
    float k = rintf(x * ORACLE_TRIG_TWO_OVER_PI);
    float r = fmaf(-k, ORACLE_TRIG_C1, x);
    r = fmaf(-k, ORACLE_TRIG_C2, r);
    r = fmaf(-k, ORACLE_TRIG_C3, r);
    /* k mod 4, exactly, for any finite float k */
    float kq = k - 4.0f * floorf(k * 0.25f);
    *q = (kq == kq) ? (int)kq : 0;
    return r;
}

static inline float oracle_cos_poly(float r)
{
    float z = r * r;
    float p = fmaf(z, ORACLE_COS_C12, ORACLE_COS_C10);
    p = fmaf(z, p, ORACLE_COS_C8);
    p = fmaf(z, p, ORACLE_COS_C6);
    p = fmaf(z, p, ORACLE_COS_C4);
    p = fmaf(z, p, ORACLE_COS_C2);
    return fmaf(z, p, 1.0f);
}

static inline float oracle_sin_poly(float r)
{
    float z = r * r;
    float p = fmaf(z, ORACLE_SIN_S11, ORACLE_SIN_S9);
    p = fmaf(z, p, ORACLE_SIN_S7);
    p = fmaf(z, p, ORACLE_SIN_S5);
    p = fmaf(z, p, ORACLE_SIN_S3);
    return fmaf(r * z, p, r);
}

static inline float oracle_rng_cos(float x)
{
    int q;
    float r = oracle_trig_reduce(x, &q);
    float c = oracle_cos_poly(r);
    float s = oracle_sin_poly(r);
    switch (q) {
    case 0: return c;
    case 1: return -s;
    case 2: return -c;
    default: return s;
    }
}

static inline float oracle_rng_sin(float x)
{
    int q;
    float r = oracle_trig_reduce(x, &q);
    float c = oracle_cos_poly(r);
    float s = oracle_sin_poly(r);
    switch (q) {
    case 0: return s;
    case 1: return c;
    case 2: return -s;
    default: return -c;
    }
}

#endif /* ORACLE_RNG_TRIG_H */
