/*
 * ecmg_tmath.h -- deterministic single-precision atan / sin / cos.
 *
 * The ORCA agent constraint (ECMAgentSimulator/ORCA.cpp:375-378) rotates the
 * velocity-obstacle centre by +/- atan(r/d) through MathUtility::RotateVector
 * (ECMGenerator/UtilityFunctions.cpp:233-242), i.e. one atanf, one cosf and one
 * sinf per neighbour.  The host C library and the CUDA math library round those
 * differently, so a GPU tick and a CPU tick that call their "own" libm can never
 * agree bit for bit.  This header gives one implementation that the CUDA kernels
 * and the CPU oracle both compile, so that both sides round identically.
 *
 * Method (own derivation, no vendor constants):
 *   atan : reduce |x| > 1 with atan(x) = pi/2 - atan(1/x); reduce t > tan(pi/8)
 *          with atan(t) = pi/4 + atan((t-1)/(t+1)); on |u| <= tan(pi/8) use
 *          u + u^3 P(u^2), P a degree-4 polynomial fitted by weighted least
 *          squares on Chebyshev nodes (relative error).  pi/4 and pi/2 are
 *          added as hi + lo float pairs (Cody & Waite style).
 *   sin/cos : on |a| <= pi/4 use a + a^3 S(a^2) and 1 - (a^2/2 - a^4 C(a^2)),
 *          S and C fitted the same way; pi/4 < |a| <= pi/2 uses the complement
 *          angle (pi/2_hi - |a|) + pi/2_lo.  Larger |a| (never produced by the
 *          callers, whose argument is an atan result) is reduced in double up
 *          to |a| = 1e6; beyond that both functions return NaN.
 * Accuracy over the argument ranges used: atan <= 2.1 ulp, sin <= 1.2 ulp,
 * cos <= 1.5 ulp against float64 (tests/test_tmath.py measures it).
 *
 * Every operation is a separately rounded IEEE-754 binary32 operation: the CUDA
 * sources that include this file are built with -fmad=false and the C oracle
 * with -ffp-contract=off, so no multiply-add is fused on either side.
 */
#ifndef ECMG_TMATH_H
#define ECMG_TMATH_H

#if defined(__CUDACC__)
#define ECMG_TM_HD __host__ __device__ __forceinline__
#else
#define ECMG_TM_HD static inline
#endif

#define ECMG_TM_PI4_HI 0.785398185253143310546875f
#define ECMG_TM_PI4_LO (-2.18556943121302206e-08f)
#define ECMG_TM_PI2_HI 1.57079637050628662109375f
#define ECMG_TM_PI2_LO (-4.37113886242604412e-08f)

ECMG_TM_HD float ecmg_atanf(float x)
{
    if (x != x) return x; /* NaN */
    float a = x < 0.0f ? -x : x;
    if (a == 0.0f) return x; /* keeps the sign of zero */
    int inv = a > 1.0f;
    float t = inv ? 1.0f / a : a; /* 1/inf = 0 -> pi/2 */
    int mid = t > 0.41421356f;
    float u = mid ? (t - 1.0f) / (t + 1.0f) : t;
    float z = u * u;
    float p = -0.060462791472673416f;
    p = 0.10582651942968369f + z * p;
    p = -0.1424226611852646f + z * p;
    p = 0.19998420774936676f + z * p;
    p = -0.3333331346511841f + z * p;
    float r = u + (u * z) * p;
    if (mid) r = ECMG_TM_PI4_HI + (ECMG_TM_PI4_LO + r);
    if (inv) r = ECMG_TM_PI2_HI - (r - ECMG_TM_PI2_LO);
    return x < 0.0f ? -r : r;
}

/* kernels on |u| <= pi/4 */
ECMG_TM_HD float ecmg_tm_sin_k(float u)
{
    float z = u * u;
    float p = -0.00019511666323523968f;
    p = 0.008332139812409878f + z * p;
    p = -0.16666653752326965f + z * p;
    return u + (u * z) * p;
}

ECMG_TM_HD float ecmg_tm_cos_k(float u)
{
    float z = u * u;
    float p = -2.719883980262239e-07f;
    p = 2.4799375751172192e-05f + z * p;
    p = -0.0013888883404433727f + z * p;
    p = 0.0416666679084301f + z * p;
    float r = 0.5f * z - (z * z) * p;
    return 1.0f - r;
}

/* sin and cos of one argument; the callers need both (RotateVector). */
ECMG_TM_HD void ecmg_sincosf(float a, float* s, float* c)
{
    if (a != a) { *s = a; *c = a; return; }
    float b = a < 0.0f ? -a : a;
    if (b <= ECMG_TM_PI4_HI) {
        *s = ecmg_tm_sin_k(a);
        *c = ecmg_tm_cos_k(a);
        return;
    }
    if (b <= ECMG_TM_PI2_HI) {
        float cpl = (ECMG_TM_PI2_HI - b) + ECMG_TM_PI2_LO; /* pi/2 - |a| */
        float sv = ecmg_tm_cos_k(cpl);
        *s = a < 0.0f ? -sv : sv;
        *c = ecmg_tm_sin_k(cpl);
        return;
    }
    /* outside [-pi/2, pi/2]: quadrant reduction in double (not reached by the
       ORCA callers; kept so the functions are total) */
    if (!(b <= 1.0e6f)) { *s = (a - a) / (a - a); *c = *s; return; } /* NaN beyond the supported range */
    double ad = (double)a;
    double k = ad * 0.63661977236758138; /* 2/pi */
    k = (k >= 0.0) ? (double)(long long)(k + 0.5) : -(double)(long long)(-k + 0.5);
    double rd = ad - k * 1.5707963267948966; /* pi/2 in double */
    float r = (float)rd;
    long long q = (long long)k;
    int qm = (int)(q & 3);
    float sk = ecmg_tm_sin_k(r), ck = ecmg_tm_cos_k(r);
    if (qm == 0) { *s = sk; *c = ck; }
    else if (qm == 1) { *s = ck; *c = -sk; }
    else if (qm == 2) { *s = -sk; *c = -ck; }
    else { *s = -ck; *c = sk; }
}

#endif /* ECMG_TMATH_H */
