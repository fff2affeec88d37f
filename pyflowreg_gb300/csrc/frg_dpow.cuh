// Float64 power x^b for the data-term nonlinearity of the float64 solver,
// psi = a (E + 1e-5)^(a - 1) (core/level_solver.py:247), in 15 float64
// operations instead of the ~100 the general pow costs on a float64 pipe that
// runs at 1/64 of the float32 rate.
//
// Method: the table-driven logarithm and exponential of P. T. P. Tang
// ("Table-driven implementation of the logarithm function in IEEE
// floating-point arithmetic", ACM TOMS 16(4), 1990; "Table-driven
// implementation of the exponential function ...", ACM TOMS 15(2), 1989),
// in base 2, with the product b * log2(x) carried as a double-double:
//   x = 2^e m, m in [1, 2); j = the top 8 bits of m's fraction;
//   c_j = 1 + (j + 1/2) / 256, inv_j = double(1 / c_j), r = m inv_j - 1
//     (one fused multiply-add, |r| <= 2^-9);
//   log2 x = e - log2(inv_j) + log2(1 + r), log2(1 + r) by its Taylor series
//     to r^5 (truncation below 2^-56, a tenth of an ulp of the result);
//     -log2(inv_j) is tabulated as Lhi + Llo with Lhi a multiple of 2^-42, so
//     e + Lhi is exact (and formed by integer operations from the fixed-point
//     sum, as is the double of k below);
//   y = b log2 x = yh + yl: yh = b (e + Lhi) rounded, yl its rounding error
//     (an fma) plus b (Llo + log2(1 + r)), so |yl| <= |b| 2^-8.5;
//   k = round(256 yh), f = yh - k / 256 + yl, |f| <= 2^-9 + |b| 2^-8.5;
//   2^y = 2^(k >> 8) * 2^((k & 255) / 256) * (1 + q(f)), q the Taylor series
//     of 2^f - 1 to f^5 (truncation below 2^-60 for |b| <= 1).
// Both series keep their first three terms in float64 and evaluate the r^4 and
// r^5 (f^4 and f^5) terms in float32 (below 2^-36 and 2^-30: float32 rounding
// of them, and a truncated float32 copy of r or f, stay below 2^-60), moved
// between the two formats by integer operations, so that each series costs
// three float64 fused multiply-adds.
// An exact emulation of these steps (rational arithmetic for every float64
// rounding, float32 arithmetic for the tails) stays within 1 ulp of the
// correctly rounded power (0.98 ulp at most on 15000 arguments, exponents
// -0.95 to 1); without the f^5 term of the exp series it is off by up to
// 11 ulp (f includes yl).
// Every step is one rounding of a value below the result's ulp except the
// final two, so the result is within a few ulp of x^b.  Positive normal x
// with |b log2 x| < 512 take this path; anything else (0, denormals,
// infinities, NaN, huge results) goes to pow().  Range tests are integer
// tests on the high words, which keeps them off the float64 pipe.
#pragma once

#include <cuda_runtime.h>

#include "frg_internal.h"

namespace frg {

constexpr int kDpowLogN = 256;   // log table entries: (inv_j, Lhi 2^42 as a 64-bit integer, Llo)
constexpr int kDpowExpN = 256;   // exp table entries: 2^(i / 256)

// The tables (device memory of this translation unit; the library is built
// without relocatable device code, so only frg_sor64.cu includes this header),
// filled by upload_dpow_tables().
__device__ double g_dpow_log[3 * kDpowLogN];
__device__ double g_dpow_exp[kDpowExpN];

// 1 / (i ln 2) with alternating signs: log2(1 + r) = sum_i (-1)^(i+1) r^i / (i ln 2)
constexpr double kL1 = 1.4426950408889634074;
constexpr double kL2 = -0.72134752044448170368;
constexpr double kL3 = 0.48089834696298780245;
constexpr double kL4 = -0.36067376022224085184;
constexpr double kL5 = 0.28853900817779268147;
// (ln 2)^i / i!: 2^f - 1 = sum_i (f ln 2)^i / i!
constexpr double kE1 = 0.69314718055994530942;
constexpr double kE2 = 0.24022650695910071233;
constexpr double kE3 = 0.055504108664821579953;
constexpr double kE4 = 0.0096181291076284771620;
constexpr double kE5 = 0.0013333558146428443423;

// float64 -> float32 by truncation and float32 -> float64, on the integer pipe
// (the conversion instructions run on the float64 pipe); values below 2^-126
// become zero.  For the series tails only: finite, below 1 in magnitude.
__device__ __forceinline__ float dpow_tail_f(double x)
{
    const int h = __double2hiint(x);
    const unsigned l = (unsigned)__double2loint(x);
    const int e = (h >> 20) & 0x7ff;
    const unsigned s = (unsigned)h & 0x80000000u;
    if (e < 897) return __uint_as_float(s);
    return __uint_as_float(s | ((unsigned)(e - 896) << 23) | (((unsigned)h & 0xfffffu) << 3) | (l >> 29));
}

__device__ __forceinline__ double dpow_tail_d(float x)
{
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    const unsigned s = b & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)s, 0);
    return __hiloint2double((int)(s | ((e + 896u) << 20) | ((b >> 3) & 0xfffffu)), (int)(b << 29));
}

// c4 t^4 + c5 t^5 in float32 from a truncated copy of t
__device__ __forceinline__ double dpow_tail(double t, float c4, float c5)
{
    const float tf = dpow_tail_f(t);
    const float t2 = __fmul_rn(tf, tf);
    return dpow_tail_d(__fmul_rn(__fmul_rn(t2, t2), __fadd_rn(c4, __fmul_rn(tf, c5))));
}

__device__ __forceinline__ double dpow_tab(double x, double b)
{
    const int hi = __double2hiint(x);
    const int lo = __double2loint(x);
    if (hi < 0x00100000 || hi >= 0x7ff00000) return pow(x, b);  // not a positive normal finite number
    const int eb = hi >> 20;                                     // biased exponent
    const int j = (hi >> 12) & 0xff;
    const double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);
    const double* lt = g_dpow_log + 3 * j;
    const double r = __fma_rn(m, __ldg(lt), -1.0);
    double p = __fma_rn(r, kL3, kL2);
    p = __fma_rn(r, p, kL1);
    p = __fma_rn(r, p, dpow_tail(r, (float)kL4, (float)kL5));
    // e + Lhi, exact: the fixed-point integer N = (eb - 1023) 2^42 + Lhi 2^42
    // (0 < |N| < 2^52) written as a double by integer operations
    const long long N = ((long long)(eb - 1023) << 42) + __double_as_longlong(__ldg(lt + 1));
    const unsigned long long aN = (unsigned long long)(N < 0 ? -N : N);
    const int pN = 63 - __clzll((long long)aN);
    const double lh = __longlong_as_double((long long)(((unsigned long long)(N < 0) << 63) |
                                                       ((unsigned long long)(981 + pN) << 52) |
                                                       ((aN << (52 - pN)) & 0xFFFFFFFFFFFFFull)));
    const double ll = __dadd_rn(__ldg(lt + 2), p);
    const double yh = __dmul_rn(b, lh);
    double yl = __fma_rn(b, lh, -yh);
    yl = __fma_rn(b, ll, yl);
    if ((__double2hiint(yh) & 0x7fffffff) >= 0x40800000) return pow(x, b);  // |yh| >= 512, or NaN
    const double t = __fma_rn(yh, 256.0, 6755399441055744.0);  // 1.5 * 2^52: round(256 yh) in the low word
    const int k = __double2loint(t);
    // k as a double (|k| <= 2^17) by integer operations
    const unsigned ak = (unsigned)(k < 0 ? -k : k);
    const int pk = 31 - __clz((int)ak);
    const double kd = ak == 0u ? 0.0
                               : __hiloint2double((int)(((unsigned)(k < 0) << 31) | ((unsigned)(1023 + pk) << 20) |
                                                        ((ak << (20 - pk)) & 0xfffffu)), 0);
    double f = __fma_rn(kd, -0.00390625, yh);
    f = __dadd_rn(f, yl);
    double q = __fma_rn(f, kE3, kE2);
    q = __fma_rn(f, q, kE1);
    q = __fma_rn(f, q, dpow_tail(f, (float)kE4, (float)kE5));
    const double E = __ldg(g_dpow_exp + (k & 255));
    const double res = __fma_rn(E, q, E);
    return __hiloint2double(__double2hiint(res) + (k >> 8) * 0x100000, __double2loint(res));
}

// x^b for |b| <= 1 from the exponent's own table (PowTab64, built on the host by
// make_pow_table): with x = 2^e m, j the top 8 bits of m's fraction and
// r = m inv_j - 1 as in dpow_tab,
//   x^b = [2^(e b) (1 / inv_j)^b] (1 + r)^b,
// the bracket a tabulated double-double T.x + T.y (64 exponents x 256 j, from
// the host's long double), (1 + r)^b - 1 = s by its binomial series to r^6
// (|r| <= 2^-9 and |b| <= 1: the r^7 term is below 2^-63), the terms to r^3
// in float64 and r^4 to r^6 in float32 (below 2^-36), and the result
// T.x + fma(T.x, s, T.y): one rounding of a value within 2^-60 of x^b, so
// within about half an ulp.  6 float64 operations.  x outside [2^-17, 2^47)
// (or not a positive normal number) and a null table take dpow_tab.
__device__ __forceinline__ double dpow_b(double x, double b, const PowTab64& P)
{
    const int hi = __double2hiint(x);
    const unsigned idx = (unsigned)((hi >> 12) - ((1023 + kPowEMin) << 8));
    if (P.t == nullptr || idx >= (unsigned)kPowTabN) return dpow_tab(x, b);
    const int j = (hi >> 12) & 0xff;
    const double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, __double2loint(x));
    const double r = __fma_rn(m, __ldg(g_dpow_log + 3 * j), -1.0);
    const float rf = dpow_tail_f(r);
    const float r2 = __fmul_rn(rf, rf);
    const float tail = __fmul_rn(__fmul_rn(r2, r2), __fadd_rn(P.c4, __fmul_rn(rf, __fadd_rn(P.c5, __fmul_rn(rf, P.c6)))));
    const double s = __fma_rn(r, __fma_rn(r, __fma_rn(r, P.c3, P.c2), b), dpow_tail_d(tail));
    const double2 T = __ldg(P.t + idx);
    return __dadd_rn(T.x, __fma_rn(T.x, s, T.y));
}

// Host: fills the tables on the current device (once per device).
cudaError_t upload_dpow_tables();

}  // namespace frg
