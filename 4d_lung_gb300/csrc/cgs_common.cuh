// cgs_common.cuh -- shared device helpers for the CG-SENSE kernels (sm_103a).
//
// Complex values are float2 (re, im), bit-compatible with fftwf_complex, the
// element type of every grid, image and sample buffer of the reference
// (Reco.h:77-91).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include <utility>

#define CGS_HD __host__ __device__ __forceinline__
#define CGS_D __device__ __forceinline__

namespace cgs {

CGS_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
CGS_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
CGS_HD float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
CGS_HD float2 cmulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
CGS_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
CGS_HD float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }

// CG vector updates (addToArrayScaled / addArraysScaled, Reco.cpp:153-173)
// with the step size (ar, ai) rounded to float.  Every product and sum is
// rounded on its own (no fused multiply-add), so that the separate update
// kernels and the forward z pass that applies the same updates in a fused
// solve store the same bits.
// y + a v
CGS_D float2 cg_axpy(float2 y, float ar, float ai, float2 v)
{
    const float re = __fsub_rn(__fmul_rn(ar, v.x), __fmul_rn(ai, v.y));
    const float im = __fadd_rn(__fmul_rn(ar, v.y), __fmul_rn(ai, v.x));
    return make_float2(__fadd_rn(y.x, re), __fadd_rn(y.y, im));
}
// y - a v
CGS_D float2 cg_axmy(float2 y, float ar, float ai, float2 v)
{
    const float re = __fsub_rn(__fmul_rn(ar, v.x), __fmul_rn(ai, v.y));
    const float im = __fadd_rn(__fmul_rn(ar, v.y), __fmul_rn(ai, v.x));
    return make_float2(__fsub_rn(y.x, re), __fsub_rn(y.y, im));
}

// ---------------------------------------------------------------------------
// Compile-time helpers
// ---------------------------------------------------------------------------

template <int Begin, int End, class F>
CGS_D void static_for(F&& f)
{
    if constexpr (Begin < End) {
        f(std::integral_constant<int, Begin>{});
        static_for<Begin + 1, End>(f);
    }
}

constexpr int smallest_factor(int n)
{
    for (int p = 2; p * p <= n; ++p)
        if (n % p == 0) return p;
    return n;
}

// cos(2*pi*m/n) and sin(2*pi*m/n) evaluated at compile time by their Taylor
// series after reducing the angle to [-pi, pi]; used only for codelet
// constants, which are then rounded to float.
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double taylor_cos(double x)
{
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 40; ++k) {
        term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
        sum += term;
    }
    return sum;
}
constexpr double taylor_sin(double x)
{
    double term = x, sum = x;
    for (int k = 1; k < 40; ++k) {
        term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
        sum += term;
    }
    return sum;
}
constexpr double reduced_angle(long long m, long long n)
{
    long long r = m % n;
    if (r < 0) r += n;
    // angle in (-pi, pi]
    if (2 * r > n) r -= n;
    return 2.0 * kPi * (double)r / (double)n;
}
constexpr double ccos(long long m, long long n) { return taylor_cos(reduced_angle(m, n)); }
constexpr double csin(long long m, long long n) { return taylor_sin(reduced_angle(m, n)); }

// v * exp(SIGN * 2*pi*i * M / N) with compile-time constants; the trivial
// multiples of pi/2 are handled without multiplications.
template <int SIGN, int M, int N>
CGS_D float2 twiddle_const(float2 v)
{
    constexpr int m = ((M % N) + N) % N;
    if constexpr (m == 0) {
        return v;
    } else if constexpr (2 * m == N) {
        return cneg(v);
    } else if constexpr (4 * m == N) {
        // multiply by SIGN * i
        return (SIGN < 0) ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
    } else if constexpr (4 * m == 3 * N) {
        return (SIGN < 0) ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
    } else {
        constexpr float c = (float)ccos(m, N);
        constexpr float s = (float)(SIGN * csin(m, N));
        return make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
    }
}

}  // namespace cgs
