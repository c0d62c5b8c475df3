// fft_codelets.cuh -- register-resident DFT codelets of compile-time size.
//
// Dft<N, SIGN>::run(v) replaces v[0..N) by X[k] = sum_n v[n] exp(SIGN*2*pi*i*n*k/N)
// (FFTW's sign convention: SIGN = -1 forward, +1 backward, unnormalised).
// Composite sizes split recursively (Cooley-Tukey, radix 4 first, then the
// smallest prime factor); odd primes use the symmetric direct form.  All
// indices and twiddles are compile-time constants, so the arrays stay in
// registers.
#pragma once
#include "cgs_common.cuh"

namespace cgs {

template <int N, int SIGN>
struct Dft;

template <int SIGN>
struct Dft<1, SIGN> {
    static CGS_D void run(float2 (&)[1]) {}
};

template <int SIGN>
struct Dft<2, SIGN> {
    static CGS_D void run(float2 (&v)[2])
    {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <int SIGN>
struct Dft<4, SIGN> {
    static CGS_D void run(float2 (&v)[4])
    {
        const float2 t0 = cadd(v[0], v[2]);
        const float2 t1 = csub(v[0], v[2]);
        const float2 t2 = cadd(v[1], v[3]);
        const float2 d = csub(v[1], v[3]);
        // t3 = SIGN * i * d
        const float2 t3 = (SIGN < 0) ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    }
};

// Odd prime N: X_k = x0 + sum_{n=1}^{(N-1)/2} [ (x_n + x_{N-n}) cos(2 pi n k / N)
//                                            + SIGN i (x_n - x_{N-n}) sin(2 pi n k / N) ]
template <int N, int SIGN>
CGS_D void dft_odd_prime(float2 (&v)[N])
{
    constexpr int H = (N - 1) / 2;
    float2 s[H + 1], d[H + 1];
    float2 x0 = v[0];
    float2 sum = v[0];
    static_for<1, H + 1>([&](auto n_) {
        constexpr int n = decltype(n_)::value;
        s[n] = cadd(v[n], v[N - n]);
        d[n] = csub(v[n], v[N - n]);
        sum = cadd(sum, s[n]);
    });
    v[0] = sum;
    static_for<1, H + 1>([&](auto k_) {
        constexpr int k = decltype(k_)::value;
        float cr = x0.x, ci = x0.y;   // cosine part
        float sr = 0.f, si = 0.f;      // sine part (times i applied below)
        static_for<1, H + 1>([&](auto n_) {
            constexpr int n = decltype(n_)::value;
            constexpr float c = (float)ccos((long long)n * k, N);
            constexpr float sn = (float)csin((long long)n * k, N);
            cr += s[n].x * c;
            ci += s[n].y * c;
            sr += d[n].x * sn;
            si += d[n].y * sn;
        });
        // SIGN * i * (sr + i si) = SIGN * (-si + i sr)
        const float tr = (SIGN < 0) ? si : -si;
        const float ti = (SIGN < 0) ? -sr : sr;
        v[k] = make_float2(cr + tr, ci + ti);
        v[N - k] = make_float2(cr - tr, ci - ti);
    });
}

constexpr int split_factor(int n)
{
    return (n % 4 == 0 && n > 4) ? 4 : smallest_factor(n);
}

template <int N, int SIGN>
struct Dft {
    static CGS_D void run(float2 (&v)[N])
    {
        constexpr int p = split_factor(N);
        if constexpr (p == N) {
            dft_odd_prime<N, SIGN>(v);
        } else {
            constexpr int q = N / p;
            // n = q*n1 + n2, k = k1 + p*k2
            float2 t[N];
            static_for<0, q>([&](auto n2_) {
                constexpr int n2 = decltype(n2_)::value;
                float2 a[p];
                static_for<0, p>([&](auto n1_) {
                    constexpr int n1 = decltype(n1_)::value;
                    a[n1] = v[q * n1 + n2];
                });
                Dft<p, SIGN>::run(a);
                static_for<0, p>([&](auto k1_) {
                    constexpr int k1 = decltype(k1_)::value;
                    t[n2 * p + k1] = twiddle_const<SIGN, n2 * k1, N>(a[k1]);
                });
            });
            static_for<0, p>([&](auto k1_) {
                constexpr int k1 = decltype(k1_)::value;
                float2 b[q];
                static_for<0, q>([&](auto n2_) {
                    constexpr int n2 = decltype(n2_)::value;
                    b[n2] = t[n2 * p + k1];
                });
                Dft<q, SIGN>::run(b);
                static_for<0, q>([&](auto k2_) {
                    constexpr int k2 = decltype(k2_)::value;
                    v[k1 + p * k2] = b[k2];
                });
            });
        }
    }
};

// Dft<N, SIGN> of a vector whose entries outside [N/4, 3N/4) are zero (the
// zero-padded half of a 2x oversampled line), N a multiple of 4.  With the
// radix-4 first level n = q n1 + n2 (q = N/4) the non-zero inputs are
// n1 = 1, 2, and each 4-point DFT of (0, a, b, 0),
//   X_0 = a + b,  X_1 = SIGN i a - b,  X_2 = b - a,  X_3 = -SIGN i a - b,
// takes four complex additions instead of eight (an addition of a zero is
// not removed by the compiler, as x + 0 differs from x for x = -0).  The
// results equal Dft<N, SIGN>'s up to the sign of zeros.
template <int SIGN>
CGS_D void dft4_mid(float2 a, float2 b, float2 (&o)[4])
{
    const float2 ia = (SIGN < 0) ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);   // SIGN i a
    o[0] = cadd(a, b);
    o[1] = csub(ia, b);
    o[2] = csub(b, a);
    o[3] = make_float2(-ia.x - b.x, -ia.y - b.y);
}

template <int N, int SIGN>
struct DftMid {
    static_assert(N % 4 == 0, "the zero pattern needs N % 4 == 0");
    static CGS_D void run(float2 (&v)[N])
    {
        constexpr int q = N / 4;
        if constexpr (q == 1) {
            float2 o[4];
            dft4_mid<SIGN>(v[1], v[2], o);
            static_for<0, 4>([&](auto k_) {
                constexpr int k = decltype(k_)::value;
                v[k] = o[k];
            });
        } else {
            float2 t[N];
            static_for<0, q>([&](auto n2_) {
                constexpr int n2 = decltype(n2_)::value;
                float2 a[4];
                dft4_mid<SIGN>(v[q + n2], v[2 * q + n2], a);
                static_for<0, 4>([&](auto k1_) {
                    constexpr int k1 = decltype(k1_)::value;
                    t[n2 * 4 + k1] = twiddle_const<SIGN, n2 * k1, N>(a[k1]);
                });
            });
            static_for<0, 4>([&](auto k1_) {
                constexpr int k1 = decltype(k1_)::value;
                float2 b[q];
                static_for<0, q>([&](auto n2_) {
                    constexpr int n2 = decltype(n2_)::value;
                    b[n2] = t[n2 * 4 + k1];
                });
                Dft<q, SIGN>::run(b);
                static_for<0, q>([&](auto k2_) {
                    constexpr int k2 = decltype(k2_)::value;
                    v[k1 + 4 * k2] = b[k2];
                });
            });
        }
    }
};

}  // namespace cgs
