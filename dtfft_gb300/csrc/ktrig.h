// Compile-time cos / sin of 2*pi*e/n for the constant twiddles of the
// in-register DFT codelets (fft_2f.cuh).  Plain C++ (no CUDA), evaluated by
// the compiler: the angle is reduced exactly on the integer fraction e/n to an
// octant, then the Taylor series of sin and cos are summed on |x| <= pi/4,
// where 13 terms leave a truncation error below 1e-22.
#pragma once

namespace gb {
namespace ktrig {

constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double sin_series(double x) {
    const double x2 = x * x;
    double term = x, sum = x;
    for (int k = 1; k <= 13; ++k) {
        term *= -x2 / (double)((2 * k) * (2 * k + 1));
        sum += term;
    }
    return sum;
}

constexpr double cos_series(double x) {
    const double x2 = x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 13; ++k) {
        term *= -x2 / (double)((2 * k - 1) * (2 * k));
        sum += term;
    }
    return sum;
}

// (cos, sin) of 2*pi*e/n
struct CS { double c, s; };

constexpr CS cs2pi(long long e, long long n) {
    e %= n;
    if (e < 0) e += n;
    // 8e = o*n + r: angle = o*pi/4 + (pi/4)(r/n), 0 <= r < n
    const long long o = (8 * e) / n, r = 8 * e - o * n;
    const double x = (kPi / 4) * ((double)r / (double)n);
    double c = 0, s = 0;   // of the angle inside its quadrant, phi in [0, pi/2)
    if (o % 2 == 0) {
        c = cos_series(x);
        s = sin_series(x);
    } else {                       // phi = pi/4 + x = pi/2 - y
        const double y = (kPi / 4) * ((double)(n - r) / (double)n);
        c = sin_series(y);
        s = cos_series(y);
    }
    switch (o / 2) {               // rotate by the quadrant
    case 0: return CS{c, s};
    case 1: return CS{-s, c};
    case 2: return CS{-c, -s};
    default: return CS{s, -c};
    }
}

constexpr double cos2pi(long long e, long long n) { return cs2pi(e, n).c; }
constexpr double sin2pi(long long e, long long n) { return cs2pi(e, n).s; }

}  // namespace ktrig
}  // namespace gb
