// Modified Bessel functions I0, I1, K0, K1 from the polynomial
// approximations of Abramowitz & Stegun 9.8.1-9.8.8, with the branch points
// of src/bessi0.f90, src/bessi1.f90, src/bessk0.f90, src/bessk1.f90 (K = 0
// beyond x = 500).  Accurate to about 1e-7: parity needs these, not exact
// Bessel functions.
#pragma once

namespace crgpu {

// ---------------------------------------------------------------------------
// modified Bessel functions: Abramowitz & Stegun 9.8.1-9.8.8 polynomial
// approximations, with the branch points the reference uses
// ---------------------------------------------------------------------------
__device__ __forceinline__ double as_i0(double x) {
    double ax = fabs(x);
    if (ax < 3.75) {  // 9.8.1
        double t = (x / 3.75) * (x / 3.75);
        return 1.0 + t * (3.5156229 + t * (3.0899424 + t * (1.2067492 +
               t * (0.2659732 + t * (0.0360768 + t * 0.0045813)))));
    }
    double u = 3.75 / ax;  // 9.8.2
    return (exp(ax) / sqrt(ax)) * (0.39894228 + u * (0.01328592 + u * (0.00225319 +
           u * (-0.00157565 + u * (0.00916281 + u * (-0.02057706 + u * (0.02635537 +
           u * (-0.01647633 + u * 0.00392377))))))));
}

__device__ __forceinline__ double as_i1(double x) {
    double ax = fabs(x);
    if (ax < 3.75) {  // 9.8.3
        double t = (x / 3.75) * (x / 3.75);
        return x * (0.5 + t * (0.87890594 + t * (0.51498869 + t * (0.15084934 +
               t * (0.02658733 + t * (0.00301532 + t * 0.00032411))))));
    }
    double u = 3.75 / ax;  // 9.8.4
    return (exp(ax) / sqrt(ax)) * (0.39894228 + u * (-0.03988024 + u * (-0.00362018 +
           u * (0.00163801 + u * (-0.01031555 + u * (0.02282967 + u * (-0.02895312 +
           u * (0.01787654 + u * -0.00420059))))))));
}

__device__ __forceinline__ double as_k0(double x) {
    if (x <= 2.0) {  // 9.8.5
        double t = x * x / 4.0;
        return (-log(x / 2.0) * as_i0(x)) + (-0.57721566 + t * (0.42278420 +
               t * (0.23069756 + t * (0.03488590 + t * (0.00262698 +
               t * (0.00010750 + t * 0.0000074))))));
    }
    if (x > 500.0) return 0.0;
    double u = 2.0 / x;  // 9.8.6
    return (exp(-x) / sqrt(x)) * (1.25331414 + u * (-0.07832358 + u * (0.02189568 +
           u * (-0.01062446 + u * (0.00587872 + u * (-0.00251540 + u * 0.00053208))))));
}

__device__ __forceinline__ double as_k1(double x) {
    if (x <= 2.0) {  // 9.8.7
        double t = x * x / 4.0;
        return (log(x / 2.0) * as_i1(x)) + (1.0 / x) * (1.0 + t * (0.15443144 +
               t * (-0.67278579 + t * (-0.18156897 + t * (-0.01919402 +
               t * (-0.00110404 + t * -0.00004686))))));
    }
    if (x > 500.0) return 0.0;
    double u = 2.0 / x;  // 9.8.8
    return (exp(-x) / sqrt(x)) * (1.25331414 + u * (0.23498619 + u * (-0.03655620 +
           u * (0.01504268 + u * (-0.00780353 + u * (0.00325614 + u * -0.00068245))))));
}


}  // namespace crgpu
