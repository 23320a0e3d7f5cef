// Complex arithmetic for the kernels: double2 (complex128) and float2
// (complex64) with the reference's conventions -- principal-branch square
// root, textbook quotient (the reference is built with -ffast-math).
#pragma once

#include <cuda_runtime.h>

namespace crgpu {

__host__ __device__ __forceinline__ double2 cz(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ float2 cf(float r, float i) { return make_float2(r, i); }

// ----- complex128 -----
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cz(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return cz(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return cz(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// s - a*b with four fused multiply-adds
__device__ __forceinline__ double2 cfms(double2 s, double2 a, double2 b) {
    double re = fma(-a.x, b.x, s.x);
    re = fma(a.y, b.y, re);
    double im = fma(-a.x, b.y, s.y);
    im = fma(-a.y, b.x, im);
    return cz(re, im);
}
// 1 / d = conj(d) / |d|^2
__device__ __forceinline__ double2 crecip(double2 d) {
    double q = 1.0 / (d.x * d.x + d.y * d.y);
    return cz(d.x * q, -d.y * q);
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return cz(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    double d = b.x * b.x + b.y * b.y;
    return cz((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double cabsd(double2 a) { return sqrt(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ double2 csqrtd(double2 z) {
    double r = cabsd(z);
    if (r == 0.0) return cz(0.0, 0.0);
    if (z.x >= 0.0) {
        double t = sqrt(0.5 * (r + z.x));
        return cz(t, z.y / (2.0 * t));
    }
    double t = sqrt(0.5 * (r - z.x));
    return cz(fabs(z.y) / (2.0 * t), copysign(t, z.y));
}
__device__ __forceinline__ double2 cconj(double2 a) { return cz(a.x, -a.y); }

// ----- complex64 -----
__device__ __forceinline__ float2 caddf(float2 a, float2 b) { return cf(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csubf(float2 a, float2 b) { return cf(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return cf(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cfmsf(float2 s, float2 a, float2 b) {
    // s - a*b with fused multiply-adds
    float re = fmaf(-a.x, b.x, s.x);
    re = fmaf(a.y, b.y, re);
    float im = fmaf(-a.x, b.y, s.y);
    im = fmaf(-a.y, b.x, im);
    return cf(re, im);
}
__device__ __forceinline__ float2 cfmaf(float2 s, float2 a, float2 b) {
    // s + a*b
    float re = fmaf(a.x, b.x, s.x);
    re = fmaf(-a.y, b.y, re);
    float im = fmaf(a.x, b.y, s.y);
    im = fmaf(a.y, b.x, im);
    return cf(re, im);
}
__device__ __forceinline__ float2 crecipf(float2 d) {
    float q = 1.0f / (d.x * d.x + d.y * d.y);
    return cf(d.x * q, -d.y * q);
}
__device__ __forceinline__ float2 cdivf(float2 a, float2 b) {
    float d = b.x * b.x + b.y * b.y;
    return cf((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ float cabsf_(float2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ float2 csqrtf_(float2 z) {
    float r = cabsf_(z);
    if (r == 0.0f) return cf(0.0f, 0.0f);
    if (z.x >= 0.0f) {
        float t = sqrtf(0.5f * (r + z.x));
        return cf(t, z.y / (2.0f * t));
    }
    float t = sqrtf(0.5f * (r - z.x));
    return cf(fabsf(z.y) / (2.0f * t), copysignf(t, z.y));
}

__device__ __forceinline__ float2 to_f(double2 a) { return cf((float)a.x, (float)a.y); }
__device__ __forceinline__ double2 to_d(float2 a) { return cz((double)a.x, (double)a.y); }

}  // namespace crgpu
