// rp_math.cuh -- FP64 vector / complex helpers for the GB300 tracing kernels.
//
// The plain path is compiled with --fmad=false and IEEE division/square root so
// that every real operation rounds exactly as the reference's C does
// (raypier/core/ctracer.pyx:83-262 for the vector helpers).  Where a reference
// expression contains an operation that is an identity up to the sign of a
// zero (a complex multiply by x + 0i, an addition of y*0.0), the cheaper form
// is written here: the FP64 pipe is the scarce resource on GB300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rp {

struct v3 {
    double x, y, z;
};

__device__ __forceinline__ v3 mkv(double x, double y, double z) {
    v3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__device__ __forceinline__ v3 addv(v3 a, v3 b) { return mkv(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 subv(v3 a, v3 b) { return mkv(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 mulvs(v3 a, double s) { return mkv(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ v3 negv(v3 a) { return mkv(-a.x, -a.y, -a.z); }
__device__ __forceinline__ double dotv(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double magsq(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ double magv(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ v3 crossv(v3 a, v3 b) {
    return mkv(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// norm_ (ctracer.pyx:249-254): three IEEE divisions by the magnitude.
__device__ __forceinline__ v3 normv(v3 a) {
    double m = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return mkv(a.x / m, a.y / m, a.z / m);
}
// Normalisation with one reciprocal instead of three divisions: within an ulp
// of norm_, used where the result is a direction / polarisation vector
// (materials, face normals) rather than a distance that selects a face.
__device__ __forceinline__ v3 normv_fast(v3 a) {
    double inv = 1.0 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return mkv(a.x * inv, a.y * inv, a.z * inv);
}
// sep_ (ctracer.pyx:108-113)
__device__ __forceinline__ double sepv(v3 p1, v3 p2) {
    double a = p2.x - p1.x, b = p2.y - p1.y, c = p2.z - p1.z;
    return sqrt((a * a) + (b * b) + (c * c));
}
// transform_c / rotate_c (ctracer.pyx:83-95); m row-major, t translation.
__device__ __forceinline__ v3 xform(const double *m, const double *t, v3 p) {
    return mkv(p.x * m[0] + p.y * m[1] + p.z * m[2] + t[0], p.x * m[3] + p.y * m[4] + p.z * m[5] + t[1],
               p.x * m[6] + p.y * m[7] + p.z * m[8] + t[2]);
}
__device__ __forceinline__ v3 rotv(const double *m, v3 p) {
    return mkv(p.x * m[0] + p.y * m[1] + p.z * m[2], p.x * m[3] + p.y * m[4] + p.z * m[5],
               p.x * m[6] + p.y * m[7] + p.z * m[8]);
}

// ---- integer powers -------------------------------------------------------
// x**k for a small non-negative integer k, rounded from a double-double
// product chain (Dekker / Ogita-Rump-Oishi TwoProduct with an explicit FMA).
// The result is the correctly rounded power except when the exact value lies
// within ~2^-100 relative of a rounding boundary, so it agrees with a libm
// pow() whose error is below one ulp in all but such hard cases.
struct dd {
    double hi, lo;
};
__device__ __forceinline__ dd dd_mul_d(dd a, double x) {
    double p = a.hi * x;
    double e = fma(a.hi, x, -p);
    double l = e + a.lo * x;
    double s = p + l;
    return dd{s, l - (s - p)};
}
__device__ __forceinline__ double ipow(double x, int k) {
    if (k == 0) return 1.0;
    dd a{x, 0.0};
    for (int i = 1; i < k; i++) a = dd_mul_d(a, x);
    return a.hi;
}
// Fills pw[0..kmax] with x**0 .. x**kmax from one product chain.
__device__ __forceinline__ void ipow_table(double x, int kmax, double *pw) {
    pw[0] = 1.0;
    if (kmax < 1) return;
    pw[1] = x;
    dd a{x, 0.0};
    for (int i = 2; i <= kmax; i++) {
        a = dd_mul_d(a, x);
        pw[i] = a.hi;
    }
}

// ---- complex numbers (double2: x = re, y = im) -----------------------------
typedef double2 cx;
__device__ __forceinline__ cx mkc(double re, double im) { return make_double2(re, im); }
__device__ __forceinline__ cx cadd(cx a, cx b) { return mkc(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cx csub(cx a, cx b) { return mkc(a.x - b.x, a.y - b.y); }
// C99 complex product as GCC emits it without -ffast-math: (ac - bd, ad + bc).
__device__ __forceinline__ cx cmul(cx a, cx b) { return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// Complex times (s + 0i): equals cmul(a, (s,0)) up to the sign of zero.
__device__ __forceinline__ cx cmuls(cx a, double s) { return mkc(a.x * s, a.y * s); }
// Complex division a / b = a conj(b) / |b|^2 with one reciprocal.  The
// operands here (refractive indices, Fresnel denominators) are of order one,
// far from the range where |b|^2 could overflow or underflow.
__device__ __forceinline__ cx cdiv(cx a, cx b) {
    double inv = 1.0 / (b.x * b.x + b.y * b.y);
    return mkc((a.x * b.x + a.y * b.y) * inv, (a.y * b.x - a.x * b.y) * inv);
}
// Principal complex square root (W. Kahan, "Branch cuts for complex elementary
// functions", 1987): t = sqrt((|x| + |z|)/2).
__device__ __forceinline__ cx csqrt_(cx z) {
    double x = z.x, y = z.y;
    if (x == 0.0 && y == 0.0) return mkc(0.0, y);
    double t = sqrt((fabs(x) + sqrt(x * x + y * y)) * 0.5);
    double h = 0.5 / t;
    if (x >= 0.0) return mkc(t, y * h);
    return mkc(fabs(y) * h, copysign(t, y));
}
// |z|^2 (the reference squares cabs(z))
__device__ __forceinline__ double cabs2_(cx z) { return z.x * z.x + z.y * z.y; }

__device__ __forceinline__ double inf_d() { return __longlong_as_double(0x7ff0000000000000LL); }
__device__ __forceinline__ double nan_d() { return __longlong_as_double(0x7ff8000000000000LL); }

}  // namespace rp
