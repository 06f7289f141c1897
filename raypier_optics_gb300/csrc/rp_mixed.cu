// rp_mixed.cu -- the mixed-precision generation kernel.
//
// GB300 runs FP64 arithmetic, and every conversion instruction between double
// and float, at about 1/64 of its FP32 rate, so this kernel keeps the FP64 pipe
// almost idle and splits the work by what precision it needs:
//
//   float-float (a pair of floats, about 48 significant bits)
//         ray origins and hit points, the face-list-frame origin and direction,
//         the ray parameter of a hit, Euclidean lengths and the optical path.
//         A hit on a curved face is found in FP32 and then corrected by a
//         Newton step whose residual is evaluated at the float-float ray point
//         (relative to the face vertex, where FP32 resolves well below a
//         nanometre), so roots reach float-float accuracy without FP64.
//   FP32  directions of children, face normals, the S/P projection, Fresnel
//         coefficients, polarisation amplitudes and E-vectors, Snell's law,
//         aperture and shape tests, the asphere Newton iterations.
//   integer pipe
//         every conversion between the double-precision ray records and
//         float / float-float (bit manipulation instead of F2F instructions).
//   FP64  one addition per stored origin coordinate, length and optical path
//         (float-float -> double); the faces and materials this kernel does not
//         specialise (distortion, extended polynomial, polygons, elliptical
//         plane; partial mirror, polarisers, waveplate, apertures) reuse the
//         plain path's FP64 device functions.
//
// The TU is compiled with FMA contraction on.  Index fields agree with the
// FP64 oracle except for rays that graze an aperture edge or a face, which is
// why parity for this path is statistical (see the precision report).
#include <cuda_fp16.h>
#include <map>
#include <mutex>
#include <tuple>

#include "rp_gen_common.cuh"

namespace rp {
namespace mx {

// ---- float-float arithmetic ------------------------------------------------
// Error-free transforms: TwoSum (Knuth), Fast2Sum (Dekker), the FMA product.
// The double-word operations follow Joldes, Muller & Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word arithmetic",
// ACM TOMS 44(2), 2017 (DWPlusDW, DWPlusFP, DWTimesDW, DWTimesFP).
struct ff {
    float hi, lo;
};
__device__ __forceinline__ ff ffm(float hi, float lo) {
    ff r;
    r.hi = hi;
    r.lo = lo;
    return r;
}
__device__ __forceinline__ ff two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    return ffm(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    float s = a + b;
    return ffm(s, b - (s - a));
}
__device__ __forceinline__ ff two_prod(float a, float b) {
    float p = a * b;
    return ffm(p, fmaf(a, b, -p));
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ffm(-a.hi, -a.lo); }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    ff p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
// a / b: FP32 quotient, float-float residual, one correction
__device__ __forceinline__ ff ff_div(ff a, ff b) {
    float q1 = __fdividef(a.hi, b.hi);
    ff r = ff_sub(a, ff_mul_f(b, q1));
    return fast_two_sum(q1, __fdividef(r.hi, b.hi));
}
__device__ __forceinline__ ff ff_sqrt(ff a) {
    if (!(a.hi > 0.0f)) return ffm(sqrtf(a.hi), 0.0f);
    float s = sqrtf(a.hi);
    ff e = ff_sub(a, two_prod(s, s));
    return fast_two_sum(s, e.hi * (0.5f / s));
}
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool ff_eq(ff a, ff b) { return a.hi == b.hi && a.lo == b.lo; }

struct ff3 {
    ff x, y, z;
};
__device__ __forceinline__ ff3 mkff3(ff x, ff y, ff z) {
    ff3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__device__ __forceinline__ ff ff_dot3(const ff3 &a, const ff3 &b) {
    return ff_add(ff_add(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}
__device__ __forceinline__ ff3 ff3_scale(const ff3 &a, ff s) { return mkff3(ff_mul(a.x, s), ff_mul(a.y, s), ff_mul(a.z, s)); }
__device__ __forceinline__ ff3 ff3_sub(const ff3 &a, const ff3 &b) {
    return mkff3(ff_sub(a.x, b.x), ff_sub(a.y, b.y), ff_sub(a.z, b.z));
}
__device__ __forceinline__ ff3 ff3_neg(const ff3 &a) { return mkff3(ff_neg(a.x), ff_neg(a.y), ff_neg(a.z)); }
__device__ __forceinline__ ff3 ff3_unit(const ff3 &a) {
    return ff3_scale(a, ff_div(ffm(1.0f, 0.0f), ff_sqrt(ff_dot3(a, a))));
}

// ---- conversions on the integer pipe ---------------------------------------
// double -> float, round to nearest even; magnitudes below 2^-126 flush to a
// signed zero, above the float range to infinity.
__device__ __forceinline__ float f_of_d(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned s = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;  // exponent re-biased for float
    unsigned r = ((unsigned)e << 23) + (((hi & 0xfffffu) << 3) | (lo >> 29));
    const unsigned rest = lo & 0x1fffffffu;
    r += (unsigned)(rest > 0x10000000u) | ((unsigned)(rest == 0x10000000u) & (r & 1u));
    if (e <= 0) r = 0u;
    else if (e >= 255) r = (((hi & 0x7ff00000u) == 0x7ff00000u) && (((hi & 0xfffffu) | lo) != 0u)) ? 0x7fc00000u : 0x7f800000u;
    return __uint_as_float(s | r);
}
// float -> double, exact; float subnormals flush to a signed zero.
__device__ __forceinline__ double d_of_f(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned hi = s | ((e + 896u) << 20) | (m >> 3), lo = m << 29;
    if (e == 0u) {
        hi = s;
        lo = 0u;
    } else if (e == 255u) {
        hi = s | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u);
    }
    return __hiloint2double((int)hi, (int)lo);
}
// double -> float-float: the top 24 significant bits and the remaining 29 bits
// rounded to a float (about 48 bits in all), renormalised.  Magnitudes outside
// [2^-74, 2^128) keep only the rounded float.
__device__ __forceinline__ ff ff_of_d(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int E = (int)((hi >> 20) & 0x7ffu) - 1023;
    if (E < -74 || E > 127) return ffm(f_of_d(x), 0.0f);
    const unsigned s = hi & 0x80000000u;
    const float h = __uint_as_float(s | ((unsigned)(E + 127) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
    float l = __uint2float_rn(lo & 0x1fffffffu) * __uint_as_float((unsigned)(E + 75) << 23);
    return fast_two_sum(h, s ? -l : l);
}
// float-float -> double: hi + lo is exact in double (one FP64 addition)
__device__ __forceinline__ double d_of_ff(ff a) { return d_of_f(a.hi) + d_of_f(a.lo); }

// ---- FP32 vectors and complex numbers ----------------------------------------
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 mul3(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 norm3(f3 a) { return mul3(a, rsqrtf(dot3(a, a))); }
__device__ __forceinline__ f3 f3_of_d(double x, double y, double z) { return mk3(f_of_d(x), f_of_d(y), f_of_d(z)); }

typedef float2 cf;
__device__ __forceinline__ cf cfm(float r, float i) { return make_float2(r, i); }
__device__ __forceinline__ cf cadd(cf a, cf b) { return cfm(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cf csub(cf a, cf b) { return cfm(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ cf cmul(cf a, cf b) { return cfm(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cf cmuls(cf a, float s) { return cfm(a.x * s, a.y * s); }
__device__ __forceinline__ cf cdiv(cf a, cf b) {
    float inv = 1.0f / (b.x * b.x + b.y * b.y);
    return cfm((a.x * b.x + a.y * b.y) * inv, (a.y * b.x - a.x * b.y) * inv);
}
__device__ __forceinline__ cf csqrtf_(cf z) {  // Kahan's principal square root, as the FP64 path
    float x = z.x, y = z.y;
    if (x == 0.0f && y == 0.0f) return cfm(0.0f, y);
    float t = sqrtf((fabsf(x) + sqrtf(x * x + y * y)) * 0.5f);
    float h = 0.5f / t;
    if (x >= 0.0f) return cfm(t, y * h);
    return cfm(fabsf(y) * h, copysignf(t, y));
}
__device__ __forceinline__ float cabs2(cf z) { return z.x * z.x + z.y * z.y; }
__device__ __forceinline__ cf cf_of_d(double2 z) { return cfm(f_of_d(z.x), f_of_d(z.y)); }

// ---- per-block tables ----------------------------------------------------------
// A face list's maps in the forms used here, as float-float: global -> local
// (rotation and translation) and the local -> global rotation for normals,
// with a flag for an identity rotation.
struct MxList {
    float ri_hi[9], ri_lo[9];
    float ti_hi[3], ti_lo[3];
    float r_hi[9], r_lo[9];
    int ident;
    int pad[1];
};
// A face's parameters in FP32, its plane / vertex height as float-float and its
// smallest accepted ray parameter (tolerance * max_length, the reference's
// h < tolerance test with h = t / max_length).
struct MxFace {
    float p[RP_FACE_NPARAM];
    float zv_hi, zv_lo;
    float rq_hi, rq_lo;  // the quadric's Rq as float-float (sphere: -curvature; conic, asphere: -p[0])
    float ic_hi, ic_lo;  // a sphere's 1 / curvature as float-float (its unit normal is (p - centre) / c)
    float tmin;
    float tol;   // Face.tolerance (a distance) in FP32
    float btol;  // DistortionFace: its base face's tolerance (a fraction of the segment)
    int spec;    // 1: the face is tested here (face_t32), 0: by the FP64 path
};

__host__ __device__ __forceinline__ size_t mx_tables_bytes(int n_lists, int n_faces) {
    return (size_t)n_lists * sizeof(MxList) + (size_t)n_faces * sizeof(MxFace);
}

// Index of the parameter that holds the plane height / vertex z of each face type.
__device__ __forceinline__ int vertex_param(int type) {
    switch (type) {
        case RP_FACE_CIRCULAR: return 2;
        case RP_FACE_RECTANGULAR: return 3;
        case RP_FACE_SHAPED_PLANAR: return 0;
        case RP_FACE_SPHERICAL: return 2;
        case RP_FACE_SHAPED_SPHERICAL: return 1;
        case RP_FACE_CONIC: return 1;
        case RP_FACE_ASPHERIC: return 1;
        case RP_FACE_EXTPOLY: return 3;
        default: return -1;
    }
}

// A DistortionFace the mixed path tests itself: a ShapedPlanarFace base and a
// distortion with an FP32 table (or the closed-form J7 test distortion); the
// scene set-up makes the same test when it boxes the face for this path.
__device__ __forceinline__ bool mx_distortion_ok(const DevScene &S, const rp_face &F) {
    if (F.base < 0 || F.base >= S.n_recs || F.distortion < 0 || F.distortion >= S.n_dists) return false;
    if (S.faces[F.base].type != RP_FACE_SHAPED_PLANAR) return false;
    const rp_distortion &D = S.dists[F.distortion];
    return D.type == RP_DIST_SIMPLE_J7 || (S.zk32_off && S.zk32_off[F.distortion] >= 0);
}

__device__ __forceinline__ float zk_horner(const float *c, int n, float r) {
    float v = c[n - 1];
    for (int k = n - 2; k >= 0; k--) v = fmaf(v, r, c[k]);
    return v;
}

// A distortion at local (x, y) in FP32: z as ZernikeDistortion.z_offset_c
// (cdistortions.pyx:416-450), or with grad (dz/dx, dz/dy, z) as
// z_offset_and_gradient_c (456-514); SimpleTestZernikeJ7 in closed form
// (48-81).  Zernike distortions use their polynomial table (the groups in
// ascending |m|: cos / sin of m theta step up by the Chebyshev recurrence).
// The distortion is a small height (N(0, 0.5 um) coefficients on the
// clutter workload), so FP32 resolves it to far below a picometre.
__device__ __noinline__ void zk_eval32(const DevScene &S, int dist, float x, float y, bool grad, float &zx, float &zy,
                                       float &z) {
    const rp_distortion &D = S.dists[dist];
    zx = 0.0f;
    zy = 0.0f;
    z = 0.0f;
    if (D.type == RP_DIST_SIMPLE_J7) {
        const float R = f_of_d(D.unit_radius), a = 2.8284271247461903f * f_of_d(D.amplitude);  // sqrt(8) A
        x /= R;
        y /= R;
        z = a * (3.0f * (x * x + y * y) - 2.0f) * y;
        zx = a * 6.0f * x * y / R;
        zy = a * (3.0f * x * x + 9.0f * y * y - 2.0f) / R;
        return;
    }
    const float *T = S.zk32 + S.zk32_off[dist];
    const int ng = (int)T[0], st = (int)T[1];
    const float iur = T[3];
    x *= iur;
    y *= iur;
    const float r = sqrtf(x * x + y * y);
    float ct, sn;
    if (r > 0.0f) {
        ct = x / r;
        sn = y / r;
    } else {
        sincosf(atan2f(y, x), &sn, &ct);  // the reference's atan2 of signed zeros
    }
    float cp = ct, sp = -sn, cc = 1.0f, sc = 0.0f;  // cos / sin of (k - 1) theta and k theta
    int k = 0;
    const float *g = T + 4;
    for (int i = 0; i < ng; i++, g += 4 + 4 * st) {
        const int m = (int)g[0], kind = (int)g[1];
        for (; k < m; k++) {
            const float cn = 2.0f * ct * cc - cp, sn2 = 2.0f * ct * sc - sp;
            cp = cc;
            sp = sc;
            cc = cn;
            sc = sn2;
        }
        const float A = kind ? sc : cc;                            // cos(m theta) or sin(|m| theta)
        const float Ad = kind ? (float)m * cc : -(float)m * sc;   // its derivative in theta
        const float *P = g + 4;
        if (!grad) {
            z = fmaf(zk_horner(P, st, r), A, z);
            continue;
        }
        const float G = zk_horner(P + st, st, r), Q = zk_horner(P + 2 * st, st, r), W = zk_horner(P + 3 * st, st, r);
        z = fmaf(G, A, z);
        zx += Q * ct * A - W * sn * Ad;
        zy += Q * sn * A + W * ct * Ad;
    }
    zx *= iur;
    zy *= iur;
}

// zk_eval32 in FP64 over the FP64 tables (Zernike distortions with a table).
__device__ void zk_eval64(const DevScene &S, int dist, double x, double y, bool grad, double &zx, double &zy,
                          double &z) {
    zx = 0.0;
    zy = 0.0;
    z = 0.0;
    const double *T = S.zk64 + S.zk32_off[dist];
    const int ng = (int)T[0], st = (int)T[1];
    const double iur = T[3];
    x *= iur;
    y *= iur;
    const double r = sqrt(x * x + y * y);
    double ct, sn;
    polar_cs(x, y, r, ct, sn);
    double cp = ct, sp = -sn, cc = 1.0, sc = 0.0;
    int k = 0;
    const double *g = T + 4;
    for (int i = 0; i < ng; i++, g += 4 + 4 * st) {
        const int m = (int)g[0], kind = (int)g[1];
        for (; k < m; k++) {
            const double cn = 2.0 * ct * cc - cp, sn2 = 2.0 * ct * sc - sp;
            cp = cc;
            sp = sc;
            cc = cn;
            sc = sn2;
        }
        const double A = kind ? sc : cc, Ad = kind ? (double)m * cc : -(double)m * sc;
        const double *P = g + 4;
        auto horner = [&](const double *c) {
            double v = c[st - 1];
            for (int q = st - 2; q >= 0; q--) v = fma(v, r, c[q]);
            return v;
        };
        if (!grad) {
            z += horner(P) * A;
            continue;
        }
        const double G = horner(P + st), Q = horner(P + 2 * st), W = horner(P + 3 * st);
        z += G * A;
        zx += Q * ct * A - W * sn * Ad;
        zy += Q * sn * A + W * ct * Ad;
    }
    zx *= iur;
    zy *= iur;
}

// Fills the tables from the FP64 tables in global memory (the shared copies of
// those are not complete until the caller's next barrier).
__device__ __forceinline__ void stage_mixed(const GenArgs &A, MxList *ml, MxFace *mf, float max_len) {
    for (int l = threadIdx.x; l < A.S.n_lists; l += blockDim.x) {
        const rp_facelist &L = A.S.lists[l];
        MxList &o = ml[l];
        for (int k = 0; k < 9; k++) {
            ff v = ff_of_d(L.inv_trans.m[k]);
            o.ri_hi[k] = v.hi;
            o.ri_lo[k] = v.lo;
            ff w = ff_of_d(L.trans.m[k]);
            o.r_hi[k] = w.hi;
            o.r_lo[k] = w.lo;
        }
        for (int k = 0; k < 3; k++) {
            ff v = ff_of_d(L.inv_trans.t[k]);
            o.ti_hi[k] = v.hi;
            o.ti_lo[k] = v.lo;
        }
        const double *m = L.inv_trans.m;
        const double *w = L.trans.m;
        o.ident = (m[0] == 1.0 && m[4] == 1.0 && m[8] == 1.0 && m[1] == 0.0 && m[2] == 0.0 && m[3] == 0.0 &&
                   m[5] == 0.0 && m[6] == 0.0 && m[7] == 0.0) &&
                  (w[0] == 1.0 && w[4] == 1.0 && w[8] == 1.0 && w[1] == 0.0 && w[2] == 0.0 && w[3] == 0.0 &&
                   w[5] == 0.0 && w[6] == 0.0 && w[7] == 0.0);
    }
    for (int f = threadIdx.x; f < A.S.n_faces; f += blockDim.x) {
        const rp_face &F = A.S.faces[f];
        MxFace &o = mf[f];
        for (int k = 0; k < RP_FACE_NPARAM; k++) o.p[k] = f_of_d(F.p[k]);
        int vp = vertex_param(F.type);
        ff z = vp >= 0 ? ff_of_d(F.p[vp]) : ffm(0.0f, 0.0f);
        o.spec = vp >= 0 ? 1 : 0;
        o.btol = 0.0f;
        if (F.type == RP_FACE_DISTORTION && mx_distortion_ok(A.S, F)) {
            const rp_face &Bf = A.S.faces[F.base];
            z = ff_of_d(Bf.p[0]);  // the ShapedPlanarFace base's z_height
            o.btol = f_of_d(Bf.tolerance);
            o.spec = 1;
        }
        o.zv_hi = z.hi;
        o.zv_lo = z.lo;
        double rq = 0.0;
        if (F.type == RP_FACE_SPHERICAL) rq = -F.p[1];
        else if (F.type == RP_FACE_SHAPED_SPHERICAL) rq = -F.p[0];
        else if (F.type == RP_FACE_CONIC || F.type == RP_FACE_ASPHERIC) rq = -F.p[0];
        else if (F.type == RP_FACE_EXTPOLY) rq = F.p[0];  // extpoly_t.R (cfaces.pyx:2030)
        const ff r = ff_of_d(rq);
        o.rq_hi = r.hi;
        o.rq_lo = r.lo;
        const bool sph = F.type == RP_FACE_SPHERICAL || F.type == RP_FACE_SHAPED_SPHERICAL;
        const ff ic = sph && rq != 0.0 ? ff_of_d(-1.0 / rq) : ffm(0.0f, 0.0f);
        o.ic_hi = ic.hi;
        o.ic_lo = ic.lo;
        o.tmin = f_of_d(F.tolerance) * max_len;
        o.tol = f_of_d(F.tolerance);
    }
}

// ---- rays in a face list's frame ---------------------------------------------
struct LRay {
    ff px, py, pz;  // origin
    ff dx, dy, dz;  // direction (the world direction rotated; not renormalised)
};

__device__ __forceinline__ ff ff_of(const float *hi, const float *lo, int k) { return ffm(hi[k], lo[k]); }

// v' = R v (+ t), float-float
__device__ __forceinline__ void ff_rotate(const MxList &L, const ff v[3], ff out[3], bool translate) {
#pragma unroll
    for (int r = 0; r < 3; r++) {
        ff acc = ff_mul(ff_of(L.ri_hi, L.ri_lo, 3 * r), v[0]);
        acc = ff_add(acc, ff_mul(ff_of(L.ri_hi, L.ri_lo, 3 * r + 1), v[1]));
        acc = ff_add(acc, ff_mul(ff_of(L.ri_hi, L.ri_lo, 3 * r + 2), v[2]));
        if (translate) acc = ff_add(acc, ff_of(L.ti_hi, L.ti_lo, r));
        out[r] = acc;
    }
}

__device__ __forceinline__ LRay local_ray(const MxList &L, const ff O[3], const ff D[3]) {
    LRay R;
    if (L.ident) {
        R.px = ff_add(O[0], ff_of(L.ti_hi, L.ti_lo, 0));
        R.py = ff_add(O[1], ff_of(L.ti_hi, L.ti_lo, 1));
        R.pz = ff_add(O[2], ff_of(L.ti_hi, L.ti_lo, 2));
        R.dx = D[0];
        R.dy = D[1];
        R.dz = D[2];
    } else {
        ff p[3], d[3];
        ff_rotate(L, O, p, true);
        ff_rotate(L, D, d, false);
        R.px = p[0];
        R.py = p[1];
        R.pz = p[2];
        R.dx = d[0];
        R.dy = d[1];
        R.dz = d[2];
    }
    return R;
}

// ---- shapes in FP32 (cshapes.pyx) ----------------------------------------------
// The postfix program of rp_shape_op with the operand stack kept as bits.
__device__ int shape_in_f(const DevScene &S, int prog, float x, float y, unsigned *err) {
    if (prog < 0) return 1;
    unsigned bits = 0u;
    int sp = 0;
    for (int k = prog; k < S.n_shapes; k++) {
        const rp_shape_op &op = S.shapes[k];
        unsigned v;
        switch (op.op) {
            case RP_SHAPE_END: return sp > 0 ? (int)(bits & 1u) : 1;
            case RP_SHAPE_TRUE: v = 1u; break;
            case RP_SHAPE_CIRCLE: {
                float dx = x - f_of_d(op.a), dy = y - f_of_d(op.b), c = f_of_d(op.c);
                v = (dx * dx + dy * dy < c * c) ? 1u : 0u;
                break;
            }
            case RP_SHAPE_RECT: {
                float dx = x - f_of_d(op.a), dy = y - f_of_d(op.b);
                v = ((2.0f * fabsf(dx) < f_of_d(op.c)) && (2.0f * fabsf(dy) < f_of_d(op.d))) ? 1u : 0u;
                break;
            }
            case RP_SHAPE_POLYGON: v = (unsigned)poly_shape_inside(S.aux + op.aux, op.n, d_of_f(x), d_of_f(y)); break;
            case RP_SHAPE_AND:
            case RP_SHAPE_OR:
            case RP_SHAPE_XOR: {
                if (sp < 2) goto bad;
                unsigned b = bits & 1u, a = (bits >> 1) & 1u;
                bits >>= 2;
                sp -= 2;
                v = op.op == RP_SHAPE_AND ? (a & b) : op.op == RP_SHAPE_OR ? (a | b) : (a ^ b);
                break;
            }
            case RP_SHAPE_NOT: {
                if (sp < 1) goto bad;
                v = (~bits) & 1u;
                bits >>= 1;
                sp -= 1;
                break;
            }
            default: goto bad;
        }
        bits = (bits << 1) | v;
        if (++sp >= 31) goto bad;
    }
    return sp > 0 ? (int)(bits & 1u) : 1;
bad:
    atomicOr(err, ERR_SHAPE_STACK);
    return 0;
}

// ---- face intersections --------------------------------------------------------
#define MX_MISS_T (-1.0f)
__device__ __forceinline__ ff miss_t() { return ffm(MX_MISS_T, 0.0f); }

// U = P + t Dl relative to the face vertex, in float-float.
__device__ __forceinline__ void vertex_point_ff(const LRay &R, ff zv, ff t, ff &X, ff &Y, ff &Z) {
    X = ff_add(R.px, ff_mul(t, R.dx));
    Y = ff_add(R.py, ff_mul(t, R.dy));
    Z = ff_sub(ff_add(R.pz, ff_mul(t, R.dz)), zv);
}
// The same point rounded to FP32 (the coordinates are of the order of the
// aperture: FP32 places them within ~1 nm, enough for aperture tests and
// derivatives, not for the residual of a root).
__device__ __forceinline__ f3 vertex_point(const LRay &R, ff zv, ff t) {
    ff X, Y, Z;
    vertex_point_ff(R, zv, t, X, Y, Z);
    return mk3(X.hi + X.lo, Y.hi + Y.lo, Z.hi + Z.lo);
}
__device__ __forceinline__ ff ff_sqr(ff a) {
    ff p = two_prod(a.hi, a.hi);
    p.lo = fmaf(2.0f * a.hi, a.lo, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// Newton correction of a quadric root: F = beta z^2 - 2 Rq z + x^2 + y^2 in
// vertex coordinates (a sphere is beta = 1, Rq = -curvature).  At the root the
// terms of F cancel to a part in 10^9 of their size, so F is evaluated in
// float-float at the float-float point (the residual at FP32-rounded
// coordinates would leave ~0.3 nm along the ray); its derivative along the
// ray needs only FP32.  One step takes the FP32 root (error ~1e-5 mm) to
// ~1e-12 mm; a second is taken when the first moved the root by more than a
// micrometre (grazing hits, where the FP32 root is poorer).
__device__ __forceinline__ ff refine_quadric(const LRay &R, ff zv, float t0, float beta, ff Rq) {
    ff t = ffm(t0, 0.0f);
    const float dx = R.dx.hi, dy = R.dy.hi, dz = R.dz.hi;
    const ff two_rq = ffm(2.0f * Rq.hi, 2.0f * Rq.lo);
    for (int it = 0; it < 2; it++) {
        ff X, Y, Z;
        vertex_point_ff(R, zv, t, X, Y, Z);
        const ff F = ff_add(ff_add(ff_sqr(X), ff_sqr(Y)), ff_mul(Z, ff_sub(ff_mul_f(Z, beta), two_rq)));
        const float G = 2.0f * ((beta * Z.hi - Rq.hi) * dz + X.hi * dx + Y.hi * dy);
        const float step = -F.hi / G;
        if (!isfinite(step)) break;
        t = ff_add_f(t, step);
        if (fabsf(step) <= 1e-3f) break;
    }
    return t;
}

// Asphere sag residual f = sag(r^2) - z and its derivative along the ray, FP32.
__device__ __forceinline__ void asph_fg(const MxFace &M, float Rq, float beta, f3 u, float dx, float dy, float dz,
                                        float &fv, float &g) {
    const float R2 = Rq * Rq;
    const float A4 = M.p[3], A6 = M.p[4], A8 = M.p[5], A10 = M.p[6], A12 = M.p[7], A14 = M.p[8], A16 = M.p[9];
    float r2 = u.x * u.x + u.y * u.y;
    float root = sqrtf(1.0f - beta * r2 / R2);
    float poly = r2 * r2 * (A4 + r2 * (A6 + r2 * (A8 + r2 * (A10 + r2 * (A12 + r2 * (A14 + r2 * A16))))));
    float inv = 1.0f / (Rq * (1.0f + root));
    fv = r2 * inv - u.z + poly;
    float dr2 = 2.0f * (dx * u.x + dy * u.y);
    float dsag = inv + beta * r2 * inv * inv / (2.0f * Rq * root);
    float dpoly = r2 * (2.0f * A4 + r2 * (3.0f * A6 + r2 * (4.0f * A8 + r2 * (5.0f * A10 +
                  r2 * (6.0f * A12 + r2 * (7.0f * A14 + r2 * 8.0f * A16))))));
    g = (dsag + dpoly) * dr2 - dz;
}

// The asphere's sag residual sag(r^2) - z at a float-float point: the conic
// part r^2 / (Rq (1 + sqrt(1 - beta r^2 / Rq^2))), of the size of z and
// cancelling against it, in float-float; the polynomial part (a small
// fraction of the sag) in FP32.
__device__ __forceinline__ float asph_residual_ff(const MxFace &M, ff Rq, float beta, ff X, ff Y, ff Z) {
    const ff r2 = ff_add(ff_sqr(X), ff_sqr(Y));
    const float k = beta / (Rq.hi * Rq.hi);
    const ff root = ff_sqrt(ff_add_f(ff_neg(ff_mul_f(r2, k)), 1.0f));
    const ff conic = ff_div(r2, ff_mul(Rq, ff_add_f(root, 1.0f)));
    const float A4 = M.p[3], A6 = M.p[4], A8 = M.p[5], A10 = M.p[6], A12 = M.p[7], A14 = M.p[8], A16 = M.p[9];
    const float q = r2.hi;
    const float poly = q * q * (A4 + q * (A6 + q * (A8 + q * (A10 + q * (A12 + q * (A14 + q * A16))))));
    return ff_sub(ff_add_f(conic, poly), Z).hi;
}

// intersect_conic (cfaces.pyx:1695-1747) in vertex coordinates, FP32: the
// ray parameter (units of the direction d) of the quadric of vertex radius Rq
// and beta = 1 + conic constant, the reference's choice of root by the sign
// of Rq beta d_z; -tmax (its -1, a fraction of the segment) without a root.
__device__ __forceinline__ float conic_root32(float Rq, float beta, float px, float py, float pz, float dx, float dy,
                                              float dz, float tmax) {
    const float b2 = beta * beta;
    float A = b2 * dz * dz + beta * (dx * dx + dy * dy);
    float B = -2.0f * Rq * beta * dz + 2.0f * beta * (px * dx + py * dy) + 2.0f * pz * b2 * dz;
    float C = -2.0f * Rq * pz * beta + beta * (px * px + py * py) + pz * pz * b2;
    float disc = B * B - 4.0f * A * C;
    if (disc < 0.0f) return -tmax;
    float sd = sqrtf(disc);
    bool plus = Rq * beta * dz <= 0.0f;
    if (A == 0.0f) return plus ? (-B + sd) / (2.0f * A) : (-B - sd) / (2.0f * A);
    if (plus) return (B > 0.0f) ? (2.0f * C) / (-B - sd) : (-B + sd) / (2.0f * A);
    return (B < 0.0f) ? (2.0f * C) / (-B + sd) : (-B - sd) / (2.0f * A);
}

// The 2D polynomial of an ExtendedPolynomialFace at normalised (xs, ys)
// (cfaces.pyx:2066-2068) and its derivatives in xs and ys (2092-2100), in
// FP32 from the face's table E = [Nx, Ny, E[0][0], E[0][1], ...].
__device__ __forceinline__ void ep_eval32(const float *E, float xs, float ys, float &P, float &Px, float &Py) {
    const int nx = (int)E[0], ny = (int)E[1];
    const float *c = E + 2;
    P = 0.0f;
    Px = 0.0f;
    Py = 0.0f;
    for (int i = nx - 1; i >= 0; i--) {
        // row i at ys and its derivative in ys
        float q = 0.0f, qd = 0.0f;
        for (int j = ny - 1; j >= 0; j--) {
            qd = fmaf(qd, ys, q);
            q = fmaf(q, ys, c[i * ny + j]);
        }
        Px = fmaf(Px, xs, P);
        P = fmaf(P, xs, q);
        Py = fmaf(Py, xs, qd);
    }
}

// The extended polynomial's residual conic(r^2) + P(x, y) - z at a
// float-float point in vertex coordinates (eval_extpoly_impf,
// cfaces.pyx:2043-2070, relative to z_height): the conic part in
// float-float, the polynomial part (a small height) in FP32; and its FP32
// derivative along the ray direction d (eval_extpoly_grad, 2073-2104).
__device__ __forceinline__ float ep_residual_ff(const float *E, ff Rq, float beta, float irho, ff X, ff Y, ff Z) {
    const ff r2 = ff_add(ff_sqr(X), ff_sqr(Y));
    const float k = beta / (Rq.hi * Rq.hi);
    const ff root = ff_sqrt(ff_add_f(ff_neg(ff_mul_f(r2, k)), 1.0f));
    const ff conic = ff_div(r2, ff_mul(Rq, ff_add_f(root, 1.0f)));
    float P, Px, Py;
    ep_eval32(E, X.hi * irho, Y.hi * irho, P, Px, Py);
    return ff_sub(ff_add_f(conic, P), Z).hi;
}
__device__ __forceinline__ void ep_fg32(const float *E, float Rq, float beta, float irho, f3 u, float dx, float dy,
                                        float dz, float &fv, float &g) {
    const float r2 = u.x * u.x + u.y * u.y;
    const float rt = sqrtf(1.0f - beta * r2 / (Rq * Rq));
    const float denom = Rq * (rt + 1.0f);
    const float nom = 2.0f * (dx * u.x + dy * u.y);
    float P, Px, Py;
    ep_eval32(E, u.x * irho, u.y * irho, P, Px, Py);
    fv = r2 / denom + P - u.z;
    g = nom / denom + beta * nom * r2 / (2.0f * Rq * rt * denom * denom) + (Px * dx + Py * dy) * irho - dz;
}

// ExtendedPolynomialFace.intersect_c (cfaces.pyx:2182-2234): the conic root,
// then Newton on the residual in FP32 (in vertex coordinates), a miss when it
// stops converging above the FP32 rounding of the residual or takes 100
// steps; the winner is refined in float-float (face_refine).  Out of line, so
// that scenes without such faces do not carry its registers.
__device__ __noinline__ float extpoly_t32(const DevScene &S, const rp_face &F, const MxFace &M, const LRay &R,
                                          float tmax, unsigned *err, bool &fb) {
    const ff zv = ffm(M.zv_hi, M.zv_lo);
    if (!S.ep32_off || S.ep32_off[&F - S.faces] < 0) {
        fb = true;
        return MX_MISS_T;
    }
    const float *E = S.ep32 + S.ep32_off[&F - S.faces];
    const float Rq = M.p[0], beta = M.p[1], irho = 1.0f / M.p[2];
    const float px = R.px.hi, py = R.py.hi, pz = ff_sub(R.pz, zv).hi;
    const float dx = R.dx.hi, dy = R.dy.hi, dz = R.dz.hi;
    float tf = conic_root32(Rq, beta, px, py, pz, dx, dy, dz, tmax);
    float fv, g;
    ep_fg32(E, Rq, beta, irho, mk3(fmaf(tf, dx, px), fmaf(tf, dy, py), fmaf(tf, dz, pz)), dx, dy, dz, fv, g);
    float f_last = fv, step = -fv / g;
    bool conv = false;
    for (int it = 0; it < 100; it++) {
        tf += step;
        if (fabsf(step) <= 1e-5f * (1.0f + fabsf(tf))) {
            conv = true;
            break;
        }
        const f3 u = mk3(fmaf(tf, dx, px), fmaf(tf, dy, py), fmaf(tf, dz, pz));
        ep_fg32(E, Rq, beta, irho, u, dx, dy, dz, fv, g);
        if (fabsf(fv) > fabsf(f_last) && fabsf(fv) > 1e-6f * (1.0f + fabsf(u.z))) return MX_MISS_T;
        f_last = fv;
        step = -fv / g;
    }
    if (!conv || !isfinite(tf)) return MX_MISS_T;
    if (!shape_in_f(S, F.shape, fmaf(tf, dx, px), fmaf(tf, dy, py), err)) return MX_MISS_T;
    if (!(tf <= tmax) || !(tf >= M.tmin)) return MX_MISS_T;  // a1 > 1 or a1 < tolerance
    return tf;
}

// DistortionFace.intersect_c (cfaces.pyx:2341-2407) over a ShapedPlanarFace
// base z = zb, after the plain path's exact cull of lines that never pass
// over the shape (box: the face's entry in S.bounds).  The base plane's hit
// is exact in float-float (tb, distance ab); the points the reference visits
// lie on the ray a distance del from it -- for a hit on the surface a small
// one, the distortion's height over the slope -- so the iteration runs in
// FP32 on del: the first estimate from the tangent plane at the distorted
// point above the base hit, then per step the base hit of the ray shifted
// down by z_offset, the tangent plane there and its ray distance, until two
// estimates agree within the face's accuracy, the reference's sequence of
// points and tests.  The hit is tb + del / |D| in float-float (*exact set).
// A shifted ray that misses the base, 20 steps without agreement, or an
// agreement away from the surface set fb: the FP64 path then decides.
__device__ __noinline__ float distortion_t32(const DevScene &S, const rp_face &F, const MxFace &M, const LRay &R, float tmax,
                                float dl, const float *box, unsigned *err, ff *tff, bool *exact, bool &fb) {
    // the exact cull of the plain path (distortion_line_misses), in FP32 on
    // its padded rectangle: a line that never passes over it cannot hit
    if (box[6] == 2.0f) {
        const float px = R.px.hi, py = R.py.hi, vx = R.dx.hi, vy = R.dy.hi;
        if (vx == 0.0f && vy == 0.0f) {
            if (px < box[0] || px > box[1] || py < box[2] || py > box[3]) return MX_MISS_T;
        } else {
            const float s00 = vx * (box[2] - py) - vy * (box[0] - px), s01 = vx * (box[3] - py) - vy * (box[0] - px);
            const float s10 = vx * (box[2] - py) - vy * (box[1] - px), s11 = vx * (box[3] - py) - vy * (box[1] - px);
            if ((s00 > 0.0f && s01 > 0.0f && s10 > 0.0f && s11 > 0.0f) ||
                (s00 < 0.0f && s01 < 0.0f && s10 < 0.0f && s11 < 0.0f))
                return MX_MISS_T;
        }
    }
    const ff zb = ffm(M.zv_hi, M.zv_lo);
    // ShapedPlanarFace.intersect_c, is_base_ray 0 (cfaces.pyx:213-221): h in [tolerance, 1]
    const ff tb = ff_div(ff_sub(zb, R.pz), R.dz);
    const float h = tb.hi / tmax;
    if (!(h >= M.btol) || h > 1.0f) return MX_MISS_T;
    const float seg = tmax * dl;  // the segment's length (h of intersect_c)
    const float ab = tb.hi * dl;  // a2: the base hit's distance
    if (ab > seg || ab < M.tol) return MX_MISS_T;  // cfaces.pyx:2355
    const float ux = R.dx.hi / dl, uy = R.dy.hi / dl, uz = R.dz.hi / dl;
    const float xb = ff_add(R.px, ff_mul(tb, R.dx)).hi, yb = ff_add(R.py, ff_mul(tb, R.dy)).hi;
    float gx, gy, gz;
    zk_eval32(S, F.distortion, xb, yb, true, gx, gy, gz);
    // the tangent plane at the distorted point, normal (-gx, -gy, 1): a1 - ab
    float del = gz / (uz - gx * ux - gy * uy);
    if (ab + del < fabsf(gz)) return MX_MISS_T;  // cfaces.pyx:2375-2377
    const float acc = M.p[0];                    // DistortionFace.accuracy
    float dprev = 0.0f, x = xb, y = yb;
    bool conv = false;
    for (int it = 0; it < 20; it++) {
        x = fmaf(ux, del, xb);  // the ray point at a1
        y = fmaf(uy, del, yb);
        if (fabsf(del - dprev) < acc) {
            conv = true;
            break;
        }
        float zs, wx, wy;
        zk_eval32(S, F.distortion, x, y, false, wx, wy, zs);
        const float d2 = zs / uz;  // the base hit of the ray shifted by -z_offset
        const float h2 = (ab + d2) / seg;
        if (!(h2 >= M.btol) || h2 > 1.0f) {
            fb = true;
            return MX_MISS_T;
        }
        x = fmaf(ux, d2, xb);
        y = fmaf(uy, d2, yb);
        zk_eval32(S, F.distortion, x, y, true, gx, gy, gz);
        const float dnew = (gz - d2 * (gx * ux + gy * uy)) / (uz - gx * ux - gy * uy);
        dprev = del;
        del = dnew;
    }
    if (!conv || !isfinite(del)) {
        fb = true;
        return MX_MISS_T;
    }
    // A converged estimate lies on the distorted surface.  The reference's
    // iteration can also settle where no surface is: a base hit far outside
    // the face, where the polynomials are large, whose tangent plane meets
    // the ray far from the plane; FP32 cannot follow it there (del is then
    // tens of millimetres), so the FP64 path decides such a ray.
    {
        float zs, wx, wy;
        zk_eval32(S, F.distortion, x, y, false, wx, wy, zs);
        if (!(fabsf(uz * del - zs) < 1e-3f)) {
            fb = true;
            return MX_MISS_T;
        }
    }
    if (!shape_in_f(S, F.shape, x, y, err)) return MX_MISS_T;  // cfaces.pyx:2402
    const ff t = ff_add_f(tb, del / dl);
    *tff = t;
    *exact = true;
    return t.hi;
}

// Phase one of a face test: the FP32 ray parameter of face F's hit (hit =
// P + t Dl), with bounds and aperture tested at the FP32 hit point, or
// MX_MISS_T; `fb` is set for face types left to the FP64 path.  A plane's
// parameter costs one float-float division, so it is returned exactly in *tff
// (*exact set); curved faces are refined by face_refine only if they win.
template <bool DIST>
__device__ float face_t32(const DevScene &S, const rp_face &F, const MxFace &M, const LRay &R, float tmax, float dl,
                          unsigned *err, ff *tff, bool *exact, bool &fb) {
    fb = false;
    *exact = false;
    const ff zv = ffm(M.zv_hi, M.zv_lo);
    switch (F.type) {
        case RP_FACE_CIRCULAR:
        case RP_FACE_RECTANGULAR:
        case RP_FACE_SHAPED_PLANAR: {
            // cfaces.pyx:147-175, 364-396, 201-227: plane z = zv
            ff t = ff_div(ff_sub(zv, R.pz), R.dz);
            if (!(t.hi >= M.tmin) || t.hi > tmax) return MX_MISS_T;
            float X = fmaf(t.hi, R.dx.hi, R.px.hi), Y = fmaf(t.hi, R.dy.hi, R.py.hi);
            if (F.type == RP_FACE_CIRCULAR) {
                X -= M.p[1];
                if (X * X + Y * Y > M.p[0] * M.p[0] * 0.25f) return MX_MISS_T;
            } else if (F.type == RP_FACE_RECTANGULAR) {
                X -= M.p[2];
                if (X * X > M.p[0] * M.p[0] * 0.25f) return MX_MISS_T;
                if (Y * Y > M.p[1] * M.p[1] * 0.25f) return MX_MISS_T;
            } else if (!shape_in_f(S, F.shape, X, Y, err)) {
                return MX_MISS_T;
            }
            *tff = t;
            *exact = true;
            return t.hi;
        }
        case RP_FACE_SPHERICAL:
        case RP_FACE_SHAPED_SPHERICAL: {
            // cfaces.pyx:418-482, 512-592, in vertex coordinates: centre at z = -c
            const bool plain = F.type == RP_FACE_SPHERICAL;
            const float c = plain ? M.p[1] : M.p[0];
            const float px = R.px.hi, py = R.py.hi;
            const ff pzr = ff_sub(R.pz, zv);
            const float pz = pzr.hi;
            const float dx = R.dx.hi, dy = R.dy.hi, dz = R.dz.hi;
            float a = dx * dx + dy * dy + dz * dz;
            float b = 2.0f * (dx * px + dy * py + dz * (pz + c));
            float cc = px * px + py * py + pz * (pz + 2.0f * c);
            float disc = b * b - 4.0f * a * cc;
            if (disc < 0.0f) return MX_MISS_T;
            float q = -0.5f * (b + copysignf(sqrtf(disc), b));
            float t1 = q / a, t2 = (q != 0.0f) ? cc / q : t1;
            const float INF = __int_as_float(0x7f800000);
            float zc1 = pz + c + t1 * dz, zc2 = pz + c + t2 * dz;  // z relative to the centre
            if (c >= 0.0f) {
                if (zc1 < 0.0f) t1 = INF;
                if (zc2 < 0.0f) t2 = INF;
            } else {
                if (zc1 > 0.0f) t1 = INF;
                if (zc2 > 0.0f) t2 = INF;
            }
            float x1 = px + t1 * dx, y1 = py + t1 * dy, x2 = px + t2 * dx, y2 = py + t2 * dy;
            if (plain) {
                float DD = M.p[0] * M.p[0] * 0.25f;
                if (x1 * x1 + y1 * y1 > DD) t1 = INF;
                if (x2 * x2 + y2 * y2 > DD) t2 = INF;
            } else {
                if (t1 != INF && !shape_in_f(S, F.shape, x1, y1, err)) t1 = INF;
                if (t2 != INF && !shape_in_f(S, F.shape, x2, y2, err)) t2 = INF;
            }
            float t = fminf(t1, t2);
            if (!(t <= tmax) || !(t >= M.tmin)) return MX_MISS_T;
            return t;
        }
        case RP_FACE_CONIC:
        case RP_FACE_ASPHERIC: {
            const float Rq = -M.p[0], beta = 1.0f + M.p[2];
            const float px = R.px.hi, py = R.py.hi;
            const float pz = ff_sub(R.pz, zv).hi;
            const float dx = R.dx.hi, dy = R.dy.hi, dz = R.dz.hi;
            float t = conic_root32(Rq, beta, px, py, pz, dx, dy, dz, tmax);
            if (F.type == RP_FACE_CONIC) {
                if (!(t <= tmax) || !(t >= M.tmin)) return MX_MISS_T;  // D < 0 gives -1: a miss
            } else {
                // asphere: Newton on the sag residual in FP32 from the conic root
                // (cfaces.pyx:1908-1974)
                float tf = t, f_last = 0.0f;
                bool conv = false;
                const f3 p0 = mk3(px, py, pz);
                for (int it = 0; it < 100; it++) {
                    f3 u = add3(p0, mul3(mk3(dx, dy, dz), tf));
                    float fv, g;
                    asph_fg(M, Rq, beta, u, dx, dy, dz, fv, g);
                    if (it > 0 && fabsf(fv) > fabsf(f_last) && fabsf(fv) > 1e-6f * (1.0f + fabsf(u.z))) return MX_MISS_T;
                    f_last = fv;
                    float step = -fv / g;
                    tf += step;
                    if (fabsf(step) <= 1e-5f * (1.0f + fabsf(tf))) {
                        conv = true;
                        break;
                    }
                }
                if (!conv || !isfinite(tf)) return MX_MISS_T;
                if (!(tf <= tmax) || !(tf >= M.tmin)) return MX_MISS_T;
                t = tf;
            }
            if (!shape_in_f(S, F.shape, fmaf(t, dx, px), fmaf(t, dy, py), err)) return MX_MISS_T;
            return t;
        }
        case RP_FACE_EXTPOLY:  // (as the DistortionFace: scenes that have one carry the FP64 path)
            if constexpr (DIST) return extpoly_t32(S, F, M, R, tmax, err, fb);
            fb = true;
            return MX_MISS_T;
        case RP_FACE_DISTORTION:  // (only scenes that also carry the FP64 path specialise it)
            if constexpr (DIST)
                if (M.spec) return distortion_t32(S, F, M, R, tmax, dl, S.bounds + 16 * (&F - S.faces), err, tff,
                                                  exact, fb);
            fb = true;
            return MX_MISS_T;
        default: fb = true; return MX_MISS_T;
    }
}

// An ExtendedPolynomialFace hit in float-float from its FP32 ray parameter:
// Newton steps on the residual in float-float (ep_residual_ff).
__device__ __noinline__ ff extpoly_refine(const DevScene &S, const rp_face &F, const MxFace &M, const LRay &R,
                                          float t32) {
    const ff zv = ffm(M.zv_hi, M.zv_lo);
    const ff Rq = ffm(M.rq_hi, M.rq_lo);
    const float *E = S.ep32 + S.ep32_off[&F - S.faces];
    const float beta = M.p[1], irho = 1.0f / M.p[2];
    ff tt = ffm(t32, 0.0f);
    const float dx = R.dx.hi, dy = R.dy.hi, dz = R.dz.hi;
    for (int it = 0; it < 2; it++) {
        ff X, Y, Z;
        vertex_point_ff(R, zv, tt, X, Y, Z);
        float fv, g;
        ep_fg32(E, Rq.hi, beta, irho, mk3(X.hi, Y.hi, Z.hi), dx, dy, dz, fv, g);
        fv = ep_residual_ff(E, Rq, beta, irho, X, Y, Z);
        const float step = -fv / g;
        if (!isfinite(step)) break;
        tt = ff_add_f(tt, step);
        if (fabsf(step) <= 1e-3f) break;
    }
    return tt;
}

// Phase two, for a face that may be the nearest: its ray parameter in
// float-float from the FP32 one, by Newton steps whose residuals are
// evaluated in float-float (refine_quadric; the asphere's sag residual by
// asph_residual_ff, its derivative in FP32).  The FP32 root is within
// ~1e-5 mm, so one step suffices unless it moved the root by more than a
// micrometre.
template <bool DIST>
__device__ __forceinline__ ff face_refine(const DevScene &S, const rp_face &F, const MxFace &M, const LRay &R,
                                          float t32) {
    const ff zv = ffm(M.zv_hi, M.zv_lo);
    const ff Rq = ffm(M.rq_hi, M.rq_lo);
    if (F.type == RP_FACE_SPHERICAL || F.type == RP_FACE_SHAPED_SPHERICAL) return refine_quadric(R, zv, t32, 1.0f, Rq);
    if constexpr (DIST)
        if (F.type == RP_FACE_EXTPOLY) return extpoly_refine(S, F, M, R, t32);
    const float beta = 1.0f + M.p[2];
    if (F.type == RP_FACE_CONIC) return refine_quadric(R, zv, t32, beta, Rq);
    ff tt = ffm(t32, 0.0f);
    const float dx = R.dx.hi, dy = R.dy.hi, dz = R.dz.hi;
    for (int it = 0; it < 2; it++) {
        ff X, Y, Z;
        vertex_point_ff(R, zv, tt, X, Y, Z);
        float fv, g;
        asph_fg(M, Rq.hi, beta, mk3(X.hi, Y.hi, Z.hi), dx, dy, dz, fv, g);
        fv = asph_residual_ff(M, Rq, beta, X, Y, Z);
        const float step = -fv / g;
        if (!isfinite(step)) break;
        tt = ff_add_f(tt, step);
        if (fabsf(step) <= 1e-3f) break;
    }
    return tt;
}

// Unit normal of a specialised face in float-float at a hit given in vertex
// coordinates (x, y and z relative to the vertex); false for faces left to the
// FP64 path.  Face parameters are the FP32 copies.
template <bool DIST>
__device__ __forceinline__ bool face_normal_ff(const DevScene &S, const rp_face &F, const MxFace &M, ff x, ff y, ff z,
                                               ff3 &n) {
    const ff zero = ffm(0.0f, 0.0f);
    switch (F.type) {
        case RP_FACE_CIRCULAR: n = mkff3(zero, zero, ffm(F.invert_normals ? 1.0f : -1.0f, 0.0f)); return true;
        case RP_FACE_SHAPED_PLANAR: n = mkff3(zero, zero, ffm(1.0f, 0.0f)); return true;
        case RP_FACE_RECTANGULAR: n = mkff3(zero, zero, ffm(-1.0f, 0.0f)); return true;
        case RP_FACE_SPHERICAL:
        case RP_FACE_SHAPED_SPHERICAL: {
            // cfaces.pyx:485-498, 594-606: (p - centre) normalised, flipped for
            // c < 0.  At a hit |p - centre| = |c| to float-float accuracy, so
            // the unit normal is (p - centre) / c: (x, y, z + c) times 1 / c.
            const ff ic = ffm(M.ic_hi, M.ic_lo);
            const ff zc = ff_sub(z, ffm(M.rq_hi, M.rq_lo));  // z + c, with c = -Rq
            n = mkff3(ff_mul(x, ic), ff_mul(y, ic), ff_mul(zc, ic));
            return true;
        }
        case RP_FACE_CONIC: {  // cfaces.pyx:1796-1820
            float Rq = -M.p[0], beta = 1.0f + M.p[2];
            float sign = F.invert_normals ? -1.0f : 1.0f;
            if (Rq * beta < 0.0f) sign = -sign;
            ff3 g = mkff3(ff_mul_f(x, -2.0f * beta * sign), ff_mul_f(y, -2.0f * beta * sign),
                          ff_mul_f(ff_add_f(ff_mul_f(z, -beta), Rq), 2.0f * beta * sign));
            n = ff3_unit(g);
            return true;
        }
        case RP_FACE_ASPHERIC: {  // cfaces.pyx:1976-2005
            float Rq = -M.p[0], beta = 1.0f + M.p[2];
            float sign = F.invert_normals ? -1.0f : 1.0f;
            float xf = x.hi + x.lo, yf = y.hi + y.lo;
            float r2 = xf * xf + yf * yf;
            float root = sqrtf(1.0f - beta * r2 / (Rq * Rq));
            float df = r2 * (4.0f * M.p[3] + r2 * (6.0f * M.p[4] + r2 * (8.0f * M.p[5] + r2 * (10.0f * M.p[6] +
                       r2 * (12.0f * M.p[7] + r2 * (14.0f * M.p[8] + r2 * 16.0f * M.p[9]))))));
            float inv = 1.0f / (Rq * (1.0f + root));
            df += 2.0f * inv + beta * r2 * inv * inv / (Rq * root);
            n = ff3_unit(mkff3(ff_mul_f(x, -df * sign), ff_mul_f(y, -df * sign), ffm(sign, 0.0f)));
            return true;
        }
        case RP_FACE_EXTPOLY: {  // cfaces.pyx:2236-2293: the conic's unit normal, then the polynomial's gradient
            if constexpr (!DIST) return false;
            if (!S.ep32_off || S.ep32_off[&F - S.faces] < 0) return false;
            const float *E = S.ep32 + S.ep32_off[&F - S.faces];
            const float Rq = M.p[0], beta = M.p[1], irho = 1.0f / M.p[2];
            float sign = F.invert_normals ? -1.0f : 1.0f;
            if (Rq * beta < 0.0f) sign = -sign;
            ff3 g = mkff3(ff_mul_f(x, -2.0f * beta * sign), ff_mul_f(y, -2.0f * beta * sign),
                          ff_mul_f(ff_add_f(ff_mul_f(z, -beta), Rq), 2.0f * beta * sign));
            g = ff3_unit(g);
            float P, Px, Py;
            ep_eval32(E, x.hi * irho, y.hi * irho, P, Px, Py);
            const float s2 = F.invert_normals ? irho : -irho;  // added with invert_normals, else subtracted
            g.x = ff_add_f(g.x, s2 * Px);
            g.y = ff_add_f(g.y, s2 * Py);
            n = ff3_unit(g);
            return true;
        }
        case RP_FACE_DISTORTION: {  // cfaces.pyx:2409-2422 over a plane: (-dz/dx, -dz/dy, 1) normalised
            if constexpr (DIST) {
                if (!M.spec) return false;
                float gx, gy, gz;
                zk_eval32(S, F.distortion, x.hi, y.hi, true, gx, gy, gz);
                n = ff3_unit(mkff3(ffm(-gx, 0.0f), ffm(-gy, 0.0f), ffm(1.0f, 0.0f)));
                return true;
            }
            return false;
        }
        default: return false;
    }
}

// ---- materials in FP32 ------------------------------------------------------------
struct RayF {
    f3 d;         // direction (unit to FP32 rounding)
    f3 E;         // E_vector
    cf e1, e2;    // E1_amp, E2_amp
    double2 n;    // refractive_index (copied to transparent / PEC children)
    unsigned type, wl;
};
struct ChildF {
    ff3 d;
    cf e1, e2;
    double2 n;
    unsigned type;
};

// convert_to_sp in FP32 (cmaterials.pyx:49-91)
__device__ __forceinline__ void sp_f(f3 d, f3 E, cf e1, cf e2, f3 normal, f3 &Eo, cf &e1o, cf &e2o) {
    f3 E2v = norm3(cross3(d, E));
    f3 E1v = norm3(cross3(E2v, d));
    f3 Sv = cross3(d, normal);
    if (fabsf(Sv.x) < 1e-10f && fabsf(Sv.y) < 1e-10f && fabsf(Sv.z) < 1e-10f) {
        Eo = E;
        e1o = e1;
        e2o = e2;
        return;
    }
    Sv = norm3(Sv);
    f3 Pv = norm3(cross3(d, Sv));
    float A = dot3(E1v, Sv), B = dot3(E2v, Sv);
    e1o = cfm(e1.x * A + e2.x * B, e1.y * A + e2.y * B);
    B = dot3(E1v, Pv);
    A = dot3(E2v, Pv);
    e2o = cfm(e1.x * B + e2.x * A, e1.y * B + e2.y * A);
    Eo = Sv;
}

__device__ __forceinline__ bool mat_specialised(int type) {
    return type == RP_MAT_NONE || type == RP_MAT_OPAQUE || type == RP_MAT_PEC || type == RP_MAT_DIELECTRIC ||
           type == RP_MAT_FULL_DIELECTRIC || type == RP_MAT_FULL_DIELECTRIC_DISPERSIVE || type == RP_MAT_TRANSPARENT;
}

// Children of a hit for the specialised materials (cmaterials.pyx:260-278
// Transparent, 292-319 PEC, 589-680 Dielectric, 756-872 FullDielectric,
// 897-1013 FullDielectricDispersive).  Directions (reflection, Snell's law) are
// float-float from the float-float ray direction D, its unit vector ind and
// the unit normal nn; the S/P projection, Fresnel coefficients and amplitudes
// are FP32.  Eo receives the children's shared E_vector; returns the number of
// children.  nt_in / nt_out: a dispersive material's complex indices inside
// and outside at the ray's wavelength (loaded by the caller ahead of use).
__device__ int eval_f(const DevScene &S, const rp_material &m, const RayF &r, const ff3 &D, const ff3 &ind,
                      const ff3 &nn, f3 &Eo, ChildF *ch, unsigned *err, double2 nt_in, double2 nt_out) {
    if (m.type == RP_MAT_NONE || m.type == RP_MAT_OPAQUE) return 0;
    const f3 normal = mk3(nn.x.hi, nn.y.hi, nn.z.hi);
    cf E1, E2;
    sp_f(r.d, r.E, r.e1, r.e2, normal, Eo, E1, E2);
    if (m.type == RP_MAT_TRANSPARENT) {
        ch[0].d = D;
        ch[0].n = r.n;
        ch[0].e1 = E1;
        ch[0].e2 = E2;
        ch[0].type = r.type & ~RP_REFL_RAY;
        return 1;
    }
    const ff cosT = ff_dot3(nn, m.type == RP_MAT_PEC ? D : ind);
    const ff3 ctn2 = ff3_scale(nn, ff_mul_f(cosT, 2.0f));
    if (m.type == RP_MAT_PEC) {
        ch[0].d = ff3_sub(D, ctn2);
        ch[0].n = r.n;
        ch[0].e1 = cfm(-E1.x, -E1.y);
        ch[0].e2 = E2;
        ch[0].type = r.type | RP_REFL_RAY;
        return 1;
    }
    const float cosTheta = cosT.hi;
    const float cos1 = fabsf(cosTheta);
    const bool out_to_in = cosTheta < 0.0f;
    const float flip = out_to_in ? 1.0f : -1.0f;
    // Snell's law in vector form: tg2 = (ind - cos n) n1/n2, t = tg2 - n sqrt(1 - |tg2|^2) flip
    auto refract = [&](ff ratio, float &cos2) -> ff3 {
        ff3 tg2 = ff3_scale(ff3_sub(ind, ff3_scale(nn, cosT)), ratio);
        ff c2 = ff_sqrt(ff_sub(ffm(1.0f, 0.0f), ff_dot3(tg2, tg2)));
        ff3 tr = ff3_sub(tg2, ff3_scale(nn, ff_mul_f(c2, flip)));
        cos2 = fabsf(ff_dot3(tr, nn).hi);
        return tr;
    };
    if (m.type == RP_MAT_DIELECTRIC) {
        const double n1d = out_to_in ? m.n_outside[0] : m.n_inside[0];
        const double n2d = out_to_in ? m.n_inside[0] : m.n_outside[0];
        const float n1 = f_of_d(n1d), n2 = f_of_d(n2d);
        ch[0].n = out_to_in ? make_double2(m.n_inside[0], m.n_inside[1]) : make_double2(m.n_outside[0], m.n_outside[1]);
        float q = n2 / n1;
        float N2_sin2 = cosTheta * cosTheta + (q * q - 1.0f);
        if (N2_sin2 < 0.0f) {
            ch[0].d = ff3_sub(ind, ctn2);
            ch[0].e1 = cfm(-E1.x, -E1.y);
            ch[0].e2 = cfm(-E2.x, -E2.y);
            ch[0].type = r.type | RP_REFL_RAY;
        } else {
            float cos2;
            ch[0].d = refract(ff_div(ff_of_d(n1d), ff_of_d(n2d)), cos2);
            float aspect = sqrtf(cos2 / cos1) * (2.0f * n1) * cos1;
            float T_p = aspect / (n2 * cos1 + n1 * cos2);
            float T_s = aspect / (n2 * cos2 + n1 * cos1);
            ch[0].e1 = cmuls(E1, T_s);
            ch[0].e2 = cmuls(E2, T_p);
            ch[0].type = r.type & ~RP_REFL_RAY;
        }
        return 1;
    }
    // FullDielectric / FullDielectricDispersive
    double2 n1d, n2d;
    if (m.type == RP_MAT_FULL_DIELECTRIC) {
        double2 ni = make_double2(m.n_inside[0], m.n_inside[1]), no = make_double2(m.n_outside[0], m.n_outside[1]);
        n1d = out_to_in ? no : ni;
        n2d = out_to_in ? ni : no;
    } else {
        if ((long long)r.wl >= S.n_wl) {
            atomicOr(err, ERR_WAVELENGTH);
            return 0;
        }
        n1d = out_to_in ? nt_out : nt_in;
        n2d = out_to_in ? nt_in : nt_out;
    }
    const cf n1 = cf_of_d(n1d), n2 = cf_of_d(n2d);
    const float sin1 = sqrtf(fabsf(1.0f - cos1 * cos1));
    cf sin2 = cdiv(cmuls(n1, sin1), n2);
    cf cos2 = csqrtf_(csub(cfm(1.0f, 0.0f), cmul(sin2, sin2)));
    const float P_in = n1.x * (cabs2(E1) + cabs2(E2));
    if (P_in == 0.0f) return 0;
    cf n2c1 = cmuls(n2, cos1), n1c2 = cmul(n1, cos2), n2c2 = cmul(n2, cos2), n1c1 = cmuls(n1, cos1);
    cf den_p = cadd(n2c1, n1c2), den_s = cadd(n2c2, n1c1);
    cf R_p = cmul(cdiv(csub(n1c2, n2c1), den_p), E2);
    cf R_s = cmul(cdiv(csub(n1c1, n2c2), den_s), E1);
    int nc = 0;
    if ((n1.x * (cabs2(R_s) + cabs2(R_p))) / P_in > f_of_d(m.reflection_threshold)) {
        ch[0].d = ff3_sub(ind, ctn2);
        ch[0].e1 = R_s;
        ch[0].e2 = cfm(-R_p.x, -R_p.y);
        ch[0].n = n1d;
        ch[0].type = r.type | RP_REFL_RAY;
        nc = 1;
    }
    float aspect = sqrtf(cos2.x / cos1);
    cf num = cmuls(n1, 2.0f * cos1 * aspect);
    cf T_p = cmul(cdiv(num, den_p), E2);
    cf T_s = cmul(cdiv(num, den_s), E1);
    if ((n2.x * (cabs2(T_s) + cabs2(T_p))) / P_in > f_of_d(m.transmission_threshold)) {
        float c2unused;
        ChildF tc;  // filled here and copied to a fixed slot, so the children stay in registers
        tc.d = refract(ff_div(ff_of_d(n1d.x), ff_of_d(n2d.x)), c2unused);
        tc.e1 = T_s;
        tc.e2 = T_p;
        tc.n = n2d;
        tc.type = r.type & ~RP_REFL_RAY;
        if (nc)
            ch[1] = tc;
        else
            ch[0] = tc;
        nc++;
    }
    return nc;
}

// Writes one child from FP32 fields (exact widening on the integer pipe).
__device__ __forceinline__ void store_child_f(const RaySoA &out, unsigned long long k, const double *origin,
                                              f3 normal, f3 E, double opl, const ChildF &c, double phase,
                                              unsigned wl, unsigned parent, unsigned endf, unsigned ident) {
    out.ox[k] = origin[0];
    out.oy[k] = origin[1];
    out.oz[k] = origin[2];
    out.dx[k] = d_of_ff(c.d.x);
    out.dy[k] = d_of_ff(c.d.y);
    out.dz[k] = d_of_ff(c.d.z);
    out.nx[k] = d_of_f(normal.x);
    out.ny[k] = d_of_f(normal.y);
    out.nz[k] = d_of_f(normal.z);
    out.ex[k] = d_of_f(E.x);
    out.ey[k] = d_of_f(E.y);
    out.ez[k] = d_of_f(E.z);
    out.n[k] = c.n;
    out.e1[k] = make_double2(d_of_f(c.e1.x), d_of_f(c.e1.y));
    out.e2[k] = make_double2(d_of_f(c.e2.x), d_of_f(c.e2.y));
    out.len[k] = __longlong_as_double(0x7ff0000000000000LL);
    out.phase[k] = phase;
    out.opl[k] = opl;
    out.wl[k] = wl;
    out.parent[k] = parent;
    out.endf[k] = endf;
    out.ident[k] = ident;
    out.type[k] = c.type;
}

// ---- the nearest-hit search --------------------------------------------------------
struct Best {
    ff len;  // Euclidean distance of the nearest hit so far
    ff t;    // its ray parameter
    int face, list;
};

// The FP64 paths for faces and materials this kernel does not specialise are
// kept out of line so that their registers and stack do not weigh on the
// specialised path.

// DistortionFace.intersect_c in FP64 (distortion_isect, the same iteration
// step for step) with the distortion from its FP64 polynomial table instead
// of the reference's recursion: for the rays the FP32 iteration hands over
// (those that wander where the polynomials are large), which then need no
// workspace in local memory.
__device__ __noinline__ double distortion_t64(const DevScene &S, const rp_face &f, v3 p1, v3 p2, unsigned *err) {
    const rp_face &face = S.faces[f.base];
    double a1, a2, h = sepv(p2, p1);
    const double tolerance = f.p[0];
    a2 = face_isect_base(S, face, p1, p2, 0, err);
    if (a2 > h || a2 < f.tolerance) return RP_MISS;
    const v3 d = subv(p2, p1);
    v3 pt1 = addv(p1, mulvs(d, a2 / h));
    double gx, gy, gz;
    zk_eval64(S, f.distortion, pt1.x, pt1.y, true, gx, gy, gz);
    v3 n = face_normal_base(S, face, pt1);
    pt1.z += gz;
    n.x /= n.z;
    n.y /= n.z;
    n.x -= gx;
    n.y -= gy;
    v3 o = subv(p1, pt1);
    a1 = -h * dotv(o, n) / dotv(d, n);
    if (a1 < fabs(gz)) return RP_MISS;
    for (int i = 0; i < 20; i++) {
        pt1 = addv(p1, mulvs(d, a1 / h));
        if (fabs(a1 - a2) < tolerance) break;
        double zs, wx, wy;
        zk_eval64(S, f.distortion, pt1.x, pt1.y, false, wx, wy, zs);
        v3 q1 = p1, q2 = p2;
        q1.z -= zs;
        q2.z -= zs;
        a2 = face_isect_base(S, face, q1, q2, 0, err);
        pt1 = addv(q1, mulvs(d, a2 / h));
        n = face_normal_base(S, face, pt1);
        zk_eval64(S, f.distortion, pt1.x, pt1.y, true, gx, gy, gz);
        pt1.z += gz;
        n.x /= n.z;
        n.y /= n.z;
        n.x -= gx;
        n.y -= gy;
        o = subv(p1, pt1);
        a2 = a1;
        a1 = -h * dotv(o, n) / dotv(d, n);
    }
    if (!shape_inside(S, f.shape, pt1.x, pt1.y, err)) return RP_MISS;
    return a1;
}

// FP64 distance for a face type this kernel does not specialise (and for a
// DistortionFace its FP32 iteration handed over).
__device__ __forceinline__ double fallback_dist(const GenArgs &A, const DevScene &S, const rp_face &F, int f, int l,
                                                unsigned long long i) {
    const rp_facelist &L = S.lists[l];
    v3 o = mkv(A.in.ox[i], A.in.oy[i], A.in.oz[i]);
    v3 d = mkv(A.in.dx[i], A.in.dy[i], A.in.dz[i]);
    v3 pend = addv(o, mulvs(d, A.max_len));
    const v3 p1 = xform(L.inv_trans.m, L.inv_trans.t, o), p2 = xform(L.inv_trans.m, L.inv_trans.t, pend);
    if (distortion_line_misses(S.bounds + 16 * f, p1, p2)) return -1.0;  // cfaces.pyx NO_INTERSECTION
    if (F.type == RP_FACE_DISTORTION && mx_distortion_ok(S, F) && S.dists[F.distortion].type == RP_DIST_ZERNIKE)
        return distortion_t64(S, F, p1, p2, A.err);
    return face_isect(S, F, p1, p2, A.err);
}

// World normal of a face type this kernel does not specialise: the FP64
// normal at the local hit point, rotated, as float-float.
__device__ __noinline__ ff3 fallback_normal_ff(const DevScene &S, const rp_face &F, int l, v3 lp, unsigned *err) {
    v3 n64 = face_normal(S, F, lp, err);
    if (F.invert_normal) n64 = negv(n64);
    n64 = rotv(S.lists[l].trans.m, n64);
    return mkff3(ff_of_d(n64.x), ff_of_d(n64.y), ff_of_d(n64.z));
}

// Children of a material this kernel does not specialise (polarisers,
// waveplate, partial mirror, apertures, ...) through the FP64 path, after the
// termination filter; *term receives the number of children dropped by it.
__device__ __noinline__ int fallback_children(const GenArgs &A, const DevScene &S, const rp_face &F,
                                              const rp_material &Mt, int l, const RaySoA &Rr, unsigned long long i,
                                              double len, const double *origin, f3 nrm, ChildCommon *ccd, Child *chd,
                                              unsigned *term) {
    v3 tng = face_tangent(F);
    if (F.invert_normal) tng = negv(tng);
    tng = rotv(S.lists[l].trans.m, tng);
    RayState r;
    r.o = mkv(Rr.ox[i], Rr.oy[i], Rr.oz[i]);
    r.d = mkv(Rr.dx[i], Rr.dy[i], Rr.dz[i]);
    r.E = mkv(Rr.ex[i], Rr.ey[i], Rr.ez[i]);
    r.n = Rr.n[i];
    r.e1 = Rr.e1[i];
    r.e2 = Rr.e2[i];
    r.len = len;
    r.opl = Rr.opl[i];
    r.type = Rr.type[i];
    r.wl = Rr.wl[i];
    int nc = eval_children(S, Mt, r, mkv(origin[0], origin[1], origin[2]),
                           mkv(d_of_f(nrm.x), d_of_f(nrm.y), d_of_f(nrm.z)), tng, *ccd, chd, A.err);
    if (A.e2_term > 0.0 && nc > 0) {
        int w = 0;
        for (int k = 0; k < nc; k++) {
            if (!(child_e2(chd[k]) < A.e2_term)) {
                if (w != k) chd[w] = chd[k];
                w++;
            }
        }
        *term = (unsigned)(nc - w);
        nc = w;
    }
    return nc;
}


// Keeps the hit if it is nearer than b (the reference's strict `dist < length`,
// ties to the lower face index as in the oracle's order of evaluation).
__device__ __forceinline__ void keep_nearest(ff dist, ff t, int f, int l, Best &b) {
    if (ff_lt(dist, b.len) || (ff_eq(dist, b.len) && b.face >= 0 && f < b.face)) {
        b.len = dist;
        b.t = t;
        b.face = f;
        b.list = l;
    }
}

// A candidate for the nearest hit from phase one of a face test.
struct Cand {
    float d, t;   // FP32 distance along the ray and ray parameter
    int face, list;
    bool exact;   // a plane: tx is its float-float parameter already
    ff tx;
};
__device__ __forceinline__ void cand_clear(Cand &c) {
    c.d = __int_as_float(0x7f800000);
    c.t = 0.0f;
    c.face = -1;
    c.list = -1;
    c.exact = false;
    c.tx = ffm(0.0f, 0.0f);
}

// Phase one of a specialised face test (the caller checks MxFace.spec):
// keeps the two nearest candidates by FP32 distance (ties to the lower face
// record, as the exact comparison does).  True when the face's FP32 test
// could not decide (a DistortionFace's iteration that the FP64 path must run).
template <bool DIST>
__device__ __forceinline__ bool try_face32(const DevScene &S, const MxList *ml, const MxFace *mf, int f, int l,
                                           int &cur, LRay &R, const ff *O, const ff *D, float dl, float tmax,
                                           unsigned *err, Cand &c1, Cand &c2) {
    if (l != cur) {
        R = local_ray(ml[l], O, D);
        cur = l;
    }
    bool fb, exact;
    ff tx;
    const float t = face_t32<DIST>(S, S.faces[f], mf[f], R, tmax, dl, err, &tx, &exact, fb);
    if (fb) return true;
    if (!(t >= 0.0f)) return false;
    const float d = t * dl;
    if (!(mf[f].tol < d)) return false;
    Cand c;
    c.d = d;
    c.t = t;
    c.face = f;
    c.list = l;
    c.exact = exact;
    c.tx = tx;
    if (d < c1.d || (d == c1.d && f < c1.face)) {
        c2 = c1;
        c1 = c;
    } else if (d < c2.d || (d == c2.d && f < c2.face)) {
        c2 = c;
    }
    return false;
}

// Phase two for one candidate: its float-float parameter (bounds and the
// tolerance checked again on the refined value), kept in b when nearer.
template <bool DIST>
__device__ __forceinline__ void settle(const DevScene &S, const MxList *ml, const MxFace *mf, const Cand &c, int &cur,
                                       LRay &R, const ff *O, const ff *D, ff dlen, float tmax, Best &b) {
    if (c.face < 0) return;
    ff t;
    if (c.exact) {
        t = c.tx;
    } else {
        if (c.list != cur) {
            R = local_ray(ml[c.list], O, D);
            cur = c.list;
        }
        t = face_refine<DIST>(S, S.faces[c.face], mf[c.face], R, c.t);
        if (!(t.hi <= tmax) || !(t.hi >= mf[c.face].tmin)) return;
    }
    const ff dist = ff_mul(t, dlen);
    if (!(mf[c.face].tol < dist.hi)) return;
    keep_nearest(dist, t, c.face, c.list, b);
}

// The two candidates' refinement: the nearer always; the other when its FP32
// distance is within the FP32 roots' error of the nearer (so that the exact
// comparison, not FP32 rounding, decides between close hits) or when the
// nearer fails its refined checks.
template <bool DIST>
__device__ __forceinline__ void settle_best(const DevScene &S, const MxList *ml, const MxFace *mf, const Cand &c1,
                                            const Cand &c2, int &cur, LRay &R, const ff *O, const ff *D, ff dlen,
                                            float tmax, Best &b) {
    settle<DIST>(S, ml, mf, c1, cur, R, O, D, dlen, tmax, b);
    if (c2.face >= 0 && (b.face < 0 || c2.d <= fmaf(c1.d, 1.000244140625f, 1e-3f)))
        settle<DIST>(S, ml, mf, c2, cur, R, O, D, dlen, tmax, b);
}

// Tests a face through the FP64 path.  Out of line: called only for face types
// the specialised path does not handle, after the specialised search.
__device__ __noinline__ void try_face_fp64(const GenArgs &A, const DevScene &S, int f, int l, unsigned long long i,
                                           ff dlen, Best &b) {
    const rp_face &F = S.faces[f];
    double dd = fallback_dist(A, S, F, f, l, i);
    if (!(F.tolerance < dd)) return;  // also rejects NO_INTERSECTION (-1)
    ff dist = ff_of_d(dd);
    keep_nearest(dist, ff_div(dist, dlen), f, l, b);
}

// ---- input prefetch ----------------------------------------------------------
// One tile's input fields in shared memory (structure of arrays, one slot per
// thread).  Each thread copies its own ray's fields with cp.async, so a tile's
// loads are in flight while the previous tile computes, and a thread waits
// only for its own copies (cp.async.wait_group).
// The input fields of one sub-tile (32 rays, one warp).
struct TileIn {
    double ox[RP_SUB], oy[RP_SUB], oz[RP_SUB], dx[RP_SUB], dy[RP_SUB], dz[RP_SUB];
    double ex[RP_SUB], ey[RP_SUB], ez[RP_SUB];
    double2 n[RP_SUB], e1[RP_SUB], e2[RP_SUB];
    double opl[RP_SUB], phase[RP_SUB];
    unsigned wl[RP_SUB], type[RP_SUB], ident[RP_SUB];
    unsigned src[RP_SUB];  // the ray's index in `in` (through the gather map, or its own)
};
// The fields of a gathered input ray the kernel only passes through to its
// final record (one buffer per warp, filled while the sub-tile is searched).
struct PassIn {
    double nx[RP_SUB], ny[RP_SUB], nz[RP_SUB];
    unsigned parent[RP_SUB];
};

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
// Writes the traced input ray's record to its final place dst of `wb`: the
// prefetched fields from shared memory, normal and parent index from the
// record at src of `in`, and the segment's length and end face.
// Writes the traced input ray's record to its final place dst of `wb`: the
// prefetched fields from shared memory and the segment's length and end face.
__device__ __forceinline__ void write_back(const TileIn &b, const PassIn &p, unsigned t, const RaySoA &wb,
                                           unsigned long long dst, double len, unsigned endf) {
    const double nx = p.nx[t], ny = p.ny[t], nz = p.nz[t];
    const unsigned parent = p.parent[t];
    wb.ox[dst] = b.ox[t]; wb.oy[dst] = b.oy[t]; wb.oz[dst] = b.oz[t];
    wb.dx[dst] = b.dx[t]; wb.dy[dst] = b.dy[t]; wb.dz[dst] = b.dz[t];
    wb.ex[dst] = b.ex[t]; wb.ey[dst] = b.ey[t]; wb.ez[dst] = b.ez[t];
    wb.n[dst] = b.n[t]; wb.e1[dst] = b.e1[t]; wb.e2[dst] = b.e2[t];
    wb.len[dst] = len; wb.phase[dst] = b.phase[t]; wb.opl[dst] = b.opl[t];
    wb.wl[dst] = b.wl[t]; wb.endf[dst] = endf; wb.ident[dst] = b.ident[t]; wb.type[dst] = b.type[t];
    wb.nx[dst] = nx; wb.ny[dst] = ny; wb.nz[dst] = nz; wb.parent[dst] = parent;
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev2() { asm volatile("cp.async.wait_group 2;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Queues the copy of ray i's fields into the lane's slot of `buf` (nothing
// for i beyond the generation) and closes the thread's copy group.
// Only origin and direction are copied for a ray traced in place (`full`
// false): the search kernel then writes just its length and end face.
__device__ __forceinline__ void prefetch_ray(TileIn *buf, const RaySoA &in, unsigned long long i, unsigned long long n,
                                             unsigned long long s, bool full) {
    if (i < n) {  // ray i of the generation; its record is s of `in`
        const unsigned t = threadIdx.x & 31;
        buf->src[t] = (unsigned)s;
        cp_async8(&buf->ox[t], &in.ox[s]);
        cp_async8(&buf->oy[t], &in.oy[s]);
        cp_async8(&buf->oz[t], &in.oz[s]);
        cp_async8(&buf->dx[t], &in.dx[s]);
        cp_async8(&buf->dy[t], &in.dy[s]);
        cp_async8(&buf->dz[t], &in.dz[s]);
        if (full) {
            cp_async8(&buf->ex[t], &in.ex[s]);
            cp_async8(&buf->ey[t], &in.ey[s]);
            cp_async8(&buf->ez[t], &in.ez[s]);
            cp_async16(&buf->n[t], &in.n[s]);
            cp_async16(&buf->e1[t], &in.e1[s]);
            cp_async16(&buf->e2[t], &in.e2[s]);
            cp_async8(&buf->opl[t], &in.opl[s]);
            cp_async8(&buf->phase[t], &in.phase[s]);
            cp_async4(&buf->wl[t], &in.wl[s]);
            cp_async4(&buf->type[t], &in.type[s]);
            cp_async4(&buf->ident[t], &in.ident[s]);
        }
    }
    cp_async_commit();
}

// Queues the copy of the pass-through fields of record s (no commit).
__device__ __forceinline__ void prefetch_pass(PassIn *p, const RaySoA &in, unsigned long long s) {
    const unsigned t = threadIdx.x & 31;
    cp_async8(&p->nx[t], &in.nx[s]);
    cp_async8(&p->ny[t], &in.ny[s]);
    cp_async8(&p->nz[t], &in.nz[s]);
    cp_async4(&p->parent[t], &in.parent[s]);
}

// Takes the warp's next sub-tile from the launch-wide counter.
__device__ __forceinline__ unsigned claim_sub_tile(unsigned *counter, unsigned lane) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(counter, 1u);
    return __shfl_sync(0xffffffffu, t, 0);
}

// The gather-map entry of this lane's ray in sub-tile `tile` (0 when there is
// none), loaded a sub-tile ahead of its use so that its latency is hidden.
__device__ __forceinline__ unsigned map_entry(const GenArgs &A, unsigned tile, unsigned lane, unsigned long long n_sub) {
    const unsigned long long i = (unsigned long long)tile * RP_SUB + lane;
    return (A.in_map && tile < n_sub && i < A.n_in) ? A.in_map[i] : 0u;
}

}  // namespace mx

// A ray's entry distance into a padded world box b (lo xyz, hi xyz;
// rp_bounds.h): the FP32 slab test with the inverse direction (ix, iy, iz),
// infinity when the ray misses the box or it lies behind.
__device__ __forceinline__ float mx_box_enter(const float *b, float ox, float oy, float oz, float ix, float iy,
                                              float iz) {
    float t1 = (b[0] - ox) * ix, t2 = (b[3] - ox) * ix;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b[1] - oy) * iy;
    t2 = (b[4] - oy) * iy;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    t1 = (b[2] - oz) * iz;
    t2 = (b[5] - oz) * iz;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    if (!(tmax >= tmin) || tmax < 0.0f) return __int_as_float(0x7f800000);
    return fmaxf(tmin, 0.0f);
}

// A face's entry distance in the mixed search.  b: its 16 floats of
// S.bounds; b[6] = 1, its box's entry; 3, the nearer entry of its two boxes
// (b[0..7], b[8..15]); 2 (a DistortionFace, in the form of the kernels that
// carry its code), its prism's entry (prism_enter, u the ray's unit
// direction); otherwise 0 (a face without a box is always tested).
template <bool FB>
__device__ __forceinline__ float mx_face_enter(const float *b, float ox, float oy, float oz, float ix, float iy,
                                               float iz, float ux, float uy, float uz) {
    if (b[6] != 1.0f) {
        if (b[6] == 3.0f)
            return fminf(mx_box_enter(b, ox, oy, oz, ix, iy, iz), mx_box_enter(b + 8, ox, oy, oz, ix, iy, iz));
        if constexpr (FB)
            if (b[6] == 2.0f) return prism_enter(b, ox, oy, oz, ux, uy, uz);
        return 0.0f;
    }
    return mx_box_enter(b, ox, oy, oz, ix, iy, iz);
}


namespace mx {
// Inserts box entry te of face f into the ordered queue (q0, f0) <= (q1, f1)
// <= (q2, f2) of the three nearest entries.
__device__ __forceinline__ void queue_insert(float te, int f, float &q0, float &q1, float &q2, int &f0, int &f1,
                                             int &f2) {
    if (te < q2) {
        if (te < q1) {
            q2 = q1;
            f2 = f1;
            if (te < q0) {
                q1 = q0;
                f1 = f0;
                q0 = te;
                f0 = f;
            } else {
                q1 = te;
                f1 = f;
            }
        } else {
            q2 = te;
            f2 = f;
        }
    }
}

// A thread's box-entry table in shared memory: face f's entry at
// tb[f * RP_BLOCK], as FP32, or as FP16 rounded down (a lower bound: the
// nearest-first order and its stopping test stay valid) for tables of more
// than 32 faces, which then still take 16 KB a block at most.
__device__ __forceinline__ void tb_put(float *tb, int f, float te) { tb[f * RP_BLOCK] = te; }
__device__ __forceinline__ void tb_put(__half *tb, int f, float te) { tb[f * RP_BLOCK] = __float2half_rd(te); }
__device__ __forceinline__ float tb_get(const float *tb, int f) { return tb[f * RP_BLOCK]; }
__device__ __forceinline__ float tb_get(const __half *tb, int f) { return __half2float(tb[f * RP_BLOCK]); }

// Position of the r-th (from 0) set bit of m; m has more than r set bits.
__device__ __forceinline__ unsigned nth_set_bit(unsigned m, unsigned r) {
    unsigned pos = 0;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) {
        const unsigned low = __popc(m & ((1u << w) - 1u));
        if (r >= low) {
            r -= low;
            m >>= w;
            pos += w;
        }
    }
    return pos;
}

// Whether a hit on face record f goes to the material kernel (its material
// can produce children).
__device__ __forceinline__ bool makes_children(const DevScene &S, int f) {
    const int mat = S.faces[f].material;
    if (mat < 0) return false;
    const int t = S.mats[mat].type;
    return t != RP_MAT_NONE && t != RP_MAT_OPAQUE;
}
}  // namespace mx

// Resident blocks per SM the two kernels are compiled for: three (168
// registers a thread) for both; at four (128 registers) the spills cost more
// than the extra warps hide (config 2: 20.3 against 19.4 ms per step; the
// material kernel alone at two blocks: 22.3 ms).
#define MX_SEARCH_MIN_BLOCKS 3
#define MX_MAT_MIN_BLOCKS 3

// The nearest hit of one ray (origin and direction od[0..5], its record src
// of A.in for the FP64 faces): culled nearest-first FP32 candidates among the
// specialised faces, the winner (and a close second) refined in float-float,
// then the faces left to the FP64 path.  tb is the thread's table of the box
// entries of the first 64 faces in shared memory (tb_put / tb_get).
template <bool FB, typename TbT>
__device__ __forceinline__ mx::Best nearest_mx(const GenArgs &A, const DevScene &S, const mx::MxList *ml,
                                               const mx::MxFace *mf, TbT *tb, float max_len, const double *od,
                                               unsigned long long src) {
    using namespace mx;
    Best b;
    b.len = ffm(max_len, 0.0f);
    b.t = ffm(0.0f, 0.0f);
    b.face = -1;
    b.list = -1;
    ff O[3], D[3];
    O[0] = ff_of_d(od[0]);
    O[1] = ff_of_d(od[1]);
    O[2] = ff_of_d(od[2]);
    D[0] = ff_of_d(od[3]);
    D[1] = ff_of_d(od[4]);
    D[2] = ff_of_d(od[5]);
    const ff dlen = ff_sqrt(ff_add(ff_add(ff_mul(D[0], D[0]), ff_mul(D[1], D[1])), ff_mul(D[2], D[2])));
    int cur = -1;
    LRay R;
    unsigned long long pend = 0;  // culled faces left to the FP64 path
    Cand c1, c2;                  // the two nearest FP32 candidates of the specialised faces
    cand_clear(c1);
    cand_clear(c2);
    const float dl = dlen.hi;
    if (A.one_list >= 0) {
        // sequential trace: one face of one list (FaceList.intersect_one_face_c, ctracer.pyx:1861-1879)
        const int f = S.lists[A.one_list].first_face + A.one_face;
        bool fp64 = !mf[f].spec;
        if (!fp64) {
            fp64 = try_face32<FB>(S, ml, mf, f, A.one_list, cur, R, O, D, dl, max_len, A.err, c1, c2);
            settle_best<FB>(S, ml, mf, c1, c2, cur, R, O, D, dlen, max_len, b);
        }
        if constexpr (FB)
            if (fp64) try_face_fp64(A, S, f, A.one_list, src, dlen, b);
    } else {
        // culled nearest-first search over the first 64 faces, then the rest in order
        const float dfx = D[0].hi, dfy = D[1].hi, dfz = D[2].hi;
        const float il = rsqrtf(dfx * dfx + dfy * dfy + dfz * dfz);
        const float ix = 1.0f / ((fabsf(dfx * il) < 1e-30f) ? copysignf(1e-30f, dfx) : dfx * il);
        const float iy = 1.0f / ((fabsf(dfy * il) < 1e-30f) ? copysignf(1e-30f, dfy) : dfy * il);
        const float iz = 1.0f / ((fabsf(dfz * il) < 1e-30f) ? copysignf(1e-30f, dfz) : dfz * il);
        const float ox = O[0].hi, oy = O[1].hi, oz = O[2].hi;
        const float ux = dfx * il, uy = dfy * il, uz = dfz * il;  // (FB: distortion faces' prisms)
        const int nf = S.n_faces;
        const int nmask = nf < 64 ? nf : 64;
        const float lim0 = max_len * 1.000001f + 1e-4f;
        unsigned long long cand = 0;
        // the three nearest box entries, in order, kept in registers while the
        // boxes are entered: most rays test one to three faces, so the
        // selection below rarely has to scan the candidates again
        const float INF = __int_as_float(0x7f800000);
        float q0 = INF, q1 = INF, q2 = INF;
        int f0 = -1, f1 = -1, f2 = -1;
        for (int f = 0; f < nmask; f++) {
            const float te = mx_face_enter<FB>(S.bounds + 16 * f, ox, oy, oz, ix, iy, iz, ux, uy, uz);
            tb_put(tb, f, te);
            if (te <= lim0) {
                cand |= 1ull << f;
                queue_insert(te, f, q0, q1, q2, f0, f1, f2);
            }
        }
        while (cand) {
            if (f0 < 0) {
                // the queue ran out: refill it with the three nearest entries
                // of the candidates left, in one pass over them
                q0 = q1 = q2 = INF;
                f1 = f2 = -1;
                for (unsigned long long m = cand; m; m &= m - 1) {
                    const int f = __ffsll((long long)m) - 1;
                    queue_insert(tb_get(tb, f), f, q0, q1, q2, f0, f1, f2);
                }
            }
            // the front of the register queue: no candidate left in `cand`
            // enters its box before it
            const float tsel = q0;
            const int sel = f0;
            q0 = q1;
            f0 = f1;
            q1 = q2;
            f1 = f2;
            f2 = -1;
            // boxes entered beyond the nearest FP32 candidate (with a
            // margin above the FP32 roots' error) cannot hold a nearer hit
            if (sel < 0 || tsel > fmaf(c1.d, 1.000244140625f, 1e-3f)) break;
            cand &= ~(1ull << sel);
            int l = S.face_list[sel];
            if (l < 0 || l >= S.n_lists) {
                atomicOr(A.err, ERR_SHAPE_STACK);
                break;
            }
            // a face the FP32 test cannot decide goes to the FP64 faces below
            // (a scene without FP64 faces has only faces the FP32 test decides)
            if constexpr (FB) {
                if (!mf[sel].spec || try_face32<FB>(S, ml, mf, sel, l, cur, R, O, D, dl, max_len, A.err, c1, c2))
                    pend |= 1ull << sel;
            } else {
                try_face32<FB>(S, ml, mf, sel, l, cur, R, O, D, dl, max_len, A.err, c1, c2);
            }
        }
        for (int f = nmask; f < nf; f++) {
            if (!mf[f].spec) continue;
            const float te = mx_face_enter<FB>(S.bounds + 16 * f, ox, oy, oz, ix, iy, iz, ux, uy, uz);
            if (te > fmaf(c1.d, 1.000244140625f, 1e-3f)) continue;
            int l = S.face_list[f];
            if (l < 0 || l >= S.n_lists) {
                atomicOr(A.err, ERR_SHAPE_STACK);
                break;
            }
            const bool fp64 = try_face32<FB>(S, ml, mf, f, l, cur, R, O, D, dl, max_len, A.err, c1, c2);
            if constexpr (FB)
                if (fp64) try_face_fp64(A, S, f, l, src, dlen, b);
        }
        settle_best<FB>(S, ml, mf, c1, c2, cur, R, O, D, dlen, max_len, b);
        // the FP64 faces: the nearest hit does not depend on the order of
        // the tests, and the box bound stays valid against the final length
        for (int f = 0; FB && f < nf; f++) {
            if (f < nmask) {
                if (!((pend >> f) & 1ull)) continue;
                if (tb_get(tb, f) > b.len.hi * 1.000001f + 1e-4f) continue;
            } else {
                if (mf[f].spec) continue;
                const float te = mx_face_enter<FB>(S.bounds + 16 * f, ox, oy, oz, ix, iy, iz, ux, uy, uz);
                if (te > b.len.hi * 1.000001f + 1e-4f) continue;
            }
            int l = S.face_list[f];
            if (l < 0 || l >= S.n_lists) {
                atomicOr(A.err, ERR_SHAPE_STACK);
                break;
            }
            if constexpr (FB) try_face_fp64(A, S, f, l, src, dlen, b);
        }
    }
    return b;
}

// ---- the search kernel ------------------------------------------------------------
// One block stages the tables once; then each of its warps takes 32-ray
// sub-tiles from a launch-wide counter until none are left, with no barrier
// between warps, so the staging is paid once per resident block and neither
// a slow sub-tile nor a slow warp holds up the others.  The next sub-tile's
// fields are copied into the warp's other shared-memory buffer (cp.async)
// while the current one is searched.  For each ray: the nearest hit (culled
// nearest-first over the specialised faces, then the FP64 faces), then the
// ray's final record with its length and end face (gathered input) or just
// those two fields (in place), and, when the generation keeps children, the
// hit's ray parameter and face record for the material kernel.
// Dynamic shared memory: the plain kernel's tables, the mixed tables at
// mx_off, each thread's box-entry distance per culled face at tb_off, the
// warps' input buffers at in_off and pass-through buffers at pass_off.
// TbT: the type of the box-entry table (tb_put), which the refills of the
// queue of nearest entries read instead of entering the boxes again: FP32
// for scenes of up to RP_MX_TB_F32_FACES faces, FP16 above (the first 64
// faces; 16 KB a block, so three blocks still fit an SM).  The FP16 table's
// conversions cost about 2 % of the search on an 11-face scene; a 41-face
// scene's search takes 15 % less with it than re-entering the boxes.
#define RP_MX_TB_F32_FACES 32
// (The form with the FP64 fallback is compiled for two blocks per SM: the
// scenes that need it hold two by shared memory already -- the 64-face clutter
// scene, 109 KB a block -- and at 255 registers it spills 0.3 instead of 1.4 KB
// a thread: 797 against 834 ms per 1M-ray clutter step.)
template <bool FB, typename TbT>
__global__ void __launch_bounds__(RP_BLOCK, FB ? 2 : MX_SEARCH_MIN_BLOCKS)
    mixed_search_kernel(GenArgs A, unsigned mx_off, unsigned tb_off, unsigned in_off, unsigned pass_off) {
    using namespace mx;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_hits;
    const unsigned lane = threadIdx.x & 31;
    TileIn *bufs = reinterpret_cast<TileIn *>(smem + in_off) + 2 * (threadIdx.x >> 5);
    PassIn *pass = reinterpret_cast<PassIn *>(smem + pass_off) + (threadIdx.x >> 5);
    unsigned *s_counts;
    DevScene S = stage_tables(A, smem, &s_counts);
    MxList *ml = reinterpret_cast<MxList *>(smem + mx_off);
    MxFace *mf = reinterpret_cast<MxFace *>(ml + A.S.n_lists);
    TbT *tb = reinterpret_cast<TbT *>(smem + tb_off) + threadIdx.x;  // tb[f * RP_BLOCK]
    const float max_len = f_of_d(A.max_len);  // exact: max_length is a float
    stage_mixed(A, ml, mf, max_len);
    if (threadIdx.x == 0) s_hits = 0;
    const unsigned long long n_sub = rp_n_sub(A.n_in);
    __syncthreads();  // the staged tables and the counter are ready

    const bool gathered = A.in_map != nullptr;
    unsigned tile = claim_sub_tile(A.tile_next, lane);
    if (tile < n_sub) {
        const unsigned long long i0 = (unsigned long long)tile * RP_SUB + lane;
        prefetch_ray(&bufs[0], A.in, i0, A.n_in, gathered ? (unsigned long long)map_entry(A, tile, lane, n_sub) : i0,
                     gathered);
    }
    unsigned next = claim_sub_tile(A.tile_next, lane);
    unsigned next_src = map_entry(A, next, lane, n_sub);
    for (unsigned k = 0;; k++) {
        if (tile >= n_sub) break;
        const unsigned next2 = claim_sub_tile(A.tile_next, lane);
        const unsigned next2_src = map_entry(A, next2, lane, n_sub);
        const TileIn &in = bufs[k & 1];
        const unsigned t = lane;
        const unsigned long long i = (unsigned long long)tile * RP_SUB + lane;
        const bool active = i < A.n_in;
        if (gathered) {
            // pass-through fields of this sub-tile: their own copy group, awaited at the write-back
            if (active) prefetch_pass(pass, A.in, in.src[t]);
            cp_async_commit();
        }
        const unsigned long long ni = (unsigned long long)next * RP_SUB + lane;
        if (next < n_sub)
            prefetch_ray(&bufs[(k + 1) & 1], A.in, ni, A.n_in, gathered ? (unsigned long long)next_src : ni, gathered);
        else
            cp_async_commit();
        // this thread's copies for `tile` have landed (the pass-through group
        // and the next sub-tile's group may still be in flight)
        if (gathered)
            cp_async_wait_prev2();
        else
            cp_async_wait_prev();
        const unsigned long long src = active && gathered ? (unsigned long long)in.src[t] : i;  // the record in A.in

        if (active) {
            const double od[6] = {in.ox[t], in.oy[t], in.oz[t], in.dx[t], in.dy[t], in.dz[t]};
            const Best b = nearest_mx<FB, TbT>(A, S, ml, mf, tb, max_len, od, src);
            const double len64 = d_of_ff(b.len);
            const unsigned endf = b.face >= 0 ? (unsigned)S.faces[b.face].idx : 0xFFFFFFFFu;
            if (gathered) {
                cp_async_wait_prev();  // the pass-through group
                write_back(in, *pass, t, A.wb, i, len64, endf);
            } else {
                A.in.len[i] = len64;
                A.in.endf[i] = endf;
            }
            if (A.emit) {
                A.hit_t[i] = make_float2(b.t.hi, b.t.lo);
                A.hit_face[i] = b.face;
            }
            if (b.face >= 0) {
                atomicAdd(&s_counts[b.face], 1u);
                atomicAdd(&s_hits, 1u);
            }
        }
        tile = next;
        next = next2;
        next_src = next2_src;
    }
    flush_counts(A, S, s_counts);
    if (threadIdx.x == 0) atomicAdd(&A.stats[0], (unsigned long long)s_hits);
}

// ---- the material kernel ----------------------------------------------------------
namespace mx {
// One chunk's inputs for the material kernel: the fields of up to 32 hit
// rays (structure of arrays, one slot per lane) with their hand-over.
struct MatIn {
    double ox[RP_SUB], oy[RP_SUB], oz[RP_SUB], dx[RP_SUB], dy[RP_SUB], dz[RP_SUB];
    double ex[RP_SUB], ey[RP_SUB], ez[RP_SUB];
    double2 n[RP_SUB], e1[RP_SUB], e2[RP_SUB];
    double opl[RP_SUB], phase[RP_SUB];
    float2 t[RP_SUB];
    unsigned wl[RP_SUB], type[RP_SUB], ident[RP_SUB];
    int face[RP_SUB];
    unsigned idx[RP_SUB];  // the ray's index in the generation; 0xffffffff for an idle lane
};

// A group's rays that go to the material kernel: per 32-ray quarter the
// ballot of hits whose material can produce children, and their prefix counts.
struct GroupMask {
    unsigned q;           // the group (within its job); n_groups when none is left
    unsigned m[RP_GROUP / 32];
    unsigned p1, p2, p3, total;
    int job;              // its job in a batch (0 otherwise)
};

// A group claimed a group ahead of its use: its index and this lane's four
// hit-face records, loaded when it is claimed so that the loads (and the
// claim's atomic) complete while the warp evaluates the current group.
struct GroupAhead {
    unsigned q;
    int hf[RP_GROUP / 32];
};

__device__ __forceinline__ void claim_ahead(const GenArgs &A, unsigned long long n_groups, unsigned lane,
                                            GroupAhead &H) {
    H.q = claim_sub_tile(A.group_next, lane);
    const unsigned long long g0 = (unsigned long long)H.q * RP_GROUP;
#pragma unroll
    for (int c = 0; c < RP_GROUP / 32; c++) {
        const unsigned long long i = g0 + 32 * c + lane;
        H.hf[c] = (H.q < n_groups && i < A.n_in) ? A.hit_face[i] : -1;
    }
}

// Takes the group claimed ahead in H (claiming the next one into H at once)
// until one has material rays (a group without any gets its zero child count
// at once); G.q = n_groups when none is left.
__device__ __forceinline__ void next_group(const GenArgs &A, const DevScene &S, unsigned long long n_groups,
                                           unsigned lane, GroupAhead &H, GroupMask &G) {
    G.job = 0;
    for (;;) {
        const GroupAhead cur = H;
        G.q = cur.q;
        G.total = 0;
        if (cur.q >= n_groups) return;
        claim_ahead(A, n_groups, lane, H);
#pragma unroll
        for (int c = 0; c < RP_GROUP / 32; c++) {
            const int f = cur.hf[c];
            G.m[c] = __ballot_sync(0xffffffffu, f >= 0 && f < S.n_faces && makes_children(S, f));
        }
        G.p1 = __popc(G.m[0]);
        G.p2 = G.p1 + __popc(G.m[1]);
        G.p3 = G.p2 + __popc(G.m[2]);
        G.total = G.p3 + __popc(G.m[3]);
        if (G.total > 0) return;
        if (lane == 0) A.tile_counts[cur.q] = 0u;
    }
}

// The same over a batch: global groups taken from the batch's counter, each
// returned as its job and its group within the job; G.job = -1 when none is
// left.
// (claimed ahead as in the single-job kernel: the global group, its job and
// this lane's four hit-face records)
struct BatchAhead {
    unsigned u;
    int j;
    int hf[RP_GROUP / 32];
};

__device__ __forceinline__ void claim_ahead_batch(const BatchDev *Bt, unsigned *ctr, unsigned lane, BatchAhead &H) {
    H.u = claim_sub_tile(&ctr[1], lane);
    H.j = -1;
#pragma unroll
    for (int c = 0; c < RP_GROUP / 32; c++) H.hf[c] = -1;
    if (H.u >= Bt->total_units) return;
    H.j = batch_job_of(Bt, H.u);
    const GenArgs &A = Bt->jobs[H.j].a;
    const unsigned long long g0 = (unsigned long long)(H.u - Bt->unit_start[H.j]) * RP_GROUP;
#pragma unroll
    for (int c = 0; c < RP_GROUP / 32; c++) {
        const unsigned long long i = g0 + 32 * c + lane;
        if (i < A.n_in && A.emit) H.hf[c] = A.hit_face[i];
    }
}

__device__ __forceinline__ void next_group_batch(const BatchDev *Bt, unsigned *ctr, unsigned lane, BatchAhead &H,
                                                 GroupMask &G) {
    for (;;) {
        const BatchAhead cur = H;
        G.total = 0;
        if (cur.u >= Bt->total_units) {
            G.job = -1;
            G.q = 0;
            return;
        }
        claim_ahead_batch(Bt, ctr, lane, H);
        const GenArgs &A = Bt->jobs[cur.j].a;
        G.job = cur.j;
        G.q = cur.u - Bt->unit_start[cur.j];
#pragma unroll
        for (int c = 0; c < RP_GROUP / 32; c++) {
            const int f = cur.hf[c];
            G.m[c] = __ballot_sync(0xffffffffu, f >= 0 && f < A.S.n_faces && makes_children(A.S, f));
        }
        G.p1 = __popc(G.m[0]);
        G.p2 = G.p1 + __popc(G.m[1]);
        G.p3 = G.p2 + __popc(G.m[2]);
        G.total = G.p3 + __popc(G.m[3]);
        if (G.total > 0) return;
        if (lane == 0) A.tile_counts[G.q] = 0u;
    }
}

// The ray of chunk k of group G that this lane evaluates (in ray order), or
// ~0 when the chunk has fewer rays than lanes.
__device__ __forceinline__ unsigned long long chunk_ray(const GroupMask &G, unsigned k, unsigned lane) {
    const unsigned o = 32 * k + lane;
    if (o >= G.total) return ~0ull;
    unsigned c, base, m;
    if (o < G.p1) {
        c = 0; base = 0; m = G.m[0];
    } else if (o < G.p2) {
        c = 1; base = G.p1; m = G.m[1];
    } else if (o < G.p3) {
        c = 2; base = G.p2; m = G.m[2];
    } else {
        c = 3; base = G.p3; m = G.m[3];
    }
    return (unsigned long long)G.q * RP_GROUP + 32 * c + nth_set_bit(m, o - base);
}

// Queues the copies of ray i's inputs into the lane's slot of B (nothing for
// i = ~0) and closes the lane's copy group.
__device__ __forceinline__ void prefetch_mat(MatIn *B, const GenArgs &A, const RaySoA &Rr, unsigned long long i,
                                             unsigned lane) {
    B->idx[lane] = i == ~0ull ? 0xffffffffu : (unsigned)i;
    if (i != ~0ull) {
        cp_async8(&B->ox[lane], &Rr.ox[i]);
        cp_async8(&B->oy[lane], &Rr.oy[i]);
        cp_async8(&B->oz[lane], &Rr.oz[i]);
        cp_async8(&B->dx[lane], &Rr.dx[i]);
        cp_async8(&B->dy[lane], &Rr.dy[i]);
        cp_async8(&B->dz[lane], &Rr.dz[i]);
        cp_async8(&B->ex[lane], &Rr.ex[i]);
        cp_async8(&B->ey[lane], &Rr.ey[i]);
        cp_async8(&B->ez[lane], &Rr.ez[i]);
        cp_async16(&B->n[lane], &Rr.n[i]);
        cp_async16(&B->e1[lane], &Rr.e1[i]);
        cp_async16(&B->e2[lane], &Rr.e2[i]);
        cp_async8(&B->opl[lane], &Rr.opl[i]);
        cp_async8(&B->phase[lane], &Rr.phase[i]);
        cp_async8(&B->t[lane], &A.hit_t[i]);
        cp_async4(&B->wl[lane], &Rr.wl[i]);
        cp_async4(&B->type[lane], &Rr.type[i]);
        cp_async4(&B->ident[lane], &Rr.ident[i]);
        cp_async4(&B->face[lane], &A.hit_face[i]);
    }
    cp_async_commit();
}
}  // namespace mx

// The material evaluation of one hit ray of a chunk (lane t of buffer B, ray
// i of the generation's records Rr): hit point, normal and optical path
// rebuilt from the record and the hand-over's ray parameter, then the
// material's children (FP32 / float-float, or the FP64 path's for materials
// not specialised here) with the |E|^2 rule applied.
template <bool FB>
__device__ __forceinline__ void material_mx(const GenArgs &A, const DevScene &S, const mx::MxList *ml,
                                            const mx::MxFace *mf, const RaySoA &Rr, const mx::MatIn &B, unsigned t,
                                            unsigned long long i, float e2t, unsigned *s_term, int &nc,
                                            mx::ChildF *ch, mx::f3 &nrm, mx::f3 &Eo, double *origin, double &opl,
                                            bool &fp64_children, Child *chd, ChildCommon &ccd, int &face) {
    using namespace mx;
    face = B.face[t];
    const ff tt = ffm(B.t[t].x, B.t[t].y);
    const rp_face &F = S.faces[face];
    const int l = S.face_list[face];
    // a dispersive material's indices at the ray's wavelength: scattered
    // loads, issued here so that they land while the hit point and normal
    // are computed
    double2 nt_in = make_double2(0.0, 0.0), nt_out = make_double2(0.0, 0.0);
    {
        const rp_material &Mn = S.mats[F.material];
        const long long w = (long long)B.wl[t];
        if (Mn.type == RP_MAT_FULL_DIELECTRIC_DISPERSIVE && w < S.n_wl) {
            nt_in = S.ntab[(long long)Mn.curve_inside * S.n_wl + w];
            nt_out = S.ntab[(long long)Mn.curve_outside * S.n_wl + w];
        }
    }
    if (l < 0 || l >= S.n_lists) {
        atomicOr(A.err, ERR_SHAPE_STACK);
    } else {
        const MxFace &M = mf[face];
        const MxList &L = ml[l];
        ff O[3], D[3];
        O[0] = ff_of_d(B.ox[t]);
        O[1] = ff_of_d(B.oy[t]);
        O[2] = ff_of_d(B.oz[t]);
        D[0] = ff_of_d(B.dx[t]);
        D[1] = ff_of_d(B.dy[t]);
        D[2] = ff_of_d(B.dz[t]);
        const ff dlen = ff_sqrt(ff_add(ff_add(ff_mul(D[0], D[0]), ff_mul(D[1], D[1])), ff_mul(D[2], D[2])));
        const ff lenff = ff_mul(tt, dlen);
        ff P[3];
        P[0] = ff_add(O[0], ff_mul(tt, D[0]));
        P[1] = ff_add(O[1], ff_mul(tt, D[1]));
        P[2] = ff_add(O[2], ff_mul(tt, D[2]));
        origin[0] = d_of_ff(P[0]);
        origin[1] = d_of_ff(P[1]);
        origin[2] = d_of_ff(P[2]);
        // the hit in the face list's frame, relative to the face vertex
        ff lp[3];
        if (L.ident) {
            lp[0] = ff_add(P[0], ff_of(L.ti_hi, L.ti_lo, 0));
            lp[1] = ff_add(P[1], ff_of(L.ti_hi, L.ti_lo, 1));
            lp[2] = ff_add(P[2], ff_of(L.ti_hi, L.ti_lo, 2));
        } else {
            ff_rotate(L, P, lp, true);
        }
        ff3 nn;
        if (face_normal_ff<FB>(S, F, M, lp[0], lp[1], ff_sub(lp[2], ffm(M.zv_hi, M.zv_lo)), nn)) {
            if (F.invert_normal) nn = ff3_neg(nn);
            if (!L.ident) {
                ff v[3] = {nn.x, nn.y, nn.z}, w[3];
#pragma unroll
                for (int rr = 0; rr < 3; rr++)
                    w[rr] = ff_add(ff_add(ff_mul(ff_of(L.r_hi, L.r_lo, 3 * rr), v[0]),
                                          ff_mul(ff_of(L.r_hi, L.r_lo, 3 * rr + 1), v[1])),
                                   ff_mul(ff_of(L.r_hi, L.r_lo, 3 * rr + 2), v[2]));
                nn = mkff3(w[0], w[1], w[2]);
            }
        } else if constexpr (FB) {
            nn = fallback_normal_ff(S, F, l, mkv(d_of_ff(lp[0]), d_of_ff(lp[1]), d_of_ff(lp[2])), A.err);
        }
        nrm = mk3(nn.x.hi, nn.y.hi, nn.z.hi);
        const rp_material &Mt = S.mats[F.material];
        const double2 nin = B.n[t];
        opl = d_of_ff(ff_add(ff_of_d(B.opl[t]), ff_mul(lenff, ff_of_d(nin.x))));
        if (mat_specialised(Mt.type)) {
            RayF r;
            r.d = mk3(D[0].hi, D[1].hi, D[2].hi);
            r.E = f3_of_d(B.ex[t], B.ey[t], B.ez[t]);
            r.e1 = cf_of_d(B.e1[t]);
            r.e2 = cf_of_d(B.e2[t]);
            r.n = nin;
            r.type = B.type[t];
            r.wl = B.wl[t];
            const ff3 Dff = mkff3(D[0], D[1], D[2]);
            const ff idl = ff_div(ffm(1.0f, 0.0f), dlen);
            nc = eval_f(S, Mt, r, Dff, ff3_scale(Dff, idl), nn, Eo, ch, A.err, nt_in, nt_out);
            if (A.e2_term > 0.0 && nc > 0) {
                // the |E|^2 rule, children kept in order (fixed indices: registers)
                const bool k0 = !(cabs2(ch[0].e1) + cabs2(ch[0].e2) < e2t);
                const bool k1 = nc > 1 && !(cabs2(ch[1].e1) + cabs2(ch[1].e2) < e2t);
                if (!k0 && k1) ch[0] = ch[1];
                const int w = (int)k0 + (int)k1;
                if (w < nc) atomicAdd(s_term, (unsigned)(nc - w));
                nc = w;
            }
        } else if constexpr (FB) {
            unsigned term = 0;
            nc = fallback_children(A, S, F, Mt, l, Rr, i, d_of_ff(lenff), origin, nrm, &ccd, chd, &term);
            fp64_children = true;
            if (term) atomicAdd(s_term, term);
        }
    }
}

// Each warp takes groups of RP_GROUP rays from a launch-wide counter.  The
// rays of a group whose hit material can produce children are compacted, in
// ray order, into chunks of 32 (ballots of the hand-over's face records), so
// that every lane of a chunk evaluates a hit: misses, absorbing faces and
// faces without a material never occupy a lane.  The next chunk's inputs --
// scattered records of the group's window -- are copied into the warp's other
// shared-memory buffer (cp.async) while the current chunk computes, so the
// loads' latency is hidden behind the arithmetic.  Each lane rebuilds its hit
// point, normal and optical path from the ray's record and the hand-over's
// float-float ray parameter, evaluates the material and keeps the children
// above the |E|^2 threshold; a warp scan of the chunk's child counts plus the
// group's running count places them in the group's slot range
// (RP_TILE_SLOTS slots) in parent order, reflected before transmitted, and
// the group's total goes to tile_counts[group].
template <bool FB>
__global__ void __launch_bounds__(RP_BLOCK, MX_MAT_MIN_BLOCKS) mixed_material_kernel(GenArgs A, unsigned mx_off,
                                                                                    unsigned buf_off) {
    using namespace mx;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_term;
    const unsigned lane = threadIdx.x & 31;
    MatIn *bufs = reinterpret_cast<MatIn *>(smem + buf_off) + 2 * (threadIdx.x >> 5);
    unsigned *s_counts;
    DevScene S = stage_tables(A, smem, &s_counts);
    MxList *ml = reinterpret_cast<MxList *>(smem + mx_off);
    MxFace *mf = reinterpret_cast<MxFace *>(ml + A.S.n_lists);
    const float max_len = f_of_d(A.max_len);
    stage_mixed(A, ml, mf, max_len);
    if (threadIdx.x == 0) s_term = 0;
    const float e2t = f_of_d(A.e2_term);
    const RaySoA Rr = A.in_map ? A.wb : A.in;  // the generation's records, written by the search kernel
    const unsigned long long n_groups = rp_n_units(A.n_in, RP_GROUP);
    __syncthreads();

    GroupMask G;
    GroupAhead H;
    claim_ahead(A, n_groups, lane, H);
    next_group(A, S, n_groups, lane, H, G);
    if (G.q < n_groups) prefetch_mat(&bufs[0], A, Rr, chunk_ray(G, 0, lane), lane);
    unsigned k = 0, carry = 0;
    for (unsigned step = 0; G.q < n_groups; step++) {
        // the chunk after this one: the same group's next, or the next group's first
        GroupMask Gn = G;
        unsigned kn = k + 1;
        const bool last_of_group = kn * 32 >= G.total;
        if (last_of_group) {
            next_group(A, S, n_groups, lane, H, Gn);
            kn = 0;
        }
        if (Gn.q < n_groups)
            prefetch_mat(&bufs[(step + 1) & 1], A, Rr, chunk_ray(Gn, kn, lane), lane);
        else
            cp_async_commit();
        cp_async_wait_prev();  // this lane's copies for the current chunk have landed
        const MatIn &B = bufs[step & 1];
        const unsigned t = lane;
        const unsigned ridx = B.idx[t];
        const bool act = ridx != 0xffffffffu;
        const unsigned long long i = act ? (unsigned long long)ridx : 0ull;

        int nc = 0;
        ChildF ch[2];
        f3 nrm = mk3(0.0f, 0.0f, 0.0f), Eo = mk3(0.0f, 0.0f, 0.0f);  // unit normal (FP32 copy), E_vector
        double origin[3] = {0.0, 0.0, 0.0}, opl = 0.0;
        bool fp64_children = false;
        Child chd[2];
        ChildCommon ccd;
        int face = -1;
        if (act)
            material_mx<FB>(A, S, ml, mf, Rr, B, t, i, e2t, &s_term, nc, ch, nrm, Eo, origin, opl, fp64_children, chd,
                            ccd, face);
        // the chunk's children go to the group's slot range in parent
        // order: the group's running count plus the exclusive warp scan
        unsigned chunk_children;
        const unsigned excl = warp_scan((unsigned)nc, &chunk_children);
        if (nc > 0) {
            const double phase = B.phase[t];
            const unsigned wl = B.wl[t], ident = B.ident[t];
            const unsigned endf = (unsigned)S.faces[face].idx;
            const unsigned long long slot = (unsigned long long)G.q * RP_TILE_SLOTS + carry + excl;
            if (FB && fp64_children) {
                for (int kk = 0; kk < nc; kk++)
                    store_child(A.scratch, slot + kk, ccd, chd[kk], phase, wl, (unsigned)i, endf, ident);
            } else {
                store_child_f(A.scratch, slot, origin, nrm, Eo, opl, ch[0], phase, wl, (unsigned)i, endf, ident);
                if (nc > 1)
                    store_child_f(A.scratch, slot + 1, origin, nrm, Eo, opl, ch[1], phase, wl, (unsigned)i, endf,
                                  ident);
            }
        }
        carry += chunk_children;
        if (last_of_group) {
            if (lane == 0) A.tile_counts[G.q] = carry;
            carry = 0;
        }
        G = Gn;
        k = kn;
    }
    cp_async_wait_all();
    __syncthreads();
    if (threadIdx.x == 0 && s_term) atomicAdd(&A.stats[1], (unsigned long long)s_term);
}

// ---- batches of jobs ---------------------------------------------------------------
// The search kernel over a batch: warps take global sub-tiles from the
// batch's counter; each sub-tile belongs to one job (a job's generation
// starts on a group boundary of the global numbering) and runs with that
// job's arguments and tables from global memory.  The next sub-tile's origins
// and directions are prefetched as in the single-job kernel; rays are traced
// in place (length and end face written to the job's records) and the hit
// goes to the job's hand-over.  Face hits are added to the job's counters by
// one atomic per distinct face of a warp.
__global__ void __launch_bounds__(RP_BLOCK, MX_SEARCH_MIN_BLOCKS)
    mixed_search_batch_kernel(const BatchDev *Bt, unsigned *ctr, unsigned in_off) {
    using namespace mx;
    extern __shared__ __align__(16) unsigned char smem[];
    const unsigned lane = threadIdx.x & 31;
    TileIn *bufs = reinterpret_cast<TileIn *>(smem + in_off) + 2 * (threadIdx.x >> 5);
    // each thread's box entries of the first 64 faces of its ray's job, after the input buffers
    __half *tb = reinterpret_cast<__half *>(smem + in_off + 2 * RP_SUB_PER_BLOCK * sizeof(TileIn)) + threadIdx.x;
    const unsigned subs = RP_GROUP / RP_SUB;
    const unsigned long long n_sub = (unsigned long long)Bt->total_units * subs;
    // global sub-tile -> job and this lane's ray (~0 past the job's rays)
    auto locate = [&](unsigned tile, int &j, unsigned long long &i) {
        j = batch_job_of(Bt, tile / subs);
        const unsigned long long lt = tile - (unsigned long long)Bt->unit_start[j] * subs;
        i = lt * RP_SUB + lane;
        if (i >= Bt->jobs[j].a.n_in || !Bt->jobs[j].mixed) i = ~0ull;
    };
    unsigned tile = claim_sub_tile(&ctr[0], lane);
    int j = 0;
    unsigned long long i = ~0ull;
    if (tile < n_sub) {
        locate(tile, j, i);
        const GenArgs &A = Bt->jobs[j].a;
        prefetch_ray(&bufs[0], A.in, i, A.n_in, i, false);
    }
    for (unsigned k = 0; tile < n_sub; k++) {
        const unsigned next = claim_sub_tile(&ctr[0], lane);
        int jn = 0;
        unsigned long long in_ = ~0ull;
        if (next < n_sub) {
            locate(next, jn, in_);
            const GenArgs &An = Bt->jobs[jn].a;
            prefetch_ray(&bufs[(k + 1) & 1], An.in, in_, An.n_in, in_, false);
        } else {
            cp_async_commit();
        }
        cp_async_wait_prev();  // this lane's copies for `tile` have landed
        const BatchJob &J = Bt->jobs[j];
        const GenArgs &A = J.a;
        int face = -1;
        if (i != ~0ull) {
            const TileIn &in = bufs[k & 1];
            const double od[6] = {in.ox[lane], in.oy[lane], in.oz[lane], in.dx[lane], in.dy[lane], in.dz[lane]};
            const Best b = nearest_mx<false, __half>(A, A.S, static_cast<const MxList *>(J.mx_lists),
                                                     static_cast<const MxFace *>(J.mx_faces), tb, f_of_d(A.max_len),
                                                     od, i);
            A.in.len[i] = d_of_ff(b.len);
            A.in.endf[i] = b.face >= 0 ? (unsigned)A.S.faces[b.face].idx : 0xFFFFFFFFu;
            if (A.emit) {
                A.hit_t[i] = make_float2(b.t.hi, b.t.lo);
                A.hit_face[i] = b.face;
            }
            face = b.face;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, face);
        if (face >= 0 && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&A.face_counts[face], (unsigned)__popc(peers));
        tile = next;
        j = jn;
        i = in_;
    }
}

// The material kernel over a batch: global groups, each evaluated with its
// job's arguments and tables; the chunks' inputs are prefetched as in the
// single-job kernel, and children go to the job's own slot arena at its
// group's range.
__global__ void __launch_bounds__(RP_BLOCK, MX_MAT_MIN_BLOCKS)
    mixed_material_batch_kernel(const BatchDev *Bt, unsigned *ctr, unsigned buf_off) {
    using namespace mx;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_term;  // not reported per job
    const unsigned lane = threadIdx.x & 31;
    MatIn *bufs = reinterpret_cast<MatIn *>(smem + buf_off) + 2 * (threadIdx.x >> 5);
    if (threadIdx.x == 0) s_term = 0;
    __syncthreads();
    GroupMask G;
    BatchAhead H;
    claim_ahead_batch(Bt, ctr, lane, H);
    next_group_batch(Bt, ctr, lane, H, G);
    if (G.job >= 0) {
        const GenArgs &A = Bt->jobs[G.job].a;
        prefetch_mat(&bufs[0], A, A.in, chunk_ray(G, 0, lane), lane);
    }
    unsigned k = 0, carry = 0;
    for (unsigned step = 0; G.job >= 0; step++) {
        GroupMask Gn = G;
        unsigned kn = k + 1;
        const bool last_of_group = kn * 32 >= G.total;
        if (last_of_group) {
            next_group_batch(Bt, ctr, lane, H, Gn);
            kn = 0;
        }
        if (Gn.job >= 0) {
            const GenArgs &An = Bt->jobs[Gn.job].a;
            prefetch_mat(&bufs[(step + 1) & 1], An, An.in, chunk_ray(Gn, kn, lane), lane);
        } else {
            cp_async_commit();
        }
        cp_async_wait_prev();
        const BatchJob &J = Bt->jobs[G.job];
        const GenArgs &A = J.a;
        const MatIn &B = bufs[step & 1];
        const unsigned t = lane;
        const unsigned ridx = B.idx[t];
        const bool act = ridx != 0xffffffffu;
        const unsigned long long i = act ? (unsigned long long)ridx : 0ull;
        int nc = 0;
        ChildF ch[2];
        f3 nrm = mk3(0.0f, 0.0f, 0.0f), Eo = mk3(0.0f, 0.0f, 0.0f);
        double origin[3] = {0.0, 0.0, 0.0}, opl = 0.0;
        bool fp64_children = false;
        Child chd[2];
        ChildCommon ccd;
        int face = -1;
        if (act)
            material_mx<false>(A, A.S, static_cast<const MxList *>(J.mx_lists), static_cast<const MxFace *>(J.mx_faces),
                               A.in, B, t, i, f_of_d(A.e2_term), &s_term, nc, ch, nrm, Eo, origin, opl, fp64_children,
                               chd, ccd, face);
        unsigned chunk_children;
        const unsigned excl = warp_scan((unsigned)nc, &chunk_children);
        if (nc > 0) {
            const double phase = B.phase[t];
            const unsigned wl = B.wl[t], ident = B.ident[t];
            const unsigned endf = (unsigned)A.S.faces[face].idx;
            const unsigned long long slot = (unsigned long long)G.q * RP_TILE_SLOTS + carry + excl;
            const unsigned parent = (unsigned)(i + A.parent_base);  // within the job's generation
            store_child_f(A.scratch, slot, origin, nrm, Eo, opl, ch[0], phase, wl, parent, endf, ident);
            if (nc > 1)
                store_child_f(A.scratch, slot + 1, origin, nrm, Eo, opl, ch[1], phase, wl, parent, endf, ident);
        }
        carry += chunk_children;
        if (last_of_group) {
            if (lane == 0) A.tile_counts[G.q] = carry;
            carry = 0;
        }
        G = Gn;
        k = kn;
    }
    cp_async_wait_all();
}

// One job's float / float-float tables for the batch kernels (the single-job
// kernels build them in shared memory per block).
__global__ void batch_tables_kernel(GenArgs a, mx::MxList *ml, mx::MxFace *mf) {
    mx::stage_mixed(a, ml, mf, mx::f_of_d(a.max_len));
}

size_t batch_tables_bytes(int n_lists, int n_faces) { return mx::mx_tables_bytes(n_lists, n_faces); }

cudaError_t launch_batch_tables(const GenArgs &a, void *tables, cudaStream_t st) {
    mx::MxList *ml = static_cast<mx::MxList *>(tables);
    batch_tables_kernel<<<1, RP_BLOCK, 0, st>>>(a, ml, reinterpret_cast<mx::MxFace *>(ml + a.S.n_lists));
    return cudaGetLastError();
}

// ---- launches ---------------------------------------------------------------------
// Resident blocks for one kernel and shared-memory size, cached per (kernel,
// device, size) under a lock: several host threads (server lanes) launch.
template <typename K>
static cudaError_t resident_grid(K kernel, size_t total, int *blocks) {
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, size_t>, int> cache;
    static std::map<std::pair<const void *, int>, size_t> limit;  // shared-memory limit set per (kernel, device)
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const void *key = reinterpret_cast<const void *>(kernel);
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({key, dev, total});
    if (it != cache.end()) {
        *blocks = it->second;
        return cudaSuccess;
    }
    size_t &lim = limit[{key, dev}];
    if (lim < total) {
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)total);
        if (e != cudaSuccess) return e;
        lim = total;
    }
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, RP_BLOCK, total);
    if (e != cudaSuccess) return e;
    *blocks = (per_sm > 0 ? per_sm : 1) * sms;
    cache[{key, dev, total}] = *blocks;
    return cudaSuccess;
}

struct MixedLayout {
    size_t mx_off, tb_off, in_off, pass_off, search_total, mat_buf_off, mat_total;
    bool tb;  // the search kernel's box-entry table is FP32 (else FP16)
};

static MixedLayout mixed_layout(const GenArgs &a, size_t smem) {
    MixedLayout L;
    L.mx_off = (smem + 15) & ~(size_t)15;
    L.tb_off = L.mx_off + mx::mx_tables_bytes(a.S.n_lists, a.S.n_faces);
    L.mat_buf_off = (L.tb_off + 15) & ~(size_t)15;
    L.mat_total = L.mat_buf_off + 2 * RP_SUB_PER_BLOCK * sizeof(mx::MatIn);
    L.tb = a.S.n_faces <= RP_MX_TB_F32_FACES;  // an FP32 table (else FP16)
    const int nmask = a.S.n_faces < 64 ? a.S.n_faces : 64;
    L.in_off = (L.tb_off + (size_t)nmask * RP_BLOCK * (L.tb ? sizeof(float) : sizeof(__half)) + 15) & ~(size_t)15;
    L.pass_off = L.in_off + 2 * RP_SUB_PER_BLOCK * sizeof(mx::TileIn);
    L.search_total = L.pass_off + (a.in_map ? RP_SUB_PER_BLOCK * sizeof(mx::PassIn) : 0);
    return L;
}

static cudaError_t mixed_grids(const GenArgs &a, const MixedLayout &L, int *search_blocks, int *mat_blocks) {
    cudaError_t e;
    if (L.tb)
        e = a.mixed_fallback ? resident_grid(mixed_search_kernel<true, float>, L.search_total, search_blocks)
                             : resident_grid(mixed_search_kernel<false, float>, L.search_total, search_blocks);
    else
        e = a.mixed_fallback ? resident_grid(mixed_search_kernel<true, __half>, L.search_total, search_blocks)
                             : resident_grid(mixed_search_kernel<false, __half>, L.search_total, search_blocks);
    if (e != cudaSuccess) return e;
    return a.mixed_fallback ? resident_grid(mixed_material_kernel<true>, L.mat_total, mat_blocks)
                            : resident_grid(mixed_material_kernel<false>, L.mat_total, mat_blocks);
}

// Runs the one-time per-size set-up of the launches (attributes, occupancy)
// so that a later launch of the same configuration makes no other CUDA call,
// as stream capture requires.
cudaError_t prepare_generation_mixed(const GenArgs &a, size_t smem) {
    const MixedLayout L = mixed_layout(a, smem);
    if (L.search_total > 220 * 1024) return cudaErrorInvalidConfiguration;
    int sb = 0, mb = 0;
    return mixed_grids(a, L, &sb, &mb);
}

// The search kernel, then (when the generation keeps children) the material
// kernel.  The scene's faces and materials decide the instantiation: without
// FP64 fallbacks the kernels carry no out-of-line calls and their register
// cost.  The caller has zeroed the tile and group counters.
cudaError_t launch_generation_mixed(const GenArgs &a, size_t smem, cudaStream_t st, cudaEvent_t mid) {
    if (a.n_in == 0) return cudaSuccess;
    if (a.emit && (!a.hit_t || !a.hit_face || !a.group_next || a.unit_rays != RP_GROUP))
        return cudaErrorInvalidValue;  // the hand-over and the group unit are set up by the caller
    const MixedLayout L = mixed_layout(a, smem);
    if (L.search_total > 220 * 1024) return cudaErrorInvalidConfiguration;  // scene too large for the tables
    int sb = 0, mb = 0;
    cudaError_t e = mixed_grids(a, L, &sb, &mb);
    if (e != cudaSuccess) return e;
    const unsigned long long n_tiles = (a.n_in + RP_BLOCK - 1) / RP_BLOCK;
    const unsigned sgrid = (unsigned)(n_tiles < (unsigned long long)sb ? n_tiles : sb);
    const unsigned o1 = (unsigned)L.mx_off, o2 = (unsigned)L.tb_off, o3 = (unsigned)L.in_off, o4 = (unsigned)L.pass_off;
    if (L.tb) {
        if (a.mixed_fallback)
            mixed_search_kernel<true, float><<<sgrid, RP_BLOCK, L.search_total, st>>>(a, o1, o2, o3, o4);
        else
            mixed_search_kernel<false, float><<<sgrid, RP_BLOCK, L.search_total, st>>>(a, o1, o2, o3, o4);
    } else {
        if (a.mixed_fallback)
            mixed_search_kernel<true, __half><<<sgrid, RP_BLOCK, L.search_total, st>>>(a, o1, o2, o3, o4);
        else
            mixed_search_kernel<false, __half><<<sgrid, RP_BLOCK, L.search_total, st>>>(a, o1, o2, o3, o4);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess && mid) e = cudaEventRecord(mid, st);
    if (e != cudaSuccess || !a.emit) return e;
    // one warp per group: RP_SUB_PER_BLOCK groups per block
    const unsigned long long n_groups = rp_n_units(a.n_in, RP_GROUP);
    const unsigned long long need = (n_groups + RP_SUB_PER_BLOCK - 1) / RP_SUB_PER_BLOCK;
    const unsigned mgrid = (unsigned)(need < (unsigned long long)mb ? need : mb);
    const unsigned o5 = (unsigned)L.mat_buf_off;
    if (a.mixed_fallback)
        mixed_material_kernel<true><<<mgrid, RP_BLOCK, L.mat_total, st>>>(a, o1, o5);
    else
        mixed_material_kernel<false><<<mgrid, RP_BLOCK, L.mat_total, st>>>(a, o1, o5);
    return cudaGetLastError();
}


// Shared memory and resident grids of the batch kernels (their tables come
// from global memory: the warps' input buffers and, for the search, each
// thread's box entries of up to 64 faces are in shared memory).
cudaError_t prepare_batch_mixed(size_t *search_smem, size_t *mat_smem, int *search_blocks, int *mat_blocks) {
    *search_smem = 2 * RP_SUB_PER_BLOCK * sizeof(mx::TileIn) + 64 * RP_BLOCK * sizeof(__half);
    *mat_smem = 2 * RP_SUB_PER_BLOCK * sizeof(mx::MatIn);
    cudaError_t e = resident_grid(mixed_search_batch_kernel, *search_smem, search_blocks);
    if (e != cudaSuccess) return e;
    return resident_grid(mixed_material_batch_kernel, *mat_smem, mat_blocks);
}

// The two kernels of one batch step, on persistent grids (the same launch
// for every step: the batch's size is read from device memory).
cudaError_t launch_batch_mixed(const BatchDev *batch, unsigned *ctr, cudaStream_t st) {
    size_t ss = 0, ms = 0;
    int sb = 0, mb = 0;
    cudaError_t e = prepare_batch_mixed(&ss, &ms, &sb, &mb);
    if (e != cudaSuccess) return e;
    mixed_search_batch_kernel<<<sb, RP_BLOCK, ss, st>>>(batch, ctr, 0u);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    mixed_material_batch_kernel<<<mb, RP_BLOCK, ms, st>>>(batch, ctr, 0u);
    return cudaGetLastError();
}

}  // namespace rp
