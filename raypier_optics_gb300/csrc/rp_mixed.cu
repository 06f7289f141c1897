// rp_mixed.cu -- mixed FP32/FP64 generation kernel.
//
// Same generation structure as the plain kernel (rp_trace.cu): culled
// nearest-first face search, orientation, material, per-ray child slots.  The
// arithmetic is split by what needs 64-bit precision:
//
//   FP64  ray origins and hit points; the distance along the ray to a face
//         (planes: one FP64 division; spheres and conics: the quadratic root;
//         aspheres and polynomial faces: FP32 Newton iterations followed by a
//         final FP64 Newton step); the Euclidean length correction for a
//         direction that is not exactly unit; accumulated optical path length.
//   FP32  directions (stored as double), face normals, the S/P projection,
//         Fresnel coefficients, polarisation amplitudes and E-vectors, the
//         Snell direction update, aperture and shape tests.
//
// The TU is compiled with FMA contraction on.  Distortion faces and the rarer
// materials reuse the FP64 device functions of the plain path.  Results agree
// with the FP64 oracle to the accuracy reported in the precision test (nm in
// position / OPL, rad in direction); index fields can differ for rays that
// graze an aperture edge, which is why parity for this path is statistical.
#include "rp_gen_common.cuh"

namespace rp {
namespace mx {

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
__device__ __forceinline__ f3 tof(v3 a) { return mk3((float)a.x, (float)a.y, (float)a.z); }
__device__ __forceinline__ v3 tod(f3 a) { return mkv(a.x, a.y, a.z); }
__device__ __forceinline__ f3 rot3(const double *m, f3 p) {
    return mk3(p.x * (float)m[0] + p.y * (float)m[1] + p.z * (float)m[2],
               p.x * (float)m[3] + p.y * (float)m[4] + p.z * (float)m[5],
               p.x * (float)m[6] + p.y * (float)m[7] + p.z * (float)m[8]);
}

// complex float
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
__device__ __forceinline__ cf csqrtf_(cf z) {
    float x = z.x, y = z.y;
    if (x == 0.0f && y == 0.0f) return cfm(0.0f, y);
    float t = sqrtf((fabsf(x) + sqrtf(x * x + y * y)) * 0.5f);
    if (x >= 0.0f) return cfm(t, y / (2.0f * t));
    return cfm(fabsf(y) / (2.0f * t), copysignf(t, y));
}
__device__ __forceinline__ float cabs2(cf z) { return z.x * z.x + z.y * z.y; }

// 1/x in FP64 from an FP32 estimate and two Newton steps (relative error ~1e-16)
__device__ __forceinline__ double drcp(double x) {
    double r = (double)(1.0f / (float)x);
    r = r * (2.0 - x * r);
    r = r * (2.0 - x * r);
    return r;
}

// Ray in a face list's frame: FP64 origin, FP32 unit direction, the same
// direction as double, and the Euclidean-length factor |d| of the stored
// direction (distances are Euclidean in the reference).
struct LRay {
    v3 p;      // local origin (FP64)
    f3 df;     // local direction (FP32)
    v3 dd;     // local direction (FP64 copy of df)
};

#define MX_MISS (-1.0)

__device__ __forceinline__ double plane_t(double z, const LRay &R) {
    // t with p.z + t d.z = z; FP64 numerator, FP64-refined reciprocal
    if (R.dd.z == 0.0) return MX_MISS;
    return (z - R.p.z) * drcp(R.dd.z);
}

__device__ __forceinline__ int shape_in(const DevScene &S, int prog, float x, float y, unsigned *err) {
    return shape_inside(S, prog, (double)x, (double)y, err);
}

// Sphere / conic: roots of a t^2 + b t + c = 0 in FP64 (the quadratic that
// loses precision to cancellation at large radius and grazing incidence).
__device__ __forceinline__ bool quad_roots(double a, double b, double c, double &t1, double &t2) {
    double disc = b * b - 4.0 * a * c;
    if (disc < 0.0) return false;
    double sd = sqrt(disc);
    double inv2a = 0.5 * drcp(a);
    t1 = (-b + sd) * inv2a;
    t2 = (-b - sd) * inv2a;
    return true;
}

__device__ double face_t_mixed(const DevScene &S, const rp_face &f, const LRay &R, double tmax, unsigned *err) {
    // Returns the ray parameter of a valid hit (hit = p + t d), or MX_MISS.
    const double tol_t = f.tolerance;  // faces compare their tolerance to the fraction h = t / tmax
    switch (f.type) {
        case RP_FACE_CIRCULAR: {
            double t = plane_t(f.p[2], R);
            if (t < tol_t * tmax || t > tmax) return MX_MISS;
            float X = (float)(R.p.x + t * R.dd.x - f.p[1]), Y = (float)(R.p.y + t * R.dd.y);
            float dd = (float)f.p[0];
            if (X * X + Y * Y > dd * dd * 0.25f) return MX_MISS;
            return t;
        }
        case RP_FACE_RECTANGULAR: {
            double t = plane_t(f.p[3], R);
            if (t < tol_t * tmax || t > tmax) return MX_MISS;
            float X = (float)(R.p.x + t * R.dd.x - f.p[2]), Y = (float)(R.p.y + t * R.dd.y);
            if (X * X > (float)(f.p[0] * f.p[0] / 4)) return MX_MISS;
            if (Y * Y > (float)(f.p[1] * f.p[1] / 4)) return MX_MISS;
            return t;
        }
        case RP_FACE_SHAPED_PLANAR: {
            double t = plane_t(f.p[0], R);
            if (t < tol_t * tmax || t > tmax) return MX_MISS;
            float X = (float)(R.p.x + t * R.dd.x), Y = (float)(R.p.y + t * R.dd.y);
            if (!shape_in(S, f.shape, X, Y, err)) return MX_MISS;
            return t;
        }
        case RP_FACE_SPHERICAL:
        case RP_FACE_SHAPED_SPHERICAL: {
            bool plain = f.type == RP_FACE_SPHERICAL;
            double c = plain ? f.p[1] : f.p[0], zh = plain ? f.p[2] : f.p[1];
            double cz = zh - c;
            v3 q = mkv(R.p.x, R.p.y, R.p.z - cz);
            double a = dotv(R.dd, R.dd), b = 2.0 * dotv(R.dd, q), cc = dotv(q, q) - c * c;
            double t1, t2;
            if (!quad_roots(a, b, cc, t1, t2)) return MX_MISS;
            const double INF = inf_d();
            float z1 = (float)(q.z + t1 * R.dd.z), z2 = (float)(q.z + t2 * R.dd.z);
            if (c >= 0) {
                if (z1 < 0.0f) t1 = INF;
                if (z2 < 0.0f) t2 = INF;
            } else {
                if (z1 > 0.0f) t1 = INF;
                if (z2 > 0.0f) t2 = INF;
            }
            float x1 = (float)(R.p.x + t1 * R.dd.x), y1 = (float)(R.p.y + t1 * R.dd.y);
            float x2 = (float)(R.p.x + t2 * R.dd.x), y2 = (float)(R.p.y + t2 * R.dd.y);
            if (plain) {
                float DD = (float)(f.p[0] * f.p[0] / 4.0);
                if (x1 * x1 + y1 * y1 > DD) t1 = INF;
                if (x2 * x2 + y2 * y2 > DD) t2 = INF;
            } else {
                if (!shape_in(S, f.shape, x1, y1, err)) t1 = INF;
                if (!shape_in(S, f.shape, x2, y2, err)) t2 = INF;
            }
            if (t2 < t1) t1 = t2;
            if (t1 > tmax || t1 < tol_t * tmax) return MX_MISS;
            return t1;
        }
        case RP_FACE_CONIC: {
            // beta z^2 - 2 R z + r^2 = 0 along the ray (cfaces.pyx:1695-1747)
            double Rr = -f.p[0], beta = 1 + f.p[2];
            v3 a = mkv(R.p.x, R.p.y, R.p.z - f.p[1]);
            v3 d = R.dd;
            double A = beta * beta * d.z * d.z + beta * (d.x * d.x + d.y * d.y);
            double B = -2 * Rr * beta * d.z + 2 * beta * (a.x * d.x + a.y * d.y) + 2 * a.z * beta * beta * d.z;
            double C = -2 * Rr * a.z * beta + beta * (a.x * a.x + a.y * a.y) + a.z * a.z * beta * beta;
            double disc = B * B - 4 * A * C;
            if (disc < 0) return MX_MISS;
            double sd = sqrt(disc), inv2a = 0.5 * drcp(A);
            double t = (Rr * beta * d.z <= 0) ? (-B + sd) * inv2a : (-B - sd) * inv2a;
            float X = (float)(a.x + t * d.x), Y = (float)(a.y + t * d.y);
            if (!shape_in(S, f.shape, X, Y, err)) return MX_MISS;
            if (t > tmax || t < tol_t * tmax) return MX_MISS;
            return t;
        }
        case RP_FACE_ASPHERIC: {
            // conic start, FP32 Newton on the sag residual, one FP64 step last
            double Rr = -f.p[0], beta = 1 + f.p[2];
            v3 a = mkv(R.p.x, R.p.y, R.p.z - f.p[1]);
            v3 d = R.dd;
            double A = beta * beta * d.z * d.z + beta * (d.x * d.x + d.y * d.y);
            double B = -2 * Rr * beta * d.z + 2 * beta * (a.x * d.x + a.y * d.y) + 2 * a.z * beta * beta * d.z;
            double C = -2 * Rr * a.z * beta + beta * (a.x * a.x + a.y * a.y) + a.z * a.z * beta * beta;
            double disc = B * B - 4 * A * C;
            double t = MX_MISS;
            if (disc >= 0) {
                double sd = sqrt(disc), inv2a = 0.5 * drcp(A);
                t = (Rr * beta * d.z <= 0) ? (-B + sd) * inv2a : (-B - sd) * inv2a;
            }
            const float Rf = (float)Rr, bf = (float)beta, R2f = Rf * Rf;
            const float A4 = (float)f.p[3], A6 = (float)f.p[4], A8 = (float)f.p[5], A10 = (float)f.p[6],
                        A12 = (float)f.p[7], A14 = (float)f.p[8], A16 = (float)f.p[9];
            // residual f(t) = sag(r(t)) - z(t) and df/dt in FP32, relative to the start t0
            float ax = (float)a.x, ay = (float)a.y, az = (float)a.z;
            float dx = R.df.x, dy = R.df.y, dz = R.df.z;
            float tf = (float)t;
            float f_last = 0.0f;
            bool conv = false;
            for (int it = 0; it < 100; it++) {
                float ux = ax + tf * dx, uy = ay + tf * dy;
                float r2 = ux * ux + uy * uy;
                float root = sqrtf(1.0f - bf * r2 / R2f);
                float poly = r2 * r2 * (A4 + r2 * (A6 + r2 * (A8 + r2 * (A10 + r2 * (A12 + r2 * (A14 + r2 * A16))))));
                float fv = r2 / (Rf * (1.0f + root)) - (az + tf * dz) + poly;
                if (it > 0 && fabsf(fv) > fabsf(f_last) && fabsf(fv) > 1e-6f * (1.0f + fabsf(az))) return MX_MISS;
                f_last = fv;
                float dr2 = 2.0f * (dx * ux + dy * uy);
                float dsag = 1.0f / (Rf * (1.0f + root)) + bf * r2 / (2.0f * Rf * R2f * root * (1.0f + root) * (1.0f + root));
                float dpoly = r2 * (2.0f * A4 + r2 * (3.0f * A6 + r2 * (4.0f * A8 + r2 * (5.0f * A10 +
                              r2 * (6.0f * A12 + r2 * (7.0f * A14 + r2 * 8.0f * A16))))));
                float g = (dsag + dpoly) * dr2 - dz;
                float step = -fv / g;
                tf += step;
                if (!(fabsf(step) <= 1e-5f * (1.0f + fabsf(tf)))) continue;
                conv = true;
                break;
            }
            if (!conv || !isfinite(tf)) return MX_MISS;
            // last Newton step in FP64
            double td = (double)tf;
            {
                double ux = a.x + td * d.x, uy = a.y + td * d.y;
                double r2 = ux * ux + uy * uy;
                double root = sqrt(1.0 - beta * r2 / (Rr * Rr));
                double poly = r2 * r2 * (f.p[3] + r2 * (f.p[4] + r2 * (f.p[5] + r2 * (f.p[6] +
                              r2 * (f.p[7] + r2 * (f.p[8] + r2 * f.p[9]))))));
                double fv = r2 / (Rr * (1.0 + root)) - (a.z + td * d.z) + poly;
                double dr2 = 2.0 * (d.x * ux + d.y * uy);
                double dsag = 1.0 / (Rr * (1.0 + root)) +
                              beta * r2 / (2.0 * Rr * Rr * Rr * root * (1.0 + root) * (1.0 + root));
                double dpoly = r2 * (2.0 * f.p[3] + r2 * (3.0 * f.p[4] + r2 * (4.0 * f.p[5] + r2 * (5.0 * f.p[6] +
                               r2 * (6.0 * f.p[7] + r2 * (7.0 * f.p[8] + r2 * 8.0 * f.p[9]))))));
                double g = (dsag + dpoly) * dr2 - d.z;
                td = td - fv / g;
            }
            if (!isfinite(td)) return MX_MISS;
            float X = (float)(a.x + td * d.x), Y = (float)(a.y + td * d.y);
            if (!shape_in(S, f.shape, X, Y, err)) return MX_MISS;
            if (td > tmax || td < tol_t * tmax) return MX_MISS;
            return td;
        }
        default:
            return MX_MISS - 1.0;  // not handled here: use the FP64 path
    }
}

// FP32 face normals (local frame) from an FP64 local hit point.
__device__ f3 face_normal_mixed(const DevScene &S, const rp_face &f, v3 p, unsigned *err, bool &handled) {
    handled = true;
    switch (f.type) {
        case RP_FACE_CIRCULAR: return mk3(0, 0, f.invert_normals ? 1.0f : -1.0f);
        case RP_FACE_SHAPED_PLANAR: return mk3(0, 0, 1);
        case RP_FACE_RECTANGULAR: return mk3(0, 0, -1);
        case RP_FACE_SPHERICAL:
        case RP_FACE_SHAPED_SPHERICAL: {
            bool plain = f.type == RP_FACE_SPHERICAL;
            double c = plain ? f.p[1] : f.p[0], zh = plain ? f.p[2] : f.p[1];
            f3 q = mk3((float)p.x, (float)p.y, (float)(p.z - (zh - c)));
            if (c < 0) q = mk3(-q.x, -q.y, -q.z);
            return norm3(q);
        }
        case RP_FACE_CONIC: {
            float Rr = (float)(-f.p[0]), beta = (float)(1 + f.p[2]);
            float sign = f.invert_normals ? -1.0f : 1.0f;
            float pz = (float)(p.z - f.p[1]);
            f3 g = mk3(-(float)p.x * 2 * beta, -(float)p.y * 2 * beta, 2 * beta * (Rr - beta * pz));
            if (Rr * beta < 0) sign = -sign;
            return norm3(mul3(g, sign));
        }
        case RP_FACE_ASPHERIC: {
            float Rr = (float)(-f.p[0]), beta = (float)(1 + f.p[2]);
            float sign = f.invert_normals ? -1.0f : 1.0f;
            float x = (float)p.x, y = (float)p.y;
            float r2 = x * x + y * y;
            float root = sqrtf(1.0f - beta * r2 / (Rr * Rr));
            float A4 = (float)f.p[3], A6 = (float)f.p[4], A8 = (float)f.p[5], A10 = (float)f.p[6],
                  A12 = (float)f.p[7], A14 = (float)f.p[8], A16 = (float)f.p[9];
            float df = r2 * (4 * A4 + r2 * (6 * A6 + r2 * (8 * A8 + r2 * (10 * A10 + r2 * (12 * A12 +
                       r2 * (14 * A14 + r2 * 16 * A16))))));
            df += 2.0f / (Rr * (1.0f + root));
            df += beta * r2 / (Rr * Rr * Rr * root * (1.0f + root) * (1.0f + root));
            return norm3(mul3(mk3(-df * x, -df * y, 1.0f), sign));
        }
        default: handled = false; return mk3(0, 0, 0);
    }
}

// convert_to_sp in FP32 (cmaterials.pyx:49-91)
__device__ __forceinline__ void sp_mixed(f3 d, f3 E, cf e1, cf e2, f3 normal, f3 &Eo, cf &e1o, cf &e2o) {
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

// Material evaluation for the common materials in FP32 (OPL and the hit point
// stay FP64).  Returns -1 for materials left to the FP64 path.
__device__ int eval_mixed(const DevScene &S, const rp_material &m, const RayState &r, v3 point, f3 nrm_in,
                          ChildCommon &cc, Child *ch, unsigned *err) {
    const double INF = inf_d();
    if (m.type == RP_MAT_NONE || m.type == RP_MAT_OPAQUE) return 0;
    if (m.type != RP_MAT_PEC && m.type != RP_MAT_DIELECTRIC && m.type != RP_MAT_FULL_DIELECTRIC &&
        m.type != RP_MAT_FULL_DIELECTRIC_DISPERSIVE && m.type != RP_MAT_TRANSPARENT)
        return -1;
    f3 normal = norm3(nrm_in);
    f3 d = tof(r.d);
    f3 ind = norm3(d);
    f3 E = tof(r.E);
    cf e1 = cfm((float)r.e1.x, (float)r.e1.y), e2 = cfm((float)r.e2.x, (float)r.e2.y);
    f3 Eo;
    cf E1, E2;
    sp_mixed(d, E, e1, e2, normal, Eo, E1, E2);
    cc.E = tod(Eo);
    cc.opl = r.opl + r.len * r.n.x;  // FP64
    cc.origin = point;
    cc.normal = tod(normal);
    if (m.type == RP_MAT_TRANSPARENT) {
        ch[0].d = r.d;
        ch[0].n = r.n;
        ch[0].e1 = make_double2(E1.x, E1.y);
        ch[0].e2 = make_double2(E2.x, E2.y);
        ch[0].len = INF;
        ch[0].type = r.type & ~RP_REFL_RAY;
        return 1;
    }
    float cosTheta = dot3(normal, m.type == RP_MAT_PEC ? d : ind);
    f3 ctn = mul3(normal, cosTheta);
    if (m.type == RP_MAT_PEC) {
        ch[0].d = tod(sub3(d, mul3(ctn, 2.0f)));
        ch[0].n = r.n;
        ch[0].e1 = make_double2(-E1.x, -E1.y);
        ch[0].e2 = make_double2(E2.x, E2.y);
        ch[0].len = INF;
        ch[0].type = r.type | RP_REFL_RAY;
        return 1;
    }
    float cos1 = fabsf(cosTheta);
    bool out_to_in = cosTheta < 0.0f;
    if (m.type == RP_MAT_DIELECTRIC) {
        float n1 = (float)(out_to_in ? m.n_outside[0] : m.n_inside[0]);
        float n2 = (float)(out_to_in ? m.n_inside[0] : m.n_outside[0]);
        ch[0].n = out_to_in ? make_double2(m.n_inside[0], m.n_inside[1]) : make_double2(m.n_outside[0], m.n_outside[1]);
        float flip = out_to_in ? 1.0f : -1.0f;
        float q = n2 / n1;
        float N2_sin2 = cosTheta * cosTheta + (q * q - 1.0f);
        ch[0].len = INF;
        if (N2_sin2 < 0.0f) {
            ch[0].d = tod(sub3(ind, mul3(ctn, 2.0f)));
            ch[0].e1 = make_double2(-E1.x, -E1.y);
            ch[0].e2 = make_double2(-E2.x, -E2.y);
            ch[0].type = r.type | RP_REFL_RAY;
        } else {
            f3 tg2 = mul3(sub3(ind, ctn), n1 / n2);
            float c2 = sqrtf(1.0f - dot3(tg2, tg2));
            f3 tr = sub3(tg2, mul3(normal, c2 * flip));
            float cos2 = fabsf(dot3(tr, normal));
            float aspect = sqrtf(cos2 / cos1) * (2 * n1) * cos1;
            float T_p = aspect / (n2 * cos1 + n1 * cos2);
            float T_s = aspect / (n2 * cos2 + n1 * cos1);
            ch[0].d = tod(tr);
            ch[0].e1 = make_double2(E1.x * T_s, E1.y * T_s);
            ch[0].e2 = make_double2(E2.x * T_p, E2.y * T_p);
            ch[0].type = r.type & ~RP_REFL_RAY;
        }
        return 1;
    }
    // FullDielectric / FullDielectricDispersive (cmaterials.pyx:756-872, 897-1013)
    float sin1 = sqrtf(fabsf(1.0f - cos1 * cos1));
    cf n1, n2;
    double2 n1d, n2d;
    if (m.type == RP_MAT_FULL_DIELECTRIC) {
        double2 ni = make_double2(m.n_inside[0], m.n_inside[1]), no = make_double2(m.n_outside[0], m.n_outside[1]);
        n1d = out_to_in ? no : ni;
        n2d = out_to_in ? ni : no;
    } else {
        long long w = (long long)r.wl;
        if (w >= S.n_wl) {
            atomicOr(err, ERR_WAVELENGTH);
            return 0;
        }
        n1d = S.ntab[(long long)(out_to_in ? m.curve_outside : m.curve_inside) * S.n_wl + w];
        n2d = S.ntab[(long long)(out_to_in ? m.curve_inside : m.curve_outside) * S.n_wl + w];
    }
    n1 = cfm((float)n1d.x, (float)n1d.y);
    n2 = cfm((float)n2d.x, (float)n2d.y);
    float flip = out_to_in ? 1.0f : -1.0f;
    cf sin2 = cdiv(cmuls(n1, sin1), n2);
    cf cos2 = csqrtf_(csub(cfm(1.0f, 0.0f), cmul(sin2, sin2)));
    float P_in = n1.x * (cabs2(E1) + cabs2(E2));
    if (P_in == 0.0f) return 0;
    cf n2c1 = cmuls(n2, cos1), n1c2 = cmul(n1, cos2), n2c2 = cmul(n2, cos2), n1c1 = cmuls(n1, cos1);
    cf den_p = cadd(n2c1, n1c2), den_s = cadd(n2c2, n1c1);
    cf R_p = cmul(cdiv(cfm(n1c2.x - n2c1.x, n1c2.y - n2c1.y), den_p), E2);
    cf R_s = cmul(cdiv(cfm(n1c1.x - n2c2.x, n1c1.y - n2c2.y), den_s), E1);
    int nc = 0;
    if ((n1.x * (cabs2(R_s) + cabs2(R_p))) / P_in > (float)m.reflection_threshold) {
        ch[0].d = tod(sub3(ind, mul3(ctn, 2.0f)));
        ch[0].len = INF;
        ch[0].e1 = make_double2(R_s.x, R_s.y);
        ch[0].e2 = make_double2(-R_p.x, -R_p.y);
        ch[0].n = n1d;
        ch[0].type = r.type | RP_REFL_RAY;
        nc = 1;
    }
    f3 tg2 = mul3(sub3(ind, ctn), n1.x / n2.x);
    float c2 = sqrtf(1.0f - dot3(tg2, tg2));
    f3 tr = sub3(tg2, mul3(normal, c2 * flip));
    float aspect = sqrtf(cos2.x / cos1);
    cf num = cmuls(n1, 2.0f * cos1 * aspect);
    cf T_p = cmul(cdiv(num, den_p), E2);
    cf T_s = cmul(cdiv(num, den_s), E1);
    if ((n2.x * (cabs2(T_s) + cabs2(T_p))) / P_in > (float)m.transmission_threshold) {
        ch[nc].d = tod(tr);
        ch[nc].len = INF;
        ch[nc].e1 = make_double2(T_s.x, T_s.y);
        ch[nc].e2 = make_double2(T_p.x, T_p.y);
        ch[nc].n = n2d;
        ch[nc].type = r.type & ~RP_REFL_RAY;
        nc++;
    }
    return nc;
}

}  // namespace mx

__device__ __forceinline__ float mx_box_enter(const float *b, float ox, float oy, float oz, float ix, float iy,
                                              float iz) {
    if (b[6] == 0.0f) return 0.0f;
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

__global__ void __launch_bounds__(RP_BLOCK) generation_mixed_kernel(GenArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_hits, s_term;
    unsigned *s_counts;
    DevScene S = stage_tables(A, smem, &s_counts);
    if (threadIdx.x == 0) {
        s_hits = 0;
        s_term = 0;
    }
    __syncthreads();
    const unsigned tile = blockIdx.x;
    const unsigned long long i = (unsigned long long)tile * RP_BLOCK + threadIdx.x;
    const bool active = i < A.n_in;

    int best = -1, best_list = -1;
    double len = A.max_len;   // Euclidean distance of the current nearest hit
    v3 o = mkv(0, 0, 0), d = mkv(0, 0, 0);
    double dlen = 1.0;        // |d| of the stored direction
    if (active) {
        o = mkv(A.in.ox[i], A.in.oy[i], A.in.oz[i]);
        d = mkv(A.in.dx[i], A.in.dy[i], A.in.dz[i]);
        double d2 = d.x * d.x + d.y * d.y + d.z * d.z;
        dlen = 1.0 + 0.5 * (d2 - 1.0);  // first order in |d|^2 - 1 (directions are unit to FP32 rounding)
        const double tmax = A.max_len;  // the far point is origin + d * max_length (ray parameter)
        mx::f3 df = mx::mk3((float)d.x, (float)d.y, (float)d.z);
        float il = rsqrtf(mx::dot3(df, df));
        float ix = 1.0f / ((fabsf(df.x * il) < 1e-30f) ? copysignf(1e-30f, df.x) : df.x * il);
        float iy = 1.0f / ((fabsf(df.y * il) < 1e-30f) ? copysignf(1e-30f, df.y) : df.y * il);
        float iz = 1.0f / ((fabsf(df.z * il) < 1e-30f) ? copysignf(1e-30f, df.z) : df.z * il);
        float ox = (float)o.x, oy = (float)o.y, oz = (float)o.z;
        const int nf = S.n_faces;
        const int nmask = nf < 64 ? nf : 64;
        const float lim0 = (float)A.max_len * 1.000001f + 1e-4f;
        unsigned long long cand = 0;
        if (A.one_list >= 0) {
            int f = S.lists[A.one_list].first_face + A.one_face;
            if (f < 64) cand = 1ull << f;
        } else {
            for (int f = 0; f < nmask; f++)
                if (mx_box_enter(S.bounds + 8 * f, ox, oy, oz, ix, iy, iz) <= lim0) cand |= 1ull << f;
        }
        int cur_list = -1;
        mx::LRay R;
        v3 p1 = o, p2 = o;
        v3 pend = addv(o, mulvs(d, A.max_len));
        while (cand) {
            float tsel = __int_as_float(0x7f800000);
            int sel = -1;
            for (unsigned long long m = cand; m; m &= m - 1) {
                int f = __ffsll((long long)m) - 1;
                float t = mx_box_enter(S.bounds + 8 * f, ox, oy, oz, ix, iy, iz);
                if (t < tsel) {
                    tsel = t;
                    sel = f;
                }
            }
            if (sel < 0 || tsel > (float)len * 1.000001f + 1e-4f) break;
            cand &= ~(1ull << sel);
            int l = S.face_list[sel];
            if (l < 0 || l >= S.n_lists) {
                atomicOr(A.err, ERR_SHAPE_STACK);
                break;
            }
            const rp_facelist &L = S.lists[l];
            if (l != cur_list) {
                R.p = xform(L.inv_trans.m, L.inv_trans.t, o);
                R.df = mx::rot3(L.inv_trans.m, df);
                R.dd = mkv(R.df.x, R.df.y, R.df.z);
                p1 = R.p;
                p2 = xform(L.inv_trans.m, L.inv_trans.t, pend);
                cur_list = l;
            }
            const rp_face &F = S.faces[sel];
            double t = mx::face_t_mixed(S, F, R, tmax, A.err);
            double dist;
            if (t < MX_MISS - 0.5) {
                dist = face_isect(S, F, p1, p2, A.err);  // FP64 path (distortion, polygons, ...)
            } else {
                dist = (t == MX_MISS) ? MX_MISS : t * dlen;
            }
            if (F.tolerance < dist && (dist < len || (dist == len && best >= 0 && sel < best))) {
                len = dist;
                best = sel;
                best_list = l;
            }
        }
        for (int f = nmask; f < nf && A.one_list < 0; f++) {  // faces beyond the first 64: FP64 path
            int l = S.face_list[f];
            if (l < 0 || l >= S.n_lists) break;
            const rp_facelist &L = S.lists[l];
            v3 q1 = xform(L.inv_trans.m, L.inv_trans.t, o), q2 = xform(L.inv_trans.m, L.inv_trans.t, pend);
            const rp_face &F = S.faces[f];
            double dist = face_isect(S, F, q1, q2, A.err);
            if (F.tolerance < dist && (dist < len || (dist == len && best >= 0 && f < best))) {
                len = dist;
                best = f;
                best_list = l;
            }
        }
        A.in.len[i] = len;
        A.in.endf[i] = best >= 0 ? (unsigned)S.faces[best].idx : 0xFFFFFFFFu;
        if (best >= 0) {
            atomicAdd(&s_counts[best], 1u);
            atomicAdd(&s_hits, 1u);
        }
    }

    if (!A.emit) {
        flush_counts(A, S, s_counts);
        if (threadIdx.x == 0) atomicAdd(&A.stats[0], (unsigned long long)s_hits);
        return;
    }

    Child ch[2];
    ChildCommon cc;
    int nc = 0;
    if (active && best >= 0) {
        const rp_facelist &L = S.lists[best_list];
        const rp_face &F = S.faces[best];
        v3 point = addv(o, mulvs(d, len / dlen));  // FP64 hit point
        v3 lp = xform(L.inv_trans.m, L.inv_trans.t, point);
        bool handled;
        mx::f3 nl = mx::face_normal_mixed(S, F, lp, A.err, handled);
        v3 nrm, tng = face_tangent(F);
        if (handled) {
            if (F.invert_normal) nl = mx::mk3(-nl.x, -nl.y, -nl.z);
            nrm = mx::tod(mx::rot3(L.trans.m, nl));
        } else {
            nrm = face_normal(S, F, lp, A.err);
            if (F.invert_normal) nrm = negv(nrm);
            nrm = rotv(L.trans.m, nrm);
        }
        if (F.invert_normal) tng = negv(tng);
        tng = rotv(L.trans.m, tng);
        if (F.material >= 0) {
            RayState r;
            r.o = o;
            r.d = d;
            r.E = mkv(A.in.ex[i], A.in.ey[i], A.in.ez[i]);
            r.n = A.in.n[i];
            r.e1 = A.in.e1[i];
            r.e2 = A.in.e2[i];
            r.len = len;
            r.opl = A.in.opl[i];
            r.type = A.in.type[i];
            r.wl = A.in.wl[i];
            const rp_material &M = S.mats[F.material];
            nc = mx::eval_mixed(S, M, r, point, mx::tof(nrm), cc, ch, A.err);
            if (nc < 0) nc = eval_children(S, M, r, point, nrm, tng, cc, ch, A.err);
            if (A.e2_term > 0.0 && nc > 0) {
                int w = 0;
                for (int k = 0; k < nc; k++) {
                    if (!(child_e2(ch[k]) < A.e2_term)) {
                        if (w != k) ch[w] = ch[k];
                        w++;
                    }
                }
                if (w < nc) atomicAdd(&s_term, (unsigned)(nc - w));
                nc = w;
            }
        }
    }
    // children go to the tile's slot range in parent order: the exclusive
    // block scan of the per-ray counts is each ray's first slot
    unsigned tile_children;
    const unsigned excl = block_scan((unsigned)nc, &tile_children);
    if (nc > 0) {
        double phase = A.in.phase[i];
        unsigned wl = A.in.wl[i], ident = A.in.ident[i];
        unsigned endf = (unsigned)S.faces[best].idx;
        const unsigned long long slot = (unsigned long long)tile * RP_TILE_SLOTS + excl;
        for (int k = 0; k < nc; k++) store_child(A.scratch, slot + k, cc, ch[k], phase, wl, (unsigned)i, endf, ident);
    }
    flush_counts(A, S, s_counts);
    if (threadIdx.x == 0) A.tile_counts[tile] = tile_children;
    if (threadIdx.x == 0) {
        atomicAdd(&A.stats[0], (unsigned long long)s_hits);
        if (s_term) atomicAdd(&A.stats[1], (unsigned long long)s_term);
    }
}

cudaError_t launch_generation_mixed(const GenArgs &a, size_t smem, cudaStream_t st) {
    if (a.n_in == 0) return cudaSuccess;
    unsigned grid = (unsigned)((a.n_in + RP_BLOCK - 1) / RP_BLOCK);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(generation_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    generation_mixed_kernel<<<grid, RP_BLOCK, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace rp
