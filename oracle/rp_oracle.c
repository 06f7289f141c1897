/*
 * rp_oracle.c -- CPU restatement of raypier's non-sequential tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GB300 kernels are
 * checked against: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it; the product package never does.  It restates, in plain C99, the
 * reference algorithm of raypier/core/{ctracer,cfaces,cmaterials,cshapes,
 * cdistortions}.pyx and raypier/core/tracer.py, function by function, with the
 * same operation order and the same libm / C99-complex calls, so that when it
 * is built with the reference's compiler flags (gcc -O2 -ffp-contract=off, no
 * -march=native) it reproduces the reference bit for bit.  It is pinned to the
 * reference by the golden vectors in tests/golden (generated from the reference
 * build by tests/golden/make_golden.py).
 *
 * Layout: rays are the reference's packed 188-byte AoS record (rp_ray); the
 * scene is the table form declared in include/rp_gb300.h.
 */
#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/rp_gb300.h"

typedef double complex cplx;
typedef struct { double x, y, z; } vec;
typedef struct { vec normal, tangent; } orient_t;
typedef struct { double dist; int face_idx; int piece_idx; } isect_t;

/* ctracer.pyx:15 / cfaces.pyx:26: INF = DBL_MAX + DBL_MAX */
static double rp_inf(void) { volatile double m = DBL_MAX; return m + m; }
#define SP_TOL 1.0e-10 /* cmaterials.pyx:31 */

/* Cython's __pyx_t_double_complex_from_parts: x + y*I */
static inline cplx cfp(double x, double y) { return x + y * (cplx)_Complex_I; }
static inline cplx ld_c(const double *p) { cplx z; memcpy(&z, p, sizeof z); return z; }
static inline void st_c(double *p, cplx z) { memcpy(p, &z, sizeof z); }
static inline vec ld_v(const double *p) { vec v = {p[0], p[1], p[2]}; return v; }
static inline void st_v(double *p, vec v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

/* ---- vector maths: ctracer.pyx:83-262 ----------------------------------- */
static inline vec transform_c(const rp_transform *t, vec p) { /* 83-88 */
    vec o;
    o.x = p.x * t->m[0] + p.y * t->m[1] + p.z * t->m[2] + t->t[0];
    o.y = p.x * t->m[3] + p.y * t->m[4] + p.z * t->m[5] + t->t[1];
    o.z = p.x * t->m[6] + p.y * t->m[7] + p.z * t->m[8] + t->t[2];
    return o;
}
static inline vec rotate_c(const rp_transform *t, vec p) { /* 90-95 */
    vec o;
    o.x = p.x * t->m[0] + p.y * t->m[1] + p.z * t->m[2];
    o.y = p.x * t->m[3] + p.y * t->m[4] + p.z * t->m[5];
    o.z = p.x * t->m[6] + p.y * t->m[7] + p.z * t->m[8];
    return o;
}
static inline double sep_(vec p1, vec p2) { /* 108-113 */
    double a = p2.x - p1.x, b = p2.y - p1.y, c = p2.z - p1.z;
    return sqrt((a * a) + (b * b) + (c * c));
}
static inline vec invert_(vec v) { v.x = -v.x; v.y = -v.y; v.z = -v.z; return v; } /* 119-123 */
static inline vec multvs_(vec a, double b) { vec o = {a.x * b, a.y * b, a.z * b}; return o; }
static inline vec addvv_(vec a, vec b) { vec o = {a.x + b.x, a.y + b.y, a.z + b.z}; return o; }
static inline vec subvv_(vec a, vec b) { vec o = {a.x - b.x, a.y - b.y, a.z - b.z}; return o; }
static inline double mag_(vec a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline double mag_sq_(vec a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double dotprod_(vec a, vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline vec cross_(vec a, vec b) { /* 234-239 */
    vec c;
    c.x = a.y * b.z - a.z * b.y;
    c.y = a.z * b.x - a.x * b.z;
    c.z = a.x * b.y - a.y * b.x;
    return c;
}
static inline vec norm_(vec a) { /* 249-254 */
    double mag = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    a.x /= mag; a.y /= mag; a.z /= mag;
    return a;
}

/* ---- shapes: cshapes.pyx ------------------------------------------------- */
static int point_in_polygon_shape(const double *xy, int n, double X, double Y) {
    /* PolygonShape.point_inside_c, cshapes.pyx:147-168 */
    int ct = 0;
    double y1 = xy[2 * (n - 1) + 1], x1 = xy[2 * (n - 1)];
    for (int i = 0; i < n; i++) {
        double y2 = xy[2 * i + 1], x2 = xy[2 * i];
        if ((y1 <= Y && Y < y2) || (y2 <= Y && Y < y1)) {
            if ((x1 + (Y - y1) * (x2 - x1) / (y2 - y1)) > X) ct = !ct;
        }
        y1 = y2; x1 = x2;
    }
    return ct;
}

static int shape_inside(const rp_scene_desc *s, int prog, double x, double y) {
    /* Evaluates a postfix shape program; each op restates one Shape subclass. */
    if (prog < 0) return 1; /* base Shape: ctracer.pyx:1653-1655 */
    int stack[32], sp = 0;
    for (int k = prog; k < s->n_shape_ops; k++) {
        const rp_shape_op *op = &s->shape_ops[k];
        switch (op->op) {
        case RP_SHAPE_END: return sp > 0 ? stack[sp - 1] : 1;
        case RP_SHAPE_TRUE: stack[sp++] = 1; break;
        case RP_SHAPE_CIRCLE: { /* cshapes.pyx:109-116 */
            double dx = x - op->a, dy = y - op->b;
            stack[sp++] = ((dx * dx) + (dy * dy) < (op->c * op->c)) ? 1 : 0;
            break;
        }
        case RP_SHAPE_RECT: { /* cshapes.pyx:128-136 */
            double dx = x - op->a, dy = y - op->b;
            stack[sp++] = ((2 * fabs(dx) < op->c) && (2 * fabs(dy)) < op->d) ? 1 : 0;
            break;
        }
        case RP_SHAPE_POLYGON:
            stack[sp++] = point_in_polygon_shape(s->aux + op->aux, op->n, x, y);
            break;
        case RP_SHAPE_AND: sp--; stack[sp - 1] = stack[sp - 1] & stack[sp]; break;  /* 48-50 */
        case RP_SHAPE_OR:  sp--; stack[sp - 1] = stack[sp - 1] | stack[sp]; break;  /* 53-55 */
        case RP_SHAPE_XOR: sp--; stack[sp - 1] = stack[sp - 1] ^ stack[sp]; break;  /* 58-60 */
        case RP_SHAPE_NOT: stack[sp - 1] = 1 & (~stack[sp - 1]); break;             /* 35-36 */
        default: return 0;
        }
        if (sp >= 31) return 0;
    }
    return sp > 0 ? stack[sp - 1] : 1;
}

/* ---- Zernike distortion: cdistortions.pyx ----------------------------- */
#define ZK_MAXK 64
typedef struct { double w[3][ZK_MAXK]; } zk_ws;

static double zernike_R_c(double r, int k, int n, int m, zk_ws *ws) { /* 149-178 */
    if (n < m) return 0.0;
    if (n == 0) return 1.0;
    double val = ws->w[0][k];
    if (isnan(val)) {
        int nA = n - 1, mA = abs(m - 1), half_n = nA / 2;
        int kA = half_n * (half_n + 1) + abs(mA);
        int nB = nA, mB = m + 1;
        int kB = half_n * (half_n + 1) + abs(mB);
        int nC = n - 2, mC = m;
        half_n = nC / 2;
        int kC = half_n * (half_n + 1) + abs(mC);
        val = r * (zernike_R_c(r, kA, nA, mA, ws) + zernike_R_c(r, kB, nB, mB, ws));
        val -= zernike_R_c(r, kC, nC, mC, ws);
        ws->w[0][k] = val;
        return val;
    }
    return val;
}

static double zernike_Rprime_c(double r, int k, int n, int m, zk_ws *ws) { /* 189-219 */
    if (n < m) return 0.0;
    if (n == 0) return 0.0;
    double val = ws->w[1][k];
    if (isnan(val)) {
        int nA = n - 1, mA = abs(m - 1), half_n = nA / 2;
        int kA = half_n * (half_n + 1) + abs(mA);
        int nB = nA, mB = m + 1;
        int kB = half_n * (half_n + 1) + abs(mB);
        int nC = n - 2, mC = m;
        int kC = (half_n - 1) * half_n + abs(mC); /* 209: as in the reference */
        val = zernike_R_c(r, kA, nA, mA, ws) + zernike_R_c(r, kB, nB, mB, ws);
        val += r * (zernike_Rprime_c(r, kA, nA, mA, ws) + zernike_Rprime_c(r, kB, nB, mB, ws));
        val -= zernike_Rprime_c(r, kC, nC, mC, ws);
        ws->w[1][k] = val;
        return val;
    }
    return val;
}

static double zernike_R_over_r_c(double r, int k, int n, int m, zk_ws *ws) { /* 288-316 */
    if (n < m) return 0.0;
    double val = ws->w[2][k];
    if (isnan(val)) {
        int nA = n - 1, mA = abs(m - 1), half_n = nA / 2;
        int kA = half_n * (half_n + 1) + abs(mA);
        int nB = nA, mB = m + 1;
        int kB = half_n * (half_n + 1) + abs(mB);
        int nC = n - 2, mC = m;
        half_n = nC / 2;
        int kC = half_n * (half_n + 1) + abs(mC);
        val = zernike_R_c(r, kA, nA, mA, ws) + zernike_R_c(r, kB, nB, mB, ws);
        val -= zernike_R_over_r_c(r, kC, nC, mC, ws);
        ws->w[2][k] = val;
    }
    return val;
}

/* coefficient record in aux: j, n, m, k, value */
#define ZC(i, f) (s->aux[d->aux + 5 * (i) + (f)])

static double z_offset_c(const rp_scene_desc *s, const rp_distortion *d, double x, double y) {
    if (d->type == RP_DIST_SIMPLE_J7) { /* cdistortions.pyx:48-60 */
        x /= d->unit_radius;
        y /= d->unit_radius;
        double Z = sqrt(8.0) * (3 * (x * x + y * y) - 2) * y;
        return Z * d->amplitude;
    }
    /* ZernikeDistortion.z_offset_c, cdistortions.pyx:416-450 */
    zk_ws ws;
    double Z = 0.0;
    x /= d->unit_radius;
    y /= d->unit_radius;
    double r = sqrt(x * x + y * y);
    double theta = atan2(y, x);
    for (int i = 0; i < d->k_max; i++) ws.w[0][i] = NAN;
    ws.w[0][0] = 1.0;
    for (int i = 0; i < d->n_coefs; i++) {
        int n = (int)ZC(i, 1), m = (int)ZC(i, 2), k = (int)ZC(i, 3);
        double value = ZC(i, 4), N, PH;
        if (m == 0) N = sqrt(n + 1);
        else N = sqrt(2 * (n + 1));
        N *= value;
        if (m >= 0) PH = cos(m * theta);
        else PH = -sin(m * theta);
        double R = zernike_R_c(r, k, n, abs(m), &ws);
        Z += N * R * PH;
    }
    return Z;
}

static vec z_offset_and_gradient_c(const rp_scene_desc *s, const rp_distortion *d, double x, double y) {
    vec Z;
    if (d->type == RP_DIST_SIMPLE_J7) { /* cdistortions.pyx:62-81 */
        double root8 = sqrt(8) * d->amplitude, R = d->unit_radius;
        x /= R;
        y /= R;
        Z.x = root8 * 6 * x * y / R;
        Z.y = root8 * (3 * x * x + 9 * y * y - 2) / R;
        Z.z = root8 * (3 * (x * x + y * y) - 2) * y;
        return Z;
    }
    /* ZernikeDistortion.z_offset_and_gradient_c, cdistortions.pyx:456-514 */
    zk_ws ws;
    x /= d->unit_radius;
    y /= d->unit_radius;
    double r = sqrt(x * x + y * y);
    double theta = atan2(y, x);
    for (int i = 0; i < d->k_max; i++) { ws.w[0][i] = NAN; ws.w[1][i] = NAN; ws.w[2][i] = NAN; }
    Z.x = 0.0; Z.y = 0.0; Z.z = 0.0;
    for (int i = 0; i < d->n_coefs; i++) {
        int n = (int)ZC(i, 1), m = (int)ZC(i, 2), k = (int)ZC(i, 3);
        double value = ZC(i, 4), N, PH, PHprime;
        if (m >= 0) {
            PH = cos(m * theta);
            PHprime = -m * sin(m * theta);
        } else {
            PH = -sin(m * theta);
            PHprime = -m * cos(m * theta);
        }
        double R = zernike_R_c(r, k, n, abs(m), &ws);
        double Rprime = zernike_Rprime_c(r, k, n, abs(m), &ws);
        double R_over_r = zernike_R_over_r_c(r, k, n, abs(m), &ws);
        if (m == 0) N = sqrt(n + 1);
        else N = sqrt(2 * (n + 1));
        N *= value;
        Z.z += N * R * PH;
        Z.x += N * (Rprime * cos(theta) * PH + R_over_r * (-sin(theta)) * PHprime);
        Z.y += N * (Rprime * sin(theta) * PH + R_over_r * (cos(theta)) * PHprime);
    }
    Z.x /= d->unit_radius;
    Z.y /= d->unit_radius;
    return Z;
}
#undef ZC

/* ---- faces: cfaces.pyx --------------------------------------------------- */
static const isect_t NO_INTERSECTION = {-1.0, -1, 0}; /* cfaces.pyx:40-44 */

static double intersect_conic(vec a, vec d, double curvature, double conic_const) {
    /* cfaces.pyx:1695-1747 */
    double beta = 1 + conic_const;
    double R = -curvature;
    double A = pow(beta, 2.0) * pow(d.z, 2.0) + beta * pow(d.x, 2.0) + beta * pow(d.y, 2.0);
    double B = -2 * R * beta * d.z + 2 * a.x * beta * d.x + 2 * a.y * beta * d.y + 2 * a.z * pow(beta, 2.0) * d.z;
    double C = -2 * R * a.z * beta + pow(a.x, 2.0) * beta + pow(a.y, 2.0) * beta + pow(a.z, 2.0) * pow(beta, 2.0);
    double D = B * B - 4 * A * C;
    if (D < 0) return -1;
    D = sqrt(D);
    if (R * beta * d.z <= 0) return (-B + D) / (2 * A);
    return (-B - D) / (2 * A);
}

typedef struct {
    double R, beta, A4, A6, A8, A10, A12, A14, A16;
    vec a, d;
} aspheric_t;

static double eval_aspheric_impf(aspheric_t A, double alpha) { /* cfaces.pyx:1854-1863 */
    double r2 = (pow((A.a.x + alpha * A.d.x), 2.0) + pow((A.a.y + alpha * A.d.y), 2.0));
    double out = r2;
    out /= A.R * (1 + sqrt(1 - A.beta * r2 / (pow(A.R, 2.0))));
    out -= A.a.z + alpha * A.d.z;
    out += A.A4 * (pow(r2, 2.0)) + A.A6 * (pow(r2, 3.0)) + A.A8 * (pow(r2, 4.0)) + A.A10 * (pow(r2, 5.0))
         + A.A12 * (pow(r2, 6.0)) + A.A14 * (pow(r2, 7.0)) + A.A16 * (pow(r2, 8.0));
    return out;
}

static double eval_aspheric_grad(aspheric_t A, double alpha) { /* cfaces.pyx:1866-1882 */
    double r2 = (pow((A.a.x + alpha * A.d.x), 2.0) + pow((A.a.y + alpha * A.d.y), 2.0));
    double dx = A.d.x * (A.a.x + alpha * A.d.x);
    double dy = A.d.y * (A.a.y + alpha * A.d.y);
    double out = A.A10 * (10 * dx + 10 * dy) * (pow(r2, 4.0));
    out += A.A12 * (12 * dx + 12 * dy) * (pow(r2, 5.0));
    out += A.A14 * (14 * dx + 14 * dy) * (pow(r2, 6.0));
    out += A.A16 * (16 * dx + 16 * dy) * (pow(r2, 7.0));
    out += A.A4 * (4 * dx + 4 * dy) * (r2);
    out += A.A6 * (6 * dx + 6 * dy) * (pow(r2, 2.0));
    out += A.A8 * (8 * dx + 8 * dy) * (pow(r2, 3.0)) - A.d.z;
    out += (2 * dx + 2 * dy) / (A.R * (sqrt(1 - A.beta * (r2) / pow(A.R, 2.0)) + 1));
    out += A.beta * (2 * dx + 2 * dy) * (r2)
         / (2 * (pow(A.R, 3.0)) * sqrt(1 - A.beta * r2 / (pow(A.R, 2.0))) * pow((sqrt(1 - A.beta * r2 / (pow(A.R, 2.0))) + 1), 2.0));
    return out;
}

/* ExtendedPolynomialFace helpers: cfaces.pyx:2043-2126.  f->p: R, beta, norm_radius, z_height, atol */
static double eval_extpoly_impf(const rp_scene_desc *s, const rp_face *f, vec a, vec d, double alpha) {
    const double *E = s->aux + f->aux;
    int Nx = f->n_aux0, Ny = f->n_aux1;
    double x = a.x + alpha * d.x;
    double y = a.y + alpha * d.y;
    double r2 = pow(x, 2.0) + pow(y, 2.0);
    double R = f->p[0], beta = f->p[1];
    double out = r2;
    if (R >= 0) out /= (R + sqrt(R * R - beta * r2));
    else out /= (R - sqrt(R * R - beta * r2));
    out -= a.z + alpha * d.z;
    x /= f->p[2];
    y /= f->p[2];
    for (int i = 0; i < Nx; i++)
        for (int j = 0; j < Ny; j++)
            out += E[i * Ny + j] * pow(x, (double)i) * pow(y, (double)j);
    out += f->p[3];
    return out;
}

static double eval_extpoly_grad(const rp_scene_desc *s, const rp_face *f, vec a, vec d, double alpha) {
    const double *E = s->aux + f->aux;
    int Nx = f->n_aux0, Ny = f->n_aux1;
    double R = f->p[0], beta = f->p[1];
    double dEdx = 0.0, dEdy = 0.0;
    double x = a.x + alpha * d.x;
    double y = a.y + alpha * d.y;
    double r2 = pow(x, 2.0) + pow(y, 2.0);
    double R2 = R * R;
    double rt = sqrt(1 - (beta * r2 / R2));
    double denom = R * (rt + 1);
    double nom = (2 * d.x * x + 2 * d.y * y);
    double inv_rad = 1. / f->p[2];
    double out = -d.z;
    out += nom / denom;
    out += beta * nom * r2 / (2 * R * rt * denom * denom);
    x *= inv_rad;
    y *= inv_rad;
    for (int i = 1; i < Nx; i++)
        for (int j = 0; j < Ny; j++)
            dEdx += (i) * E[i * Ny + j] * pow(x, (double)(i - 1)) * pow(y, (double)j);
    for (int i = 0; i < Nx; i++)
        for (int j = 1; j < Ny; j++)
            dEdy += (j) * E[i * Ny + j] * pow(x, (double)i) * pow(y, (double)(j - 1));
    dEdx *= inv_rad;
    dEdy *= inv_rad;
    out += dEdx * d.x;
    out += dEdy * d.y;
    return out;
}

static int point_in_polygon_c(const double *xy, int size, double X, double Y) { /* cfaces.pyx:1050-1068 */
    int ct = 0;
    double y1 = xy[2 * (size - 1) + 1], x1 = xy[2 * (size - 1)];
    for (int i = 0; i < size; i++) {
        double y2 = xy[2 * i + 1], x2 = xy[2 * i];
        double h = (Y - y1) / (y2 - y1);
        if (0 < h && h <= 1.0) {
            double x = x1 + h * (x2 - x1);
            if (x > X) ct = !ct;
        }
        y1 = y2; x1 = x2;
    }
    return ct;
}

static vec face_normal(const rp_scene_desc *s, const rp_face *f, vec p, int piece);

static isect_t face_intersect(const rp_scene_desc *s, const rp_face *f, vec p1, vec p2, int is_base_ray) {
    isect_t out = NO_INTERSECTION;
    switch (f->type) {
    case RP_FACE_NONE: /* Face.intersect_c, ctracer.pyx:1747-1757 */
        out.dist = 0.0; out.face_idx = f->idx; out.piece_idx = 0;
        return out;
    case RP_FACE_CIRCULAR: { /* cfaces.pyx:147-175 */
        double max_length = sep_(p1, p2);
        double h = (f->p[2] - p1.z) / (p2.z - p1.z);
        double d = f->p[0];
        if ((h < f->tolerance) || (h > 1.0)) return NO_INTERSECTION;
        double X = p1.x + h * (p2.x - p1.x) - f->p[1];
        double Y = p1.y + h * (p2.y - p1.y);
        if (is_base_ray && (X * X + Y * Y) > (d * d / 4)) return NO_INTERSECTION;
        out.dist = h * max_length;
        return out;
    }
    case RP_FACE_SHAPED_PLANAR: { /* cfaces.pyx:201-227 */
        double max_length = sep_(p1, p2);
        double h = (f->p[0] - p1.z) / (p2.z - p1.z);
        if ((h < f->tolerance) || (h > 1.0)) return NO_INTERSECTION;
        double X = p1.x + h * (p2.x - p1.x);
        double Y = p1.y + h * (p2.y - p1.y);
        if (is_base_ray && !shape_inside(s, f->shape, X, Y)) return NO_INTERSECTION;
        out.dist = h * max_length;
        return out;
    }
    case RP_FACE_ELLIPTICAL_PLANE: { /* cfaces.pyx:323-340 */
        double max_length = sep_(p1, p2);
        double gx = f->p[0], gy = f->p[1], d = f->p[2];
        double h = (gx * p1.x + gy * p1.y - p1.z) / ((p2.z - p1.z) - gx * (p2.x - p1.x) - gy * (p2.y - p1.y));
        if ((h < f->tolerance) || (h > 1.0)) return NO_INTERSECTION;
        double X = p1.x + h * (p2.x - p1.x);
        double Y = p1.y + h * (p2.y - p1.y);
        if (is_base_ray && (X * X + Y * Y) > (d * d / 4)) return NO_INTERSECTION;
        out.dist = h * max_length;
        return out;
    }
    case RP_FACE_RECTANGULAR: { /* cfaces.pyx:364-396; p: length, width, offset, z_plane */
        double max_length = sep_(p1, p2);
        double h = (f->p[3] - p1.z) / (p2.z - p1.z);
        double lngth = f->p[0], wdth = f->p[1];
        if ((h < f->tolerance) || (h > 1.0)) return NO_INTERSECTION;
        if (is_base_ray) {
            double X = p1.x + h * (p2.x - p1.x) - f->p[2];
            double Y = p1.y + h * (p2.y - p1.y);
            if (X * X > lngth * lngth / 4) return NO_INTERSECTION;
            if (Y * Y > wdth * wdth / 4) return NO_INTERSECTION;
        }
        out.dist = h * max_length;
        return out;
    }
    case RP_FACE_POLYGON: { /* cfaces.pyx:1096-1108 */
        double max_length = sep_(p1, p2);
        double h = (f->p[0] - p1.z) / (p2.z - p1.z);
        if ((h < f->tolerance) || (h > 1.0)) return NO_INTERSECTION;
        double X = p1.x + h * (p2.x - p1.x);
        double Y = p1.y + h * (p2.y - p1.y);
        if (is_base_ray && point_in_polygon_c(s->aux + f->aux, f->n_aux0, X, Y) == 1)
            out.dist = h * max_length;
        return out;
    }
    case RP_FACE_SPHERICAL:
    case RP_FACE_SHAPED_SPHERICAL: { /* cfaces.pyx:418-482 and 512-592 */
        double curvature, z_height;
        if (f->type == RP_FACE_SPHERICAL) { curvature = f->p[1]; z_height = f->p[2]; }
        else { curvature = f->p[0]; z_height = f->p[1]; }
        vec r = p1;
        vec sv = subvv_(p2, r);
        double cz = z_height - curvature;
        vec d = r;
        d.z -= cz;
        double A = mag_sq_(sv);
        double B = 2 * dotprod_(sv, d);
        double C = mag_sq_(d) - pow(curvature, 2.0);
        double D = B * B - 4 * A * C;
        if (D < 0) return NO_INTERSECTION;
        D = sqrt(D);
        double a1 = (-B + D) / (2 * A);
        vec pt1 = addvv_(r, multvs_(sv, a1));
        double a2 = (-B - D) / (2 * A);
        vec pt2 = addvv_(r, multvs_(sv, a2));
        if (curvature >= 0) {
            if (pt1.z < cz) a1 = rp_inf();
            if (pt2.z < cz) a2 = rp_inf();
        } else {
            if (pt1.z > cz) a1 = rp_inf();
            if (pt2.z > cz) a2 = rp_inf();
        }
        if (f->type == RP_FACE_SPHERICAL) {
            D = f->p[0] * f->p[0] / 4.;
            if (is_base_ray) {
                if ((pt1.x * pt1.x + pt1.y * pt1.y) > D) a1 = rp_inf();
                if ((pt2.x * pt2.x + pt2.y * pt2.y) > D) a2 = rp_inf();
            }
        } else if (is_base_ray) {
            if (!shape_inside(s, f->shape, pt1.x, pt1.y)) a1 = rp_inf();
            if (!shape_inside(s, f->shape, pt2.x, pt2.y)) a2 = rp_inf();
        }
        if (a2 < a1) a1 = a2;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(r, p2);
        return out;
    }
    case RP_FACE_CONIC: { /* cfaces.pyx:1766-1794; p: curvature, z_height, conic_const */
        vec d = subvv_(p2, p1);
        vec a = p1;
        a.z -= f->p[1];
        double a1 = intersect_conic(a, d, f->p[0], f->p[2]);
        vec pt1 = addvv_(a, multvs_(d, a1));
        if (is_base_ray && !shape_inside(s, f->shape, pt1.x, pt1.y)) return NO_INTERSECTION;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(p1, p2);
        return out;
    }
    case RP_FACE_ASPHERIC: { /* cfaces.pyx:1908-1974; p: curvature, z_height, conic, A4..A16, atol */
        double tol = pow(f->p[10], 2.0);
        vec d = subvv_(p2, p1);
        vec a = p1;
        a.z -= f->p[1];
        double a1 = intersect_conic(a, d, f->p[0], f->p[2]);
        aspheric_t A;
        A.R = -f->p[0];
        A.beta = 1 + f->p[2];
        A.A4 = f->p[3]; A.A6 = f->p[4]; A.A8 = f->p[5]; A.A10 = f->p[6];
        A.A12 = f->p[7]; A.A14 = f->p[8]; A.A16 = f->p[9];
        A.a = a;
        A.d = d;
        double f_, f_last, dz;
        f_ = f_last = eval_aspheric_impf(A, a1);
        dz = -f_ / eval_aspheric_grad(A, a1);
        int converged = 0;
        for (int i = 0; i < 100; i++) {
            a1 += dz;
            if (dz * dz < tol) { converged = 1; break; }
            f_ = eval_aspheric_impf(A, a1);
            if (fabs(f_) > fabs(f_last)) return NO_INTERSECTION;
            f_last = f_;
            dz = -f_ / eval_aspheric_grad(A, a1);
        }
        if (!converged) return NO_INTERSECTION;
        vec pt1 = addvv_(a, multvs_(d, a1));
        if (is_base_ray && !shape_inside(s, f->shape, pt1.x, pt1.y)) return NO_INTERSECTION;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(p1, p2);
        return out;
    }
    case RP_FACE_EXTPOLY: { /* cfaces.pyx:2182-2234; p: R, beta, norm_radius, z_height, atol */
        double tol = pow(f->p[4], 2.0);
        vec d = subvv_(p2, p1);
        vec a = p1;
        a.z -= f->p[3];
        double a1 = intersect_conic(a, d, -f->p[0], f->p[1] - 1.0);
        double f_, f_last, dz;
        /* the reference evaluates the polynomial from p1 (not a): cfaces.pyx:2211-2212 */
        f_ = f_last = eval_extpoly_impf(s, f, p1, d, a1);
        dz = -f_ / eval_extpoly_grad(s, f, p1, d, a1);
        int converged = 0;
        for (int i = 0; i < 100; i++) {
            a1 += dz;
            if (dz * dz < tol) { converged = 1; break; }
            f_ = eval_extpoly_impf(s, f, p1, d, a1);
            if (fabs(f_) > fabs(f_last)) return NO_INTERSECTION;
            f_last = f_;
            dz = -f_ / eval_extpoly_grad(s, f, p1, d, a1);
        }
        if (!converged) return NO_INTERSECTION;
        vec pt1 = addvv_(a, multvs_(d, a1));
        if (is_base_ray && !shape_inside(s, f->shape, pt1.x, pt1.y)) return NO_INTERSECTION;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(p1, p2);
        return out;
    }
    case RP_FACE_ORIENTED_POLYGON: { /* cfaces.pyx:1189-1215 */
        vec n = ld_v(&f->p[3]), o = ld_v(&f->p[0]);
        vec xa = ld_v(&f->p[6]), ya = ld_v(&f->p[9]);
        vec line = subvv_(p2, p1);
        double max_length = mag_(line);
        line = norm_(line);
        double h = dotprod_(line, n);
        if (h == 0.0) return NO_INTERSECTION;
        h = dotprod_(subvv_(o, p1), n) / h;
        if ((h < f->tolerance) || (h > max_length)) return NO_INTERSECTION;
        if (is_base_ray) {
            line = subvv_(addvv_(p1, multvs_(line, h)), o);
            double X = dotprod_(line, xa);
            double Y = dotprod_(line, ya);
            if (point_in_polygon_c(s->aux + f->aux, f->n_aux0, X, Y) == 1) out.dist = h;
        } else {
            out.dist = h;
        }
        return out;
    }
    case RP_FACE_OFF_AXIS_PARABOLIC: { /* cfaces.pyx:1228-1297; p: EFL, diameter, height */
        double efl = f->p[0], A = 1 / (2 * f->p[0]);
        double a, b, c, d, a1, a2;
        vec sv = subvv_(p2, p1), r = p1, pt1, pt2;
        r.z += efl / 2.;
        a = A * (pow(sv.x, 2.0) + pow(sv.y, 2.0));
        b = 2 * A * (r.x * sv.x + r.y * sv.y) - sv.z;
        c = A * (pow(r.x, 2.0) + pow(r.y, 2.0)) - r.z;
        d = pow(b, 2.0) - 4 * a * c;
        if (d < 0) return NO_INTERSECTION;
        if (a < 1e-10) {
            a1 = -c / b;
            pt1 = addvv_(r, multvs_(sv, a1));
            pt1.x -= efl;
            if ((pt1.x * pt1.x + pt1.y * pt1.y) > (f->p[1] / 2)) return NO_INTERSECTION;
            if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
            out.dist = a1 * sep_(p1, p2);
            return out;
        }
        d = sqrt(d);
        a1 = (-b + d) / (2 * a);
        pt1 = addvv_(r, multvs_(sv, a1));
        a2 = (-b - d) / (2 * a);
        pt2 = addvv_(r, multvs_(sv, a2));
        pt1.x -= efl;
        pt2.x -= efl;
        if (is_base_ray) {
            d = f->p[1];
            d *= d / 4.;
            if ((pt1.x * pt1.x + pt1.y * pt1.y) > d) a1 = rp_inf();
            if ((pt2.x * pt2.x + pt2.y * pt2.y) > d) a2 = rp_inf();
        }
        if (a2 < a1) a1 = a2;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(p1, p2);
        return out;
    }
    case RP_FACE_ELLIPSOIDAL: { /* cfaces.pyx:1339-1384; p: major, minor, x1, x2, y1, y2, z1, z2 */
        const rp_transform *trans = (const rp_transform *)(s->aux + f->aux);
        vec S = subvv_(p2, p1);
        vec r = transform_c(trans, p1);
        vec sv = transform_c(trans, p2);
        double A, B, a, b, c, d, root1, root2;
        sv = subvv_(sv, r);
        B = pow(f->p[1], 2.0);
        A = pow(f->p[0], 2.0);
        a = A * (sv.z * sv.z + sv.y * sv.y) + B * sv.x * sv.x;
        b = 2 * (A * (r.z * sv.z + r.y * sv.y) + B * r.x * sv.x);
        c = A * (r.z * r.z + r.y * r.y) + B * r.x * r.x - A * B;
        d = b * b - 4 * a * c;
        d = sqrt(d);
        root1 = (-b + d) / (2 * a);
        root2 = (-b - d) / (2 * a);
        p2 = addvv_(p1, multvs_(S, root2));
        p1 = addvv_(p1, multvs_(S, root1));
        if (is_base_ray) {
            if (!(f->p[2] < p2.x && p2.x < f->p[3])) root2 = 2;
            if (!(f->p[4] < p2.y && p2.y < f->p[5])) root2 = 2;
            if (!(f->p[6] < p2.z && p2.z < f->p[7])) root2 = 2;
            if (!(f->p[2] < p1.x && p1.x < f->p[3])) root1 = 2;
            if (!(f->p[4] < p1.y && p1.y < f->p[5])) root1 = 2;
            if (!(f->p[6] < p1.z && p1.z < f->p[7])) root1 = 2;
        }
        if (root1 < f->tolerance) root1 = 2;
        if (root2 < f->tolerance) root2 = 2;
        if (root1 > root2) root1 = root2;
        if (root1 > 1) return NO_INTERSECTION;
        out.dist = root1 * mag_(S);
        return out;
    }
    case RP_FACE_SADDLE: { /* cfaces.pyx:1421-1495; p: z_height, curvature */
        double A = sqrt(6.0), root, denom, a1, a2;
        vec d, p, pt1, pt2;
        A *= f->p[1];
        p = p1;
        p.z -= f->p[0];
        d = subvv_(p2, p1);
        if (d.x == 0.0) {
            a1 = (-A * (p.x * p.y) + p.z) / (A * d.y * p.x - d.z);
            a2 = rp_inf();
        } else if (d.y == 0.0) {
            a1 = (-A * (p.x * p.y) + p.z) / (A * d.x * p.y - d.z);
            a2 = rp_inf();
        } else {
            root = (pow(A, 2.0)) * (pow(d.x, 2.0)) * (pow(p.y, 2.0)) - 2 * (pow(A, 2.0)) * d.x * d.y * p.x * p.y +
                   (pow(A, 2.0)) * (pow(d.y, 2.0)) * (pow(p.x, 2.0)) + 4 * A * d.x * d.y * p.z -
                   2 * A * d.x * d.z * p.y - 2 * A * d.y * d.z * p.x + pow(d.z, 2.0);
            if (root < 0) return NO_INTERSECTION;
            root = sqrt(root);
            denom = 2 * A * (d.x * d.y);
            a1 = a2 = -A * d.x * p.y - A * d.y * p.x + d.z;
            a1 += root;
            a2 -= root;
            a1 /= denom;
            a2 /= denom;
        }
        pt1 = addvv_(p1, multvs_(d, a1));
        pt2 = addvv_(p1, multvs_(d, a2));
        if (a1 < 0.0) a1 = rp_inf();
        if (a2 < 0.0) a2 = rp_inf();
        if (is_base_ray) {
            if (!shape_inside(s, f->shape, pt1.x, pt1.y)) a1 = rp_inf();
            if (!shape_inside(s, f->shape, pt2.x, pt2.y)) a2 = rp_inf();
        }
        if (a2 < a1) a1 = a2;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(p1, p2);
        return out;
    }
    case RP_FACE_CYLINDRICAL: { /* cfaces.pyx:1524-1582; p: z_height, radius */
        double R = f->p[1], R2 = R * R, a1, a2, cz, ox2, oz2, dx2, dz2, denom, root;
        vec d, o, pt1, pt2;
        o = p1;
        o.z -= f->p[0];
        d = subvv_(p2, p1);
        ox2 = o.x * o.x;
        oz2 = o.z * o.z;
        dx2 = d.x * d.x;
        dz2 = d.z * d.z;
        root = R2 * dz2 - 2 * R * dx2 * o.z + 2 * R * d.x * d.z * o.x - dx2 * oz2 + 2 * d.x * d.z * o.x * o.z -
               dz2 * ox2;
        if (root < 0) return NO_INTERSECTION;
        root = sqrt(root);
        denom = dx2 + dz2;
        a1 = a2 = -R * d.z - d.x * o.x - d.z * o.z;
        a1 += root;
        a2 -= root;
        a1 /= denom;
        a2 /= denom;
        pt1 = addvv_(p1, multvs_(d, a1));
        pt2 = addvv_(p1, multvs_(d, a2));
        cz = f->p[0] - f->p[1];
        if (R >= 0) {
            if (pt1.z < cz) a1 = rp_inf();
            if (pt2.z < cz) a2 = rp_inf();
        } else {
            if (pt1.z > cz) a1 = rp_inf();
            if (pt2.z > cz) a2 = rp_inf();
        }
        if (is_base_ray) {
            if (!shape_inside(s, f->shape, pt1.x, pt1.y)) a1 = rp_inf();
            if (!shape_inside(s, f->shape, pt2.x, pt2.y)) a2 = rp_inf();
        }
        if (a2 < a1) a1 = a2;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(p1, p2);
        return out;
    }
    case RP_FACE_AXICON: { /* cfaces.pyx:1617-1664; p: z_height, gradient */
        double a1, a2, root, ox2, oy2, oz2, dx2, dy2, dz2, beta2, denom, beta = f->p[1];
        vec o, d, pt1, pt2;
        d = subvv_(p2, p1);
        o = p1;
        o.z -= f->p[0];
        beta2 = beta * beta;
        ox2 = o.x * o.x;
        oy2 = o.y * o.y;
        oz2 = o.z * o.z;
        dx2 = d.x * d.x;
        dy2 = d.y * d.y;
        dz2 = d.z * d.z;
        root = -beta2 * dx2 * oy2 + 2 * beta2 * d.x * d.y * o.x * o.y - beta2 * dy2 * ox2 + dx2 * oz2 -
               2 * d.x * d.z * o.x * o.z + dy2 * oz2 - 2 * d.y * d.z * o.y * o.z + dz2 * ox2 + dz2 * oy2;
        denom = (beta2 * dx2 + beta2 * dy2 - dz2);
        if (root < 0) return NO_INTERSECTION;
        root = beta * sqrt(root);
        a1 = -beta2 * d.x * o.x - beta2 * d.y * o.y + d.z * o.z;
        a2 = a1 + root;
        a1 -= root;
        a1 /= denom;
        a2 /= denom;
        pt1 = addvv_(p1, multvs_(d, a1));
        pt2 = addvv_(p1, multvs_(d, a2));
        if (pt1.z > f->p[0]) a1 = rp_inf();
        if (pt2.z > f->p[0]) a2 = rp_inf();
        if (is_base_ray) {
            if (!shape_inside(s, f->shape, pt1.x, pt1.y)) a1 = rp_inf();
            if (!shape_inside(s, f->shape, pt2.x, pt2.y)) a2 = rp_inf();
        }
        if (a2 < a1) a1 = a2;
        if (a1 > 1.0 || a1 < f->tolerance) return NO_INTERSECTION;
        out.dist = a1 * sep_(p1, p2);
        return out;
    }
    case RP_FACE_DISTORTION: { /* cfaces.pyx:2341-2407 */
        const rp_face *face = &s->faces[f->base];
        const rp_distortion *dist = &s->distortions[f->distortion];
        double z_shift = 0.0, a1, a2, h = sep_(p2, p1);
        double tolerance = f->p[0];
        isect_t fout = face_intersect(s, face, p1, p2, 0);
        a2 = fout.dist;
        if (a2 > h || a2 < f->tolerance) return NO_INTERSECTION;
        vec d = subvv_(p2, p1);
        vec pt1 = addvv_(p1, multvs_(d, a2 / h));
        vec dxdyz = z_offset_and_gradient_c(s, dist, pt1.x, pt1.y);
        vec n = face_normal(s, face, pt1, fout.piece_idx);
        pt1.z += dxdyz.z;
        n.x /= n.z;
        n.y /= n.z;
        n.x -= dxdyz.x;
        n.y -= dxdyz.y;
        vec o = subvv_(p1, pt1);
        a1 = -h * dotprod_(o, n) / dotprod_(d, n);
        if (a1 < fabs(dxdyz.z)) return NO_INTERSECTION;
        for (int i = 0; i < 20; i++) {
            pt1 = addvv_(p1, multvs_(d, a1 / h));
            if (fabs(a1 - a2) < tolerance) break;
            z_shift = z_offset_c(s, dist, pt1.x, pt1.y);
            vec q1 = p1, q2 = p2;
            q1.z -= z_shift;
            q2.z -= z_shift;
            fout = face_intersect(s, face, q1, q2, 0);
            a2 = fout.dist;
            pt1 = addvv_(q1, multvs_(d, a2 / h));
            n = face_normal(s, face, pt1, fout.piece_idx);
            dxdyz = z_offset_and_gradient_c(s, dist, pt1.x, pt1.y);
            pt1.z += dxdyz.z;
            n.x /= n.z;
            n.y /= n.z;
            n.x -= dxdyz.x;
            n.y -= dxdyz.y;
            o = subvv_(p1, pt1);
            a2 = a1;
            a1 = -h * dotprod_(o, n) / dotprod_(d, n);
        }
        if (!shape_inside(s, f->shape, pt1.x, pt1.y)) return NO_INTERSECTION;
        fout.dist = a1;
        return fout;
    }
    default:
        return NO_INTERSECTION;
    }
}

static vec face_normal(const rp_scene_desc *s, const rp_face *f, vec p, int piece) {
    vec nrm;
    (void)piece;
    switch (f->type) {
    case RP_FACE_CIRCULAR: /* cfaces.pyx:177-191 */
        nrm.x = 0; nrm.y = 0; nrm.z = f->invert_normals ? 1 : -1;
        return nrm;
    case RP_FACE_SHAPED_PLANAR: /* cfaces.pyx:229-237 */
        nrm.x = 0; nrm.y = 0; nrm.z = 1;
        return nrm;
    case RP_FACE_ELLIPTICAL_PLANE: /* cfaces.pyx:342-351 */
        nrm.x = f->p[0]; nrm.y = f->p[1]; nrm.z = -1;
        return norm_(nrm);
    case RP_FACE_RECTANGULAR: /* cfaces.pyx:398-407 */
    case RP_FACE_POLYGON:     /* cfaces.pyx:1110-1118 */
        nrm.x = 0; nrm.y = 0; nrm.z = -1;
        return nrm;
    case RP_FACE_SPHERICAL:
    case RP_FACE_SHAPED_SPHERICAL: { /* cfaces.pyx:485-498, 594-606 */
        double curvature = f->type == RP_FACE_SPHERICAL ? f->p[1] : f->p[0];
        double z_height = f->type == RP_FACE_SPHERICAL ? f->p[2] : f->p[1];
        p.z -= (z_height - curvature);
        if (curvature < 0) { p.z = -p.z; p.y = -p.y; p.x = -p.x; }
        return norm_(p);
    }
    case RP_FACE_CONIC: { /* cfaces.pyx:1796-1820 */
        double R = -f->p[0];
        double beta = 1 + f->p[2];
        vec g;
        int sign = f->invert_normals ? -1 : 1;
        p.z -= f->p[1];
        g.z = 2 * beta * (R - beta * p.z);
        g.x = -p.x * 2 * beta;
        g.y = -p.y * 2 * beta;
        if ((R * beta) < 0) sign *= -1;
        g.z *= sign; g.y *= sign; g.x *= sign;
        return norm_(g);
    }
    case RP_FACE_ASPHERIC: { /* cfaces.pyx:1976-2005 */
        double R = -f->p[0];
        double beta = 1 + f->p[2];
        vec g;
        int sign = f->invert_normals ? -1 : 1;
        p.z -= f->p[1];
        double r2 = p.x * p.x + p.y * p.y;
        double root = sqrt(1 - (beta * (r2) / (R * R)));
        double df = 10 * f->p[6] * (pow(r2, 4.0)) + 8 * f->p[5] * (pow(r2, 3.0)) + 6 * f->p[4] * (pow(r2, 2.0)) + 4 * f->p[3] * r2;
        df += 16 * f->p[9] * (pow(r2, 7.0)) + 14 * f->p[8] * (pow(r2, 6.0)) + 12 * f->p[7] * (pow(r2, 5.0));
        df += 2 / (R * (1 + root));
        df += beta * (r2) / ((pow(R, 3.0)) * root * (pow((1 + root), 2.0)));
        g.z = 1.0;
        g.x = -df * p.x;
        g.y = -df * p.y;
        g.z *= sign; g.y *= sign; g.x *= sign;
        return norm_(g);
    }
    case RP_FACE_EXTPOLY: { /* cfaces.pyx:2236-2293 */
        const double *E = s->aux + f->aux;
        int Nx = f->n_aux0, Ny = f->n_aux1;
        double R = f->p[0], beta = f->p[1];
        vec g;
        int sign = f->invert_normals ? -1 : 1;
        double inv_rad = 1. / f->p[2];
        double x = p.x * inv_rad;
        double y = p.y * inv_rad;
        p.z -= f->p[3];
        g.z = 2 * beta * (R - beta * p.z);
        g.x = -p.x * 2 * beta;
        g.y = -p.y * 2 * beta;
        if ((R * beta) < 0) sign *= -1;
        g.z *= sign; g.y *= sign; g.x *= sign;
        g = norm_(g);
        if (f->invert_normals) {
            for (int i = 1; i < Nx; i++)
                for (int j = 0; j < Ny; j++)
                    g.x += i * E[i * Ny + j] * inv_rad * pow(x, (double)(i - 1)) * pow(y, (double)j);
            for (int i = 0; i < Nx; i++)
                for (int j = 1; j < Ny; j++)
                    g.y += j * E[i * Ny + j] * inv_rad * pow(x, (double)i) * pow(y, (double)(j - 1));
        } else {
            for (int i = 1; i < Nx; i++)
                for (int j = 0; j < Ny; j++)
                    g.x -= i * E[i * Ny + j] * inv_rad * pow(x, (double)(i - 1)) * pow(y, (double)j);
            for (int i = 0; i < Nx; i++)
                for (int j = 1; j < Ny; j++)
                    g.y -= j * E[i * Ny + j] * inv_rad * pow(x, (double)i) * pow(y, (double)(j - 1));
        }
        return norm_(g);
    }
    case RP_FACE_ORIENTED_POLYGON: /* cfaces.pyx:1183-1184 */
        return ld_v(&f->p[3]);
    case RP_FACE_OFF_AXIS_PARABOLIC: { /* cfaces.pyx:1299-1315 */
        double A = 1 / (2 * f->p[0]), B, dz, m2;
        vec n;
        m2 = p.x * p.x + p.y * p.y;
        B = 4 * m2 * A * A;
        dz = -sqrt(B / (B + 1));
        m2 = sqrt(m2);
        n.x = -(dz * p.x) / m2;
        n.y = -(dz * p.y) / m2;
        n.z = -1 / sqrt(B + 1);
        return n;
    }
    case RP_FACE_ELLIPSOIDAL: { /* cfaces.pyx:1386-1396 */
        const rp_transform *trans = (const rp_transform *)(s->aux + f->aux);
        vec n;
        p = transform_c(trans, p);
        n.x = p.x / -(pow(f->p[0], 2.0));
        n.y = p.y / -(pow(f->p[1], 2.0));
        n.z = p.z / -(pow(f->p[1], 2.0));
        n = rotate_c(trans + 1, n);
        return norm_(n);
    }
    case RP_FACE_SADDLE: { /* cfaces.pyx:1497-1508 */
        double rt6 = sqrt(6) * f->p[1];
        vec n;
        n.z = 1.0;
        n.x = -rt6 * p.y;
        n.y = -rt6 * p.x;
        return norm_(n);
    }
    case RP_FACE_CYLINDRICAL: /* cfaces.pyx:1584-1595 */
        p.z -= (f->p[0] - f->p[1]);
        if (f->p[1] < 0) {
            p.z = -p.z;
            p.x = -p.x;
        }
        p.y = 0;
        return norm_(p);
    case RP_FACE_AXICON: { /* cfaces.pyx:1666-1677 */
        double beta = f->p[1], r = sqrt(p.x * p.x + p.y * p.y);
        p.z = 1.0;
        p.x = beta * p.x / r;
        p.y = beta * p.y / r;
        return p;
    }
    case RP_FACE_DISTORTION: { /* cfaces.pyx:2409-2422 */
        const rp_face *base = &s->faces[f->base];
        vec dxdyz = z_offset_and_gradient_c(s, &s->distortions[f->distortion], p.x, p.y);
        vec p1 = p;
        p1.z -= dxdyz.z;
        vec n = face_normal(s, base, p1, piece);
        n.x /= n.z;
        n.y /= n.z;
        n.z = 1.0;
        n.x -= dxdyz.x;
        n.y -= dxdyz.y;
        return norm_(n);
    }
    default: /* Face.compute_normal_c returns p: ctracer.pyx:1783-1784 */
        return p;
    }
}

static vec face_tangent(const rp_face *f) {
    if (f->type == RP_FACE_ORIENTED_POLYGON) return ld_v(&f->p[6]); /* cfaces.pyx:1186-1187 */
    vec t = {1.0, 0.0, 0.0}; /* ctracer.pyx:1786-1791 */
    return t;
}

/* ---- materials: cmaterials.pyx ------------------------------------------- */
static rp_ray convert_to_sp(rp_ray ray, vec normal) { /* cmaterials.pyx:49-91 */
    cplx E1_amp = ld_c(ray.E1_amp), E2_amp = ld_c(ray.E2_amp);
    vec dir = ld_v(ray.direction), Ev = ld_v(ray.E_vector);
    vec E2_vector = norm_(cross_(dir, Ev));
    vec E1_vector = norm_(cross_(E2_vector, dir));
    normal = norm_(normal);
    vec S_vector = cross_(dir, normal);
    if (fabs(S_vector.x) < SP_TOL && fabs(S_vector.y) < SP_TOL && fabs(S_vector.z) < SP_TOL) return ray;
    S_vector = norm_(S_vector);
    vec v = cross_(dir, S_vector);
    vec P_vector = norm_(v);
    double A = dotprod_(E1_vector, S_vector);
    double B = dotprod_(E2_vector, S_vector);
    double S_re = creal(E1_amp) * A + creal(E2_amp) * B;
    double S_im = cimag(E1_amp) * A + cimag(E2_amp) * B;
    B = dotprod_(E1_vector, P_vector);
    A = dotprod_(E2_vector, P_vector);
    double P_re = creal(E1_amp) * B + creal(E2_amp) * A;
    double P_im = cimag(E1_amp) * B + cimag(E2_amp) * A;
    st_v(ray.E_vector, S_vector);
    ray.E1_amp[0] = S_re; ray.E1_amp[1] = S_im;
    ray.E2_amp[0] = P_re; ray.E2_amp[1] = P_im;
    return ray;
}

typedef struct {
    rp_ray *rays;
    uint64_t n, cap;
    int overflow;
} ray_sink;

static void add_ray(ray_sink *o, const rp_ray *r) { /* RayCollection.add_ray_c, ctracer.pyx:1004-1012 */
    if (o->n >= o->cap) { o->overflow = 1; return; }
    o->rays[o->n++] = *r;
}

/* The complex index seen by a material for wavelength index wl: for a
 * FullDielectricDispersiveMaterial it is the table value computed by
 * on_set_wavelengths (cmaterials.pyx:883-887). */
typedef struct {
    const rp_scene_desc *s;
    const cplx *n_tab;   /* [n_dispersions][n_wl] */
    int64_t n_wl;
    const double *wl;    /* the wavelengths (InterfaceMaterial._wavelengths) */
} mat_ctx;

static void fresnel_split(const mat_ctx *mc, const rp_material *m, cplx n1_in, cplx n2_in,
                          int use_table, const rp_ray *in_ray, uint32_t idx, vec point,
                          orient_t orient, ray_sink *out) {
    /* FullDielectricMaterial.eval_child_ray_c (cmaterials.pyx:756-872) and
     * FullDielectricDispersiveMaterial.eval_child_ray_c (cmaterials.pyx:897-1013) */
    cplx n1, n2, cos2, sin2, R_p, R_s, T_p, T_s, E1_amp, E2_amp;
    double cosTheta, cos1, sin1, P_in, tan_mag_sq, c2, aspect;
    int flip;
    vec normal = norm_(orient.normal);
    vec in_direction = norm_(ld_v(in_ray->direction));
    rp_ray sp_ray = convert_to_sp(*in_ray, normal);
    sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
    E1_amp = cfp(sp_ray.E1_amp[0], 0) + (cfp(0, 1.0) * cfp(sp_ray.E1_amp[1], 0));
    E2_amp = cfp(sp_ray.E2_amp[0], 0) + (cfp(0, 1.0) * cfp(sp_ray.E2_amp[1], 0));
    cosTheta = dotprod_(normal, in_direction);
    cos1 = fabs(cosTheta);
    sin1 = sqrt(fabs(1 - cos1 * cos1));
    if (cosTheta < 0.0) {
        if (use_table) {
            n1 = mc->n_tab[m->curve_outside * mc->n_wl + in_ray->wavelength_idx];
            n2 = mc->n_tab[m->curve_inside * mc->n_wl + in_ray->wavelength_idx];
        } else {
            n1 = cfp(creal(n2_in), 0) + (cfp(0, 1.0) * cfp(cimag(n2_in), 0)); /* n_outside */
            n2 = cfp(creal(n1_in), 0) + (cfp(0, 1.0) * cfp(cimag(n1_in), 0)); /* n_inside */
        }
        flip = 1;
    } else {
        if (use_table) {
            n1 = mc->n_tab[m->curve_inside * mc->n_wl + in_ray->wavelength_idx];
            n2 = mc->n_tab[m->curve_outside * mc->n_wl + in_ray->wavelength_idx];
        } else {
            n1 = cfp(creal(n1_in), 0) + (cfp(0, 1.0) * cfp(cimag(n1_in), 0));
            n2 = cfp(creal(n2_in), 0) + (cfp(0, 1.0) * cfp(cimag(n2_in), 0));
        }
        flip = -1;
    }
    sin2 = (n1 * cfp(sin1, 0)) / n2;
    cos2 = csqrt(cfp(1, 0) - (sin2 * sin2));
    vec cosThetaNormal = multvs_(normal, cosTheta);
    P_in = creal(n1) * (((pow(creal(E1_amp), 2.0) + pow(cimag(E1_amp), 2.0)) + pow(creal(E2_amp), 2.0)) + pow(cimag(E2_amp), 2.0));
    if (P_in == 0.0) return;
    R_p = (-((n2 * cfp(cos1, 0)) - (n1 * cos2))) / ((n2 * cfp(cos1, 0)) + (n1 * cos2));
    R_s = (-((n2 * cos2) - (n1 * cfp(cos1, 0)))) / ((n2 * cos2) + (n1 * cfp(cos1, 0)));
    R_s = R_s * E1_amp;
    R_p = R_p * E2_amp;
    if (((creal(n1) * (pow(cabs(R_s), 2.0) + pow(cabs(R_p), 2.0))) / P_in) > m->reflection_threshold) {
        vec reflected = subvv_(in_direction, multvs_(cosThetaNormal, 2.0));
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, reflected);
        sp_ray.length = rp_inf();
        sp_ray.E1_amp[0] = creal(R_s); sp_ray.E1_amp[1] = cimag(R_s);
        sp_ray.E2_amp[0] = -creal(R_p); sp_ray.E2_amp[1] = -cimag(R_p);
        sp_ray.parent_idx = idx;
        sp_ray.refractive_index[0] = creal(n1); sp_ray.refractive_index[1] = cimag(n1);
        sp_ray.ray_type_id |= RP_REFL_RAY;
        add_ray(out, &sp_ray);
    }
    vec tangent = subvv_(in_direction, cosThetaNormal);
    vec tg2 = multvs_(tangent, creal(n1) / creal(n2));
    tan_mag_sq = mag_sq_(tg2);
    c2 = sqrt(1 - tan_mag_sq);
    vec transmitted = subvv_(tg2, multvs_(normal, (c2 * flip)));
    aspect = sqrt(creal(cos2) / cos1);
    T_p = (cfp(aspect, 0) * (cfp(2.0 * cos1, 0) * n1)) / ((n2 * cfp(cos1, 0)) + (n1 * cos2));
    T_s = (cfp(aspect, 0) * (cfp(2.0 * cos1, 0) * n1)) / ((n2 * cos2) + (n1 * cfp(cos1, 0)));
    T_s = T_s * E1_amp;
    T_p = T_p * E2_amp;
    if (((creal(n2) * (pow(cabs(T_s), 2.0) + pow(cabs(T_p), 2.0))) / P_in) > m->transmission_threshold) {
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, transmitted);
        sp_ray.length = rp_inf();
        sp_ray.E1_amp[0] = creal(T_s); sp_ray.E1_amp[1] = cimag(T_s);
        sp_ray.E2_amp[0] = creal(T_p); sp_ray.E2_amp[1] = cimag(T_p);
        sp_ray.parent_idx = idx;
        sp_ray.refractive_index[0] = creal(n2); sp_ray.refractive_index[1] = cimag(n2);
        sp_ray.ray_type_id &= ~RP_REFL_RAY;
        add_ray(out, &sp_ray);
    }
}

static inline cplx cplx_of_parts(double re, double im) { /* x.real + I*x.imag as Cython emits it */
    return cfp(re, 0) + (cfp(0, 1.0) * cfp(im, 0));
}

static void coated_split(const mat_ctx *mc, const rp_material *m, const rp_ray *in_ray, uint32_t idx, vec point,
                         orient_t orient, ray_sink *out) {
    /* SingleLayerCoatedMaterial.eval_child_ray_c (cmaterials.pyx:1026-1184) and
     * CoatedDispersiveMaterial.eval_child_ray_c (cmaterials.pyx:1228-1381) */
    cplx n1, n2, n3, cos2, sin2, cos3, sin3, R_p, R_s, T_p, T_s, E1_amp, E2_amp;
    cplx n1cos1, n2cos2, n3cos3, n1cos2, n2cos1, n2cos3, n3cos2, ep1, ep2, M00, M01, M10, M11, phi;
    double cosTheta, cos1, sin1, P_in, tan_mag_sq, c2, aspect, wavelength, dwc, thickness;
    int flip;
    const int disp = m->type == RP_MAT_COATED_DISPERSIVE;
    const uint32_t w = in_ray->wavelength_idx;
    wavelength = mc->wl[w];
    vec normal = norm_(orient.normal);
    vec in_direction = norm_(ld_v(in_ray->direction));
    rp_ray sp_ray = convert_to_sp(*in_ray, normal);
    sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
    E1_amp = cplx_of_parts(sp_ray.E1_amp[0], sp_ray.E1_amp[1]);
    E2_amp = cplx_of_parts(sp_ray.E2_amp[0], sp_ray.E2_amp[1]);
    cosTheta = dotprod_(normal, in_direction);
    cos1 = fabs(cosTheta);
    sin1 = sqrt(fabs((1.0 - (cos1 * cos1))));
    cplx ni, no;
    if (disp) {
        cplx ctemp = mc->n_tab[(int64_t)m->p[0] * mc->n_wl + w];
        n2 = cplx_of_parts(creal(ctemp), cimag(ctemp));
        ni = mc->n_tab[m->curve_inside * mc->n_wl + w];
        no = mc->n_tab[m->curve_outside * mc->n_wl + w];
        thickness = m->p[1];
    } else {
        n2 = cplx_of_parts(m->p[0], m->p[1]);
        ni = cfp(m->n_inside[0], m->n_inside[1]);
        no = cfp(m->n_outside[0], m->n_outside[1]);
        thickness = m->p[2];
    }
    if (cosTheta < 0.0) {
        n1 = cplx_of_parts(creal(no), cimag(no));
        n3 = cplx_of_parts(creal(ni), cimag(ni));
        flip = 1;
    } else {
        n1 = cplx_of_parts(creal(ni), cimag(ni));
        n3 = cplx_of_parts(creal(no), cimag(no));
        flip = -1;
    }
    sin2 = (n1 * cfp(sin1, 0)) / n2;
    cos2 = csqrt(cfp(1, 0) - (sin2 * sin2));
    sin3 = (n1 * cfp(sin1, 0)) / n3;
    cos3 = csqrt(cfp(1, 0) - (sin3 * sin3));
    vec cosThetaNormal = multvs_(normal, cosTheta);
    P_in = creal(n1) * (((pow(creal(E1_amp), 2.0) + pow(cimag(E1_amp), 2.0)) + pow(creal(E2_amp), 2.0)) +
                        pow(cimag(E2_amp), 2.0));
    if (P_in == 0.0) return;
    n1cos1 = n1 * cfp(cos1, 0);
    n2cos2 = n2 * cos2;
    n3cos3 = n3 * cos3;
    dwc = ((2.0 * M_PI) * thickness) / wavelength;
    phi = (((-cfp(0, 1.0)) * cfp(dwc, 0)) * (n2 - (sin2 * sin2))) / cos2;
    ep1 = cexp(phi) / ((cfp(4, 0) * n2cos2) * n3cos3);
    ep2 = cexp(cfp(-2L, 0) * phi);
    M00 = (-ep1) * (((n1cos1 - n2cos2) * (n2cos2 + n3cos3)) + (((n1cos1 + n2cos2) * (n2cos2 - n3cos3)) * ep2));
    M01 = ep1 * ((((n1cos1 - n2cos2) * (n2cos2 - n3cos3)) * ep2) + ((n1cos1 + n2cos2) * (n2cos2 + n3cos3)));
    M10 = ep1 * (((n1cos1 - n2cos2) * (n2cos2 - n3cos3)) + (((n1cos1 + n2cos2) * (n2cos2 + n3cos3)) * ep2));
    M11 = (-ep1) * ((((n1cos1 - n2cos2) * (n2cos2 + n3cos3)) * ep2) + ((n1cos1 + n2cos2) * (n2cos2 - n3cos3)));
    R_s = (-M00) / M01;
    T_s = M10 + (M11 * R_s);
    n1cos2 = n1 * cos2;
    n2cos1 = n2 * cfp(cos1, 0);
    n2cos3 = n2 * cos3;
    n3cos2 = n3 * cos2;
    M00 = (-ep1) * (((n1cos2 - n2cos1) * (n2cos3 + n3cos2)) + (((n1cos2 + n2cos1) * (n2cos3 - n3cos2)) * ep2));
    M01 = ep1 * ((((n1cos2 - n2cos1) * (n2cos3 - n3cos2)) * ep2) + ((n1cos2 + n2cos1) * (n2cos3 + n3cos2)));
    M10 = ep1 * (((n1cos2 - n2cos1) * (n2cos3 - n3cos2)) + (((n1cos2 + n2cos1) * (n2cos3 + n3cos2)) * ep2));
    M11 = (-ep1) * ((((n1cos2 - n2cos1) * (n2cos3 + n3cos2)) * ep2) + ((n1cos2 + n2cos1) * (n2cos3 - n3cos2)));
    R_p = (-M00) / M01;
    T_p = M10 + (M11 * R_p);
    R_s = R_s * E1_amp;
    R_p = R_p * E2_amp;
    if (((creal(n1) * (pow(cabs(R_s), 2.0) + pow(cabs(R_p), 2.0))) / P_in) > m->reflection_threshold) {
        vec reflected = subvv_(in_direction, multvs_(cosThetaNormal, 2.0));
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, reflected);
        sp_ray.length = rp_inf();
        sp_ray.E1_amp[0] = creal(R_s); sp_ray.E1_amp[1] = cimag(R_s);
        sp_ray.E2_amp[0] = -creal(R_p); sp_ray.E2_amp[1] = -cimag(R_p);
        sp_ray.parent_idx = idx;
        sp_ray.refractive_index[0] = creal(n1); sp_ray.refractive_index[1] = cimag(n1);
        sp_ray.ray_type_id |= RP_REFL_RAY;
        add_ray(out, &sp_ray);
    }
    vec tangent = subvv_(in_direction, cosThetaNormal);
    vec tg2 = multvs_(tangent, creal(n1) / creal(n3));
    tan_mag_sq = mag_sq_(tg2);
    c2 = sqrt(1 - tan_mag_sq);
    vec transmitted = subvv_(tg2, multvs_(normal, (c2 * flip)));
    aspect = sqrt(creal(cos3) / cos1);
    T_s = T_s * (E1_amp * cfp(aspect, 0));
    T_p = T_p * (E2_amp * cfp(aspect, 0));
    if (((creal(n3) * (pow(cabs(T_s), 2.0) + pow(cabs(T_p), 2.0))) / P_in) > m->transmission_threshold) {
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, transmitted);
        sp_ray.length = rp_inf();
        sp_ray.E1_amp[0] = creal(T_s); sp_ray.E1_amp[1] = cimag(T_s);
        sp_ray.E2_amp[0] = creal(T_p); sp_ray.E2_amp[1] = cimag(T_p);
        sp_ray.parent_idx = idx;
        sp_ray.refractive_index[0] = creal(n3); sp_ray.refractive_index[1] = cimag(n3);
        sp_ray.ray_type_id &= ~RP_REFL_RAY;
        add_ray(out, &sp_ray);
    }
}

static void eval_child_ray(const mat_ctx *mc, const rp_material *m, const rp_ray *in_ray, uint32_t idx,
                           vec point, orient_t orient, ray_sink *out) {
    switch (m->type) {
    case RP_MAT_NONE:   /* ctracer.pyx:1580-1586 */
    case RP_MAT_OPAQUE: /* cmaterials.pyx:245-251 */
        return;
    case RP_MAT_TRANSPARENT: { /* cmaterials.pyx:260-278 */
        vec normal = norm_(orient.normal);
        rp_ray sp_ray = convert_to_sp(*in_ray, normal);
        sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        sp_ray.length = rp_inf();
        sp_ray.parent_idx = idx;
        sp_ray.ray_type_id &= ~RP_REFL_RAY;
        add_ray(out, &sp_ray);
        return;
    }
    case RP_MAT_PEC: { /* cmaterials.pyx:285-319 */
        vec normal = norm_(orient.normal);
        rp_ray sp_ray = convert_to_sp(*in_ray, normal);
        vec dir = ld_v(in_ray->direction);
        double cosTheta = dotprod_(normal, dir);
        vec cosThetaNormal = multvs_(normal, cosTheta);
        vec reflected = subvv_(dir, multvs_(cosThetaNormal, 2));
        sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, reflected);
        sp_ray.length = rp_inf();
        sp_ray.E1_amp[0] = -sp_ray.E1_amp[0];
        sp_ray.E1_amp[1] = -sp_ray.E1_amp[1];
        sp_ray.parent_idx = idx;
        sp_ray.ray_type_id |= RP_REFL_RAY;
        add_ray(out, &sp_ray);
        return;
    }
    case RP_MAT_PARTIAL: { /* cmaterials.pyx:344-397 */
        vec normal = norm_(orient.normal);
        vec in_direction = norm_(ld_v(in_ray->direction));
        rp_ray sp_ray = convert_to_sp(*in_ray, normal), sp_ray2;
        sp_ray2 = sp_ray;
        double cosTheta = dotprod_(normal, in_direction);
        vec cosThetaNormal = multvs_(normal, cosTheta);
        sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
        sp_ray2.accumulated_path = sp_ray.accumulated_path;
        double R = sqrt(m->p[0]);
        double T = sqrt(1.0 - m->p[0]);
        vec reflected = subvv_(in_direction, multvs_(cosThetaNormal, 2.0));
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, reflected);
        sp_ray.length = rp_inf();
        st_c(sp_ray.E1_amp, ld_c(sp_ray.E1_amp) * cfp(R, 0));
        st_c(sp_ray.E2_amp, ld_c(sp_ray.E2_amp) * cfp(R, 0));
        sp_ray.parent_idx = idx;
        sp_ray.ray_type_id |= RP_REFL_RAY;
        add_ray(out, &sp_ray);
        st_v(sp_ray2.origin, point);
        st_v(sp_ray2.normal, normal);
        st_v(sp_ray2.direction, in_direction);
        sp_ray2.length = rp_inf();
        st_c(sp_ray2.E1_amp, ld_c(sp_ray2.E1_amp) * cfp(T, 0));
        st_c(sp_ray2.E2_amp, ld_c(sp_ray2.E2_amp) * cfp(T, 0));
        sp_ray2.parent_idx = idx;
        sp_ray2.ray_type_id &= ~RP_REFL_RAY;
        add_ray(out, &sp_ray2);
        return;
    }
    case RP_MAT_LINEAR_POLARISING: { /* cmaterials.pyx:404-455 */
        vec normal = norm_(orient.normal);
        vec in_direction = norm_(ld_v(in_ray->direction));
        rp_ray sp_ray = convert_to_sp(*in_ray, normal), sp_ray2;
        sp_ray2 = sp_ray;
        double cosTheta = dotprod_(normal, in_direction);
        vec cosThetaNormal = multvs_(normal, cosTheta);
        sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
        sp_ray2.accumulated_path = sp_ray.accumulated_path;
        vec reflected = subvv_(in_direction, multvs_(cosThetaNormal, 2.0));
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, reflected);
        sp_ray.length = rp_inf();
        sp_ray.E2_amp[0] = 0.0; sp_ray.E2_amp[1] = 0.0;
        sp_ray.parent_idx = idx;
        sp_ray.ray_type_id |= RP_REFL_RAY;
        add_ray(out, &sp_ray);
        st_v(sp_ray2.origin, point);
        st_v(sp_ray2.normal, normal);
        st_v(sp_ray2.direction, in_direction);
        sp_ray2.length = rp_inf();
        sp_ray2.E1_amp[0] = 0.0; sp_ray2.E1_amp[1] = 0.0;
        sp_ray2.parent_idx = idx;
        sp_ray2.ray_type_id &= ~RP_REFL_RAY;
        add_ray(out, &sp_ray2);
        return;
    }
    case RP_MAT_WAVEPLATE: { /* cmaterials.pyx:527-551; p: retardance re, im, fast axis */
        vec normal = norm_(orient.normal);
        vec in_direction = norm_(ld_v(in_ray->direction));
        rp_ray out_ray = convert_to_sp(*in_ray, ld_v(&m->p[2]));
        out_ray.accumulated_path = out_ray.accumulated_path + (out_ray.length * out_ray.refractive_index[0]);
        st_v(out_ray.origin, point);
        st_v(out_ray.normal, normal);
        st_v(out_ray.direction, in_direction);
        out_ray.length = rp_inf();
        out_ray.parent_idx = idx;
        out_ray.ray_type_id &= ~RP_REFL_RAY;
        /* apply_retardance_c, cmaterials.pyx:496-503 */
        double E1r = out_ray.E1_amp[0], E1i = out_ray.E1_amp[1];
        out_ray.E1_amp[0] = (E1r * m->p[0]) - (E1i * m->p[1]);
        out_ray.E1_amp[1] = (E1i * m->p[0]) + (E1r * m->p[1]);
        add_ray(out, &out_ray);
        return;
    }
    case RP_MAT_DIELECTRIC: { /* cmaterials.pyx:589-680 */
        vec normal = norm_(orient.normal);
        vec in_direction = norm_(ld_v(in_ray->direction));
        rp_ray sp_ray = convert_to_sp(*in_ray, normal);
        double n1, n2, flip;
        sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
        double cosTheta = dotprod_(normal, in_direction);
        double cos1 = fabs(cosTheta);
        if (cosTheta < 0.0) {
            n1 = m->n_outside[0]; n2 = m->n_inside[0];
            sp_ray.refractive_index[0] = m->n_inside[0]; sp_ray.refractive_index[1] = m->n_inside[1];
            flip = 1;
        } else {
            n1 = m->n_inside[0]; n2 = m->n_outside[0];
            sp_ray.refractive_index[0] = m->n_outside[0]; sp_ray.refractive_index[1] = m->n_outside[1];
            flip = -1;
        }
        double N2 = pow((n2 / n1), 2.0);
        double N2_sin2 = ((cosTheta * cosTheta) + (N2 - 1.0));
        vec cosThetaNormal = multvs_(normal, cosTheta);
        if (N2_sin2 < 0.0) {
            vec reflected = subvv_(in_direction, multvs_(cosThetaNormal, 2));
            st_v(sp_ray.origin, point);
            st_v(sp_ray.normal, normal);
            st_v(sp_ray.direction, reflected);
            sp_ray.length = rp_inf();
            sp_ray.E1_amp[0] *= -1; sp_ray.E1_amp[1] *= -1;
            sp_ray.E2_amp[0] *= -1; sp_ray.E2_amp[1] *= -1;
            sp_ray.parent_idx = idx;
            sp_ray.ray_type_id |= RP_REFL_RAY;
        } else {
            vec tangent = subvv_(in_direction, cosThetaNormal);
            vec tg2 = multvs_(tangent, (n1 / n2));
            double tan_mag_sq = mag_sq_(tg2);
            double c2 = sqrt((1.0 - tan_mag_sq));
            vec transmitted = subvv_(tg2, multvs_(normal, (c2 * flip)));
            double cos2 = fabs(dotprod_(transmitted, normal));
            double Two_n1_cos1 = (2 * n1) * cos1;
            double aspect = (sqrt((cos2 / cos1)) * Two_n1_cos1);
            double T_p = (aspect / ((n2 * cos1) + (n1 * cos2)));
            double T_s = (aspect / ((n2 * cos2) + (n1 * cos1)));
            st_v(sp_ray.origin, point);
            st_v(sp_ray.normal, normal);
            st_v(sp_ray.direction, transmitted);
            sp_ray.length = rp_inf();
            sp_ray.E1_amp[0] *= T_s; sp_ray.E1_amp[1] *= T_s;
            sp_ray.E2_amp[0] *= T_p; sp_ray.E2_amp[1] *= T_p;
            sp_ray.parent_idx = idx;
            sp_ray.ray_type_id &= ~RP_REFL_RAY;
        }
        add_ray(out, &sp_ray);
        return;
    }
    case RP_MAT_FULL_DIELECTRIC:
        fresnel_split(mc, m, ld_c(m->n_inside), ld_c(m->n_outside), 0, in_ray, idx, point, orient, out);
        return;
    case RP_MAT_FULL_DIELECTRIC_DISPERSIVE:
        fresnel_split(mc, m, 0, 0, 1, in_ray, idx, point, orient, out);
        return;
    case RP_MAT_SINGLE_LAYER_COATED:
    case RP_MAT_COATED_DISPERSIVE:
        coated_split(mc, m, in_ray, idx, point, orient, out);
        return;
    case RP_MAT_DIFFRACTION_GRATING: { /* cmaterials.pyx:1474-1543; p: lines_per_mm, order, efficiency, origin */
        vec normal = norm_(orient.normal);
        vec tangent = norm_(orient.tangent);
        vec tangent2 = cross_(normal, tangent);
        double wavelen = mc->wl[in_ray->wavelength_idx];
        double line_spacing = (1000.0 / m->p[0]);
        vec reflected = norm_(ld_v(in_ray->direction));
        double k_z = dotprod_(normal, reflected);
        double k_y = dotprod_(tangent2, reflected);
        double k_x = dotprod_(tangent, reflected);
        int sign = (k_z < 0.0) ? 1 : -1;
        int order = (int)m->p[1];
        k_x = (k_x - ((order * wavelen) / (line_spacing * in_ray->refractive_index[0])));
        k_z = ((1.0 - (k_x * k_x)) - (k_y * k_y));
        if (k_z < 0) return;
        k_z = (sign * sqrt(k_z));
        reflected = multvs_(tangent, k_x);
        reflected = addvv_(reflected, multvs_(tangent2, k_y));
        reflected = addvv_(reflected, multvs_(normal, k_z));
        rp_ray sp_ray = convert_to_sp(*in_ray, normal);
        sp_ray.accumulated_path = (sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]));
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        st_v(sp_ray.direction, reflected);
        double eff = m->p[2];
        sp_ray.E1_amp[0] = ((-sp_ray.E1_amp[0]) * eff);
        sp_ray.E1_amp[1] = ((-sp_ray.E1_amp[1]) * eff);
        sp_ray.E2_amp[0] = (sp_ray.E2_amp[0] * eff);
        sp_ray.E2_amp[1] = (sp_ray.E2_amp[1] * eff);
        sp_ray.parent_idx = idx;
        sp_ray.ray_type_id |= RP_REFL_RAY;
        sp_ray.phase = (sp_ray.phase + (((((1000.0 * dotprod_(subvv_(ld_v(&m->p[3]), point), tangent)) * order) *
                                          2.0) * M_PI) / line_spacing));
        add_ray(out, &sp_ray);
        return;
    }
    case RP_MAT_CIRCULAR_APERTURE: { /* cmaterials.pyx:1639-1662; p: outer_radius, radius, edge_width, invert, origin */
        vec origin = ld_v(&m->p[4]);
        double width = m->p[2];
        double r = sqrt(mag_sq_(subvv_(origin, point)));
        if (r > m->p[0]) return;
        double atten = (0.5 + (0.5 * erf(((m->p[1] - r) / width))));
        if (m->p[3] != 0.0) atten = (1.0 - atten);
        vec normal = norm_(orient.normal);
        rp_ray sp_ray = convert_to_sp(*in_ray, normal);
        sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        sp_ray.parent_idx = idx;
        sp_ray.ray_type_id &= ~RP_REFL_RAY;
        sp_ray.E1_amp[0] *= atten; sp_ray.E1_amp[1] *= atten;
        sp_ray.E2_amp[0] *= atten; sp_ray.E2_amp[1] *= atten;
        add_ray(out, &sp_ray);
        return;
    }
    case RP_MAT_RECT_APERTURE: { /* cmaterials.pyx:1719-1763; p: outer_w, outer_h, w, h, edge, invert, origin */
        vec origin = ld_v(&m->p[6]);
        double width = m->p[4];
        double x = m->p[2] / 2.;
        double y = m->p[3] / 2.;
        vec pp = subvv_(point, origin);
        double px = dotprod_(pp, orient.tangent);
        double py = dotprod_(pp, cross_(orient.normal, orient.tangent));
        if (fabs(px) > m->p[0] / 2.) return;
        if (fabs(py) > m->p[1] / 2.) return;
        double atten = (0.5 - (0.5 * erf(((px - x) / width))));
        atten = (atten * (0.5 - (0.5 * erf(((-(px + x)) / width)))));
        atten = (atten * (0.5 - (0.5 * erf(((py - y) / width)))));
        atten = (atten * (0.5 - (0.5 * erf(((-(py + y)) / width)))));
        if (m->p[5] != 0.0) atten = (1.0 - atten);
        vec normal = norm_(orient.normal);
        rp_ray sp_ray = convert_to_sp(*in_ray, normal);
        sp_ray.accumulated_path = sp_ray.accumulated_path + (sp_ray.length * sp_ray.refractive_index[0]);
        st_v(sp_ray.origin, point);
        st_v(sp_ray.normal, normal);
        sp_ray.parent_idx = idx;
        sp_ray.ray_type_id &= ~RP_REFL_RAY;
        sp_ray.E1_amp[0] *= atten; sp_ray.E1_amp[1] *= atten;
        sp_ray.E2_amp[0] *= atten; sp_ray.E2_amp[1] *= atten;
        add_ray(out, &sp_ray);
        return;
    }
    default:
        return;
    }
}

/* ---- dispersion curves: cmaterials.pyx:107-239 --------------------------- */
static double curve_eval(const rp_scene_desc *s, const rp_dispersion *c, double wavelen) {
    const double *coefs = s->aux + c->aux;
    int n_coefs = c->n_coefs;
    switch (c->formula_id) {
    case 0: return coefs[0]; /* nondispersive_0, 107-108 */
    case 1: { /* sellmeier_1, 110-119 */
        double n2 = 1.0, wl2 = wavelen * wavelen;
        n2 += coefs[0];
        for (int i = 0; i < (n_coefs - 1) / 2; i++)
            n2 += coefs[2 * i + 1] * wl2 / (wl2 - pow(coefs[2 * i + 2], 2.0));
        return sqrt(n2);
    }
    case 2: { /* sellmeier_2, 121-130 */
        double n2 = 1.0, wl2 = wavelen * wavelen;
        n2 += coefs[0];
        for (int i = 0; i < (n_coefs - 1) / 2; i++)
            n2 += coefs[2 * i + 1] * wl2 / (wl2 - coefs[2 * i + 2]);
        return sqrt(n2);
    }
    case 3: { /* sellmeier_3, 133-140 */
        double n2 = coefs[0];
        for (int i = 1; i < n_coefs - 1; i += 2) n2 += coefs[i] * (pow(wavelen, coefs[i + 1]));
        return sqrt(n2);
    }
    default: return NAN;
    }
}

/* c_evaluate_n, cmaterials.pyx:206-228.  Returns 0, or -1 when a wavelength is
 * outside the curve's range (the reference raises ValueError). */
static int build_n_tables(const rp_scene_desc *s, const double *wl, int64_t n_wl, cplx **out) {
    *out = NULL;
    if (s->n_dispersions == 0 || n_wl == 0) return 0;
    cplx *tab = (cplx *)malloc(sizeof(cplx) * (size_t)s->n_dispersions * (size_t)n_wl);
    if (!tab) return -2;
    for (int c = 0; c < s->n_dispersions; c++) {
        const rp_dispersion *d = &s->dispersions[c];
        double n_imag = 0.0001 * d->absorption / (4 * M_PI);
        for (int64_t i = 0; i < n_wl; i++) {
            double wvl = wl[i];
            if ((wvl < d->wavelength_min) || (wvl > d->wavelength_max)) { free(tab); return -1; }
            double re = curve_eval(s, d, wvl);
            double im = n_imag * wvl;
            double parts[2] = {re, im};
            tab[c * n_wl + i] = ld_c(parts);
        }
    }
    *out = tab;
    return 0;
}

/* ---- FaceList / trace: ctracer.pyx ------------------------------------ */
static isect_t facelist_intersect(const rp_scene_desc *s, const rp_facelist *fl, rp_ray *ray, vec ray_end,
                                  int only_face) {
    /* FaceList.intersect_c (ctracer.pyx:1882-1904) and intersect_one_face_c (1861-1879) */
    vec p1 = transform_c(&fl->inv_trans, ld_v(ray->origin));
    vec p2 = transform_c(&fl->inv_trans, ray_end);
    isect_t out;
    out.face_idx = -1;
    out.dist = 0; out.piece_idx = 0;
    for (int i = 0; i < fl->n_faces; i++) {
        if (only_face >= 0 && i != only_face) continue;
        const rp_face *face = &s->faces[fl->first_face + i];
        isect_t th = face_intersect(s, face, p1, p2, 1);
        if (face->tolerance < th.dist && th.dist < ray->length) {
            ray->length = th.dist;
            th.face_idx = face->idx;
            out = th;
            ray->end_face_idx = (uint32_t)face->idx;
        }
    }
    return out;
}

static orient_t compute_orientation(const rp_scene_desc *s, const rp_facelist *fl, const rp_face *face,
                                    vec point, const isect_t *it) {
    /* FaceList.compute_orientation_c, ctracer.pyx:1939-1953 */
    orient_t o;
    point = transform_c(&fl->inv_trans, point);
    o.normal = face_normal(s, face, point, it->piece_idx);
    o.tangent = face_tangent(face);
    if (face->invert_normal) {
        o.normal = invert_(o.normal);
        o.tangent = invert_(o.tangent);
    }
    o.normal = rotate_c(&fl->trans, o.normal);
    o.tangent = rotate_c(&fl->trans, o.tangent);
    return o;
}

static int find_face_record(const rp_scene_desc *s, int idx) {
    /* all_faces[idx]: the face whose Face.idx is idx (core/tracer.py:28-30) */
    for (int k = 0; k < s->n_faces; k++) if (s->faces[k].idx == idx) return k;
    return -1;
}

static int owning_list(const rp_scene_desc *s, int rec) {
    for (int l = 0; l < s->n_lists; l++)
        if (rec >= s->lists[l].first_face && rec < s->lists[l].first_face + s->lists[l].n_faces) return l;
    return -1;
}

static double ray_e2(const rp_ray *r) {
    return r->E1_amp[0] * r->E1_amp[0] + r->E1_amp[1] * r->E1_amp[1]
         + r->E2_amp[0] * r->E2_amp[0] + r->E2_amp[1] * r->E2_amp[1];
}

/* trace_segment_c (ctracer.pyx:2062-2118); one_list/one_face select
 * trace_one_face_segment_c (2121-2170).  Children beyond out_cap set *overflow. */
static int trace_generation(const rp_scene_desc *s, const mat_ctx *mc, rp_ray *rays, uint64_t n_rays,
                            float max_length, int one_list, int one_face, double e2_terminate,
                            rp_ray *out, uint64_t out_cap, uint64_t *n_out, uint32_t *face_counts) {
    ray_sink sink = {out, 0, out_cap, 0};
    int nearest_set = -1;
    isect_t nearest_it = {0, -1, 0};
    for (uint64_t i = 0; i < n_rays; i++) {
        rp_ray *ray = rays + i;
        ray->length = max_length;
        ray->end_face_idx = (uint32_t)-1;
        int nearest_idx = -1;
        vec point = addvv_(ld_v(ray->origin), multvs_(ld_v(ray->direction), max_length));
        if (one_list >= 0) {
            isect_t it = facelist_intersect(s, &s->lists[one_list], ray, point, one_face);
            if (it.face_idx >= 0) { nearest_set = one_list; nearest_it = it; nearest_idx = it.face_idx; }
        } else {
            for (int j = 0; j < s->n_lists; j++) {
                isect_t it = facelist_intersect(s, &s->lists[j], ray, point, -1);
                if (it.face_idx >= 0) { nearest_set = j; nearest_it = it; nearest_idx = it.face_idx; }
            }
        }
        if (nearest_idx >= 0) {
            int rec = find_face_record(s, nearest_idx);
            if (rec < 0) return -1;
            const rp_face *face = &s->faces[rec];
            if (face_counts) face_counts[rec] += 1;
            point = addvv_(ld_v(ray->origin), multvs_(ld_v(ray->direction), ray->length));
            orient_t orient = compute_orientation(s, &s->lists[nearest_set], face, point, &nearest_it);
            uint64_t before = sink.n;
            if (face->material >= 0)
                eval_child_ray(mc, &s->materials[face->material], ray, (uint32_t)i, point, orient, &sink);
            if (e2_terminate > 0) {
                /* |E|^2 termination between generations, applied as a stable
                 * filter on this ray's children (new; not in the reference). */
                uint64_t w = before;
                for (uint64_t k = before; k < sink.n; k++)
                    if (!(ray_e2(&sink.rays[k]) < e2_terminate)) sink.rays[w++] = sink.rays[k];
                sink.n = w;
            }
        }
    }
    *n_out = sink.n;
    return sink.overflow ? -2 : 0;
}

/* ---- Gausslets: ctracer.pyx:2214-2385 ------------------------------------ */
/* InterfaceMaterial.eval_parabasal_ray_c and its overrides:
 * ctracer.pyx:1588-1610 (base), cmaterials.pyx:683-724 (DielectricMaterial, and
 * so FullDielectric and SingleLayerCoated), 1393-1433 (CoatedDispersive),
 * 1544-1600 (DiffractionGrating). */
static rp_para eval_parabasal_ray(const mat_ctx *mc, const rp_material *m, const rp_ray *base_ray, vec direction,
                                  vec point, orient_t orient, uint32_t ray_type_id) {
    rp_para para_out;
    vec normal = norm_(orient.normal), out_dir;
    switch (m->type) {
    case RP_MAT_DIELECTRIC:
    case RP_MAT_FULL_DIELECTRIC:
    case RP_MAT_SINGLE_LAYER_COATED:
    case RP_MAT_COATED_DISPERSIVE: {
        double cosTheta, n1, n2, n_in, n_out;
        int flip;
        if (m->type == RP_MAT_COATED_DISPERSIVE) {
            n_in = creal(mc->n_tab[(int64_t)m->curve_inside * mc->n_wl + base_ray->wavelength_idx]);
            n_out = creal(mc->n_tab[(int64_t)m->curve_outside * mc->n_wl + base_ray->wavelength_idx]);
        } else {
            n_in = m->n_inside[0];
            n_out = m->n_outside[0];
        }
        direction = norm_(direction);
        cosTheta = dotprod_(normal, direction);
        vec cosThetaNormal = multvs_(normal, cosTheta);
        if (cosTheta < 0.0) { n1 = n_out; n2 = n_in; flip = 1; }
        else { n1 = n_in; n2 = n_out; flip = -1; }
        if (ray_type_id & RP_REFL_RAY) {
            out_dir = subvv_(direction, multvs_(cosThetaNormal, 2));
        } else {
            vec tangent = subvv_(direction, cosThetaNormal);
            vec tg2 = multvs_(tangent, n1 / n2);
            double tan_mag_sq = mag_sq_(tg2);
            double c2 = sqrt(1 - tan_mag_sq);
            out_dir = subvv_(tg2, multvs_(normal, c2 * flip));
        }
        break;
    }
    case RP_MAT_DIFFRACTION_GRATING: {
        vec tangent = norm_(orient.tangent), tangent2 = cross_(normal, tangent), reflected;
        double wavelen = mc->wl[base_ray->wavelength_idx];
        double line_spacing = 1000.0 / m->p[0];
        double k_x, k_y, k_z;
        int sign;
        reflected = norm_(direction);
        k_z = dotprod_(normal, reflected);
        k_y = dotprod_(tangent2, reflected);
        k_x = dotprod_(tangent, reflected);
        sign = k_z < 0.0 ? 1 : -1;
        k_x = k_x - (int)m->p[1] * wavelen / (line_spacing * base_ray->refractive_index[0]);
        k_z = 1 - (k_x * k_x) - (k_y * k_y);
        k_z = sign * sqrt(k_z);
        reflected = multvs_(tangent, k_x);
        reflected = addvv_(reflected, multvs_(tangent2, k_y));
        reflected = addvv_(reflected, multvs_(normal, k_z));
        out_dir = reflected;
        break;
    }
    default:
        if (ray_type_id & RP_REFL_RAY) {
            double cosTheta = dotprod_(normal, direction);
            vec cosThetaNormal = multvs_(normal, cosTheta);
            out_dir = subvv_(direction, multvs_(cosThetaNormal, 2));
        } else {
            out_dir = direction;
        }
        break;
    }
    st_v(para_out.direction, out_dir);
    st_v(para_out.origin, point);
    st_v(para_out.normal, normal);
    para_out.length = rp_inf();
    return para_out;
}

typedef struct {
    rp_gausslet *g;
    uint64_t n, cap;
    int overflow;
} gausslet_sink;

/* trace_parabasal_rays, ctracer.pyx:2353-2385 */
static void trace_parabasal_rays(const rp_scene_desc *s, const mat_ctx *mc, rp_gausslet *g_in, const rp_ray *base_rays,
                                 uint64_t n_base, const rp_face *face, const rp_facelist *fl, gausslet_sink *out,
                                 double max_length) {
    vec point[6];
    orient_t orient[6];
    for (int j = 0; j < 6; j++) {
        rp_para *para_ray = &g_in->para[j];
        vec ray_end = addvv_(ld_v(para_ray->origin), multvs_(ld_v(para_ray->direction), max_length));
        /* FaceList.intersect_para_c, ctracer.pyx:1914-1926 */
        vec p1 = transform_c(&fl->inv_trans, ld_v(para_ray->origin));
        vec p2 = transform_c(&fl->inv_trans, ray_end);
        isect_t it_para = face_intersect(s, face, p1, p2, 0);
        if (face->tolerance < it_para.dist && it_para.dist < para_ray->length) {
            para_ray->length = it_para.dist;
            it_para.face_idx = face->idx;
        }
        if (it_para.face_idx < 0) return;
        point[j] = addvv_(ld_v(para_ray->origin), multvs_(ld_v(para_ray->direction), para_ray->length));
        orient[j] = compute_orientation(s, fl, face, point[j], &it_para);
    }
    const rp_material *m = &s->materials[face->material];
    for (uint64_t i = 0; i < n_base; i++) {
        rp_gausslet gausslet;
        gausslet.base_ray = base_rays[i];
        for (int j = 0; j < 6; j++)
            gausslet.para[j] = eval_parabasal_ray(mc, m, &base_rays[i], ld_v(g_in->para[j].direction), point[j],
                                                  orient[j], gausslet.base_ray.ray_type_id);
        if (out->n >= out->cap) { out->overflow = 1; return; }
        out->g[out->n++] = gausslet;
    }
}

/* trace_gausslet_c (ctracer.pyx:2214-2282); one_list/one_face select
 * trace_one_face_gausslet_c (2285-2350).  captured[i] = 1 + material index of
 * a ResampleGaussletMaterial that captured gausslet i (its
 * eval_child_ray_c, cmaterials.pyx:1806-1818); the decomposition itself and
 * the final reset_length_c are left to the caller. */
static int trace_gausslet_generation(const rp_scene_desc *s, const mat_ctx *mc, rp_gausslet *gausslets, uint64_t n,
                                     double max_length, int one_list, int one_face, gausslet_sink *out,
                                     uint32_t *face_counts, int32_t *captured) {
    int nearest_set = -1;
    isect_t nearest_it = {0, -1, 0};
    for (uint64_t i = 0; i < n; i++) {
        rp_gausslet *gausslet = gausslets + i;
        rp_ray *ray = &gausslet->base_ray;
        if (captured) captured[i] = 0;
        ray->end_face_idx = (uint32_t)-1;
        int nearest_idx = -1;
        vec point = addvv_(ld_v(ray->origin), multvs_(ld_v(ray->direction), max_length));
        if (one_list >= 0) {
            isect_t it = facelist_intersect(s, &s->lists[one_list], ray, point, one_face);
            if (it.face_idx >= 0) { nearest_set = one_list; nearest_it = it; nearest_idx = it.face_idx; }
        } else {
            for (int j = 0; j < s->n_lists; j++) {
                isect_t it = facelist_intersect(s, &s->lists[j], ray, point, -1);
                if (it.face_idx >= 0) { nearest_set = j; nearest_it = it; nearest_idx = it.face_idx; }
            }
        }
        if (nearest_idx >= 0) {
            int rec = find_face_record(s, nearest_idx);
            if (rec < 0) return -1;
            const rp_face *face = &s->faces[rec];
            if (face_counts) face_counts[rec] += 1;
            point = addvv_(ld_v(ray->origin), multvs_(ld_v(ray->direction), ray->length));
            const rp_facelist *fl = &s->lists[nearest_set];
            orient_t orient = compute_orientation(s, fl, face, point, &nearest_it);
            rp_ray kids[2];
            ray_sink child_rays = {kids, 0, 2, 0};
            const rp_material *m = &s->materials[face->material];
            if (m->type == RP_MAT_RESAMPLE_GAUSSLET) {
                if ((ray->ray_type_id & RP_GAUSSLET_RAY) && captured) captured[i] = face->material + 1;
            } else {
                eval_child_ray(mc, m, ray, (uint32_t)i, point, orient, &child_rays);
            }
            trace_parabasal_rays(s, mc, gausslet, kids, child_rays.n, face, fl, out, max_length);
        }
    }
    return out->overflow ? -2 : 0;
}

/* ---- exported oracle API ------------------------------------------------ */
int rp_oracle_version(void) { return RP_ABI_VERSION; }

int rp_oracle_trace_segment(const rp_scene_desc *s, const double *wl, int64_t n_wl, rp_ray *rays, uint64_t n,
                            float max_length, int one_list, int one_face, double e2_terminate,
                            rp_ray *out, uint64_t out_cap, uint64_t *n_out, uint32_t *face_counts) {
    mat_ctx mc = {s, NULL, n_wl, wl};
    cplx *tab = NULL;
    int rc = build_n_tables(s, wl, n_wl, &tab);
    if (rc) return rc;
    mc.n_tab = tab;
    rc = trace_generation(s, &mc, rays, n, max_length, one_list, one_face, e2_terminate, out, out_cap, n_out,
                          face_counts);
    free(tab);
    return rc;
}

/* trace_rays, core/tracer.py:9-47: generations concatenated into `out`,
 * gen_offsets[g] = start of generation g, gen_offsets[n_gens] = total. */
int rp_oracle_trace_rays(const rp_scene_desc *s, const double *wl, int64_t n_wl, const rp_ray *in, uint64_t n,
                         int recursion_limit, float max_length, double e2_terminate, rp_ray *out,
                         uint64_t out_cap, uint64_t *gen_offsets, int max_gens, int *n_gens,
                         uint32_t *face_counts) {
    mat_ctx mc = {s, NULL, n_wl, wl};
    cplx *tab = NULL;
    int rc = build_n_tables(s, wl, n_wl, &tab);
    if (rc) return rc;
    mc.n_tab = tab;
    if (n > out_cap) { free(tab); return -2; }
    memcpy(out, in, sizeof(rp_ray) * n);
    /* input_rays.reset_length(max_length): core/tracer.py:22 (double argument) */
    for (uint64_t i = 0; i < n; i++) out[i].length = (double)max_length;
    uint64_t start = 0, count = n;
    int g = 0;
    gen_offsets[0] = 0;
    while (count > 0 && g < recursion_limit) {
        if (g >= max_gens) { free(tab); return -2; }
        uint64_t n_new = 0;
        uint64_t next = start + count;
        rc = trace_generation(s, &mc, out + start, count, max_length, -1, -1, e2_terminate, out + next,
                              out_cap - next, &n_new, face_counts);
        if (rc) { free(tab); return rc; }
        g++;
        gen_offsets[g] = next;
        start = next;
        count = n_new;
    }
    *n_gens = g;
    free(tab);
    return 0;
}

/* ---- unit-level entry points (single plugin calls, for known-answer tests) */
double rp_oracle_face_intersect(const rp_scene_desc *s, int rec, const double *p1, const double *p2,
                                int is_base_ray) {
    isect_t it = face_intersect(s, &s->faces[rec], ld_v(p1), ld_v(p2), is_base_ray);
    return it.dist;
}

void rp_oracle_face_normal(const rp_scene_desc *s, int rec, const double *p, double *n) {
    st_v(n, face_normal(s, &s->faces[rec], ld_v(p), 0));
}

int rp_oracle_shape_inside(const rp_scene_desc *s, int prog, double x, double y) {
    return shape_inside(s, prog, x, y);
}

void rp_oracle_distortion(const rp_scene_desc *s, int d, double x, double y, double *out3, double *z) {
    st_v(out3, z_offset_and_gradient_c(s, &s->distortions[d], x, y));
    *z = z_offset_c(s, &s->distortions[d], x, y);
}

void rp_oracle_convert_to_sp(const rp_ray *in, const double *normal, rp_ray *out) {
    *out = convert_to_sp(*in, ld_v(normal));
}

int rp_oracle_eval_child_ray(const rp_scene_desc *s, const double *wl, int64_t n_wl, int mat, const rp_ray *in,
                             uint32_t idx, const double *point, const double *normal, const double *tangent,
                             rp_ray *out2) {
    mat_ctx mc = {s, NULL, n_wl, wl};
    cplx *tab = NULL;
    if (build_n_tables(s, wl, n_wl, &tab)) return -1;
    mc.n_tab = tab;
    ray_sink sink = {out2, 0, 2, 0};
    orient_t o = {ld_v(normal), ld_v(tangent)};
    eval_child_ray(&mc, &s->materials[mat], in, idx, ld_v(point), o, &sink);
    free(tab);
    return (int)sink.n;
}

int rp_oracle_dispersion_n(const rp_scene_desc *s, int curve, const double *wl, int64_t n, double *out_re_im) {
    for (int64_t i = 0; i < n; i++) {
        const rp_dispersion *d = &s->dispersions[curve];
        if ((wl[i] < d->wavelength_min) || (wl[i] > d->wavelength_max)) return -1;
        out_re_im[2 * i] = curve_eval(s, d, wl[i]);
        out_re_im[2 * i + 1] = 0.0001 * d->absorption / (4 * M_PI) * wl[i];
    }
    return 0;
}

int rp_oracle_owning_list(const rp_scene_desc *s, int rec) { return owning_list(s, rec); }

/* One Gausslet generation; see trace_gausslet_generation.  The children's
 * lengths are left as the materials wrote them (the caller appends any
 * decomposition output and then resets lengths, ctracer.pyx:2274-2281). */
int rp_oracle_trace_gausslet_segment(const rp_scene_desc *s, const double *wl, int64_t n_wl, rp_gausslet *g,
                                     uint64_t n, double max_length, int one_list, int one_face, rp_gausslet *out,
                                     uint64_t out_cap, uint64_t *n_out, uint32_t *face_counts, int32_t *captured) {
    mat_ctx mc = {s, NULL, n_wl, wl};
    cplx *tab = NULL;
    int rc = build_n_tables(s, wl, n_wl, &tab);
    if (rc) return rc;
    mc.n_tab = tab;
    gausslet_sink sink = {out, 0, out_cap, 0};
    rc = trace_gausslet_generation(s, &mc, g, n, max_length, one_list, one_face, &sink, face_counts, captured);
    *n_out = sink.n;
    free(tab);
    return rc;
}

/* InterfaceMaterial.eval_parabasal_ray (ctracer.pyx:1634-1644) of material `mat`. */
int rp_oracle_eval_parabasal(const rp_scene_desc *s, const double *wl, int64_t n_wl, int mat, const rp_ray *base,
                             const double *direction, const double *point, const double *normal,
                             const double *tangent, uint32_t ray_type, rp_para *out) {
    mat_ctx mc = {s, NULL, n_wl, wl};
    cplx *tab = NULL;
    if (build_n_tables(s, wl, n_wl, &tab)) return -1;
    mc.n_tab = tab;
    orient_t o = {ld_v(normal), ld_v(tangent)};
    *out = eval_parabasal_ray(&mc, &s->materials[mat], base, ld_v(direction), ld_v(point), o, ray_type);
    free(tab);
    return 0;
}

/* select_ray_intersections' per-collection loop (ctracer.pyx:1996-2008): a
 * copy of each ray is intersected with face list `list` from its origin to
 * origin + direction * length; the copies that meet a face are appended with
 * wavelength_idx + wl_offset. */
int rp_oracle_select_intersections(const rp_scene_desc *s, int list, const rp_ray *rays, uint64_t n,
                                   uint32_t wl_offset, rp_ray *out, uint64_t *n_out) {
    uint64_t k = 0;
    for (uint64_t i = 0; i < n; i++) {
        rp_ray ray = rays[i];
        vec point = addvv_(ld_v(ray.origin), multvs_(ld_v(ray.direction), ray.length));
        isect_t it = facelist_intersect(s, &s->lists[list], &ray, point, -1);
        if (it.face_idx >= 0) {
            ray.wavelength_idx += wl_offset;
            out[k++] = ray;
        }
    }
    *n_out = k;
    return 0;
}

/* ---- E-field summation: raypier/core/cfields.pyx -------------------------- */
/* evaluate_one_mode (cfields.pyx:150-222): closed-form least-squares fit of
 * the Gaussian mode coefficients to a gausslet's parabasal offsets (x, y) and
 * slopes (dx, dy).  Returns -1 where the reference raises ZeroDivisionError
 * (its divisions here are not cdivision). */
static int evaluate_one_mode(double complex *out, const double *x, const double *y, const double *dx,
                             const double *dy, double blending, int size) {
    double a00 = 0, a01 = 0, a02 = 0, a11 = 0, a12 = 0, a22 = 0, b0 = 0, b1 = 0, b2 = 0, xi2, yi2, num, den;
    double re[3], im[3];
    for (int i = 0; i < size; i++) {
        xi2 = x[i] * x[i];
        yi2 = y[i] * y[i];
        a00 = a00 + xi2 * xi2;
        a01 = a01 + ((2 * xi2) * x[i]) * y[i];
        a02 = a02 + xi2 * yi2;
        a11 = a11 + (4 * xi2) * yi2;
        a12 = a12 + ((2 * x[i]) * y[i]) * yi2;
        a22 = a22 + yi2 * yi2;
        b0 = b0 + xi2;
        b1 = b1 + (2 * x[i]) * y[i];
        b2 = b2 + yi2;
    }
    den = (((((-a00) * a11) * a22) + (a00 * pow(a12, 2.0))) + (pow(a01, 2.0) * a22)) - (((2.0 * a01) * a02) * a12)
          + (pow(a02, 2.0) * a11);
    if (den == 0) return -1;
    num = blending * ((((-b0) * ((a11 * a22) - pow(a12, 2.0))) + (b1 * ((a01 * a22) - (a02 * a12))))
                      - (b2 * ((a01 * a12) - (a02 * a11))));
    im[0] = num / den;
    num = (-blending) * (((b0 * ((a01 * a22) - (a02 * a12))) - (b1 * ((a00 * a22) - pow(a02, 2.0))))
                         + (b2 * ((a00 * a12) - (a01 * a02))));
    im[1] = num / den;
    num = blending * ((((-b0) * ((a01 * a12) - (a02 * a11))) + (b1 * ((a00 * a12) - (a01 * a02))))
                      - (b2 * ((a00 * a11) - pow(a01, 2.0))));
    im[2] = num / den;
    a00 = 0; a01 = 0; a02 = 0; a11 = 0; a12 = 0; a22 = 0; b0 = 0; b1 = 0; b2 = 0;
    for (int i = 0; i < size; i++) {
        xi2 = x[i] * x[i];
        yi2 = y[i] * y[i];
        a00 = a00 + xi2;
        a01 = a01 + x[i] * y[i];
        a11 = a11 + (xi2 + yi2);
        a22 = a22 + yi2;
        b0 = b0 + dx[i] * x[i];
        b1 = b1 + ((dx[i] * y[i]) + (dy[i] * x[i]));
        b2 = b2 + dy[i] * y[i];
    }
    a12 = a01 * a01;
    den = ((a00 * a12) - ((a00 * a11) * a22)) + (a12 * a22);
    if (den == 0) return -1;
    re[0] = ((((-a12) * b2) + ((a01 * a22) * b1)) + (b0 * (a12 - (a11 * a22)))) / den;
    re[1] = (-((((a00 * a01) * b2) - ((a00 * a22) * b1)) + ((a01 * a22) * b0))) / den;
    re[2] = ((((a00 * a01) * b1) - (a12 * b0)) - (b2 * ((a00 * a11) - a12))) / den;
    for (int k = 0; k < 3; k++) {
        __real__ out[k] = re[k];
        __imag__ out[k] = im[k];
    }
    return 0;
}

/* evaluate_modes (cfields.pyx:225-234): n rows of `size` parabasal samples;
 * modes[n][3] complex as (re, im) pairs.  Returns -1 on a zero denominator. */
int rp_oracle_evaluate_modes(const double *x, const double *y, const double *dx, const double *dy, int64_t n,
                             int size, double blending, double *modes) {
    for (int64_t i = 0; i < n; i++) {
        double complex m[3];
        if (evaluate_one_mode(m, x + i * size, y + i * size, dx + i * size, dy + i * size, blending, size))
            return -1;
        for (int k = 0; k < 3; k++) {
            modes[(i * 3 + k) * 2] = creal(m[k]);
            modes[(i * 3 + k) * 2 + 1] = cimag(m[k]);
        }
    }
    return 0;
}

/* calc_mode_U (cfields.pyx:120-147) */
static double complex calc_mode_U(double complex A, double complex B, double complex C, double complex detG0, vec pt,
                                  vec E, vec H, vec direction, double complex k, double phase,
                                  double inv_root_area, double complex rootI) {
    double x = dotprod_(pt, E), y = dotprod_(pt, H), z = dotprod_(pt, direction);
    double complex denom = (1 + (z * (A + C)) + (z * z) * detG0) * 2;
    double complex AA = (A + z * detG0) / denom;
    double complex CC = (C + z * detG0) / denom;
    double complex U = cexp(I * (phase + k * (z + AA * (x * x) + B * (2 * x * y) / denom + CC * (y * y))));
    U /= csqrt(((1 + z * A) * (1 + z * C) - (z * B) * (z * B)) * I);
    U *= inv_root_area * rootI;
    return U;
}

/* sum_gaussian_modes (cfields.pyx:49-117): E[n_points][3] complex as (re, im)
 * pairs, summed over the rays in order for every point. */
int rp_oracle_sum_gaussian_modes(const rp_ray *rays, int64_t n_rays, const double *modes, const double *wavelengths,
                                 const double *points, int64_t n_points, double time_ps, double *E_out) {
    const double complex rootI = csqrt(I);
    double c = 0.299792458;
    c *= time_ps;
    double complex *out = calloc((size_t)(n_points > 0 ? n_points : 1) * 3, sizeof(double complex));
    if (!out) return -1;
    for (int64_t iray = 0; iray < n_rays; iray++) {
        rp_ray ray = rays[iray];
        vec E = norm_(ld_v(ray.E_vector));
        vec D = ld_v(ray.direction);
        vec H = norm_(cross_(D, E));
        double k = 2000.0 * M_PI / wavelengths[ray.wavelength_idx];
        double phase = ray.phase + (ray.accumulated_path * k) - (c * k / ray.refractive_index[0]);
        double complex kz = ld_c(ray.refractive_index);
        kz *= k;
        double invk = 2. / creal(kz);
        double complex A = ld_c(modes + iray * 6 + 0);
        double complex B = ld_c(modes + iray * 6 + 2);
        double complex C = ld_c(modes + iray * 6 + 4);
        double inv_root_area = sqrt(sqrt(cimag(A) * cimag(C) - (cimag(B) * cimag(B))) * (2.0 / M_PI));
        __imag__ A = __imag__ A * invk;
        __imag__ B = __imag__ B * invk;
        __imag__ C = __imag__ C * invk;
        double complex detG0 = (A * C) - (B * B);
        double complex E1a = ld_c(ray.E1_amp), E2a = ld_c(ray.E2_amp);
        vec O = ld_v(ray.origin);
        for (int64_t ipt = 0; ipt < n_points; ipt++) {
            vec pt = {points[ipt * 3], points[ipt * 3 + 1], points[ipt * 3 + 2]};
            pt = subvv_(pt, O);
            double complex U = calc_mode_U(A, B, C, detG0, pt, E, H, D, kz, phase, inv_root_area, rootI);
            double complex E1 = E1a * U, E2 = E2a * U;
            out[ipt * 3 + 0] += (E1 * E.x + E2 * H.x);
            out[ipt * 3 + 1] += (E1 * E.y + E2 * H.y);
            out[ipt * 3 + 2] += (E1 * E.z + E2 * H.z);
        }
    }
    for (int64_t i = 0; i < n_points * 3; i++) {
        E_out[2 * i] = creal(out[i]);
        E_out[2 * i + 1] = cimag(out[i]);
    }
    free(out);
    return 0;
}

/* calc_mode_curvature (cfields.pyx:232-290): A, B, C and the local bases
 * x', y', z' (n x 3) from the slopes and second derivatives. */
void rp_oracle_mode_curvature(const double *dx, const double *dy, const double *dx2, const double *dy2,
                              const double *dxdy, int64_t n, double *A, double *B, double *C, double *X, double *Y,
                              double *Z) {
    for (int64_t i = 0; i < n; i++) {
        vec c = {-dx[i], -dy[i], 1.0};
        c = norm_(c);
        vec b = {0.0, 0.0, 1.0};
        vec a = norm_(cross_(b, c));
        b = cross_(c, a);
        st_v(X + 3 * i, a);
        st_v(Y + 3 * i, b);
        st_v(Z + 3 * i, c);
        double Fz = c.x * dx[i] + c.y * dy[i] + c.z;
        A[i] = -(a.x * a.x * dx2[i] + 2 * a.x * a.y * dxdy[i] + a.y * a.y * dy2[i]) / Fz;
        B[i] = -(a.x * b.x * dx2[i] + (a.x * b.y + b.x * a.y) * dxdy[i] + a.y * b.y * dy2[i]) / Fz;
        C[i] = -(b.x * b.x * dx2[i] + 2 * b.x * b.y * dxdy[i] + b.y * b.y * dy2[i]) / Fz;
    }
}

/* build_interaction_matrix (cfields.pyx:295-395): every (mode i, test point j)
 * pair within max_spacing, in loop order; returns the number of pairs and
 * writes the first `cap` of them (data as (re, im) pairs). */
int64_t rp_oracle_interaction_matrix(const double *rx, const double *ry, int64_t n, const double *tx,
                                     const double *ty, int64_t L, const double *A, const double *B, const double *C,
                                     const double *X, const double *Y, const double *Z, double wavelength,
                                     double spacing, double max_spacing, double blending, int64_t cap, double *data,
                                     uint64_t *row, uint64_t *col) {
    const double complex rootI = csqrt(I);
    double phase = 0.0, inv_root_area = 1.0;
    double k = 2000.0 * M_PI / wavelength;
    double impart = 2 * (blending * blending) / (k * spacing * spacing);
    int64_t ct = 0;
    for (int64_t i = 0; i < n; i++) {
        vec o = {rx[i], ry[i], 0.0};
        vec a = ld_v(X + 3 * i), b = ld_v(Y + 3 * i), c = ld_v(Z + 3 * i);
        double complex _A, _B, _C;
        __real__ _A = A[i];
        __real__ _B = B[i];
        __real__ _C = C[i];
        __imag__ _A = impart;
        __imag__ _B = 0;
        __imag__ _C = impart;
        double complex detG0 = (_A * _C);
        for (int64_t j = 0; j < L; j++) {
            vec pt = {tx[j], ty[j], 0.0};
            pt = subvv_(pt, o);
            if (((pt.x * pt.x) + (pt.y * pt.y)) <= (max_spacing * max_spacing)) {
                if (ct < cap) {
                    double complex U = calc_mode_U(_A, _B, _C, detG0, pt, a, b, c, k, phase, inv_root_area, rootI);
                    data[2 * ct] = creal(U);
                    data[2 * ct + 1] = cimag(U);
                    row[ct] = (uint64_t)i;
                    col[ct] = (uint64_t)j;
                }
                ct++;
            }
        }
    }
    return ct;
}

/* apply_mode_curvature (cfields.pyx:398-426) on gausslet records in place. */
void rp_oracle_apply_mode_curvature(rp_gausslet *g, int64_t n, const double *A, const double *B, const double *C) {
    for (int64_t i = 0; i < n; i++) {
        const rp_ray *ray = &g[i].base_ray;
        vec z = ld_v(ray->direction);
        vec x = ld_v(ray->E_vector);
        vec y = cross_(x, z);
        vec origin = ld_v(ray->origin);
        for (int j = 0; j < 6; j++) {
            rp_para *para = &g[i].para[j];
            vec r = subvv_(ld_v(para->origin), origin);
            double px = dotprod_(r, x);
            double py = dotprod_(r, y);
            vec shift = multvs_(x, (-A[i] * px - B[i] * py));
            shift = addvv_(shift, multvs_(y, (-C[i] * py - B[i] * px)));
            vec d = norm_(addvv_(shift, ld_v(para->direction)));
            st_v(para->direction, d);
        }
    }
}

/* ---- wavefront samples for the mode fit (core/fields.py:51-148) -------------
 * The reference forms these with numpy: a 3-term product sum over the last
 * axis adds x, y, z left to right and numpy.cross is the usual component
 * formula, so the C below reproduces it bit for bit. */

/* evaluate_neighbours_gc (core/fields.py:114-136): offsets and slopes of each
 * gausslet's six parabasal rays in the base ray's (E, E x d) frame. */
void rp_oracle_gausslet_samples(const rp_gausslet *g, int64_t n, double *x, double *y, double *dx, double *dy) {
    for (int64_t i = 0; i < n; i++) {
        const rp_ray *b = &g[i].base_ray;
        vec o = ld_v(b->origin), d = ld_v(b->direction), E = ld_v(b->E_vector);
        vec H = cross_(E, d);
        for (int j = 0; j < 6; j++) {
            vec u = subvv_(ld_v(g[i].para[j].origin), o);
            vec m = ld_v(g[i].para[j].direction);
            double md = dotprod_(m, d);
            x[i * 6 + j] = dotprod_(u, E);
            y[i * 6 + j] = dotprod_(u, H);
            dx[i * 6 + j] = dotprod_(m, E) / md;
            dy[i * 6 + j] = dotprod_(m, H) / md;
        }
    }
}

/* evaluate_neighbours (core/fields.py:80-111): for each ray whose six
 * neighbours all exist (kept[k] its index), the neighbours carried along
 * their directions to the ray's normal plane, then offsets and slopes in the
 * ray's (E, E x d) frame.  Returns the number of rows kept. */
int64_t rp_oracle_ray_samples(const rp_ray *r, int64_t n, const int32_t *nb, double *x, double *y, double *dx,
                              double *dy, int64_t *kept) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; i++) {
        int all = 1;
        for (int j = 0; j < 6; j++) all = all && nb[i * 6 + j] >= 0;
        if (!all) continue;
        vec o = ld_v(r[i].origin), d = ld_v(r[i].direction), E = ld_v(r[i].E_vector);
        vec H = cross_(E, d);
        for (int j = 0; j < 6; j++) {
            const rp_ray *q = &r[nb[i * 6 + j]];
            vec m = ld_v(q->direction);
            vec u = subvv_(ld_v(q->origin), o);
            double md = dotprod_(m, d);
            double s = -dotprod_(u, d) / md;
            u.x = u.x + s * m.x;
            u.y = u.y + s * m.y;
            u.z = u.z + s * m.z;
            x[k * 6 + j] = dotprod_(u, E);
            y[k * 6 + j] = dotprod_(u, H);
            dx[k * 6 + j] = dotprod_(m, E) / md;
            dy[k * 6 + j] = dotprod_(m, H) / md;
        }
        kept[k++] = i;
    }
    return k;
}

/* project_to_sphere (core/fields.py:51-77) in place: each ray that meets the
 * sphere moves to the smaller root of |o - c + a d|^2 = radius^2 and its
 * optical path by a Re(n); hit[i] = 0 for a ray that misses (unchanged). */
void rp_oracle_project_to_sphere(rp_ray *r, int64_t n, const double *c, double radius, uint8_t *hit) {
    for (int64_t i = 0; i < n; i++) {
        vec u = {r[i].origin[0] - c[0], r[i].origin[1] - c[1], r[i].origin[2] - c[2]};
        vec d = ld_v(r[i].direction);
        double cc = dotprod_(u, u) - radius * radius;
        double b = 2 * dotprod_(d, u);
        double disc = b * b - 4 * cc;
        if (!(disc >= 0.0)) {
            hit[i] = 0;
            continue;
        }
        double s = sqrt(disc);
        double r1 = (-b + s) / 2, r2 = (-b - s) / 2;
        double a = (r2 < r1 || r2 != r2) ? r2 : r1;
        r[i].origin[0] += a * d.x;
        r[i].origin[1] += a * d.y;
        r[i].origin[2] += a * d.z;
        r[i].accumulated_path += a * r[i].refractive_index[0];
        hit[i] = 1;
    }
}
