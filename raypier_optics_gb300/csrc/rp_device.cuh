// rp_device.cuh -- device-side faces, shapes, distortions and materials for the
// plain FP64 tracing path.  Each function states the reference code it
// follows (raypier/core/*.pyx); together they replace the Cython virtual
// calls Face.intersect_c / compute_normal_c, Shape.point_inside_c,
// Distortion.z_offset[_and_gradient]_c and InterfaceMaterial.eval_child_ray_c
// with a switch on the type tag of a table record (include/rp_gb300.h).
#pragma once
#include "../../include/rp_gb300.h"
#include "rp_math.cuh"

namespace rp {

// Scene tables as the kernels see them.  lists/faces/materials point into
// shared memory inside the generation kernel; the rest stays in global memory.
struct DevScene {
    const rp_facelist *lists;
    const rp_face *faces;
    const rp_material *mats;
    const rp_shape_op *shapes;
    const rp_distortion *dists;
    const double *aux;
    const double2 *ntab;  // [n_dispersions][n_wl] complex index per curve and wavelength
    const double *wl;     // [n_wl] the wavelengths (um)
    const float *bounds;  // [n_faces][16]: world box lo[3], hi[3], flag, -, and a second box (flag 3; rp_bounds.h)
    const short *face_list;  // [n_faces]: owning face list of each traced face
    const short *zk_prog;    // compiled Zernike programs (rp_zkprog.h), or null
    const int *zk_off;       // [n_dists][2]: offsets of the z and z-gradient programs in zk_prog, -1 for none
    const float *zk32;       // the mixed path's polynomial tables of the distortions (rp_zkprog.h, zkp), FP32
    const double *zk64;      // the same tables in FP64, at the same word offsets
    const int *zk32_off;     // [n_dists]: offset of a distortion's table in zk32 / zk64, -1 for none
    const float *ep32;       // the mixed path's FP32 copies of the ExtendedPolynomialFace coefficient matrices
    const int *ep32_off;     // [n_recs]: offset of a face record's matrix ([Nx, Ny, E...]) in ep32, -1 for none
    long long n_wl;
    int n_lists, n_faces, n_recs, n_mats, n_shapes, n_dists;
};

// error bits reported through the kernel's error word
enum : unsigned {
    ERR_TIMEOUT = 1u,
    ERR_ZK_STACK = 2u,
    ERR_SHAPE_STACK = 4u,
    ERR_OVERFLOW = 8u,
    ERR_WAVELENGTH = 16u,
};

// ---- shapes: cshapes.pyx --------------------------------------------------
__device__ __forceinline__ int poly_shape_inside(const double *xy, int n, double X, double Y) {
    // PolygonShape.point_inside_c, cshapes.pyx:147-168
    int ct = 0;
    if (n < 1) return 0;
    double y1 = xy[2 * (n - 1) + 1], x1 = xy[2 * (n - 1)];
    for (int i = 0; i < n; i++) {
        double y2 = xy[2 * i + 1], x2 = xy[2 * i];
        if ((y1 <= Y && Y < y2) || (y2 <= Y && Y < y1)) {
            if ((x1 + (Y - y1) * (x2 - x1) / (y2 - y1)) > X) ct = !ct;
        }
        y1 = y2;
        x1 = x2;
    }
    return ct;
}

static __device__ int shape_inside(const DevScene &S, int prog, double x, double y, unsigned *err) {
    if (prog < 0) return 1;  // base Shape: ctracer.pyx:1653-1655
    int stack[16];
    int sp = 0;
    for (int k = prog; k < S.n_shapes; k++) {
        const rp_shape_op &op = S.shapes[k];
        switch (op.op) {
            case RP_SHAPE_END: return sp > 0 ? stack[sp - 1] : 1;
            case RP_SHAPE_TRUE: stack[sp++] = 1; break;
            case RP_SHAPE_CIRCLE: {  // cshapes.pyx:109-116
                double dx = x - op.a, dy = y - op.b;
                stack[sp++] = ((dx * dx) + (dy * dy) < (op.c * op.c)) ? 1 : 0;
                break;
            }
            case RP_SHAPE_RECT: {  // cshapes.pyx:128-136
                double dx = x - op.a, dy = y - op.b;
                stack[sp++] = ((2 * fabs(dx) < op.c) && (2 * fabs(dy)) < op.d) ? 1 : 0;
                break;
            }
            case RP_SHAPE_POLYGON: stack[sp++] = poly_shape_inside(S.aux + op.aux, op.n, x, y); break;
            case RP_SHAPE_AND: if (sp < 2) goto bad; sp--; stack[sp - 1] &= stack[sp]; break;
            case RP_SHAPE_OR:  if (sp < 2) goto bad; sp--; stack[sp - 1] |= stack[sp]; break;
            case RP_SHAPE_XOR: if (sp < 2) goto bad; sp--; stack[sp - 1] ^= stack[sp]; break;
            case RP_SHAPE_NOT: if (sp < 1) goto bad; stack[sp - 1] = 1 & (~stack[sp - 1]); break;
            default: goto bad;
        }
        if (sp >= 15) goto bad;
    }
    return sp > 0 ? stack[sp - 1] : 1;
bad:
    atomicOr(err, ERR_SHAPE_STACK);
    return 0;
}

// ---- Zernike distortion: cdistortions.pyx ---------------------------------
// The reference evaluates the radial polynomials by recursion memoised in a
// per-thread workspace keyed by a slot index k (zernike_R_c 149-178,
// zernike_Rprime_c 189-219, zernike_R_over_r_c 288-316).  zernike_Rprime_c
// computes the slot of its third sub-call with a different formula (209) from
// the slot of the value it stands for, so a slot can be filled by one
// polynomial and read back for another: results depend on call order.  The
// machine below runs the same recursion with an explicit bounded stack, calls
// in the reference's order (left operand first), and the same slot keys.
#define RP_ZK_SLOTS 48
#define RP_ZK_DEPTH 24
#define RP_ZKOP_WORDS 7     // one operation of a compiled program (rp_zkprog.h)
#define RP_ZKPROG_SLOTS 96  // a compiled program's workspace (doubles; fits the recursion's)
struct ZkFrame {
    signed char fn, stage;
    short n, m, k;
    short nA, mA, kA, nB, mB, kB, nC, mC, kC;
    double acc, acc2;
};

static __device__ __noinline__ double zk_eval(int fn0, int k0, int n0, int m0, double r, double (*ws)[RP_ZK_SLOTS], unsigned *err) {
    ZkFrame st[RP_ZK_DEPTH];
    int sp = 0;
    double ret = 0.0;
    st[0].fn = (signed char)fn0;
    st[0].stage = 0;
    st[0].n = (short)n0;
    st[0].m = (short)m0;
    st[0].k = (short)k0;
    for (int guard = 0; guard < 100000; guard++) {
        ZkFrame &F = st[sp];
        int push = -1;  // fn of a child to push
        int cn = 0, cm = 0, ck = 0;
        if (F.stage == 0) {
            if (F.n < F.m) { ret = 0.0; goto pop; }
            if (F.fn == 0 && F.n == 0) { ret = 1.0; goto pop; }
            if (F.fn == 1 && F.n == 0) { ret = 0.0; goto pop; }
            if (F.k < 0 || F.k >= RP_ZK_SLOTS) { atomicOr(err, ERR_ZK_STACK); ret = 0.0; goto pop; }
            {
                double v = ws[F.fn][F.k];
                if (!isnan(v)) { ret = v; goto pop; }
            }
            {
                int nA = F.n - 1, mA = abs(F.m - 1), half_n = nA / 2;
                int kA = half_n * (half_n + 1) + abs(mA);
                int nB = nA, mB = F.m + 1;
                int kB = half_n * (half_n + 1) + abs(mB);
                int nC = F.n - 2, mC = F.m, kC;
                if (F.fn == 1) {
                    kC = (half_n - 1) * half_n + abs(mC);  // cdistortions.pyx:211
                } else {
                    half_n = nC / 2;
                    kC = half_n * (half_n + 1) + abs(mC);
                }
                F.nA = nA; F.mA = mA; F.kA = kA;
                F.nB = nB; F.mB = mB; F.kB = kB;
                F.nC = nC; F.mC = mC; F.kC = kC;
            }
            F.stage = 1;
            push = 0; cn = F.nA; cm = F.mA; ck = F.kA;  // every function starts with R(A)
        } else if (F.fn == 0) {  // zernike_R_c: val = r*(R(A)+R(B)) - R(C)
            if (F.stage == 1) { F.acc = ret; F.stage = 2; push = 0; cn = F.nB; cm = F.mB; ck = F.kB; }
            else if (F.stage == 2) { F.acc = r * (F.acc + ret); F.stage = 3; push = 0; cn = F.nC; cm = F.mC; ck = F.kC; }
            else { double val = F.acc - ret; ws[0][F.k] = val; ret = val; goto pop; }
        } else if (F.fn == 1) {  // zernike_Rprime_c: R(A)+R(B) + r*(R'(A)+R'(B)) - R'(C)
            if (F.stage == 1) { F.acc = ret; F.stage = 2; push = 0; cn = F.nB; cm = F.mB; ck = F.kB; }
            else if (F.stage == 2) { F.acc = F.acc + ret; F.stage = 3; push = 1; cn = F.nA; cm = F.mA; ck = F.kA; }
            else if (F.stage == 3) { F.acc2 = ret; F.stage = 4; push = 1; cn = F.nB; cm = F.mB; ck = F.kB; }
            else if (F.stage == 4) { F.acc = F.acc + (r * (F.acc2 + ret)); F.stage = 5; push = 1; cn = F.nC; cm = F.mC; ck = F.kC; }
            else { double val = F.acc - ret; ws[1][F.k] = val; ret = val; goto pop; }
        } else {  // zernike_R_over_r_c: R(A)+R(B) - Ro(C)
            if (F.stage == 1) { F.acc = ret; F.stage = 2; push = 0; cn = F.nB; cm = F.mB; ck = F.kB; }
            else if (F.stage == 2) { F.acc = F.acc + ret; F.stage = 3; push = 2; cn = F.nC; cm = F.mC; ck = F.kC; }
            else { double val = F.acc - ret; ws[2][F.k] = val; ret = val; goto pop; }
        }
        if (sp + 1 >= RP_ZK_DEPTH) { atomicOr(err, ERR_ZK_STACK); return 0.0; }
        sp++;
        st[sp].fn = (signed char)push;
        st[sp].stage = 0;
        st[sp].n = (short)cn;
        st[sp].m = (short)cm;
        st[sp].k = (short)ck;
        continue;
    pop:
        if (sp == 0) return ret;
        sp--;
    }
    atomicOr(err, ERR_ZK_STACK);
    return 0.0;
}

// The polar angle of (x, y) as its cosine and sine.  For r > 0 they are x / r
// and y / r (within an ulp or two of cos / sin of atan2(y, x)); at the origin
// the reference's atan2 of signed zeros decides the angle.
__device__ __forceinline__ void polar_cs(double x, double y, double r, double &c, double &s) {
    if (r > 0.0) {
        c = x / r;
        s = y / r;
    } else {
        const double t = atan2(y, x);
        c = cos(t);
        s = sin(t);
    }
}

// cos(m t) and sin(m t) for m >= 0 from c = cos t, s = sin t (Chebyshev
// recurrence).  The reference calls cos / sin of m * theta for every Zernike
// term; FP64 trigonometry costs GB300's slow FP64 pipe about fifty
// instructions a call, and a distorted face is evaluated some forty times
// per ray test, so the terms share the angle and step up from it (the
// results differ from the library calls by a few ulp).
__device__ __forceinline__ void multi_angle(int m, double c, double s, double &cm, double &sm) {
    double c0 = 1.0, s0 = 0.0, c1 = c, s1 = s;
    if (m == 0) {
        cm = 1.0;
        sm = 0.0;
        return;
    }
    for (int k = 2; k <= m; k++) {
        const double c2 = 2.0 * c * c1 - c0, s2 = 2.0 * c * s1 - s0;
        c0 = c1;
        s0 = s1;
        c1 = c2;
        s1 = s2;
    }
    cm = c1;
    sm = s1;
}

// Replays distortion d's compiled program (grad: the z-and-gradient one) at
// radius r into ws and returns its result slots, or null when the recursion
// must run instead (no program, or r not finite, where the recursion's memo
// reads see NaN values and would repeat work the program assumes done).
__device__ __forceinline__ const short *zk_program(const DevScene &S, const rp_distortion &d, bool grad, double r,
                                                   double *ws) {
    if (!S.zk_off || !isfinite(r)) return nullptr;
    const int off = S.zk_off[2 * (int)(&d - S.dists) + (grad ? 1 : 0)];
    if (off < 0) return nullptr;
    const short *p = S.zk_prog + off;
    const int n_ops = p[0];
    ws[0] = 0.0;
    ws[1] = 1.0;
    const short *o = p + 3;
    for (int j = 0; j < n_ops; j++, o += RP_ZKOP_WORDS) {
        const double a = ws[o[2]], b = ws[o[3]], c = ws[o[4]];
        double v;
        if (o[1] == 0) v = r * (a + b) - c;                          // zernike_R_c
        else if (o[1] == 1) v = (a + b) + r * (c + ws[o[5]]) - ws[o[6]];  // zernike_Rprime_c
        else v = (a + b) - c;                                        // zernike_R_over_r_c
        ws[o[0]] = v;
    }
    return o;  // the result slots follow the operations
}

// ZernikeDistortion.z_offset_c (cdistortions.pyx:416-450) and the
// SimpleTestZernikeJ7 variant (48-60).
static __device__ double dist_z(const DevScene &S, const rp_distortion &d, double x, double y, unsigned *err) {
    if (d.type == RP_DIST_SIMPLE_J7) {
        x /= d.unit_radius;
        y /= d.unit_radius;
        double Z = sqrt(8.0) * (3 * (x * x + y * y) - 2) * y;
        return Z * d.amplitude;
    }
    double ws[3][RP_ZK_SLOTS];
    double Z = 0.0;
    x /= d.unit_radius;
    y /= d.unit_radius;
    double r = sqrt(x * x + y * y);
    double ct, st;
    polar_cs(x, y, r, ct, st);
    const short *res = zk_program(S, d, false, r, &ws[0][0]);
    if (!res) {
        int kmax = min(d.k_max, RP_ZK_SLOTS);
        for (int i = 0; i < kmax; i++) ws[0][i] = nan_d();
        ws[0][0] = 1.0;
    }
    const double *c = S.aux + d.aux;
    for (int i = 0; i < d.n_coefs; i++) {
        int n = (int)c[5 * i + 1], m = (int)c[5 * i + 2], k = (int)c[5 * i + 3];
        double N, PH, cm, sm;
        if (m == 0) N = sqrt((double)(n + 1));
        else N = sqrt((double)(2 * (n + 1)));
        N *= c[5 * i + 4];
        multi_angle(abs(m), ct, st, cm, sm);
        if (m >= 0) PH = cm;  // cos(m theta)
        else PH = sm;         // -sin(m theta) = sin(|m| theta)
        double R = res ? (&ws[0][0])[res[i]] : zk_eval(0, k, n, abs(m), r, ws, err);
        Z += N * R * PH;
    }
    return Z;
}

// z_offset_and_gradient_c (cdistortions.pyx:456-514, 62-81): (dz/dx, dz/dy, z)
static __device__ v3 dist_zg(const DevScene &S, const rp_distortion &d, double x, double y, unsigned *err) {
    v3 Z;
    if (d.type == RP_DIST_SIMPLE_J7) {
        double root8 = sqrt(8.0) * d.amplitude, R = d.unit_radius;
        x /= R;
        y /= R;
        Z.x = root8 * 6 * x * y / R;
        Z.y = root8 * (3 * x * x + 9 * y * y - 2) / R;
        Z.z = root8 * (3 * (x * x + y * y) - 2) * y;
        return Z;
    }
    double ws[3][RP_ZK_SLOTS];
    x /= d.unit_radius;
    y /= d.unit_radius;
    double r = sqrt(x * x + y * y);
    double ct, st;
    polar_cs(x, y, r, ct, st);
    const short *res = zk_program(S, d, true, r, &ws[0][0]);
    if (!res) {
        int kmax = min(d.k_max, RP_ZK_SLOTS);
        for (int i = 0; i < kmax; i++) {
            ws[0][i] = nan_d();
            ws[1][i] = nan_d();
            ws[2][i] = nan_d();
        }
    }
    Z.x = 0.0;
    Z.y = 0.0;
    Z.z = 0.0;
    const double *c = S.aux + d.aux;
    for (int i = 0; i < d.n_coefs; i++) {
        int n = (int)c[5 * i + 1], m = (int)c[5 * i + 2], k = (int)c[5 * i + 3];
        double N, PH, PHprime, cm, sm;
        multi_angle(abs(m), ct, st, cm, sm);
        if (m >= 0) {
            PH = cm;             // cos(m theta)
            PHprime = -m * sm;   // -m sin(m theta)
        } else {
            PH = sm;             // -sin(m theta)
            PHprime = -m * cm;   // -m cos(m theta)
        }
        double R, Rprime, R_over_r;
        if (res) {
            R = (&ws[0][0])[res[3 * i]];
            Rprime = (&ws[0][0])[res[3 * i + 1]];
            R_over_r = (&ws[0][0])[res[3 * i + 2]];
        } else {
            R = zk_eval(0, k, n, abs(m), r, ws, err);
            Rprime = zk_eval(1, k, n, abs(m), r, ws, err);
            R_over_r = zk_eval(2, k, n, abs(m), r, ws, err);
        }
        if (m == 0) N = sqrt((double)(n + 1));
        else N = sqrt((double)(2 * (n + 1)));
        N *= c[5 * i + 4];
        Z.z += N * R * PH;
        Z.x += N * (Rprime * ct * PH + R_over_r * (-st) * PHprime);
        Z.y += N * (Rprime * st * PH + R_over_r * (ct)*PHprime);
    }
    Z.x /= d.unit_radius;
    Z.y /= d.unit_radius;
    return Z;
}

// ---- faces: cfaces.pyx ----------------------------------------------------
// intersect_conic, cfaces.pyx:1695-1747
__device__ __forceinline__ double intersect_conic(v3 a, v3 d, double curvature, double conic_const) {
    double beta = 1 + conic_const;
    double R = -curvature;
    double b2 = beta * beta;
    double A = b2 * (d.z * d.z) + beta * (d.x * d.x) + beta * (d.y * d.y);
    double B = -2 * R * beta * d.z + 2 * a.x * beta * d.x + 2 * a.y * beta * d.y + 2 * a.z * b2 * d.z;
    double C = -2 * R * a.z * beta + (a.x * a.x) * beta + (a.y * a.y) * beta + (a.z * a.z) * b2;
    double D = B * B - 4 * A * C;
    if (D < 0) return -1;
    D = sqrt(D);
    if (R * beta * d.z <= 0) return (-B + D) / (2 * A);
    return (-B - D) / (2 * A);
}

// AsphericFace sag residual and its alpha-derivative (cfaces.pyx:1854-1882).
// p: curvature, z_height, conic, A4, A6, A8, A10, A12, A14, A16, atol; p[11] = highest
// power k of r^2 with a non-zero coefficient (terms with a zero coefficient
// add only a signed zero in the reference and are skipped); p[12] = R**3 with
// R = -curvature.
__device__ __forceinline__ void asph_eval(const rp_face &f, v3 a, v3 d, double alpha, bool want_f, bool want_g,
                                          double *F, double *G) {
    double R = -f.p[0], beta = 1 + f.p[2];
    int kmax = min(max((int)f.p[11], 2), 8);
    double ux = a.x + alpha * d.x, uy = a.y + alpha * d.y;
    double r2 = (ux * ux) + (uy * uy);
    double pw[9];
    ipow_table(r2, kmax < 2 ? 2 : kmax, pw);
    double R2 = R * R;
    double root = sqrt(1 - beta * r2 / R2);
    if (want_f) {
        double out = r2;
        out /= R * (1 + root);
        out -= a.z + alpha * d.z;
        double poly = f.p[3] * pw[2];
        if (kmax >= 3) poly = poly + f.p[4] * pw[3];
        if (kmax >= 4) poly = poly + f.p[5] * pw[4];
        if (kmax >= 5) poly = poly + f.p[6] * pw[5];
        if (kmax >= 6) poly = poly + f.p[7] * pw[6];
        if (kmax >= 7) poly = poly + f.p[8] * pw[7];
        if (kmax >= 8) poly = poly + f.p[9] * pw[8];
        out += poly;
        *F = out;
    }
    if (want_g) {
        double dx = d.x * ux, dy = d.y * uy;
        double out = 0.0;
        bool first = true;
        if (kmax >= 5) { out = f.p[6] * (10 * dx + 10 * dy) * pw[4]; first = false; }
        if (kmax >= 6) { double t = f.p[7] * (12 * dx + 12 * dy) * pw[5]; out = first ? t : out + t; first = false; }
        if (kmax >= 7) { double t = f.p[8] * (14 * dx + 14 * dy) * pw[6]; out = first ? t : out + t; first = false; }
        if (kmax >= 8) { double t = f.p[9] * (16 * dx + 16 * dy) * pw[7]; out = first ? t : out + t; first = false; }
        {
            double t = f.p[3] * (4 * dx + 4 * dy) * (r2);
            out = first ? t : out + t;
        }
        if (kmax >= 3) out += f.p[4] * (6 * dx + 6 * dy) * pw[2];
        if (kmax >= 4) out += f.p[5] * (8 * dx + 8 * dy) * pw[3] - d.z;
        else out += 0.0 - d.z;
        double R3 = f.p[12];  // pow(R, 3.0), evaluated once on the host with libm pow
        out += (2 * dx + 2 * dy) / (R * (root + 1));
        double rp1 = root + 1;
        out += beta * (2 * dx + 2 * dy) * (r2) / (2 * R3 * root * (rp1 * rp1));
        *G = out;
    }
}

// ExtendedPolynomialFace residual / derivative (cfaces.pyx:2043-2126).
// p: R, beta, norm_radius, z_height, atol; aux: coefs [Nx][Ny].
__device__ __forceinline__ double extpoly_impf(const DevScene &S, const rp_face &f, v3 a, v3 d, double alpha) {
    const double *E = S.aux + f.aux;
    int Nx = f.n_aux0, Ny = f.n_aux1;
    double x = a.x + alpha * d.x;
    double y = a.y + alpha * d.y;
    double r2 = (x * x) + (y * y);
    double R = f.p[0], beta = f.p[1];
    double out = r2;
    if (R >= 0) out /= (R + sqrt(R * R - beta * r2));
    else out /= (R - sqrt(R * R - beta * r2));
    out -= a.z + alpha * d.z;
    x /= f.p[2];
    y /= f.p[2];
    double px[8], py[8];
    ipow_table(x, Nx - 1, px);
    ipow_table(y, Ny - 1, py);
    for (int i = 0; i < Nx; i++)
        for (int j = 0; j < Ny; j++) out += E[i * Ny + j] * px[i] * py[j];
    out += f.p[3];
    return out;
}

__device__ __forceinline__ double extpoly_grad(const DevScene &S, const rp_face &f, v3 a, v3 d, double alpha) {
    const double *E = S.aux + f.aux;
    int Nx = f.n_aux0, Ny = f.n_aux1;
    double R = f.p[0], beta = f.p[1];
    double dEdx = 0.0, dEdy = 0.0;
    double x = a.x + alpha * d.x;
    double y = a.y + alpha * d.y;
    double r2 = (x * x) + (y * y);
    double R2 = R * R;
    double rt = sqrt(1 - (beta * r2 / R2));
    double denom = R * (rt + 1);
    double nom = (2 * d.x * x + 2 * d.y * y);
    double inv_rad = 1. / f.p[2];
    double out = -d.z;
    out += nom / denom;
    out += beta * nom * r2 / (2 * R * rt * denom * denom);
    x *= inv_rad;
    y *= inv_rad;
    double px[8], py[8];
    ipow_table(x, Nx - 1, px);
    ipow_table(y, Ny - 1, py);
    for (int i = 1; i < Nx; i++)
        for (int j = 0; j < Ny; j++) dEdx += (i)*E[i * Ny + j] * px[i - 1] * py[j];
    for (int i = 0; i < Nx; i++)
        for (int j = 1; j < Ny; j++) dEdy += (j)*E[i * Ny + j] * px[i] * py[j - 1];
    dEdx *= inv_rad;
    dEdy *= inv_rad;
    out += dEdx * d.x;
    out += dEdy * d.y;
    return out;
}

__device__ __forceinline__ int point_in_polygon(const double *xy, int size, double X, double Y) {
    // point_in_polygon_c, cfaces.pyx:1050-1068
    int ct = 0;
    if (size < 1) return 0;
    double y1 = xy[2 * (size - 1) + 1], x1 = xy[2 * (size - 1)];
    for (int i = 0; i < size; i++) {
        double y2 = xy[2 * i + 1], x2 = xy[2 * i];
        double h = (Y - y1) / (y2 - y1);
        if (0 < h && h <= 1.0) {
            double x = x1 + h * (x2 - x1);
            if (x > X) ct = !ct;
        }
        y1 = y2;
        x1 = x2;
    }
    return ct;
}

#define RP_MISS (-1.0)

// Face.intersect_c of every face type except DistortionFace.  Returns the
// distance, or -1 for NO_INTERSECTION (cfaces.pyx:40-44).
static __device__ double face_isect_base(const DevScene &S, const rp_face &f, v3 p1, v3 p2, int is_base_ray,
                                  unsigned *err) {
    switch (f.type) {
        case RP_FACE_NONE: return 0.0;  // ctracer.pyx:1747-1757
        case RP_FACE_CIRCULAR: {        // cfaces.pyx:147-175
            double h = (f.p[2] - p1.z) / (p2.z - p1.z);
            if ((h < f.tolerance) || (h > 1.0)) return RP_MISS;
            double X = p1.x + h * (p2.x - p1.x) - f.p[1];
            double Y = p1.y + h * (p2.y - p1.y);
            double dd = f.p[0];
            if (is_base_ray && (X * X + Y * Y) > (dd * dd / 4)) return RP_MISS;
            return h * sepv(p1, p2);
        }
        case RP_FACE_SHAPED_PLANAR: {  // cfaces.pyx:201-227
            double h = (f.p[0] - p1.z) / (p2.z - p1.z);
            if ((h < f.tolerance) || (h > 1.0)) return RP_MISS;
            double X = p1.x + h * (p2.x - p1.x);
            double Y = p1.y + h * (p2.y - p1.y);
            if (is_base_ray && !shape_inside(S, f.shape, X, Y, err)) return RP_MISS;
            return h * sepv(p1, p2);
        }
        case RP_FACE_ELLIPTICAL_PLANE: {  // cfaces.pyx:323-340
            double gx = f.p[0], gy = f.p[1], dd = f.p[2];
            double h = (gx * p1.x + gy * p1.y - p1.z) / ((p2.z - p1.z) - gx * (p2.x - p1.x) - gy * (p2.y - p1.y));
            if ((h < f.tolerance) || (h > 1.0)) return RP_MISS;
            double X = p1.x + h * (p2.x - p1.x);
            double Y = p1.y + h * (p2.y - p1.y);
            if (is_base_ray && (X * X + Y * Y) > (dd * dd / 4)) return RP_MISS;
            return h * sepv(p1, p2);
        }
        case RP_FACE_RECTANGULAR: {  // cfaces.pyx:364-396
            double h = (f.p[3] - p1.z) / (p2.z - p1.z);
            if ((h < f.tolerance) || (h > 1.0)) return RP_MISS;
            if (is_base_ray) {
                double X = p1.x + h * (p2.x - p1.x) - f.p[2];
                double Y = p1.y + h * (p2.y - p1.y);
                if (X * X > f.p[0] * f.p[0] / 4) return RP_MISS;
                if (Y * Y > f.p[1] * f.p[1] / 4) return RP_MISS;
            }
            return h * sepv(p1, p2);
        }
        case RP_FACE_POLYGON: {  // cfaces.pyx:1096-1108
            double h = (f.p[0] - p1.z) / (p2.z - p1.z);
            if ((h < f.tolerance) || (h > 1.0)) return RP_MISS;
            double X = p1.x + h * (p2.x - p1.x);
            double Y = p1.y + h * (p2.y - p1.y);
            if (is_base_ray && point_in_polygon(S.aux + f.aux, f.n_aux0, X, Y) == 1) return h * sepv(p1, p2);
            return RP_MISS;
        }
        case RP_FACE_SPHERICAL:
        case RP_FACE_SHAPED_SPHERICAL: {  // cfaces.pyx:418-482, 512-592
            bool plain = f.type == RP_FACE_SPHERICAL;
            double curvature = plain ? f.p[1] : f.p[0];
            double z_height = plain ? f.p[2] : f.p[1];
            v3 s = subv(p2, p1);
            double cz = z_height - curvature;
            v3 d = p1;
            d.z -= cz;
            double A = magsq(s);
            double B = 2 * dotv(s, d);
            double C = magsq(d) - curvature * curvature;
            double D = B * B - 4 * A * C;
            if (D < 0) return RP_MISS;
            D = sqrt(D);
            double twoA = 2 * A;
            double a1 = (-B + D) / twoA;
            double a2 = (-B - D) / twoA;
            v3 pt1 = addv(p1, mulvs(s, a1));
            v3 pt2 = addv(p1, mulvs(s, a2));
            double INF = inf_d();
            if (curvature >= 0) {
                if (pt1.z < cz) a1 = INF;
                if (pt2.z < cz) a2 = INF;
            } else {
                if (pt1.z > cz) a1 = INF;
                if (pt2.z > cz) a2 = INF;
            }
            if (is_base_ray) {
                if (plain) {
                    double DD = f.p[0] * f.p[0] / 4.;
                    if ((pt1.x * pt1.x + pt1.y * pt1.y) > DD) a1 = INF;
                    if ((pt2.x * pt2.x + pt2.y * pt2.y) > DD) a2 = INF;
                } else {
                    if (!shape_inside(S, f.shape, pt1.x, pt1.y, err)) a1 = INF;
                    if (!shape_inside(S, f.shape, pt2.x, pt2.y, err)) a2 = INF;
                }
            }
            if (a2 < a1) a1 = a2;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        case RP_FACE_CONIC: {  // cfaces.pyx:1766-1794
            v3 d = subv(p2, p1);
            v3 a = p1;
            a.z -= f.p[1];
            double a1 = intersect_conic(a, d, f.p[0], f.p[2]);
            v3 pt1 = addv(a, mulvs(d, a1));
            if (is_base_ray && !shape_inside(S, f.shape, pt1.x, pt1.y, err)) return RP_MISS;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        case RP_FACE_ASPHERIC: {  // cfaces.pyx:1908-1974
            double tol = f.p[10] * f.p[10];
            v3 d = subv(p2, p1);
            v3 a = p1;
            a.z -= f.p[1];
            double a1 = intersect_conic(a, d, f.p[0], f.p[2]);
            double fv, gv, f_last, dz;
            asph_eval(f, a, d, a1, true, true, &fv, &gv);
            f_last = fv;
            dz = -fv / gv;
            bool conv = false;
            for (int i = 0; i < 100; i++) {
                a1 += dz;
                if (dz * dz < tol) { conv = true; break; }
                asph_eval(f, a, d, a1, true, true, &fv, &gv);  // f and its derivative share r^2 and the root
                if (fabs(fv) > fabs(f_last)) return RP_MISS;
                f_last = fv;
                dz = -fv / gv;
            }
            if (!conv) return RP_MISS;
            v3 pt1 = addv(a, mulvs(d, a1));
            if (is_base_ray && !shape_inside(S, f.shape, pt1.x, pt1.y, err)) return RP_MISS;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        case RP_FACE_EXTPOLY: {  // cfaces.pyx:2182-2234
            double tol = f.p[4] * f.p[4];
            v3 d = subv(p2, p1);
            v3 a = p1;
            a.z -= f.p[3];
            double a1 = intersect_conic(a, d, -f.p[0], f.p[1] - 1.0);
            double fv = extpoly_impf(S, f, p1, d, a1);
            double f_last = fv;
            double dz = -fv / extpoly_grad(S, f, p1, d, a1);
            bool conv = false;
            for (int i = 0; i < 100; i++) {
                a1 += dz;
                if (dz * dz < tol) { conv = true; break; }
                fv = extpoly_impf(S, f, p1, d, a1);
                if (fabs(fv) > fabs(f_last)) return RP_MISS;
                f_last = fv;
                dz = -fv / extpoly_grad(S, f, p1, d, a1);
            }
            if (!conv) return RP_MISS;
            v3 pt1 = addv(a, mulvs(d, a1));
            if (is_base_ray && !shape_inside(S, f.shape, pt1.x, pt1.y, err)) return RP_MISS;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        case RP_FACE_ORIENTED_POLYGON: {  // cfaces.pyx:1189-1215
            v3 o = mkv(f.p[0], f.p[1], f.p[2]), n = mkv(f.p[3], f.p[4], f.p[5]);
            v3 line = subv(p2, p1);
            double max_length = magv(line);
            line = normv(line);
            double h = dotv(line, n);
            if (h == 0.0) return RP_MISS;
            h = dotv(subv(o, p1), n) / h;
            if ((h < f.tolerance) || (h > max_length)) return RP_MISS;
            if (is_base_ray) {
                line = subv(addv(p1, mulvs(line, h)), o);
                double X = dotv(line, mkv(f.p[6], f.p[7], f.p[8]));
                double Y = dotv(line, mkv(f.p[9], f.p[10], f.p[11]));
                if (point_in_polygon(S.aux + f.aux, f.n_aux0, X, Y) == 1) return h;
                return RP_MISS;
            }
            return h;
        }
        case RP_FACE_OFF_AXIS_PARABOLIC: {  // cfaces.pyx:1228-1297; p: EFL, diameter
            // paraboloid z + efl/2 = A (x^2 + y^2), aperture centred on x = efl
            const double efl = f.p[0], A = 1 / (2 * efl);
            v3 s = subv(p2, p1);
            v3 r = p1;
            r.z += efl / 2.;
            double a = A * (s.x * s.x + s.y * s.y);
            double b = 2 * A * (r.x * s.x + r.y * s.y) - s.z;
            double c = A * (r.x * r.x + r.y * r.y) - r.z;
            double d = b * b - 4 * a * c;
            if (d < 0) return RP_MISS;
            if (a < 1e-10) {
                // near-axial ray: the linear root; the aperture test here
                // compares r^2 with diameter/2, as the reference does
                double a1 = -c / b;
                v3 pt1 = addv(r, mulvs(s, a1));
                pt1.x -= efl;
                if ((pt1.x * pt1.x + pt1.y * pt1.y) > (f.p[1] / 2)) return RP_MISS;
                if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
                return a1 * sepv(p1, p2);
            }
            d = sqrt(d);
            double a1 = (-b + d) / (2 * a);
            v3 pt1 = addv(r, mulvs(s, a1));
            double a2 = (-b - d) / (2 * a);
            v3 pt2 = addv(r, mulvs(s, a2));
            pt1.x -= efl;
            pt2.x -= efl;
            if (is_base_ray) {
                double dd = f.p[1];
                dd *= dd / 4.;
                if ((pt1.x * pt1.x + pt1.y * pt1.y) > dd) a1 = inf_d();
                if ((pt2.x * pt2.x + pt2.y * pt2.y) > dd) a2 = inf_d();
            }
            if (a2 < a1) a1 = a2;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        case RP_FACE_ELLIPSOIDAL: {  // cfaces.pyx:1339-1384; p: major, minor, x1, x2, y1, y2, z1, z2
            const double *T = S.aux + f.aux;  // trans (m, t): the face-list frame -> the ellipse frame
            v3 Sv = subv(p2, p1);
            v3 r = xform(T, T + 9, p1);
            v3 s = subv(xform(T, T + 9, p2), r);
            double B = f.p[1] * f.p[1], A = f.p[0] * f.p[0];
            double a = A * (s.z * s.z + s.y * s.y) + B * s.x * s.x;
            double b = 2 * (A * (r.z * s.z + r.y * s.y) + B * r.x * s.x);
            double c = A * (r.z * r.z + r.y * r.y) + B * r.x * r.x - A * B;
            double d = sqrt(b * b - 4 * a * c);  // NaN for a miss: every bound test below fails
            double root1 = (-b + d) / (2 * a);
            double root2 = (-b - d) / (2 * a);
            v3 q2 = addv(p1, mulvs(Sv, root2));
            v3 q1 = addv(p1, mulvs(Sv, root1));
            if (is_base_ray) {
                if (!(f.p[2] < q2.x && q2.x < f.p[3])) root2 = 2;
                if (!(f.p[4] < q2.y && q2.y < f.p[5])) root2 = 2;
                if (!(f.p[6] < q2.z && q2.z < f.p[7])) root2 = 2;
                if (!(f.p[2] < q1.x && q1.x < f.p[3])) root1 = 2;
                if (!(f.p[4] < q1.y && q1.y < f.p[5])) root1 = 2;
                if (!(f.p[6] < q1.z && q1.z < f.p[7])) root1 = 2;
            }
            if (root1 < f.tolerance) root1 = 2;
            if (root2 < f.tolerance) root2 = 2;
            if (root1 > root2) root1 = root2;
            if (root1 > 1) return RP_MISS;
            return root1 * magv(Sv);  // NaN (never a hit) when the ray misses a non-base test
        }
        case RP_FACE_SADDLE: {  // cfaces.pyx:1421-1495; p: z_height, curvature; z = sqrt(6) c x y
            double A = sqrt(6.0) * f.p[1];
            v3 p = p1;
            p.z -= f.p[0];
            v3 d = subv(p2, p1);
            double a1, a2;
            if (d.x == 0.0) {
                a1 = (-A * (p.x * p.y) + p.z) / (A * d.y * p.x - d.z);
                a2 = inf_d();
            } else if (d.y == 0.0) {
                a1 = (-A * (p.x * p.y) + p.z) / (A * d.x * p.y - d.z);
                a2 = inf_d();
            } else {
                double A2 = A * A;
                double root = A2 * (d.x * d.x) * (p.y * p.y) - 2 * A2 * d.x * d.y * p.x * p.y +
                              A2 * (d.y * d.y) * (p.x * p.x) + 4 * A * d.x * d.y * p.z - 2 * A * d.x * d.z * p.y -
                              2 * A * d.y * d.z * p.x + d.z * d.z;
                if (root < 0) return RP_MISS;
                root = sqrt(root);
                double denom = 2 * A * (d.x * d.y);
                a1 = a2 = -A * d.x * p.y - A * d.y * p.x + d.z;
                a1 += root;
                a2 -= root;
                a1 /= denom;
                a2 /= denom;
            }
            v3 pt1 = addv(p1, mulvs(d, a1));
            v3 pt2 = addv(p1, mulvs(d, a2));
            if (a1 < 0.0) a1 = inf_d();
            if (a2 < 0.0) a2 = inf_d();
            if (is_base_ray) {
                if (!shape_inside(S, f.shape, pt1.x, pt1.y, err)) a1 = inf_d();
                if (!shape_inside(S, f.shape, pt2.x, pt2.y, err)) a2 = inf_d();
            }
            if (a2 < a1) a1 = a2;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        case RP_FACE_CYLINDRICAL: {  // cfaces.pyx:1524-1582; p: z_height, radius (axis along y)
            const double R = f.p[1], R2 = R * R;
            v3 o = p1;
            o.z -= f.p[0];
            v3 d = subv(p2, p1);
            double ox2 = o.x * o.x, oz2 = o.z * o.z, dx2 = d.x * d.x, dz2 = d.z * d.z;
            double root = R2 * dz2 - 2 * R * dx2 * o.z + 2 * R * d.x * d.z * o.x - dx2 * oz2 +
                          2 * d.x * d.z * o.x * o.z - dz2 * ox2;
            if (root < 0) return RP_MISS;
            root = sqrt(root);
            double denom = dx2 + dz2;
            double a1, a2;
            a1 = a2 = -R * d.z - d.x * o.x - d.z * o.z;
            a1 += root;
            a2 -= root;
            a1 /= denom;
            a2 /= denom;
            v3 pt1 = addv(p1, mulvs(d, a1));
            v3 pt2 = addv(p1, mulvs(d, a2));
            double cz = f.p[0] - R;
            if (R >= 0) {
                if (pt1.z < cz) a1 = inf_d();
                if (pt2.z < cz) a2 = inf_d();
            } else {
                if (pt1.z > cz) a1 = inf_d();
                if (pt2.z > cz) a2 = inf_d();
            }
            if (is_base_ray) {
                if (!shape_inside(S, f.shape, pt1.x, pt1.y, err)) a1 = inf_d();
                if (!shape_inside(S, f.shape, pt2.x, pt2.y, err)) a2 = inf_d();
            }
            if (a2 < a1) a1 = a2;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        case RP_FACE_AXICON: {  // cfaces.pyx:1617-1664; p: z_height, gradient; z = z_height - gradient r
            const double beta = f.p[1], beta2 = beta * beta;
            v3 d = subv(p2, p1);
            v3 o = p1;
            o.z -= f.p[0];
            double ox2 = o.x * o.x, oy2 = o.y * o.y, oz2 = o.z * o.z;
            double dx2 = d.x * d.x, dy2 = d.y * d.y, dz2 = d.z * d.z;
            double root = -beta2 * dx2 * oy2 + 2 * beta2 * d.x * d.y * o.x * o.y - beta2 * dy2 * ox2 + dx2 * oz2 -
                          2 * d.x * d.z * o.x * o.z + dy2 * oz2 - 2 * d.y * d.z * o.y * o.z + dz2 * ox2 + dz2 * oy2;
            double denom = (beta2 * dx2 + beta2 * dy2 - dz2);
            if (root < 0) return RP_MISS;
            root = beta * sqrt(root);
            double a1 = -beta2 * d.x * o.x - beta2 * d.y * o.y + d.z * o.z;
            double a2 = a1 + root;
            a1 -= root;
            a1 /= denom;
            a2 /= denom;
            v3 pt1 = addv(p1, mulvs(d, a1));
            v3 pt2 = addv(p1, mulvs(d, a2));
            if (pt1.z > f.p[0]) a1 = inf_d();
            if (pt2.z > f.p[0]) a2 = inf_d();
            if (is_base_ray) {
                if (!shape_inside(S, f.shape, pt1.x, pt1.y, err)) a1 = inf_d();
                if (!shape_inside(S, f.shape, pt2.x, pt2.y, err)) a2 = inf_d();
            }
            if (a2 < a1) a1 = a2;
            if (a1 > 1.0 || a1 < f.tolerance) return RP_MISS;
            return a1 * sepv(p1, p2);
        }
        default: return RP_MISS;
    }
}

// Face.compute_normal_c of every face type except DistortionFace.
static __device__ v3 face_normal_base(const DevScene &S, const rp_face &f, v3 p) {
    switch (f.type) {
        case RP_FACE_CIRCULAR: return mkv(0, 0, f.invert_normals ? 1 : -1);  // cfaces.pyx:177-191
        case RP_FACE_SHAPED_PLANAR: return mkv(0, 0, 1);                      // 229-237
        case RP_FACE_ELLIPTICAL_PLANE: return normv(mkv(f.p[0], f.p[1], -1)); // 342-351
        case RP_FACE_RECTANGULAR:                                              // 398-407
        case RP_FACE_POLYGON: return mkv(0, 0, -1);                           // 1110-1118
        case RP_FACE_SPHERICAL:
        case RP_FACE_SHAPED_SPHERICAL: {  // 485-498, 594-606
            bool plain = f.type == RP_FACE_SPHERICAL;
            double curvature = plain ? f.p[1] : f.p[0];
            double z_height = plain ? f.p[2] : f.p[1];
            p.z -= (z_height - curvature);
            if (curvature < 0) p = negv(p);
            return normv(p);
        }
        case RP_FACE_CONIC: {  // 1796-1820
            double R = -f.p[0], beta = 1 + f.p[2];
            int sign = f.invert_normals ? -1 : 1;
            p.z -= f.p[1];
            v3 g;
            g.z = 2 * beta * (R - beta * p.z);
            g.x = -p.x * 2 * beta;
            g.y = -p.y * 2 * beta;
            if ((R * beta) < 0) sign *= -1;
            g.z *= sign;
            g.y *= sign;
            g.x *= sign;
            return normv(g);
        }
        case RP_FACE_ASPHERIC: {  // 1976-2005
            double R = -f.p[0], beta = 1 + f.p[2];
            int sign = f.invert_normals ? -1 : 1;
            p.z -= f.p[1];
            double r2 = p.x * p.x + p.y * p.y;
            double root = sqrt(1 - (beta * (r2) / (R * R)));
            double pw[9];
            ipow_table(r2, 7, pw);
            double df = 10 * f.p[6] * pw[4] + 8 * f.p[5] * pw[3] + 6 * f.p[4] * pw[2] + 4 * f.p[3] * r2;
            df += 16 * f.p[9] * pw[7] + 14 * f.p[8] * pw[6] + 12 * f.p[7] * pw[5];
            df += 2 / (R * (1 + root));
            double rp1 = 1 + root;
            df += beta * (r2) / (f.p[12] * root * (rp1 * rp1));
            v3 g = mkv(-df * p.x, -df * p.y, 1.0);
            g.z *= sign;
            g.y *= sign;
            g.x *= sign;
            return normv(g);
        }
        case RP_FACE_EXTPOLY: {  // 2236-2293
            const double *E = S.aux + f.aux;
            int Nx = f.n_aux0, Ny = f.n_aux1;
            double R = f.p[0], beta = f.p[1];
            int sign = f.invert_normals ? -1 : 1;
            double inv_rad = 1. / f.p[2];
            double x = p.x * inv_rad;
            double y = p.y * inv_rad;
            p.z -= f.p[3];
            v3 g;
            g.z = 2 * beta * (R - beta * p.z);
            g.x = -p.x * 2 * beta;
            g.y = -p.y * 2 * beta;
            if ((R * beta) < 0) sign *= -1;
            g.z *= sign;
            g.y *= sign;
            g.x *= sign;
            g = normv(g);
            double px[8], py[8];
            ipow_table(x, Nx - 1, px);
            ipow_table(y, Ny - 1, py);
            if (f.invert_normals) {
                for (int i = 1; i < Nx; i++)
                    for (int j = 0; j < Ny; j++) g.x += i * E[i * Ny + j] * inv_rad * px[i - 1] * py[j];
                for (int i = 0; i < Nx; i++)
                    for (int j = 1; j < Ny; j++) g.y += j * E[i * Ny + j] * inv_rad * px[i] * py[j - 1];
            } else {
                for (int i = 1; i < Nx; i++)
                    for (int j = 0; j < Ny; j++) g.x -= i * E[i * Ny + j] * inv_rad * px[i - 1] * py[j];
                for (int i = 0; i < Nx; i++)
                    for (int j = 1; j < Ny; j++) g.y -= j * E[i * Ny + j] * inv_rad * px[i] * py[j - 1];
            }
            return normv(g);
        }
        case RP_FACE_ORIENTED_POLYGON: return mkv(f.p[3], f.p[4], f.p[5]);  // 1183-1184
        case RP_FACE_OFF_AXIS_PARABOLIC: {  // 1299-1315 (unit length by construction)
            double A = 1 / (2 * f.p[0]);
            double m2 = p.x * p.x + p.y * p.y;
            double B = 4 * m2 * A * A;
            double dz = -sqrt(B / (B + 1));
            m2 = sqrt(m2);
            return mkv(-(dz * p.x) / m2, -(dz * p.y) / m2, -1 / sqrt(B + 1));
        }
        case RP_FACE_ELLIPSOIDAL: {  // 1386-1396: gradient in the ellipse frame, rotated back
            const double *T = S.aux + f.aux;
            p = xform(T, T + 9, p);
            double ma2 = f.p[0] * f.p[0], mi2 = f.p[1] * f.p[1];
            v3 n = mkv(p.x / -ma2, p.y / -mi2, p.z / -mi2);
            return normv(rotv(T + 12, n));
        }
        case RP_FACE_SADDLE: {  // 1497-1508
            double rt6 = sqrt(6.0) * f.p[1];
            return normv(mkv(-rt6 * p.y, -rt6 * p.x, 1.0));
        }
        case RP_FACE_CYLINDRICAL: {  // 1584-1595
            p.z -= (f.p[0] - f.p[1]);
            if (f.p[1] < 0) {
                p.z = -p.z;
                p.x = -p.x;
            }
            p.y = 0;
            return normv(p);
        }
        case RP_FACE_AXICON: {  // 1666-1677: not normalised, as in the reference
            double beta = f.p[1];
            double r = sqrt(p.x * p.x + p.y * p.y);
            return mkv(beta * p.x / r, beta * p.y / r, 1.0);
        }
        default: return p;  // Face.compute_normal_c, ctracer.pyx:1783-1784
    }
}

// DistortionFace.intersect_c, cfaces.pyx:2341-2407
// Out of line (as is zk_eval): inlined at every face-test site, the distorted
// face's iteration and Zernike code made the plain kernel's instruction
// footprint the bottleneck on scenes that use it (instruction-fetch stalls
// 24 per issued instruction on the 64-face clutter scene); one shared copy
// made that scene 1.8x faster and the lens-train scene's plain path 5 %.
static __device__ __noinline__ double distortion_isect(const DevScene &S, const rp_face &f, v3 p1, v3 p2, unsigned *err) {
    const rp_face &face = S.faces[f.base];
    const rp_distortion &dist = S.dists[f.distortion];
    double a1, a2, h = sepv(p2, p1);
    double tolerance = f.p[0];
    a2 = face_isect_base(S, face, p1, p2, 0, err);
    if (a2 > h || a2 < f.tolerance) return RP_MISS;
    v3 d = subv(p2, p1);
    v3 pt1 = addv(p1, mulvs(d, a2 / h));
    v3 dxdyz = dist_zg(S, dist, pt1.x, pt1.y, err);
    v3 n = face_normal_base(S, face, pt1);
    pt1.z += dxdyz.z;
    n.x /= n.z;
    n.y /= n.z;
    n.x -= dxdyz.x;
    n.y -= dxdyz.y;
    v3 o = subv(p1, pt1);
    a1 = -h * dotv(o, n) / dotv(d, n);
    if (a1 < fabs(dxdyz.z)) return RP_MISS;
    for (int i = 0; i < 20; i++) {
        pt1 = addv(p1, mulvs(d, a1 / h));
        if (fabs(a1 - a2) < tolerance) break;
        double z_shift = dist_z(S, dist, pt1.x, pt1.y, err);
        v3 q1 = p1, q2 = p2;
        q1.z -= z_shift;
        q2.z -= z_shift;
        a2 = face_isect_base(S, face, q1, q2, 0, err);
        pt1 = addv(q1, mulvs(d, a2 / h));
        n = face_normal_base(S, face, pt1);
        dxdyz = dist_zg(S, dist, pt1.x, pt1.y, err);
        pt1.z += dxdyz.z;
        n.x /= n.z;
        n.y /= n.z;
        n.x -= dxdyz.x;
        n.y -= dxdyz.y;
        o = subv(p1, pt1);
        a2 = a1;
        a1 = -h * dotv(o, n) / dotv(d, n);
    }
    if (!shape_inside(S, f.shape, pt1.x, pt1.y, err)) return RP_MISS;
    return a1;
}

__device__ __forceinline__ double face_isect(const DevScene &S, const rp_face &f, v3 p1, v3 p2, unsigned *err) {
    if (f.type == RP_FACE_DISTORTION) return distortion_isect(S, f, p1, p2, err);
    return face_isect_base(S, f, p1, p2, 1, err);
}

static __device__ v3 face_normal(const DevScene &S, const rp_face &f, v3 p, unsigned *err) {
    if (f.type == RP_FACE_DISTORTION) {  // cfaces.pyx:2409-2422
        v3 dxdyz = dist_zg(S, S.dists[f.distortion], p.x, p.y, err);
        v3 p1 = p;
        p1.z -= dxdyz.z;
        v3 n = face_normal_base(S, S.faces[f.base], p1);
        n.x /= n.z;
        n.y /= n.z;
        n.z = 1.0;
        n.x -= dxdyz.x;
        n.y -= dxdyz.y;
        return normv(n);
    }
    return face_normal_base(S, f, p);
}

__device__ __forceinline__ v3 face_tangent(const rp_face &f) {
    if (f.type == RP_FACE_ORIENTED_POLYGON) return mkv(f.p[6], f.p[7], f.p[8]);  // cfaces.pyx:1186-1187
    return mkv(1.0, 0.0, 0.0);                                                     // ctracer.pyx:1786-1791
}

// ---- rays and materials: cmaterials.pyx -----------------------------------
// The fields of a ray a material reads or writes (the rest is copied).
struct RayState {
    v3 o, d, E;        // origin, direction, E_vector
    cx n, e1, e2;      // refractive_index, E1_amp, E2_amp
    double len, phase, opl;
    unsigned wl, endf, ident, type;
};

// One emitted child: the fields that differ between children of one parent.
struct Child {
    v3 d;
    cx n, e1, e2;
    double len;
    unsigned type;
};

// The per-parent part every child of a hit shares.
struct ChildCommon {
    v3 origin, normal, E;
    double opl;
    double dphase;  // added to the parent's phase (the grating phase; 0 otherwise)
};

// convert_to_sp (cmaterials.pyx:49-91).  Returns false at normal incidence,
// where the reference returns the ray unchanged.
__device__ __forceinline__ void convert_to_sp(const RayState &r, v3 normal, v3 &E_out, cx &e1_out, cx &e2_out) {
    v3 E2_vector = normv_fast(crossv(r.d, r.E));
    v3 E1_vector = normv_fast(crossv(E2_vector, r.d));
    normal = normv_fast(normal);
    v3 S = crossv(r.d, normal);
    if (fabs(S.x) < 1.0e-10 && fabs(S.y) < 1.0e-10 && fabs(S.z) < 1.0e-10) {
        E_out = r.E;
        e1_out = r.e1;
        e2_out = r.e2;
        return;
    }
    S = normv_fast(S);
    v3 P = normv_fast(crossv(r.d, S));
    double A = dotv(E1_vector, S);
    double B = dotv(E2_vector, S);
    e1_out = mkc(r.e1.x * A + r.e2.x * B, r.e1.y * A + r.e2.y * B);
    B = dotv(E1_vector, P);
    A = dotv(E2_vector, P);
    e2_out = mkc(r.e1.x * B + r.e2.x * A, r.e1.y * B + r.e2.y * A);
    E_out = S;
}

// e^z (CUDA's exp, sin and cos; the reference calls glibc's cexp)
__device__ __forceinline__ cx cexp_(cx z) {
    double e = exp(z.x), s, c;
    sincos(z.y, &s, &c);
    return mkc(e * c, e * s);
}

// SingleLayerCoatedMaterial.eval_child_ray_c (cmaterials.pyx:1026-1184) and
// CoatedDispersiveMaterial.eval_child_ray_c (1228-1381): Fresnel coefficients
// of a single thin film (index n2, thickness in um) between n1 and n3 by the
// reference's characteristic-matrix product, with its phase
// phi = -i (2 pi t / lambda) (n2 - sin2^2) / cos2.
static __device__ int coated_children(const DevScene &S, const rp_material &m, const RayState &r, v3 point,
                                      v3 onormal, ChildCommon &cc, Child *ch, unsigned *err) {
    const double INF = inf_d();
    const long long w = (long long)r.wl;
    if (w >= S.n_wl) {
        atomicOr(err, ERR_WAVELENGTH);
        return 0;
    }
    const double wavelength = S.wl[w];
    v3 normal = normv_fast(onormal);
    v3 ind = normv_fast(r.d);
    cx E1, E2;
    convert_to_sp(r, normal, cc.E, E1, E2);
    cc.opl = r.opl + (r.len * r.n.x);
    cc.origin = point;
    cc.normal = normal;
    const double cosTheta = dotv(normal, ind);
    const double cos1 = fabs(cosTheta);
    const double sin1 = sqrt(fabs(1 - cos1 * cos1));
    const bool out_to_in = cosTheta < 0.0;
    cx n1, n2, n3;
    double thickness;
    if (m.type == RP_MAT_SINGLE_LAYER_COATED) {
        cx ni = mkc(m.n_inside[0], 0.0 + m.n_inside[1]), no = mkc(m.n_outside[0], 0.0 + m.n_outside[1]);
        n2 = mkc(m.p[0], 0.0 + m.p[1]);
        n1 = out_to_in ? no : ni;
        n3 = out_to_in ? ni : no;
        thickness = m.p[2];
    } else {
        const cx ni = S.ntab[(long long)m.curve_inside * S.n_wl + w];
        const cx no = S.ntab[(long long)m.curve_outside * S.n_wl + w];
        const cx nc = S.ntab[(long long)m.p[0] * S.n_wl + w];
        n2 = mkc(nc.x, 0.0 + nc.y);
        n1 = out_to_in ? mkc(no.x, 0.0 + no.y) : mkc(ni.x, 0.0 + ni.y);
        n3 = out_to_in ? mkc(ni.x, 0.0 + ni.y) : mkc(no.x, 0.0 + no.y);
        thickness = m.p[1];
    }
    const double flip = out_to_in ? 1 : -1;
    const cx sin2 = cdiv(cmuls(n1, sin1), n2);
    const cx cos2 = csqrt_(csub(mkc(1.0, 0.0), cmul(sin2, sin2)));
    const cx sin3 = cdiv(cmuls(n1, sin1), n3);
    const cx cos3 = csqrt_(csub(mkc(1.0, 0.0), cmul(sin3, sin3)));
    const v3 ctn = mulvs(normal, cosTheta);
    const double P_in = n1.x * (((E1.x * E1.x + E1.y * E1.y) + E2.x * E2.x) + E2.y * E2.y);
    if (P_in == 0.0) return 0;
    const cx n1cos1 = cmuls(n1, cos1), n2cos2 = cmul(n2, cos2), n3cos3 = cmul(n3, cos3);
    const double dwc = ((2.0 * 3.141592653589793) * thickness) / wavelength;
    // -i dwc = (0, -dwc)
    const cx phi = cdiv(cmul(mkc(0.0, -dwc), csub(n2, cmul(sin2, sin2))), cos2);
    const cx ep1 = cdiv(cexp_(phi), cmul(cmuls(n2cos2, 4.0), n3cos3));
    const cx ep2 = cexp_(cmuls(phi, -2.0));
    // s polarisation
    cx a = csub(n1cos1, n2cos2), bq = cadd(n1cos1, n2cos2), c = cadd(n2cos2, n3cos3), d = csub(n2cos2, n3cos3);
    cx M00 = cmul(mkc(-ep1.x, -ep1.y), cadd(cmul(a, c), cmul(cmul(bq, d), ep2)));
    cx M01 = cmul(ep1, cadd(cmul(cmul(a, d), ep2), cmul(bq, c)));
    cx M10 = cmul(ep1, cadd(cmul(a, d), cmul(cmul(bq, c), ep2)));
    cx M11 = cmul(mkc(-ep1.x, -ep1.y), cadd(cmul(cmul(a, c), ep2), cmul(bq, d)));
    cx R_s = cdiv(mkc(-M00.x, -M00.y), M01);
    cx T_s = cadd(M10, cmul(M11, R_s));
    // p polarisation
    const cx n1cos2 = cmul(n1, cos2), n2cos1 = cmuls(n2, cos1), n2cos3 = cmul(n2, cos3), n3cos2 = cmul(n3, cos2);
    a = csub(n1cos2, n2cos1);
    bq = cadd(n1cos2, n2cos1);
    c = cadd(n2cos3, n3cos2);
    d = csub(n2cos3, n3cos2);
    M00 = cmul(mkc(-ep1.x, -ep1.y), cadd(cmul(a, c), cmul(cmul(bq, d), ep2)));
    M01 = cmul(ep1, cadd(cmul(cmul(a, d), ep2), cmul(bq, c)));
    M10 = cmul(ep1, cadd(cmul(a, d), cmul(cmul(bq, c), ep2)));
    M11 = cmul(mkc(-ep1.x, -ep1.y), cadd(cmul(cmul(a, c), ep2), cmul(bq, d)));
    cx R_p = cdiv(mkc(-M00.x, -M00.y), M01);
    cx T_p = cadd(M10, cmul(M11, R_p));
    R_s = cmul(R_s, E1);
    R_p = cmul(R_p, E2);
    int nc = 0;
    if (((n1.x * (cabs2_(R_s) + cabs2_(R_p))) / P_in) > m.reflection_threshold) {
        ch[0].d = subv(ind, mulvs(ctn, 2.0));
        ch[0].len = INF;
        ch[0].e1 = R_s;
        ch[0].e2 = mkc(-R_p.x, -R_p.y);
        ch[0].n = n1;
        ch[0].type = r.type | RP_REFL_RAY;
        nc = 1;
    }
    v3 tg2 = mulvs(subv(ind, ctn), n1.x / n3.x);
    double c2 = sqrt(1 - magsq(tg2));
    v3 transmitted = subv(tg2, mulvs(normal, (c2 * flip)));
    double aspect = sqrt(cos3.x / cos1);
    T_s = cmul(T_s, cmuls(E1, aspect));
    T_p = cmul(T_p, cmuls(E2, aspect));
    if (((n3.x * (cabs2_(T_s) + cabs2_(T_p))) / P_in) > m.transmission_threshold) {
        ch[nc].d = transmitted;
        ch[nc].len = INF;
        ch[nc].e1 = T_s;
        ch[nc].e2 = T_p;
        ch[nc].n = n3;
        ch[nc].type = r.type & ~RP_REFL_RAY;
        nc++;
    }
    return nc;
}

// InterfaceMaterial.eval_child_ray_c for every material type.  Writes up to two
// children in emission order; returns their number.  `ntab` rows hold the
// complex index of each dispersion curve per wavelength index.
static __device__ int eval_children(const DevScene &S, const rp_material &m, const RayState &r, v3 point, v3 onormal,
                             v3 otangent, ChildCommon &cc, Child *ch, unsigned *err) {
    const double INF = inf_d();
    cc.dphase = 0.0;
    switch (m.type) {
        case RP_MAT_NONE:
        case RP_MAT_OPAQUE: return 0;  // cmaterials.pyx:245-251
        case RP_MAT_TRANSPARENT: {     // cmaterials.pyx:260-278
            v3 normal = normv_fast(onormal);
            cx e1, e2;
            convert_to_sp(r, normal, cc.E, e1, e2);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            ch[0].d = r.d;
            ch[0].n = r.n;
            ch[0].e1 = e1;
            ch[0].e2 = e2;
            ch[0].len = INF;
            ch[0].type = r.type & ~RP_REFL_RAY;
            return 1;
        }
        case RP_MAT_PEC: {  // cmaterials.pyx:285-319
            v3 normal = normv_fast(onormal);
            cx e1, e2;
            convert_to_sp(r, normal, cc.E, e1, e2);
            double cosTheta = dotv(normal, r.d);
            v3 ctn = mulvs(normal, cosTheta);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            ch[0].d = subv(r.d, mulvs(ctn, 2));
            ch[0].n = r.n;
            ch[0].e1 = mkc(-e1.x, -e1.y);
            ch[0].e2 = e2;
            ch[0].len = INF;
            ch[0].type = r.type | RP_REFL_RAY;
            return 1;
        }
        case RP_MAT_PARTIAL:               // cmaterials.pyx:344-397
        case RP_MAT_LINEAR_POLARISING: {   // cmaterials.pyx:404-455
            v3 normal = normv_fast(onormal);
            v3 ind = normv_fast(r.d);
            cx e1, e2;
            convert_to_sp(r, normal, cc.E, e1, e2);
            double cosTheta = dotv(normal, ind);
            v3 ctn = mulvs(normal, cosTheta);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            ch[0].d = subv(ind, mulvs(ctn, 2.0));
            ch[1].d = ind;
            ch[0].n = r.n;
            ch[1].n = r.n;
            if (m.type == RP_MAT_PARTIAL) {
                double R = sqrt(m.p[0]);
                double T = sqrt(1.0 - m.p[0]);
                ch[0].e1 = cmuls(e1, R);
                ch[0].e2 = cmuls(e2, R);
                ch[1].e1 = cmuls(e1, T);
                ch[1].e2 = cmuls(e2, T);
            } else {
                ch[0].e1 = e1;
                ch[0].e2 = mkc(0.0, 0.0);
                ch[1].e1 = mkc(0.0, 0.0);
                ch[1].e2 = e2;
            }
            ch[0].len = INF;
            ch[1].len = INF;
            ch[0].type = r.type | RP_REFL_RAY;
            ch[1].type = r.type & ~RP_REFL_RAY;
            return 2;
        }
        case RP_MAT_WAVEPLATE: {  // cmaterials.pyx:527-551
            v3 normal = normv_fast(onormal);
            v3 ind = normv_fast(r.d);
            cx e1, e2;
            convert_to_sp(r, mkv(m.p[2], m.p[3], m.p[4]), cc.E, e1, e2);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            ch[0].d = ind;
            ch[0].n = r.n;
            // apply_retardance_c, cmaterials.pyx:496-503
            ch[0].e1 = mkc((e1.x * m.p[0]) - (e1.y * m.p[1]), (e1.y * m.p[0]) + (e1.x * m.p[1]));
            ch[0].e2 = e2;
            ch[0].len = INF;
            ch[0].type = r.type & ~RP_REFL_RAY;
            return 1;
        }
        case RP_MAT_DIELECTRIC: {  // cmaterials.pyx:589-680
            v3 normal = normv_fast(onormal);
            v3 ind = normv_fast(r.d);
            cx e1, e2;
            convert_to_sp(r, normal, cc.E, e1, e2);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            double cosTheta = dotv(normal, ind);
            double cos1 = fabs(cosTheta);
            double n1, n2, flip;
            if (cosTheta < 0.0) {
                n1 = m.n_outside[0];
                n2 = m.n_inside[0];
                ch[0].n = mkc(m.n_inside[0], m.n_inside[1]);
                flip = 1;
            } else {
                n1 = m.n_inside[0];
                n2 = m.n_outside[0];
                ch[0].n = mkc(m.n_outside[0], m.n_outside[1]);
                flip = -1;
            }
            double q = n2 / n1;
            double N2 = q * q;
            double N2_sin2 = ((cosTheta * cosTheta) + (N2 - 1.0));
            v3 ctn = mulvs(normal, cosTheta);
            ch[0].len = INF;
            if (N2_sin2 < 0.0) {
                ch[0].d = subv(ind, mulvs(ctn, 2));
                ch[0].e1 = mkc(e1.x * -1, e1.y * -1);
                ch[0].e2 = mkc(e2.x * -1, e2.y * -1);
                ch[0].type = r.type | RP_REFL_RAY;
            } else {
                v3 tangent = subv(ind, ctn);
                v3 tg2 = mulvs(tangent, (n1 / n2));
                double tan_mag_sq = magsq(tg2);
                double c2 = sqrt((1.0 - tan_mag_sq));
                v3 transmitted = subv(tg2, mulvs(normal, (c2 * flip)));
                double cos2 = fabs(dotv(transmitted, normal));
                double Two_n1_cos1 = (2 * n1) * cos1;
                double aspect = (sqrt((cos2 / cos1)) * Two_n1_cos1);
                double T_p = (aspect / ((n2 * cos1) + (n1 * cos2)));
                double T_s = (aspect / ((n2 * cos2) + (n1 * cos1)));
                ch[0].d = transmitted;
                ch[0].e1 = mkc(e1.x * T_s, e1.y * T_s);
                ch[0].e2 = mkc(e2.x * T_p, e2.y * T_p);
                ch[0].type = r.type & ~RP_REFL_RAY;
            }
            return 1;
        }
        case RP_MAT_FULL_DIELECTRIC:
        case RP_MAT_FULL_DIELECTRIC_DISPERSIVE: {  // cmaterials.pyx:756-872, 897-1013
            v3 normal = normv_fast(onormal);
            v3 ind = normv_fast(r.d);
            cx E1, E2;
            convert_to_sp(r, normal, cc.E, E1, E2);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            double cosTheta = dotv(normal, ind);
            double cos1 = fabs(cosTheta);
            double sin1 = sqrt(fabs(1 - cos1 * cos1));
            cx n1, n2;
            double flip;
            bool out_to_in = cosTheta < 0.0;
            if (m.type == RP_MAT_FULL_DIELECTRIC) {
                cx ni = mkc(m.n_inside[0], m.n_inside[1]), no = mkc(m.n_outside[0], m.n_outside[1]);
                n1 = out_to_in ? no : ni;
                n2 = out_to_in ? ni : no;
            } else {
                long long w = (long long)r.wl;
                if (w >= S.n_wl) {  // the reference indexes its n tables unchecked here
                    atomicOr(err, ERR_WAVELENGTH);
                    return 0;
                }
                n1 = S.ntab[(long long)(out_to_in ? m.curve_outside : m.curve_inside) * S.n_wl + w];
                n2 = S.ntab[(long long)(out_to_in ? m.curve_inside : m.curve_outside) * S.n_wl + w];
            }
            flip = out_to_in ? 1 : -1;
            cx sin2 = cdiv(cmuls(n1, sin1), n2);
            cx cos2 = csqrt_(csub(mkc(1.0, 0.0), cmul(sin2, sin2)));
            v3 ctn = mulvs(normal, cosTheta);
            double P_in = n1.x * (((E1.x * E1.x + E1.y * E1.y) + E2.x * E2.x) + E2.y * E2.y);
            if (P_in == 0.0) return 0;
            cx n2c1 = cmuls(n2, cos1), n1c2 = cmul(n1, cos2);
            cx n2c2 = cmul(n2, cos2), n1c1 = cmuls(n1, cos1);
            cx den_p = cadd(n2c1, n1c2), den_s = cadd(n2c2, n1c1);
            cx R_p = cdiv(mkc(-(n2c1.x - n1c2.x), -(n2c1.y - n1c2.y)), den_p);
            cx R_s = cdiv(mkc(-(n2c2.x - n1c1.x), -(n2c2.y - n1c1.y)), den_s);
            R_s = cmul(R_s, E1);
            R_p = cmul(R_p, E2);
            int nc = 0;
            if (((n1.x * (cabs2_(R_s) + cabs2_(R_p))) / P_in) > m.reflection_threshold) {
                ch[0].d = subv(ind, mulvs(ctn, 2.0));
                ch[0].len = INF;
                ch[0].e1 = R_s;
                ch[0].e2 = mkc(-R_p.x, -R_p.y);
                ch[0].n = n1;
                ch[0].type = r.type | RP_REFL_RAY;
                nc = 1;
            }
            v3 tangent = subv(ind, ctn);
            v3 tg2 = mulvs(tangent, n1.x / n2.x);
            double tan_mag_sq = magsq(tg2);
            double c2 = sqrt(1 - tan_mag_sq);
            v3 transmitted = subv(tg2, mulvs(normal, (c2 * flip)));
            double aspect = sqrt(cos2.x / cos1);
            cx num = cmuls(cmuls(n1, 2.0 * cos1), aspect);
            cx T_p = cmul(cdiv(num, den_p), E2);
            cx T_s = cmul(cdiv(num, den_s), E1);
            if (((n2.x * (cabs2_(T_s) + cabs2_(T_p))) / P_in) > m.transmission_threshold) {
                ch[nc].d = transmitted;
                ch[nc].len = INF;
                ch[nc].e1 = T_s;
                ch[nc].e2 = T_p;
                ch[nc].n = n2;
                ch[nc].type = r.type & ~RP_REFL_RAY;
                nc++;
            }
            return nc;
        }
        case RP_MAT_SINGLE_LAYER_COATED:
        case RP_MAT_COATED_DISPERSIVE:
            return coated_children(S, m, r, point, onormal, cc, ch, err);
        case RP_MAT_DIFFRACTION_GRATING: {  // cmaterials.pyx:1474-1543
            const long long w = (long long)r.wl;
            if (w >= S.n_wl) {
                atomicOr(err, ERR_WAVELENGTH);
                return 0;
            }
            v3 normal = normv_fast(onormal);
            v3 tangent = normv_fast(otangent);  // the grating vector
            v3 tangent2 = crossv(normal, tangent);  // along the lines
            const double wavelen = S.wl[w];
            const double line_spacing = 1000.0 / m.p[0];  // um
            v3 refl = normv_fast(r.d);
            double k_z = dotv(normal, refl), k_y = dotv(tangent2, refl), k_x = dotv(tangent, refl);
            const double sign = k_z < 0.0 ? 1.0 : -1.0;
            const double order = m.p[1];
            k_x = k_x - ((order * wavelen) / (line_spacing * r.n.x));
            k_z = ((1.0 - (k_x * k_x)) - (k_y * k_y));
            if (k_z < 0) return 0;  // evanescent order
            k_z = sign * sqrt(k_z);
            refl = addv(addv(mulvs(tangent, k_x), mulvs(tangent2, k_y)), mulvs(normal, k_z));
            cx e1, e2;
            convert_to_sp(r, normal, cc.E, e1, e2);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            cc.dphase = ((((1000.0 * dotv(subv(mkv(m.p[3], m.p[4], m.p[5]), point), tangent)) * order) * 2.0) *
                         3.141592653589793) / line_spacing;
            const double eff = m.p[2];
            ch[0].d = refl;
            ch[0].n = r.n;
            ch[0].e1 = mkc((-e1.x) * eff, (-e1.y) * eff);
            ch[0].e2 = mkc(e2.x * eff, e2.y * eff);
            ch[0].len = r.len;  // the reference keeps the parent's length here
            ch[0].type = r.type | RP_REFL_RAY;
            return 1;
        }
        case RP_MAT_CIRCULAR_APERTURE: {  // cmaterials.pyx:1639-1662
            double r_ = sqrt(magsq(subv(mkv(m.p[4], m.p[5], m.p[6]), point)));
            if (r_ > m.p[0]) return 0;
            double atten = (0.5 + (0.5 * erf(((m.p[1] - r_) / m.p[2]))));
            if (m.p[3] != 0.0) atten = (1.0 - atten);
            v3 normal = normv_fast(onormal);
            cx e1, e2;
            convert_to_sp(r, normal, cc.E, e1, e2);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            ch[0].d = r.d;
            ch[0].n = r.n;
            ch[0].len = r.len;  // the aperture keeps the parent's length
            ch[0].e1 = mkc(e1.x * atten, e1.y * atten);
            ch[0].e2 = mkc(e2.x * atten, e2.y * atten);
            ch[0].type = r.type & ~RP_REFL_RAY;
            return 1;
        }
        case RP_MAT_RECT_APERTURE: {  // cmaterials.pyx:1719-1763
            double width = m.p[4];
            double x = m.p[2] / 2., y = m.p[3] / 2.;
            v3 pp = subv(point, mkv(m.p[6], m.p[7], m.p[8]));
            double px = dotv(pp, otangent);
            double py = dotv(pp, crossv(onormal, otangent));
            if (fabs(px) > m.p[0] / 2.) return 0;
            if (fabs(py) > m.p[1] / 2.) return 0;
            double atten = (0.5 - (0.5 * erf(((px - x) / width))));
            atten = (atten * (0.5 - (0.5 * erf(((-(px + x)) / width)))));
            atten = (atten * (0.5 - (0.5 * erf(((py - y) / width)))));
            atten = (atten * (0.5 - (0.5 * erf(((-(py + y)) / width)))));
            if (m.p[5] != 0.0) atten = (1.0 - atten);
            v3 normal = normv_fast(onormal);
            cx e1, e2;
            convert_to_sp(r, normal, cc.E, e1, e2);
            cc.opl = r.opl + (r.len * r.n.x);
            cc.origin = point;
            cc.normal = normal;
            ch[0].d = r.d;
            ch[0].n = r.n;
            ch[0].len = r.len;
            ch[0].e1 = mkc(e1.x * atten, e1.y * atten);
            ch[0].e2 = mkc(e2.x * atten, e2.y * atten);
            ch[0].type = r.type & ~RP_REFL_RAY;
            return 1;
        }
        default: return 0;
    }
}

// ---- Gausslets ------------------------------------------------------------
// FaceList.intersect_para_c's face test (ctracer.pyx:1914-1926): the face's
// intersect_c with is_base_ray = 0, i.e. without its aperture or shape
// (DistortionFace checks its shape either way, cfaces.pyx:2412).
__device__ __forceinline__ double face_isect_para(const DevScene &S, const rp_face &f, v3 p1, v3 p2, unsigned *err) {
    if (f.type == RP_FACE_DISTORTION) return distortion_isect(S, f, p1, p2, err);
    return face_isect_base(S, f, p1, p2, 0, err);
}

// InterfaceMaterial.eval_parabasal_ray_c of every material type: the
// direction and normal of a parabasal ray that met the face at a point with
// orientation (onormal, otangent), for the child base ray `base` (its
// refractive index, wavelength index and type).  Normalisations are the
// reference's norm_ (three divisions).
__device__ __forceinline__ void eval_parabasal(const DevScene &S, const rp_material &m, cx base_n, unsigned base_wl,
                                               unsigned base_type, v3 direction, v3 onormal, v3 otangent,
                                               v3 &dir_out, v3 &normal_out, unsigned *err) {
    v3 normal = normv(onormal);
    normal_out = normal;
    switch (m.type) {
        case RP_MAT_DIELECTRIC:
        case RP_MAT_FULL_DIELECTRIC:
        case RP_MAT_SINGLE_LAYER_COATED:
        case RP_MAT_COATED_DISPERSIVE: {  // cmaterials.pyx:683-724 and 1393-1433
            double n_in, n_out;
            if (m.type == RP_MAT_COATED_DISPERSIVE) {
                const long long w = (long long)base_wl;
                if (w >= S.n_wl) {
                    atomicOr(err, ERR_WAVELENGTH);
                    dir_out = direction;
                    return;
                }
                n_in = S.ntab[(long long)m.curve_inside * S.n_wl + w].x;
                n_out = S.ntab[(long long)m.curve_outside * S.n_wl + w].x;
            } else {
                n_in = m.n_inside[0];
                n_out = m.n_outside[0];
            }
            direction = normv(direction);
            double cosTheta = dotv(normal, direction);
            v3 cosThetaNormal = mulvs(normal, cosTheta);
            double n1, n2;
            int flip;
            if (cosTheta < 0.0) {
                n1 = n_out;
                n2 = n_in;
                flip = 1;
            } else {
                n1 = n_in;
                n2 = n_out;
                flip = -1;
            }
            if (base_type & RP_REFL_RAY) {
                dir_out = subv(direction, mulvs(cosThetaNormal, 2));
            } else {
                v3 tg2 = mulvs(subv(direction, cosThetaNormal), n1 / n2);
                double c2 = sqrt(1 - magsq(tg2));
                dir_out = subv(tg2, mulvs(normal, c2 * flip));
            }
            return;
        }
        case RP_MAT_DIFFRACTION_GRATING: {  // cmaterials.pyx:1544-1600
            const long long w = (long long)base_wl;
            if (w >= S.n_wl) {
                atomicOr(err, ERR_WAVELENGTH);
                dir_out = direction;
                return;
            }
            v3 tangent = normv(otangent);
            v3 tangent2 = crossv(normal, tangent);
            const double wavelen = S.wl[w];
            const double line_spacing = 1000.0 / m.p[0];
            v3 refl = normv(direction);
            double k_z = dotv(normal, refl), k_y = dotv(tangent2, refl), k_x = dotv(tangent, refl);
            const int sign = k_z < 0.0 ? 1 : -1;
            k_x = k_x - m.p[1] * wavelen / (line_spacing * base_n.x);
            k_z = 1 - (k_x * k_x) - (k_y * k_y);
            k_z = sign * sqrt(k_z);  // NaN for an evanescent order, as in the reference
            refl = mulvs(tangent, k_x);
            refl = addv(refl, mulvs(tangent2, k_y));
            dir_out = addv(refl, mulvs(normal, k_z));
            return;
        }
        default: {  // InterfaceMaterial, ctracer.pyx:1588-1610
            if (base_type & RP_REFL_RAY) {
                double cosTheta = dotv(normal, direction);
                v3 cosThetaNormal = mulvs(normal, cosTheta);
                dir_out = subv(direction, mulvs(cosThetaNormal, 2));
            } else {
                dir_out = direction;
            }
            return;
        }
    }
}

}  // namespace rp
