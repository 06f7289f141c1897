// rp_bounds.h -- conservative bounding boxes of the points where a face can
// report a hit, used to skip faces a ray cannot reach before its current
// nearest hit.  Skipping such a face never changes the result: the nearest
// hit is the face with the smallest distance in (tolerance, length), ties to
// the earlier face, which does not depend on the order faces are tested in.
//
// A box is computed in the face list's local frame from the face parameters
// and mapped to world coordinates; faces whose hit set is not bounded by their
// parameters (DistortionFace returns its last iterate without a surface
// check, cfaces.pyx:2404-2407; a shape containing an inversion) are marked
// "always test".
#pragma once
#include <algorithm>
#include <cmath>

#include "../../include/rp_gb300.h"

namespace rp {

struct Box2 {
    double x0, x1, y0, y1;
    bool bounded;
    double rmax;  // largest distance from the local z axis of an inside point
};

// Bounding box of the inside of a shape program (cshapes.pyx).
inline Box2 shape_box(const rp_scene_desc *d, int prog) {
    const double inf = INFINITY;
    Box2 unb{-inf, inf, -inf, inf, false, inf};
    if (prog < 0) return unb;
    Box2 st[16];
    int sp = 0;
    for (int k = prog; k < d->n_shape_ops; k++) {
        const rp_shape_op &op = d->shape_ops[k];
        if (op.op == RP_SHAPE_END) break;
        if (sp >= 15) return unb;
        switch (op.op) {
            case RP_SHAPE_TRUE: st[sp++] = unb; break;
            case RP_SHAPE_CIRCLE: {
                double r = std::fabs(op.c);
                st[sp++] = Box2{op.a - r, op.a + r, op.b - r, op.b + r, true, std::hypot(op.a, op.b) + r};
                break;
            }
            case RP_SHAPE_RECT: {
                double w = std::fabs(op.c) / 2, h = std::fabs(op.d) / 2;
                st[sp++] = Box2{op.a - w, op.a + w, op.b - h, op.b + h, true,
                                std::hypot(std::fabs(op.a) + w, std::fabs(op.b) + h)};
                break;
            }
            case RP_SHAPE_POLYGON: {
                Box2 b{inf, -inf, inf, -inf, true, 0.0};
                const double *xy = d->aux + op.aux;
                for (int i = 0; i < op.n; i++) {
                    b.rmax = std::max(b.rmax, std::hypot(xy[2 * i], xy[2 * i + 1]));
                    b.x0 = std::min(b.x0, xy[2 * i]);
                    b.x1 = std::max(b.x1, xy[2 * i]);
                    b.y0 = std::min(b.y0, xy[2 * i + 1]);
                    b.y1 = std::max(b.y1, xy[2 * i + 1]);
                }
                st[sp++] = b;
                break;
            }
            case RP_SHAPE_AND: {
                if (sp < 2) return unb;
                Box2 b = st[--sp], a = st[sp - 1];
                st[sp - 1] = Box2{std::max(a.x0, b.x0), std::min(a.x1, b.x1), std::max(a.y0, b.y0),
                                  std::min(a.y1, b.y1), a.bounded || b.bounded, std::min(a.rmax, b.rmax)};
                if (!a.bounded) st[sp - 1] = b;
                if (!b.bounded) st[sp - 1] = a;
                break;
            }
            case RP_SHAPE_OR:
            case RP_SHAPE_XOR: {
                if (sp < 2) return unb;
                Box2 b = st[--sp], a = st[sp - 1];
                if (!a.bounded || !b.bounded) st[sp - 1] = unb;
                else st[sp - 1] = Box2{std::min(a.x0, b.x0), std::max(a.x1, b.x1), std::min(a.y0, b.y0),
                                       std::max(a.y1, b.y1), true, std::max(a.rmax, b.rmax)};
                break;
            }
            case RP_SHAPE_NOT:
                if (sp < 1) return unb;
                st[sp - 1] = unb;
                break;
            default: return unb;
        }
    }
    if (sp != 1) return unb;
    return st[0];
}

// z range of the conic quadric beta z^2 - 2 R z + r^2 = 0 (both sheets) for
// r in [0, rmax] (cfaces.pyx:1695-1747 intersects it and returns either root).
inline bool conic_z_range(double R, double beta, double rmax, double &z0, double &z1) {
    if (!(std::isfinite(R) && std::isfinite(beta) && std::isfinite(rmax))) return false;
    z0 = INFINITY;
    z1 = -INFINITY;
    auto take = [&](double z) {
        z0 = std::min(z0, z);
        z1 = std::max(z1, z);
    };
    if (beta == 0.0) {
        if (R == 0.0) return false;
        take(0.0);
        take(rmax * rmax / (2 * R));
        return true;
    }
    double r2max = rmax * rmax;
    if (beta > 0) r2max = std::min(r2max, R * R / beta);
    for (double r2 : {0.0, r2max}) {
        double disc = R * R - beta * r2;
        if (disc < 0) disc = 0;
        take((R + std::sqrt(disc)) / beta);
        take((R - std::sqrt(disc)) / beta);
    }
    return true;
}

// The same z values by sheet: [a0, a1] for the sheet through the vertex
// (z = 0 at r = 0) and [b0, b1] for the other one, whose points the reference
// also returns when its choice of root falls on them.  Each root is monotonic
// in r^2, so its range lies between its values at r = 0 and r = rmax.  False
// for a paraboloid (one sheet) or a non-finite input.
inline bool conic_sheet_ranges(double R, double beta, double rmax, double &a0, double &a1, double &b0,
                               double &b1) {
    if (!(std::isfinite(R) && std::isfinite(beta) && std::isfinite(rmax)) || beta == 0.0 || R == 0.0) return false;
    double r2max = rmax * rmax;
    if (beta > 0) r2max = std::min(r2max, R * R / beta);
    const double d0 = std::fabs(R), d1 = std::sqrt(std::max(R * R - beta * r2max, 0.0));
    // the vertex sheet takes the root R - sign(R) sqrt(disc): 0 at r = 0
    const double s = R > 0 ? -1.0 : 1.0;
    const double va0 = (R + s * d0) / beta, va1 = (R + s * d1) / beta;
    const double vb0 = (R - s * d0) / beta, vb1 = (R - s * d1) / beta;
    a0 = std::min(va0, va1);
    a1 = std::max(va0, va1);
    b0 = std::min(vb0, vb1);
    b1 = std::max(vb0, vb1);
    return std::isfinite(a0) && std::isfinite(a1) && std::isfinite(b0) && std::isfinite(b1);
}

// Local-frame box of face record `f`; returns false if the face is not bounded.
inline bool face_local_box(const rp_scene_desc *d, const rp_face &f, double lo[3], double hi[3]) {
    const double *p = f.p;
    auto set = [&](double x0, double x1, double y0, double y1, double z0, double z1) {
        lo[0] = x0; hi[0] = x1;
        lo[1] = y0; hi[1] = y1;
        lo[2] = z0; hi[2] = z1;
        for (int k = 0; k < 3; k++)
            if (!(std::isfinite(lo[k]) && std::isfinite(hi[k]) && lo[k] <= hi[k])) return false;
        return true;
    };
    switch (f.type) {
        case RP_FACE_CIRCULAR: {
            double r = std::fabs(p[0]) / 2;
            return set(p[1] - r, p[1] + r, -r, r, p[2], p[2]);
        }
        case RP_FACE_RECTANGULAR:
            return set(p[2] - std::fabs(p[0]) / 2, p[2] + std::fabs(p[0]) / 2, -std::fabs(p[1]) / 2,
                       std::fabs(p[1]) / 2, p[3], p[3]);
        case RP_FACE_ELLIPTICAL_PLANE: {
            double r = std::fabs(p[2]) / 2, dz = (std::fabs(p[0]) + std::fabs(p[1])) * r;
            return set(-r, r, -r, r, -dz, dz);
        }
        case RP_FACE_POLYGON:
        case RP_FACE_ORIENTED_POLYGON: {
            if (f.n_aux0 < 1) return false;
            const double *xy = d->aux + f.aux;
            double b0[3] = {INFINITY, INFINITY, INFINITY}, b1[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int i = 0; i < f.n_aux0; i++) {
                double q[3];
                if (f.type == RP_FACE_POLYGON) {
                    q[0] = xy[2 * i];
                    q[1] = xy[2 * i + 1];
                    q[2] = p[0];
                } else {
                    for (int k = 0; k < 3; k++) q[k] = p[k] + xy[2 * i] * p[6 + k] + xy[2 * i + 1] * p[9 + k];
                }
                for (int k = 0; k < 3; k++) {
                    b0[k] = std::min(b0[k], q[k]);
                    b1[k] = std::max(b1[k], q[k]);
                }
            }
            return set(b0[0], b1[0], b0[1], b1[1], b0[2], b1[2]);
        }
        case RP_FACE_SHAPED_PLANAR: {
            Box2 b = shape_box(d, f.shape);
            if (!b.bounded) return false;
            return set(b.x0, b.x1, b.y0, b.y1, p[0], p[0]);
        }
        case RP_FACE_SPHERICAL:
        case RP_FACE_SHAPED_SPHERICAL: {
            double c, zh, x0, x1, y0, y1, rcirc = INFINITY;
            if (f.type == RP_FACE_SPHERICAL) {
                c = p[1];
                zh = p[2];
                double r = std::fabs(p[0]) / 2;  // circular aperture x^2 + y^2 <= d^2/4
                x0 = -r; x1 = r; y0 = -r; y1 = r;
                rcirc = r;
            } else {
                c = p[0];
                zh = p[1];
                Box2 b = shape_box(d, f.shape);
                if (!b.bounded) return false;
                x0 = b.x0; x1 = b.x1; y0 = b.y0; y1 = b.y1;
            }
            double ac = std::fabs(c);
            x0 = std::max(x0, -ac); x1 = std::min(x1, ac);
            y0 = std::max(y0, -ac); y1 = std::min(y1, ac);
            if (f.type == RP_FACE_SHAPED_SPHERICAL) rcirc = shape_box(d, f.shape).rmax;
            double rx = std::max(std::fabs(x0), std::fabs(x1)), ry = std::max(std::fabs(y0), std::fabs(y1));
            double r2 = std::min(rx * rx + ry * ry, rcirc * rcirc);
            double low = std::sqrt(std::max(c * c - r2, 0.0));  // smallest |z - cz| on the cap
            double cz = zh - c;
            // valid hits lie on the hemisphere z >= cz (c >= 0) or z <= cz (c < 0): cfaces.pyx:460-469
            if (c >= 0) return set(x0, x1, y0, y1, cz + low, cz + ac);
            return set(x0, x1, y0, y1, cz - ac, cz - low);
        }
        case RP_FACE_CONIC: {
            Box2 b = shape_box(d, f.shape);
            if (!b.bounded) return false;
            double z0, z1;
            if (!conic_z_range(-p[0], 1 + p[2], b.rmax, z0, z1)) return false;
            return set(b.x0, b.x1, b.y0, b.y1, z0 + p[1], z1 + p[1]);
        }
        case RP_FACE_ASPHERIC: {
            // converged hits satisfy z = sag(r) (eval_aspheric_impf, cfaces.pyx:1854-1863)
            Box2 b = shape_box(d, f.shape);
            if (!b.bounded) return false;
            double rmax = b.rmax;
            double R = -p[0], beta = 1 + p[2];
            if (R == 0.0 || !std::isfinite(rmax)) return false;
            const int N = 8192;
            auto sag = [&](double r, bool &ok) {
                double r2 = r * r;
                double q = 1 - beta * r2 / (R * R);
                ok = q >= 0;
                double z = r2 / (R * (1 + std::sqrt(std::max(q, 0.0))));
                double pw = r2 * r2;
                for (int k = 0; k < 7; k++) {
                    z += p[3 + k] * pw;
                    pw *= r2;
                }
                return z;
            };
            double z0 = INFINITY, z1 = -INFINITY;
            bool ok = true;
            double prev = sag(0.0, ok);
            for (int i = 1; i <= N && ok; i++) {
                double z = sag(rmax * i / N, ok);
                if (!ok) break;
                // between two samples the smooth sag stays within the pair's range
                // widened by their difference
                double step = std::fabs(z - prev);
                z0 = std::min(z0, std::min(z, prev) - step);
                z1 = std::max(z1, std::max(z, prev) + step);
                prev = z;
            }
            if (!(z0 <= z1)) z0 = z1 = prev;
            return set(b.x0, b.x1, b.y0, b.y1, z0 + p[1], z1 + p[1]);
        }
        case RP_FACE_EXTPOLY: {
            // z = conic(r) + sum E_ij (x/rho)^i (y/rho)^j + z_height (cfaces.pyx:2043-2081)
            Box2 b = shape_box(d, f.shape);
            if (!b.bounded) return false;
            double rx = std::max(std::fabs(b.x0), std::fabs(b.x1)), ry = std::max(std::fabs(b.y0), std::fabs(b.y1));
            double R = p[0], beta = p[1], rho = p[2];
            double z0, z1;
            if (!conic_z_range(R, beta, std::min(b.rmax, std::sqrt(rx * rx + ry * ry)), z0, z1)) return false;
            double bound = 0;
            const double *E = d->aux + f.aux;
            for (int i = 0; i < f.n_aux0; i++)
                for (int j = 0; j < f.n_aux1; j++)
                    bound += std::fabs(E[i * f.n_aux1 + j]) * std::pow(rx / std::fabs(rho), i) *
                             std::pow(ry / std::fabs(rho), j);
            return set(b.x0, b.x1, b.y0, b.y1, z0 - bound + p[3], z1 + bound + p[3]);
        }
        case RP_FACE_ELLIPSOIDAL:  // hits lie strictly inside the block (cfaces.pyx:1362-1376)
            return set(p[2], p[3], p[4], p[5], p[6], p[7]);
        case RP_FACE_SADDLE: {  // z = z_height + sqrt(6) c x y: extremes at the corners of the shape box
            Box2 b = shape_box(d, f.shape);
            if (!b.bounded) return false;
            double A = std::sqrt(6.0) * p[1];
            double z0 = INFINITY, z1 = -INFINITY;
            for (double x : {b.x0, b.x1})
                for (double y : {b.y0, b.y1}) {
                    z0 = std::min(z0, A * x * y);
                    z1 = std::max(z1, A * x * y);
                }
            return set(b.x0, b.x1, b.y0, b.y1, p[0] + z0, p[0] + z1);
        }
        case RP_FACE_CYLINDRICAL: {  // the kept half lies between the vertex and the axis
            Box2 b = shape_box(d, f.shape);
            if (!b.bounded) return false;
            double cz = p[0] - p[1];
            return set(b.x0, b.x1, b.y0, b.y1, std::min(p[0], cz), std::max(p[0], cz));
        }
        case RP_FACE_AXICON: {  // |z - z_height| = |gradient| r with z <= z_height
            Box2 b = shape_box(d, f.shape);
            if (!b.bounded) return false;
            return set(b.x0, b.x1, b.y0, b.y1, p[0] - std::fabs(p[1]) * b.rmax, p[0]);
        }
        default:
            return false;  // DistortionFace, OffAxisParabolicFace and the base Face: always tested
    }
}

// World-space box, padded for the FP32 test in the kernel.  out[0..2] = lo,
// out[3..5] = hi, out[6] = 1 if the face may be skipped, 0 if always tested.
// A DistortionFace with a bounded shape gets out[6] = 2 and, in out[0..3],
// the shape's local x0, x1, y0, y1 (padded): the reference accepts its hit
// only where the point it returns -- always a point of the ray's line in the
// list's frame, converged or not (cfaces.pyx:2372-2407) -- has local (x, y)
// inside the shape, so a ray whose line never passes over that rectangle
// cannot hit it (distortion_line_misses).
inline void world_from_local(const rp_facelist &L, const double lo[3], const double hi[3], float out[8]);

inline void face_world_box(const rp_scene_desc *d, const rp_facelist &L, const rp_face &f, float out[8]) {
    double lo[3], hi[3];
    out[6] = 0.0f;
    out[7] = 0.0f;
    for (int k = 0; k < 6; k++) out[k] = 0.0f;
    if (f.type == RP_FACE_DISTORTION) {
        const Box2 b = shape_box(d, f.shape);
        if (!b.bounded || !std::isfinite(b.x0) || !std::isfinite(b.x1) || !std::isfinite(b.y0) ||
            !std::isfinite(b.y1))
            return;
        const double scale = std::max(std::max(std::fabs(b.x0), std::fabs(b.x1)), std::max(std::fabs(b.y0), std::fabs(b.y1)));
        if (scale > 1e7) return;
        const double pad = 1e-3 + 1e-5 * scale;
        out[0] = (float)(b.x0 - pad);
        out[1] = (float)(b.x1 + pad);
        out[2] = (float)(b.y0 - pad);
        out[3] = (float)(b.y1 + pad);
        out[6] = 2.0f;
        return;
    }
    if (!face_local_box(d, f, lo, hi)) return;
    world_from_local(L, lo, hi, out);
}

// The world box of a local box (its eight corners through the list's
// transform), padded as above, with out[6] = 1.
inline void world_from_local(const rp_facelist &L, const double lo[3], const double hi[3], float out[8]) {
    double w0[3] = {INFINITY, INFINITY, INFINITY}, w1[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; c++) {
        double q[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
        for (int k = 0; k < 3; k++) {
            double w = L.trans.m[3 * k] * q[0] + L.trans.m[3 * k + 1] * q[1] + L.trans.m[3 * k + 2] * q[2] +
                       L.trans.t[k];
            w0[k] = std::min(w0[k], w);
            w1[k] = std::max(w1[k], w);
        }
    }
    double scale = 0;
    for (int k = 0; k < 3; k++) scale = std::max(scale, std::max(std::fabs(w0[k]), std::fabs(w1[k])));
    if (!std::isfinite(scale) || scale > 1e7) return;
    double pad = 1e-3 + 1e-5 * scale;  // far above FP32 rounding of the kernel's test
    for (int k = 0; k < 3; k++) {
        out[k] = (float)(w0[k] - pad);
        out[3 + k] = (float)(w1[k] + pad);
    }
    out[6] = 1.0f;
}

// The boxes of the searches: out[0..7] as face_world_box; for a distortion
// face (flag 2) out[8..15] the x and y rows of its list's world-to-list map;
// for a ConicRevolutionFace, out[0..7] and out[8..15] the world boxes of its
// two sheets' parts over the aperture (out[6] = 3 when the two boxes are set):
// each a thin slab where the union of both can span hundreds of millimetres,
// so a ray that starts between the sheets enters neither.  A face's entry
// distance is the nearer of its boxes' entries.
inline void face_world_boxes(const rp_scene_desc *d, const rp_facelist &L, const rp_face &f, float out[16]) {
    for (int k = 0; k < 16; k++) out[k] = 0.0f;
    face_world_box(d, L, f, out);
    if (out[6] == 2.0f) {
        // a distortion face: rows x and y of its list's world-to-list map
        // (m[0..2], t[0]; m[3..5], t[1]) for the searches' prism entry
        for (int r = 0; r < 2; r++) {
            for (int c = 0; c < 3; c++) out[8 + 4 * r + c] = (float)L.inv_trans.m[3 * r + c];
            out[8 + 4 * r + 3] = (float)L.inv_trans.t[r];
        }
        return;
    }
    if (f.type != RP_FACE_CONIC || out[6] != 1.0f) return;
    const Box2 b = shape_box(d, f.shape);
    double a0, a1, b0, b1;
    if (!b.bounded || !conic_sheet_ranges(-f.p[0], 1 + f.p[2], b.rmax, a0, a1, b0, b1)) return;
    float wa[8] = {0}, wb[8] = {0};
    double lo[3] = {b.x0, b.y0, a0 + f.p[1]}, hi[3] = {b.x1, b.y1, a1 + f.p[1]};
    world_from_local(L, lo, hi, wa);
    lo[2] = b0 + f.p[1];
    hi[2] = b1 + f.p[1];
    world_from_local(L, lo, hi, wb);
    if (wa[6] != 1.0f || wb[6] != 1.0f) return;  // keep the single box
    for (int k = 0; k < 8; k++) {
        out[k] = wa[k];
        out[8 + k] = wb[k];
    }
    out[6] = 3.0f;
}

}  // namespace rp
