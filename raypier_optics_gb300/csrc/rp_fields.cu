// rp_fields.cu -- E-field summation over Gaussian modes (raypier/core/cfields.pyx),
// the consumer of traced rays and gausslets: the least-squares mode fit of
// each gausslet (evaluate_modes, 150-234) and the coherent sum of every mode
// at every evaluation point (sum_gaussian_modes with calc_mode_U, 49-147).
// Compiled with --fmad=false, like the tracing kernels.
//
// The sum is points x rays complex exponentials of FP64 arguments (phases of
// 1e4 .. 1e6 rad): one thread per evaluation point accumulates the three
// field components over all modes in the reference's order (ray by ray), the
// block staging the per-mode constants in shared memory one tile at a time.
// The per-mode constants (basis, scaled curvature, determinant, phase at the
// requested time) are computed once per evaluation by a small kernel.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <new>

#include "rp_internal.h"

namespace rp {

// Per-mode constants of sum_gaussian_modes (cfields.pyx:76-100).
#define RP_MODE_WORDS 28
#define RP_FIELD_BLOCK 128
#define RP_FIELD_TILE 32

enum : unsigned { FERR_ZERO_DIV = 1u, FERR_WAVELENGTH = 2u };

// Complex quotient by Smith's method (R. L. Smith, "Algorithm 116: Complex
// division", CACM 5(8), 1962).
__device__ __forceinline__ cx cdiv_smith(cx a, cx b) {
    if (fabs(b.x) < fabs(b.y)) {
        double r = b.x / b.y;
        double den = (b.x * r) + b.y;
        return mkc(((a.x * r) + a.y) / den, ((a.y * r) - a.x) / den);
    }
    double r = b.y / b.x;
    double den = (b.y * r) + b.x;
    return mkc(((a.y * r) + a.x) / den, (a.y - (a.x * r)) / den);
}

__device__ __forceinline__ cx cexp_f(cx z) {
    double e = exp(z.x), s, c;
    sincos(z.y, &s, &c);
    return mkc(e * c, e * s);
}

// evaluate_one_mode (cfields.pyx:150-222).  Returns false on a zero
// denominator, where the reference raises ZeroDivisionError.
__device__ bool eval_one_mode(const double *x, const double *y, const double *dx, const double *dy, int size,
                              double blending, cx *out) {
    double a00 = 0, a01 = 0, a02 = 0, a11 = 0, a12 = 0, a22 = 0, b0 = 0, b1 = 0, b2 = 0;
    for (int i = 0; i < size; i++) {
        double xi2 = x[i] * x[i], yi2 = y[i] * y[i];
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
    double den = ((((((-a00) * a11) * a22) + (a00 * (a12 * a12))) + ((a01 * a01) * a22)) - (((2.0 * a01) * a02) * a12)) +
                 ((a02 * a02) * a11);
    if (den == 0) return false;
    double im0 = (blending * ((((-b0) * ((a11 * a22) - (a12 * a12))) + (b1 * ((a01 * a22) - (a02 * a12)))) -
                              (b2 * ((a01 * a12) - (a02 * a11))))) / den;
    double im1 = ((-blending) * (((b0 * ((a01 * a22) - (a02 * a12))) - (b1 * ((a00 * a22) - (a02 * a02)))) +
                                 (b2 * ((a00 * a12) - (a01 * a02))))) / den;
    double im2 = (blending * ((((-b0) * ((a01 * a12) - (a02 * a11))) + (b1 * ((a00 * a12) - (a01 * a02)))) -
                              (b2 * ((a00 * a11) - (a01 * a01))))) / den;
    a00 = a01 = a02 = a11 = a12 = a22 = b0 = b1 = b2 = 0;
    for (int i = 0; i < size; i++) {
        double xi2 = x[i] * x[i], yi2 = y[i] * y[i];
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
    if (den == 0) return false;
    out[0] = mkc(((((-a12) * b2) + ((a01 * a22) * b1)) + (b0 * (a12 - (a11 * a22)))) / den, im0);
    out[1] = mkc((-((((a00 * a01) * b2) - ((a00 * a22) * b1)) + ((a01 * a22) * b0))) / den, im1);
    out[2] = mkc(((((a00 * a01) * b1) - (a12 * b0)) - (b2 * ((a00 * a11) - a12))) / den, im2);
    return true;
}

// x, y, dx, dy: n rows of `size` (at most 64) samples; modes: n x 3 complex.
__global__ void modes_kernel(const double *x, const double *y, const double *dx, const double *dy,
                             unsigned long long n, int size, double blending, cx *modes, unsigned *err) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long o = i * (unsigned long long)size;
    cx m[3];
    if (!eval_one_mode(x + o, y + o, dx + o, dy + o, size, blending, m)) {
        atomicOr(err, FERR_ZERO_DIV);
        m[0] = m[1] = m[2] = mkc(nan_d(), nan_d());
    }
    modes[3 * i] = m[0];
    modes[3 * i + 1] = m[1];
    modes[3 * i + 2] = m[2];
}

// Per-mode constants (cfields.pyx:76-100) for time `time_ps`.
__global__ void mode_constants_kernel(RaySoA r, unsigned long long n, const cx *modes, const double *wl, long long n_wl,
                                      double time_ps, double *P, unsigned *err) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double c = 0.299792458;
    c *= time_ps;
    v3 D = mkv(r.dx[i], r.dy[i], r.dz[i]);
    v3 E = normv(mkv(r.ex[i], r.ey[i], r.ez[i]));
    v3 H = normv(crossv(D, E));
    unsigned w = r.wl[i];
    if ((long long)w >= n_wl) {
        atomicOr(err, FERR_WAVELENGTH);
        w = 0;
    }
    double k = 2000.0 * 3.14159265358979323846 / wl[w];
    cx n_idx = r.n[i];
    double phase = r.phase[i] + (r.opl[i] * k) - (c * k / n_idx.x);
    cx kz = mkc(n_idx.x * k, n_idx.y * k);
    double invk = 2. / kz.x;
    cx A = modes[3 * i], B = modes[3 * i + 1], C = modes[3 * i + 2];
    double inv_root_area = sqrt(sqrt(A.y * C.y - (B.y * B.y)) * (2.0 / 3.14159265358979323846));
    A.y *= invk;
    B.y *= invk;
    C.y *= invk;
    cx detG0 = csub(cmul(A, C), cmul(B, B));
    double *p = P + i * RP_MODE_WORDS;
    p[0] = r.ox[i]; p[1] = r.oy[i]; p[2] = r.oz[i];
    p[3] = E.x; p[4] = E.y; p[5] = E.z;
    p[6] = H.x; p[7] = H.y; p[8] = H.z;
    p[9] = D.x; p[10] = D.y; p[11] = D.z;
    p[12] = A.x; p[13] = A.y; p[14] = B.x; p[15] = B.y; p[16] = C.x; p[17] = C.y;
    p[18] = detG0.x; p[19] = detG0.y;
    p[20] = kz.x; p[21] = kz.y;
    p[22] = phase;
    p[23] = inv_root_area;
    cx e1 = r.e1[i], e2 = r.e2[i];
    p[24] = e1.x; p[25] = e1.y; p[26] = e2.x; p[27] = e2.y;
}

// calc_mode_U (cfields.pyx:120-147) of the mode whose constants are `p`.
__device__ __forceinline__ cx mode_U(const double *p, double px, double py, double pz) {
    v3 pt = mkv(px - p[0], py - p[1], pz - p[2]);
    double x = dotv(pt, mkv(p[3], p[4], p[5]));
    double y = dotv(pt, mkv(p[6], p[7], p[8]));
    double z = dotv(pt, mkv(p[9], p[10], p[11]));
    const cx A = mkc(p[12], p[13]), B = mkc(p[14], p[15]), C = mkc(p[16], p[17]), G = mkc(p[18], p[19]);
    const cx k = mkc(p[20], p[21]);
    cx denom = cmuls(cadd(cadd(mkc(1.0, 0.0), cmuls(cadd(A, C), z)), cmuls(G, z * z)), 2.0);
    cx AA = cdiv_smith(cadd(A, cmuls(G, z)), denom);
    cx CC = cdiv_smith(cadd(C, cmuls(G, z)), denom);
    cx t = cadd(cadd(cadd(mkc(z, 0.0), cmuls(AA, x * x)), cdiv_smith(cmuls(B, 2 * x * y), denom)), cmuls(CC, y * y));
    cx w = cmul(k, t);
    w.x = p[22] + w.x;
    cx U = cexp_f(mkc(-w.y, w.x));  // exp(i w)
    cx q = csub(cmul(cadd(mkc(1.0, 0.0), cmuls(A, z)), cadd(mkc(1.0, 0.0), cmuls(C, z))),
                cmul(cmuls(B, z), cmuls(B, z)));
    U = cdiv_smith(U, csqrt_(mkc(-q.y, q.x)));  // csqrt(q i)
    const double h = 0.70710678118654752440;  // sqrt(i) = (1 + i) / sqrt(2)
    return cmul(U, mkc(p[23] * h, p[23] * h));
}

__global__ void __launch_bounds__(RP_FIELD_BLOCK) field_sum_kernel(const double *P, unsigned long long n_modes,
                                                                   const double *pts, unsigned long long n_pts,
                                                                   cx *E_out) {
    __shared__ double sp[RP_FIELD_TILE * RP_MODE_WORDS];
    const unsigned long long ipt = (unsigned long long)blockIdx.x * RP_FIELD_BLOCK + threadIdx.x;
    const bool active = ipt < n_pts;
    double px = 0, py = 0, pz = 0;
    if (active) {
        px = pts[3 * ipt];
        py = pts[3 * ipt + 1];
        pz = pts[3 * ipt + 2];
    }
    cx o0 = mkc(0, 0), o1 = mkc(0, 0), o2 = mkc(0, 0);
    for (unsigned long long t0 = 0; t0 < n_modes; t0 += RP_FIELD_TILE) {
        const unsigned nt = (unsigned)(n_modes - t0 < RP_FIELD_TILE ? n_modes - t0 : RP_FIELD_TILE);
        __syncthreads();
        for (unsigned k = threadIdx.x; k < nt * RP_MODE_WORDS; k += RP_FIELD_BLOCK) sp[k] = P[t0 * RP_MODE_WORDS + k];
        __syncthreads();
        if (active) {
            for (unsigned j = 0; j < nt; j++) {
                const double *p = sp + j * RP_MODE_WORDS;
                cx U = mode_U(p, px, py, pz);
                cx E1 = cmul(mkc(p[24], p[25]), U), E2 = cmul(mkc(p[26], p[27]), U);
                o0 = cadd(o0, cadd(cmuls(E1, p[3]), cmuls(E2, p[6])));
                o1 = cadd(o1, cadd(cmuls(E1, p[4]), cmuls(E2, p[7])));
                o2 = cadd(o2, cadd(cmuls(E1, p[5]), cmuls(E2, p[8])));
            }
        }
    }
    if (active) {
        E_out[3 * ipt] = o0;
        E_out[3 * ipt + 1] = o1;
        E_out[3 * ipt + 2] = o2;
    }
}

// ---- decomposition helpers (cfields.pyx:232-426) -------------------------------
// calc_mode_curvature (cfields.pyx:232-290): one thread per point; X, Y, Z
// are n x 3 (the local basis x', y', z').
__global__ void mode_curvature_kernel(const double *dx, const double *dy, const double *dx2, const double *dy2,
                                      const double *dxdy, unsigned long long n, double *A, double *B, double *C,
                                      double *X, double *Y, double *Z) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const v3 c = normv(mkv(-dx[i], -dy[i], 1.0));
    const v3 a = normv(crossv(mkv(0.0, 0.0, 1.0), c));
    const v3 b = crossv(c, a);
    X[3 * i] = a.x; X[3 * i + 1] = a.y; X[3 * i + 2] = a.z;
    Y[3 * i] = b.x; Y[3 * i + 1] = b.y; Y[3 * i + 2] = b.z;
    Z[3 * i] = c.x; Z[3 * i + 1] = c.y; Z[3 * i + 2] = c.z;
    const double Fz = c.x * dx[i] + c.y * dy[i] + c.z;
    A[i] = -(a.x * a.x * dx2[i] + 2 * a.x * a.y * dxdy[i] + a.y * a.y * dy2[i]) / Fz;
    B[i] = -(a.x * b.x * dx2[i] + (a.x * b.y + b.x * a.y) * dxdy[i] + a.y * b.y * dy2[i]) / Fz;
    C[i] = -(b.x * b.x * dx2[i] + 2 * b.x * b.y * dxdy[i] + b.y * b.y * dy2[i]) / Fz;
}

// The pair test of build_interaction_matrix (cfields.pyx:376-380): the test
// point relative to the mode's origin, both in the decomposition plane.
__device__ __forceinline__ bool im_in_range(double ox, double oy, double tx, double ty, double ms2) {
    const double px = tx - ox, py = ty - oy;
    return (px * px) + (py * py) <= ms2;
}

struct IMArgs {
    const double *rx, *ry, *tx, *ty, *A, *B, *C, *X, *Y, *Z;
    unsigned long long n, L;
    double ms2, k, impart;
    unsigned *counts;                  // [n] pairs of each mode
    const unsigned long long *offsets; // [n] exclusive prefix of counts
    cx *data;                          // [cap] entries
    unsigned long long *row, *col;
    unsigned long long cap;
};

// One warp per mode i counts the test points within reach, 32 at a time.
__global__ void __launch_bounds__(256) interaction_count_kernel(IMArgs M) {
    const unsigned long long i = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (i >= M.n) return;  // whole warps
    const double ox = M.rx[i], oy = M.ry[i];
    unsigned c = 0;
    for (unsigned long long j = lane; j < M.L; j += 32) c += im_in_range(ox, oy, M.tx[j], M.ty[j], M.ms2) ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) M.counts[i] = c;
}

// One warp per mode i writes its entries from offsets[i] on, in ascending j
// (ballot + prefix popcount), each the calc_mode_U of the mode at the test
// point (cfields.pyx:350-393: curvature as the real parts, the 1/e^2 width
// as the imaginary parts of A and C, detG0 = A C, phase 0, unit area).
__global__ void __launch_bounds__(256) interaction_fill_kernel(IMArgs M) {
    const unsigned long long i = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (i >= M.n) return;  // whole warps
    double p[RP_MODE_WORDS];
    p[0] = M.rx[i]; p[1] = M.ry[i]; p[2] = 0.0;
    p[3] = M.X[3 * i]; p[4] = M.X[3 * i + 1]; p[5] = M.X[3 * i + 2];
    p[6] = M.Y[3 * i]; p[7] = M.Y[3 * i + 1]; p[8] = M.Y[3 * i + 2];
    p[9] = M.Z[3 * i]; p[10] = M.Z[3 * i + 1]; p[11] = M.Z[3 * i + 2];
    const cx A = mkc(M.A[i], M.impart), B = mkc(M.B[i], 0.0), C = mkc(M.C[i], M.impart);
    const cx G = cmul(A, C);
    p[12] = A.x; p[13] = A.y; p[14] = B.x; p[15] = B.y; p[16] = C.x; p[17] = C.y;
    p[18] = G.x; p[19] = G.y;
    p[20] = M.k; p[21] = 0.0;
    p[22] = 0.0;  // phase
    p[23] = 1.0;  // inv_root_area
    unsigned long long pos = M.offsets[i];
    for (unsigned long long j0 = 0; j0 < M.L; j0 += 32) {
        const unsigned long long j = j0 + lane;
        const bool hit = j < M.L && im_in_range(p[0], p[1], M.tx[j], M.ty[j], M.ms2);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const unsigned long long q = pos + __popc(m & ((1u << lane) - 1u));
            if (q < M.cap) {
                M.data[q] = mode_U(p, M.tx[j], M.ty[j], 0.0);
                M.row[q] = i;
                M.col[q] = j;
            }
        }
        pos += __popc(m);
    }
}

// ---- wavefront samples around a base ray ---------------------------------------
// A base ray (origin o, direction d, polarisation E taken as unit, as the
// reference does) spans the frame (E, H = E x d, d).  Each neighbouring ray
// (origin q, direction m) samples the wavefront near the base ray: its offset
// u = q - o expressed as (u.E, u.H) and its slope (m.E, m.H) / (m.d).  A ray of
// a lattice is first carried along m to the plane through o normal to d
// (u + s m, s = -(u.d) / (m.d)); the parabasal rays of a gausslet already
// start in that plane (core/fields.py:83-148 describe both).  The mode fit
// then takes six samples per base ray.  Dot products add x, y, z in that
// order.
__device__ __forceinline__ double dot_xyz(v3 a, v3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }

struct SampleFrame {
    v3 o, d, E, H;
};

__device__ __forceinline__ SampleFrame sample_frame(v3 o, v3 d, v3 E) {
    SampleFrame f;
    f.o = o;
    f.d = d;
    f.E = E;
    f.H = mkv((E.y * d.z) - (E.z * d.y), (E.z * d.x) - (E.x * d.z), (E.x * d.y) - (E.y * d.x));
    return f;
}

__device__ __forceinline__ void wavefront_sample(const SampleFrame &f, v3 q, v3 m, bool to_plane, double *x, double *y,
                                                 double *sx, double *sy) {
    v3 u = mkv(q.x - f.o.x, q.y - f.o.y, q.z - f.o.z);
    const double md = dot_xyz(m, f.d);
    if (to_plane) {
        const double s = (-dot_xyz(u, f.d)) / md;
        u = mkv(u.x + (s * m.x), u.y + (s * m.y), u.z + (s * m.z));
    }
    *x = dot_xyz(u, f.E);
    *y = dot_xyz(u, f.H);
    *sx = dot_xyz(m, f.E) / md;
    *sy = dot_xyz(m, f.H) / md;
}

// Stores sample row r (6 values per array) of x, y, dx, dy at xs[k * rows * 6 + r * 6 + j].
__device__ __forceinline__ void store_samples(double *xs, unsigned long long rows, unsigned long long r, const double *x,
                                              const double *y, const double *sx, const double *sy) {
    const unsigned long long plane = rows * 6;
    for (int j = 0; j < 6; j++) {
        xs[r * 6 + j] = x[j];
        xs[plane + r * 6 + j] = y[j];
        xs[2 * plane + r * 6 + j] = sx[j];
        xs[3 * plane + r * 6 + j] = sy[j];
    }
}

// One gausslet per thread: its six parabasal samples, then (modes != null)
// the mode fit.  xs (or null) receives the samples.
__global__ void gausslet_samples_kernel(RaySoA base, const double *para, unsigned long long cap, unsigned long long n,
                                        double blending, double *xs, cx *modes, unsigned *err) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SampleFrame f = sample_frame(mkv(base.ox[i], base.oy[i], base.oz[i]), mkv(base.dx[i], base.dy[i], base.dz[i]),
                                       mkv(base.ex[i], base.ey[i], base.ez[i]));
    double x[6], y[6], sx[6], sy[6];
    for (int j = 0; j < 6; j++) {
        const double *p = para + (unsigned long long)j * RP_PARA_FIELDS * cap + i;  // field k at p[k * cap]
        wavefront_sample(f, mkv(p[0], p[cap], p[2 * cap]), mkv(p[3 * cap], p[4 * cap], p[5 * cap]), false, &x[j], &y[j],
                         &sx[j], &sy[j]);
    }
    if (xs) store_samples(xs, n, i, x, y, sx, sy);
    if (modes) {
        cx m[3];
        if (!eval_one_mode(x, y, sx, sy, 6, blending, m)) {
            atomicOr(err, FERR_ZERO_DIV);
            m[0] = m[1] = m[2] = mkc(nan_d(), nan_d());
        }
        modes[3 * i] = m[0];
        modes[3 * i + 1] = m[1];
        modes[3 * i + 2] = m[2];
    }
}

// One kept ray per thread (kept[k]: a ray whose six lattice neighbours nb[6
// kept[k] + j] all exist): its samples, the mode fit (modes != null) and the
// copy of its record to row k of dst (dst.ox != null).
__global__ void ray_samples_kernel(RaySoA r, const int *nb, const unsigned long long *kept, unsigned long long n_kept,
                                   double blending, double *xs, cx *modes, RaySoA dst, unsigned *err) {
    const unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_kept) return;
    const unsigned long long i = kept[k];
    const SampleFrame f =
        sample_frame(mkv(r.ox[i], r.oy[i], r.oz[i]), mkv(r.dx[i], r.dy[i], r.dz[i]), mkv(r.ex[i], r.ey[i], r.ez[i]));
    double x[6], y[6], sx[6], sy[6];
    for (int j = 0; j < 6; j++) {
        const unsigned long long q = (unsigned long long)nb[6 * i + j];
        wavefront_sample(f, mkv(r.ox[q], r.oy[q], r.oz[q]), mkv(r.dx[q], r.dy[q], r.dz[q]), true, &x[j], &y[j], &sx[j],
                         &sy[j]);
    }
    if (xs) store_samples(xs, n_kept, k, x, y, sx, sy);
    if (modes) {
        cx m[3];
        if (!eval_one_mode(x, y, sx, sy, 6, blending, m)) {
            atomicOr(err, FERR_ZERO_DIV);
            m[0] = m[1] = m[2] = mkc(nan_d(), nan_d());
        }
        modes[3 * k] = m[0];
        modes[3 * k + 1] = m[1];
        modes[3 * k + 2] = m[2];
    }
    if (dst.ox) {
        dst.ox[k] = r.ox[i]; dst.oy[k] = r.oy[i]; dst.oz[k] = r.oz[i];
        dst.dx[k] = r.dx[i]; dst.dy[k] = r.dy[i]; dst.dz[k] = r.dz[i];
        dst.nx[k] = r.nx[i]; dst.ny[k] = r.ny[i]; dst.nz[k] = r.nz[i];
        dst.ex[k] = r.ex[i]; dst.ey[k] = r.ey[i]; dst.ez[k] = r.ez[i];
        dst.n[k] = r.n[i]; dst.e1[k] = r.e1[i]; dst.e2[k] = r.e2[i];
        dst.len[k] = r.len[i]; dst.phase[k] = r.phase[i]; dst.opl[k] = r.opl[i];
        dst.wl[k] = r.wl[i]; dst.parent[k] = r.parent[i]; dst.endf[k] = r.endf[i];
        dst.ident[k] = r.ident[i]; dst.type[k] = r.type[i];
    }
}

// Every record of src to the same row of dst.
__global__ void copy_rays_kernel(RaySoA s, RaySoA d, unsigned long long n) {
    const unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    d.ox[k] = s.ox[k]; d.oy[k] = s.oy[k]; d.oz[k] = s.oz[k];
    d.dx[k] = s.dx[k]; d.dy[k] = s.dy[k]; d.dz[k] = s.dz[k];
    d.nx[k] = s.nx[k]; d.ny[k] = s.ny[k]; d.nz[k] = s.nz[k];
    d.ex[k] = s.ex[k]; d.ey[k] = s.ey[k]; d.ez[k] = s.ez[k];
    d.n[k] = s.n[k]; d.e1[k] = s.e1[k]; d.e2[k] = s.e2[k];
    d.len[k] = s.len[k]; d.phase[k] = s.phase[k]; d.opl[k] = s.opl[k];
    d.wl[k] = s.wl[k]; d.parent[k] = s.parent[k]; d.endf[k] = s.endf[k];
    d.ident[k] = s.ident[k]; d.type[k] = s.type[k];
}

// Moves each ray back (or on) along its direction to the sphere of `radius`
// about c (core/fields.py:51-77): the nearer-behind root alpha of
// |o - c + alpha d|^2 = radius^2 (the smaller of the two), the optical path
// adjusted by alpha times the real refractive index.  hit[i] = 0 for a ray
// that misses the sphere (left unchanged); *n_miss counts them.
__global__ void sphere_project_kernel(RaySoA r, unsigned long long n, double cx_, double cy_, double cz_, double radius,
                                      unsigned char *hit, unsigned *n_miss) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const v3 u = mkv(r.ox[i] - cx_, r.oy[i] - cy_, r.oz[i] - cz_);
    const v3 d = mkv(r.dx[i], r.dy[i], r.dz[i]);
    const double c = dot_xyz(u, u) - (radius * radius);
    const double b = 2.0 * dot_xyz(d, u);
    const double disc = (b * b) - (4.0 * c);
    if (!(disc >= 0.0)) {
        hit[i] = 0;
        atomicAdd(n_miss, 1u);
        return;
    }
    const double s = sqrt(disc);
    const double r1 = ((-b) + s) / 2.0, r2 = ((-b) - s) / 2.0;
    const double alpha = (r2 < r1 || r2 != r2) ? r2 : r1;  // the smaller root (NaN propagates as numpy's min)
    r.ox[i] = r.ox[i] + (alpha * d.x);
    r.oy[i] = r.oy[i] + (alpha * d.y);
    r.oz[i] = r.oz[i] + (alpha * d.z);
    r.opl[i] = r.opl[i] + (alpha * r.n[i].x);
    hit[i] = 1;
}

// apply_mode_curvature (cfields.pyx:398-426): each parabasal direction of
// gausslet i tilted by the curvature A, B, C in the base ray's (E, E x d)
// frame and renormalised.
__global__ void apply_curvature_kernel(RaySoA base, double *para, unsigned long long cap, unsigned long long n,
                                       const double *A, const double *B, const double *C) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const v3 z = mkv(base.dx[i], base.dy[i], base.dz[i]);
    const v3 x = mkv(base.ex[i], base.ey[i], base.ez[i]);
    const v3 y = crossv(x, z);
    const v3 o = mkv(base.ox[i], base.oy[i], base.oz[i]);
    const double a = A[i], b = B[i], c = C[i];
    for (int j = 0; j < 6; j++) {
        double *f = para + (unsigned long long)j * RP_PARA_FIELDS * cap + i;  // field k at f[k * cap]
        const v3 r = subv(mkv(f[0], f[cap], f[2 * cap]), o);
        const double px = dotv(r, x), py = dotv(r, y);
        v3 shift = mulvs(x, ((-a) * px) - (b * py));
        shift = addv(shift, mulvs(y, ((-c) * py) - (b * px)));
        const v3 d = normv(addv(shift, mkv(f[3 * cap], f[4 * cap], f[5 * cap])));
        f[3 * cap] = d.x;
        f[4 * cap] = d.y;
        f[5 * cap] = d.z;
    }
}

}  // namespace rp

using namespace rp;

// ---- C ABI ----------------------------------------------------------------------
struct rp_field {
    rp_ctx *ctx;
    uint64_t n_modes;
    rp_rays *rays;     // the modes' base rays
    cx *modes;         // n_modes x 3
    double *wl;        // the wavelength table
    int64_t n_wl;
    double *consts;    // n_modes x RP_MODE_WORDS
    unsigned *err;
    size_t modes_bytes, wl_bytes, consts_bytes, err_bytes;
};

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

#define FCK(call)                                              \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return rp__cuda_fail(_e, #call); \
    } while (0)

extern "C" {

int rp_field_evaluate_modes(rp_ctx *ctx, const double *x, const double *y, const double *dx, const double *dy,
                            uint64_t n, int32_t size, double blending, double *modes_out) {
    if (!ctx || (n && (!x || !y || !dx || !dy || !modes_out)) || size < 1 || size > 64) return RP_ERR_INVALID;
    if (n == 0) return RP_OK;
    FCK(cudaSetDevice(ctx->device));
    // every array of the block starts on a 256-byte boundary (the modes are
    // 16-byte double2 stores)
    const size_t in_b = align_up((size_t)n * size * sizeof(double)), out_b = align_up((size_t)n * 3 * sizeof(cx));
    unsigned char *blk = nullptr;
    size_t got = 0;
    int rc = rp__ctx_alloc(ctx, (void **)&blk, 4 * in_b + out_b + 256, &got);
    if (rc) return rc;
    double *d[4];
    for (int k = 0; k < 4; k++) d[k] = (double *)(blk + k * in_b);
    cx *m = (cx *)(blk + 4 * in_b);
    unsigned *err = (unsigned *)(blk + 4 * in_b + out_b);
    const size_t copy_b = (size_t)n * size * sizeof(double);
    const double *h[4] = {x, y, dx, dy};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(d[k], h[k], copy_b, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(unsigned), ctx->stream);
    if (e == cudaSuccess) {
        modes_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(d[0], d[1], d[2], d[3], n, size, blending,
                                                                         m, err);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(modes_out, m, (size_t)n * 3 * sizeof(cx), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_pinned, err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    unsigned ferr = (unsigned)(ctx->h_pinned[0] & 0xffffffffu);
    rp__ctx_free(ctx, blk, got);
    if (e != cudaSuccess) return rp__cuda_fail(e, "rp_field_evaluate_modes");
    if (ferr & FERR_ZERO_DIV) {
        rp__set_error("float division");
        return RP_ERR_INVALID;
    }
    return RP_OK;
}

}  // extern "C"

// A field of n_modes modes with its wavelength table uploaded; the caller
// fills its rays (f->rays->n) and modes.
static int field_alloc(rp_ctx *ctx, uint64_t n_modes, const double *wavelengths, int64_t n_wl, rp_field **out) {
    *out = nullptr;
    rp_field *f = new (std::nothrow) rp_field();
    if (!f) return RP_ERR_NOMEM;
    f->ctx = ctx;
    f->n_modes = n_modes;
    f->n_wl = n_wl;
    int rc = rp_rays_alloc(ctx, n_modes ? n_modes : 1, &f->rays);
    if (rc == RP_OK) rc = rp__ctx_alloc(ctx, (void **)&f->modes, (size_t)(n_modes ? n_modes : 1) * 3 * sizeof(cx),
                                        &f->modes_bytes);
    if (rc == RP_OK) rc = rp__ctx_alloc(ctx, (void **)&f->wl, (size_t)(n_wl ? n_wl : 1) * sizeof(double), &f->wl_bytes);
    if (rc == RP_OK)
        rc = rp__ctx_alloc(ctx, (void **)&f->consts, (size_t)(n_modes ? n_modes : 1) * RP_MODE_WORDS * sizeof(double),
                           &f->consts_bytes);
    if (rc == RP_OK) rc = rp__ctx_alloc(ctx, (void **)&f->err, sizeof(unsigned), &f->err_bytes);
    if (rc == RP_OK && n_wl) {
        cudaError_t e =
            cudaMemcpyAsync(f->wl, wavelengths, (size_t)n_wl * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) rc = rp__cuda_fail(e, "field wavelengths");
    }
    if (rc) {
        rp_field_destroy(f);
        return rc;
    }
    *out = f;
    return RP_OK;
}

// Waits for the stream and turns the field's error word into a status.
static int field_status(rp_field *f, const char *what) {
    rp_ctx *ctx = f->ctx;
    cudaError_t e = cudaMemcpyAsync(ctx->h_pinned, f->err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return rp__cuda_fail(e, what);
    if (ctx->h_pinned[0] & FERR_ZERO_DIV) {
        rp__set_error("float division");
        return RP_ERR_INVALID;
    }
    return RP_OK;
}

// The rays of a lattice whose six neighbour indices are all >= 0 (the rays
// the mode fit keeps, core/fields.py:98); RP_ERR_INVALID when an index names
// no ray of the collection.
static int kept_rows(const int32_t *nb, uint64_t n, std::vector<unsigned long long> &kept) {
    kept.clear();
    for (uint64_t i = 0; i < n; i++) {
        bool all = true;
        for (int j = 0; j < 6; j++) {
            const int32_t v = nb[6 * i + j];
            if (v >= 0 && (uint64_t)v >= n) {
                rp__set_error("neighbour index %d of ray %llu is outside the collection of %llu rays", v,
                              (unsigned long long)i, (unsigned long long)n);
                return RP_ERR_INVALID;
            }
            all = all && v >= 0;
        }
        if (all) kept.push_back(i);
    }
    return RP_OK;
}

// Device copies of a lattice's neighbour table and kept rows, in one block.
struct LatticeDev {
    unsigned char *blk = nullptr;
    size_t got = 0;
    int *nb = nullptr;
    unsigned long long *kept = nullptr;
};

static int lattice_upload(rp_ctx *ctx, const int32_t *nb, uint64_t n, const std::vector<unsigned long long> &kept,
                          LatticeDev &L) {
    const size_t nb_b = align_up((size_t)n * 6 * sizeof(int32_t));
    const size_t k_b = align_up((kept.size() ? kept.size() : 1) * sizeof(unsigned long long));
    int rc = rp__ctx_alloc(ctx, (void **)&L.blk, nb_b + k_b, &L.got);
    if (rc) return rc;
    L.nb = (int *)L.blk;
    L.kept = (unsigned long long *)(L.blk + nb_b);
    cudaError_t e = cudaMemcpyAsync(L.nb, nb, (size_t)n * 6 * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && !kept.empty())
        e = cudaMemcpyAsync(L.kept, kept.data(), kept.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                            ctx->stream);
    // the host vectors must outlive the copies
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return rp__cuda_fail(e, "lattice upload");
    return RP_OK;
}

// Runs sphere_project_kernel on `rays` in place; RP_ERR_INVALID when rays
// miss the sphere and hit_host is null (the caller cannot drop them).
static int project_rays(rp_ctx *ctx, rp_rays *rays, const double *centre, double radius, uint8_t *hit_host) {
    const uint64_t n = rays->n;
    if (n == 0) return RP_OK;
    unsigned char *blk = nullptr;
    size_t got = 0;
    int rc = rp__ctx_alloc(ctx, (void **)&blk, 256 + align_up(n), &got);
    if (rc) return rc;
    unsigned *miss = (unsigned *)blk;
    unsigned char *hit = blk + 256;
    cudaError_t e = cudaMemsetAsync(miss, 0, sizeof(unsigned), ctx->stream);
    if (e == cudaSuccess) {
        sphere_project_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(
            rays->soa, n, centre[0], centre[1], centre[2], radius, hit, miss);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && hit_host) e = cudaMemcpyAsync(hit_host, hit, n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_pinned, miss, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    const unsigned n_miss = (unsigned)(ctx->h_pinned[0] & 0xffffffffu);
    rp__ctx_free(ctx, blk, got);
    if (e != cudaSuccess) return rp__cuda_fail(e, "sphere projection");
    if (n_miss && !hit_host) {
        rp__set_error("%u of %llu rays miss the projection sphere", n_miss, (unsigned long long)n);
        return RP_ERR_INVALID;
    }
    return RP_OK;
}

extern "C" {

int rp_field_create(rp_ctx *ctx, const void *rays, uint64_t n_rays, const double *modes, const double *wavelengths,
                    int64_t n_wl, rp_field **out) {
    if (!ctx || !out || (n_rays && (!rays || !modes)) || n_wl < 0 || (n_wl && !wavelengths)) return RP_ERR_INVALID;
    *out = nullptr;
    FCK(cudaSetDevice(ctx->device));
    rp_field *f = nullptr;
    int rc = field_alloc(ctx, n_rays, wavelengths, n_wl, &f);
    if (rc) return rc;
    rc = rp_rays_upload_aos(f->rays, rays, n_rays);
    if (rc == RP_OK) {
        cudaError_t e = cudaSuccess;
        if (n_rays) e = cudaMemcpyAsync(f->modes, modes, (size_t)n_rays * 3 * sizeof(cx), cudaMemcpyHostToDevice,
                                        ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = rp__cuda_fail(e, "rp_field_create");
    }
    if (rc) {
        rp_field_destroy(f);
        return rc;
    }
    *out = f;
    return RP_OK;
}

int rp_field_create_from_gausslets(rp_gausslets *g, const double *wavelengths, int64_t n_wl, double blending,
                                   rp_field **out) {
    if (!g || !g->base || !out || n_wl < 0 || (n_wl && !wavelengths)) return RP_ERR_INVALID;
    *out = nullptr;
    rp_ctx *ctx = g->ctx;
    FCK(cudaSetDevice(ctx->device));
    const uint64_t n = g->base->n;
    rp_field *f = nullptr;
    int rc = field_alloc(ctx, n, wavelengths, n_wl, &f);
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(f->err, 0, sizeof(unsigned), ctx->stream);
    if (e == cudaSuccess && n) {
        const unsigned blocks = (unsigned)((n + 127) / 128);
        copy_rays_kernel<<<blocks, 128, 0, ctx->stream>>>(g->base->soa, f->rays->soa, n);
        gausslet_samples_kernel<<<blocks, 128, 0, ctx->stream>>>(g->base->soa, g->para, g->cap, n, blending, nullptr,
                                                                f->modes, f->err);
        e = cudaGetLastError();
    }
    f->rays->n = n;
    rc = e != cudaSuccess ? rp__cuda_fail(e, "rp_field_create_from_gausslets")
                          : field_status(f, "rp_field_create_from_gausslets");
    if (rc) {
        rp_field_destroy(f);
        return rc;
    }
    *out = f;
    return RP_OK;
}

int rp_field_create_from_rays(rp_rays *rays, const int32_t *neighbours, const double *centre, double radius,
                              double blending, const double *wavelengths, int64_t n_wl, rp_field **out) {
    if (!rays || !out || (rays->n && !neighbours) || n_wl < 0 || (n_wl && !wavelengths) || (radius != 0.0 && !centre))
        return RP_ERR_INVALID;
    *out = nullptr;
    rp_ctx *ctx = rays->ctx;
    FCK(cudaSetDevice(ctx->device));
    const uint64_t n = rays->n;
    std::vector<unsigned long long> kept;
    int rc = kept_rows(neighbours, n, kept);
    if (rc) return rc;
    const uint64_t nk = kept.size();
    LatticeDev L;
    rp_rays *proj = nullptr;
    rp_field *f = nullptr;
    rc = lattice_upload(ctx, neighbours, n, kept, L);
    RaySoA src = rays->soa;
    if (rc == RP_OK && radius != 0.0 && n) {  // core/fields.py:201-206: a non-zero radius projects first
        rc = rp_rays_alloc(ctx, n, &proj);
        if (rc == RP_OK) {
            proj->n = n;
            copy_rays_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(rays->soa, proj->soa, n);
            cudaError_t e = cudaGetLastError();
            rc = e != cudaSuccess ? rp__cuda_fail(e, "ray copy") : project_rays(ctx, proj, centre, radius, nullptr);
            src = proj->soa;
        }
    }
    if (rc == RP_OK) rc = field_alloc(ctx, nk, wavelengths, n_wl, &f);
    if (rc == RP_OK) {
        cudaError_t e = cudaMemsetAsync(f->err, 0, sizeof(unsigned), ctx->stream);
        if (e == cudaSuccess && nk) {
            ray_samples_kernel<<<(unsigned)((nk + 127) / 128), 128, 0, ctx->stream>>>(src, L.nb, L.kept, nk, blending,
                                                                                     nullptr, f->modes, f->rays->soa,
                                                                                     f->err);
            e = cudaGetLastError();
        }
        f->rays->n = nk;
        rc = e != cudaSuccess ? rp__cuda_fail(e, "rp_field_create_from_rays") : field_status(f, "rp_field_create_from_rays");
    }
    if (proj) rp_rays_free(proj);
    if (L.blk) rp__ctx_free(ctx, L.blk, L.got);
    if (rc) {
        if (f) rp_field_destroy(f);
        return rc;
    }
    *out = f;
    return RP_OK;
}

int rp_field_download(const rp_field *f, uint64_t *n_modes, void *records, double *modes) {
    if (!f || !n_modes) return RP_ERR_INVALID;
    *n_modes = f->n_modes;
    rp_ctx *ctx = f->ctx;
    FCK(cudaSetDevice(ctx->device));
    if (f->n_modes == 0) return RP_OK;
    if (records) {
        int rc = rp_rays_download_aos(f->rays, records, f->n_modes);
        if (rc) return rc;
    }
    if (modes) {
        FCK(cudaMemcpyAsync(modes, f->modes, (size_t)f->n_modes * 3 * sizeof(cx), cudaMemcpyDeviceToHost, ctx->stream));
        FCK(cudaStreamSynchronize(ctx->stream));
    }
    return RP_OK;
}

// Copies 4 x rows x 6 samples from the device block xs to the four host arrays.
static int download_samples(rp_ctx *ctx, const double *xs, uint64_t rows, double *x, double *y, double *dx,
                            double *dy) {
    const size_t b = (size_t)rows * 6 * sizeof(double);
    double *h[4] = {x, y, dx, dy};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(h[k], xs + (size_t)k * rows * 6, b, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return rp__cuda_fail(e, "sample download");
    return RP_OK;
}

int rp_field_gausslet_samples(rp_gausslets *g, double *x, double *y, double *dx, double *dy) {
    if (!g || !g->base) return RP_ERR_INVALID;
    const uint64_t n = g->base->n;
    if (n && (!x || !y || !dx || !dy)) return RP_ERR_INVALID;
    if (n == 0) return RP_OK;
    rp_ctx *ctx = g->ctx;
    FCK(cudaSetDevice(ctx->device));
    double *xs = nullptr;
    size_t got = 0;
    int rc = rp__ctx_alloc(ctx, (void **)&xs, (size_t)n * 24 * sizeof(double), &got);
    if (rc) return rc;
    gausslet_samples_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(g->base->soa, g->para, g->cap, n, 1.0,
                                                                                xs, nullptr, nullptr);
    cudaError_t e = cudaGetLastError();
    rc = e != cudaSuccess ? rp__cuda_fail(e, "rp_field_gausslet_samples") : download_samples(ctx, xs, n, x, y, dx, dy);
    rp__ctx_free(ctx, xs, got);
    return rc;
}

int rp_field_ray_samples(rp_rays *rays, const int32_t *neighbours, double *x, double *y, double *dx, double *dy,
                         uint64_t *kept_out, uint64_t *n_kept) {
    if (!rays || !n_kept) return RP_ERR_INVALID;
    const uint64_t n = rays->n;
    *n_kept = 0;
    if (n && (!neighbours || !x || !y || !dx || !dy || !kept_out)) return RP_ERR_INVALID;
    rp_ctx *ctx = rays->ctx;
    FCK(cudaSetDevice(ctx->device));
    std::vector<unsigned long long> kept;
    int rc = kept_rows(neighbours, n, kept);
    if (rc) return rc;
    const uint64_t nk = kept.size();
    *n_kept = nk;
    for (uint64_t k = 0; k < nk; k++) kept_out[k] = kept[k];
    if (nk == 0) return RP_OK;
    LatticeDev L;
    rc = lattice_upload(ctx, neighbours, n, kept, L);
    if (rc) return rc;
    double *xs = nullptr;
    size_t got = 0;
    rc = rp__ctx_alloc(ctx, (void **)&xs, (size_t)nk * 24 * sizeof(double), &got);
    if (rc == RP_OK) {
        RaySoA none;
        memset(&none, 0, sizeof none);
        ray_samples_kernel<<<(unsigned)((nk + 127) / 128), 128, 0, ctx->stream>>>(rays->soa, L.nb, L.kept, nk, 1.0, xs,
                                                                                 nullptr, none, nullptr);
        cudaError_t e = cudaGetLastError();
        rc = e != cudaSuccess ? rp__cuda_fail(e, "rp_field_ray_samples") : download_samples(ctx, xs, nk, x, y, dx, dy);
        rp__ctx_free(ctx, xs, got);
    }
    rp__ctx_free(ctx, L.blk, L.got);
    return rc;
}

int rp_rays_project_to_sphere(rp_rays *rays, const double *centre, double radius, uint8_t *hit) {
    if (!rays || !centre || (rays->n && !hit)) return RP_ERR_INVALID;
    rp_ctx *ctx = rays->ctx;
    FCK(cudaSetDevice(ctx->device));
    return project_rays(ctx, rays, centre, radius, hit);
}

int rp_field_destroy(rp_field *f) {
    if (!f) return RP_ERR_INVALID;
    rp_ctx *ctx = f->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (f->rays) rp_rays_free(f->rays);
    if (f->modes) rp__ctx_free(ctx, f->modes, f->modes_bytes);
    if (f->wl) rp__ctx_free(ctx, f->wl, f->wl_bytes);
    if (f->consts) rp__ctx_free(ctx, f->consts, f->consts_bytes);
    if (f->err) rp__ctx_free(ctx, f->err, f->err_bytes);
    delete f;
    return RP_OK;
}

int rp_field_evaluate_device(rp_field *f, const double *points_dev, uint64_t n_points, double time_ps, double *E_dev) {
    if (!f || (n_points && (!points_dev || !E_dev))) return RP_ERR_INVALID;
    // the kernel stores E as 16-byte complex pairs and reads 8-byte coordinates
    if (((uintptr_t)E_dev & 15) || ((uintptr_t)points_dev & 7)) return RP_ERR_INVALID;
    rp_ctx *ctx = f->ctx;
    FCK(cudaSetDevice(ctx->device));
    if (n_points == 0) return RP_OK;
    FCK(cudaMemsetAsync(f->err, 0, sizeof(unsigned), ctx->stream));
    if (f->n_modes) {
        mode_constants_kernel<<<(unsigned)((f->n_modes + 127) / 128), 128, 0, ctx->stream>>>(
            f->rays->soa, f->n_modes, f->modes, f->wl, f->n_wl, time_ps, f->consts, f->err);
        FCK(cudaGetLastError());
    }
    field_sum_kernel<<<(unsigned)((n_points + RP_FIELD_BLOCK - 1) / RP_FIELD_BLOCK), RP_FIELD_BLOCK, 0, ctx->stream>>>(
        f->consts, f->n_modes, points_dev, n_points, (cx *)E_dev);
    FCK(cudaGetLastError());
    FCK(cudaMemcpyAsync(ctx->h_pinned, f->err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    FCK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_pinned[0] & FERR_WAVELENGTH) {
        rp__set_error("a ray's wavelength_idx is outside the wavelength table");
        return RP_ERR_INVALID;
    }
    return RP_OK;
}

int rp_field_evaluate(rp_field *f, const double *points, uint64_t n_points, double time_ps, double *E_out) {
    if (!f || (n_points && (!points || !E_out))) return RP_ERR_INVALID;
    rp_ctx *ctx = f->ctx;
    FCK(cudaSetDevice(ctx->device));
    if (n_points == 0) return RP_OK;
    const size_t pb = (size_t)n_points * 3 * sizeof(double), eb = (size_t)n_points * 3 * sizeof(cx);
    unsigned char *blk = nullptr;
    size_t got = 0;
    int rc = rp__ctx_alloc(ctx, (void **)&blk, align_up(pb) + eb, &got);
    if (rc) return rc;
    double *dp = (double *)blk, *de = (double *)(blk + align_up(pb));  // E on a 256-byte boundary
    cudaError_t e = cudaMemcpyAsync(dp, points, pb, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        rp__ctx_free(ctx, blk, got);
        return rp__cuda_fail(e, "rp_field_evaluate");
    }
    rc = rp_field_evaluate_device(f, dp, n_points, time_ps, de);
    if (rc == RP_OK) {
        e = cudaMemcpyAsync(E_out, de, eb, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = rp__cuda_fail(e, "rp_field_evaluate");
    }
    rp__ctx_free(ctx, blk, got);
    return rc;
}

int rp_field_mode_curvature(rp_ctx *ctx, const double *dx, const double *dy, const double *dx2, const double *dy2,
                            const double *dxdy, uint64_t n, double *A, double *B, double *C, double *X, double *Y,
                            double *Z) {
    if (!ctx || (n && (!dx || !dy || !dx2 || !dy2 || !dxdy || !A || !B || !C || !X || !Y || !Z)))
        return RP_ERR_INVALID;
    if (n == 0) return RP_OK;
    FCK(cudaSetDevice(ctx->device));
    const size_t v = align_up((size_t)n * sizeof(double)), v3b = align_up((size_t)n * 3 * sizeof(double));
    unsigned char *blk = nullptr;
    size_t got = 0;
    int rc = rp__ctx_alloc(ctx, (void **)&blk, 8 * v + 3 * v3b, &got);
    if (rc) return rc;
    double *d[8];
    for (int k = 0; k < 8; k++) d[k] = (double *)(blk + k * v);
    double *dX = (double *)(blk + 8 * v), *dY = (double *)(blk + 8 * v + v3b), *dZ = (double *)(blk + 8 * v + 2 * v3b);
    const double *h[5] = {dx, dy, dx2, dy2, dxdy};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 5 && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(d[k], h[k], (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        mode_curvature_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(d[0], d[1], d[2], d[3], d[4], n,
                                                                                   d[5], d[6], d[7], dX, dY, dZ);
        e = cudaGetLastError();
    }
    double *out[6] = {A, B, C, X, Y, Z};
    const double *src[6] = {d[5], d[6], d[7], dX, dY, dZ};
    for (int k = 0; k < 6 && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(out[k], src[k], (size_t)n * (k < 3 ? 1 : 3) * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    rp__ctx_free(ctx, blk, got);
    if (e != cudaSuccess) return rp__cuda_fail(e, "rp_field_mode_curvature");
    return RP_OK;
}

int rp_field_interaction_matrix(rp_ctx *ctx, const double *rx, const double *ry, uint64_t n_modes, const double *tx,
                                const double *ty, uint64_t n_points, const double *A, const double *B,
                                const double *C, const double *X, const double *Y, const double *Z,
                                double wavelength, double spacing, double max_spacing, double blending, uint64_t cap,
                                uint64_t *count, double *data, uint64_t *row, uint64_t *col) {
    if (!ctx || !count || (n_modes && (!rx || !ry || !A || !B || !C || !X || !Y || !Z)) || (n_points && (!tx || !ty)))
        return RP_ERR_INVALID;
    if (cap && (!data || !row || !col)) return RP_ERR_INVALID;
    *count = 0;
    if (n_modes == 0 || n_points == 0) return RP_OK;
    FCK(cudaSetDevice(ctx->device));
    const size_t vn = align_up((size_t)n_modes * sizeof(double)), v3n = align_up((size_t)n_modes * 3 * sizeof(double));
    const size_t vl = align_up((size_t)n_points * sizeof(double));
    const size_t cb = align_up((size_t)n_modes * sizeof(unsigned)), ob = align_up((size_t)n_modes * 8);
    const size_t in_bytes = 5 * vn + 3 * v3n + 2 * vl + cb + ob + 256;
    unsigned char *blk = nullptr;
    size_t got = 0;
    int rc = rp__ctx_alloc(ctx, (void **)&blk, in_bytes, &got);
    if (rc) return rc;
    IMArgs M;
    memset(&M, 0, sizeof M);
    unsigned char *q = blk;
    auto take = [&](size_t b) { unsigned char *r = q; q += b; return r; };
    double *drx = (double *)take(vn), *dry = (double *)take(vn), *dA = (double *)take(vn), *dB = (double *)take(vn),
           *dC = (double *)take(vn);
    double *dX = (double *)take(v3n), *dY = (double *)take(v3n), *dZ = (double *)take(v3n);
    double *dtx = (double *)take(vl), *dty = (double *)take(vl);
    M.counts = (unsigned *)take(cb);
    unsigned long long *offs = (unsigned long long *)take(ob);
    unsigned long long *total = (unsigned long long *)take(256);
    struct { double *d; const double *h; size_t b; } up[] = {
        {drx, rx, (size_t)n_modes * 8}, {dry, ry, (size_t)n_modes * 8}, {dA, A, (size_t)n_modes * 8},
        {dB, B, (size_t)n_modes * 8},   {dC, C, (size_t)n_modes * 8},   {dX, X, (size_t)n_modes * 24},
        {dY, Y, (size_t)n_modes * 24},  {dZ, Z, (size_t)n_modes * 24},  {dtx, tx, (size_t)n_points * 8},
        {dty, ty, (size_t)n_points * 8}};
    cudaError_t e = cudaSuccess;
    for (auto &u : up)
        if (e == cudaSuccess) e = cudaMemcpyAsync(u.d, u.h, u.b, cudaMemcpyHostToDevice, ctx->stream);
    M.rx = drx; M.ry = dry; M.A = dA; M.B = dB; M.C = dC; M.X = dX; M.Y = dY; M.Z = dZ; M.tx = dtx; M.ty = dty;
    M.n = n_modes;
    M.L = n_points;
    M.ms2 = max_spacing * max_spacing;
    M.k = 2000.0 * 3.14159265358979323846 / wavelength;
    M.impart = 2 * (blending * blending) / (M.k * spacing * spacing);
    M.offsets = offs;
    const unsigned grid = (unsigned)((n_modes * 32 + 255) / 256);
    if (e == cudaSuccess) {
        interaction_count_kernel<<<grid, 256, 0, ctx->stream>>>(M);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_count_scan(M.counts, n_modes, offs, total, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_pinned, total, 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    const uint64_t n_pairs = ctx->h_pinned[0];
    if (e == cudaSuccess) *count = n_pairs;
    if (e == cudaSuccess && n_pairs > cap) {
        rp__ctx_free(ctx, blk, got);
        rp__set_error("%llu matrix entries do not fit %llu", (unsigned long long)n_pairs, (unsigned long long)cap);
        return RP_ERR_CAPACITY;
    }
    unsigned char *ob2 = nullptr;
    size_t got2 = 0;
    const size_t db = align_up((size_t)n_pairs * sizeof(cx)), ib = align_up((size_t)n_pairs * 8);
    if (e == cudaSuccess && n_pairs) {
        rc = rp__ctx_alloc(ctx, (void **)&ob2, db + 2 * ib, &got2);
        if (rc) {
            rp__ctx_free(ctx, blk, got);
            return rc;
        }
        M.data = (cx *)ob2;
        M.row = (unsigned long long *)(ob2 + db);
        M.col = (unsigned long long *)(ob2 + db + ib);
        M.cap = n_pairs;
        interaction_fill_kernel<<<grid, 256, 0, ctx->stream>>>(M);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(data, M.data, (size_t)n_pairs * sizeof(cx), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(row, M.row, (size_t)n_pairs * 8, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(col, M.col, (size_t)n_pairs * 8, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    if (ob2) rp__ctx_free(ctx, ob2, got2);
    rp__ctx_free(ctx, blk, got);
    if (e != cudaSuccess) return rp__cuda_fail(e, "rp_field_interaction_matrix");
    return RP_OK;
}

int rp_field_apply_mode_curvature(rp_gausslets *g, const double *A, const double *B, const double *C) {
    if (!g || !g->base) return RP_ERR_INVALID;
    const uint64_t n = g->base->n;
    if (n && (!A || !B || !C)) return RP_ERR_INVALID;
    if (n == 0) return RP_OK;
    rp_ctx *ctx = g->ctx;
    FCK(cudaSetDevice(ctx->device));
    const size_t v = align_up((size_t)n * sizeof(double));
    unsigned char *blk = nullptr;
    size_t got = 0;
    int rc = rp__ctx_alloc(ctx, (void **)&blk, 3 * v, &got);
    if (rc) return rc;
    double *d[3] = {(double *)blk, (double *)(blk + v), (double *)(blk + 2 * v)};
    const double *h[3] = {A, B, C};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 3 && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(d[k], h[k], (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        apply_curvature_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(g->base->soa, g->para, g->cap, n,
                                                                                    d[0], d[1], d[2]);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    rp__ctx_free(ctx, blk, got);
    if (e != cudaSuccess) return rp__cuda_fail(e, "rp_field_apply_mode_curvature");
    return RP_OK;
}

int rp_field_sum_gaussian_modes(rp_ctx *ctx, const void *rays, uint64_t n_rays, const double *modes,
                                const double *wavelengths, int64_t n_wl, const double *points, uint64_t n_points,
                                double time_ps, double *E_out) {
    rp_field *f = nullptr;
    int rc = rp_field_create(ctx, rays, n_rays, modes, wavelengths, n_wl, &f);
    if (rc) return rc;
    rc = rp_field_evaluate(f, points, n_points, time_ps, E_out);
    rp_field_destroy(f);
    return rc;
}

}  // extern "C"
