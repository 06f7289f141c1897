// rp_lens.cu -- the differentiable sequential lens: an FP64 forward trace of a
// stack of even aspheres and a hand-written adjoint of it.
//
// Forward: every ray crosses the surfaces in order.  Each surface is an
// AsphericFace (cfaces.pyx:1840-2025: conic start, Newton on the sag residual,
// circular aperture), its normal is AsphericFace.compute_normal (1976-2005) and
// the ray is refracted as DielectricMaterial.eval_child_ray (cmaterials.pyx:
// 589-680) does, from the index before the surface to the index after it; the
// image plane is a CircularFace.  These are the plain path's device functions
// with its operation order, so the forward equals rp_trace_rays on the same
// faces bit for bit.  A ray that misses an aperture or is totally internally
// reflected is dropped from the loss.
//
// Loss: the RMS spot radius on the image plane, sqrt(mean |x - xbar|^2) over
// the surviving rays.
//
// Adjoint: nothing of the forward is kept but each ray's image point and
// reached flag.  The backward pass walks the surfaces in reverse and, for
// each, re-traces the ray through the surfaces before it (the forward per
// generation, recomputed; no per-surface state in memory): from a checkpoint
// in registers, the ray in front of the middle surface, for the later
// surfaces, from its input for the earlier ones (n^2/4 + n surface
// evaluations for n surfaces instead of n^2/2), recomputes that surface's hit,
// normal and refraction, and applies the chain rule:
//   hit     h = p + t d with F(h) = z - z_k - s(x^2 + y^2) = 0, so
//           dt = (ds - dz_k - G.dp - t G.dd) / (G.d) with G = grad F
//   normal  n = m / |m|, m = (-2 s' x, -2 s' y, 1)
//   Snell   d' = mu d + (sign(c) w - mu c) n, c = n.d, w = sqrt(1 - mu^2 (1 - c^2))
// with the sag s(u) = u / (R (1 + q)) + A4 u^2 + A6 u^3, q = sqrt(1 - beta u / R^2),
// R = -curvature, beta = 1 + conic.  Gradients are accumulated per block and
// summed on the host in a fixed order.
#include "rp_kernels.cuh"

namespace rp {

#define RP_LENS_BLOCK 128

// Block-wide sum of one double (all threads call it); thread 0 gets the total.
__device__ __forceinline__ double lens_block_sum(double v, double *s_red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < RP_LENS_BLOCK / 32; w++) t += s_red[w];
    return t;
}

// One surface of the forward trace (shared by the forward and the adjoint so
// that both see the same hit): returns false when the ray is lost.
__device__ __forceinline__ bool lens_surface(const LensArgs &L, int k, v3 p, v3 d, v3 &h, v3 &dout, double &t,
                                             unsigned *err) {
    const rp_face &F = L.faces[k];
    v3 pend = addv(p, mulvs(d, L.max_len));
    double dist = face_isect_base(L.S, F, p, pend, 1, err);
    if (!(F.tolerance < dist)) return false;
    t = dist;
    h = addv(p, mulvs(d, dist));
    // DielectricMaterial, n1 -> n2 along the trace (cmaterials.pyx:589-680)
    v3 normal = normv_fast(face_normal_base(L.S, F, h));
    v3 ind = normv_fast(d);
    double cosTheta = dotv(normal, ind);
    double n1 = L.nidx[k], n2 = L.nidx[k + 1];
    double flip = cosTheta < 0.0 ? 1.0 : -1.0;
    double q = n2 / n1;
    double N2 = q * q;
    double N2_sin2 = ((cosTheta * cosTheta) + (N2 - 1.0));
    if (N2_sin2 < 0.0) return false;  // total internal reflection leaves the lens
    v3 ctn = mulvs(normal, cosTheta);
    v3 tg2 = mulvs(subv(ind, ctn), (n1 / n2));
    double c2 = sqrt((1.0 - magsq(tg2)));
    dout = subv(tg2, mulvs(normal, (c2 * flip)));
    return true;
}

__global__ void __launch_bounds__(RP_LENS_BLOCK) lens_forward_kernel(LensArgs L) {
    __shared__ double s_red[RP_LENS_BLOCK / 32];
    const unsigned long long i = (unsigned long long)blockIdx.x * RP_LENS_BLOCK + threadIdx.x;
    double cnt = 0.0, sx = 0.0, sy = 0.0;
    if (i < L.n) {
        v3 p = mkv(L.in.ox[i], L.in.oy[i], L.in.oz[i]);
        v3 d = mkv(L.in.dx[i], L.in.dy[i], L.in.dz[i]);
        bool ok = true;
        for (int k = 0; k < L.n_surf; k++) {
            if (!ok) continue;
            v3 h, dn;
            double t;
            ok = lens_surface(L, k, p, d, h, dn, t, L.err);
            if (ok) {
                p = h;
                d = dn;
            }
        }
        double x = 0.0, y = 0.0;
        if (ok) {
            // image plane: CircularFace (cfaces.pyx:147-175)
            const rp_face &F = L.faces[L.n_surf];
            double dist = face_isect_base(L.S, F, p, addv(p, mulvs(d, L.max_len)), 1, L.err);
            ok = F.tolerance < dist;
            if (ok) {
                v3 h = addv(p, mulvs(d, dist));
                x = h.x;
                y = h.y;
            }
        }
        L.img[2 * i] = x;
        L.img[2 * i + 1] = y;
        L.valid[i] = ok ? 1 : 0;
        if (ok) {
            cnt = 1.0;
            sx = x;
            sy = y;
        }
    }
    cnt = lens_block_sum(cnt, s_red);
    sx = lens_block_sum(sx, s_red);
    sy = lens_block_sum(sy, s_red);
    if (threadIdx.x == 0) {
        L.part[3 * blockIdx.x] = cnt;
        L.part[3 * blockIdx.x + 1] = sx;
        L.part[3 * blockIdx.x + 2] = sy;
    }
}

__global__ void __launch_bounds__(RP_LENS_BLOCK) lens_spread_kernel(LensArgs L) {
    __shared__ double s_red[RP_LENS_BLOCK / 32];
    const unsigned long long i = (unsigned long long)blockIdx.x * RP_LENS_BLOCK + threadIdx.x;
    double v = 0.0;
    if (i < L.n && L.valid[i]) {
        double dx = L.img[2 * i] - L.xm, dy = L.img[2 * i + 1] - L.ym;
        v = dx * dx + dy * dy;
    }
    v = lens_block_sum(v, s_red);
    if (threadIdx.x == 0) L.part[blockIdx.x] = v;
}

// Sag and its derivatives at u = x^2 + y^2 (R = -curvature, beta = 1 + conic).
struct SagD {
    double s1, s2;                 // ds/du, d2s/du2
    double sR, sB, sA4, sA6;       // ds/dR, ds/dbeta, ds/dA4, ds/dA6
    double s1R, s1B, s1A4, s1A6;   // d(ds/du)/dR, ... for the normal
};
__device__ __forceinline__ SagD sag_derivs(double u, double R, double beta, double A4, double A6) {
    SagD g;
    const double R2 = R * R, q = sqrt(1.0 - beta * u / R2), q1 = 1.0 + q;
    const double R3 = R2 * R, q3 = q * q * q;
    g.s1 = 1.0 / (2.0 * R * q) + 2.0 * A4 * u + 3.0 * A6 * u * u;
    g.s2 = beta / (4.0 * R3 * q3) + 2.0 * A4 + 6.0 * A6 * u;
    g.sR = -u / (R2 * q1) - beta * u * u / (R2 * R2 * q * q1 * q1);
    g.sB = u * u / (2.0 * R3 * q * q1 * q1);
    g.sA4 = u * u;
    g.sA6 = u * u * u;
    g.s1R = -1.0 / (2.0 * R2 * q) - beta * u / (2.0 * R2 * R2 * q3);
    g.s1B = u / (4.0 * R3 * q3);
    g.s1A4 = 2.0 * u;
    g.s1A6 = 3.0 * u * u;
    return g;
}

// The ray i in front of surface k (k = n_surf: in front of the image plane):
// its input re-traced through surfaces 0 .. k-1 with the forward's arithmetic.
// Only called for rays the forward kept, which pass every surface again.
// From surface j0 with the ray (p, d) in front of it (j0 = 0: the input).
__device__ __forceinline__ void lens_prefix_from(const LensArgs &L, int j0, int k, v3 &p, v3 &d) {
    for (int j = j0; j < k; j++) {
        v3 h, dn;
        double t;
        if (lens_surface(L, j, p, d, h, dn, t, L.err)) {
            p = h;
            d = dn;
        }
    }
}

__device__ __forceinline__ void lens_prefix(const LensArgs &L, unsigned long long i, int k, v3 &p, v3 &d) {
    p = mkv(L.in.ox[i], L.in.oy[i], L.in.oz[i]);
    d = mkv(L.in.dx[i], L.in.dy[i], L.in.dz[i]);
    for (int j = 0; j < k; j++) {
        v3 h, dn;
        double t;
        if (lens_surface(L, j, p, d, h, dn, t, L.err)) {
            p = h;
            d = dn;
        }
    }
}

// Per ray: the adjoint of the loss through the image plane and every surface
// in reverse.  gpart[block][5 * k + j] receives the block's sum of dL/dR,
// dL/dbeta, dL/dA4, dL/dA6, dL/dz_k for surface k, and gpart[block][5 n] dL/dz_image.
__global__ void __launch_bounds__(RP_LENS_BLOCK) lens_backward_kernel(LensArgs L) {
    __shared__ double s_red[RP_LENS_BLOCK / 32];
    const unsigned long long i = (unsigned long long)blockIdx.x * RP_LENS_BLOCK + threadIdx.x;
    const int np = 5 * L.n_surf + 1;
    double *out = L.gpart + (size_t)blockIdx.x * np;
    const bool ok = i < L.n && L.valid[i];
    v3 hb = mkv(0, 0, 0), db = mkv(0, 0, 0);
    double zimg_b = 0.0;
    // one checkpoint, in registers: the ray in front of the middle surface,
    // from which the prefixes of the later surfaces are re-traced (the same
    // arithmetic as from the input, so the same states); the earlier ones
    // start from the input
    const int km = L.n_surf / 2;
    v3 pm = mkv(0, 0, 0), dm = mkv(0, 0, 1);
    if (ok) lens_prefix(L, i, km, pm, dm);
    if (ok) {
        // image plane z = z_img: h = p + t d, t = (z_img - p_z) / d_z
        const int k = L.n_surf;
        v3 p = pm, d = dm;
        lens_prefix_from(L, km, k, p, d);
        const double zi = L.faces[k].p[2];
        const double t = (zi - p.z) / d.z;
        v3 h = addv(p, mulvs(d, t));
        v3 hbar = mkv((h.x - L.xm) * L.scale, (h.y - L.ym) * L.scale, 0.0);
        const double tb = dotv(hbar, d);
        hb = mkv(hbar.x, hbar.y, hbar.z - tb / d.z);
        db = mkv(t * hbar.x, t * hbar.y, t * hbar.z - t * tb / d.z);
        zimg_b = tb / d.z;
    }
    double v = lens_block_sum(zimg_b, s_red);
    if (threadIdx.x == 0) out[5 * L.n_surf] = v;
    for (int k = L.n_surf - 1; k >= 0; k--) {
        double gR = 0.0, gB = 0.0, gA4 = 0.0, gA6 = 0.0, gZ = 0.0;
        if (ok) {
            v3 p, d;
            if (k >= km) {
                p = pm;
                d = dm;
                lens_prefix_from(L, km, k, p, d);
            } else {
                lens_prefix(L, i, k, p, d);
            }
            v3 h, dn;
            double t = 0.0;
            lens_surface(L, k, p, d, h, dn, t, L.err);  // the forward kept this ray, so it hits again
            const rp_face &F = L.faces[k];
            const double R = -F.p[0], beta = 1.0 + F.p[2], A4 = F.p[3], A6 = F.p[4];
            const double u = h.x * h.x + h.y * h.y;
            const SagD g = sag_derivs(u, R, beta, A4, A6);
            // normal and refraction, recomputed in the model's terms
            const v3 m = mkv(-2.0 * g.s1 * h.x, -2.0 * g.s1 * h.y, 1.0);
            const double mm = magv(m);
            const v3 n = mulvs(m, 1.0 / mm);
            const double c = dotv(n, d);
            const double mu = L.nidx[k] / L.nidx[k + 1];
            const double w = sqrt(1.0 - mu * mu * (1.0 - c * c));
            const double sg = c < 0.0 ? -1.0 : 1.0;
            const double gam = sg * w - mu * c;
            const double dgdc = sg * mu * mu * c / w - mu;
            // d' = mu d + gam n
            const double sdn = dotv(n, db);
            v3 dbar = addv(mulvs(db, mu), mulvs(n, sdn * dgdc));
            v3 nbar = addv(mulvs(db, gam), mulvs(d, sdn * dgdc));
            // n = m / |m|
            const double nn = dotv(nbar, n);
            const v3 mb = mulvs(subv(nbar, mulvs(n, nn)), 1.0 / mm);
            // m = (-2 s1 x, -2 s1 y, 1), s1 = s'(x^2 + y^2)
            v3 hbar = hb;
            hbar.x += mb.x * (-2.0 * g.s1 - 4.0 * h.x * h.x * g.s2) + mb.y * (-4.0 * h.x * h.y * g.s2);
            hbar.y += mb.x * (-4.0 * h.x * h.y * g.s2) + mb.y * (-2.0 * g.s1 - 4.0 * h.y * h.y * g.s2);
            const double mxy = -2.0 * (h.x * mb.x + h.y * mb.y);
            gR += mxy * g.s1R;
            gB += mxy * g.s1B;
            gA4 += mxy * g.s1A4;
            gA6 += mxy * g.s1A6;
            // h = p + t d with F(h) = z - z_k - s(u) = 0; grad F = m
            const double Gd = dotv(m, d);
            const double tb = dotv(hbar, d);
            const double r = tb / Gd;
            hb = subv(hbar, mulvs(m, r));
            db = addv(dbar, subv(mulvs(hbar, t), mulvs(m, t * r)));
            gR += r * g.sR;
            gB += r * g.sB;
            gA4 += r * g.sA4;
            gA6 += r * g.sA6;
            gZ += r;
        }
        gR = lens_block_sum(gR, s_red);
        gB = lens_block_sum(gB, s_red);
        gA4 = lens_block_sum(gA4, s_red);
        gA6 = lens_block_sum(gA6, s_red);
        gZ = lens_block_sum(gZ, s_red);
        if (threadIdx.x == 0) {
            out[5 * k] = gR;
            out[5 * k + 1] = gB;
            out[5 * k + 2] = gA4;
            out[5 * k + 3] = gA6;
            out[5 * k + 4] = gZ;
        }
    }
}

static unsigned lens_blocks(const LensArgs &L) { return (unsigned)((L.n + RP_LENS_BLOCK - 1) / RP_LENS_BLOCK); }

cudaError_t launch_lens_forward(const LensArgs &L, cudaStream_t st) {
    if (L.n == 0) return cudaSuccess;
    lens_forward_kernel<<<lens_blocks(L), RP_LENS_BLOCK, 0, st>>>(L);
    return cudaGetLastError();
}
cudaError_t launch_lens_spread(const LensArgs &L, cudaStream_t st) {
    if (L.n == 0) return cudaSuccess;
    lens_spread_kernel<<<lens_blocks(L), RP_LENS_BLOCK, 0, st>>>(L);
    return cudaGetLastError();
}
cudaError_t launch_lens_backward(const LensArgs &L, cudaStream_t st) {
    if (L.n == 0) return cudaSuccess;
    lens_backward_kernel<<<lens_blocks(L), RP_LENS_BLOCK, 0, st>>>(L);
    return cudaGetLastError();
}
unsigned lens_block_count(unsigned long long n) { return (unsigned)((n + RP_LENS_BLOCK - 1) / RP_LENS_BLOCK); }

}  // namespace rp
