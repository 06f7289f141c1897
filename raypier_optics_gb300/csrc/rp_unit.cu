// rp_unit.cu -- single-plugin entry points: one face, shape, distortion,
// material or dispersion curve evaluated on the GPU for a batch of
// independent inputs.  They are the device counterparts of the reference's
// Python-visible unit calls (Face.intersect ctracer.pyx:1769-1777,
// Face.compute_normal 1793-1800, Shape.point_inside 1657-1658,
// Distortion.z_offset[_and_gradient] 1703-1729, InterfaceMaterial.eval_child_ray
// 1620-1632, Convert_to_SP cmaterials.pyx:94-101, BaseDispersionCurve.evaluate_n
// 230-239) and use exactly the device functions of the generation kernel.
// Compiled with --fmad=false like the plain path.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "../../include/rp_gb300.h"
#include "rp_kernels.cuh"

using namespace rp;

namespace rp {

__global__ void unit_face_isect(DevScene S, int rec, const double *p1, const double *p2, unsigned long long n,
                                int is_base_ray, double *out, unsigned *err) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 a = mkv(p1[3 * i], p1[3 * i + 1], p1[3 * i + 2]);
    v3 b = mkv(p2[3 * i], p2[3 * i + 1], p2[3 * i + 2]);
    const rp_face &F = S.faces[rec];
    out[i] = (F.type == RP_FACE_DISTORTION) ? distortion_isect(S, F, a, b, err)
                                            : face_isect_base(S, F, a, b, is_base_ray, err);
}

__global__ void unit_face_normal(DevScene S, int rec, const double *p, unsigned long long n, double *out,
                                 unsigned *err) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v3 q = face_normal(S, S.faces[rec], mkv(p[3 * i], p[3 * i + 1], p[3 * i + 2]), err);
    out[3 * i] = q.x;
    out[3 * i + 1] = q.y;
    out[3 * i + 2] = q.z;
}

__global__ void unit_shape(DevScene S, int prog, const double *xy, unsigned long long n, int *out, unsigned *err) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = shape_inside(S, prog, xy[2 * i], xy[2 * i + 1], err);
}

__global__ void unit_distortion(DevScene S, int d, const double *xy, unsigned long long n, double *out,
                                unsigned *err) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const rp_distortion &D = S.dists[d];
    v3 g = dist_zg(S, D, xy[2 * i], xy[2 * i + 1], err);
    out[4 * i] = g.x;
    out[4 * i + 1] = g.y;
    out[4 * i + 2] = g.z;
    out[4 * i + 3] = dist_z(S, D, xy[2 * i], xy[2 * i + 1], err);
}

// Reads / writes the packed 188-byte record through 4-byte words.
__device__ __forceinline__ double rd(const unsigned char *r, int off) {
    const unsigned *w = reinterpret_cast<const unsigned *>(r + off);
    return __hiloint2double((int)w[1], (int)w[0]);
}
__device__ __forceinline__ void wr(unsigned char *r, int off, double v) {
    unsigned *w = reinterpret_cast<unsigned *>(r + off);
    w[0] = (unsigned)__double2loint(v);
    w[1] = (unsigned)__double2hiint(v);
}
__device__ __forceinline__ unsigned rdu(const unsigned char *r, int off) {
    return *reinterpret_cast<const unsigned *>(r + off);
}
__device__ __forceinline__ void wru(unsigned char *r, int off, unsigned v) {
    *reinterpret_cast<unsigned *>(r + off) = v;
}

static __device__ RayState load_record(const unsigned char *r) {
    RayState s;
    s.o = mkv(rd(r, 0), rd(r, 8), rd(r, 16));
    s.d = mkv(rd(r, 24), rd(r, 32), rd(r, 40));
    s.E = mkv(rd(r, 72), rd(r, 80), rd(r, 88));
    s.n = make_double2(rd(r, 96), rd(r, 104));
    s.e1 = make_double2(rd(r, 112), rd(r, 120));
    s.e2 = make_double2(rd(r, 128), rd(r, 136));
    s.len = rd(r, 144);
    s.phase = rd(r, 152);
    s.opl = rd(r, 160);
    s.wl = rdu(r, 168);
    s.endf = rdu(r, 176);
    s.ident = rdu(r, 180);
    s.type = rdu(r, 184);
    return s;
}

static __device__ void write_child_record(unsigned char *dst, const unsigned char *parent, const ChildCommon &cc,
                                   const Child &ch, unsigned pidx, double phase) {
    for (int k = 0; k < RP_RAY_BYTES / 4; k++)
        reinterpret_cast<unsigned *>(dst)[k] = reinterpret_cast<const unsigned *>(parent)[k];
    wr(dst, 0, cc.origin.x); wr(dst, 8, cc.origin.y); wr(dst, 16, cc.origin.z);
    wr(dst, 24, ch.d.x); wr(dst, 32, ch.d.y); wr(dst, 40, ch.d.z);
    wr(dst, 48, cc.normal.x); wr(dst, 56, cc.normal.y); wr(dst, 64, cc.normal.z);
    wr(dst, 72, cc.E.x); wr(dst, 80, cc.E.y); wr(dst, 88, cc.E.z);
    wr(dst, 96, ch.n.x); wr(dst, 104, ch.n.y);
    wr(dst, 112, ch.e1.x); wr(dst, 120, ch.e1.y);
    wr(dst, 128, ch.e2.x); wr(dst, 136, ch.e2.y);
    wr(dst, 144, ch.len);
    wr(dst, 152, phase + cc.dphase);
    wr(dst, 160, cc.opl);
    wru(dst, 172, pidx);
    wru(dst, 184, ch.type);
}

__global__ void unit_material(DevScene S, int mat, const unsigned char *rays, const unsigned *idx,
                              const double *pts, const double *nrm, const double *tng, unsigned long long n,
                              unsigned char *children, int *n_children, unsigned *err) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned char *rec = rays + i * RP_RAY_BYTES;
    RayState r = load_record(rec);
    ChildCommon cc;
    Child ch[2];
    v3 point = mkv(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    v3 on = mkv(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    v3 ot = mkv(tng[3 * i], tng[3 * i + 1], tng[3 * i + 2]);
    int nc = eval_children(S, S.mats[mat], r, point, on, ot, cc, ch, err);
    for (int k = 0; k < nc; k++)
        write_child_record(children + (2 * i + k) * RP_RAY_BYTES, rec, cc, ch[k], idx[i], r.phase);
    n_children[i] = nc;
}

__global__ void unit_convert_sp(const unsigned char *rays, const double *nrm, unsigned long long n,
                                unsigned char *out) {
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned char *rec = rays + i * RP_RAY_BYTES;
    unsigned char *dst = out + i * RP_RAY_BYTES;
    for (int k = 0; k < RP_RAY_BYTES / 4; k++)
        reinterpret_cast<unsigned *>(dst)[k] = reinterpret_cast<const unsigned *>(rec)[k];
    RayState r = load_record(rec);
    v3 E;
    cx e1, e2;
    convert_to_sp(r, mkv(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]), E, e1, e2);
    wr(dst, 72, E.x); wr(dst, 80, E.y); wr(dst, 88, E.z);
    wr(dst, 112, e1.x); wr(dst, 120, e1.y);
    wr(dst, 128, e2.x); wr(dst, 136, e2.y);
}

}  // namespace rp

// ---- host side ------------------------------------------------------------------
extern "C" int rp__scene_view(rp_scene *s, rp::DevScene *out, cudaStream_t *st, int *device);
extern "C" int rp__ctx_stream(rp_ctx *c, cudaStream_t *st, int *device);
extern "C" int rp__scene_curve(rp_scene *s, const rp_dispersion **dcurve, int *n_curves);

namespace {

// A device staging area for a batch call: copies inputs in, runs, copies out.
struct Batch {
    std::vector<void *> bufs;
    ~Batch() {
        for (void *p : bufs) cudaFree(p);
    }
    void *in(const void *h, size_t bytes, cudaStream_t st, cudaError_t &e) {
        void *d = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&d, bytes ? bytes : 16);
        if (e == cudaSuccess) {
            bufs.push_back(d);
            if (bytes) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
        }
        return d;
    }
    void *out(size_t bytes, cudaStream_t st, cudaError_t &e) {
        void *d = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&d, bytes ? bytes : 16);
        if (e == cudaSuccess) {
            bufs.push_back(d);
            e = cudaMemsetAsync(d, 0, bytes ? bytes : 16, st);
        }
        return d;
    }
};

unsigned grid_of(unsigned long long n) { return (unsigned)((n + 127) / 128); }

int finish(cudaError_t e, cudaStream_t st, unsigned *derr) {
    unsigned herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof herr, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return RP_ERR_CUDA;
    return herr ? RP_ERR_INVALID : RP_OK;
}

}  // namespace

extern "C" {

int rp_face_intersect(rp_scene *s, int32_t rec, const double *p1, const double *p2, uint64_t n, int is_base_ray,
                      double *dist) {
    DevScene S;
    cudaStream_t st;
    int dev;
    if (!s || rp__scene_view(s, &S, &st, &dev) || rec < 0 || rec >= S.n_recs || (n && (!p1 || !p2 || !dist)))
        return RP_ERR_INVALID;
    if (!n) return RP_OK;
    cudaSetDevice(dev);
    cudaError_t e = cudaSuccess;
    Batch b;
    auto *d1 = (const double *)b.in(p1, 24 * n, st, e);
    auto *d2 = (const double *)b.in(p2, 24 * n, st, e);
    auto *dout = (double *)b.out(8 * n, st, e);
    auto *derr = (unsigned *)b.out(4, st, e);
    if (e == cudaSuccess) {
        unit_face_isect<<<grid_of(n), 128, 0, st>>>(S, rec, d1, d2, n, is_base_ray, dout, derr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(dist, dout, 8 * n, cudaMemcpyDeviceToHost, st);
    return finish(e, st, derr);
}

int rp_face_normal(rp_scene *s, int32_t rec, const double *p, uint64_t n, double *normal) {
    DevScene S;
    cudaStream_t st;
    int dev;
    if (!s || rp__scene_view(s, &S, &st, &dev) || rec < 0 || rec >= S.n_recs || (n && (!p || !normal)))
        return RP_ERR_INVALID;
    if (!n) return RP_OK;
    cudaSetDevice(dev);
    cudaError_t e = cudaSuccess;
    Batch b;
    auto *dp = (const double *)b.in(p, 24 * n, st, e);
    auto *dout = (double *)b.out(24 * n, st, e);
    auto *derr = (unsigned *)b.out(4, st, e);
    if (e == cudaSuccess) {
        unit_face_normal<<<grid_of(n), 128, 0, st>>>(S, rec, dp, n, dout, derr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(normal, dout, 24 * n, cudaMemcpyDeviceToHost, st);
    return finish(e, st, derr);
}

int rp_shape_inside(rp_scene *s, int32_t prog, const double *xy, uint64_t n, int32_t *inside) {
    DevScene S;
    cudaStream_t st;
    int dev;
    if (!s || rp__scene_view(s, &S, &st, &dev) || prog >= S.n_shapes || (n && (!xy || !inside)))
        return RP_ERR_INVALID;
    if (!n) return RP_OK;
    cudaSetDevice(dev);
    cudaError_t e = cudaSuccess;
    Batch b;
    auto *dxy = (const double *)b.in(xy, 16 * n, st, e);
    auto *dout = (int *)b.out(4 * n, st, e);
    auto *derr = (unsigned *)b.out(4, st, e);
    if (e == cudaSuccess) {
        unit_shape<<<grid_of(n), 128, 0, st>>>(S, prog, dxy, n, dout, derr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(inside, dout, 4 * n, cudaMemcpyDeviceToHost, st);
    return finish(e, st, derr);
}

int rp_distortion_eval(rp_scene *s, int32_t d, const double *xy, uint64_t n, double *out4) {
    DevScene S;
    cudaStream_t st;
    int dev;
    if (!s || rp__scene_view(s, &S, &st, &dev) || d < 0 || d >= S.n_dists || (n && (!xy || !out4)))
        return RP_ERR_INVALID;
    if (!n) return RP_OK;
    cudaSetDevice(dev);
    cudaError_t e = cudaSuccess;
    Batch b;
    auto *dxy = (const double *)b.in(xy, 16 * n, st, e);
    auto *dout = (double *)b.out(32 * n, st, e);
    auto *derr = (unsigned *)b.out(4, st, e);
    if (e == cudaSuccess) {
        unit_distortion<<<grid_of(n), 128, 0, st>>>(S, d, dxy, n, dout, derr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out4, dout, 32 * n, cudaMemcpyDeviceToHost, st);
    return finish(e, st, derr);
}

int rp_material_eval(rp_scene *s, int32_t mat, const void *rays, const uint32_t *idx, const double *points,
                     const double *normals, const double *tangents, uint64_t n, void *children,
                     int32_t *n_children) {
    DevScene S;
    cudaStream_t st;
    int dev;
    if (!s || rp__scene_view(s, &S, &st, &dev) || mat < 0 || mat >= S.n_mats ||
        (n && (!rays || !idx || !points || !normals || !tangents || !children || !n_children)))
        return RP_ERR_INVALID;
    if (!n) return RP_OK;
    cudaSetDevice(dev);
    cudaError_t e = cudaSuccess;
    Batch b;
    auto *dr = (const unsigned char *)b.in(rays, (size_t)RP_RAY_BYTES * n, st, e);
    auto *di = (const unsigned *)b.in(idx, 4 * n, st, e);
    auto *dp = (const double *)b.in(points, 24 * n, st, e);
    auto *dn = (const double *)b.in(normals, 24 * n, st, e);
    auto *dt = (const double *)b.in(tangents, 24 * n, st, e);
    auto *dc = (unsigned char *)b.out((size_t)RP_RAY_BYTES * 2 * n, st, e);
    auto *dnc = (int *)b.out(4 * n, st, e);
    auto *derr = (unsigned *)b.out(4, st, e);
    if (e == cudaSuccess) {
        unit_material<<<grid_of(n), 128, 0, st>>>(S, mat, dr, di, dp, dn, dt, n, dc, dnc, derr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(children, dc, (size_t)RP_RAY_BYTES * 2 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(n_children, dnc, 4 * n, cudaMemcpyDeviceToHost, st);
    return finish(e, st, derr);
}

int rp_convert_to_sp(rp_ctx *c, const void *rays, const double *normals, uint64_t n, void *out) {
    cudaStream_t st;
    int dev;
    if (!c || rp__ctx_stream(c, &st, &dev) || (n && (!rays || !normals || !out))) return RP_ERR_INVALID;
    if (!n) return RP_OK;
    cudaSetDevice(dev);
    cudaError_t e = cudaSuccess;
    Batch b;
    auto *dr = (const unsigned char *)b.in(rays, (size_t)RP_RAY_BYTES * n, st, e);
    auto *dn = (const double *)b.in(normals, 24 * n, st, e);
    auto *dout = (unsigned char *)b.out((size_t)RP_RAY_BYTES * n, st, e);
    auto *derr = (unsigned *)b.out(4, st, e);
    if (e == cudaSuccess) {
        unit_convert_sp<<<grid_of(n), 128, 0, st>>>(dr, dn, n, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)RP_RAY_BYTES * n, cudaMemcpyDeviceToHost, st);
    return finish(e, st, derr);
}

int rp_dispersion_eval(rp_scene *s, int32_t curve, const double *wl, uint64_t n, double *out_re_im) {
    DevScene S;
    cudaStream_t st;
    int dev;
    if (!s || rp__scene_view(s, &S, &st, &dev) || (n && (!wl || !out_re_im))) return RP_ERR_INVALID;
    const rp_dispersion *dc = nullptr;
    int nc = 0;
    if (rp__scene_curve(s, &dc, &nc) || curve < 0 || curve >= nc) return RP_ERR_INVALID;
    if (!n) return RP_OK;
    cudaSetDevice(dev);
    cudaError_t e = cudaSuccess;
    Batch b;
    auto *dwl = (const double *)b.in(wl, 8 * n, st, e);
    auto *dout = (double2 *)b.out(16 * n, st, e);
    auto *derr = (unsigned *)b.out(4, st, e);
    if (e == cudaSuccess) e = launch_dispersion_table(dc + curve, 1, S.aux, dwl, (long long)n, dout, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_re_im, dout, 16 * n, cudaMemcpyDeviceToHost, st);
    return finish(e, st, derr);
}

}  // extern "C"
