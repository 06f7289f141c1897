/*
 * rp_gb300.h -- C ABI of the GB300 (sm_103a) non-sequential ray-tracing hot path.
 *
 * This library replaces raypier's Cython hot path
 *   raypier/core/ctracer.pyx:2062-2118   trace_segment_c
 *   raypier/core/ctracer.pyx:2173-2182   trace_segment (Python entry)
 *   raypier/core/tracer.py:9-47          trace_rays (generation driver)
 * and the per-face / per-material plugin calls it dispatches to
 *   raypier/core/ctracer.pxd:231-235     Face.intersect_c / compute_normal_c / compute_tangent_c
 *   raypier/core/ctracer.pxd:189-193     InterfaceMaterial.eval_child_ray_c
 *   raypier/core/ctracer.pxd:212-213     Shape.point_inside_c
 *   raypier/core/ctracer.pxd:207-209     Distortion.z_offset_and_gradient_c / z_offset_c
 * The reference dispatches through Cython virtual methods; here a scene is a set
 * of plain tables (faces, face lists, materials, shapes, distortions, dispersion
 * curves) and each face/material/shape/distortion is selected by a type tag.
 *
 * Conventions: every entry point returns an int status (RP_OK == 0, negative on
 * error); no C++ exception crosses this boundary.  The context owns all device
 * memory; the caller owns every host buffer it passes.  A context is bound to one
 * CUDA device and one stream and is not thread-safe.
 */
#ifndef RP_GB300_H
#define RP_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RP_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------- */
#define RP_OK               0
#define RP_ERR_INVALID     -1   /* bad argument or malformed scene            */
#define RP_ERR_CAPACITY    -2   /* an output buffer is too small              */
#define RP_ERR_BUDGET      -3   /* the context's device-memory budget is hit  */
#define RP_ERR_TIMEOUT     -4   /* a bounded device-side wait gave up         */
#define RP_ERR_CUDA        -5   /* a CUDA runtime call failed                 */
#define RP_ERR_UNSUPPORTED -6   /* face/material/shape type not implemented   */
#define RP_ERR_NOMEM       -7   /* host allocation failed                     */

/* ---- ray record --------------------------------------------------------- */
/* Byte-identical to ctracer.ray_t / ctracer.ray_dtype: 188 bytes, packed
 * (raypier/core/ctracer.pxd:40-48, raypier/core/ctracer.pyx:45-60). */
#pragma pack(push, 1)
typedef struct rp_ray {
    double origin[3], direction[3], normal[3], E_vector[3];
    double refractive_index[2], E1_amp[2], E2_amp[2];   /* complex: re, im */
    double length, phase, accumulated_path;
    uint32_t wavelength_idx, parent_idx, end_face_idx, ray_ident, ray_type_id;
} rp_ray;
#pragma pack(pop)

#define RP_RAY_BYTES 188
#define RP_REFL_RAY  1u          /* ctracer.pyx:19 REFL_RAY */
#define RP_GAUSSLET_RAY 2u       /* ctracer.pyx:21 GAUSSLET */

/* Gausslet record: a base ray and six parabasal rays, byte-identical to
 * ctracer.gausslet_dtype (ctracer.pxd:54-64 para_t / gausslet_t,
 * ctracer.pyx:66-76): 80 + 668 bytes, packed. */
#pragma pack(push, 1)
typedef struct rp_para {
    double origin[3], direction[3], normal[3];
    double length;
} rp_para;
typedef struct rp_gausslet {
    rp_ray base_ray;
    rp_para para[6];
} rp_gausslet;
#pragma pack(pop)
#define RP_PARA_BYTES 80
#define RP_GAUSSLET_BYTES 668
#define RP_NO_FACE   0xFFFFFFFFu /* end_face_idx of a ray that hit nothing */

/* ---- scene tables ------------------------------------------------------- */
/* Affine map: out = m * p + t, m row-major (ctracer.pxd:62-64 transform_t). */
typedef struct rp_transform {
    double m[9];
    double t[3];
} rp_transform;

/* A FaceList: faces [first_face, first_face + n_faces) share one transform
 * (ctracer.pxd:238-251). */
typedef struct rp_facelist {
    rp_transform trans;       /* local -> global */
    rp_transform inv_trans;   /* global -> local */
    int32_t first_face;
    int32_t n_faces;
} rp_facelist;

/* Face types (raypier/core/cfaces.pyx). */
enum rp_face_type {
    RP_FACE_NONE = 0,          /* base Face: never hit (ctracer.pyx:1747-1757) */
    RP_FACE_CIRCULAR = 1,      /* CircularFace          cfaces.pyx:140-191  p: diameter, offset, z_plane */
    RP_FACE_RECTANGULAR = 2,   /* RectangularFace       cfaces.pyx:354-407  p: length, width, offset, z_plane */
    RP_FACE_SHAPED_PLANAR = 3, /* ShapedPlanarFace      cfaces.pyx:194-242  p: z_height */
    RP_FACE_SPHERICAL = 4,     /* SphericalFace         cfaces.pyx:410-498  p: diameter, curvature, z_height */
    RP_FACE_SHAPED_SPHERICAL = 5, /* ShapedSphericalFace cfaces.pyx:501-608 p: curvature, z_height */
    RP_FACE_CONIC = 6,         /* ConicRevolutionFace   cfaces.pyx:1751-1837 p: curvature, z_height, conic_const */
    RP_FACE_ASPHERIC = 7,      /* AsphericFace          cfaces.pyx:1840-2025 p: curvature, z_height, conic_const, A4..A16, atol */
    RP_FACE_EXTPOLY = 8,       /* ExtendedPolynomialFace cfaces.pyx:2028-2320 p: R, beta, norm_radius, z_height, atol; aux: coefs[n_aux0][n_aux1] */
    RP_FACE_DISTORTION = 9,    /* DistortionFace        cfaces.pyx:2323-2438 p: accuracy; base, distortion */
    RP_FACE_ORIENTED_POLYGON = 10, /* OrientedPolygonFace cfaces.pyx:1121-1222 p: origin[3], normal[3], x_axis[3], y_axis[3]; aux: xy[n_aux0][2] */
    RP_FACE_POLYGON = 11,      /* PolygonFace           cfaces.pyx:1077-1118 p: z_plane; aux: xy[n_aux0][2] */
    RP_FACE_ELLIPTICAL_PLANE = 12, /* ElipticalPlaneFace cfaces.pyx:313-351  p: g_x, g_y, diameter */
    RP_FACE_OFF_AXIS_PARABOLIC = 13, /* OffAxisParabolicFace cfaces.pyx:1224-1315 p: EFL, diameter, height */
    RP_FACE_ELLIPSOIDAL = 14,  /* EllipsoidalFace       cfaces.pyx:1318-1410 p: major, minor, x1, x2, y1, y2, z1, z2;
                                  aux: trans m[9] t[3], inv_trans m[9] t[3] (24 doubles) */
    RP_FACE_SADDLE = 15,       /* SaddleFace            cfaces.pyx:1413-1511 p: z_height, curvature */
    RP_FACE_CYLINDRICAL = 16,  /* CylindericalFace      cfaces.pyx:1516-1602 p: z_height, radius */
    RP_FACE_AXICON = 17        /* AxiconFace            cfaces.pyx:1605-1680 p: z_height, gradient */
};

#define RP_FACE_NPARAM 16
typedef struct rp_face {
    int32_t type;            /* rp_face_type */
    int32_t idx;             /* Face.idx: the value written to end_face_idx */
    int32_t material;        /* index into the material table, -1 for sub-faces */
    int32_t invert_normal;   /* Face.invert_normal (ctracer.pxd:228) */
    int32_t invert_normals;  /* CircularFace / ShapedFace .invert_normals (cfaces.pyx:53,136) */
    int32_t shape;           /* first op of this face's shape program, -1: no shape */
    int32_t aux;             /* offset into the aux double table */
    int32_t n_aux0, n_aux1;  /* aux extents (see face type) */
    int32_t base;            /* DistortionFace: record index of the base face */
    int32_t distortion;      /* DistortionFace: index into the distortion table */
    int32_t reserved;
    double tolerance;        /* Face.tolerance */
    double p[RP_FACE_NPARAM];
} rp_face;

/* Shapes (raypier/core/cshapes.pyx) as a postfix program of boolean ops,
 * terminated by RP_SHAPE_END. */
enum rp_shape_op_type {
    RP_SHAPE_END = 0,
    RP_SHAPE_TRUE = 1,     /* base Shape: always inside (ctracer.pyx:1653-1655) */
    RP_SHAPE_CIRCLE = 2,   /* CircleShape    cshapes.pyx:102-116  a,b = centre, c = radius */
    RP_SHAPE_RECT = 3,     /* RectangleShape cshapes.pyx:119-136  a,b = centre, c = width, d = height */
    RP_SHAPE_POLYGON = 4,  /* PolygonShape   cshapes.pyx:139-168  aux: xy[n][2] */
    RP_SHAPE_AND = 5,      /* BooleanAND     cshapes.pyx:48-50 */
    RP_SHAPE_OR = 6,       /* BooleanOR      cshapes.pyx:53-55 */
    RP_SHAPE_XOR = 7,      /* BooleanXOR     cshapes.pyx:58-60 */
    RP_SHAPE_NOT = 8       /* InvertShape    cshapes.pyx:30-36 */
};
typedef struct rp_shape_op {
    int32_t op;
    int32_t aux;
    int32_t n;
    int32_t reserved;
    double a, b, c, d;
} rp_shape_op;

/* Distortions (raypier/core/cdistortions.pyx). */
enum rp_distortion_type {
    RP_DIST_ZERNIKE = 1,     /* ZernikeDistortion   cdistortions.pyx:323-514; aux: n_coefs x (j,n,m,k,value) */
    RP_DIST_SIMPLE_J7 = 2    /* SimpleTestZernikeJ7 cdistortions.pyx:39-81  */
};
typedef struct rp_distortion {
    int32_t type;
    int32_t n_coefs;
    int32_t k_max;
    int32_t aux;
    double unit_radius;
    double amplitude;
} rp_distortion;

/* Materials (raypier/core/cmaterials.pyx). */
enum rp_material_type {
    RP_MAT_NONE = 0,                 /* base InterfaceMaterial: no child (ctracer.pyx:1580-1586) */
    RP_MAT_OPAQUE = 1,               /* OpaqueMaterial            cmaterials.pyx:242-251 */
    RP_MAT_TRANSPARENT = 2,          /* TransparentMaterial       cmaterials.pyx:254-278 */
    RP_MAT_PEC = 3,                  /* PECMaterial               cmaterials.pyx:281-319 */
    RP_MAT_PARTIAL = 4,              /* PartiallyReflectiveMaterial cmaterials.pyx:322-397  p0 = reflectivity */
    RP_MAT_LINEAR_POLARISING = 5,    /* LinearPolarisingMaterial  cmaterials.pyx:400-455 */
    RP_MAT_WAVEPLATE = 6,            /* WaveplateMaterial         cmaterials.pyx:458-551  p0,p1 = retardance (re,im), p2..p4 = fast axis */
    RP_MAT_DIELECTRIC = 7,           /* DielectricMaterial        cmaterials.pyx:554-680 */
    RP_MAT_FULL_DIELECTRIC = 8,      /* FullDielectricMaterial    cmaterials.pyx:727-872 */
    RP_MAT_FULL_DIELECTRIC_DISPERSIVE = 9, /* FullDielectricDispersiveMaterial cmaterials.pyx:875-1013 */
    RP_MAT_CIRCULAR_APERTURE = 10,   /* CircularApertureMaterial  cmaterials.pyx:1602-1662
                                        p: outer_radius, radius, edge_width, invert, origin[3] */
    RP_MAT_RECT_APERTURE = 11,       /* RectangularApertureMaterial cmaterials.pyx:1665-1763
                                        p: outer_width, outer_height, width, height, edge_width, invert, origin[3] */
    RP_MAT_SINGLE_LAYER_COATED = 12, /* SingleLayerCoatedMaterial cmaterials.pyx:1017-1184
                                        n_inside, n_outside; p: n_coating (re, im), thickness (um) */
    RP_MAT_COATED_DISPERSIVE = 13,   /* CoatedDispersiveMaterial  cmaterials.pyx:1187-1381
                                        curve_inside, curve_outside; p: curve_coating, coating_thickness (um) */
    RP_MAT_DIFFRACTION_GRATING = 14, /* DiffractionGratingMaterial cmaterials.pyx:1437-1543
                                        p: lines_per_mm, order, efficiency, origin[3] */
    RP_MAT_RESAMPLE_GAUSSLET = 15    /* ResampleGaussletMaterial  cmaterials.pyx:1766-1830: emits no
                                        child; a Gausslet generation reports the gausslets it captured */
};
typedef struct rp_material {
    int32_t type;
    int32_t curve_inside;    /* dispersive: index into the dispersion table */
    int32_t curve_outside;
    int32_t reserved;
    double n_inside[2];      /* complex (re, im) */
    double n_outside[2];
    double reflection_threshold;
    double transmission_threshold;
    double p[10];
} rp_material;

/* Dispersion curves: BaseDispersionCurve (cmaterials.pyx:152-239). */
typedef struct rp_dispersion {
    int32_t formula_id;      /* 0, 1, 2 or 3 (formula 5 has no return value in the reference) */
    int32_t n_coefs;
    int32_t aux;             /* offset of the coefficients in the aux table */
    int32_t reserved;
    double absorption;       /* cm^-1 */
    double wavelength_min, wavelength_max;
} rp_dispersion;

/* A whole scene.  faces[0 .. n_faces) are the traced faces in FaceList order
 * (the reference's all_faces order); records after n_faces are sub-faces
 * (DistortionFace base faces) that are only reached through rp_face.base. */
typedef struct rp_scene_desc {
    int32_t n_lists;
    int32_t n_faces;
    int32_t n_face_records;
    int32_t n_materials;
    int32_t n_shape_ops;
    int32_t n_distortions;
    int32_t n_dispersions;
    int32_t n_aux;
    const rp_facelist *lists;
    const rp_face *faces;
    const rp_material *materials;
    const rp_shape_op *shape_ops;
    const rp_distortion *distortions;
    const rp_dispersion *dispersions;
    const double *aux;
} rp_scene_desc;

/* Per-call statistics. */
typedef struct rp_stats {
    uint64_t rays_in;        /* rays traced (segments) */
    uint64_t rays_out;       /* children kept */
    uint64_t hits;           /* rays that hit a face */
    uint64_t terminated;     /* children dropped by the |E|^2 rule */
    double   device_ms;      /* device time of the call (CUDA events on the context stream) */
    double   kernel_ms;      /* summed device time of the generation kernels alone */
    uint64_t launches;       /* kernels this library launched for the call */
    uint64_t generations;    /* generations traced */
    double   search_ms;      /* RP_TRACE_MIXED: the part of kernel_ms spent in the search kernels (the rest is
                                the material kernels); 0 on the plain path */
} rp_stats;

/* Trace flags. */
#define RP_TRACE_PLAIN_FP64  0u  /* all-FP64 path, bit-parity with the reference */
#define RP_TRACE_MIXED       1u  /* FP32 bulk, FP64 roots / last Newton step / OPL */

typedef struct rp_ctx rp_ctx;
typedef struct rp_scene rp_scene;
typedef struct rp_rays rp_rays;

/* ---- library ------------------------------------------------------------ */
int rp_version(void);
const char *rp_status_string(int status);
/* Last CUDA error text seen by this thread (empty if none). */
const char *rp_last_error(void);

/* ---- context ------------------------------------------------------------ */
/* Bind to `device`; hbm_budget 0 = no limit.  Replaces nothing in the
 * reference (which has no device); owns the stream and scratch arenas. */
int rp_ctx_create(int device, uint64_t hbm_budget, rp_ctx **out);
int rp_ctx_destroy(rp_ctx *ctx);
int rp_ctx_synchronize(rp_ctx *ctx);
/* Bytes of device memory the context holds (live buffers, cached blocks and scratch). */
int rp_ctx_memory(rp_ctx *ctx, uint64_t *bytes_in_use);
/* Return cached device blocks of freed ray buffers to CUDA. */
int rp_ctx_trim(rp_ctx *ctx);
/* Page-locked host memory for fast host<->device copies of ray records. */
int rp_host_alloc(uint64_t bytes, void **ptr);
int rp_host_free(void *ptr);

/* ---- scenes ------------------------------------------------------------- */
/* Upload a scene.  `wavelengths` is the RayCollection.wavelengths array that
 * the reference pushes into each material (core/tracer.py:28-34,
 * ctracer.pyx:1647-1650); dispersion tables are evaluated once here, as the
 * reference's on_set_wavelengths does (cmaterials.pyx:883-887).  Returns
 * RP_ERR_INVALID when a wavelength lies outside a curve's range
 * (cmaterials.pyx:220-224 raises ValueError there). */
int rp_scene_create(rp_ctx *ctx, const rp_scene_desc *desc,
                    const double *wavelengths, int64_t n_wavelengths,
                    rp_scene **out);
int rp_scene_destroy(rp_scene *scene);
/* Per-face hit counters accumulated since the last reset (Face.count,
 * ctracer.pyx:2108). counts has n_faces entries. */
int rp_scene_face_counts(rp_scene *scene, uint32_t *counts, int32_t n_faces, int reset);

/* Host-only: one world-space box per face that holds every point where the
 * face can report a hit (no counterpart in the reference, which tests every
 * face): out[8*f .. 8*f+5] = lo xyz, hi xyz, out[8*f+6] = 1 if face f may be
 * skipped, 0 if it is always tested (2: a distortion face's local rectangle).
 * For a conic face it spans both sheets; the searches use
 * rp_scene_search_bounds. */
int rp_scene_bounds(const rp_scene_desc *desc, float *out, int32_t n_faces);
/* Host-only: the boxes the nearest-hit searches use to skip faces a ray cannot
 * reach before its current nearest hit, 16 floats per face: out[16*f ..
 * 16*f+7] as rp_scene_bounds and, for a ConicRevolutionFace, the boxes of its
 * two sheets' parts over the aperture in out[16*f .. +7] and out[16*f+8 ..
 * +15] (out[16*f+6] = 3 when the two boxes are set; a ray that may hit the
 * face enters one of them). */
int rp_scene_search_bounds(const rp_scene_desc *desc, float *out, int32_t n_faces);

/* ---- device ray buffers (structure-of-arrays) ---------------------------- */
int rp_rays_alloc(rp_ctx *ctx, uint64_t capacity, rp_rays **out);
int rp_rays_free(rp_rays *rays);
int rp_rays_count(const rp_rays *rays, uint64_t *n);
int rp_rays_capacity(const rp_rays *rays, uint64_t *cap);
/* Copy n packed 188-byte records in (RayCollection.from_array, ctracer.pyx:1142-1154)
 * or out (RayCollection.copy_as_array, ctracer.pyx:1048-1054). */
int rp_rays_upload_aos(rp_rays *rays, const void *records, uint64_t n);
int rp_rays_download_aos(const rp_rays *rays, void *records, uint64_t n);
/* Device pointer of one SoA field (for zero-copy consumers); field names follow
 * ray_dtype: "origin_x", ..., "E1_amp" (double2), "wavelength_idx", ... */
int rp_rays_field(const rp_rays *rays, const char *name, void **dev_ptr);

/* ---- tracing ------------------------------------------------------------ */
/* One generation: replaces trace_segment_c (ctracer.pyx:2062-2118).
 * `in` is mutated as in the reference (length, end_face_idx); children are
 * written to `out` in the reference's append order (parent ascending,
 * reflected before transmitted).  When e2_terminate > 0 a child with
 * |E1|^2 + |E2|^2 < e2_terminate is dropped (stable).  `max_length` is a C
 * float as in the reference (ctracer.pxd:261).  Returns RP_ERR_CAPACITY if
 * `out` cannot hold the children (out is then left with count 0). */
int rp_trace_segment(rp_ctx *ctx, rp_scene *scene, rp_rays *in, rp_rays *out,
                     float max_length, uint32_t flags, double e2_terminate,
                     rp_stats *stats);

/* Sequential variant: only face `face_idx` of face list `list_idx` is tested
 * (trace_one_face_segment_c, ctracer.pyx:2121-2170). */
int rp_trace_one_face_segment(rp_ctx *ctx, rp_scene *scene, rp_rays *in, rp_rays *out,
                              int32_t list_idx, int32_t face_idx, float max_length,
                              uint32_t flags, double e2_terminate, rp_stats *stats);

/* Whole non-sequential trace (trace_rays, core/tracer.py:9-47): generation g+1
 * is traced from generation g while it is non-empty and g < recursion_limit.
 * gens[0] must hold the input rays; gens[1..max_gens) are allocated by the
 * library as needed (free them with rp_rays_free).  *n_gens receives the
 * number of traced generations (the reference's len(traced_rays)). */
int rp_trace_rays(rp_ctx *ctx, rp_scene *scene, rp_rays **gens, int32_t max_gens,
                  int32_t recursion_limit, float max_length, uint32_t flags,
                  double e2_terminate, int32_t *n_gens, rp_stats *stats);

/* Host-buffer convenience: upload `n` input records, trace all generations,
 * download them into `out_records` (capacity `out_cap` records, generations
 * concatenated) with `gen_offsets[0..n_gens]` the start of each generation.
 * Reference counterpart: trace_rays + RayCollection.copy_as_array. */
int rp_trace_rays_host(rp_ctx *ctx, rp_scene *scene, const void *in_records, uint64_t n,
                       int32_t recursion_limit, float max_length, uint32_t flags,
                       double e2_terminate, void *out_records, uint64_t out_cap,
                       uint64_t *gen_offsets, int32_t max_gens, int32_t *n_gens,
                       rp_stats *stats);

/* ---- Gausslets ----------------------------------------------------------- */
/* Device Gausslet buffers: the base rays as a ray buffer plus the six
 * parabasal rays as structure-of-arrays. */
typedef struct rp_gausslets rp_gausslets;
int rp_gausslets_alloc(rp_ctx *ctx, uint64_t capacity, rp_gausslets **out);
int rp_gausslets_free(rp_gausslets *g);
int rp_gausslets_count(const rp_gausslets *g, uint64_t *n);
/* Copy n packed 668-byte records in (GaussletCollection.from_array,
 * ctracer.pyx:1303-1318) or out (GaussletCollection.copy_as_array, 1286-1292). */
int rp_gausslets_upload(rp_gausslets *g, const void *records, uint64_t n);
int rp_gausslets_download(const rp_gausslets *g, void *records, uint64_t n);
/* GaussletCollection.config_parabasal_rays (ctracer.pyx:1430-1476) on the
 * device: the six parabasal rays of a circular Gaussian mode of 1/e^2 waist
 * `radius` (mm) whose waist lies working_dist beyond each base ray's origin,
 * at the base ray's wavelength (wavelengths[wavelength_idx], um). */
int rp_gausslets_config_parabasal(rp_gausslets *g, const double *wavelengths, int64_t n_wavelengths, double radius,
                                  double working_dist);
/* GaussletCollection.total_power (ctracer.pyx:1482-1496): the sum over the
 * base rays of (|E1|^2 + |E2|^2) Re(n), reduced on the device in a fixed
 * order. */
int rp_gausslets_total_power(const rp_gausslets *g, double *power);

/* One Gausslet generation: replaces trace_gausslet_c (ctracer.pyx:2214-2282)
 * and, with list_idx / face_idx >= 0, trace_one_face_gausslet_c (2285-2350),
 * both through trace_parabasal_rays (2353-2385).  The base ray finds its face
 * as a ray does (its length is not reset first: the reference resets lengths
 * at the end of each generation); the six parabasal rays are then tested
 * against that face alone without its aperture; if every one meets it, each
 * child of the base ray becomes a child gausslet whose parabasal rays the
 * material bends (eval_parabasal_ray_c, cmaterials.pyx:683-724, 1393-1433,
 * 1544-1600, ctracer.pyx:1588-1610).  `in` is mutated as in the reference
 * (base length and end_face_idx, lengths of the parabasal rays tested); the
 * children's base and parabasal lengths are set to max_length
 * (reset_length_c, ctracer.pyx:1224-1230).  `max_length` is a double here, as
 * in the reference's Gausslet path.  captured (optional, host array of n_in
 * int32) receives for each input gausslet 1 + the material index of the
 * RP_MAT_RESAMPLE_GAUSSLET material that captured it, else 0: the caller runs
 * the decomposition (eval_decomposed_rays_c, cmaterials.pyx:1820-1830). */
int rp_trace_gausslet_segment(rp_ctx *ctx, rp_scene *scene, rp_gausslets *in, rp_gausslets *out,
                              int32_t list_idx, int32_t face_idx, double max_length,
                              int32_t *captured, rp_stats *stats);

/* ---- post-trace capture -------------------------------------------------- */
/* Replaces select_ray_intersections (ctracer.pyx:1981-2015) for one traced
 * collection: a copy of every ray of `in` (which is not modified) is
 * intersected with the faces of face list `list_idx` of `scene`, from its
 * origin to origin + direction * length (FaceList.intersect_c, 1882-1904);
 * the copies that meet a face are written to `out` in input order, with the
 * nearest face's distance as length, its index as end_face_idx and
 * wavelength_idx + wl_offset (the collection's offset in the concatenated
 * wavelength lists; the caller maps the concatenation onto its unique values,
 * 2010-2015). */
int rp_select_intersections(rp_ctx *ctx, rp_scene *scene, int32_t list_idx, rp_rays *in, rp_rays *out,
                            uint32_t wl_offset);
/* The same for gausslets, by their base rays (select_gausslet_intersections,
 * ctracer.pyx:2018-2058); the parabasal rays are copied unchanged. */
int rp_select_gausslet_intersections(rp_ctx *ctx, rp_scene *scene, int32_t list_idx, rp_gausslets *in,
                                     rp_gausslets *out, uint32_t wl_offset);

/* ---- E-field summation ---------------------------------------------------- */
/* Gaussian-mode coefficients of each gausslet (evaluate_modes,
 * cfields.pyx:150-234): x, y, dx, dy are n rows of `size` (1..64) parabasal
 * offsets and slopes in the base ray's frame (core/fields.py:122-148
 * evaluate_neighbours_gc); modes_out receives n x 3 complex (re, im)
 * coefficients A, B, C.  RP_ERR_INVALID where the reference raises
 * ZeroDivisionError (a degenerate fit). */
int rp_field_evaluate_modes(rp_ctx *ctx, const double *x, const double *y, const double *dx, const double *dy,
                            uint64_t n, int32_t size, double blending, double *modes_out);

/* A set of Gaussian modes held on the device for repeated evaluation
 * (core/fields.py:239-266 EFieldSummation): the modes' base rays (188-byte
 * records), their n x 3 complex coefficients and the wavelength table. */
typedef struct rp_field rp_field;
int rp_field_create(rp_ctx *ctx, const void *rays, uint64_t n_rays, const double *modes,
                    const double *wavelengths, int64_t n_wavelengths, rp_field **out);
int rp_field_destroy(rp_field *field);
/* sum_gaussian_modes (cfields.pyx:49-117): the complex E-field at n_points
 * points (x, y, z), E_out n_points x 3 complex (re, im), summed over the modes
 * in order for every point, at time time_ps.  Host buffers. */
int rp_field_evaluate(rp_field *field, const double *points, uint64_t n_points, double time_ps, double *E_out);
/* The same with device buffers (points and E on the context's device). */
int rp_field_evaluate_device(rp_field *field, const double *points_dev, uint64_t n_points, double time_ps,
                             double *E_dev);
/* calc_mode_curvature (cfields.pyx:232-290): the wavefront curvature A, B, C
 * (d2z'/dx'2, d2z'/dx'dy', d2z'/dy'2) and the local basis x', y', z' (X, Y, Z:
 * n x 3) at n points of a decomposition plane from the wavefront slopes dx, dy
 * and second derivatives dx2, dy2, dxdy there (the reference's rx, ry are
 * not used by it).  Host buffers. */
int rp_field_mode_curvature(rp_ctx *ctx, const double *dx, const double *dy, const double *dx2, const double *dy2,
                            const double *dxdy, uint64_t n, double *A, double *B, double *C, double *X, double *Y,
                            double *Z);
/* build_interaction_matrix (cfields.pyx:295-395): the field of mode i (origin
 * rx[i], ry[i]; curvature A, B, C; basis rows X, Y, Z) at test point j (tx[j],
 * ty[j]) for every pair no further apart than max_spacing, as COO entries
 * (data: complex (re, im); row = i, col = j) ordered by i, then j.  *count
 * receives the number of pairs; RP_ERR_CAPACITY (nothing written) when it
 * exceeds cap.  Host buffers. */
int rp_field_interaction_matrix(rp_ctx *ctx, const double *rx, const double *ry, uint64_t n_modes, const double *tx,
                                const double *ty, uint64_t n_points, const double *A, const double *B,
                                const double *C, const double *X, const double *Y, const double *Z,
                                double wavelength, double spacing, double max_spacing, double blending, uint64_t cap,
                                uint64_t *count, double *data, uint64_t *row, uint64_t *col);
/* apply_mode_curvature (cfields.pyx:398-426): tilts the parabasal rays of
 * every gausslet of a device collection by its curvature A[i], B[i], C[i]
 * (host arrays, one per gausslet). */
int rp_field_apply_mode_curvature(rp_gausslets *gausslets, const double *A, const double *B, const double *C);
/* One-shot sum_gaussian_modes: create, evaluate, destroy. */
int rp_field_sum_gaussian_modes(rp_ctx *ctx, const void *rays, uint64_t n_rays, const double *modes,
                                const double *wavelengths, int64_t n_wavelengths, const double *points,
                                uint64_t n_points, double time_ps, double *E_out);
/* The modes of a device gausslet collection, fitted on the device and kept
 * there: replaces the set-up of EFieldSummation / eval_Efield_from_gausslets
 * (core/fields.py:239-247, 269-277: evaluate_neighbours_gc, 122-148, then
 * cfields.evaluate_modes).  Each gausslet's six parabasal rays are sampled in
 * its base ray's (E, E x d) frame and fitted in closed form; the field's base
 * rays are the gausslets' base rays.  RP_ERR_INVALID ("float division") for a
 * degenerate fit, where the reference raises ZeroDivisionError. */
int rp_field_create_from_gausslets(rp_gausslets *gausslets, const double *wavelengths, int64_t n_wavelengths,
                                   double blending, rp_field **out);
/* The modes of a device ray lattice (eval_Efield_from_rays, core/fields.py:
 * 195-224): with radius != 0 the rays are first moved to their intercept with
 * the sphere of that radius about centre[3] (project_to_sphere, 51-77; every
 * ray must meet it); each ray whose six neighbour indices (neighbours: host,
 * n x 6 int32, -1 for none) all exist is sampled against its neighbours
 * carried to its normal plane (evaluate_neighbours, 80-111) and fitted.  The
 * field keeps those rays, in order. */
int rp_field_create_from_rays(rp_rays *rays, const int32_t *neighbours, const double *centre, double radius,
                              double blending, const double *wavelengths, int64_t n_wavelengths, rp_field **out);
/* A field's mode count and, where the pointers are non-null, its base rays
 * (188-byte records) and n x 3 complex mode coefficients.  Host buffers. */
int rp_field_download(const rp_field *field, uint64_t *n_modes, void *records, double *modes);
/* The wavefront samples the mode fit takes, as host arrays of n x 6:
 * evaluate_neighbours_gc (core/fields.py:114-136) of a device gausslet
 * collection ... */
int rp_field_gausslet_samples(rp_gausslets *gausslets, double *x, double *y, double *dx, double *dy);
/* ... and evaluate_neighbours (80-111) of a device ray lattice; kept[] (host,
 * capacity n) receives the rows kept, *n_kept their number (the samples fill
 * the first *n_kept rows). */
int rp_field_ray_samples(rp_rays *rays, const int32_t *neighbours, double *x, double *y, double *dx, double *dy,
                         uint64_t *kept, uint64_t *n_kept);
/* project_to_sphere (core/fields.py:51-77) in place on a device buffer: each
 * ray moves along its direction to the nearer-behind intercept with the
 * sphere (radius about centre[3]) and its optical path by that distance
 * times the real refractive index; hit[i] (host, n bytes) is 0 for a ray that
 * misses the sphere (left unchanged). */
int rp_rays_project_to_sphere(rp_rays *rays, const double *centre, double radius, uint8_t *hit);

/* ---- measurement support -------------------------------------------------- */
/* No counterpart in the reference: the device's measured arithmetic peaks,
 * the denominators of the pipe rooflines reported beside the HBM one.  FP64
 * and FP32 fused multiply-add throughput (counted as two floating-point
 * operations each) and 32-bit integer multiply-add throughput, per second,
 * from many independent chains per thread timed with CUDA events (best of
 * three launches after a warm-up).  Takes about a tenth of a second. */
int rp_measure_peaks(int device, double *fp64_flops, double *fp32_flops, double *int32_ops);
/* The host link's copy rates in bytes per second, device to page-locked host
 * memory and back (one 256 MB cudaMemcpyAsync each way, best of three after a
 * warm-up, CUDA events): the bound of the host-buffer entry points, which
 * move every generation over it. */
int rp_measure_host_link(int device, double *d2h_bytes_per_s, double *h2d_bytes_per_s);

/* ---- differentiable sequential lens ------------------------------------- */
/* No counterpart in the reference: raypier has no gradients.  A stack of even
 * aspheres traced in order (each surface an AsphericFace with a circular
 * aperture, cfaces.pyx:1840-2025, refracting as DielectricMaterial,
 * cmaterials.pyx:589-680, from n_index[k] to n_index[k+1]) onto an image plane
 * (CircularFace); the loss is the RMS spot radius of the rays that reach it.
 * The forward runs the plain path's FP64 face and material arithmetic, so it
 * equals rp_trace_rays on the same faces bit for bit; the backward is a
 * hand-written adjoint that re-traces each ray from its input up to every
 * surface (no per-surface state is kept between the passes).
 * params[5 * n_surfaces]: curvature[n] (raypier sign, R = -curvature),
 * conic[n], A4[n], A6[n], thickness[n] (vertex to next vertex; the last one
 * from the last vertex to the image plane).  Surface 0's vertex is at z0. */
typedef struct rp_lens_desc {
    int32_t n_surfaces;            /* 1 .. 64 */
    int32_t reserved;
    double z0;
    double max_length;             /* segment length of the intersection tests (trace max_length) */
    double atol;                   /* AsphericFace.atol */
    double tolerance;              /* Face.tolerance */
    const double *semi_diameter;   /* [n_surfaces] aperture radius */
    const double *n_index;         /* [n_surfaces + 1] real index before surface 0 and after each surface */
} rp_lens_desc;
typedef struct rp_lens rp_lens;
int rp_lens_create(rp_ctx *ctx, const rp_lens_desc *desc, uint64_t max_rays, rp_lens **out);
int rp_lens_destroy(rp_lens *lens);
/* Traces `rays` (origins and directions of a device buffer; unit directions)
 * and returns the RMS spot radius and the number of rays that reached the
 * image.  RP_ERR_INVALID when an aperture reaches a conic's rim. */
int rp_lens_forward(rp_lens *lens, const double *params, const rp_rays *rays, double *loss, uint64_t *n_valid);
/* d loss / d params of the last forward (same rays, unchanged since). */
int rp_lens_backward(rp_lens *lens, double *grad);
/* Image-plane x, y and reached flags of the last forward's first n rays. */
int rp_lens_image(const rp_lens *lens, double *xy, uint8_t *valid, uint64_t n);

/* ---- trace-job server ----------------------------------------------------- */
/* No counterpart in the reference (its traces run one at a time in the caller's
 * thread).  A server holds up to `lanes` jobs in flight (at most 64) on one
 * device; submitted jobs wait in one FIFO queue and are admitted as soon as a
 * slot is free and the HBM budget holds their estimated footprint.  A job is
 * a whole trace_rays (core/tracer.py:9-47) of rays generated on the device
 * from a source description.  The server advances in steps: each step moves
 * every admitted job forward by one generation, the RP_TRACE_MIXED jobs
 * together in one launch of each mixed-path kernel (their rays numbered in
 * 128-ray groups across the jobs), as one CUDA graph replayed every step, and
 * the plain FP64 jobs through their own kernels in the same step; one
 * read-back per step gives every job's next generation size.  Jobs that
 * arrive while others trace join at the next step.  The result is the job's
 * counters and the tallies of the rays that ended on its detector face,
 * reduced on the device in a fixed order within the job (the same whether the
 * job runs alone or among others).  RP_TRACE_MIXED jobs need scenes of the
 * faces and materials the mixed kernels specialise (else RP_ERR_UNSUPPORTED
 * in the result).  Submit and wait may be called from any thread. */
#define RP_SOURCE_POINT_CONE      1  /* point at `origin`, directions uniform in a cone of `half_angle` about +z */
#define RP_SOURCE_COLLIMATED_DISC 2  /* directions +z, origins uniform over a disc of `radius` about `origin` */
typedef struct rp_source_desc {
    int32_t type;
    int32_t reserved;
    uint64_t n_rays;
    uint64_t seed;            /* counter-based: ray i depends only on (seed, i) */
    double origin[3];
    double half_angle;        /* rad */
    double radius;            /* mm */
    /* every ray: E linearly polarised at a uniform angle about the ray,
     * E1 = 1, n = 1, wavelength_idx uniform over the job's wavelengths */
} rp_source_desc;

typedef struct rp_job_desc {
    const rp_scene_desc *scene;   /* copied at submit */
    const double *wavelengths;    /* copied at submit */
    int64_t n_wl;
    rp_source_desc source;
    int32_t recursion_limit;
    float max_length;
    uint32_t flags;               /* RP_TRACE_PLAIN_FP64 / RP_TRACE_MIXED */
    int32_t detector_face;        /* Face.idx whose hits are tallied, -1: none */
    double e2_terminate;
} rp_job_desc;

typedef struct rp_job_result {
    int32_t status;               /* RP_OK or the failing call's status */
    int32_t generations;
    uint64_t segments;            /* rays traced over all generations */
    uint64_t detector_hits;
    double detector_power;        /* sum of (|E1|^2 + |E2|^2) Re(n) over the detector hits */
    double sum_x, sum_y, sum_xx, sum_yy;  /* of the detector hit points */
    double t_submit_ms, t_start_ms, t_done_ms;  /* server clock */
} rp_job_result;

/* The source rays of a job into a device buffer (capacity >= n_rays), for
 * tracing them with the other entry points. */
int rp_source_generate(rp_ctx *ctx, const rp_source_desc *source, uint32_t n_wl, rp_rays *out);

typedef struct rp_server rp_server;
int rp_server_create(int device, uint64_t hbm_budget, int32_t lanes, rp_server **out);
int rp_server_submit(rp_server *server, const rp_job_desc *job, uint64_t *job_id);
/* Blocks until the job is done; copies its per-face hit counts (n_faces of
 * them) when face_counts is not NULL.  A job id can be waited for once. */
int rp_server_wait(rp_server *server, uint64_t job_id, rp_job_result *result, uint32_t *face_counts,
                   int32_t n_faces);
/* The work of a step: a mixed job's generation of more than `groups` 128-ray
 * groups (what is left of the step's budget after the smaller generations,
 * and at least `min_chunk` groups) is traced over several steps, so that
 * small jobs' steps stay short; results do not depend on it.  Defaults
 * 32768 and 1024. */
int rp_server_set_step_groups(rp_server *server, uint32_t groups, uint32_t min_chunk);
/* Counters of the step loop since the server was created: how busy the GPU
 * was while jobs were in the steps (step_gpu_ms / step_wall_ms) and what the
 * host adds per step. */
typedef struct rp_server_stats {
    uint64_t steps;               /* batch steps run */
    uint64_t step_jobs;           /* sum over the steps of the jobs in each */
    double step_gpu_ms;           /* device time of the steps' work (CUDA events on the step stream) */
    double step_wall_ms;          /* host time inside the steps: preparation, launch, wait, bookkeeping */
    double idle_wall_ms;          /* host time between steps while jobs were in flight */
} rp_server_stats;
int rp_server_get_stats(rp_server *server, rp_server_stats *out);
/* Finishes the queued jobs, then stops the step loop. */
int rp_server_destroy(rp_server *server);

/* Allocation-free rp_trace_segment.  No counterpart in the reference: this is
 * an addition of this library.  Same arguments, results and status codes as
 * rp_trace_segment, for callers that must not allocate device memory during a
 * trace: a process whose HBM is already claimed by another caching allocator
 * (so a cudaMalloc would fail or force that allocator to give memory back),
 * or a loop that cannot afford the device-wide synchronisation cudaFree
 * implies while other streams run.  The call makes no cudaMalloc, cudaFree,
 * host allocation or allocating library call: its scratch (child slots,
 * per-tile counts and offsets, counters) is one fixed device array of about
 * 6.2 MB inside this library, sized for RP_NOALLOC_MAX_RAYS input rays.
 *  - More than RP_NOALLOC_MAX_RAYS rays in `in`: RP_ERR_CAPACITY, nothing
 *    launched, rp_last_error() says so.
 *  - The first call on each device does a one-time set-up (it looks up the
 *    scratch array's device address, which loads this library's device code
 *    on that device): make that first call before any stream capture.  The
 *    address is kept per device until rp_ctx_create is called for that
 *    device again: after a reset of the device (cudaDeviceReset), create a
 *    new context before the next call.
 *  - The counters at the start of the scratch must be zero when the
 *    generation kernel starts; the call clears them itself on its stream.
 *    Every other scratch byte is written before it is read.
 *  - There is one scratch array per device: calls on the same device must
 *    not overlap (another host thread, or another context on that device).
 *    Overlapping calls race on the scratch and corrupt each other's results.
 * stats->kernel_ms and stats->device_ms both receive the generation kernel's
 * time. */
#define RP_NOALLOC_MAX_RAYS 16384
int rp_trace_segment_noalloc(rp_ctx *ctx, rp_scene *scene, rp_rays *in, rp_rays *out,
                             float max_length, uint32_t flags, double e2_terminate,
                             rp_stats *stats);

/* ---- single-plugin calls (batches of independent inputs, host buffers) ---- */
/* Face.intersect (ctracer.pyx:1769-1777): distance along p1->p2 (local
 * coordinates, 3 doubles per point) to face record `rec`, -1 for a miss. */
int rp_face_intersect(rp_scene *scene, int32_t rec, const double *p1, const double *p2, uint64_t n,
                      int is_base_ray, double *dist);
/* Face.compute_normal (ctracer.pyx:1793-1800), local coordinates. */
int rp_face_normal(rp_scene *scene, int32_t rec, const double *p, uint64_t n, double *normal);
/* Shape.point_inside (ctracer.pyx:1657-1658) for the shape program at `prog`. */
int rp_shape_inside(rp_scene *scene, int32_t prog, const double *xy, uint64_t n, int32_t *inside);
/* Distortion.z_offset_and_gradient / z_offset (ctracer.pyx:1703-1729):
 * out4[i] = (dz/dx, dz/dy, z, z_offset). */
int rp_distortion_eval(rp_scene *scene, int32_t distortion, const double *xy, uint64_t n, double *out4);
/* InterfaceMaterial.eval_child_ray (ctracer.pyx:1620-1632): children of ray i
 * in records 2i, 2i+1 (188-byte format), their number in n_children[i]. */
int rp_material_eval(rp_scene *scene, int32_t material, const void *rays, const uint32_t *ray_idx,
                     const double *points, const double *normals, const double *tangents, uint64_t n,
                     void *children, int32_t *n_children);
/* Convert_to_SP (cmaterials.pyx:94-101). */
int rp_convert_to_sp(rp_ctx *ctx, const void *rays, const double *normals, uint64_t n, void *out_rays);
/* BaseDispersionCurve.evaluate_n (cmaterials.pyx:230-239) for curve `curve`
 * of the scene: complex index per wavelength (re, im pairs). */
int rp_dispersion_eval(rp_scene *scene, int32_t curve, const double *wavelengths, uint64_t n,
                       double *out_re_im);

#ifdef __cplusplus
}
#endif
#endif /* RP_GB300_H */
