/*
 * CPU oracle for the GB300 light-transport core -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference renderer's hot path
 * (Iscandel/Raytracer, RaytracerNew2/src): PathTracingMIS, VolPathTracing,
 * the binary SAH BVH, the BSDFs, lights, media, camera and film they use.
 * Each function cites the reference file:line it follows.  Only the test
 * suite, __graft_entry__.smoke() and bench.py's CPU baseline may load it;
 * the product library never links or calls it.
 *
 * Parity status: the PCG32 stream (tools/Rng.h) and the CDF sampler
 * (core/CDF.h) are pinned against the reference's own headers compiled here
 * (oracle/ref_pin.c + oracle/build_oracle.py); the rest of the restatement
 * is parity unpinned, because the reference needs Eigen, SFML, OpenEXR and
 * OpenVDB, none of which exist on this machine, and it ships no tests or
 * golden vectors.
 *
 * Arithmetic: IEEE binary32 with no contraction (-ffp-contract=off), every
 * expression evaluated in the reference's left-to-right order.
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H

#include <stdint.h>
#include <math.h>
#include "rtgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- basic types ---------------- */
typedef struct { float x, y, z; } v3;
typedef struct { float x, y; } v2;
typedef struct { float r, g, b; } c3;

#define O_PI 3.14159265358979323846f
#define O_INV_PI 0.3183098861837906715377f
#define O_INV_FOUR_PI 0.07957747154594766788450883936693f
#define O_MAX_REAL 10e7f
#define O_EPSILON 1e-4f

/* std::min / std::max argument semantics (first argument wins ties/NaN) */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }
static inline int imin(int a, int b) { return (b < a) ? b : a; }
static inline int imax(int a, int b) { return (a < b) ? b : a; }

static inline v3 mk3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v2 mk2(float x, float y) { v2 r = {x, y}; return r; }
static inline c3 mkc(float r, float g, float b) { c3 c = {r, g, b}; return c; }
static inline c3 cfill(float v) { c3 c = {v, v, v}; return c; }
static inline float v3_get(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline v3 v3_add(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 v3_sub(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 v3_neg(v3 a) { return mk3(-a.x, -a.y, -a.z); }
static inline v3 v3_muls(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline v3 v3_smul(float s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline v3 v3_divs(v3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
/* Eigen 3-vector redux order: (a0*b0 + a1*b1) + a2*b2 */
static inline float v3_dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 v3_cross(v3 a, v3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float v3_sqnorm(v3 a) { return v3_dot(a, a); }
static inline float v3_norm(v3 a) { return sqrtf(v3_sqnorm(a)); }
/* Eigen normalized()/normalize(): v / sqrt(squaredNorm) when non-zero */
static inline v3 v3_normalized(v3 a)
{
    float n = v3_sqnorm(a);
    if (n > 0.f) return v3_divs(a, sqrtf(n));
    return a;
}
static inline c3 c3_add(c3 a, c3 b) { return mkc(a.r + b.r, a.g + b.g, a.b + b.b); }
static inline c3 c3_mul(c3 a, c3 b) { return mkc(a.r * b.r, a.g * b.g, a.b * b.b); }
static inline c3 c3_muls(c3 a, float s) { return mkc(a.r * s, a.g * s, a.b * s); }
static inline c3 c3_divs(c3 a, float s) { return mkc(a.r / s, a.g / s, a.b / s); }
static inline c3 c3_div(c3 a, c3 b) { return mkc(a.r / b.r, a.g / b.g, a.b / b.b); }
/* core/Color.h:151-158 average(): sum from 0 in channel order, then / 3 */
static inline float c3_avg(c3 a) { float s = 0.f; s += a.r; s += a.g; s += a.b; return s / 3.f; }
/* core/Color.h:423-426 */
static inline float c3_lum(c3 a) { return 0.2126f * a.r + 0.7152f * a.g + 0.0722f * a.b; }
/* core/Color.h:163-171 isZero(1e-5): all |c| <= 1e-5 */
static inline int c3_iszero(c3 a) { return fabsf(a.r) <= 1e-5f && fabsf(a.g) <= 1e-5f && fabsf(a.b) <= 1e-5f; }
static inline int c3_isnan(c3 a) { return isnan(a.r) || isnan(a.g) || isnan(a.b); }
/* core/Color.h max(): math::max(c0, c1, c2) = std::max(c0, std::max(c1, c2)) */
static inline float c3_max(c3 a) { return smax(a.r, smax(a.g, a.b)); }
static inline c3 c3_from(const float *p) { return mkc(p[0], p[1], p[2]); }
static inline v3 v3_from(const float *p) { return mk3(p[0], p[1], p[2]); }

/* ---------------- transforms (core/Transform.h:90-99,118-125) ---------------- */
v3 xf_point(const float *m, v3 p);
v3 xf_vector(const float *m, v3 v);
/* normal transform: transpose of the inverse's 3x3 (Transform.h:181-189) */
v3 xf_normal(const float *inv, v3 n);

/* ---------------- PCG32 (tools/Rng.h:81-141) ---------------- */
typedef struct { uint64_t state, inc; } o_pcg32;
void o_pcg_seed(o_pcg32 *r, uint64_t initstate, uint64_t initseq);
uint32_t o_pcg_next(o_pcg32 *r);
float o_pcg_float(o_pcg32 *r);
uint64_t o_mix64(uint64_t x);

typedef struct { o_pcg32 rng; } o_sampler;
void o_sampler_seed_path(o_sampler *s, uint64_t seed, uint32_t pixel, uint32_t sample);
float o_next1d(o_sampler *s);
v2 o_next2d(o_sampler *s);

/* ---------------- CDF (core/CDF.h:8-92) ---------------- */
typedef struct { float *cdf; int n; int cap; float sum; int normalized; } o_cdf;
void o_cdf_init(o_cdf *c);
void o_cdf_free(o_cdf *c);
void o_cdf_add(o_cdf *c, float pdf);
void o_cdf_normalize(o_cdf *c);
int o_cdf_sample(const o_cdf *c, float u);
int o_cdf_sample_pdf(const o_cdf *c, float u, float *pdf);
int o_cdf_sample_reuse(const o_cdf *c, float *u);
int o_cdf_sample_reuse_pdf(const o_cdf *c, float *u, float *pdf);

/* ---------------- scene (flattened, host) ---------------- */
typedef struct o_bvh o_bvh;

typedef struct {
    o_cdf cdf;              /* triangle area CDF (Mesh.cpp:19-31)          */
    float area;             /* mySurfaceArea                                */
} o_mesh_rt;

typedef struct {
    /* environment light (EnvironmentLight.cpp:8-73) */
    o_cdf *row;             /* H row CDFs                                   */
    o_cdf marginal;
    float *weight;          /* sin weights per row                          */
    float sphere_radius;    /* EnvironmentLight::initialize                 */
    v3 center;
} o_env_rt;

typedef struct {
    /* Heterogeneous medium derived data (Heterogeneous.cpp:281-369) */
    float world_to_array[16];
    float array_to_world[16];
    float wbox_min[3], wbox_max[3];
    float max_sigma_t;
} o_medium_rt;

typedef struct o_scene {
    const rt_scene_desc *d;
    int *tri_mesh;          /* mesh of each triangle                        */
    o_mesh_rt *mesh;
    o_env_rt *env;          /* per light (only env lights filled)           */
    o_medium_rt *med;
    o_cdf light_cdf;        /* Integrator::myLightWeights                   */
    float bmin[3], bmax[3]; /* scene bounding box                           */
    o_bvh *top;             /* two-level BVH (Scene.cpp:117, MeshFactory.h:123) */
    int strategy;
} o_scene;

/* BSDF sample record (bsdf/BSDF.h BSDFSamplingInfos) */
typedef struct {
    v3 wi, wo;
    int sampled_type;
    float relative_eta;
    float pdf;
} o_bsdf_rec;

enum { O_BSDF_UNKNOWN = 0, O_BSDF_DIFFUSE_REFLECTION = 1, O_BSDF_DELTA_REFLECTION = 2,
       O_BSDF_GLOSSY_REFLECTION = 4, O_BSDF_DELTA_TRANSMISSION = 8,
       O_BSDF_GLOSSY_TRANSMISSION = 0x10, O_BSDF_DIFFUSE = 0x200,
       O_BSDF_DELTA = 2 | 8, O_BSDF_ALL = (1 | 2 | 4) | (8 | 4) };

/* ImageTextures (texture/ImageTexture.cpp): the BSDF at a hit, with its
 * textured parameters replaced by their values at uv.  Returns b itself when
 * it has no texture, else `tmp` filled in. */
const rt_bsdf_desc *o_bsdf_at(const rt_scene_desc *d, const rt_bsdf_desc *b, v2 uv, rt_bsdf_desc *tmp);
c3 o_tex_eval(const rt_texture_desc *t, v2 uv);

c3 o_bsdf_eval(const rt_bsdf_desc *b, const o_bsdf_rec *r);
float o_bsdf_pdf(const rt_bsdf_desc *b, const o_bsdf_rec *r);
/* aux_key: the side-stream key of a LayeredBSDF sample (o_ly_sample) */
c3 o_bsdf_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s, uint64_t aux_key);

/* light sample record (light/Light.h LightSamplingInfos) */
typedef struct {
    v3 point, to_light, normal;
    c3 intensity;
    float distance, pdf;
    int light;
} o_light_rec;

void o_light_sample(const o_scene *sc, int light, v3 p, v2 s, o_light_rec *out);
float o_light_pdf(const o_scene *sc, int light, v3 p, const o_light_rec *rec);
int o_light_is_delta(const o_scene *sc, int light);   /* Light::isDelta */
c3 o_env_le(const o_scene *sc, int light, v3 dir);

/* ---------------- ray / intersection ---------------- */
typedef struct { v3 o, d, inv; float mint, maxt; } o_ray;
o_ray o_ray_make(v3 o, v3 d, float mint, float maxt);
/* Sphere::intersection's uv (Sphere.cpp:98-104): spherical angles of the
 * object-space hit point of ray r at t */
v2 o_sphere_uv(const rt_sphere_desc *sp, const o_ray *r, float t);

typedef struct {
    float t; float u, v;
    int prim;               /* triangle index, -(sphere)-2 for spheres, -1 none */
    v3 p;                   /* hit point                                    */
    v3 ng;                  /* true normal                                  */
    v3 n, s, tt;            /* shading frame (N, S, T)                      */
    v2 uv;                  /* texture coordinates (Intersection::myUv)     */
} o_hit;

o_bvh *o_bvh_build_scene(const o_scene *sc);
int32_t oracle_export_bvh(const o_scene *sc, rt_bvh_node *nodes, int32_t cap_nodes, int32_t *prims,
                          int32_t cap_prims, int32_t *n_nodes, int32_t *n_prims);
void o_bvh_free(o_bvh *b);
int o_intersect(const o_scene *sc, const o_ray *ray, o_hit *hit, int shadow);
int o_bvh_node_count(const o_bvh *b);
void o_bvh_root_box(const o_bvh *b, float *out6);

/* ---------------- camera (camera/NoriPerspective.cpp:80-118) ---------------- */
o_ray o_camera_ray(const rt_camera_desc *c, float px, float py, v2 lens);

/* ---------------- media ---------------- */
int o_medium_sample_distance(const o_scene *sc, int m, const o_ray *ray, o_sampler *s,
                             float *t, c3 *weight, c3 *emission);
c3 o_medium_transmittance(const o_scene *sc, int m, const o_ray *ray, o_sampler *s);
float o_phase_sample(const rt_medium_desc *m, v3 wi, v2 u, v3 *wo, float *pdf);
float o_phase_eval(const rt_medium_desc *m, v3 wi, v3 wo);
float o_sphere_light_pdf(const rt_sphere_desc *s, v3 p, v3 sampled, v3 n);
float o_plane_area(const rt_sphere_desc *s);
v3 o_plane_normal(const rt_sphere_desc *s);

/* ---------------- public oracle API (ctypes) ---------------- */
int32_t oracle_version(void);
o_scene *oracle_scene_create(const rt_scene_desc *d, int32_t strategy);
void oracle_scene_destroy(o_scene *sc);
int32_t oracle_scene_info(const o_scene *sc, float bounds[6], int32_t *nodes);
int32_t oracle_render(o_scene *sc, const rt_render_desc *rd, float *film_rgbw, int32_t nthreads);
int32_t oracle_render_tiles(o_scene *sc, const rt_render_desc *rd, int32_t tile0, int32_t tile1,
                            float *film_rgbw, int32_t nthreads);
int32_t oracle_render_tiles_strided(o_scene *sc, const rt_render_desc *rd, int32_t tile0, int32_t count,
                                    int32_t stride, float *film_rgbw, int32_t nthreads);
int32_t oracle_render_paths(o_scene *sc, const rt_render_desc *rd, const int32_t *pixels,
                            const int32_t *samples, int32_t n, float *rad_out);
int32_t oracle_trace(const o_scene *sc, const rt_ray *rays, int32_t n, int32_t anyhit, rt_hit *hits);
int32_t oracle_bsdf_query(const rt_bsdf_desc *b, int32_t op, const rt_bsdf_q *q, int32_t n,
                          rt_bsdf_r *r);
int32_t oracle_light_query(const o_scene *sc, int32_t light, const rt_light_q *q, int32_t n,
                           rt_light_r *r);
/* Medium::sampleDistance / Medium::transmittance for n ray segments, each
 * drawing from the path stream (seed, pixel, sample) (rt_medium_query). */
int32_t oracle_medium_query(const o_scene *sc, int32_t medium, int32_t op, const rt_medium_q *q, int32_t n,
                            rt_medium_r *r);
/* pin hooks: single functions of the restatement, for comparison with the
 * reference's own (oracle_core.c, oracle_bvh.c) */
int32_t oracle_tri_query(const float *tri_v, const rt_ray *rays, int32_t n, rt_hit *hits);
int32_t oracle_fresnel_query(int32_t op, const float *in, int32_t n, float *out);
int32_t oracle_mapping_query(int32_t op, const float *u, int32_t n, float *out);
int32_t oracle_microfacet_query(int32_t type, int32_t op, float alpha, const float *in, int32_t n, float *out);
int32_t oracle_phase_query(float g, int32_t op, const float *in, int32_t n, float *out);
int32_t oracle_env_sphere(const o_scene *sc, int32_t light, float *out4);
void oracle_pcg_stream(uint64_t initstate, uint64_t initseq, int32_t n, uint32_t *out);
void oracle_cdf_sample_reuse(const float *pdfs, int32_t n, const float *u, int32_t m,
                             int32_t *index, float *u_out, float *pdf_out, float *sum_out);
void oracle_cdf_sample(const float *pdfs, int32_t n, const float *u, int32_t m, int32_t *index, float *pdf_out);
void oracle_pcg_reals(uint64_t initstate, uint64_t initseq, int32_t n, float *out);
void oracle_camera_rays(const rt_scene_desc *d, const float *pxy, const float *lens, int32_t n,
                        rt_ray *out);

#ifdef __cplusplus
}
#endif
#endif
