/*
 * rtgpu.h -- C ABI of the GB300 light-transport core (librtgpu.so).
 *
 * The library replaces the per-sample render loop of Iscandel/Raytracer for
 * its two path-tracing integrators (PathTracingMIS, VolPathTracing).  A host
 * plugin flattens an initialised reference Scene into the plain structs below
 * and calls these entry points; nothing here uses C++ types, exceptions or
 * torch types.  Every entry point returns an rt_status; rt_last_error()
 * returns a thread-local description of the last failure.
 *
 * Reference interfaces each entry point stands in for (paths relative to
 * RaytracerNew2/src):
 *   rt_scene_create  Scene::initialize              core/Scene.cpp:115-138
 *                    (Bvh build Bvh.cpp:51-79, light init
 *                     EnvironmentLight.cpp:256-262, Integrator::initialize
 *                     integrator/Integrator.cpp:24-38, Mesh CDF Mesh.cpp:8-32,
 *                     Heterogeneous::setOwnerBBox Heterogeneous.cpp:281-369)
 *   rt_render        Scene::compute render step     core/Scene.cpp:83-101
 *                    + SampleJob::run               core/SampleJob.cpp:28-72
 *                    + Integrator::li (PathTracingMIS.cpp:27-262,
 *                      VolPathTracing.cpp:25-367)
 *                    + Screen::addSample/merge      core/Screen.cpp:44-97,136-157
 *   rt_trace         Scene::computeIntersection     core/Scene.cpp:106-113
 *                    (Bvh::intersection Bvh.cpp:392-481)
 *   rt_bsdf_query    BSDF::eval/sample/pdf          bsdf/BSDF.h
 *   rt_light_query   Light::sample/pdf/le           light/Light.h
 *   rt_medium_query  Medium::sampleDistance/transmittance  medium/Medium.h
 */
#ifndef RTGPU_H
#define RTGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTGPU_ABI_VERSION 1

typedef int32_t rt_status;
enum {
    RT_OK = 0,
    RT_ERR_INVALID = 1,     /* bad argument or malformed scene            */
    RT_ERR_CUDA = 2,        /* a CUDA runtime call failed                 */
    RT_ERR_LIMIT = 3,       /* a device loop hit its iteration cap        */
    RT_ERR_NOMEM = 4,       /* device or host allocation failed           */
    RT_ERR_UNSUPPORTED = 5  /* feature not provided by this build         */
};

/* ------------------------------------------------------------------ */
/* Scene description (host memory, caller-owned, read during create)  */
/* All matrices are 4x4 row-major float[16], applied to column        */
/* vectors exactly as core/Transform.h:90-99 applies them.            */
/* ------------------------------------------------------------------ */

enum { RT_BSDF_DIFFUSE = 0, RT_BSDF_ROUGH_CONDUCTOR = 1,
       RT_BSDF_ROUGH_DIELECTRIC = 2, RT_BSDF_SMOOTH_LAYERED = 3,
       RT_BSDF_LAYERED = 4,
       /* smooth (delta) BSDFs: bsdf/Dielectric.cpp, Conductor.cpp, Mirror.cpp.
        * Dielectric reads reflectance, transmittance, eta_int and eta_ext;
        * Conductor reads reflectance, eta and k; Mirror reads nothing. */
       RT_BSDF_DIELECTRIC = 5, RT_BSDF_CONDUCTOR = 6, RT_BSDF_MIRROR = 7,
       /* bsdf/SheetDielectric.cpp (reflectance, transmittance, eta_int,
        * eta_ext) and bsdf/Microfacet.cpp (albedo = kd, alpha, eta_int,
        * eta_ext, distribution, ks = probabilitySpecular) */
       RT_BSDF_SHEET_DIELECTRIC = 8, RT_BSDF_MICROFACET = 9 };
/* bsdf/MicrofacetDistribution.h:9-13 name order */
enum { RT_DIST_BECKMANN = 0, RT_DIST_PHONG = 1, RT_DIST_GGX = 2 };

typedef struct rt_bsdf_desc {
    int32_t type;            /* RT_BSDF_*                                        */
    int32_t distribution;    /* RT_DIST_* (rough conductor / dielectric)         */
    float albedo[3];         /* Diffuse albedo; SmoothLayered: base Diffuse albedo */
    float reflectance[3];    /* "reflectanceTexture" (constant), default 1       */
    float transmittance[3];  /* "transmittedTexture" (constant), default 1       */
    float eta[3];            /* RoughConductor eta                               */
    float k[3];              /* RoughConductor absorption                        */
    float alpha;             /* "alpha" (constant texture), default 0.2          */
    float eta_int;           /* default 1.5046                                   */
    float eta_ext;           /* default 1.000277                                 */
    float thickness;         /* SmoothLayered / Layered, default 1.2             */
    float absorbance[3];     /* SmoothLayered / Layered, default 0               */
    /* LayeredBSDF (bsdf/LayeredBSDF.cpp:17-36): `distribution` (default ggx) and
     * `alpha` ("alphaTop", default 0.01) describe the coat; the base
     * RoughConductor takes eta, k, reflectance and these two: */
    int32_t distribution_base; /* default beckmann                               */
    float alpha_base;          /* default 0.2                                    */
    /* 1: wrapped in a TwoSides (bsdf/TwoSides.cpp) with this BSDF on both
     * sides (the one-child form, where "bsdf2" defaults to "bsdf") */
    int32_t two_sided;
    /* ImageTextures replacing the constants above at each hit's texture
     * coordinates: index + 1 into rt_scene_desc.textures, 0 = the constant.
     * albedo: Diffuse, Microfacet (kd); reflectance: RoughConductor,
     * RoughDielectric, Dielectric, Conductor, SheetDielectric; transmittance:
     * RoughDielectric, Dielectric, SheetDielectric;
     * alpha (the texel's channel average): RoughConductor, RoughDielectric. */
    int32_t tex_albedo, tex_reflectance, tex_transmittance, tex_alpha;
    float ks;                /* Microfacet "probabilitySpecular", default 1      */
} rt_bsdf_desc;

/* ImageTexture (texture/ImageTexture.cpp:8-70): a linear RGB image as
 * ImageLoader::load leaves it (8-bit images decoded from sRGB, HDR images
 * as stored), indexed (x, y) = rgb[3 * (x + y * width)], looked up with the
 * reference's wrap and bilinear rules (math::interp2, core/BasicMath.h). */
typedef struct rt_texture_desc {
    int32_t width, height;
    const float *rgb;
    float scale;             /* "scale" (its absolute value), default 1          */
    int32_t invert_x;        /* "invertX", default 0                             */
    int32_t invert_y;        /* "invertY", default 0                             */
} rt_texture_desc;

/* One reference Mesh (factory/MeshFactory.h:39-139): a contiguous range of
 * triangles with one BSDF, an optional area light and its media. */
typedef struct rt_mesh_desc {
    int32_t first_tri;
    int32_t n_tris;
    int32_t bsdf;            /* index into bsdfs, -1 = no BSDF (null boundary)   */
    int32_t light;           /* index into lights, -1 = not emissive             */
    int32_t interior;        /* index into media, -1 = none                      */
    int32_t exterior;        /* index into media, -1 = none                      */
} rt_mesh_desc;

/* Analytic shapes, listed in rt_scene_desc.spheres: a Sphere
   (geometricShape/Sphere.cpp), object space centred at 0, or a Plane
   (geometricShape/Plane.cpp), the object-space square [-1,1]^2 at z = 0 with
   normal +z.  Hits on entry i carry prim = -i - 2.                            */
enum { RT_ANALYTIC_SPHERE = 0, RT_ANALYTIC_PLANE = 1 };
typedef struct rt_sphere_desc {
    float radius;            /* Sphere only                                      */
    float to_world[16];
    float to_object[16];     /* inverse of to_world                              */
    int32_t bsdf, light, interior, exterior;
    int32_t kind;            /* RT_ANALYTIC_* (0 for a zero-filled entry: sphere) */
} rt_sphere_desc;

enum { RT_LIGHT_AREA = 0,    /* AreaLight / MeshLight bound to a shape           */
       RT_LIGHT_ENV = 1,     /* EnvironmentLight (lat-long map)                  */
       RT_LIGHT_POINT = 2,   /* PointLight (light/PointLight.cpp), delta         */
       RT_LIGHT_SPOT = 3 };  /* SpotLight (light/SpotLight.cpp), delta           */
enum { RT_SHAPE_MESH = 0,
       RT_SHAPE_SPHERE = 1 };  /* an entry of spheres[]: a Sphere or a Plane      */

typedef struct rt_light_desc {
    int32_t type;            /* RT_LIGHT_*                                       */
    int32_t mesh_light;      /* 1: MeshLight::sample (light/MeshLight.cpp:32-64),
                                0: AreaLight::sample (light/AreaLight.cpp:31-55) */
    int32_t shape_kind;      /* RT_SHAPE_*                                       */
    int32_t shape;           /* mesh or sphere index                             */
    float radiance[3];
    /* environment map: width*height RGB floats, row-major (y*W+x)              */
    int32_t env_width, env_height;
    const float *env_rgb;
    float env_scale;         /* "scale"                                          */
    float env_to_world[16];  /* "toWorld"                                        */
    float env_to_light[16];  /* inverse of env_to_world                          */
    /* PointLight / SpotLight: sample() returns intensity / distance^2 with pdf
       1, and pdf() is 0 (they cannot be hit).                                  */
    float position[3];       /* PointLight "position"; SpotLight toWorld (0,0,0) */
    float intensity[3];      /* "intensity"                                      */
    float spot_to_light[16]; /* SpotLight: inverse of "toWorld"                  */
    float cos_falloff_start; /* SpotLight: cos(falloffStart), default cos(30 deg)*/
    float cos_total_width;   /* SpotLight: cos(totalWidth), default cos(60 deg)  */
} rt_light_desc;

enum { RT_MEDIUM_HOMOGENEOUS = 0, RT_MEDIUM_HETEROGENEOUS = 1 };
enum { RT_PHASE_ISOTROPIC = 0, RT_PHASE_HG = 1 };

typedef struct rt_medium_desc {
    int32_t type;            /* RT_MEDIUM_*                                      */
    int32_t phase;           /* RT_PHASE_*                                       */
    float g;                 /* HG asymmetry                                     */
    float sigma_a[3];        /* Homogeneous                                      */
    float sigma_s[3];        /* Homogeneous                                      */
    float scale;             /* both types                                       */
    float albedo[3];         /* Heterogeneous                                    */
    int32_t res[3];          /* GridVolume resolution                            */
    const float *density;    /* res[0]*res[1]*res[2] floats, x fastest           */
    float grid_min[3];       /* GridVolume bounding box from the .vol header     */
    float grid_max[3];
    float to_world[16];      /* Heterogeneous "toWorld"                          */
    int32_t centered;        /* Heterogeneous "centered" (default 1)             */
} rt_medium_desc;

typedef struct rt_camera_desc {
    int32_t width, height;
    float sample_to_camera[16];  /* NoriPerspective.cpp:32-34                    */
    float camera_to_world[16];   /* Camera world transform                       */
    float near_clip, far_clip;
    float aperture_radius;       /* 0 = pinhole                                  */
    float focal_plane;
    int32_t medium;              /* camera medium or -1                          */
    /* reconstruction filter of the camera's screen (the filter/ sources): RT_FILTER_*,
     * radii "radiusX"/"radiusY" (default 0.5) and two parameters: Gaussian
     * "alpha", "omega" (GaussianFilter.cpp:16-17); Mitchell-Netravali "B", "C"
     * (MitchellNetravaliFilter.cpp:17-18) */
    int32_t filter;
    float filter_radius[2];
    float filter_param[2];
} rt_camera_desc;

enum { RT_FILTER_BOX = 0, RT_FILTER_GAUSSIAN = 1, RT_FILTER_MITCHELL = 2 };

typedef struct rt_scene_desc {
    int32_t n_vertices;
    const float *vertices;       /* 3 floats per vertex, world space             */
    const float *normals;        /* 3 floats per vertex or NULL (face normals);  
                                    a NaN x marks a vertex of a mesh without normals */
    int32_t n_triangles;
    const int32_t *indices;      /* 3 vertex indices per triangle                */
    int32_t n_meshes;
    const rt_mesh_desc *meshes;
    int32_t n_spheres;
    const rt_sphere_desc *spheres;
    int32_t n_bsdfs;
    const rt_bsdf_desc *bsdfs;
    int32_t n_lights;
    const rt_light_desc *lights; /* scene light order (Scene::getLights)          */
    int32_t env_light;           /* index of the environment light or -1         */
    int32_t n_media;
    const rt_medium_desc *media;
    rt_camera_desc camera;
    int32_t n_textures;
    const rt_texture_desc *textures;
    const float *uvs;            /* 2 floats per vertex or NULL; a NaN u marks a
                                    vertex of a mesh without texture coordinates
                                    (its hits use their barycentric (u, v),
                                    Triangle.cpp:155-170) */
} rt_scene_desc;

/* ------------------------------------------------------------------ */
/* Render description                                                  */
/* ------------------------------------------------------------------ */
enum { RT_INTEGRATOR_PATH_MIS = 0, RT_INTEGRATOR_VOLPATH = 1 };
/* integrator/Integrator.h:11-15 strategy names.  ALL_LIGHTS: PathTracingMIS
 * samples every light at every vertex (PathTracingMIS.cpp:80-117);
 * VolPathTracing then selects one light uniformly, as the reference does. */
enum { RT_STRATEGY_ALL_LIGHTS = 0, RT_STRATEGY_ONE_LIGHT_UNIFORM = 1,
       RT_STRATEGY_ONE_LIGHT_WEIGHTED = 2 };

typedef struct rt_render_desc {
    int32_t integrator;      /* RT_INTEGRATOR_*                                  */
    int32_t max_depth;       /* "maxDepth" (default 1000)                        */
    int32_t min_depth;       /* "minDepth" (default 3)                           */
    int32_t strategy;        /* RT_STRATEGY_*                                    */
    int32_t spp;             /* samples per pixel rendered by this call          */
    int32_t sample_begin;    /* first sample index (progressive rendering)       */
    uint64_t seed;           /* path-stream sampler seed                         */
    int32_t block_x, block_y;/* tile size of the reference job grid (default 32) */
    int32_t flags;           /* RT_RENDER_* bits, 0 for a plain render           */
} rt_render_desc;

/* rt_render_desc.flags: add this call's (rgb sum, weight) to the film instead
 * of overwriting it, for progressive rendering over disjoint sample ranges.
 * Not part of the reference: there Screen::addSample always accumulates
 * into one film per render (core/Screen.cpp:44-80). */
#define RT_RENDER_ACCUMULATE 1

/* Per-path sample stream ("PathStreamSampler"): path (pixel p, sample s)
 * draws from a PCG32 (tools/Rng.h:81-141) seeded with
 *   initstate = rt_mix64((seed << 32) ^ p), initseq = s
 * where p = y*width + x and rt_mix64 is the splitmix64 finaliser.  The
 * draw order per path follows SampleJob.cpp:49-58 and the integrators. */

typedef struct rt_ray {
    float o[3]; float mint;
    float d[3]; float maxt;
} rt_ray;

typedef struct rt_hit {
    float t;
    float u, v;              /* barycentrics of the hit (Triangle.cpp:73,78)     */
    int32_t prim;            /* triangle index, or -(sphere index)-2, -1 = miss  */
} rt_hit;

/* BSDF point queries in the local shading frame (test hook). */
enum { RT_BSDF_OP_EVAL = 0, RT_BSDF_OP_PDF = 1, RT_BSDF_OP_SAMPLE = 2 };
typedef struct rt_bsdf_q {
    float wi[3];
    float wo[3];             /* eval / pdf                                       */
    float u[2];              /* sample                                           */
} rt_bsdf_q;
typedef struct rt_bsdf_r {
    float value[3];          /* eval value, or sample weight                     */
    float pdf;
    float wo[3];             /* sampled direction                                */
    float relative_eta;
    int32_t sampled_type;    /* BSDF::BSDFType bits (bsdf/BSDF.h)                */
    int32_t pad;
} rt_bsdf_r;

/* Light queries (test hook): sample light `light` from point p with u. */
typedef struct rt_light_q {
    float p[3];
    float u[2];
} rt_light_q;
typedef struct rt_light_r {
    float intensity[3];
    float pdf;
    float to_light[3];
    float distance;
    float point[3];
    float normal[3];
    float pdf_eval;          /* Light::pdf(p, infos) for the sampled point       */
    float pad;
} rt_light_r;

/* Medium queries (test hook): Medium::sampleDistance or
 * Medium::transmittance (medium/Medium.h, Homogeneous.cpp:30-78,
 * Heterogeneous.cpp:419-546) for a ray segment, drawing from the per-path
 * sample stream of (seed, pixel, sample). */
enum { RT_MEDIUM_OP_SAMPLE = 0, RT_MEDIUM_OP_TRANSMITTANCE = 1 };
typedef struct rt_medium_q {
    float o[3]; float mint;
    float d[3]; float maxt;
    uint64_t seed;
    uint32_t pixel, sample;
} rt_medium_q;
typedef struct rt_medium_r {
    float weight[3];         /* sample: MediumSamplingInfos weight; else Tr     */
    float t;                 /* sample: distance reached (scatter point or maxT) */
    int32_t scattered;       /* sample: 1 when the ray scattered in the medium  */
    int32_t limit;           /* 1 when a tracking loop reached its cap          */
} rt_medium_r;

typedef struct rt_render_stats {
    double kernel_ms;        /* device time of the last render (events)          */
    double camera_ms;        /* per-kernel device time, summed over launches;    */
    double trace_closest_ms; /* filled when profiling is enabled                 */
    double trace_any_ms;
    double shade_ms;
    double volpath_ms;
    double film_ms;
    int64_t paths;           /* path samples rendered                            */
    int64_t closest_rays;    /* closest-hit rays traced                          */
    int64_t shadow_rays;     /* any-hit rays traced                              */
    int64_t launches;        /* kernels launched by the last render              */
    int64_t trace_closest_launches;
    int64_t trace_any_launches;
    int64_t nodes_closest;   /* BVH nodes fetched by closest-hit rays (level 2)  */
    int64_t tris_closest;    /* triangle slots tested by closest-hit rays        */
    int64_t nodes_any;       /* ... by any-hit rays                              */
    int64_t tris_any;
    int64_t limit_hits;      /* device loops that hit their cap                  */
    int64_t nan_samples;     /* samples dropped as NaN (Screen.cpp:46-50)        */
    double resolve_ms;       /* part of shade_ms spent in the resolve kernel     */
    double sort_ms;          /* ray reordering before the traces                 */
} rt_render_stats;

typedef struct rt_ctx rt_ctx;
typedef struct rt_scene rt_scene;

/* Library ------------------------------------------------------------ */
int32_t rt_abi_version(void);
const char *rt_last_error(void);
uint64_t rt_mix64(uint64_t x);

/* Context: one device, one CUDA stream.  Not thread-safe. */
rt_status rt_ctx_create(int32_t device, rt_ctx **out);
rt_status rt_ctx_destroy(rt_ctx *ctx);
/* Optional stream override (cudaStream_t passed as an opaque pointer). */
rt_status rt_ctx_set_stream(rt_ctx *ctx, void *stream);

/* Scene: flatten + BVH build on the host, upload to device memory. */
rt_status rt_scene_create(rt_ctx *ctx, const rt_scene_desc *desc, rt_scene **out);
rt_status rt_scene_destroy(rt_scene *scene);
/* Scene axis-aligned bounds (min xyz, max xyz) and device bytes held. */
rt_status rt_scene_info(const rt_scene *scene, float bounds[6], int64_t *device_bytes,
                        int32_t *bvh_nodes);

/* Render spp samples per pixel starting at sample_begin; film_rgbw receives
 * width*height*4 floats (rgb sum, weight), accumulated in sample order, in
 * host memory (on_device = 0) or device memory (on_device = 1).  The film is
 * overwritten unless rd->flags has RT_RENDER_ACCUMULATE. */
rt_status rt_render(rt_ctx *ctx, rt_scene *scene, const rt_render_desc *rd,
                    float *film_rgbw, int32_t on_device);
rt_status rt_render_stats_get(const rt_ctx *ctx, rt_render_stats *out);
/* Radiance (3 floats each) of n path samples: pixel index y * width + x and
 * absolute sample index, drawn from the same per-path streams and traced
 * through the same kernels as rt_render.  Stands in for Integrator::li
 * (integrator/Integrator.h:68) called per sample by SampleJob::run
 * (core/SampleJob.cpp:46-61): a plugin's li() issues a 1-path launch of the
 * sample it is asked for.  Not a film: nothing is reduced or splatted. */
rt_status rt_render_paths(rt_ctx *ctx, rt_scene *scene, const rt_render_desc *rd,
                          const int32_t *pixels, const int32_t *samples, int32_t n, float *rgb);
/* Profiling level of later renders: 0 off, 1 per-kernel CUDA-event timing,
 * 2 timing plus BVH traversal counters (slower; for roofline accounting). */
rt_status rt_ctx_set_profiling(rt_ctx *ctx, int32_t level);
/* Tree used by later renders and rt_trace: 2 (binary BVH, the default), 4
 * (4-wide BVH collapsed from the binary one, same boxes) or 8 (compressed
 * 8-wide BVH); all report the same closest hits (a tie at equal distance may
 * name another triangle) and the same occlusion.  Stands in for the
 * reference's binary traversal, Bvh::intersection (accelStruct/Bvh.cpp:392-481). */
rt_status rt_ctx_set_bvh_width(rt_ctx *ctx, int32_t width);
/* Builder of the binary tree for scenes created later on this context:
 * RT_BUILDER_HOST_SAH (the default: binned SAH on the host, plus the 4- and
 * 8-wide trees) or RT_BUILDER_DEVICE (a linear BVH over Morton codes built on
 * the device in milliseconds, one triangle per leaf, no wide trees, slower
 * to traverse; for scenes that arrive with the job, as in serving).  A
 * device tree deeper than the traversal stack falls back to the host build.
 * Both give the same closest hits (a tie at equal distance may name another
 * triangle).  Stands in for Bvh::build (accelStruct/Bvh.cpp:51-79). */
enum { RT_BUILDER_HOST_SAH = 0, RT_BUILDER_DEVICE = 1 };
rt_status rt_ctx_set_bvh_builder(rt_ctx *ctx, int32_t builder);
/* Paths per wavefront batch of later renders (whole tiles x all samples are
 * batched up to this count): 2^16..2^26.  Device memory for path state is
 * about 240 bytes per path. */
rt_status rt_ctx_set_wave_paths(rt_ctx *ctx, int32_t paths);
/* Regroup the rays of every bounce after the first by direction octant and
 * origin cell before tracing them (0 off, 1 on); results are unchanged. */
rt_status rt_ctx_set_ray_sort(rt_ctx *ctx, int32_t on);
/* Launch each PathTracingMIS wavefront batch of later renders as one CUDA
 * graph (0 off, 1 on): camera rays, the bounce rounds as a device-controlled
 * conditional loop (it stops when no path is left, with no host round trip)
 * and the film reduction.  Graphs are kept and reused for renders with
 * identical parameters.  Renders with profiling or ray sorting on launch
 * kernel by kernel.  Results are identical either way. */
rt_status rt_ctx_set_graphs(rt_ctx *ctx, int32_t on);

/* Launch shapes, queue capacities and scheduling choices of later renders.
 * None of them changes a result: a film is the same bit for bit under any
 * tuning.  (The tile size, blockSizeX/Y of the scene file, is not among
 * them: it decides which neighbours a sample on a pixel edge reaches.) */
typedef struct rt_tuning {
    int32_t wave_paths;          /* paths per wavefront batch of this context's
                                    renders (queue capacity), 2^16..2^26     */
    int32_t lane_wave_paths;     /* the same for each lane of rt_batch_render
                                    and of servers started from the context   */
    int32_t trace_blocks_per_sm; /* traversal grid: 128-thread blocks per SM,
                                    1..64                                      */
    int32_t shade_blocks_per_sm; /* finish and shading grid, 1..64            */
    int32_t sort_threshold;      /* bounces with fewer closest-hit rays than
                                    this shade in one unsorted queue instead
                                    of per-material queues (0: always sorted) */
    int32_t lanes;               /* worker lanes of rt_batch_render, 1..16    */
    int32_t graphs;              /* one CUDA graph per batch, 0 or 1          */
    int32_t volpath_wavefront;   /* VolPathTracing as a wavefront of kernels
                                    over queues (1, the default) or as one
                                    persistent kernel per path (0)            */
    int32_t batch_wavefront;     /* rt_batch_render: the PathTracingMIS jobs
                                    (box filter) in one wavefront whose path
                                    slots span their scenes, batches of up to
                                    wave_paths (1, the default), or every job
                                    as its own render on the lanes (0)        */
} rt_tuning;
rt_status rt_ctx_get_tuning(rt_ctx *ctx, rt_tuning *out);
rt_status rt_ctx_set_tuning(rt_ctx *ctx, const rt_tuning *t);

/* Autotuner.  Searches rt_tuning for the fastest rt_batch_render of the
 * given jobs (a representative sample of a workload, e.g. a few of its jobs
 * at reduced spp) by coordinate descent over a fixed candidate grid, with at
 * most max_trials timed trials (each one untimed warm-up and the best of two
 * timed runs).  The jobs render into scratch device films.  The best tuning
 * is left set on the context and returned with its measured path samples
 * per second (samples_per_s may be null). */
rt_status rt_autotune(rt_ctx *ctx, rt_scene *const *scenes, const rt_render_desc *descs, int32_t n,
                      int32_t max_trials, rt_tuning *best, double *samples_per_s);

/* Allocation-free tile render.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory while rendering (plugins
 * whose host application owns the device memory through its own pool under
 * a hard budget, real-time loops that forbid cudaMalloc/cudaFree after
 * start-up because they can synchronise the device).  Renders every sample
 * of tile (tile_x, tile_y) of the block_x x block_y job grid into
 * film_rgbw_device (a device pointer to the full width*height*4 film; only
 * the tile's pixels are written, or added to with RT_RENDER_ACCUMULATE),
 * with the same results as rt_render for those pixels.
 * Limits: tile pixels * spp * ~240 bytes of path state must fit the 32 MiB
 * static scratch (about 130k path samples, e.g. 32x32 at 128 spp);
 * PathTracingMIS max_depth <= 1024; at most 256 lights; larger requests
 * return RT_ERR_LIMIT.  The call synchronises the context's stream, so that
 * stream must not be under stream capture (RT_ERR_UNSUPPORTED otherwise).
 * The first call on a device looks up the scratch address
 * (cudaGetSymbolAddress).  All calls on one device share the scratch and
 * keep its last contents: calls that overlap on the GPU (other threads or
 * streams) race. */
rt_status rt_render_tile_static(rt_ctx *ctx, rt_scene *scene, const rt_render_desc *rd,
                                int32_t tile_x, int32_t tile_y, float *film_rgbw_device);

/* Batched rendering: n independent jobs (scenes[i] rendered with descs[i]
 * into films[i], each width*height*4 floats on the host or, with
 * on_device = 1, on the device).  With rt_tuning.batch_wavefront (the
 * default), the PathTracingMIS jobs with the box filter of radius 0.5 that
 * share max_depth and min_depth run together as one wavefront: every batch
 * of up to wave_paths path slots holds whole tiles of several jobs, each
 * path carries its job's scene, and one launch per kernel per bounce serves
 * all of them.  Other jobs (VolPathTracing, other filters) run meanwhile as
 * one rt_render each, largest first, on up to rt_ctx_set_lanes() worker
 * lanes of the context's device (one stream, wavefront buffers and host
 * thread each).  Each film equals what rt_render writes for that job alone.
 * Returns after every job has finished; on failures the other jobs still
 * run and the first error is returned.  rt_render_stats_get then reports
 * the sums over the jobs, with kernel_ms the wall time of the batch.  The
 * reference renders one scene per process (core/main.cpp:439-447) and cuts
 * a frame into tile jobs (core/Scene.cpp:83-95); this call replaces a loop
 * of such runs. */
rt_status rt_batch_render(rt_ctx *ctx, rt_scene *const *scenes, const rt_render_desc *descs,
                          int32_t n, float *const *films, int32_t on_device);
/* Worker lanes of rt_batch_render: 1..16, default 4. */
rt_status rt_ctx_set_lanes(rt_ctx *ctx, int32_t lanes);

/* Served rendering, with continuous batching.  No counterpart in the
 * reference, which renders one scene per process.  PathTracingMIS jobs with
 * the box filter (rt_render's requirements for one multi-scene wavefront)
 * are admitted from the queue, in order, while the device budget allows:
 * a job holds its scene's device bytes (rt_scene_info) and its films (one,
 * or three for a progressive job) until it finishes, and the wavefront's
 * and lanes' path state count from the start.  A scheduler thread then runs
 * steps: each renders the next chunk of every admitted job together in one
 * wavefront (jobs that arrive meanwhile join at the next step), updates the
 * progressive estimates and retires finished jobs.  Other jobs run on worker
 * lanes (one stream, wavefront buffers and host thread each) under the same
 * budget. */
typedef struct rt_server rt_server;
typedef int64_t rt_job_id;
typedef struct rt_server_opts {
    int32_t lanes;                /* lanes for jobs the wavefront cannot take,
                                     1..16 (0: 4)                                   */
    int32_t max_queue;            /* queued jobs before submit fails (0: 4096)      */
    int64_t device_budget_bytes;  /* device memory of path state (the wavefront's
                                     slots and every lane's, at
                                     rt_path_state_bytes each), admitted jobs'
                                     scenes and films; 0 = unlimited               */
    int32_t lanes_only;           /* 0: continuous batching in one wavefront (the
                                     default); 1: every job on a lane               */
    int32_t rmse_display;         /* 0: target RMSE over the pixel means (linear
                                     radiance); 1: over the pixel means clipped to
                                     [0, 1] per channel, the range a display shows */
} rt_server_opts;
enum { RT_JOB_QUEUED = 0, RT_JOB_RUNNING = 1, RT_JOB_DONE = 2, RT_JOB_FAILED = 3 };
typedef struct rt_job_info {
    int32_t state;                /* RT_JOB_*                                       */
    int32_t spp_done;             /* samples per pixel in the film                  */
    float rmse_estimate;          /* progressive jobs: estimated RMSE, else -1     */
    float queue_ms, run_ms;       /* time queued, time rendering                    */
    char error[128];              /* RT_JOB_FAILED: rt_last_error of the job        */
} rt_job_info;
rt_status rt_server_start(rt_ctx *ctx, const rt_server_opts *opts, rt_server **out);
/* Device bytes of wavefront path state per path slot for an integrator
 * (RT_INTEGRATOR_*): the per-slot part of a render's working memory, and
 * what a server counts against its budget per slot (lanes at the
 * VolPathTracing figure, since a lane may take either kind of job).  0 for
 * an unknown integrator. */
int64_t rt_path_state_bytes(int32_t integrator);
/* Queue a render of `scene` (which must outlive the job).  A job whose
 * scene and films alone exceed the budget is refused (RT_ERR_LIMIT).
 * target_rmse <= 0: render desc->spp samples, the film equals rt_render's.  target_rmse > 0:
 * render progressively from desc->sample_begin, at most desc->spp samples,
 * until the RMSE of the film's pixel means (rgb / weight, over pixels and
 * channels) estimated from two half films falls to target_rmse. */
rt_status rt_job_submit(rt_server *srv, rt_scene *scene, const rt_render_desc *desc,
                        float target_rmse, rt_job_id *id);
/* Job state; when the job has finished and film is not NULL, copy its
 * width*height*4 floats to film (host memory) and release the job. */
rt_status rt_job_poll(rt_server *srv, rt_job_id id, rt_job_info *info, float *film);
/* As rt_job_poll after waiting up to timeout_ms (< 0: no limit) for the job. */
rt_status rt_job_wait(rt_server *srv, rt_job_id id, int32_t timeout_ms, rt_job_info *info,
                      float *film);
/* Finish running jobs, drop queued ones, release the lanes. */
rt_status rt_server_stop(rt_server *srv);

/* Trace n rays (closest hit, or any hit when anyhit != 0).  Returns
 * RT_ERR_LIMIT if a traversal had to drop a subtree (a stack was full); the
 * builder bounds the tree depth so that this does not happen. */
rt_status rt_trace(rt_ctx *ctx, rt_scene *scene, const rt_ray *rays, int32_t n,
                   int32_t anyhit, rt_hit *hits, int32_t on_device);

/* Move a resident scene's triangles: `vertices` holds new positions for all
 * of the scene's vertices (3 floats each, the count and order of
 * rt_scene_desc.vertices; `normals` likewise, required when and only when
 * the scene has vertex normals), in host memory or, with on_device = 1, in
 * device memory.  On the device, the triangle arrays are rewritten and the
 * binary tree's boxes are recomputed bottom-up over its unchanged topology
 * (widened as the build widens them), then the 4-wide tree's; the
 * compressed 8-wide tree is dropped (renders at width 8 use the binary
 * one).  Closest hits and occlusion afterwards equal those of a scene built
 * from the new positions (a tie at equal distance may name another
 * triangle); traversal slows as the positions drift from the ones the tree
 * was built for.  Refused (RT_ERR_UNSUPPORTED) for scenes with an emissive
 * mesh or a mesh bounding a grid medium, whose light CDFs or medium boxes
 * would change.  Stands in for rebuilding the scene: the reference rebuilds
 * every BVH per scene load (core/Scene.cpp:115-138). */
rt_status rt_scene_refit(rt_ctx *ctx, rt_scene *scene, const float *vertices, const float *normals,
                         int32_t on_device);
/* A binary BVH built by the caller, as topology: node i is internal when
 * count == 0 (children left, right), else a leaf over prims[first, first +
 * count) (indices of the scene's triangles, the order of rt_scene_desc's
 * indices).  Node 0 is the root; every node is reached once and every
 * triangle is in exactly one leaf. */
typedef struct rt_bvh_node {
    int32_t left, right, first, count;
} rt_bvh_node;
/* rt_scene_create with the caller's tree instead of the library's SAH build:
 * the device traverses the reference's own tree.  Stands in for Bvh::build
 * and Bvh::flatten (accelStruct/Bvh.cpp:51-79, 587-607) over the primitives
 * MeshFactory and Scene::initialize arrange in two levels
 * (factory/MeshFactory.h:123, core/Scene.cpp:117): the plugin flattens the
 * top-level tree with every mesh leaf replaced by that mesh's tree (analytic
 * spheres and planes are left out: they are tested after the tree).  Boxes
 * are recomputed from the triangles and widened as the library's own build
 * widens them; leaves of more than 8 triangles are split in halves of their
 * range; a tree deeper than 62 levels is refused (RT_ERR_INVALID), as is a
 * malformed one.  The 4-wide tree is collapsed from this one. */
rt_status rt_scene_create_bvh(rt_ctx *ctx, const rt_scene_desc *desc, const rt_bvh_node *nodes, int32_t n_nodes,
                              const int32_t *prims, int32_t n_prims, rt_scene **out);
/* Host-only check of such a tree over n triangles (9 floats each): the
 * device image rt_scene_create_bvh would upload, checked structurally; its
 * depth and internal node count.  Needs no GPU. */
rt_status rt_bvh_import_check(const float *tri_v, int32_t n, const rt_bvh_node *nodes, int32_t n_nodes,
                              const int32_t *prims, int32_t n_prims, int32_t *max_depth, int32_t *n_device_nodes);

/* Host-only: build the device tree (width 2: binary, 4: 4-wide collapsed
 * from the binary one, 8: compressed 8-wide) over n triangles (9 floats
 * each) as rt_scene_create would, and report its deepest level (root 0) and
 * node count; the binary and 4-wide trees are also checked structurally
 * (RT_ERR_INVALID if malformed).  Stands in for
 * Bvh::build (accelStruct/Bvh.cpp:51-79), whose traversal keeps a fixed
 * stack of 64 (Bvh.cpp:402): the builder here splits at the object median
 * wherever the SAH tree would grow deeper than depth_cap levels (<= 0: the
 * default 62, which rt_scene_create uses; at most 62; 2^depth_cap >= n), so
 * the traversal stacks cannot overflow.  Needs no GPU. */
rt_status rt_bvh_stats(const float *tri_v, int32_t n, int32_t width, int32_t depth_cap,
                       int32_t *max_depth, int32_t *n_nodes);

/* Evaluate BSDF `bsdf` of the scene for n queries (host arrays). */
rt_status rt_bsdf_query(rt_ctx *ctx, rt_scene *scene, int32_t bsdf, int32_t op,
                        const rt_bsdf_q *q, int32_t n, rt_bsdf_r *r);

/* Sample light `light` (Light::sample + Light::pdf) for n queries. */
rt_status rt_light_query(rt_ctx *ctx, rt_scene *scene, int32_t light,
                         const rt_light_q *q, int32_t n, rt_light_r *r);

/* Scene ingestion: a Wavefront OBJ file as the reference's ObjLoader reads
 * it (io/ObjLoader.cpp:97-290): positions and normals transformed by
 * to_world (row-major 4x4, NULL = identity), corners de-duplicated by their
 * (position, uv, normal) indices in order of first use, quads split into
 * (a b c) (d a c).  Arrays are allocated by the library (normals / uvs NULL
 * when the file has none); release them with rt_mesh_data_free. */
typedef struct rt_mesh_data {
    int32_t n_vertices;
    float *vertices;             /* 3 per vertex, world space                  */
    float *normals;              /* 3 per vertex or NULL                       */
    float *uvs;                  /* 2 per vertex or NULL                       */
    int32_t n_triangles;
    int32_t *indices;            /* 3 per triangle                             */
} rt_mesh_data;
rt_status rt_obj_load(const char *path, const float *to_world, rt_mesh_data *out);
void rt_mesh_data_free(rt_mesh_data *mesh);
/* A Radiance RGBE (.hdr) environment map as the reference reads it
 * (io/ImageLoader.cpp:78-99): width*height RGB floats, top row first, in a
 * library allocation released with rt_host_free. */
rt_status rt_hdr_load(const char *path, int32_t *width, int32_t *height, float **rgb);
void rt_host_free(void *p);

/* Sample or evaluate medium `medium` of the scene for n queries. */
rt_status rt_medium_query(rt_ctx *ctx, rt_scene *scene, int32_t medium, int32_t op,
                          const rt_medium_q *q, int32_t n, rt_medium_r *r);

#ifdef __cplusplus
}
#endif

#endif /* RTGPU_H */
