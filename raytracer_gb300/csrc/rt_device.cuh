// rt_device.cuh -- device-resident scene layout and the per-vertex physics
// of the reference renderer (BSDFs, lights, camera, media, ray casting).
//
// Reference paths are relative to RaytracerNew2/src of Iscandel/Raytracer.
// Each routine keeps the reference's operation order so that, fed the same
// sample stream, the device reproduces the CPU renderer's arithmetic
// (transcendental functions excepted: CUDA's expf/logf/sinf/... differ from
// the C library by at most a few ulp).
#pragma once
#include "rt_math.cuh"

// ------------------------------------------------------------------ layout
struct DevMesh {
    int first_tri, n_tris, bsdf, light, interior, exterior;
    int cdf_off;      // offset of this mesh's area CDF (n_tris + 1 floats)
    float area;       // Mesh::mySurfaceArea
};

// An analytic shape: kind 0 Sphere, kind 1 Plane (RT_ANALYTIC_*)
struct DevSphere {
    float radius;
    float to_world[16];
    float to_object[16];
    int bsdf, light, interior, exterior;
    int kind;
    float area;   // Plane: Plane::surfaceArea (Plane.cpp:13-17)
};

struct DevBsdf {
    int type, distribution;
    float albedo[3], reflectance[3], transmittance[3], eta[3], k[3];
    float alpha;      // raw "alpha" texture value
    float alpha_avg;  // Color(alpha).average() as the BSDFs read it
    float eta_int, eta_ext, thickness;
    float absorbance[3];
    // LayeredBSDF: its base RoughConductor's distribution and alpha (the
    // base's eta, k and reflectance use the fields above)
    int dist_base;
    float alpha_base_avg;
    int two_sided;    // wrapped in TwoSides (bsdf/TwoSides.cpp) with itself on both sides
    // ImageTextures (index into DevScene::textures, -1 = the constant) for
    // albedo, reflectance, transmittance and alpha; textured = any of them
    int tex[4];
    int textured;
    float ks;         // Microfacet "probabilitySpecular"
};
enum { TEX_ALBEDO = 0, TEX_REFLECTANCE = 1, TEX_TRANSMITTANCE = 2, TEX_ALPHA = 3 };

// ImageTexture (texture/ImageTexture.cpp): linear RGB texels, (x, y) at
// rgb[3 * (x + y * w)]
struct DevTexture {
    int w, h;
    const float *rgb;
    float scale;
    int invert_x, invert_y;
};

// Shading queue of a BSDF.  The heavy types (0-4) get a queue and a shading
// kernel each; the smooth (delta) types Dielectric, Conductor and Mirror
// (5-7) are cheap and share one; textured BSDFs of any type go to the mixed
// queue, whose kernel dispatches at run time and applies the textures.
#define RT_QUEUE_DELTA 5
#define RT_QUEUE_MIXED 6
__host__ __device__ __forceinline__ int bsdf_queue(int type) { return type < RT_QUEUE_DELTA ? type : RT_QUEUE_DELTA; }
// (Microfacet, type 9, shades from the mixed queue too)
__host__ __device__ __forceinline__ int bsdf_queue_of(const DevBsdf &b)
{
    return (b.textured || b.type == 9) ? RT_QUEUE_MIXED : bsdf_queue(b.type);
}

struct DevLight {
    int type, mesh_light, shape_kind, shape;
    float radiance[3];
    // environment map
    int env_w, env_h;
    float env_scale;
    const float *env_rgb;       // W*H*3
    const float *env_row_cdf;   // H * (W + 1)
    const float *env_marginal;  // H + 1
    const float *env_weight;    // H
    const int *env_marg_guide;  // env_gm + 1 entries (cdf_guide of env_marginal)
    const int *env_row_guide;   // H * (env_gr + 1) entries
    int env_gm, env_gr;         // guide cells, powers of two
    float env_marginal_sum;
    float env_radius;           // bounding sphere radius (EnvironmentLight::initialize)
    float env_to_world[16], env_to_light[16];
    // PointLight / SpotLight (type 2 / 3)
    float position[3], intensity[3];
    float spot_to_light[16];
    float cos_falloff_start, cos_total_width;
};

struct DevMedium {
    int type, phase;
    float g;
    float sigma_t[3], sigma_s[3];  // Homogeneous, scale applied (Homogeneous.cpp:16-22)
    float scale;
    float albedo[3];
    int res[3];
    const float *density;
    float world_to_array[16];
    float wbox_min[3], wbox_max[3];
    float max_sigma_t;
};

struct DevCamera {
    int width, height;
    float sample_to_camera[16], camera_to_world[16];
    float near_clip, far_clip, aperture_radius, focal_plane;
    float inv_w, inv_h;
    int medium;
    // reconstruction filter: type, radii, screen overlap (Screen::setFilter,
    // Screen.cpp:98-108) and the 32 x 32 weight table of
    // ReconstructionFilter::precompute (ReconstructionFilter.cpp:27-40)
    int filter, ov_x, ov_y;
    float frx, fry;
    const float *filter_table;
};

struct DevScene {
    // BVH2 (two child boxes per node, 64 B): see rt_bvh.cpp for the layout
    const float4 *nodes;
    const float4 *tri_slots;    // 3 float4 per leaf slot: (p0, id), (e1, 0), (e2, 0)
    int n_nodes;
    // 4-wide BVH collapsed from the BVH2 (128-byte nodes, see rt_bvh.h); its
    // leaves are the BVH2's triangle slots
    const float4 *nodes4;
    int n_nodes4;
    // compressed 8-wide BVH (80-byte nodes, see rt_bvh.h) and its triangle slots
    const float4 *wnodes;
    const float4 *wtri;
    int n_wnodes;
    // original geometry
    const float *tri_v;         // 9 floats per triangle (p0, p1, p2)
    const float *tri_n;         // 9 floats per triangle (n0, n1, n2) or null
    const int *tri_mesh;
    const uint8_t *tri_type;    // shading queue (bsdf_queue_of) of the triangle's mesh BSDF, 255 = no BSDF
    const float *tri_uv;        // 6 floats per triangle (uv0, uv1, uv2) or null; NaN: mesh without uvs
    const DevTexture *textures;
    int n_textures;
    int has_textured;           // some BSDF is textured (hits carry texture coordinates)
    int has_mixed;              // some BSDF shades from the mixed queue (bsdf_queue_of)
    const DevMesh *meshes;
    const float *mesh_cdf;
    int n_meshes;
    const DevSphere *spheres;
    int n_spheres;
    const DevBsdf *bsdfs;
    const DevLight *lights;
    int n_lights;
    int env_light;
    const float *light_cdf;     // n_lights + 1 (Integrator::myLightWeights)
    const DevMedium *media;
    DevCamera cam;
    float bmin[3], bmax[3];
    // set to 1 by device code that had to cut a loop or drop work (the host
    // turns it into RT_ERR_LIMIT); filled in per launch, null in none
    int *limit_flag;
};

// ------------------------------------------------------------------ rays / hits
struct Ray {
    V3 o, d;
    float mint, maxt;
};
__device__ __forceinline__ Ray make_ray(V3 o, V3 d, float mint, float maxt)
{
    Ray r; r.o = o; r.d = d; r.mint = mint; r.maxt = maxt; return r;
}

struct Hit {
    float t, u, v;
    int prim;   // triangle id, -(sphere)-2, -1 = none
};

struct Frame {
    V3 p;       // hit point
    V3 n, s, t; // shading frame
};

// BoundingBox::intersection (core/BoundingBox.h:154-183)
__device__ __forceinline__ bool ref_box_hit(const float *bmin, const float *bmax, V3 o, V3 d, float mint,
                                            float maxt, float &nearT, float &farT)
{
    nearT = -RT_MAX_REAL;
    farT = RT_MAX_REAL;
    V3 inv = v3(1.f / d.x, 1.f / d.y, 1.f / d.z);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float oo = vget(o, i), dd = vget(d, i), iv = vget(inv, i);
        float mn = bmin[i], mx = bmax[i];
        if (dd == 0) {
            if (oo < mn || oo > mx) return false;
        } else {
            float t1 = (mn - oo) * iv;
            float t2 = (mx - oo) * iv;
            if (t1 > t2) { float q = t1; t1 = t2; t2 = q; }
            nearT = smax(t1, nearT);
            farT = smin(t2, farT);
            if (!(nearT <= farT)) return false;
        }
    }
    return (mint <= farT && maxt >= nearT);
}

// ------------------------------------------------------------------ traversal
// |det| < 1e-8 (double compare in Triangle.cpp:66) <=> |det| <= float32(1e-8)
#define RT_DET_EPS 9.99999993922529e-09f
#define RT_STACK 64
// Bits of the limit flag a render reads back: which device cap tripped
// (the host names them in the RT_ERR_LIMIT message).
enum {
    RT_LIM_STACK2 = 1,     // BVH2 traversal stack full (the build bounds the depth)
    RT_LIM_STACK4 = 2,     // 4-wide traversal stack full (deeper trees are not uploaded)
    RT_LIM_STACK8 = 4,     // 8-wide group stack full (deeper trees are not uploaded)
    RT_LIM_VOLPATH = 8,    // a VolPathTracing loop cap (boundaries, tracking steps, iterations)
};

// Triangle::intersection (geometricShape/Triangle.cpp:46-88), exact order
__device__ __forceinline__ bool mt_test(float4 a, float4 b, float4 c, V3 o, V3 d, float mint, float maxt,
                                        float &t, float &u, float &v)
{
    V3 p0 = v3(a.x, a.y, a.z), e1 = v3(b.x, b.y, b.z), e2 = v3(c.x, c.y, c.z);
    V3 s = o - p0;
    V3 s1 = cross(d, e2), s2 = cross(s, e1);
    float det = dot(s1, e1);
    if (fabsf(det) <= RT_DET_EPS) return false;
    float inv = 1 / det;
    float b1 = inv * dot(s1, s);
    if (b1 < 0.f || b1 > 1.f) return false;
    float b2 = inv * dot(s2, d);
    if (b2 < 0.f || b1 + b2 > 1.f) return false;
    float tt = inv * dot(s2, e2);
    if (tt < mint || tt > maxt) return false;
    t = tt; u = b1; v = b2;
    return true;
}

// Sphere::intersection (geometricShape/Sphere.cpp:38-111)
__device__ __forceinline__ bool sphere_test(const DevSphere &sp, V3 o, V3 d, float mint, float maxt, float &t)
{
    V3 lo = xf_point(sp.to_object, o);
    V3 ld = xf_vector(sp.to_object, d);
    V3 sto = lo - v3(0.f, 0.f, 0.f);
    float a = 1;
    float b = 2 * dot(ld, sto);
    float c = dot(sto, sto) - sp.radius * sp.radius;
    float delta = b * b - 4 * a * c;
    if (delta < 0) return false;
    float t1 = (-b + sqrtf(delta)) / (2 * a);
    float t2 = (-b - sqrtf(delta)) / (2 * a);
    float tn = t1, tf = t2;
    if (tn > tf) { float q = tn; tn = tf; tf = q; }
    if (tn <= mint) {
        if (tf > mint && tf < maxt) { t = tf; return true; }
        return false;
    } else if (tn > mint && tn < maxt) { t = tn; return true; }
    return false;
}

// Plane::intersection (geometricShape/Plane.cpp:63-79).  A ray lying in the
// plane gives t = NaN, which the reference's range test lets through; here it
// is a miss.
__device__ __forceinline__ bool plane_test(const DevSphere &sp, V3 o, V3 d, float mint, float maxt, float &t)
{
    V3 lo = xf_point(sp.to_object, o);
    V3 ld = xf_vector(sp.to_object, d);
    float tt = -lo.z / ld.z;
    if (!(tt >= mint && tt <= maxt)) return false;
    V3 q = lo + tt * ld;
    if (q.x < -1.f || q.x > 1.f || q.y < -1.f || q.y > 1.f) return false;
    t = tt;
    return true;
}
__device__ __noinline__ bool plane_test_call(const DevSphere &sp, V3 o, V3 d, float mint, float maxt, float &t)
{
    return plane_test(sp, o, d, mint, maxt, t);
}
// The analytic shapes are tested one by one after the triangle BVH.  The
// plane test is out of line, so that scenes with spheres only keep the
// traversal kernels' registers.
__device__ __forceinline__ bool analytic_test(const DevSphere &sp, V3 o, V3 d, float mint, float maxt, float &t)
{
    if (sp.kind == 1) return plane_test_call(sp, o, d, mint, maxt, t);
    return sphere_test(sp, o, d, mint, maxt, t);
}

// Adaptive epsilon of Bvh::intersection (accelStruct/Bvh.cpp:411-413)
__device__ __forceinline__ float adapt_mint(V3 o, float mint)
{
    if (mint == RT_EPSILON) {
        float m = smax(smax(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
        mint = smax(mint, mint * m);
    }
    return mint;
}

// Per-axis guard of the fused slab test.  A slab distance is evaluated as
// fma(plane, 1/d, -o/d); besides the rounding relative to the plane (covered
// by widening the boxes when they are built) it carries a few ulps of |o/d|.
// Every near plane is moved earlier and every far plane later by
// 2^-21 |o/d|, which in distance along the axis is 2^-21 |o|, however
// parallel the ray runs to the slab.
__device__ __forceinline__ float slab_guard(float oo) { return fabsf(oo) * 4.76837158203125e-7f; }

// Leaf encoding of BVH2 child links: c >= 0 internal node index; c < 0 leaf
// with v = ~c, first slot = v >> 3, count = (v & 7) + 1.
// Three-input min / max (sm_100 and later: min.f32 / max.f32 with three
// sources; NaN inputs are ignored as by fminf / fmaxf).  RT_MNMX3=0 builds
// them from two-input operations.
#ifndef RT_MNMX3
#define RT_MNMX3 1
#endif
__device__ __forceinline__ float rt_min3(float a, float b, float c)
{
#if RT_MNMX3
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}
__device__ __forceinline__ float rt_max3(float a, float b, float c)
{
#if RT_MNMX3
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float rt_min4(float a, float b, float c, float d) { return rt_min3(a, b, fminf(c, d)); }
__device__ __forceinline__ float rt_max4(float a, float b, float c, float d) { return rt_max3(a, b, fmaxf(c, d)); }

// Closest / any hit through the BVH2 plus the analytic spheres.  With
// COUNT, nodes fetched and triangle slots tested are added to cnt[0], cnt[1]
// (the roofline's algorithmic-bytes accounting).
template <bool ANY, bool COUNT = false>
__device__ __forceinline__ bool trace_ray(const DevScene &S, V3 o, V3 d, float mint0, float maxt, Hit &h,
                                          int *cnt = nullptr)
{
    float mint = adapt_mint(o, mint0);
    h.prim = -1;
    if (maxt < mint) return false;
    float hit_t = maxt;
    bool found = false;
    const float eps = 1e-20f;
    float idx = 1.0f / (fabsf(d.x) > eps ? d.x : copysignf(eps, d.x));
    float idy = 1.0f / (fabsf(d.y) > eps ? d.y : copysignf(eps, d.y));
    float idz = 1.0f / (fabsf(d.z) > eps ? d.z : copysignf(eps, d.z));
    const float oox = o.x * idx, ooy = o.y * idy, ooz = o.z * idz;
    // offsets for the lo and hi planes of each axis, guard applied outward
    const float lx = -(oox + copysignf(slab_guard(oox), idx)), hx = -(oox - copysignf(slab_guard(oox), idx));
    const float ly = -(ooy + copysignf(slab_guard(ooy), idy)), hy = -(ooy - copysignf(slab_guard(ooy), idy));
    const float lz = -(ooz + copysignf(slab_guard(ooz), idz)), hz = -(ooz - copysignf(slab_guard(ooz), idz));
    if (S.n_nodes > 0) {
        int stack[RT_STACK];
        int sp = 0;
        int node = 0;
        for (;;) {
            while (node >= 0) {
                if (COUNT) cnt[0]++;
                const float4 *N = S.nodes + 4 * (size_t)node;
                float4 n0 = __ldg(N), n1 = __ldg(N + 1), n2 = __ldg(N + 2);
                int4 cc = __ldg(reinterpret_cast<const int4 *>(N + 3));
                float c0lox = __fmaf_rn(n0.x, idx, lx), c0hix = __fmaf_rn(n0.y, idx, hx);
                float c0loy = __fmaf_rn(n0.z, idy, ly), c0hiy = __fmaf_rn(n0.w, idy, hy);
                float c0loz = __fmaf_rn(n2.x, idz, lz), c0hiz = __fmaf_rn(n2.y, idz, hz);
                float c1lox = __fmaf_rn(n1.x, idx, lx), c1hix = __fmaf_rn(n1.y, idx, hx);
                float c1loy = __fmaf_rn(n1.z, idy, ly), c1hiy = __fmaf_rn(n1.w, idy, hy);
                float c1loz = __fmaf_rn(n2.z, idz, lz), c1hiz = __fmaf_rn(n2.w, idz, hz);
                float c0min = rt_max4(fminf(c0lox, c0hix), fminf(c0loy, c0hiy), fminf(c0loz, c0hiz), mint);
                float c0max = rt_min4(fmaxf(c0lox, c0hix), fmaxf(c0loy, c0hiy), fmaxf(c0loz, c0hiz), hit_t);
                float c1min = rt_max4(fminf(c1lox, c1hix), fminf(c1loy, c1hiy), fminf(c1loz, c1hiz), mint);
                float c1max = rt_min4(fmaxf(c1lox, c1hix), fmaxf(c1loy, c1hiy), fmaxf(c1loz, c1hiz), hit_t);
                bool t0 = c0min <= c0max, t1 = c1min <= c1max;
                if (!t0 && !t1) {
                    if (sp == 0) { node = 0x7fffffff; break; }
                    node = stack[--sp];
                    continue;
                }
                if (t0 && t1) {
                    int nearc = cc.x, farc = cc.y;
                    if (c1min < c0min) { nearc = cc.y; farc = cc.x; }
                    // rt_scene_create refuses a tree deeper than the stack,
                    // so the stack cannot be full here.  (No flag is written:
                    // any use of the limit flag in this loop made the VolPath
                    // kernels that call it twice as slow.)
                    if (sp < RT_STACK) stack[sp++] = farc;
                    node = nearc;
                } else {
                    node = t0 ? cc.x : cc.y;
                }
            }
            if (node == 0x7fffffff) break;
            // leaf
            int v = ~node;
            int first = v >> 3, cnt_leaf = (v & 7) + 1;
            for (int i = 0; i < cnt_leaf; i++) {
                if (COUNT) cnt[1]++;
                const float4 *T = S.tri_slots + 3 * (size_t)(first + i);
                float4 a = __ldg(T), b = __ldg(T + 1), c = __ldg(T + 2);
                float t, u, w;
                if (mt_test(a, b, c, o, d, mint, hit_t, t, u, w)) {
                    h.t = t; h.u = u; h.v = w; h.prim = __float_as_int(a.w);
                    found = true;
                    if (ANY) return true;
                    hit_t = t;
                }
            }
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    for (int s = 0; s < S.n_spheres; s++) {
        float t;
        if (analytic_test(S.spheres[s], o, d, mint, hit_t, t)) {
            h.t = t; h.u = 0.f; h.v = 0.f; h.prim = -s - 2;
            found = true;
            if (ANY) return true;
            hit_t = t;
        }
    }
    return found;
}

// DifferentialGeometry::coordinateSystem (core/DifferentialGeometry.h:36-50)
__device__ __forceinline__ void frame_from(V3 n, V3 &s, V3 &t)
{
    V3 c;
    if (fabsf(n.x) > fabsf(n.y)) {
        float il = 1.0f / sqrtf(n.x * n.x + n.z * n.z);
        c = v3(n.z * il, 0.0f, -n.x * il);
    } else {
        float il = 1.0f / sqrtf(n.y * n.y + n.z * n.z);
        c = v3(0.0f, n.z * il, -n.y * il);
    }
    t = c;
    s = cross(c, n);
}

// Differential geometry of a hit: Triangle::getDifferentialGeometry
// (Triangle.cpp:130-190) or Sphere::getDifferentialGeometry (Sphere.cpp:115-139)
__device__ __forceinline__ Frame hit_frame(const DevScene &S, const Hit &h, V3 o, V3 d)
{
    Frame f;
    if (h.prim >= 0) {
        const float *P = S.tri_v + 9 * (size_t)h.prim;
        V3 p0 = vload(P), p1 = vload(P + 3), p2 = vload(P + 6);
        float sum = h.u + h.v;
        float bx = 1 - sum;
        f.p = (bx * p0 + h.u * p1) + h.v * p2;
        V3 ng = normalized(cross(p1 - p0, p2 - p0));
        V3 ns = ng;
        // a triangle of a mesh without normals carries NaN normals
        if (S.tri_n && !isnan(S.tri_n[9 * (size_t)h.prim])) {
            const float *Nn = S.tri_n + 9 * (size_t)h.prim;
            ns = normalized((bx * vload(Nn) + h.u * vload(Nn + 3)) + h.v * vload(Nn + 6));
        }
        f.n = ns;
    } else {
        const DevSphere &sp = S.spheres[-h.prim - 2];
        f.p = o + h.t * d;
        if (sp.kind == 1) {   // Plane::getDifferentialGeometry (Plane.cpp:82-92)
            f.n = normalized(xf_normal(sp.to_object, v3(0.f, 0.f, 1.f)));
        } else {
            V3 nl = normalized(xf_point(sp.to_object, f.p) - v3(0, 0, 0));
            f.n = normalized(xf_normal(sp.to_object, nl));
        }
    }
    frame_from(f.n, f.s, f.t);
    return f;
}
__device__ __forceinline__ V3 to_local(const Frame &f, V3 v) { return v3(dot(v, f.s), dot(v, f.t), dot(v, f.n)); }
__device__ __forceinline__ V3 to_world(const Frame &f, V3 v) { return (f.s * v.x + f.t * v.y) + f.n * v.z; }

// primitive attributes
__device__ __forceinline__ int prim_bsdf(const DevScene &S, int prim)
{
    return prim >= 0 ? S.meshes[S.tri_mesh[prim]].bsdf : S.spheres[-prim - 2].bsdf;
}
__device__ __forceinline__ int prim_light(const DevScene &S, int prim)
{
    return prim >= 0 ? S.meshes[S.tri_mesh[prim]].light : S.spheres[-prim - 2].light;
}
// shading queue (bsdf_queue) of a hit primitive's BSDF, or -1 without a BSDF
__device__ __forceinline__ int prim_type(const DevScene &S, int prim)
{
    if (prim >= 0) {
        int t = __ldg(S.tri_type + prim);
        return t == 255 ? -1 : t;
    }
    int b = S.spheres[-prim - 2].bsdf;
    return b < 0 ? -1 : bsdf_queue_of(S.bsdfs[b]);
}

__device__ __forceinline__ int prim_interior(const DevScene &S, int prim)
{
    return prim >= 0 ? S.meshes[S.tri_mesh[prim]].interior : S.spheres[-prim - 2].interior;
}
__device__ __forceinline__ int prim_exterior(const DevScene &S, int prim)
{
    return prim >= 0 ? S.meshes[S.tri_mesh[prim]].exterior : S.spheres[-prim - 2].exterior;
}

// ------------------------------------------------------------------ CDF (core/CDF.h:44-81)
__device__ __forceinline__ int cdf_sample(const float *cdf, int n /* entries incl. leading 0 */, float u)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if (cdf[mid] < u) lo = mid + 1; else hi = mid;
    }
    return imin(imax(0, lo - 1), n - 2);
}
// The same index as cdf_sample, with the search narrowed by a guide table:
// guide[k] = first i with cdf[i] >= k / G (G a power of two, so k = (int)(u*G)
// is exact).  For u in [k/G, (k+1)/G) the answer lies in [guide[k],
// guide[k+1]], so a binary search over that range returns exactly what the
// full lower_bound returns, in a step or two instead of log2(n).
__device__ __forceinline__ int cdf_sample_guided(const float *cdf, int n, float u, const int *guide, int G)
{
    int k = imin(imax((int)(u * (float)G), 0), G - 1);
    int lo = __ldg(guide + k), hi = __ldg(guide + k + 1);
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if (__ldg(cdf + mid) < u) lo = mid + 1; else hi = mid;
    }
    return imin(imax(0, lo - 1), n - 2);
}
__device__ __forceinline__ int cdf_sample_reuse(const float *cdf, int n, float &u, float &pdf)
{
    int i = cdf_sample(cdf, n, u);
    u = (u - cdf[i]) / (cdf[i + 1] - cdf[i]);
    pdf = cdf[i + 1] - cdf[i];
    return i;
}

// ------------------------------------------------------------------ warps (core/Mapping.h)
__device__ __forceinline__ V2 concentric_disk(V2 s)
{
    const float r1 = 2 * s.x - 1.f;
    const float r2 = 2 * s.y - 1.f;
    float rx, ry;
    if (r1 > -r2 && r1 > r2) { rx = r1; ry = (RT_PI * r2) / (4 * r1); }
    else if (r1 < r2 && r1 > -r2) { rx = r2; ry = (RT_PI / 4.f) * (2 - r1 / r2); }
    else if (r1 < -r2 && r1 < r2) { rx = -r1; ry = (RT_PI / 4.f) * (4 + r2 / r1); }
    else { rx = -r2; ry = (RT_PI / 4.f) * (6 - r1 / r2); }
    return v2(rx * cosf(ry), rx * sinf(ry));
}
__device__ __forceinline__ V3 cosine_hemisphere(V2 s)
{
    V2 t = concentric_disk(s);
    float z = sqrtf(smax(0.f, 1.f - t.x * t.x - t.y * t.y));
    return v3(t.x, t.y, z);
}
__device__ __forceinline__ V3 square_to_triangle(V2 s)
{
    float sq = sqrtf(s.x);
    return v3(1 - sq, (1 - s.y) * sq, s.y * sq);
}
__device__ __forceinline__ V3 uniform_sphere(V2 s)
{
    float phi = 2.f * RT_PI * s.x;
    float u = 2 * s.y - 1.f;
    float st = sqrtf(1.f - u * u);
    return normalized(v3(st * cosf(phi), st * sinf(phi), u));
}
__device__ __forceinline__ float cone_pdf(float c) { return 1.f / (2 * RT_PI * (1.f - c)); }
__device__ __forceinline__ float spherical_phi(V3 v)
{
    float r = atan2f(v.x, -v.z);
    return r < 0.f ? r + 2 * (float)3.14159265358979323846 : r;
}
__device__ __forceinline__ float spherical_theta(V3 v) { return acosf(v.y); }

// ------------------------------------------------------------------ textures
// Texture coordinates of a hit (Intersection::myUv): a triangle's vertex uvs
// interpolated with the barycentrics (Triangle.cpp:155-164), or the
// barycentric (u, v) themselves for a mesh without uvs (Triangle::intersection
// leaves them in myUv); a sphere's spherical angles of the object-space hit
// point (Sphere.cpp:98-104).
__device__ __forceinline__ V2 hit_uv(const DevScene &S, const Hit &h, V3 o, V3 d)
{
    if (h.prim >= 0) {
        if (S.tri_uv) {
            const float *q = S.tri_uv + 6 * (size_t)h.prim;
            if (!isnan(q[0])) {
                const float b0 = 1.f - (h.u + h.v);
                return v2((b0 * q[0] + h.u * q[2]) + h.v * q[4], (b0 * q[1] + h.u * q[3]) + h.v * q[5]);
            }
        }
        return v2(h.u, h.v);
    }
    const DevSphere &sp = S.spheres[-h.prim - 2];
    V3 lo = xf_point(sp.to_object, o), ld = xf_vector(sp.to_object, d);
    if (sp.kind == 1) {   // Plane::intersection (Plane.cpp:75-76)
        V3 q = lo + h.t * ld;
        return v2((q.x + 1) / 2.f, (q.y + 1) / 2.f);
    }
    V3 n = normalized(lo + h.t * ld);
    return v2(spherical_phi(n) / (2 * RT_PI), spherical_theta(n) / RT_PI);
}

__device__ __forceinline__ int tex_clamp(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }
__device__ __forceinline__ C3 tex_texel(const DevTexture &T, int x, int y)
{
    const float *p = T.rgb + 3 * ((size_t)y * T.w + x);
    return c3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}
// math::interp2 (core/BasicMath.h:73-90).  A texture one texel wide (high)
// has an empty clamp range there, where the reference reads index -1; here
// the index stays 0.
__device__ __forceinline__ C3 tex_interp2(const DevTexture &T, float x, float y)
{
    const float ax = x - (float)(int)x, ay = y - (float)(int)y;
    int x0 = T.w < 2 ? 0 : tex_clamp((int)x, 0, T.w - 2);
    int y0 = T.h < 2 ? 0 : tex_clamp((int)y, 0, T.h - 2);
    int x1 = tex_clamp(x0 + 1 < T.w ? x0 + 1 : x0, 0, T.w - 1);
    int y1 = tex_clamp(y0 + 1 < T.h ? y0 + 1 : y0, 0, T.h - 1);
    C3 r = ((1.f - ax) * (1.f - ay)) * tex_texel(T, x0, y0);
    r = r + ((1.f - ax) * ay) * tex_texel(T, x0, y1);
    r = r + (ax * (1.f - ay)) * tex_texel(T, x1, y0);
    return r + (ax * ay) * tex_texel(T, x1, y1);
}
__device__ __forceinline__ float tex_sign(float v) { return v >= 0.f ? 1.f : -1.f; }
// ImageTexture::eval (ImageTexture.cpp:28-70): x spans width - 1 and y spans
// height; invertX / invertY flip within the unit tile; scale repeats; values
// outside [0, size) wrap.
__device__ __noinline__ C3 tex_eval(const DevTexture &T, V2 uv)
{
    const float W = (float)T.w, H = (float)T.h;
    float x, y;
    if (!T.invert_y) y = uv.y * H;
    else y = (float)(int)uv.y + (tex_sign(uv.y) * 1.f - (uv.y - (float)(int)uv.y)) * H;
    if (!T.invert_x) x = uv.x * (W - 1.f);
    else x = (float)(int)uv.x + (tex_sign(uv.x) * 1.f - (uv.x - (float)(int)uv.x)) * W;
    x *= T.scale;
    y *= T.scale;
    if (x >= W) x = (float)((unsigned)(int)x % (unsigned)T.w) + (x - (float)(int)x);
    else if (x < 0.f) x = (float)((unsigned)T.w - (unsigned)abs((int)x) % (unsigned)T.w) + (x - (float)(int)x);
    if (y >= H) y = (float)((unsigned)(int)y % (unsigned)T.h) + (y - (float)(int)y);
    else if (y < 0.f) y = (float)((unsigned)T.h - (unsigned)abs((int)y) % (unsigned)T.h) + (y - (float)(int)y);
    return tex_interp2(T, x, y);
}
// The BSDF parameters at a hit: textured ones replaced by their texture's
// value at uv (an alpha texture by the average of its channels, as the
// rough BSDFs read it).
__device__ __noinline__ void tex_apply(const DevScene &S, DevBsdf &b, V2 uv)
{
    if (b.tex[TEX_ALBEDO] >= 0) {
        C3 c = tex_eval(S.textures[b.tex[TEX_ALBEDO]], uv);
        b.albedo[0] = c.r; b.albedo[1] = c.g; b.albedo[2] = c.b;
    }
    if (b.tex[TEX_REFLECTANCE] >= 0) {
        C3 c = tex_eval(S.textures[b.tex[TEX_REFLECTANCE]], uv);
        b.reflectance[0] = c.r; b.reflectance[1] = c.g; b.reflectance[2] = c.b;
    }
    if (b.tex[TEX_TRANSMITTANCE] >= 0) {
        C3 c = tex_eval(S.textures[b.tex[TEX_TRANSMITTANCE]], uv);
        b.transmittance[0] = c.r; b.transmittance[1] = c.g; b.transmittance[2] = c.b;
    }
    if (b.tex[TEX_ALPHA] >= 0) {
        float a = cavg(tex_eval(S.textures[b.tex[TEX_ALPHA]], uv));
        b.alpha = a;
        b.alpha_avg = a;
    }
}
__device__ __forceinline__ V3 cartesian_from_spherical(float theta, float phi)
{
    float st = sinf(theta), ct = cosf(theta), cp = cosf(phi), sp = sinf(phi);
    return v3(sp * st, ct, -cp * st);
}

// ------------------------------------------------------------------ Fresnel (core/Fresnel.h)
__device__ __forceinline__ float fresnel_conductor1(float eta, float k, float cosI)
{
    float epa = eta * eta + k * k;
    float c2 = cosI * cosI;
    float epac2 = epa * c2;
    float two = 2 * eta * cosI;
    float rpar = (epac2 - two + 1) / (epac2 + two + 1);
    float rperp = (epa - two + c2) / (epa + two + c2);
    return (rpar * rpar + rperp * rperp) * 0.5f;
}
__device__ __forceinline__ float fresnel_dielectric(float eI, float eT, float cI, float cT)
{
    float tcI = eT * cI, icT = eI * cT, icI = eI * cI, tcT = eT * cT;
    float rpar = (tcI - icT) / (tcI + icT);
    float rperp = (icI - tcT) / (icI + tcT);
    return (rpar * rpar + rperp * rperp) * 0.5f;
}
// Fresnel.h:83-114 (grey reflectance)
__device__ __forceinline__ float estimate_dielectric(float etaExt, float etaInt, float cosI, float &eI, float &eT,
                                                     float &rel, float &cT)
{
    eI = etaExt; eT = etaInt;
    bool entering = true;
    float fr;
    if (cosI <= 0.f) { entering = false; float q = eI; eI = eT; eT = q; }
    rel = eI / eT;
    float sinT = rel * sqrtf(smax(0.f, 1 - cosI * cosI));
    cT = sqrtf(smax(0.f, 1 - sinT * sinT));
    if (sinT >= 1.f) { cT = 0.f; fr = 1.f; }
    else {
        fr = fresnel_dielectric(eI, eT, fabsf(cosI), cT);
        if (entering) cT = -cT;
    }
    return fr;
}

// ------------------------------------------------------------------ microfacets (MicrofacetDistribution.cpp)
__device__ __forceinline__ float sin2t(V3 v) { return 1.f - v.z * v.z; }
__device__ __forceinline__ float sint(V3 v) { float s2 = sin2t(v); if (s2 < 0.f) return 0.f; return sqrtf(s2); }
__device__ __forceinline__ float tan2t(V3 v) { float s2 = 1.f - v.z * v.z; if (s2 <= 0.f) return 0.f; return s2 / (v.z * v.z); }

__device__ __forceinline__ V3 mf_sample_normal(int type, V2 s, float alpha)
{
    float theta;
    if (type == 0) theta = atanf(sqrtf(-alpha * alpha * logf(1 - s.x)));
    else if (type == 2) theta = atanf(alpha * sqrtf(s.x) / sqrtf(1.f - s.x));
    else theta = acosf(powf(s.x, 1.f / (alpha + 2)));
    float phi = 2 * RT_PI * s.y;
    return v3(sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta));
}
__device__ __forceinline__ float mf_D(int type, V3 wh, float alpha)
{
    if (wh.z <= 0.f) return 0.f;
    if (type == 0) {
        float c2 = wh.z * wh.z;
        float t2 = sin2t(wh) / c2;
        float a2 = alpha * alpha;
        return expf(-t2 / a2) / (RT_PI * a2 * c2 * c2);
    } else if (type == 2) {
        float a2 = alpha * alpha;
        float c2 = wh.z * wh.z;
        float t2 = tan2t(wh);
        float ss = a2 + t2;
        return a2 / (RT_PI * c2 * c2 * ss * ss);
    }
    return ((alpha + 2.f) / (2 * RT_PI)) * powf(wh.z, alpha);
}
__device__ __forceinline__ float mf_G1(int type, V3 v, V3 m, float alpha)
{
    if (dot(v, m) / v.z <= 0) return 0.f;
    if (type == 0) {
        float tv = sint(v) / v.z;
        if (tv == 0.f) return 1.f;
        float b = fabsf(1.f / (alpha * tv));
        if (b < 1.6f) return (3.535f * b + 2.181f * b * b) / (1 + 2.276f * b + 2.577f * b * b);
        return 1.f;
    } else if (type == 2) {
        float a2 = alpha * alpha;
        float t2 = tan2t(v);
        return 2.f / (1 + sqrtf(1 + a2 * t2));
    }
    float tv = sint(v) / v.z;
    float b = sqrtf(0.5f * alpha + 1) / tv;
    if (b < 1.6f) return (3.535f * b + 2.181f * b * b) / (1 + 2.276f * b + 2.577f * b * b);
    return 1.f;
}
__device__ __forceinline__ float mf_G(int type, V3 wi, V3 wo, V3 wh, float alpha)
{
    return mf_G1(type, wi, wh, alpha) * mf_G1(type, wo, wh, alpha);
}
__device__ __forceinline__ float adjusted_alpha(float a, float cosI) { return (1.2f - 0.2f * sqrtf(fabsf(cosI))) * a; }
__device__ __forceinline__ float fsign(float v) { return v >= 0.f ? 1.f : -1.f; }
__device__ __forceinline__ V3 reflect_n(V3 v, V3 n) { float d = 2 * dot(v, n); return d * n - v; }
__device__ __forceinline__ V3 refract_local(V3 v, float cT, float rel) { return v3(rel * -v.x, rel * -v.y, cT); }
__device__ __forceinline__ V3 refract_n(V3 v, V3 n, float rel, float cT)
{
    float s = dot(v, n) * rel + cT;
    return n * s - v * rel;
}
__device__ __forceinline__ V3 half_dir_transmitted(V3 wi, V3 wo, float eI, float eT)
{
    V3 s = eI * wi + eT * wo;
    return normalized(-1.f * s);
}

// ------------------------------------------------------------------ BSDFs
enum { BT_UNKNOWN = 0, BT_DIFFUSE_REFLECTION = 1, BT_DELTA_REFLECTION = 2, BT_GLOSSY_REFLECTION = 4,
       BT_DELTA_TRANSMISSION = 8, BT_GLOSSY_TRANSMISSION = 0x10, BT_DIFFUSE = 0x200,
       BT_DELTA = 2 | 8, BT_ALL = (1 | 2 | 4) | (8 | 4) };

struct BsdfRec {
    V3 wi, wo;
    int type;
    float rel_eta;
    float pdf;
};

// Diffuse (bsdf/Diffuse.cpp:28-106)
__device__ __forceinline__ C3 diffuse_eval(const float *alb, V3 wi, V3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return cfill(0.f);
    return cload(alb) * RT_INV_PI;
}
__device__ __forceinline__ float diffuse_pdf(V3 wi, V3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return 0.f;
    return RT_INV_PI * wo.z;
}
__device__ __forceinline__ C3 diffuse_sample(const float *alb, BsdfRec &r, V2 s)
{
    if (r.wi.z <= 0.f) return cfill(0.f);
    r.type = BT_DIFFUSE;
    r.wo = cosine_hemisphere(s);
    r.pdf = diffuse_pdf(r.wi, r.wo);
    return cload(alb);
}

// RoughConductor (bsdf/RoughConductor.cpp:77-145)
__device__ __forceinline__ C3 rc_eval(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z, co = wo.z;
    if (ci <= 0.f || co <= 0.f) return cfill(0.f);
    V3 wh = normalized(wi + wo);
    float D = mf_D(b.distribution, wh, b.alpha_avg);
    float G = mf_G(b.distribution, wi, wo, wh, b.alpha_avg);
    C3 F = c3(fresnel_conductor1(b.eta[0], b.k[0], ci), fresnel_conductor1(b.eta[1], b.k[1], ci),
              fresnel_conductor1(b.eta[2], b.k[2], ci));
    float den = 4 * ci * co;
    C3 r = cload(b.reflectance) * D;
    r = r * F;
    r = r * G;
    return r / den;
}
__device__ __forceinline__ float rc_pdf(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z, co = wo.z;
    if (ci <= 0.f || co <= 0.f) return 0.f;
    V3 wh = normalized(wi + wo);
    float ch = wh.z;
    float Jh = 1.f / (4 * fabsf(dot(wh, wo)));
    float D = mf_D(b.distribution, wh, b.alpha_avg);
    return D * ch * Jh;
}
__device__ __forceinline__ C3 rc_sample(const DevBsdf &b, BsdfRec &r, V2 s)
{
    if (r.wi.z <= 0.f) return cfill(0.f);
    r.type = BT_GLOSSY_REFLECTION;
    float alpha = adjusted_alpha(b.alpha_avg, r.wi.z);
    V3 n = mf_sample_normal(b.distribution, s, alpha);
    r.wo = reflect_n(r.wi, n);
    float co = r.wo.z;
    if (co <= 0.f) return cfill(0.f);
    r.pdf = rc_pdf(b, r.wi, r.wo);
    if (r.pdf <= 0) return cfill(0.f);
    C3 e = rc_eval(b, r.wi, r.wo);
    return (e * fabsf(co)) / r.pdf;
}

// RoughDielectric (bsdf/RoughDielectric.cpp:83-329)
__device__ __forceinline__ C3 rd_eval_reflection(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z, co = wo.z;
    V3 wh = normalized(wi + wo);
    wh = fsign(ci) * wh;
    float alpha = b.alpha_avg;
    float D = mf_D(b.distribution, wh, alpha);
    float eI, eT, rel, cT;
    float fr = estimate_dielectric(b.eta_ext, b.eta_int, dot(wi, wh), eI, eT, rel, cT);
    float G = mf_G(b.distribution, wi, wo, wh, alpha);
    float den = 4 * ci * co;
    C3 r = cload(b.reflectance) * D;
    r = r * fr;
    r = r * G;
    return r / den;
}
__device__ __forceinline__ C3 rd_eval_refraction(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z, co = wo.z;
    float eI, eT, rel, cT;
    float fr = estimate_dielectric(b.eta_ext, b.eta_int, ci, eI, eT, rel, cT);
    V3 wt = half_dir_transmitted(wi, wo, eI, eT);
    float alpha = b.alpha_avg;
    float left = dot(wi, wt) * dot(wo, wt) / (ci * co);
    float G = mf_G(b.distribution, wi, wo, wt, alpha);
    float D = mf_D(b.distribution, wt, alpha);
    float omf = (-1.f * fr) + 1.f;
    C3 term = cload(b.transmittance) * left;
    term = term * eT;
    term = term * eT;
    term = term * omf;
    term = term * G;
    term = term * D;
    term = term * rel;
    term = term * rel;
    float denom = eI * dot(wi, wt) + eT * dot(wo, wt);
    return term / (denom * denom);
}
__device__ __forceinline__ float rd_pdf_reflection(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z;
    float alpha = (1.2f - 0.2f * sqrtf(fabsf(ci))) * b.alpha_avg;
    V3 wh = normalized(wi + wo);
    wh = fsign(ci) * wh;
    float ch = wh.z;
    float Jh = 1.f / (4 * dot(wh, wo));
    return fabsf(mf_D(b.distribution, wh, alpha) * ch * Jh);
}
__device__ __forceinline__ float rd_pdf_refraction(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z;
    float eI, eT, rel, cT;
    estimate_dielectric(b.eta_ext, b.eta_int, ci, eI, eT, rel, cT);
    V3 wt = half_dir_transmitted(wi, wo, eI, eT);
    float cwt = wt.z;
    float alpha = (1.2f - 0.2f * sqrtf(fabsf(ci))) * b.alpha_avg;
    float hd = eI * dot(wi, wt) + eT * dot(wo, wt);
    float Jh = (eT * eT * dot(wo, wt)) / (hd * hd);
    return fabsf(mf_D(b.distribution, wt, alpha) * cwt * Jh);
}
__device__ __forceinline__ C3 rd_eval(const DevBsdf &b, V3 wi, V3 wo)
{
    if (wi.z * wo.z > 0) return rd_eval_reflection(b, wi, wo);
    return rd_eval_refraction(b, wi, wo);
}
__device__ __forceinline__ float rd_pdf(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z, co = wo.z;
    float eI, eT, rel, cT;
    if (ci * co > 0) {
        V3 wh = normalized(wi + wo);
        wh = fsign(ci) * wh;
        float fr = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, dot(wi, wh), eI, eT, rel, cT));
        return rd_pdf_reflection(b, wi, wo) * fr;
    }
    float etaI = b.eta_ext, etaT = b.eta_int;
    if (ci < 0) { float q = etaI; etaI = etaT; etaT = q; }
    V3 wt = half_dir_transmitted(wi, wo, etaI, etaT);
    float fr = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, dot(wi, wt), eI, eT, rel, cT));
    return rd_pdf_refraction(b, wi, wo) * (1.f - fr);
}
__device__ __forceinline__ C3 rd_sample(const DevBsdf &b, BsdfRec &r, V2 s)
{
    float ci = r.wi.z;
    float alpha = adjusted_alpha(b.alpha_avg, ci);
    V3 n = mf_sample_normal(b.distribution, s, alpha);
    float eI, eT, rel, cT;
    float fr = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, dot(r.wi, n), eI, eT, rel, cT));
    if (s.x <= fr) {
        r.type = BT_GLOSSY_REFLECTION;
        r.wo = reflect_n(r.wi, n);
        if (r.wi.z * r.wo.z <= 0) return cfill(0.f);
        r.pdf = rd_pdf_reflection(b, r.wi, r.wo) * fr;
        if (r.pdf <= 0) return cfill(0.f);
        V3 wh = normalized(r.wi + r.wo);
        wh = fsign(ci) * wh;
        float G = mf_G(b.distribution, r.wi, r.wo, wh, alpha);
        float v = 1.f * dot(r.wi, n);
        v = v * G;
        return cfill(v / (ci * n.z));
    }
    r.type = BT_GLOSSY_TRANSMISSION;
    r.wo = normalized(refract_n(r.wi, n, rel, cT));
    r.rel_eta = rel;
    float co = dot(r.wo, n);
    if (r.wi.z * r.wo.z >= 0) return cfill(0.f);
    r.pdf = rd_pdf_refraction(b, r.wi, r.wo) * (1.f - fr);
    if (r.pdf <= 0) return cfill(0.f);
    C3 e = rd_eval_refraction(b, r.wi, r.wo);
    return (e * fabsf(co)) / r.pdf;
}

// SmoothLayeredBSDF over a Diffuse base (bsdf/SmoothLayeredBSDF.cpp:139-403)
__device__ __forceinline__ C3 absorb(const DevBsdf &b, float wip, float wop)
{
    float s = 1.f / fabsf(wip) + 1.f / fabsf(wop);
    return c3(expf((-b.absorbance[0] * b.thickness) * s), expf((-b.absorbance[1] * b.thickness) * s),
              expf((-b.absorbance[2] * b.thickness) * s));
}
__device__ __forceinline__ C3 sl_eval(const DevBsdf &b, V3 wi, V3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return cfill(0.f);
    float ci = wi.z;
    float eI, eT, rel, cT;
    float fr1 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, ci, eI, eT, rel, cT));
    float T12 = 1.f - fr1;
    if (fr1 == 1.f) return cfill(0.f);
    V3 rwi = normalized(refract_local(wi, cT, rel));
    V3 rwo = normalized(refract_local(wo, cT, rel));
    rwi = -rwi;
    rwo = -rwo;
    ci = (-rwo).z;
    float fr2 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, ci, eI, eT, rel, cT));
    if (fr2 == 1.f) return cfill(0.f);
    float T21 = 1.f - fr2;
    C3 f2 = diffuse_eval(b.albedo, rwi, rwo);
    C3 a = absorb(b, rwi.z, rwo.z);
    float G = 1.f;
    float t = (1.f - G) + T21 * G;
    float m = b.eta_ext / b.eta_int;
    C3 r = T12 * f2;
    r = r * a;
    r = r * t;
    r = r * m;
    r = r * m;
    r = r * wo.z;
    r = r / rwo.z;
    return cfill(0.f) + r;
}
__device__ __forceinline__ float sl_pdf(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z;
    float eI, eT, rel, cT;
    float fr1 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, ci, eI, eT, rel, cT));
    if (fr1 == 1.f) return 0.f;
    V3 rwi = normalized(refract_local(wi, cT, rel));
    V3 rwo = normalized(refract_local(wo, cT, rel));
    rwi = -rwi;
    rwo = -rwo;
    float pb = diffuse_pdf(rwi, rwo);
    float m = b.eta_ext / b.eta_int;
    return 0.f + pb * (1.f - fr1) * m * m * wo.z / rwo.z;
}
__device__ __forceinline__ C3 sl_sample(const DevBsdf &b, BsdfRec &r, V2 s)
{
    if (r.wi.z <= 0.f) return cfill(0.f);
    float ci = r.wi.z;
    r.type = BT_GLOSSY_REFLECTION;
    float eI, eT, rel, cT;
    float fr1 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, ci, eI, eT, rel, cT));
    if (fr1 == 1.f) return cfill(0.f);
    if (s.x <= fr1) {
        r.wo = v3(-r.wi.x, -r.wi.y, r.wi.z);
        r.pdf = fr1;
        r.type = BT_DELTA_REFLECTION;
        return cfill(1.f);
    }
    V3 rwi = normalized(-refract_local(r.wi, cT, rel));
    r.type = BT_UNKNOWN;
    float T12 = 1.f - fr1;
    BsdfRec base;
    base.wi = rwi; base.wo = v3(0, 0, 0); base.type = BT_ALL; base.rel_eta = 1.f; base.pdf = -1.f;
    C3 f2 = diffuse_sample(b.albedo, base, s);
    if (iszero(f2)) return cfill(0.f);
    r.pdf = (1.f - fr1);
    if (r.pdf <= 0.f) return cfill(0.f);
    r.wo = -base.wo;
    float wip = rwi.z;
    float wop = (-base.wo).z;
    C3 a = absorb(b, wip, wop);
    ci = r.wo.z;
    float fr2 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, ci, eI, eT, rel, cT));
    if (fr2 == 1.f) return cfill(0.f);
    float T21 = 1.f - fr2;
    r.wo = normalized(refract_local(r.wo, cT, rel));
    float co = r.wo.z;
    C3 res = T12 * f2;
    res = res * a;
    res = res * T21;
    res = cfill(0.f) + res;
    res = res * fabsf(co);
    res = res / r.pdf;
    float m = b.eta_ext / b.eta_int;
    r.pdf *= base.pdf * m * m * r.wo.z / wop;
    return res;
}

// LayeredBSDF (bsdf/LayeredBSDF.cpp:17-310): a rough dielectric coat (GGX
// by default, alphaTop read as a plain real, so `alpha` here, not the
// texture average) over a RoughConductor base.  The reference draws the
// coat normal of sample() from a member Rng of the BSDF object (shared by
// all threads, LayeredBSDF.cpp:165), not from the sampler.  Here those two
// numbers come from a side stream keyed by the path's state after its BSDF
// sample was drawn (layered_aux), so the path's own stream advances exactly
// as in the reference and the result stays reproducible.
__device__ __forceinline__ Pcg32 layered_aux(uint64_t key)
{
    Pcg32 a;
    pcg_seed(a, key ^ 0x9E3779B97F4A7C15ull, 0x4C61796572656442ull);
    return a;
}
__device__ __forceinline__ DevBsdf layered_base(const DevBsdf &b)
{
    DevBsdf c = b;
    c.type = 1;
    c.distribution = b.dist_base;
    c.alpha_avg = b.alpha_base_avg;
    return c;
}
// LayeredBSDF::evalReflection (LayeredBSDF.cpp:150-163)
__device__ __forceinline__ C3 ly_eval_reflection(const DevBsdf &b, V3 wi, V3 wo, float fr, float alpha)
{
    float ci = wi.z, co = wo.z;
    V3 wh = normalized(wi + wo);
    wh = fsign(ci) * wh;
    C3 term = mf_D(b.distribution, wh, alpha) * cfill(fr);
    term = term * mf_G(b.distribution, wi, wo, wh, alpha);
    return term / (4 * ci * co);
}
// LayeredBSDF::eval (LayeredBSDF.cpp:79-147)
__device__ __forceinline__ C3 ly_eval(const DevBsdf &b, V3 wi, V3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return cfill(0.f);
    V3 wh = normalized(wi + wo);
    float eI, eT, rel, cT;
    float fr1 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, dot(wi, wh), eI, eT, rel, cT));
    float T12 = 1.f - fr1;
    float G = mf_G(b.distribution, wi, wo, wh, b.alpha);
    if (fr1 == 1.f) return cfill(0.f);
    V3 rwi = normalized(refract_n(wi, wh, rel, cT));
    V3 rwo = normalized(refract_n(wo, wh, rel, cT));
    C3 f1 = ly_eval_reflection(b, wi, wo, fr1, b.alpha);
    rwi = -1.f * rwi;
    rwo = -1.f * rwo;
    wh = normalized(rwi + rwo);
    float fr2 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, dot(-1.f * rwo, wh), eI, eT, rel, cT));
    if (fr2 == 1.f) return cfill(0.f);
    float T21 = 1.f - fr2;
    rel = b.eta_ext / b.eta_int;
    DevBsdf base = layered_base(b);
    C3 f2 = rc_eval(base, rwi, rwo) * rel;
    f2 = f2 * rel;
    f2 = f2 * wo.z;
    f2 = f2 / rwo.z;
    float s = 1.f / fabsf(rwi.z) + 1.f / fabsf(rwo.z);
    C3 ab = (cload(b.absorbance) * -1.f) * b.thickness;
    ab = ab * s;
    C3 a = c3(expf(ab.r), expf(ab.g), expf(ab.b));
    float t = (1.f - G) + T21 * G;
    C3 r = T12 * f2;
    r = r * a;
    r = r * t;
    return f1 + r;
}
// LayeredBSDF::pdf (LayeredBSDF.cpp:262-303)
__device__ __forceinline__ float ly_pdf(const DevBsdf &b, V3 wi, V3 wo)
{
    V3 wh = normalized(wi + wo);
    float eI, eT, rel, cT;
    float fr1 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, dot(wi, wh), eI, eT, rel, cT));
    if (fr1 == 1.f) return 0.f;
    V3 rwi = normalized(refract_n(wi, wh, rel, cT));
    V3 rwo = normalized(refract_n(wo, wh, rel, cT));
    float ch = wh.z;
    float Jh = 1.f / (4 * fabsf(dot(wh, wo)));
    float D = mf_D(b.distribution, wh, b.alpha);
    float pd = fabsf(D * ch * Jh);
    rwi = -1.f * rwi;
    rwo = -1.f * rwo;
    DevBsdf base = layered_base(b);
    float pc = rc_pdf(base, rwi, rwo);
    rel = b.eta_ext / b.eta_int;
    float q = pc * (1.f - fr1);
    q = q * rel;
    q = q * rel;
    q = q * wo.z;
    q = q / rwo.z;
    return pd * fr1 + q;
}
// LayeredBSDF::sample (LayeredBSDF.cpp:165-260)
__device__ __forceinline__ C3 ly_sample(const DevBsdf &b, BsdfRec &r, V2 s, uint64_t aux_key)
{
    if (r.wi.z <= 0.f) return cfill(0.f);
    float ci = r.wi.z;
    float alpha = (1.2f - 0.2f * sqrtf(fabsf(ci))) * b.alpha;
    Pcg32 aux = layered_aux(aux_key);
    float n1 = next1d(aux);
    float n2 = next1d(aux);
    V3 normal = mf_sample_normal(b.distribution, v2(n1, n2), alpha);
    float eI, eT, rel, cT;
    float fr1 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, dot(r.wi, normal), eI, eT, rel, cT));
    if (fr1 == 1.f) return cfill(0.f);
    if (s.x <= fr1) {
        r.wo = reflect_n(r.wi, normal);
        r.pdf = ly_pdf(b, r.wi, r.wo);
        r.type = BT_GLOSSY_REFLECTION;
        C3 f1 = ly_eval_reflection(b, r.wi, r.wo, fr1, alpha);
        if (iszero(f1)) return cfill(0.f);
    } else {
        r.type = BT_GLOSSY_REFLECTION;
        V3 rwi = normalized(-1.f * refract_n(r.wi, normal, rel, cT));
        BsdfRec rr;
        rr.wi = rwi; rr.wo = v3(0.f, 0.f, 0.f);
        rr.type = BT_ALL; rr.rel_eta = 1.f; rr.pdf = -1.f;
        DevBsdf base = layered_base(b);
        C3 f2 = rc_sample(base, rr, s);
        if (iszero(f2)) return cfill(0.f);
        r.wo = -1.f * rr.wo;
        float fr2 = cavg1(estimate_dielectric(b.eta_ext, b.eta_int, r.wo.z, eI, eT, rel, cT));
        if (fr2 == 1.f) return cfill(0.f);
        r.wo = normalized(refract_n(r.wo, normal, rel, cT));
        r.pdf = ly_pdf(b, r.wi, r.wo);
        if (r.pdf == 0.f) return cfill(0.f);
    }
    if (r.pdf == 0.f) return cfill(0.f);
    float co = r.wo.z;
    return (ly_eval(b, r.wi, r.wo) * fabsf(co)) / r.pdf;
}

// Smooth (delta) BSDFs.  Their eval and pdf are zero outside the discrete
// measure the reference attaches only to sampled directions
// (Dielectric.cpp:23-26,85-88; Conductor.cpp:26-37,55-64; Mirror.cpp:17-20,
// 36-39), so only sample() contributes.
// Dielectric::sample (bsdf/Dielectric.cpp:28-82): Fresnel-chosen delta
// reflection or refraction; relativeEta is set on both branches
__device__ __forceinline__ C3 dl_sample(const DevBsdf &b, BsdfRec &r, V2 s)
{
    float ci = r.wi.z;
    float eI = b.eta_ext, eT = b.eta_int;
    bool entering = true;
    float fr = 0.f;
    if (ci <= 0.f) { entering = false; float q = eI; eI = eT; eT = q; }
    float rel = eI / eT;
    float sinT = rel * sqrtf(smax(0.f, 1 - ci * ci));
    float cT = sqrtf(smax(0.f, 1 - sinT * sinT));
    if (sinT >= 1.f) fr = 1.f;
    else {
        fr = fresnel_dielectric(eI, eT, fabsf(ci), cT);
        if (entering) cT = -cT;
    }
    r.rel_eta = rel;
    if (s.x <= fr) {
        r.type = BT_DELTA_REFLECTION;
        r.wo = v3(-r.wi.x, -r.wi.y, r.wi.z);
        r.pdf = fr;
        return cload(b.reflectance);
    }
    r.type = BT_DELTA_TRANSMISSION;
    r.wo = refract_local(r.wi, cT, rel);
    r.pdf = 1 - fr;
    C3 t = cload(b.transmittance) * rel;
    return t * rel;
}
// Conductor::sample (bsdf/Conductor.cpp:39-53)
__device__ __forceinline__ C3 cd_sample(const DevBsdf &b, BsdfRec &r)
{
    if (r.wi.z <= 0.f) return cfill(0.f);
    r.type = BT_DELTA_REFLECTION;
    r.wo = v3(-r.wi.x, -r.wi.y, r.wi.z);
    r.pdf = 1.f;
    float ci = r.wi.z;
    C3 F = c3(fresnel_conductor1(b.eta[0], b.k[0], ci), fresnel_conductor1(b.eta[1], b.k[1], ci),
              fresnel_conductor1(b.eta[2], b.k[2], ci));
    return cload(b.reflectance) * F;
}
// Mirror::sample (bsdf/Mirror.cpp:22-34)
__device__ __forceinline__ C3 mr_sample(BsdfRec &r)
{
    if (r.wi.z <= 0.f) return cfill(0.f);
    r.type = BT_DELTA_REFLECTION;
    r.wo = v3(-r.wi.x, -r.wi.y, r.wi.z);
    r.pdf = 1.f;
    return cfill(1.f);
}

// SheetDielectric::sample (bsdf/SheetDielectric.cpp:122-174): reflection with
// the thin sheet's summed inter-reflections fr + T^2 fr / (1 - fr^2), else
// straight through (typed UNKNOWN there, not delta)
__device__ __forceinline__ C3 sd_sample(const DevBsdf &b, BsdfRec &r, V2 s)
{
    float ci = r.wi.z;
    float eI = b.eta_ext, eT = b.eta_int;
    float rel = eI / eT;
    float sinT = rel * sqrtf(smax(0.f, 1 - ci * ci));
    float cT = sqrtf(smax(0.f, 1 - sinT * sinT));
    float fr = fresnel_dielectric(eI, eT, fabsf(ci), cT);
    float T = 1.f - fr;
    if (fr < 1.f) fr = fr + ((T * T) * fr) / (1.f - fr * fr);
    r.rel_eta = 1.f;
    if (s.x <= fr) {
        r.type = BT_DELTA_REFLECTION;
        r.wo = v3(-r.wi.x, -r.wi.y, r.wi.z);
        r.pdf = fr;
        return cload(b.reflectance);
    }
    r.type = BT_UNKNOWN;
    r.wo = -r.wi;
    r.pdf = 1 - fr;
    return cload(b.transmittance);
}

// Microfacet (bsdf/Microfacet.cpp:62-182): (1 - ks) Lambertian kd plus ks
// times a dielectric-Fresnel microfacet lobe; its raw alpha; the sample's x
// both picks the lobe and samples the normal
__device__ __forceinline__ float nf_fresnel(float etaExt, float etaInt, float ci)
{
    float eI = etaExt, eT = etaInt;
    if (ci <= 0.f) { float q = eI; eI = eT; eT = q; }
    float rel = eI / eT;
    float sinT = rel * sqrtf(smax(0.f, 1 - ci * ci));
    float cT = sqrtf(smax(0.f, 1 - sinT * sinT));
    if (sinT >= 1.f) return 1.f;
    return fresnel_dielectric(eI, eT, fabsf(ci), cT);
}
__device__ __forceinline__ C3 nf_eval(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z, co = wo.z;
    if (ci <= 0.f || co <= 0.f) return cfill(0.f);
    V3 wh = normalized(wi + wo);
    C3 diffuse = ((1 - b.ks) * cload(b.albedo)) * RT_INV_PI;
    float F = nf_fresnel(b.eta_ext, b.eta_int, dot(wi, wh));
    C3 spec = cfill((b.ks * mf_D(b.distribution, wh, b.alpha)) * F);
    spec = spec * mf_G(b.distribution, wi, wo, wh, b.alpha);
    spec = spec / ((4 * ci) * co);
    return diffuse + spec;
}
__device__ __forceinline__ float nf_pdf(const DevBsdf &b, V3 wi, V3 wo)
{
    float ci = wi.z, co = wo.z;
    V3 wh = normalized(wi + wo);
    float ch = wh.z;
    float alpha = adjusted_alpha(b.alpha, ci);
    float Jh = 1.f / (4 * dot(wh, wo));
    return (((b.ks * mf_D(b.distribution, wh, alpha)) * ch) * Jh) + (((1 - b.ks) * co) * RT_INV_PI);
}
__device__ __forceinline__ C3 nf_sample(const DevBsdf &b, BsdfRec &r, V2 s)
{
    if (r.wi.z <= 0.f) return cfill(0.f);
    float alpha = adjusted_alpha(b.alpha, r.wi.z);
    V3 n = mf_sample_normal(b.distribution, s, alpha);
    if (s.x <= b.ks) {
        r.type = BT_GLOSSY_REFLECTION;
        r.wo = reflect_n(r.wi, n);
    } else {
        r.type = BT_DIFFUSE;
        r.wo = cosine_hemisphere(s);
    }
    float co = r.wo.z;
    r.pdf = nf_pdf(b, r.wi, r.wo);
    if (r.pdf == 0.f) return cfill(0.f);
    return (nf_eval(b, r.wi, r.wo) * fabsf(co)) / r.pdf;
}

// one BSDF type, no TwoSides wrapper
__device__ __forceinline__ C3 bsdf_eval1(const DevBsdf &b, V3 wi, V3 wo)
{
    switch (b.type) {
    case 0: return diffuse_eval(b.albedo, wi, wo);
    case 1: return rc_eval(b, wi, wo);
    case 2: return rd_eval(b, wi, wo);
    case 3: return sl_eval(b, wi, wo);
    case 4: return ly_eval(b, wi, wo);
    case 9: return nf_eval(b, wi, wo);
    default: return cfill(0.f);
    }
}
__device__ __forceinline__ float bsdf_pdf1(const DevBsdf &b, V3 wi, V3 wo)
{
    switch (b.type) {
    case 0: return diffuse_pdf(wi, wo);
    case 1: return rc_pdf(b, wi, wo);
    case 2: return rd_pdf(b, wi, wo);
    case 3: return sl_pdf(b, wi, wo);
    case 4: return ly_pdf(b, wi, wo);
    case 9: return nf_pdf(b, wi, wo);
    default: return 0.f;
    }
}
__device__ __forceinline__ C3 bsdf_sample1(const DevBsdf &b, BsdfRec &r, V2 s, uint64_t aux_key)
{
    switch (b.type) {
    case 0: return diffuse_sample(b.albedo, r, s);
    case 1: return rc_sample(b, r, s);
    case 2: return rd_sample(b, r, s);
    case 3: return sl_sample(b, r, s);
    case 4: return ly_sample(b, r, s, aux_key);
    case 5: return dl_sample(b, r, s);
    case 6: return cd_sample(b, r);
    case 8: return sd_sample(b, r, s);
    case 9: return nf_sample(b, r, s);
    default: return mr_sample(r);
    }
}
// TwoSides (bsdf/TwoSides.cpp:24-70): seen from below, the directions are
// mirrored to the upper side (z negated) before the wrapped BSDF and the
// sampled direction mirrored back
__device__ __forceinline__ C3 bsdf_eval(const DevBsdf &b, V3 wi, V3 wo)
{
    if (b.two_sided && !(wi.z > 0.f)) { wi.z = -wi.z; wo.z = -wo.z; }
    return bsdf_eval1(b, wi, wo);
}
__device__ __forceinline__ float bsdf_pdf(const DevBsdf &b, V3 wi, V3 wo)
{
    if (b.two_sided && !(wi.z > 0.f)) { wi.z = -wi.z; wo.z = -wo.z; }
    return bsdf_pdf1(b, wi, wo);
}
// aux_key: the side-stream key of a LayeredBSDF sample (ly_sample)
__device__ __forceinline__ C3 bsdf_sample(const DevBsdf &b, BsdfRec &r, V2 s, uint64_t aux_key)
{
    if (b.two_sided && !(r.wi.z > 0.f)) {
        r.wi.z = -r.wi.z;
        C3 res = bsdf_sample1(b, r, s, aux_key);
        r.wi.z = -r.wi.z;
        r.wo.z = -r.wo.z;
        return res;
    }
    return bsdf_sample1(b, r, s, aux_key);
}

// ------------------------------------------------------------------ lights
struct LightRec {
    V3 point, to_light, normal;
    C3 intensity;
    float distance, pdf;
    int delta;   // sampled from a delta light (Light::isDelta)
};

__device__ __forceinline__ void tri_verts(const DevScene &S, int tri, V3 &p0, V3 &p1, V3 &p2)
{
    const float *P = S.tri_v + 9 * (size_t)tri;
    p0 = vload(P); p1 = vload(P + 3); p2 = vload(P + 6);
}

// Mesh::sample (geometricShape/Mesh.cpp:38-68) + Triangle::sample (Triangle.cpp:251-273)
__device__ __forceinline__ void mesh_sample(const DevScene &S, int mesh, V2 s, V3 &pt, V3 &n)
{
    const DevMesh &M = S.meshes[mesh];
    float ux = s.x, pdf;
    int index = cdf_sample_reuse(S.mesh_cdf + M.cdf_off, M.n_tris + 1, ux, pdf);
    V2 s2 = v2(ux, s.y);
    int tri = M.first_tri + index;
    V3 p0, p1, p2;
    tri_verts(S, tri, p0, p1, p2);
    V3 b = square_to_triangle(s2);
    pt = (p0 * b.x + p1 * b.y) + p2 * b.z;
    if (S.tri_n && !isnan(S.tri_n[9 * (size_t)tri])) {
        const float *N = S.tri_n + 9 * (size_t)tri;
        n = normalized((b.x * vload(N) + b.y * vload(N + 3)) + b.z * vload(N + 6));
    } else {
        n = normalized(cross(p1 - p0, p2 - p0));
        n = normalized(n);
    }
}
// Mesh::pdf (Mesh.cpp:70-93)
__device__ __forceinline__ float mesh_pdf(const DevScene &S, int mesh, V3 p, V3 sampled, V3 n)
{
    V3 l = p - sampled;
    float dist = norm(l);
    l = normalized(l);
    float c = dot(n, l);
    if (c > 0) return dist * dist / (S.meshes[mesh].area * c);
    return 0.f;
}
__device__ __forceinline__ V3 sphere_normal(const DevSphere &s, V3 p)
{
    return normalized(xf_point(s.to_object, p) - v3(0, 0, 0));
}
// Sphere::sample (Sphere.cpp:146-173)
__device__ __forceinline__ void sphere_sample(const DevSphere &s, V2 u, V3 &pt, V3 &n)
{
    float theta = 2.f * RT_PI * u.x;
    float phi = acosf(2 * u.y - 1.f);
    float c = cosf(phi);
    float sq = sqrtf(1 - c * c);
    V3 p = v3(sq * cosf(theta), sq * sinf(theta), c);
    p = p * s.radius;
    n = normalized(xf_normal(s.to_object, sphere_normal(s, p)));
    pt = xf_point(s.to_world, p);
}
// Plane::sample (Plane.cpp:94-98)
__device__ __forceinline__ void plane_sample(const DevSphere &s, V2 u, V3 &pt, V3 &n)
{
    pt = xf_point(s.to_world, v3(1 - 2 * u.x, 1 - 2 * u.y, 0.f));
    n = normalized(xf_normal(s.to_object, v3(0.f, 0.f, 1.f)));
}
// Sphere::pdf (Sphere.cpp:183-201) with ISampledShape::pdf (ISampledShape.cpp:17-40);
// a Plane has ISampledShape::pdf alone
__device__ __forceinline__ float sphere_pdf(const DevSphere &s, V3 p, V3 sampled, V3 n)
{
    if (s.kind == 1) {
        V3 l = p - sampled;
        float dist = norm(l);
        l = normalized(l);
        float c = dot(n, l);
        if (c >= 0) return dist * dist / (s.area * c);
        return 0.f;
    }
    V3 center = xf_point(s.to_world, v3(0.f, 0.f, 0.f));
    V3 itc = p - center;
    float sqd = sqnorm(itc);
    if (dot(n, itc) < 0.f) return 0.f;
    if (sqd - s.radius * s.radius < RT_EPSILON) {
        V3 l = p - sampled;
        float dist = norm(l);
        l = normalized(l);
        float c = dot(n, l);
        float area = 4.f * RT_PI * s.radius * s.radius * s.radius;
        if (c >= 0) return dist * dist / (area * c);
        return 0.f;
    }
    float st2 = s.radius * s.radius / sqd;
    float ct = sqrtf(smax(0.f, 1 - st2));
    return cone_pdf(ct);
}

// EnvironmentLight (light/EnvironmentLight.cpp)
__device__ __forceinline__ void env_checkxy(const DevLight &L, float &x, float &y)
{
    unsigned W = (unsigned)L.env_w, H = (unsigned)L.env_h;
    if (x >= (float)W) x = (float)((unsigned)(int)x % W) + (x - (float)(int)x);
    else if (x < 0) x = (float)(W - (unsigned)abs((int)x) % W) + (x - (float)(int)x);
    if (y >= (float)H) y = (float)((unsigned)(int)y % H) + (y - (float)(int)y);
    else if (y < 0) y = (float)(H - (unsigned)abs((int)y) % H) + (y - (float)(int)y);
}
__device__ __forceinline__ int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
// core/BasicMath.h:74-90 interp2
__device__ __forceinline__ C3 env_interp(const DevLight &L, float x, float y)
{
    int W = L.env_w, H = L.env_h;
    float ax = x - (float)(int)x, ay = y - (float)(int)y;
    int x0 = iclamp((int)x, 0, W - 2), y0 = iclamp((int)y, 0, H - 2);
    int x1 = x0 + 1 < W ? x0 + 1 : x0; x1 = iclamp(x1, 0, W - 1);
    int y1 = y0 + 1 < H ? y0 + 1 : y0; y1 = iclamp(y1, 0, H - 1);
    const float *a00 = L.env_rgb + 3 * ((size_t)y0 * W + x0);
    const float *a01 = L.env_rgb + 3 * ((size_t)y1 * W + x0);
    const float *a10 = L.env_rgb + 3 * ((size_t)y0 * W + x1);
    const float *a11 = L.env_rgb + 3 * ((size_t)y1 * W + x1);
    float w00 = (1 - ax) * (1 - ay), w01 = (1 - ax) * ay, w10 = ax * (1 - ay), w11 = ax * ay;
    C3 r;
    r.r = ((w00 * a00[0] + w01 * a01[0]) + w10 * a10[0]) + w11 * a11[0];
    r.g = ((w00 * a00[1] + w01 * a01[1]) + w10 * a10[1]) + w11 * a11[1];
    r.b = ((w00 * a00[2] + w01 * a01[2]) + w10 * a10[2]) + w11 * a11[2];
    return r;
}
__device__ __forceinline__ void env_dir_xy(const DevLight &L, V3 dir, float &fx, float &fy)
{
    fx = (spherical_phi(dir) / (2 * RT_PI)) * (float)L.env_w;
    fy = (spherical_theta(dir) / RT_PI) * (float)L.env_h;
    fx += 0.f * (float)L.env_w;
    fy += 0.f * (float)L.env_h;
    env_checkxy(L, fx, fy);
}
__device__ __forceinline__ C3 env_le(const DevLight &L, V3 direction)
{
    V3 dir = normalized(xf_vector(L.env_to_light, direction));
    float fx, fy;
    env_dir_xy(L, dir, fx, fy);
    return env_interp(L, fx, fy) * L.env_scale;
}
__device__ __forceinline__ void env_sample(const DevLight &L, V3 p, V2 s, LightRec &o)
{
    int W = L.env_w, H = L.env_h;
    int row = cdf_sample_guided(L.env_marginal, H + 1, s.x, L.env_marg_guide, L.env_gm);
    int col = cdf_sample_guided(L.env_row_cdf + (size_t)row * (W + 1), W + 1, s.y,
                                L.env_row_guide + (size_t)row * (L.env_gr + 1), L.env_gr);
    float rcol = (float)col + 0.f * (float)W;
    float rrow = (float)row + 0.f * (float)H;
    env_checkxy(L, rcol, rrow);
    row = (int)rrow;
    col = (int)rcol;
    float theta = RT_PI * (float)row / (float)H;
    float phi = 2 * RT_PI * (float)col / (float)W;
    float st = sinf(theta);
    V3 dir = cartesian_from_spherical(theta, phi);
    dir = xf_vector(L.env_to_world, dir);
    o.distance = L.env_radius;
    dir = normalized(dir);
    o.to_light = dir;
    o.point = p + L.env_radius * dir;
    o.normal = v3(0, 0, 0);
    int cx = iclamp(col, 0, W - 1), cy = iclamp(row, 0, H - 1);
    o.intensity = cload(L.env_rgb + 3 * ((size_t)cy * W + cx)) * L.env_scale;
    float pdf = lum(o.intensity) * L.env_weight[row];
    float den = L.env_marginal_sum * (2 * RT_PI / (float)W);
    den = den * (RT_PI / (float)H);
    pdf = pdf / den;
    pdf /= smax(fabsf(st), RT_EPSILON);
    o.pdf = pdf;
}
__device__ __forceinline__ float env_pdf(const DevLight &L, V3 to_light)
{
    V3 dir = normalized(xf_vector(L.env_to_light, to_light));
    float fx, fy;
    env_dir_xy(L, dir, fx, fy);
    float st = sinf(fy);
    float den = L.env_marginal_sum * (2 * RT_PI / (float)L.env_w);
    den = den * (RT_PI / (float)L.env_h);
    float nf = L.env_weight[(int)fy] / den;
    float lm = lum(env_interp(L, fx, fy) * L.env_scale);
    float pdf = lm * nf;
    pdf /= smax(fabsf(st), RT_EPSILON);
    return pdf;
}

// PointLight::sample (light/PointLight.cpp:20-33) and SpotLight::sample /
// falloff (light/SpotLight.cpp:19-44): intensity / distance^2 towards the
// light's position, pdf 1.  The spot's cosine is the z of the inverse-toWorld
// image of -to_light, not renormalised, as in SpotLight::falloff.
__device__ __forceinline__ void delta_light_sample(const DevLight &L, V3 p, LightRec &o)
{
    V3 pos = vload(L.position);
    o.to_light = pos - p;
    o.distance = norm(o.to_light);
    float inv = 1.f / o.distance;
    o.to_light = o.to_light * inv;
    float f = 1.f;
    if (L.type == 3) {
        float ct = xf_vector(L.spot_to_light, -o.to_light).z;
        if (ct < L.cos_total_width) f = 0.f;
        else if (ct > L.cos_falloff_start) f = 1.f;
        else {
            float dl = (ct - L.cos_total_width) / (L.cos_falloff_start - L.cos_total_width);
            f = (dl * dl) * (dl * dl);
        }
    }
    C3 I = cload(L.intensity);
    if (L.type == 3) I = I * f;
    o.intensity = (I * inv) * inv;
    o.point = pos;
    o.normal = v3(0.f, 0.f, 0.f);
    o.pdf = 1.f;
}

__device__ __forceinline__ float light_pdf(const DevScene &S, int light, V3 p, V3 point, V3 normal, V3 to_light)
{
    const DevLight &L = S.lights[light];
    if (L.type >= 2) return 0.f;   // PointLight / SpotLight::pdf
    if (L.type == 1) return env_pdf(L, to_light);
    if (L.shape_kind == 0) return mesh_pdf(S, L.shape, p, point, normal);
    return sphere_pdf(S.spheres[L.shape], p, point, normal);
}

// Light::sample dispatch: MeshLight.cpp:32-64, AreaLight.cpp:31-55, EnvironmentLight.cpp:85-146
__device__ __forceinline__ void light_sample(const DevScene &S, int light, V3 p, V2 s, LightRec &o)
{
    const DevLight &L = S.lights[light];
    o.pdf = 0.f;
    o.distance = 0.f;
    o.intensity = cfill(0.f);
    o.delta = L.type >= 2;
    if (L.type == 1) { env_sample(L, p, s, o); return; }
    if (o.delta) { delta_light_sample(L, p, o); return; }
    V3 pt, n;
    if (L.shape_kind == 0) mesh_sample(S, L.shape, s, pt, n);
    else if (S.spheres[L.shape].kind == 1) plane_sample(S.spheres[L.shape], s, pt, n);
    else sphere_sample(S.spheres[L.shape], s, pt, n);
    o.point = pt;
    o.normal = n;
    o.to_light = pt - p;
    o.distance = norm(o.to_light);
    o.to_light = o.to_light / o.distance;
    float c = dot(n, -o.to_light);
    if (L.mesh_light && L.shape_kind == 0) {
        if (c <= 0) { o.intensity = cfill(0.f); o.pdf = 0.f; }
        else { o.intensity = cload(L.radiance); o.pdf = o.distance * o.distance / (S.meshes[L.shape].area * c); }
    } else {
        if (c < 0) { o.intensity = cfill(0.f); o.pdf = 0.f; }
        else { o.intensity = cload(L.radiance); o.pdf = light_pdf(S, light, p, o.point, o.normal, o.to_light); }
    }
}
// AreaLight::le (light/AreaLight.h:27-32)
__device__ __forceinline__ C3 area_le(const DevScene &S, int light, V3 dir, V3 n)
{
    if (dot(dir, n) > 0.f) return cload(S.lights[light].radiance);
    return cfill(0.f);
}
__device__ __forceinline__ float power_heuristic(float a, float b)
{
    float l = a * a, r = b * b;
    return l / (l + r);
}

// ------------------------------------------------------------------ camera (NoriPerspective.cpp:80-118)
__device__ __forceinline__ Ray camera_ray(const DevCamera &c, float px, float py, V2 lens)
{
    V3 nearP = xf_point(c.sample_to_camera, v3(px * c.inv_w, py * c.inv_h, 0.0f));
    V3 d = normalized(nearP);
    float invZ = 1.0f / d.z;
    V3 o = v3(0.f, 0.f, 0.f);
    if (c.aperture_radius > 0.f) {
        V2 s = concentric_disk(lens);
        s.x *= c.aperture_radius; s.y *= c.aperture_radius;
        o = v3(s.x, s.y, 0.f);
        float tdist = c.focal_plane * invZ;
        V3 fp = tdist * d;
        d = normalized(fp - o);
    }
    return make_ray(xf_point(c.camera_to_world, o), xf_vector(c.camera_to_world, d), c.near_clip * invZ,
                    c.far_clip * invZ);
}

// ------------------------------------------------------------------ phase functions
__device__ __forceinline__ float phase_eval(const DevMedium &m, V3 wi, V3 wo)
{
    if (m.phase == 0) return RT_INV_FOUR_PI;
    float g = m.g;
    float c = dot(-wi, wo);
    return RT_INV_FOUR_PI * (1 - g * g) / powf(1 + g * g - 2 * g * c, 1.5f);
}
// HGPhaseFunction::sample (HGPhaseFunction.cpp:27-42), world-frame direction
__device__ __forceinline__ float phase_sample(const DevMedium &m, V3 wi, V2 u, V3 &wo, float &pdf)
{
    if (m.phase == 0) {
        wo = uniform_sphere(u);
        pdf = RT_INV_FOUR_PI;
        return 1.f;
    }
    float g = m.g;
    float ct;
    if (g < RT_EPSILON) ct = 1.f - 2.f * u.x;
    else ct = (1 + g * g - ((1 - g * g) * (1 - g * g) / (1 - g + 2 * g * u.x))) / (2 * g);
    float theta = acosf(ct);
    float phi = 2 * RT_PI * u.y;
    wo = cartesian_from_spherical(theta, phi);
    pdf = phase_eval(m, wi, wo);
    return 1.f;
}

// ------------------------------------------------------------------ media
__device__ __forceinline__ C3 homog_tr(const DevMedium &m, float mint, float maxt)
{
    float t = maxt - mint;
    return c3(expf(-m.sigma_t[0] * t), expf(-m.sigma_t[1] * t), expf(-m.sigma_t[2] * t));
}
// GridVolume::lookupSigmaT (volume/GridVolume.cpp:118-149) * scale
__device__ __forceinline__ float grid_lookup(const DevMedium &m, V3 pa)
{
    float px = pa.x * (float)m.res[0], py = pa.y * (float)m.res[1], pz = pa.z * (float)m.res[2];
    float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    if (ix < 0 || iy < 0 || iz < 0) return 0.0f * m.scale;
    if (ix >= m.res[0] - 1 || iy >= m.res[1] - 1 || iz >= m.res[2] - 1) return 0.0f * m.scale;
    size_t row = (size_t)m.res[0], slab = row * (size_t)m.res[1];
    size_t off = (size_t)iz * slab + (size_t)iy * row + (size_t)ix;
    const float *D = m.density;
    float d000 = __ldg(D + off), d001 = __ldg(D + off + 1), d010 = __ldg(D + off + row),
          d011 = __ldg(D + off + row + 1);
    float d100 = __ldg(D + off + slab), d101 = __ldg(D + off + slab + 1), d110 = __ldg(D + off + slab + row),
          d111 = __ldg(D + off + slab + row + 1);
    float w1x = px - fx, w1y = py - fy, w1z = pz - fz;
    float w0x = 1 - w1x, w0y = 1 - w1y, w0z = 1 - w1z;
    float v = ((d000 * w0x + d001 * w1x) * w0y + (d010 * w0x + d011 * w1x) * w1y) * w0z +
              ((d100 * w0x + d101 * w1x) * w0y + (d110 * w0x + d111 * w1x) * w1y) * w1z;
    return v * m.scale;
}

#define RT_TRACK_CAP (1 << 20)

// Heterogeneous::transmittance (medium/Heterogeneous.cpp:419-489): ratio tracking + RR
__device__ __forceinline__ C3 hetero_tr(const DevMedium &m, Ray wr, Pcg32 &rng, int &limit)
{
    V3 o = xf_point(m.world_to_array, wr.o), d = xf_vector(m.world_to_array, wr.d);
    float tmax = wr.maxt - wr.mint;
    float tr = 1.f, st;
    int breaker = 0;
    float nearT, farT;
    const float bmin[3] = {0.f, 0.f, 0.f}, bmax[3] = {1.f, 1.f, 1.f};
    if (!ref_box_hit(bmin, bmax, o, d, wr.mint, wr.maxt, nearT, farT)) return cfill(1.f);
    tmax = smin(tmax, farT);
    st = smax(nearT, wr.mint);
    for (;;) {
        st += -logf(1.f - next1d(rng)) / m.max_sigma_t;
        float proba = grid_lookup(m, o + st * d);
        if (st >= tmax) return cfill(tr);
        tr *= 1 - smax(0.f, proba / m.max_sigma_t);
        const float threshold = .1f;
        if (tr < threshold) {
            float q = smax(.05f, 1 - tr);
            if (next1d(rng) < q) return cfill(0.f);
            tr /= 1 - q;
        }
        if (breaker > 1024) return cfill(0.f);
        breaker++;
    }
}

// Heterogeneous::sampleDistance (Heterogeneous.cpp:491-546): delta tracking
__device__ __forceinline__ bool hetero_sample(const DevMedium &m, Ray wr, Pcg32 &rng, float &t, C3 &w, C3 &em,
                                              int &limit)
{
    t = wr.mint;
    float cur = 0.f;
    float nearT, farT;
    if (!ref_box_hit(m.wbox_min, m.wbox_max, wr.o, wr.d, wr.mint, wr.maxt, nearT, farT)) {
        w = cfill(1.f); em = cfill(0.f); t = wr.maxt;
        return false;
    }
    float tmax = smin(wr.maxt, farT);
    int steps = 0;
    for (;;) {
        t += -logf(1.f - next1d(rng)) / m.max_sigma_t;
        if (t > tmax) { w = cfill(1.f); em = cfill(0.f); t = tmax; return false; }
        V3 pw = wr.o + t * wr.d;
        cur = grid_lookup(m, xf_point(m.world_to_array, pw));
        float proba = cur / m.max_sigma_t;
        if (next1d(rng) < proba) break;
        if (++steps >= RT_TRACK_CAP) { limit = 1; w = cfill(0.f); em = cfill(0.f); return true; }
    }
    if (cur != 0.f) w = cload(m.albedo); else w = cfill(0.f);
    em = cfill(0.f);
    return true;
}

__device__ __forceinline__ bool medium_sample(const DevMedium &m, Ray r, Pcg32 &rng, float &t, C3 &w, C3 &em,
                                              int &limit)
{
    if (m.type == 1) return hetero_sample(m, r, rng, t, w, em, limit);
    // Homogeneous::sampleDistance (Homogeneous.cpp:37-78)
    int ch = (int)(next1d(rng) * 3);
    float ext = ch == 0 ? m.sigma_t[0] : (ch == 1 ? m.sigma_t[1] : m.sigma_t[2]);
    ext += RT_EPSILON;
    t = -logf(1.f - next1d(rng)) / ext;
    if (t > r.maxt) {
        t = r.maxt;
        C3 e = c3(expf(-m.sigma_t[0] * t), expf(-m.sigma_t[1] * t), expf(-m.sigma_t[2] * t));
        float pdf = cavg(e);
        w = homog_tr(m, r.mint, r.maxt) / pdf;
        em = cfill(0.f);
        return false;
    }
    C3 e = c3(m.sigma_t[0] * expf(-m.sigma_t[0] * t), m.sigma_t[1] * expf(-m.sigma_t[1] * t),
              m.sigma_t[2] * expf(-m.sigma_t[2] * t));
    float pdf = cavg(e);
    t += r.mint;
    w = (cload(m.sigma_s) * homog_tr(m, r.mint, t)) / pdf;
    em = cfill(0.f) / cload(m.sigma_t);
    return true;
}
__device__ __forceinline__ C3 medium_tr(const DevMedium &m, Ray r, Pcg32 &rng, int &limit)
{
    if (m.type == 1) return hetero_tr(m, r, rng, limit);
    return homog_tr(m, r.mint, r.maxt);
}
