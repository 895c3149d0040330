/*
 * CPU oracle, part 3: scene set-up, the two integrators, the film and the
 * tile render loop.  TEST INFRASTRUCTURE ONLY -- see oracle.h.
 *
 * Integrators: integrator/PathTracingMIS.cpp:27-262,
 * integrator/VolPathTracing.cpp:25-424 and the light-sampling helpers of
 * integrator/Integrator.cpp:24-238.  Render loop: core/Scene.cpp:83-95,
 * core/SampleJob.cpp:28-72.  Film: core/Screen.cpp:44-157 with the box
 * filter (filter/BoxFilter.h:55, filter/ReconstructionFilter.h:54-63).
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

int32_t oracle_version(void) { return 1; }

/* ---------------- primitive attribute helpers ---------------- */
static int prim_mesh(const o_scene *sc, int prim) { return sc->tri_mesh[prim]; }
static int prim_bsdf(const o_scene *sc, int prim)
{
    if (prim >= 0) return sc->d->meshes[prim_mesh(sc, prim)].bsdf;
    return sc->d->spheres[-prim - 2].bsdf;
}
static int prim_light(const o_scene *sc, int prim)
{
    if (prim >= 0) return sc->d->meshes[prim_mesh(sc, prim)].light;
    return sc->d->spheres[-prim - 2].light;
}
static int prim_interior(const o_scene *sc, int prim)
{
    if (prim >= 0) return sc->d->meshes[prim_mesh(sc, prim)].interior;
    return sc->d->spheres[-prim - 2].interior;
}
static int prim_exterior(const o_scene *sc, int prim)
{
    if (prim >= 0) return sc->d->meshes[prim_mesh(sc, prim)].exterior;
    return sc->d->spheres[-prim - 2].exterior;
}
/* Intersection::isMediumTransition / getMedium (core/Intersection.h:43-57) */
static int hit_transition(const o_scene *sc, const o_hit *h)
{
    return prim_interior(sc, h->prim) != prim_exterior(sc, h->prim);
}
static int hit_medium(const o_scene *sc, const o_hit *h, v3 d)
{
    if (v3_dot(h->n, d) < 0.f) return prim_interior(sc, h->prim);
    return prim_exterior(sc, h->prim);
}
static v3 to_local(const o_hit *h, v3 v) { return mk3(v3_dot(v, h->s), v3_dot(v, h->tt), v3_dot(v, h->n)); }
static v3 to_world(const o_hit *h, v3 v)
{
    return v3_add(v3_add(v3_muls(h->s, v.x), v3_muls(h->tt, v.y)), v3_muls(h->n, v.z));
}
/* AreaLight::le (light/AreaLight.h:27-32) */
static c3 area_le(const o_scene *sc, int light, v3 dir, v3 n)
{
    if (v3_dot(dir, n) > 0.f) return c3_from(sc->d->lights[light].radiance);
    return cfill(0.f);
}
static float power_heuristic(float a, float b)
{
    float l = a * a, r = b * b;
    return l / (l + r);
}
static c3 c3_mul4(c3 a, c3 b, c3 c, float d, float e)
{
    c3 r = c3_mul(c3_mul(a, b), c);
    return c3_muls(c3_muls(r, d), e);
}

/* ---------------- light power (for the weighted strategy) ---------------- */
static c3 light_power(const o_scene *sc, int l)
{
    const rt_light_desc *L = &sc->d->lights[l];
    if (L->type == RT_LIGHT_ENV) {
        float R = sc->env[l].sphere_radius;
        return c3_muls(cfill(1.f), 4 * O_PI * R * R);
    }
    if (L->type == RT_LIGHT_POINT)   /* PointLight.h power(): 4 pi I */
        return c3_muls(c3_from(L->intensity), 4 * O_PI);
    if (L->type == RT_LIGHT_SPOT)    /* SpotLight.h power(): 2 pi I (1 - (cosFalloffStart + cosTotalWidth) / 2) */
        return c3_muls(c3_muls(c3_from(L->intensity), 2 * O_PI),
                       1.f - 0.5f * (L->cos_falloff_start + L->cos_total_width));
    float area;
    if (L->shape_kind == RT_SHAPE_MESH) area = sc->mesh[L->shape].area;
    else if (sc->d->spheres[L->shape].kind == RT_ANALYTIC_PLANE) area = o_plane_area(&sc->d->spheres[L->shape]);
    else { float r = sc->d->spheres[L->shape].radius; area = 4.f * O_PI * r * r * r; }
    c3 p = mkc(O_PI * L->radiance[0], O_PI * L->radiance[1], O_PI * L->radiance[2]);
    return c3_muls(p, area);
}

/* Integrator::initialize (Integrator.cpp:24-38) */
static void build_light_cdf(o_scene *sc, int strategy)
{
    if (sc->light_cdf.cdf) o_cdf_free(&sc->light_cdf);
    o_cdf_init(&sc->light_cdf);
    int n = sc->d->n_lights;
    float pu = (float)1. / (float)n;
    for (int l = 0; l < n; l++) {
        if (strategy == RT_STRATEGY_ONE_LIGHT_WEIGHTED) o_cdf_add(&sc->light_cdf, c3_lum(light_power(sc, l)));
        else o_cdf_add(&sc->light_cdf, pu);
    }
    o_cdf_normalize(&sc->light_cdf);
    sc->strategy = strategy;
}

/* ---------------- scene creation ---------------- */
static void mat_mul4(const double *a, const double *b, double *o)
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a[i * 4 + k] * b[k * 4 + j];
            o[i * 4 + j] = s;
        }
}
/* general 4x4 inverse (cofactor expansion, double) */
static int mat_inv4(const double *m, double *inv)
{
    double t[16];
    t[0] = m[5]*m[10]*m[15] - m[5]*m[11]*m[14] - m[9]*m[6]*m[15] + m[9]*m[7]*m[14] + m[13]*m[6]*m[11] - m[13]*m[7]*m[10];
    t[4] = -m[4]*m[10]*m[15] + m[4]*m[11]*m[14] + m[8]*m[6]*m[15] - m[8]*m[7]*m[14] - m[12]*m[6]*m[11] + m[12]*m[7]*m[10];
    t[8] = m[4]*m[9]*m[15] - m[4]*m[11]*m[13] - m[8]*m[5]*m[15] + m[8]*m[7]*m[13] + m[12]*m[5]*m[11] - m[12]*m[7]*m[9];
    t[12] = -m[4]*m[9]*m[14] + m[4]*m[10]*m[13] + m[8]*m[5]*m[14] - m[8]*m[6]*m[13] - m[12]*m[5]*m[10] + m[12]*m[6]*m[9];
    t[1] = -m[1]*m[10]*m[15] + m[1]*m[11]*m[14] + m[9]*m[2]*m[15] - m[9]*m[3]*m[14] - m[13]*m[2]*m[11] + m[13]*m[3]*m[10];
    t[5] = m[0]*m[10]*m[15] - m[0]*m[11]*m[14] - m[8]*m[2]*m[15] + m[8]*m[3]*m[14] + m[12]*m[2]*m[11] - m[12]*m[3]*m[10];
    t[9] = -m[0]*m[9]*m[15] + m[0]*m[11]*m[13] + m[8]*m[1]*m[15] - m[8]*m[3]*m[13] - m[12]*m[1]*m[11] + m[12]*m[3]*m[9];
    t[13] = m[0]*m[9]*m[14] - m[0]*m[10]*m[13] - m[8]*m[1]*m[14] + m[8]*m[2]*m[13] + m[12]*m[1]*m[10] - m[12]*m[2]*m[9];
    t[2] = m[1]*m[6]*m[15] - m[1]*m[7]*m[14] - m[5]*m[2]*m[15] + m[5]*m[3]*m[14] + m[13]*m[2]*m[7] - m[13]*m[3]*m[6];
    t[6] = -m[0]*m[6]*m[15] + m[0]*m[7]*m[14] + m[4]*m[2]*m[15] - m[4]*m[3]*m[14] - m[12]*m[2]*m[7] + m[12]*m[3]*m[6];
    t[10] = m[0]*m[5]*m[15] - m[0]*m[7]*m[13] - m[4]*m[1]*m[15] + m[4]*m[3]*m[13] + m[12]*m[1]*m[7] - m[12]*m[3]*m[5];
    t[14] = -m[0]*m[5]*m[14] + m[0]*m[6]*m[13] + m[4]*m[1]*m[14] - m[4]*m[2]*m[13] - m[12]*m[1]*m[6] + m[12]*m[2]*m[5];
    t[3] = -m[1]*m[6]*m[11] + m[1]*m[7]*m[10] + m[5]*m[2]*m[11] - m[5]*m[3]*m[10] - m[9]*m[2]*m[7] + m[9]*m[3]*m[6];
    t[7] = m[0]*m[6]*m[11] - m[0]*m[7]*m[10] - m[4]*m[2]*m[11] + m[4]*m[3]*m[10] + m[8]*m[2]*m[7] - m[8]*m[3]*m[6];
    t[11] = -m[0]*m[5]*m[11] + m[0]*m[7]*m[9] + m[4]*m[1]*m[11] - m[4]*m[3]*m[9] - m[8]*m[1]*m[7] + m[8]*m[3]*m[5];
    t[15] = m[0]*m[5]*m[10] - m[0]*m[6]*m[9] - m[4]*m[1]*m[10] + m[4]*m[2]*m[9] + m[8]*m[1]*m[6] - m[8]*m[2]*m[5];
    double det = m[0] * t[0] + m[1] * t[4] + m[2] * t[8] + m[3] * t[12];
    if (det == 0) return 0;
    for (int i = 0; i < 16; i++) inv[i] = t[i] / det;
    return 1;
}

/* Heterogeneous::setOwnerBBox (medium/Heterogeneous.cpp:281-369); the
 * matrix products are formed in double and rounded once to binary32. */
static void setup_hetero(o_scene *sc, int mi, const float *bmin, const float *bmax)
{
    const rt_medium_desc *m = &sc->d->media[mi];
    o_medium_rt *M = &sc->med[mi];
    double gmn[3], gmx[3], bmn[3], bmx[3];
    for (int i = 0; i < 3; i++) { gmn[i] = m->grid_min[i]; gmx[i] = m->grid_max[i]; bmn[i] = bmin[i]; bmx[i] = bmax[i]; }
    double ratio = (bmx[0] - bmn[0]) / (gmx[0] - gmn[0]);
    double ry = (bmx[1] - bmn[1]) / (gmx[1] - gmn[1]);
    if (ry < ratio) ratio = ry;
    double rz = (bmx[2] - bmn[2]) / (gmx[2] - gmn[2]);
    if (rz < ratio) ratio = rz;
    double S[16] = {0};
    double ext[3];
    for (int i = 0; i < 3; i++) { ext[i] = (gmx[i] - gmn[i]) * ratio; S[i * 5] = 1.0 / ext[i]; }
    S[15] = 1;
    double T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    for (int i = 0; i < 3; i++) {
        double tr = m->centered ? -(bmn[i] + ((bmx[i] - bmn[i]) / 2.0 - ext[i] / 2.0)) : -bmn[i];
        T[i * 4 + 3] = tr;
    }
    double W[16], Winv[16];
    for (int i = 0; i < 16; i++) W[i] = m->to_world[i];
    if (!mat_inv4(W, Winv)) memcpy(Winv, W, sizeof(W));
    double ST[16], A[16], Ainv[16];
    mat_mul4(S, T, ST);
    mat_mul4(ST, Winv, A);
    mat_inv4(A, Ainv);
    for (int i = 0; i < 16; i++) { M->world_to_array[i] = (float)A[i]; M->array_to_world[i] = (float)Ainv[i]; }
    /* world box = array_to_world applied to the unit box (Transform.h:145-158) */
    float mn[3] = {O_MAX_REAL, O_MAX_REAL, O_MAX_REAL}, mx[3] = {-O_MAX_REAL, -O_MAX_REAL, -O_MAX_REAL};
    const float c[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 1, 0}};
    for (int k = 0; k < 8; k++) {
        v3 p = xf_point(M->array_to_world, mk3(c[k][0], c[k][1], c[k][2]));
        mn[0] = smin(mn[0], p.x); mn[1] = smin(mn[1], p.y); mn[2] = smin(mn[2], p.z);
        mx[0] = smax(mx[0], p.x); mx[1] = smax(mx[1], p.y); mx[2] = smax(mx[2], p.z);
    }
    memcpy(M->wbox_min, mn, sizeof(mn));
    memcpy(M->wbox_max, mx, sizeof(mx));
    /* GridVolume::getMaxSigmaT (volume/GridVolume.cpp:106-116) * scale */
    size_t nv = (size_t)m->res[0] * m->res[1] * m->res[2];
    float mxs = m->density[0];
    for (size_t i = 1; i < nv; i++) if (m->density[i] > mxs) mxs = m->density[i];
    M->max_sigma_t = mxs * m->scale;
}

o_scene *oracle_scene_create(const rt_scene_desc *d, int32_t strategy)
{
    o_scene *sc = (o_scene *)calloc(1, sizeof(o_scene));
    sc->d = d;
    sc->tri_mesh = (int *)malloc(sizeof(int) * (size_t)(d->n_triangles > 0 ? d->n_triangles : 1));
    sc->mesh = (o_mesh_rt *)calloc((size_t)(d->n_meshes > 0 ? d->n_meshes : 1), sizeof(o_mesh_rt));
    for (int m = 0; m < d->n_meshes; m++) {
        const rt_mesh_desc *M = &d->meshes[m];
        o_cdf_init(&sc->mesh[m].cdf);
        sc->mesh[m].area = 0.f;
        for (int i = 0; i < M->n_tris; i++) {
            int tri = M->first_tri + i;
            sc->tri_mesh[tri] = m;
            const int32_t *ix = d->indices + 3 * (size_t)tri;
            v3 p0 = v3_from(d->vertices + 3 * (size_t)ix[0]);
            v3 p1 = v3_from(d->vertices + 3 * (size_t)ix[1]);
            v3 p2 = v3_from(d->vertices + 3 * (size_t)ix[2]);
            /* Triangle::triSurfaceArea (Triangle.h:128-135) */
            float a = 0.5f * v3_norm(v3_cross(v3_sub(p1, p0), v3_sub(p2, p0)));
            o_cdf_add(&sc->mesh[m].cdf, a);
            sc->mesh[m].area += a;
        }
        o_cdf_normalize(&sc->mesh[m].cdf);
    }
    /* media: owner boxes from the meshes (MeshFactory.h:133-136) */
    sc->med = (o_medium_rt *)calloc((size_t)(d->n_media > 0 ? d->n_media : 1), sizeof(o_medium_rt));
    sc->top = o_bvh_build_scene(sc);
    /* scene box = top-level root box */
    for (int i = 0; i < 3; i++) { sc->bmin[i] = O_MAX_REAL; sc->bmax[i] = -O_MAX_REAL; }
    {
        float b[6]; int nodes;
        oracle_scene_info(sc, b, &nodes);
        for (int i = 0; i < 3; i++) { sc->bmin[i] = b[i]; sc->bmax[i] = b[3 + i]; }
    }
    for (int m = 0; m < d->n_meshes; m++) {
        const rt_mesh_desc *M = &d->meshes[m];
        if (M->n_tris == 0) continue;
        float mn[3] = {O_MAX_REAL, O_MAX_REAL, O_MAX_REAL}, mx[3] = {-O_MAX_REAL, -O_MAX_REAL, -O_MAX_REAL};
        for (int i = 0; i < M->n_tris; i++) {
            const int32_t *ix = d->indices + 3 * (size_t)(M->first_tri + i);
            for (int k = 0; k < 3; k++) {
                const float *p = d->vertices + 3 * (size_t)ix[k];
                for (int a = 0; a < 3; a++) { mn[a] = smin(mn[a], p[a]); mx[a] = smax(mx[a], p[a]); }
            }
        }
        if (M->interior >= 0 && d->media[M->interior].type == RT_MEDIUM_HETEROGENEOUS) setup_hetero(sc, M->interior, mn, mx);
        if (M->exterior >= 0 && d->media[M->exterior].type == RT_MEDIUM_HETEROGENEOUS) setup_hetero(sc, M->exterior, mn, mx);
    }
    /* environment lights (EnvironmentLight.cpp:8-73, 256-262) */
    sc->env = (o_env_rt *)calloc((size_t)(d->n_lights > 0 ? d->n_lights : 1), sizeof(o_env_rt));
    for (int l = 0; l < d->n_lights; l++) {
        const rt_light_desc *L = &d->lights[l];
        if (L->type != RT_LIGHT_ENV) continue;
        o_env_rt *E = &sc->env[l];
        int W = L->env_width, H = L->env_height;
        E->row = (o_cdf *)calloc((size_t)H, sizeof(o_cdf));
        E->weight = (float *)malloc(sizeof(float) * (size_t)H);
        o_cdf_init(&E->marginal);
        for (int i = 0; i < H; i++) {
            float w = sinf(O_PI * ((float)i + 0.5f) / (float)H);
            o_cdf_init(&E->row[i]);
            for (int j = 0; j < W; j++) {
                const float *p = L->env_rgb + 3 * ((size_t)i * W + j);
                o_cdf_add(&E->row[i], c3_lum(c3_muls(c3_from(p), L->env_scale)));
            }
            E->weight[i] = w;
            o_cdf_add(&E->marginal, E->row[i].sum * w);
            o_cdf_normalize(&E->row[i]);
        }
        o_cdf_normalize(&E->marginal);
        v3 bmn = v3_from(sc->bmin), bmx = v3_from(sc->bmax);
        v3 c = v3_smul(0.5f, v3_add(bmx, bmn));
        E->center = c;
        E->sphere_radius = 2 * smax(v3_norm(v3_sub(bmn, c)), v3_norm(v3_sub(bmx, c)));
    }
    build_light_cdf(sc, strategy);
    return sc;
}

/* Pin hook: the bounding sphere (centre, radius) that
 * EnvironmentLight::initialize (EnvironmentLight.cpp:256-262) gives light
 * `light` from the scene box. */
int32_t oracle_env_sphere(const o_scene *sc, int32_t light, float *out4)
{
    if (light < 0 || light >= sc->d->n_lights || sc->d->lights[light].type != RT_LIGHT_ENV) return RT_ERR_INVALID;
    const o_env_rt *E = &sc->env[light];
    out4[0] = E->center.x; out4[1] = E->center.y; out4[2] = E->center.z; out4[3] = E->sphere_radius;
    return RT_OK;
}

void oracle_scene_destroy(o_scene *sc)
{
    if (!sc) return;
    const rt_scene_desc *d = sc->d;
    for (int m = 0; m < d->n_meshes; m++) o_cdf_free(&sc->mesh[m].cdf);
    for (int l = 0; l < d->n_lights; l++) {
        if (d->lights[l].type != RT_LIGHT_ENV) continue;
        for (int i = 0; i < d->lights[l].env_height; i++) o_cdf_free(&sc->env[l].row[i]);
        free(sc->env[l].row); free(sc->env[l].weight); o_cdf_free(&sc->env[l].marginal);
    }
    if (sc->light_cdf.cdf) o_cdf_free(&sc->light_cdf);
    o_bvh_free(sc->top);
    free(sc->env); free(sc->med); free(sc->mesh); free(sc->tri_mesh); free(sc);
}

/* ---------------- light sampling (Integrator.cpp:137-238) ---------------- */
/* Integrator::sampleOneLight (Integrator.cpp:222-238) */
static c3 sample_one_light(const o_scene *sc, int light, v3 p, v2 s, o_light_rec *li)
{
    o_light_sample(sc, light, p, s, li);
    if (li->pdf > 0 && c3_lum(li->intensity) > 0) {
        o_ray sh = o_ray_make(p, li->to_light, O_EPSILON, li->distance - O_EPSILON);
        o_hit tmp;
        if (!o_intersect(sc, &sh, &tmp, 1)) return c3_divs(li->intensity, li->pdf);
    }
    return cfill(0.f);
}
/* Integrator::sampleLightDirect (Integrator.cpp:176-218) */
static c3 sample_light_direct(const o_scene *sc, v3 p, v2 s, o_light_rec *li)
{
    if (sc->d->n_lights == 0) return cfill(0.f);
    float lw;
    int idx = o_cdf_sample_reuse_pdf(&sc->light_cdf, &s.x, &lw);
    c3 v = sample_one_light(sc, idx, p, s, li);
    li->pdf *= lw;
    return c3_divs(v, lw);
}

/* Integrator::evalTransmittance (Integrator.cpp:81-133) */
static c3 eval_transmittance(const o_scene *sc, o_ray ray, int medium, o_sampler *s)
{
    o_ray tr_ray = ray;
    o_hit it;
    c3 tr = cfill(1.f);
    float dist = ray.maxt;
    int first = 1;
    for (;;) {
        int inter = o_intersect(sc, &tr_ray, &it, 0);
        if (inter && prim_bsdf(sc, it.prim) >= 0) return cfill(0.f);
        if (inter) dist -= it.t;
        if (medium >= 0) {
            o_ray mr = o_ray_make(tr_ray.o, tr_ray.d, first ? tr_ray.mint : 0.f, inter ? it.t : dist);
            tr = c3_mul(tr, o_medium_transmittance(sc, medium, &mr, s));
        }
        first = 0;
        if (!inter || c3_iszero(tr)) return tr;
        if (c3_iszero(tr)) return tr;
        v3 np = v3_add(tr_ray.o, v3_smul(it.t, tr_ray.d));
        tr_ray = o_ray_make(np, tr_ray.d, O_EPSILON, dist);
        if (hit_transition(sc, &it)) medium = hit_medium(sc, &it, tr_ray.d);
    }
}

/* Integrator::sampleAttenuatedLightDirect (Integrator.cpp:137-172) */
static c3 sample_attenuated_light(const o_scene *sc, v3 p, o_sampler *s, o_light_rec *li, int medium)
{
    c3 value = cfill(0.f);
    if (sc->d->n_lights == 0) return value;
    v2 u = o_next2d(s);
    float lw;
    int idx = o_cdf_sample_reuse_pdf(&sc->light_cdf, &u.x, &lw);
    o_light_sample(sc, idx, p, u, li);
    if (li->pdf > 0 && c3_lum(li->intensity) > 0) {
        o_ray sh = o_ray_make(p, li->to_light, O_EPSILON, li->distance - O_EPSILON);
        c3 tr = eval_transmittance(sc, sh, medium, s);
        li->pdf *= lw;
        value = c3_divs(c3_mul(tr, li->intensity), li->pdf);
    }
    return value;
}

/* ---------------- PathTracingMIS::li (PathTracingMIS.cpp:27-262) ---------------- */
static c3 li_path_mis(const o_scene *sc, const rt_render_desc *rd, o_sampler *s, o_ray ray)
{
    c3 L = cfill(0.f), T = cfill(1.f);
    float eta = 1.f;
    int depth = 0, emission = 1;
    int env = sc->d->env_light;
    o_hit it;
    if (!o_intersect(sc, &ray, &it, 0)) {
        if (emission && env >= 0) L = c3_add(L, o_env_le(sc, env, ray.d));
        return L;
    }
    while (depth < rd->max_depth) {
        int bsdf = prim_bsdf(sc, it.prim);
        if (bsdf < 0) return L;
        rt_bsdf_desc Btex;
        const rt_bsdf_desc *B = o_bsdf_at(sc->d, &sc->d->bsdfs[bsdf], it.uv, &Btex);
        int hl = prim_light(sc, it.prim);
        if (emission && hl >= 0) L = c3_add(L, c3_mul(T, area_le(sc, hl, v3_neg(ray.d), it.n)));
        /* light sampling */
        if (sc->strategy == RT_STRATEGY_ALL_LIGHTS) {
            for (int l = 0; l < sc->d->n_lights; l++) {
                o_light_rec li;
                c3 value = sample_one_light(sc, l, it.p, o_next2d(s), &li);
                if (!c3_iszero(value)) {
                    o_bsdf_rec r;
                    r.wi = to_local(&it, li.to_light); r.wo = to_local(&it, v3_neg(ray.d));
                    float ct = fabsf(r.wi.z);
                    float bp = o_light_is_delta(sc, l) ? 0.f : o_bsdf_pdf(B, &r);   /* PathTracingMIS.cpp:102 */
                    float w = power_heuristic(li.pdf, bp);
                    L = c3_add(L, c3_mul4(T, value, o_bsdf_eval(B, &r), ct, w));
                }
            }
        } else {
            o_light_rec li;
            c3 value = sample_light_direct(sc, it.p, o_next2d(s), &li);
            if (!c3_iszero(value)) {
                o_bsdf_rec r;
                r.wi = to_local(&it, li.to_light); r.wo = to_local(&it, v3_neg(ray.d));
                float ct = fabsf(r.wi.z);
                float bp = o_light_is_delta(sc, li.light) ? 0.f : o_bsdf_pdf(B, &r);   /* PathTracingMIS.cpp:136, VolPathTracing.cpp:222 */
                float w = power_heuristic(li.pdf, bp);
                L = c3_add(L, c3_mul4(T, value, o_bsdf_eval(B, &r), ct, w));
            }
        }
        /* BSDF sampling */
        o_bsdf_rec r;
        r.wi = to_local(&it, v3_neg(ray.d)); r.wo = mk3(0, 0, 0);
        r.sampled_type = O_BSDF_ALL; r.relative_eta = 1.f; r.pdf = -1.f;
        v2 u = o_next2d(s);
        c3 f = o_bsdf_sample(B, &r, u, s->rng.state);
        if (c3_iszero(f)) break;
        o_ray refl = o_ray_make(it.p, to_world(&it, r.wo), O_EPSILON, O_MAX_REAL);
        o_hit nx;
        int caught = -1, is_env = 0;
        c3 Le = cfill(0.f);
        int hit = o_intersect(sc, &refl, &nx, 0);
        if (hit) {
            int nl = prim_light(sc, nx.prim);
            if (nl >= 0) { caught = nl; Le = area_le(sc, nl, v3_neg(refl.d), nx.n); }
        } else {
            if (env < 0) return L;
            caught = env; is_env = 1;
            Le = o_env_le(sc, env, refl.d);
        }
        if (caught >= 0) {
            o_light_rec lr;
            lr.normal = hit ? nx.n : mk3(0, 0, 0);
            lr.point = hit ? nx.p : mk3(0, 0, 0);
            lr.to_light = refl.d;
            float pl = (r.sampled_type & O_BSDF_DELTA) ? 0.f : o_light_pdf(sc, caught, it.p, &lr);
            float w = power_heuristic(r.pdf, pl);
            L = c3_add(L, c3_muls(c3_mul(c3_mul(T, Le), f), w));
            if (is_env) return L;
        }
        T = c3_mul(T, f);
        eta *= r.relative_eta;
        if (depth >= rd->min_depth) {
            float stop = smin(0.95f, c3_lum(T) * eta * eta);
            if (o_next1d(s) < stop) T = c3_divs(T, stop);
            else return L;
        }
        it = nx;
        ray = refl;
        emission = 0;
        depth++;
    }
    return L;
}

/* VolPathTracing::evalTransmittanceFromSampledBSDF (VolPathTracing.cpp:369-424) */
static c3 eval_tr_sampled(const o_scene *sc, o_ray ray, o_sampler *s, int medium, o_hit *it,
                          int *was, int *new_medium)
{
    o_ray tr_ray = ray;
    c3 tr = cfill(1.f);
    int first = 1;
    *was = 0;
    for (;;) {
        *was = o_intersect(sc, &tr_ray, it, 0);
        if (medium >= 0) {
            o_ray mr = o_ray_make(tr_ray.o, tr_ray.d, first ? tr_ray.mint : 0.f, *was ? it->t : tr_ray.maxt);
            tr = c3_mul(tr, o_medium_transmittance(sc, medium, &mr, s));
        }
        if (*was && prim_bsdf(sc, it->prim) >= 0) return tr;
        first = 0;
        if (!*was || c3_iszero(tr)) return tr;
        if (c3_iszero(tr)) return tr;
        v3 np = v3_add(tr_ray.o, v3_smul(it->t, tr_ray.d));
        tr_ray = o_ray_make(np, tr_ray.d, O_EPSILON, tr_ray.maxt);
        if (hit_transition(sc, it)) { medium = hit_medium(sc, it, tr_ray.d); *new_medium = medium; }
    }
}

/* ---------------- VolPathTracing::li (VolPathTracing.cpp:25-367) ---------------- */
static c3 li_volpath(const o_scene *sc, const rt_render_desc *rd, o_sampler *s, o_ray ray)
{
    c3 L = cfill(0.f), T = cfill(1.f);
    float eta = 1.f;
    int depth = 0, emission = 1;
    int env = sc->d->env_light;
    o_hit it;
    memset(&it, 0, sizeof(it));
    it.t = O_MAX_REAL; it.prim = -1;
    int was = o_intersect(sc, &ray, &it, 0);
    int medium = sc->d->camera.medium;
    while (depth < rd->max_depth) {
        float t;
        c3 wm = cfill(0.f), em = cfill(0.f);
        int scattered = 0;
        if (medium >= 0) {
            o_ray mr = o_ray_make(ray.o, ray.d, ray.mint, it.t);
            scattered = o_medium_sample_distance(sc, medium, &mr, s, &t, &wm, &em);
        }
        if (scattered) {
            const rt_medium_desc *M = &sc->d->media[medium];
            L = c3_add(L, c3_mul(T, em));
            T = c3_mul(T, wm);
            it.p = v3_add(ray.o, v3_smul(t, ray.d));
            o_light_rec li;
            memset(&li, 0, sizeof(li));
            c3 value = sample_attenuated_light(sc, it.p, s, &li, medium);
            if (!c3_iszero(value)) {
                float pf = o_light_is_delta(sc, li.light) ? 0.f : o_phase_eval(M, li.to_light, v3_neg(ray.d));   /* VolPathTracing.cpp:86 */
                float w = power_heuristic(li.pdf, pf);
                float ev = o_phase_eval(M, li.to_light, v3_neg(ray.d));
                L = c3_add(L, c3_muls(c3_muls(c3_mul(T, value), ev), w));
            }
            v3 wo; float pfpdf;
            float pfw = o_phase_sample(M, v3_neg(ray.d), o_next2d(s), &wo, &pfpdf);
            ray = o_ray_make(it.p, wo, 0.f, ray.maxt);
            int newm = -1;
            c3 tr = eval_tr_sampled(sc, ray, s, medium, &it, &was, &newm);
            T = c3_muls(T, pfw);
            if (was) {
                int hl = prim_light(sc, it.prim);
                if (hl >= 0) {
                    c3 Le = area_le(sc, hl, v3_neg(ray.d), it.n);
                    float pl = o_light_pdf(sc, hl, it.p, &li);
                    float w = power_heuristic(pfpdf, pl);
                    L = c3_add(L, c3_muls(c3_mul(c3_mul(T, Le), tr), w));
                }
            }
        } else {
            if (medium >= 0) {
                L = c3_add(L, c3_mul(T, em));
                T = c3_mul(T, wm);
            }
            if (!was) {
                if (emission && env >= 0) L = c3_add(L, c3_mul(T, o_env_le(sc, env, ray.d)));
                return L;
            }
            int bsdf = prim_bsdf(sc, it.prim);
            if (bsdf < 0) {
                ray = o_ray_make(it.p, ray.d, O_EPSILON, O_MAX_REAL);
                if (hit_transition(sc, &it)) medium = hit_medium(sc, &it, ray.d);
                was = o_intersect(sc, &ray, &it, 0);
                continue;
            }
            rt_bsdf_desc Btex;
        const rt_bsdf_desc *B = o_bsdf_at(sc->d, &sc->d->bsdfs[bsdf], it.uv, &Btex);
            int hl = prim_light(sc, it.prim);
            if (emission && hl >= 0) L = c3_add(L, c3_mul(T, area_le(sc, hl, v3_neg(ray.d), it.n)));
            o_light_rec li;
            memset(&li, 0, sizeof(li));
            c3 value = sample_attenuated_light(sc, it.p, s, &li, medium);
            if (!c3_iszero(value)) {
                o_bsdf_rec r;
                r.wi = to_local(&it, li.to_light); r.wo = to_local(&it, v3_neg(ray.d));
                float ct = fabsf(r.wi.z);
                float bp = o_light_is_delta(sc, li.light) ? 0.f : o_bsdf_pdf(B, &r);   /* PathTracingMIS.cpp:136, VolPathTracing.cpp:222 */
                float w = power_heuristic(li.pdf, bp);
                L = c3_add(L, c3_mul4(T, value, o_bsdf_eval(B, &r), ct, w));
            }
            o_bsdf_rec r;
            r.wi = to_local(&it, v3_neg(ray.d)); r.wo = mk3(0, 0, 0);
            r.sampled_type = O_BSDF_ALL; r.relative_eta = 1.f; r.pdf = -1.f;
            v2 bu = o_next2d(s);
            c3 f = o_bsdf_sample(B, &r, bu, s->rng.state);
            if (c3_iszero(f)) break;
            ray = o_ray_make(it.p, to_world(&it, r.wo), O_EPSILON, O_MAX_REAL);
            if (hit_transition(sc, &it)) medium = hit_medium(sc, &it, ray.d);
            int caught = -1, is_env = 0;
            c3 Le = cfill(0.f);
            v3 pfrom = it.p;
            int newm = -1;
            c3 tr = eval_tr_sampled(sc, ray, s, medium, &it, &was, &newm);
            if (was) {
                int nl = prim_light(sc, it.prim);
                if (nl >= 0) { caught = nl; Le = area_le(sc, nl, v3_neg(ray.d), it.n); }
            } else if (newm < 0) {
                if (env >= 0) { caught = env; is_env = 1; Le = o_env_le(sc, env, ray.d); }
            }
            if (caught >= 0) {
                o_light_rec lr;
                lr.normal = it.n; lr.point = it.p; lr.to_light = ray.d;
                float pl = (r.sampled_type & O_BSDF_DELTA) ? 0.f : o_light_pdf(sc, caught, pfrom, &lr);
                float w = power_heuristic(r.pdf, pl);
                L = c3_add(L, c3_muls(c3_mul(c3_mul(c3_mul(T, Le), f), tr), w));
                if (is_env && medium < 0) return L;
            }
            T = c3_mul(T, f);
            eta *= r.relative_eta;
        }
        if (depth >= rd->min_depth) {
            float stop = smin(0.95f, c3_max(T) * eta * eta);
            if (o_next1d(s) < stop) T = c3_divs(T, stop);
            else return L;
        }
        was = o_intersect(sc, &ray, &it, 0);
        emission = 0;
        depth++;
    }
    return L;
}

/* ---------------- one path sample (SampleJob.cpp:46-65) ---------------- */
static c3 render_one(const o_scene *sc, const rt_render_desc *rd, int x, int y, int sample,
                     float *xx, float *yy)
{
    const rt_camera_desc *cam = &sc->d->camera;
    o_sampler s;
    o_sampler_seed_path(&s, rd->seed, (uint32_t)(y * cam->width + x), (uint32_t)sample);
    v2 j = o_next2d(&s);
    *xx = (float)x + j.x;
    *yy = (float)y + j.y;
    v2 lens = mk2(0.f, 0.f);
    if (cam->aperture_radius > 0.f) lens = o_next2d(&s);
    o_ray ray = o_camera_ray(cam, *xx, *yy, lens);
    if (rd->integrator == RT_INTEGRATOR_VOLPATH) return li_volpath(sc, rd, &s, ray);
    return li_path_mis(sc, rd, &s, ray);
}

/* ---------------- tile jobs ---------------- */
/* ReconstructionFilter::precompute (ReconstructionFilter.cpp:27-40) with the
 * Gaussian (GaussianFilter.cpp:28-36) and Mitchell-Netravali
 * (MitchellNetravaliFilter.cpp:28-52) profiles; the box is 1 */
static float o_gauss1(float a, float w, float v)
{
    float e1 = expf(-a * v * v), e2 = expf(-a * w * w);
    float d = e1 - e2;
    return d < 0.f ? 0.f : d;
}
static float o_mitchell1(float B, float C, float v)
{
    v = fabsf(2.f * v);
    if (v > 1.f)
        return ((((-B - 6 * C) * v * v * v + (6 * B + 30 * C) * v * v) + (-12 * B - 48 * C) * v + 8 * B) + 24 * C) *
               (1.f / 6.f);
    return ((12 - 9 * B - 6 * C) * v * v * v + (-18 + 12 * B + 6 * C) * v * v + (6 - 2 * B)) * (1.f / 6.f);
}
static void o_filter_table(const rt_camera_desc *c, float *t)
{
    float rx = c->filter_radius[0], ry = c->filter_radius[1];
    for (int x = 0; x < 32; x++)
        for (int y = 0; y < 32; y++) {
            float fx = x * rx / 32, fy = y * ry / 32;
            float v = 1.f;
            if (c->filter == RT_FILTER_GAUSSIAN)
                v = o_gauss1(c->filter_param[0], c->filter_param[1], fx) * o_gauss1(c->filter_param[0], c->filter_param[1], fy);
            else if (c->filter == RT_FILTER_MITCHELL)
                v = o_mitchell1(c->filter_param[0], c->filter_param[1], fx / rx) *
                    o_mitchell1(c->filter_param[0], c->filter_param[1], fy / ry);
            t[x + y * 32] = v;
        }
}

typedef struct {
    o_scene *sc;
    const rt_render_desc *rd;
    float *subs;          /* one tile screen per tile of the range, (bx + 2ovx) x (by + 2ovy) */
    int ntx, nty, ovx, ovy, sw, sh;
    int first, next, end;  /* tiles first + k * stride for k in [0, end - first) */
    int stride;
    float table[1024];
    pthread_mutex_t mu;
    int64_t nan_count;
} o_job;

/* Screen::addSample (Screen.cpp:44-83) into a tile screen of sw x sh pixels
 * whose pixel (0, 0) is image pixel (minx - ovx, miny - ovy) */
static void film_add(const o_job *J, float *sub, int sw, int sh, int minx, int miny, float xx, float yy, c3 v,
                     int64_t *nan)
{
    if (c3_isnan(v)) { (*nan)++; return; }
    const rt_camera_desc *cam = &J->sc->d->camera;
    float rx = cam->filter_radius[0], ry = cam->filter_radius[1];
    xx = xx - 0.5f - (float)(minx - J->ovx);
    yy = yy - 0.5f - (float)(miny - J->ovy);
    int sx = (int)ceilf(xx - rx), ex = (int)floorf(xx + rx);
    int sy = (int)ceilf(yy - ry), ey = (int)floorf(yy + ry);
    sx = imax(0, sx); ex = imin(sw - 1, ex);
    sy = imax(0, sy); ey = imin(sh - 1, ey);
    for (int x = sx; x <= ex; x++)
        for (int y = sy; y <= ey; y++) {
            /* ReconstructionFilter::operator() (ReconstructionFilter.h:54-63) */
            int ix = imin((int)((32 * fabsf((float)x - xx)) / rx), 31);
            int iy = imin((int)((32 * fabsf((float)y - yy)) / ry), 31);
            float w = J->table[ix + iy * 32];
            float *p = sub + 4 * ((size_t)y * sw + x);
            p[0] += v.r * w; p[1] += v.g * w; p[2] += v.b * w; p[3] += w;
        }
}

static void *job_worker(void *arg)
{
    o_job *J = (o_job *)arg;
    const rt_render_desc *rd = J->rd;
    const rt_camera_desc *cam = &J->sc->d->camera;
    int bx = rd->block_x > 0 ? rd->block_x : 32, by = rd->block_y > 0 ? rd->block_y : 32;
    int64_t nan = 0;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int k = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (k >= J->end) break;
        int t = J->first + (k - J->first) * J->stride;
        int ox = (t % J->ntx) * bx, oy = (t / J->ntx) * by;
        int ex = imin(cam->width, ox + bx), ey = imin(cam->height, oy + by);
        int tw = ex - ox, th = ey - oy;
        int sw = tw + 2 * J->ovx, sh = th + 2 * J->ovy;
        float *sub = J->subs + 4 * (size_t)J->sw * J->sh * (size_t)(k - J->first);
        memset(sub, 0, sizeof(float) * 4 * (size_t)sw * sh);
        for (int y = oy; y < ey; y++)
            for (int x = ox; x < ex; x++)
                for (int i = 0; i < rd->spp; i++) {
                    float xx, yy;
                    c3 L = render_one(J->sc, rd, x, y, rd->sample_begin + i, &xx, &yy);
                    film_add(J, sub, sw, sh, ox, oy, xx, yy, L, &nan);
                }
    }
    pthread_mutex_lock(&J->mu);
    J->nan_count += nan;
    pthread_mutex_unlock(&J->mu);
    return NULL;
}

/* Render tiles [tile0, tile1) of the job grid (all tiles when tile1 < 0)
 * and merge their screens in tile order (Screen::merge, Screen.cpp:136-157:
 * the order of a single-threaded run) into the full screen, which has an
 * overlap border of ceil(r - 0.5) pixels; `film` receives the full screen's
 * top-left width x height block, as the reference reads it back
 * (Screen.h:52, Screen.cpp:113-122).  Pixels no tile reaches stay zero. */
static int32_t render_tile_set(o_scene *sc, const rt_render_desc *rd, int32_t tile0, int32_t count,
                               int32_t stride, float *film, int32_t nthreads);

int32_t oracle_render_tiles(o_scene *sc, const rt_render_desc *rd, int32_t tile0, int32_t tile1,
                            float *film, int32_t nthreads)
{
    if (!sc || !rd || !film) return RT_ERR_INVALID;
    const rt_camera_desc *cam = &sc->d->camera;
    int bx = rd->block_x > 0 ? rd->block_x : 32, by = rd->block_y > 0 ? rd->block_y : 32;
    int ntiles = ((cam->width + bx - 1) / bx) * ((cam->height + by - 1) / by);
    int first = tile0 < 0 ? 0 : tile0;
    int end = (tile1 < 0 || tile1 > ntiles) ? ntiles : tile1;
    return render_tile_set(sc, rd, first, end > first ? end - first : 0, 1, film, nthreads);
}

/* Render `count` tiles tile0, tile0 + stride, ... of the job grid (a sample
 * spread over the frame), merged in tile order as oracle_render_tiles does */
int32_t oracle_render_tiles_strided(o_scene *sc, const rt_render_desc *rd, int32_t tile0, int32_t count,
                                    int32_t stride, float *film, int32_t nthreads)
{
    if (!sc || !rd || !film || tile0 < 0 || count < 0 || stride < 1) return RT_ERR_INVALID;
    const rt_camera_desc *cam = &sc->d->camera;
    int bx = rd->block_x > 0 ? rd->block_x : 32, by = rd->block_y > 0 ? rd->block_y : 32;
    int ntiles = ((cam->width + bx - 1) / bx) * ((cam->height + by - 1) / by);
    if (count > 0 && (int64_t)tile0 + (int64_t)(count - 1) * stride >= ntiles) return RT_ERR_INVALID;
    return render_tile_set(sc, rd, tile0, count, stride, film, nthreads);
}

static int32_t render_tile_set(o_scene *sc, const rt_render_desc *rd, int32_t tile0, int32_t count,
                               int32_t stride, float *film, int32_t nthreads)
{
    if (sc->strategy != rd->strategy || !sc->light_cdf.cdf) build_light_cdf(sc, rd->strategy);
    const rt_camera_desc *cam = &sc->d->camera;
    int bx = rd->block_x > 0 ? rd->block_x : 32, by = rd->block_y > 0 ? rd->block_y : 32;
    o_job J;
    J.sc = sc; J.rd = rd;
    J.ntx = (cam->width + bx - 1) / bx;
    J.nty = (cam->height + by - 1) / by;
    J.ovx = (int)ceilf(cam->filter_radius[0] - 0.5f);
    J.ovy = (int)ceilf(cam->filter_radius[1] - 0.5f);
    J.sw = bx + 2 * J.ovx;
    J.sh = by + 2 * J.ovy;
    J.first = J.next = tile0;
    J.end = tile0 + count;
    J.stride = stride;
    J.nan_count = 0;
    o_filter_table(cam, J.table);
    int nt = J.end - J.first;
    if (nt < 0) nt = 0;
    J.subs = (float *)malloc(sizeof(float) * 4 * (size_t)J.sw * J.sh * (size_t)(nt > 0 ? nt : 1));
    if (!J.subs) return RT_ERR_NOMEM;
    pthread_mutex_init(&J.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, job_worker, &J);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&J.mu);
    /* merge into the full screen (width + 2 ovx) x (height + 2 ovy) */
    int FW = cam->width + 2 * J.ovx, FH = cam->height + 2 * J.ovy;
    float *full = (float *)calloc(4 * (size_t)FW * FH, sizeof(float));
    if (!full) { free(J.subs); return RT_ERR_NOMEM; }
    for (int k = J.first; k < J.end; k++) {
        int t = J.first + (k - J.first) * J.stride;
        int ox = (t % J.ntx) * bx, oy = (t / J.ntx) * by;
        int tw = imin(cam->width, ox + bx) - ox, tht = imin(cam->height, oy + by) - oy;
        int sw = tw + 2 * J.ovx, sh = tht + 2 * J.ovy;
        const float *sub = J.subs + 4 * (size_t)J.sw * J.sh * (size_t)(k - J.first);
        for (int x = 0; x < sw; x++)
            for (int y = 0; y < sh; y++) {
                float *dst = full + 4 * ((size_t)(oy + y) * FW + (ox + x));
                const float *src = sub + 4 * ((size_t)y * sw + x);
                for (int k = 0; k < 4; k++) dst[k] += src[k];
            }
    }
    for (int y = 0; y < cam->height; y++)
        memcpy(film + 4 * (size_t)y * cam->width, full + 4 * (size_t)y * FW, sizeof(float) * 4 * (size_t)cam->width);
    free(full);
    free(J.subs);
    return RT_OK;
}

int32_t oracle_render(o_scene *sc, const rt_render_desc *rd, float *film, int32_t nthreads)
{
    return oracle_render_tiles(sc, rd, 0, -1, film, nthreads);
}

/* Radiance of individual path samples (pixel index, sample index) */
int32_t oracle_render_paths(o_scene *sc, const rt_render_desc *rd, const int32_t *pixels,
                            const int32_t *samples, int32_t n, float *rad)
{
    if (sc->strategy != rd->strategy || !sc->light_cdf.cdf) build_light_cdf(sc, rd->strategy);
    int W = sc->d->camera.width;
    for (int i = 0; i < n; i++) {
        float xx, yy;
        c3 L = render_one(sc, rd, pixels[i] % W, pixels[i] / W, samples[i], &xx, &yy);
        rad[3 * i] = L.r; rad[3 * i + 1] = L.g; rad[3 * i + 2] = L.b;
    }
    return RT_OK;
}

/* ---------------- test hooks ---------------- */
int32_t oracle_scene_info(const o_scene *sc, float bounds[6], int32_t *nodes)
{
    if (nodes) *nodes = o_bvh_node_count(sc->top);
    o_bvh_root_box(sc->top, bounds);
    return RT_OK;
}

int32_t oracle_trace(const o_scene *sc, const rt_ray *rays, int32_t n, int32_t anyhit, rt_hit *hits)
{
    for (int i = 0; i < n; i++) {
        o_ray r = o_ray_make(v3_from(rays[i].o), v3_from(rays[i].d), rays[i].mint, rays[i].maxt);
        o_hit h;
        int hit = o_intersect(sc, &r, &h, anyhit);
        hits[i].t = hit ? h.t : 0.f;
        hits[i].u = hit ? h.u : 0.f;
        hits[i].v = hit ? h.v : 0.f;
        hits[i].prim = hit ? h.prim : -1;
        if (hit && anyhit) { hits[i].prim = 0; hits[i].t = 0.f; hits[i].u = hits[i].v = 0.f; }
    }
    return RT_OK;
}

/* ImageTexture::eval of one texture at n texture coordinates (uv pairs);
 * out: n rgb triples.  Test hook. */
void oracle_tex_eval(const rt_texture_desc *t, const float *uv, int32_t n, float *out)
{
    for (int i = 0; i < n; i++) {
        c3 c = o_tex_eval(t, mk2(uv[2 * i], uv[2 * i + 1]));
        out[3 * i] = c.r; out[3 * i + 1] = c.g; out[3 * i + 2] = c.b;
    }
}

int32_t oracle_bsdf_query(const rt_bsdf_desc *b, int32_t op, const rt_bsdf_q *q, int32_t n,
                          rt_bsdf_r *r)
{
    for (int i = 0; i < n; i++) {
        o_bsdf_rec rec;
        rec.wi = v3_from(q[i].wi); rec.wo = v3_from(q[i].wo);
        rec.sampled_type = O_BSDF_ALL; rec.relative_eta = 1.f; rec.pdf = -1.f;
        memset(&r[i], 0, sizeof(r[i]));
        if (op == RT_BSDF_OP_EVAL) {
            c3 v = o_bsdf_eval(b, &rec);
            r[i].value[0] = v.r; r[i].value[1] = v.g; r[i].value[2] = v.b;
        } else if (op == RT_BSDF_OP_PDF) {
            r[i].pdf = o_bsdf_pdf(b, &rec);
        } else {
            rec.wo = mk3(0, 0, 0);
            union { float f; uint32_t u; } ux, uy;
            ux.f = q[i].u[0];
            uy.f = q[i].u[1];
            c3 v = o_bsdf_sample(b, &rec, mk2(q[i].u[0], q[i].u[1]), ((uint64_t)ux.u << 32) | uy.u);
            r[i].value[0] = v.r; r[i].value[1] = v.g; r[i].value[2] = v.b;
            r[i].pdf = rec.pdf;
            r[i].wo[0] = rec.wo.x; r[i].wo[1] = rec.wo.y; r[i].wo[2] = rec.wo.z;
            r[i].relative_eta = rec.relative_eta;
            r[i].sampled_type = rec.sampled_type;
        }
    }
    return RT_OK;
}

int32_t oracle_light_query(const o_scene *sc, int32_t light, const rt_light_q *q, int32_t n,
                           rt_light_r *r)
{
    for (int i = 0; i < n; i++) {
        o_light_rec li;
        memset(&li, 0, sizeof(li));
        v3 p = v3_from(q[i].p);
        o_light_sample(sc, light, p, mk2(q[i].u[0], q[i].u[1]), &li);
        memset(&r[i], 0, sizeof(r[i]));
        r[i].intensity[0] = li.intensity.r; r[i].intensity[1] = li.intensity.g; r[i].intensity[2] = li.intensity.b;
        r[i].pdf = li.pdf;
        r[i].to_light[0] = li.to_light.x; r[i].to_light[1] = li.to_light.y; r[i].to_light[2] = li.to_light.z;
        r[i].distance = li.distance;
        r[i].point[0] = li.point.x; r[i].point[1] = li.point.y; r[i].point[2] = li.point.z;
        r[i].normal[0] = li.normal.x; r[i].normal[1] = li.normal.y; r[i].normal[2] = li.normal.z;
        r[i].pdf_eval = o_light_pdf(sc, light, p, &li);
    }
    return RT_OK;
}

int32_t oracle_medium_query(const o_scene *sc, int32_t medium, int32_t op, const rt_medium_q *q, int32_t n,
                            rt_medium_r *r)
{
    if (medium < 0 || medium >= sc->d->n_media) return RT_ERR_INVALID;
    for (int i = 0; i < n; i++) {
        o_sampler s;
        o_sampler_seed_path(&s, q[i].seed, q[i].pixel, q[i].sample);
        o_ray ray = o_ray_make(v3_from(q[i].o), v3_from(q[i].d), q[i].mint, q[i].maxt);
        memset(&r[i], 0, sizeof(r[i]));
        c3 w;
        if (op == RT_MEDIUM_OP_SAMPLE) {
            float t = 0.f;
            c3 em;
            r[i].scattered = o_medium_sample_distance(sc, medium, &ray, &s, &t, &w, &em);
            r[i].t = t;
        } else {
            w = o_medium_transmittance(sc, medium, &ray, &s);
        }
        r[i].weight[0] = w.r; r[i].weight[1] = w.g; r[i].weight[2] = w.b;
    }
    return RT_OK;
}

void oracle_pcg_stream(uint64_t initstate, uint64_t initseq, int32_t n, uint32_t *out)
{
    o_pcg32 r;
    o_pcg_seed(&r, initstate, initseq);
    for (int i = 0; i < n; i++) out[i] = o_pcg_next(&r);
}

void oracle_camera_rays(const rt_scene_desc *d, const float *pxy, const float *lens, int32_t n, rt_ray *out)
{
    for (int i = 0; i < n; i++) {
        v2 l = lens ? mk2(lens[2 * i], lens[2 * i + 1]) : mk2(0.f, 0.f);
        o_ray r = o_camera_ray(&d->camera, pxy[2 * i], pxy[2 * i + 1], l);
        out[i].o[0] = r.o.x; out[i].o[1] = r.o.y; out[i].o[2] = r.o.z; out[i].mint = r.mint;
        out[i].d[0] = r.d.x; out[i].d[1] = r.d.y; out[i].d[2] = r.d.z; out[i].maxt = r.maxt;
    }
}

/* CDF test hooks mirroring core/CDF.h:14-81 */
void oracle_cdf_sample_reuse(const float *pdfs, int32_t n, const float *u, int32_t m,
                             int32_t *index, float *u_out, float *pdf_out, float *sum_out)
{
    o_cdf c;
    o_cdf_init(&c);
    for (int i = 0; i < n; i++) o_cdf_add(&c, pdfs[i]);
    *sum_out = c.sum;
    o_cdf_normalize(&c);
    for (int k = 0; k < m; k++) {
        float v = u[k], p;
        index[k] = o_cdf_sample_reuse_pdf(&c, &v, &p);
        u_out[k] = v;
        pdf_out[k] = p;
    }
    o_cdf_free(&c);
}

void oracle_cdf_sample(const float *pdfs, int32_t n, const float *u, int32_t m, int32_t *index, float *pdf_out)
{
    o_cdf c;
    o_cdf_init(&c);
    for (int i = 0; i < n; i++) o_cdf_add(&c, pdfs[i]);
    o_cdf_normalize(&c);
    for (int k = 0; k < m; k++) index[k] = o_cdf_sample_pdf(&c, u[k], &pdf_out[k]);
    o_cdf_free(&c);
}

void oracle_pcg_reals(uint64_t initstate, uint64_t initseq, int32_t n, float *out)
{
    o_pcg32 r;
    o_pcg_seed(&r, initstate, initseq);
    for (int i = 0; i < n; i++) out[i] = o_pcg_float(&r);
}
