/*
 * CPU oracle, part 1: math, sampler, BSDFs, lights, camera, media.
 * TEST INFRASTRUCTURE ONLY -- see oracle.h.  Reference paths are relative to
 * RaytracerNew2/src of Iscandel/Raytracer.
 */
#include <math.h>
#include "oracle.h"

#include <stdlib.h>
#include <string.h>

/* ===================== transforms ===================== */
/* core/Transform.h:90-99: explicit row sums, then divide by w if w != 0,1 */
v3 xf_point(const float *m, v3 p)
{
    v3 o;
    o.x = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
    o.y = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    o.z = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
    float w = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    if (w != 1.f && w != 0.f) o = v3_divs(o, w);
    return o;
}

/* core/Transform.h:118-125: topLeftCorner<3,3>() * v */
v3 xf_vector(const float *m, v3 v)
{
    return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z,
               m[4] * v.x + m[5] * v.y + m[6] * v.z,
               m[8] * v.x + m[9] * v.y + m[10] * v.z);
}

/* core/Transform.h:181-189: inverse.topLeftCorner<3,3>().transpose() * n */
v3 xf_normal(const float *inv, v3 n)
{
    return mk3(inv[0] * n.x + inv[4] * n.y + inv[8] * n.z,
               inv[1] * n.x + inv[5] * n.y + inv[9] * n.z,
               inv[2] * n.x + inv[6] * n.y + inv[10] * n.z);
}

/* ===================== PCG32 (tools/Rng.h:57-141) ===================== */
#define O_PCG_MULT 0x5851f42d4c957f2dULL

uint32_t o_pcg_next(o_pcg32 *r)
{
    uint64_t old = r->state;
    r->state = old * O_PCG_MULT + r->inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31));
}

void o_pcg_seed(o_pcg32 *r, uint64_t initstate, uint64_t initseq)
{
    r->state = 0u;
    r->inc = (initseq << 1u) | 1u;
    o_pcg_next(r);
    r->state += initstate;
    o_pcg_next(r);
}

/* Rng.h:132-141: mantissa trick, [1,2) - 1 */
float o_pcg_float(o_pcg32 *r)
{
    union { uint32_t u; float f; } x;
    x.u = (o_pcg_next(r) >> 9) | 0x3f800000u;
    return x.f - 1.0f;
}

/* splitmix64 finaliser used to derive per-path initial states */
uint64_t o_mix64(uint64_t x)
{
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27; x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

/* Path-stream sampler: one PCG32 stream per (pixel, sample); the draw
 * interface matches sampler/RandomSampler.cpp:28-38 with x drawn first. */
void o_sampler_seed_path(o_sampler *s, uint64_t seed, uint32_t pixel, uint32_t sample)
{
    o_pcg_seed(&s->rng, o_mix64((seed << 32) ^ (uint64_t)pixel), (uint64_t)sample);
}
float o_next1d(o_sampler *s) { return o_pcg_float(&s->rng); }
v2 o_next2d(o_sampler *s)
{
    float a = o_pcg_float(&s->rng);
    float b = o_pcg_float(&s->rng);
    return mk2(a, b);
}

/* ===================== CDF (core/CDF.h:14-81) ===================== */
void o_cdf_init(o_cdf *c)
{
    c->cap = 16;
    c->cdf = (float *)malloc(sizeof(float) * c->cap);
    c->cdf[0] = 0.f;
    c->n = 1;
    c->sum = 0.f;
    c->normalized = 0;
}
void o_cdf_free(o_cdf *c) { free(c->cdf); c->cdf = NULL; c->n = 0; }

void o_cdf_add(o_cdf *c, float pdf)
{
    c->sum += pdf;
    if (c->n == c->cap) { c->cap *= 2; c->cdf = (float *)realloc(c->cdf, sizeof(float) * c->cap); }
    c->cdf[c->n++] = c->sum;
}

void o_cdf_normalize(o_cdf *c)
{
    if (c->sum != 0.f) {
        float factor = 1.f / c->sum;
        for (int i = 1; i < c->n; i++) c->cdf[i] *= factor;
        c->cdf[c->n - 1] = 1.f;
        c->normalized = 1;
    }
}

/* lower_bound, then clamp to [0, size-2] (CDF.h:44-50) */
int o_cdf_sample(const o_cdf *c, float u)
{
    int lo = 0, hi = c->n;
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (c->cdf[mid] < u) lo = mid + 1; else hi = mid;
    }
    int index = imax(0, lo - 1);
    return imin(index, c->n - 2);
}
int o_cdf_sample_pdf(const o_cdf *c, float u, float *pdf)
{
    int i = o_cdf_sample(c, u);
    *pdf = c->cdf[i + 1] - c->cdf[i];
    return i;
}
int o_cdf_sample_reuse(const o_cdf *c, float *u)
{
    int i = o_cdf_sample(c, *u);
    *u = (*u - c->cdf[i]) / (c->cdf[i + 1] - c->cdf[i]);
    return i;
}
int o_cdf_sample_reuse_pdf(const o_cdf *c, float *u, float *pdf)
{
    int i = o_cdf_sample_reuse(c, u);
    *pdf = c->cdf[i + 1] - c->cdf[i];
    return i;
}

/* ===================== warps (core/Mapping.h) ===================== */
/* Mapping.h:110-140 */
static v2 o_square_to_concentric_disk(v2 s)
{
    const float r1 = 2 * s.x - 1.f;
    const float r2 = 2 * s.y - 1.f;
    float rx, ry;
    if (r1 > -r2 && r1 > r2) { rx = r1; ry = (O_PI * r2) / (4 * r1); }
    else if (r1 < r2 && r1 > -r2) { rx = r2; ry = (O_PI / 4.f) * (2 - r1 / r2); }
    else if (r1 < -r2 && r1 < r2) { rx = -r1; ry = (O_PI / 4.f) * (4 + r2 / r1); }
    else { rx = -r2; ry = (O_PI / 4.f) * (6 - r1 / r2); }
    return mk2(rx * cosf(ry), rx * sinf(ry));
}
/* Mapping.h:62-67 */
static v3 o_square_to_cosine_hemisphere(v2 s)
{
    v2 t = o_square_to_concentric_disk(s);
    float z = sqrtf(smax(0.f, 1.f - t.x * t.x - t.y * t.y));
    return mk3(t.x, t.y, z);
}
/* Mapping.h:94-105 */
static v3 o_square_to_triangle(v2 s)
{
    float sq = sqrtf(s.x);
    return mk3(1 - sq, (1 - s.y) * sq, s.y * sq);
}
/* Mapping.h:145-164 */
static v3 o_square_to_uniform_sphere(v2 s)
{
    float phi = 2.f * O_PI * s.x;
    float u = 2 * s.y - 1.f;
    float st = sqrtf(1.f - u * u);
    return v3_normalized(mk3(st * cosf(phi), st * sinf(phi), u));
}
/* Mapping.h:199-202 */
static float o_uniform_cone_pdf(float cos_theta) { return 1.f / (2 * O_PI * (1.f - cos_theta)); }

/* core/Geometry.h:163-190 */
static float o_spherical_phi(v3 v)
{
    float r = atan2f(v.x, -v.z);
    return r < 0.f ? r + 2 * (float)3.14159265358979323846 : r;
}
static float o_spherical_theta(v3 v) { return acosf(v.y); }
static v3 o_cartesian_from_spherical(float theta, float phi)
{
    float st = sinf(theta), ct = cosf(theta), cp = cosf(phi), sp = sinf(phi);
    return mk3(sp * st, ct, -cp * st);
}

/* alpha as the rough BSDFs read it: myAlphaTexture->eval(uv).average() */
static float o_alpha(const rt_bsdf_desc *b) { return b->tex_alpha == -1 ? b->alpha : c3_avg(cfill(b->alpha)); }

/* ===================== Fresnel (core/Fresnel.h) ===================== */
/* Fresnel.h:30-49 (per channel) */
static float o_fresnel_conductor1(float eta, float k, float cosI)
{
    float epa = eta * eta + k * k;
    float cos2 = cosI * cosI;
    float epac2 = epa * cos2;
    float two = 2 * eta * cosI;
    float rpar = (epac2 - two + 1) / (epac2 + two + 1);
    float rperp = (epa - two + cos2) / (epa + two + cos2);
    return (rpar * rpar + rperp * rperp) * 0.5f;
}
/* Fresnel.h:51-63 */
static float o_fresnel_dielectric(float etaI, float etaT, float cosI, float cosT)
{
    float tcI = etaT * cosI, icT = etaI * cosT, icI = etaI * cosI, tcT = etaT * cosT;
    float rpar = (tcI - icT) / (tcI + icT);
    float rperp = (icI - tcT) / (icI + tcT);
    return (rpar * rpar + rperp * rperp) * 0.5f;
}
/* Fresnel.h:83-114: returns the (grey) reflectance; all channels equal */
static float o_estimate_dielectric(float etaExt, float etaInt, float cosI,
                                   float *etaI, float *etaT, float *relEta, float *cosT)
{
    *etaI = etaExt; *etaT = etaInt;
    int entering = 1;
    float fr;
    if (cosI <= 0.f) { entering = 0; float t = *etaI; *etaI = *etaT; *etaT = t; }
    *relEta = *etaI / *etaT;
    float sinT = *relEta * sqrtf(smax(0.f, 1 - cosI * cosI));
    *cosT = sqrtf(smax(0.f, 1 - sinT * sinT));
    if (sinT >= 1.f) { *cosT = 0.f; fr = 1.f; }
    else {
        fr = o_fresnel_dielectric(*etaI, *etaT, fabsf(cosI), *cosT);
        if (entering) *cosT = -*cosT;
    }
    return fr;
}
/* .average() of the grey Color returned by estimateDielectric */
static float o_fr_avg(float f) { return c3_avg(cfill(f)); }

/* ===================== microfacet (bsdf/MicrofacetDistribution.cpp) ===================== */
static float o_cos2(v3 v) { return v.z * v.z; }
static float o_sin2(v3 v) { return 1.f - v.z * v.z; }
static float o_sin(v3 v) { float s2 = o_sin2(v); if (s2 < 0.f) return 0.f; return sqrtf(s2); }
static float o_tan2(v3 v) { float s2 = 1.f - v.z * v.z; if (s2 <= 0.f) return 0.f; return s2 / (v.z * v.z); }

/* MicrofacetDistribution.cpp:29-52 */
static v3 o_mf_sample_normal(int type, v2 s, float alpha)
{
    float theta;
    if (type == RT_DIST_BECKMANN) theta = atanf(sqrtf(-alpha * alpha * logf(1 - s.x)));
    else if (type == RT_DIST_GGX) theta = atanf(alpha * sqrtf(s.x) / sqrtf(1.f - s.x));
    else theta = acosf(powf(s.x, 1.f / (alpha + 2)));
    float phi = 2 * O_PI * s.y;
    return mk3(sinf(theta) * cosf(phi), sinf(theta) * sinf(phi), cosf(theta));
}
/* MicrofacetDistribution.cpp:54-87 */
static float o_mf_D(int type, v3 wh, float alpha)
{
    if (wh.z <= 0.f) return 0.f;
    if (type == RT_DIST_BECKMANN) {
        float c2 = wh.z * wh.z;
        float t2 = o_sin2(wh) / c2;
        float a2 = alpha * alpha;
        return expf(-t2 / a2) / (O_PI * a2 * c2 * c2);
    } else if (type == RT_DIST_GGX) {
        float a2 = alpha * alpha;
        float c2 = o_cos2(wh);
        float t2 = o_tan2(wh);
        float ss = a2 + t2;
        return a2 / (O_PI * c2 * c2 * ss * ss);
    }
    return ((alpha + 2.f) / (2 * O_PI)) * powf(wh.z, alpha);
}
/* MicrofacetDistribution.cpp:105-159 */
static float o_mf_G1(int type, v3 v, v3 m, float alpha)
{
    if (v3_dot(v, m) / v.z <= 0) return 0.f;
    if (type == RT_DIST_BECKMANN) {
        float tanv = o_sin(v) / v.z;
        if (tanv == 0.f) return 1.f;
        float b = fabsf(1.f / (alpha * tanv));
        if (b < 1.6f) return (3.535f * b + 2.181f * b * b) / (1 + 2.276f * b + 2.577f * b * b);
        return 1.f;
    } else if (type == RT_DIST_GGX) {
        float a2 = alpha * alpha;
        float t2 = o_tan2(v);
        return 2.f / (1 + sqrtf(1 + a2 * t2));
    }
    float tanv = o_sin(v) / v.z;
    float b = sqrtf(0.5f * alpha + 1) / tanv;
    if (b < 1.6f) return (3.535f * b + 2.181f * b * b) / (1 + 2.276f * b + 2.577f * b * b);
    return 1.f;
}
static float o_mf_G(int type, v3 wi, v3 wo, v3 wh, float alpha)
{
    return o_mf_G1(type, wi, wh, alpha) * o_mf_G1(type, wo, wh, alpha);
}
/* MicrofacetDistribution.h:43-46 */
static float o_adjusted_alpha(float alpha, float cosI)
{
    return (1.2f - 0.2f * sqrtf(fabsf(cosI))) * alpha;
}
static float o_sign(float v) { return v >= 0.f ? 1.f : -1.f; }

/* bsdf/BSDF.h reflect/refract helpers */
static v3 o_reflect_local(v3 v) { return mk3(-v.x, -v.y, v.z); }
static v3 o_reflect_n(v3 v, v3 n) { float d = 2 * v3_dot(v, n); return v3_sub(v3_smul(d, n), v); }
static v3 o_refract_local(v3 v, float cosT, float rel) { return mk3(rel * -v.x, rel * -v.y, cosT); }
static v3 o_refract_n(v3 v, v3 n, float rel, float cosT)
{
    float s = v3_dot(v, n) * rel + cosT;
    return v3_sub(v3_muls(n, s), v3_muls(v, rel));
}
/* RoughDielectric.h:32-35 (both branches negate) */
static v3 o_half_dir_transmitted(v3 wi, v3 wo, float etaI, float etaT)
{
    v3 s = v3_add(v3_smul(etaI, wi), v3_smul(etaT, wo));
    return v3_normalized(v3_smul(-1.f, s));
}

/* ===================== Diffuse (bsdf/Diffuse.cpp:28-106) ===================== */
static c3 o_diffuse_eval(const float *albedo, v3 wi, v3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return cfill(0.f);
    return c3_muls(c3_from(albedo), O_INV_PI);
}
static float o_diffuse_pdf(v3 wi, v3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return 0.f;
    return O_INV_PI * wo.z;
}
static c3 o_diffuse_sample(const float *albedo, o_bsdf_rec *r, v2 s)
{
    if (r->wi.z <= 0.f) return cfill(0.f);
    r->sampled_type = O_BSDF_DIFFUSE;
    r->wo = o_square_to_cosine_hemisphere(s);
    r->pdf = o_diffuse_pdf(r->wi, r->wo);
    return c3_from(albedo);
}

/* ===================== RoughConductor (bsdf/RoughConductor.cpp:77-145) ===================== */
static c3 o_rc_eval(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z, co = wo.z;
    if (ci <= 0.f || co <= 0.f) return cfill(0.f);
    v3 wh = v3_normalized(v3_add(wi, wo));
    float a = o_alpha(b);
    float D = o_mf_D(b->distribution, wh, a);
    float G = o_mf_G(b->distribution, wi, wo, wh, a);
    c3 F = mkc(o_fresnel_conductor1(b->eta[0], b->k[0], ci),
               o_fresnel_conductor1(b->eta[1], b->k[1], ci),
               o_fresnel_conductor1(b->eta[2], b->k[2], ci));
    float den = 4 * ci * co;
    c3 r = c3_muls(c3_from(b->reflectance), D);
    r = c3_mul(r, F);
    r = c3_muls(r, G);
    return c3_divs(r, den);
}
static float o_rc_pdf(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z, co = wo.z;
    if (ci <= 0.f || co <= 0.f) return 0.f;
    v3 wh = v3_normalized(v3_add(wi, wo));
    float ch = wh.z;
    float Jh = 1.f / (4 * fabsf(v3_dot(wh, wo)));
    float D = o_mf_D(b->distribution, wh, o_alpha(b));
    return D * ch * Jh;
}
static c3 o_rc_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s)
{
    if (r->wi.z <= 0.f) return cfill(0.f);
    r->sampled_type = O_BSDF_GLOSSY_REFLECTION;
    float alpha = o_adjusted_alpha(o_alpha(b), r->wi.z);
    v3 n = o_mf_sample_normal(b->distribution, s, alpha);
    r->wo = o_reflect_n(r->wi, n);
    float co = r->wo.z;
    if (co <= 0.f) return cfill(0.f);
    r->pdf = o_rc_pdf(b, r->wi, r->wo);
    if (r->pdf <= 0) return cfill(0.f);
    c3 e = o_rc_eval(b, r->wi, r->wo);
    return c3_divs(c3_muls(e, fabsf(co)), r->pdf);
}

/* ===================== RoughDielectric (bsdf/RoughDielectric.cpp:83-329) ===================== */
static c3 o_rd_eval_reflection(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z, co = wo.z;
    v3 wh = v3_normalized(v3_add(wi, wo));
    wh = v3_smul(o_sign(ci), wh);
    float alpha = o_alpha(b);
    float D = o_mf_D(b->distribution, wh, alpha);
    float eI, eT, rel, cT;
    float fr = o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(wi, wh), &eI, &eT, &rel, &cT);
    float G = o_mf_G(b->distribution, wi, wo, wh, alpha);
    float den = 4 * ci * co;
    c3 r = c3_muls(c3_from(b->reflectance), D);
    r = c3_muls(r, fr);
    r = c3_muls(r, G);
    return c3_divs(r, den);
}
static c3 o_rd_eval_refraction(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z, co = wo.z;
    float eI, eT, rel, cT;
    float fr = o_estimate_dielectric(b->eta_ext, b->eta_int, ci, &eI, &eT, &rel, &cT);
    v3 wt = o_half_dir_transmitted(wi, wo, eI, eT);
    float alpha = o_alpha(b);
    float left = v3_dot(wi, wt) * v3_dot(wo, wt) / (ci * co);
    float G = o_mf_G(b->distribution, wi, wo, wt, alpha);
    float D = o_mf_D(b->distribution, wt, alpha);
    float one_m_fr = (-1.f * fr) + 1.f;
    c3 term = c3_muls(c3_from(b->transmittance), left);
    term = c3_muls(term, eT);
    term = c3_muls(term, eT);
    term = c3_muls(term, one_m_fr);
    term = c3_muls(term, G);
    term = c3_muls(term, D);
    term = c3_muls(term, rel);
    term = c3_muls(term, rel);
    float denom = eI * v3_dot(wi, wt) + eT * v3_dot(wo, wt);
    return c3_divs(term, denom * denom);
}
static float o_rd_pdf_reflection(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z;
    float alpha = (1.2f - 0.2f * sqrtf(fabsf(ci))) * o_alpha(b);
    v3 wh = v3_normalized(v3_add(wi, wo));
    wh = v3_smul(o_sign(ci), wh);
    float ch = wh.z;
    float Jh = 1.f / (4 * v3_dot(wh, wo));
    return fabsf(o_mf_D(b->distribution, wh, alpha) * ch * Jh);
}
static float o_rd_pdf_refraction(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z;
    float eI, eT, rel, cT;
    o_estimate_dielectric(b->eta_ext, b->eta_int, ci, &eI, &eT, &rel, &cT);
    v3 wt = o_half_dir_transmitted(wi, wo, eI, eT);
    float cwt = wt.z;
    float alpha = (1.2f - 0.2f * sqrtf(fabsf(ci))) * o_alpha(b);
    float hd = eI * v3_dot(wi, wt) + eT * v3_dot(wo, wt);
    float Jh = (eT * eT * v3_dot(wo, wt)) / (hd * hd);
    return fabsf(o_mf_D(b->distribution, wt, alpha) * cwt * Jh);
}
static c3 o_rd_eval(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    if (wi.z * wo.z > 0) return o_rd_eval_reflection(b, wi, wo);
    return o_rd_eval_refraction(b, wi, wo);
}
static float o_rd_pdf(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z, co = wo.z;
    float eI, eT, rel, cT;
    if (ci * co > 0) {
        v3 wh = v3_normalized(v3_add(wi, wo));
        wh = v3_smul(o_sign(ci), wh);
        float fr = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(wi, wh), &eI, &eT, &rel, &cT));
        return o_rd_pdf_reflection(b, wi, wo) * fr;
    }
    float etaI = b->eta_ext, etaT = b->eta_int;
    if (ci < 0) { float t = etaI; etaI = etaT; etaT = t; }
    v3 wt = o_half_dir_transmitted(wi, wo, etaI, etaT);
    float fr = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(wi, wt), &eI, &eT, &rel, &cT));
    return o_rd_pdf_refraction(b, wi, wo) * (1.f - fr);
}
static c3 o_rd_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s)
{
    float ci = r->wi.z;
    float alpha = o_adjusted_alpha(o_alpha(b), ci);
    v3 n = o_mf_sample_normal(b->distribution, s, alpha);
    float eI, eT, rel, cT;
    float fr = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(r->wi, n), &eI, &eT, &rel, &cT));
    if (s.x <= fr) {
        r->sampled_type = O_BSDF_GLOSSY_REFLECTION;
        r->wo = o_reflect_n(r->wi, n);
        if (r->wi.z * r->wo.z <= 0) return cfill(0.f);
        r->pdf = o_rd_pdf_reflection(b, r->wi, r->wo) * fr;
        if (r->pdf <= 0) return cfill(0.f);
        v3 wh = v3_normalized(v3_add(r->wi, r->wo));
        wh = v3_smul(o_sign(ci), wh);
        float G = o_mf_G(b->distribution, r->wi, r->wo, wh, alpha);
        float v = 1.f * v3_dot(r->wi, n);
        v = v * G;
        return cfill(v / (ci * n.z));
    }
    r->sampled_type = O_BSDF_GLOSSY_TRANSMISSION;
    r->wo = v3_normalized(o_refract_n(r->wi, n, rel, cT));
    r->relative_eta = rel;
    float co = v3_dot(r->wo, n);
    if (r->wi.z * r->wo.z >= 0) return cfill(0.f);
    r->pdf = o_rd_pdf_refraction(b, r->wi, r->wo) * (1.f - fr);
    if (r->pdf <= 0) return cfill(0.f);
    c3 e = o_rd_eval_refraction(b, r->wi, r->wo);
    return c3_divs(c3_muls(e, fabsf(co)), r->pdf);
}

/* ===================== SmoothLayered (bsdf/SmoothLayeredBSDF.cpp:139-403) ===================== */
static c3 o_absorb(const rt_bsdf_desc *b, float wip, float wop)
{
    float s = 1.f / fabsf(wip) + 1.f / fabsf(wop);
    return mkc(expf((-b->absorbance[0] * b->thickness) * s),
               expf((-b->absorbance[1] * b->thickness) * s),
               expf((-b->absorbance[2] * b->thickness) * s));
}
static c3 o_sl_eval(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return cfill(0.f);
    float ci = wi.z;
    float eI, eT, rel, cT;
    float fr1 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, ci, &eI, &eT, &rel, &cT));
    float T12 = 1.f - fr1;
    if (fr1 == 1.f) return cfill(0.f);
    v3 rwi = v3_normalized(o_refract_local(wi, cT, rel));
    v3 rwo = v3_normalized(o_refract_local(wo, cT, rel));
    rwi = v3_neg(rwi);
    rwo = v3_neg(rwo);
    ci = v3_neg(rwo).z;
    float fr2 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, ci, &eI, &eT, &rel, &cT));
    if (fr2 == 1.f) return cfill(0.f);
    float T21 = 1.f - fr2;
    c3 f2 = o_diffuse_eval(b->albedo, rwi, rwo);
    c3 a = o_absorb(b, rwi.z, rwo.z);
    float G = 1.f;
    float t = (1.f - G) + T21 * G;
    float m = b->eta_ext / b->eta_int;
    c3 r = mkc(T12 * f2.r, T12 * f2.g, T12 * f2.b);
    r = c3_mul(r, a);
    r = c3_muls(r, t);
    r = c3_muls(r, m);
    r = c3_muls(r, m);
    r = c3_muls(r, wo.z);
    r = c3_divs(r, rwo.z);
    return c3_add(cfill(0.f), r);
}
static float o_sl_pdf(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float ci = wi.z;
    float eI, eT, rel, cT;
    float fr1 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, ci, &eI, &eT, &rel, &cT));
    if (fr1 == 1.f) return 0.f;
    v3 rwi = v3_normalized(o_refract_local(wi, cT, rel));
    v3 rwo = v3_normalized(o_refract_local(wo, cT, rel));
    rwi = v3_neg(rwi);
    rwo = v3_neg(rwo);
    float pbase = o_diffuse_pdf(rwi, rwo);
    float m = b->eta_ext / b->eta_int;
    return 0.f + pbase * (1.f - fr1) * m * m * wo.z / rwo.z;
}
static c3 o_sl_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s)
{
    if (r->wi.z <= 0.f) return cfill(0.f);
    float ci = r->wi.z;
    r->sampled_type = O_BSDF_GLOSSY_REFLECTION;
    float eI, eT, rel, cT;
    float fr1 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, ci, &eI, &eT, &rel, &cT));
    if (fr1 == 1.f) return cfill(0.f);
    if (s.x <= fr1) {
        r->wo = o_reflect_local(r->wi);
        r->pdf = fr1;
        r->sampled_type = O_BSDF_DELTA_REFLECTION;
        return cfill(1.f);
    }
    v3 rwi = v3_normalized(v3_neg(o_refract_local(r->wi, cT, rel)));
    r->sampled_type = O_BSDF_UNKNOWN;
    float T12 = 1.f - fr1;
    o_bsdf_rec base;
    base.wi = rwi; base.wo = mk3(0, 0, 0); base.sampled_type = O_BSDF_ALL;
    base.relative_eta = 1.f; base.pdf = -1.f;
    c3 f2 = o_diffuse_sample(b->albedo, &base, s);
    if (c3_iszero(f2)) return cfill(0.f);
    r->pdf = (1.f - fr1);
    if (r->pdf <= 0.f) return cfill(0.f);
    r->wo = v3_neg(base.wo);
    float wip = rwi.z;
    float wop = v3_neg(base.wo).z;
    c3 a = o_absorb(b, wip, wop);
    ci = r->wo.z;
    float fr2 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, ci, &eI, &eT, &rel, &cT));
    if (fr2 == 1.f) return cfill(0.f);
    float T21 = 1.f - fr2;
    r->wo = v3_normalized(o_refract_local(r->wo, cT, rel));
    float co = r->wo.z;
    c3 res = mkc(T12 * f2.r, T12 * f2.g, T12 * f2.b);
    res = c3_mul(res, a);
    res = c3_muls(res, T21);
    res = c3_add(cfill(0.f), res);
    res = c3_muls(res, fabsf(co));
    res = c3_divs(res, r->pdf);
    float m = b->eta_ext / b->eta_int;
    r->pdf *= base.pdf * m * m * r->wo.z / wop;
    return res;
}

/* ===================== LayeredBSDF (bsdf/LayeredBSDF.cpp:17-310) =====================
 * A rough dielectric coat (distribution / alpha = "alphaTop", read as a plain
 * real) over a RoughConductor base (distribution_base, alpha_base, eta, k,
 * reflectance).  sample() draws its coat normal from a member Rng of the BSDF
 * in the reference (LayeredBSDF.cpp:165); here from a side stream keyed by
 * aux_key, the path stream's state after the BSDF sample was drawn, so the
 * path stream itself advances as in the reference. */
static rt_bsdf_desc o_ly_base(const rt_bsdf_desc *b)
{
    rt_bsdf_desc c = *b;
    c.type = RT_BSDF_ROUGH_CONDUCTOR;
    c.distribution = b->distribution_base;
    c.alpha = b->alpha_base;
    return c;
}
/* LayeredBSDF::evalReflection (LayeredBSDF.cpp:150-163) */
static c3 o_ly_eval_reflection(const rt_bsdf_desc *b, v3 wi, v3 wo, float fr, float alpha)
{
    float ci = wi.z, co = wo.z;
    v3 wh = v3_normalized(v3_add(wi, wo));
    wh = v3_smul(o_sign(ci), wh);
    c3 term = c3_muls(cfill(fr), o_mf_D(b->distribution, wh, alpha));
    term = c3_muls(term, o_mf_G(b->distribution, wi, wo, wh, alpha));
    return c3_divs(term, 4 * ci * co);
}
/* LayeredBSDF::eval (LayeredBSDF.cpp:79-147) */
static c3 o_ly_eval(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    if (wi.z <= 0.f || wo.z <= 0.f) return cfill(0.f);
    v3 wh = v3_normalized(v3_add(wi, wo));
    float eI, eT, rel, cT;
    float fr1 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(wi, wh), &eI, &eT, &rel, &cT));
    float T12 = 1.f - fr1;
    float G = o_mf_G(b->distribution, wi, wo, wh, b->alpha);
    if (fr1 == 1.f) return cfill(0.f);
    v3 rwi = v3_normalized(o_refract_n(wi, wh, rel, cT));
    v3 rwo = v3_normalized(o_refract_n(wo, wh, rel, cT));
    c3 f1 = o_ly_eval_reflection(b, wi, wo, fr1, b->alpha);
    rwi = v3_smul(-1.f, rwi);
    rwo = v3_smul(-1.f, rwo);
    wh = v3_normalized(v3_add(rwi, rwo));
    float fr2 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(v3_smul(-1.f, rwo), wh),
                                               &eI, &eT, &rel, &cT));
    if (fr2 == 1.f) return cfill(0.f);
    float T21 = 1.f - fr2;
    rel = b->eta_ext / b->eta_int;
    rt_bsdf_desc base = o_ly_base(b);
    c3 f2 = c3_muls(o_rc_eval(&base, rwi, rwo), rel);
    f2 = c3_muls(f2, rel);
    f2 = c3_muls(f2, wo.z);
    f2 = c3_divs(f2, rwo.z);
    float sum = 1.f / fabsf(rwi.z) + 1.f / fabsf(rwo.z);
    c3 ab = c3_muls(c3_muls(c3_from(b->absorbance), -1.f), b->thickness);
    ab = c3_muls(ab, sum);
    c3 a = mkc(expf(ab.r), expf(ab.g), expf(ab.b));
    float t = (1.f - G) + T21 * G;
    c3 r = c3_muls(f2, T12);
    r = c3_mul(r, a);
    r = c3_muls(r, t);
    return c3_add(f1, r);
}
/* LayeredBSDF::pdf (LayeredBSDF.cpp:262-303) */
static float o_ly_pdf(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    v3 wh = v3_normalized(v3_add(wi, wo));
    float eI, eT, rel, cT;
    float fr1 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(wi, wh), &eI, &eT, &rel, &cT));
    if (fr1 == 1.f) return 0.f;
    v3 rwi = v3_normalized(o_refract_n(wi, wh, rel, cT));
    v3 rwo = v3_normalized(o_refract_n(wo, wh, rel, cT));
    float ch = wh.z;
    float Jh = 1.f / (4 * fabsf(v3_dot(wh, wo)));
    float D = o_mf_D(b->distribution, wh, b->alpha);
    float pd = fabsf(D * ch * Jh);
    rwi = v3_smul(-1.f, rwi);
    rwo = v3_smul(-1.f, rwo);
    rt_bsdf_desc base = o_ly_base(b);
    float pc = o_rc_pdf(&base, rwi, rwo);
    rel = b->eta_ext / b->eta_int;
    float q = pc * (1.f - fr1);
    q = q * rel;
    q = q * rel;
    q = q * wo.z;
    q = q / rwo.z;
    return pd * fr1 + q;
}
/* LayeredBSDF::sample (LayeredBSDF.cpp:165-260) */
static c3 o_ly_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s, uint64_t aux_key)
{
    if (r->wi.z <= 0.f) return cfill(0.f);
    float ci = r->wi.z;
    float alpha = (1.2f - 0.2f * sqrtf(fabsf(ci))) * b->alpha;
    o_pcg32 aux;
    o_pcg_seed(&aux, aux_key ^ 0x9E3779B97F4A7C15ull, 0x4C61796572656442ull);
    float n1 = o_pcg_float(&aux);
    float n2 = o_pcg_float(&aux);
    v3 normal = o_mf_sample_normal(b->distribution, mk2(n1, n2), alpha);
    float eI, eT, rel, cT;
    float fr1 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, v3_dot(r->wi, normal), &eI, &eT, &rel, &cT));
    if (fr1 == 1.f) return cfill(0.f);
    if (s.x <= fr1) {
        r->wo = o_reflect_n(r->wi, normal);
        r->pdf = o_ly_pdf(b, r->wi, r->wo);
        r->sampled_type = O_BSDF_GLOSSY_REFLECTION;
        c3 f1 = o_ly_eval_reflection(b, r->wi, r->wo, fr1, alpha);
        if (c3_iszero(f1)) return cfill(0.f);
    } else {
        r->sampled_type = O_BSDF_GLOSSY_REFLECTION;
        v3 rwi = v3_normalized(v3_smul(-1.f, o_refract_n(r->wi, normal, rel, cT)));
        o_bsdf_rec rr;
        memset(&rr, 0, sizeof(rr));
        rr.wi = rwi;
        rr.relative_eta = 1.f;
        rt_bsdf_desc base = o_ly_base(b);
        c3 f2 = o_rc_sample(&base, &rr, s);
        if (c3_iszero(f2)) return cfill(0.f);
        r->wo = v3_smul(-1.f, rr.wo);
        float fr2 = o_fr_avg(o_estimate_dielectric(b->eta_ext, b->eta_int, r->wo.z, &eI, &eT, &rel, &cT));
        if (fr2 == 1.f) return cfill(0.f);
        r->wo = v3_normalized(o_refract_n(r->wo, normal, rel, cT));
        r->pdf = o_ly_pdf(b, r->wi, r->wo);
        if (r->pdf == 0.f) return cfill(0.f);
    }
    if (r->pdf == 0.f) return cfill(0.f);
    float co = r->wo.z;
    return c3_divs(c3_muls(o_ly_eval(b, r->wi, r->wo), fabsf(co)), r->pdf);
}

/* ===================== textures (texture/ImageTexture.cpp) ===================== */
v2 o_sphere_uv(const rt_sphere_desc *sp, const o_ray *r, float t)
{
    v3 lo = xf_point(sp->to_object, r->o), ld = xf_vector(sp->to_object, r->d);
    if (sp->kind == RT_ANALYTIC_PLANE) {   /* Plane::intersection (Plane.cpp:75-76) */
        v3 q = v3_add(lo, v3_smul(t, ld));
        return mk2((q.x + 1) / 2.f, (q.y + 1) / 2.f);
    }
    v3 n = v3_normalized(v3_add(lo, v3_smul(t, ld)));
    return mk2(o_spherical_phi(n) / (2 * O_PI), o_spherical_theta(n) / O_PI);
}
static int o_tclamp(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }
static c3 o_texel(const rt_texture_desc *t, int x, int y)
{
    const float *p = t->rgb + 3 * ((size_t)y * t->width + x);
    return mkc(p[0], p[1], p[2]);
}
/* math::interp2 (core/BasicMath.h:73-90); a texture one texel wide (high)
 * keeps index 0 where the reference's empty clamp range gives -1 */
static c3 o_interp2(const rt_texture_desc *t, float x, float y)
{
    float advanceX = x - (float)(int)x, advanceY = y - (float)(int)y;
    int xMin = t->width < 2 ? 0 : o_tclamp((int)x, 0, t->width - 2);
    int yMin = t->height < 2 ? 0 : o_tclamp((int)y, 0, t->height - 2);
    int xMax = xMin + 1 < t->width ? xMin + 1 : xMin;
    xMax = o_tclamp(xMax, 0, t->width - 1);
    int yMax = yMin + 1 < t->height ? yMin + 1 : yMin;
    yMax = o_tclamp(yMax, 0, t->height - 1);
    c3 r = c3_muls(o_texel(t, xMin, yMin), (1 - advanceX) * (1 - advanceY));
    r = c3_add(r, c3_muls(o_texel(t, xMin, yMax), (1 - advanceX) * advanceY));
    r = c3_add(r, c3_muls(o_texel(t, xMax, yMin), advanceX * (1 - advanceY)));
    return c3_add(r, c3_muls(o_texel(t, xMax, yMax), advanceX * advanceY));
}
/* ImageTexture::eval (ImageTexture.cpp:28-70) */
c3 o_tex_eval(const rt_texture_desc *t, v2 uv)
{
    unsigned W = (unsigned)t->width, H = (unsigned)t->height;
    float x, y;
    if (!t->invert_y) y = uv.y * (float)H;
    else y = (float)(int)uv.y + ((uv.y >= 0.f ? 1 : -1) * 1.f - (uv.y - (float)(int)uv.y)) * (float)H;
    if (!t->invert_x) x = uv.x * ((float)W - 1.f);
    else x = (float)(int)uv.x + ((uv.x >= 0.f ? 1 : -1) * 1.f - (uv.x - (float)(int)uv.x)) * (float)W;
    x *= t->scale;
    y *= t->scale;
    if (x >= (float)W) x = (float)((unsigned)(int)x % W) + (x - (float)(int)x);
    else if (x < 0) x = (float)(W - (unsigned)abs((int)x) % W) + (x - (float)(int)x);
    if (y >= (float)H) y = (float)((unsigned)(int)y % H) + (y - (float)(int)y);
    else if (y < 0) y = (float)(H - (unsigned)abs((int)y) % H) + (y - (float)(int)y);
    return o_interp2(t, x, y);
}
/* The BSDF at a hit with its textures applied.  An applied alpha texture is
 * stored as its channel average with tex_alpha = -1 (a value the ABI does not
 * use), which o_alpha reads as is; a constant alpha is averaged as a
 * ConstantTexture's Color. */
const rt_bsdf_desc *o_bsdf_at(const rt_scene_desc *d, const rt_bsdf_desc *b, v2 uv, rt_bsdf_desc *tmp)
{
    if (!(b->tex_albedo | b->tex_reflectance | b->tex_transmittance | b->tex_alpha)) return b;
    *tmp = *b;
    if (b->tex_albedo) {
        c3 c = o_tex_eval(&d->textures[b->tex_albedo - 1], uv);
        tmp->albedo[0] = c.r; tmp->albedo[1] = c.g; tmp->albedo[2] = c.b;
    }
    if (b->tex_reflectance) {
        c3 c = o_tex_eval(&d->textures[b->tex_reflectance - 1], uv);
        tmp->reflectance[0] = c.r; tmp->reflectance[1] = c.g; tmp->reflectance[2] = c.b;
    }
    if (b->tex_transmittance) {
        c3 c = o_tex_eval(&d->textures[b->tex_transmittance - 1], uv);
        tmp->transmittance[0] = c.r; tmp->transmittance[1] = c.g; tmp->transmittance[2] = c.b;
    }
    if (b->tex_alpha) {
        tmp->alpha = c3_avg(o_tex_eval(&d->textures[b->tex_alpha - 1], uv));
        tmp->tex_alpha = -1;
    }
    return tmp;
}

/* ===================== smooth (delta) BSDFs ===================== */
/* Their eval and pdf are zero away from the discrete measure the reference
 * only attaches to sampled directions (Dielectric.cpp:23-26,85-91;
 * Conductor.cpp:26-37,55-64; Mirror.cpp:22-29,43-49). */
/* Dielectric::sample (Dielectric.cpp:28-82) */
static c3 o_dl_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s)
{
    float cosThetaI = r->wi.z;
    float etaI = b->eta_ext, etaT = b->eta_int;
    int isEntering = 1;
    float fr = 0.f;
    if (cosThetaI <= 0.f) {
        isEntering = 0;
        float t = etaI; etaI = etaT; etaT = t;
    }
    float relativeEta = etaI / etaT;
    float sinThetaT = relativeEta * sqrtf(fmaxf(0.f, 1 - cosThetaI * cosThetaI));
    float cosThetaT = sqrtf(fmaxf(0.f, 1 - sinThetaT * sinThetaT));
    if (sinThetaT >= 1.f) {
        fr = 1.f;
    } else {
        fr = o_fresnel_dielectric(etaI, etaT, fabsf(cosThetaI), cosThetaT);
        if (isEntering) cosThetaT = -cosThetaT;
    }
    r->relative_eta = relativeEta;
    if (s.x <= fr) {
        r->sampled_type = O_BSDF_DELTA_REFLECTION;
        r->wo = o_reflect_local(r->wi);
        r->pdf = fr;
        return c3_from(b->reflectance);
    }
    r->sampled_type = O_BSDF_DELTA_TRANSMISSION;
    r->wo = o_refract_local(r->wi, cosThetaT, relativeEta);
    r->pdf = 1 - fr;
    return c3_muls(c3_muls(c3_from(b->transmittance), relativeEta), relativeEta);
}
/* Conductor::sample (Conductor.cpp:39-53) */
static c3 o_cd_sample(const rt_bsdf_desc *b, o_bsdf_rec *r)
{
    if (r->wi.z <= 0.f) return cfill(0.f);
    r->sampled_type = O_BSDF_DELTA_REFLECTION;
    r->wo = o_reflect_local(r->wi);
    r->pdf = 1.f;
    float cosI = r->wi.z;
    c3 f = mkc(o_fresnel_conductor1(b->eta[0], b->k[0], cosI), o_fresnel_conductor1(b->eta[1], b->k[1], cosI),
               o_fresnel_conductor1(b->eta[2], b->k[2], cosI));
    return c3_mul(c3_from(b->reflectance), f);
}
/* Mirror::sample (Mirror.cpp:31-43) */
static c3 o_mr_sample(o_bsdf_rec *r)
{
    if (r->wi.z <= 0.f) return cfill(0.f);
    r->sampled_type = O_BSDF_DELTA_REFLECTION;
    r->wo = o_reflect_local(r->wi);
    r->pdf = 1.f;
    return cfill(1.f);
}

/* SheetDielectric::sample (SheetDielectric.cpp:122-174): reflect with the
 * sheet's inter-reflections fr + T^2 fr / (1 - fr^2), else straight through,
 * typed UNKNOWN (so MIS applies to what the straight ray finds) */
static c3 o_sd_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s)
{
    float cosThetaI = r->wi.z;
    float etaI = b->eta_ext, etaT = b->eta_int;
    float relativeEta = etaI / etaT;
    float sinThetaT = relativeEta * sqrtf(fmaxf(0.f, 1 - cosThetaI * cosThetaI));
    float cosThetaT = sqrtf(fmaxf(0.f, 1 - sinThetaT * sinThetaT));
    float fr = o_fresnel_dielectric(etaI, etaT, fabsf(cosThetaI), cosThetaT);
    float T = 1.f - fr;
    if (fr < 1.f) fr += T * T * fr / (1.f - fr * fr);
    r->relative_eta = 1.f;
    if (s.x <= fr) {
        r->sampled_type = O_BSDF_DELTA_REFLECTION;
        r->wo = o_reflect_local(r->wi);
        r->pdf = fr;
        return c3_from(b->reflectance);
    }
    r->sampled_type = O_BSDF_UNKNOWN;
    r->wo = v3_neg(r->wi);
    r->pdf = 1 - fr;
    return c3_from(b->transmittance);
}

/* ===================== Microfacet (bsdf/Microfacet.cpp:62-182) ===================== */
/* Microfacet::fresnel (:92-118): a grey dielectric Fresnel term */
static float o_nf_fresnel(float etaExt, float etaInt, float cosThetaI)
{
    float etaI = etaExt, etaT = etaInt;
    if (cosThetaI <= 0.f) { float t = etaI; etaI = etaT; etaT = t; }
    float relativeEta = etaI / etaT;
    float sinThetaT = relativeEta * sqrtf(fmaxf(0.f, 1 - cosThetaI * cosThetaI));
    float cosThetaT = sqrtf(fmaxf(0.f, 1 - sinThetaT * sinThetaT));
    if (sinThetaT >= 1.f) return 1.f;
    return o_fresnel_dielectric(etaI, etaT, fabsf(cosThetaI), cosThetaT);
}
/* Microfacet::eval (:76-90) */
static c3 o_nf_eval(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float cosThetaI = wi.z, cosThetaO = wo.z;
    if (cosThetaI <= 0.f || cosThetaO <= 0.f) return cfill(0.f);
    v3 wh = v3_normalized(v3_add(wi, wo));
    c3 diffusePart = c3_muls(c3_muls(c3_from(b->albedo), 1 - b->ks), O_INV_PI);
    float F = o_nf_fresnel(b->eta_ext, b->eta_int, v3_dot(wi, wh));
    c3 specularPart = cfill(b->ks * o_mf_D(b->distribution, wh, b->alpha) * F);
    specularPart = c3_muls(specularPart, o_mf_G(b->distribution, wi, wo, wh, b->alpha));
    specularPart = c3_divs(specularPart, 4 * cosThetaI * cosThetaO);
    return c3_add(diffusePart, specularPart);
}
/* Microfacet::pdf (:166-182) */
static float o_nf_pdf(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    float cosThetaI = wi.z, cosThetaO = wo.z;
    v3 wh = v3_normalized(v3_add(wi, wo));
    float cosThetaH = wh.z;
    float alpha = o_adjusted_alpha(b->alpha, cosThetaI);
    float Jh = 1.f / (4 * v3_dot(wh, wo));
    return b->ks * o_mf_D(b->distribution, wh, alpha) * cosThetaH * Jh + (1 - b->ks) * cosThetaO * O_INV_PI;
}
/* Microfacet::sample (:120-164): the normal is drawn first, then sample.x
 * picks the specular lobe (probability ks) or the cosine lobe */
static c3 o_nf_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s)
{
    if (r->wi.z <= 0.f) return cfill(0.f);
    float alpha = o_adjusted_alpha(b->alpha, r->wi.z);
    v3 normal = o_mf_sample_normal(b->distribution, s, alpha);
    if (s.x <= b->ks) {
        r->sampled_type = O_BSDF_GLOSSY_REFLECTION;
        r->wo = o_reflect_n(r->wi, normal);
    } else {
        r->sampled_type = O_BSDF_DIFFUSE;
        r->wo = o_square_to_cosine_hemisphere(s);
    }
    float cosThetaO = r->wo.z;
    r->pdf = o_nf_pdf(b, r->wi, r->wo);
    if (r->pdf == 0.f) return cfill(0.f);
    return c3_divs(c3_muls(o_nf_eval(b, r->wi, r->wo), fabsf(cosThetaO)), r->pdf);
}

/* ===================== BSDF dispatch ===================== */
static c3 o_bsdf_eval1(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    switch (b->type) {
    case RT_BSDF_DIFFUSE: return o_diffuse_eval(b->albedo, wi, wo);
    case RT_BSDF_ROUGH_CONDUCTOR: return o_rc_eval(b, wi, wo);
    case RT_BSDF_ROUGH_DIELECTRIC: return o_rd_eval(b, wi, wo);
    case RT_BSDF_SMOOTH_LAYERED: return o_sl_eval(b, wi, wo);
    case RT_BSDF_LAYERED: return o_ly_eval(b, wi, wo);
    case RT_BSDF_MICROFACET: return o_nf_eval(b, wi, wo);
    }
    return cfill(0.f);   /* Dielectric, Conductor, Mirror, SheetDielectric */
}
static float o_bsdf_pdf1(const rt_bsdf_desc *b, v3 wi, v3 wo)
{
    switch (b->type) {
    case RT_BSDF_DIFFUSE: return o_diffuse_pdf(wi, wo);
    case RT_BSDF_ROUGH_CONDUCTOR: return o_rc_pdf(b, wi, wo);
    case RT_BSDF_ROUGH_DIELECTRIC: return o_rd_pdf(b, wi, wo);
    case RT_BSDF_SMOOTH_LAYERED: return o_sl_pdf(b, wi, wo);
    case RT_BSDF_LAYERED: return o_ly_pdf(b, wi, wo);
    case RT_BSDF_MICROFACET: return o_nf_pdf(b, wi, wo);
    }
    return 0.f;
}
static c3 o_bsdf_sample1(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s, uint64_t aux_key)
{
    switch (b->type) {
    case RT_BSDF_DIFFUSE: return o_diffuse_sample(b->albedo, r, s);
    case RT_BSDF_ROUGH_CONDUCTOR: return o_rc_sample(b, r, s);
    case RT_BSDF_ROUGH_DIELECTRIC: return o_rd_sample(b, r, s);
    case RT_BSDF_SMOOTH_LAYERED: return o_sl_sample(b, r, s);
    case RT_BSDF_LAYERED: return o_ly_sample(b, r, s, aux_key);
    case RT_BSDF_DIELECTRIC: return o_dl_sample(b, r, s);
    case RT_BSDF_CONDUCTOR: return o_cd_sample(b, r);
    case RT_BSDF_MIRROR: return o_mr_sample(r);
    case RT_BSDF_SHEET_DIELECTRIC: return o_sd_sample(b, r, s);
    case RT_BSDF_MICROFACET: return o_nf_sample(b, r, s);
    }
    return cfill(0.f);
}
/* TwoSides (TwoSides.cpp:22-70), both sides the same BSDF: a query with
 * cosTheta(wi) <= 0 goes to the BSDF with wi.z and wo.z negated, and the
 * direction it samples comes back with wo.z negated. */
c3 o_bsdf_eval(const rt_bsdf_desc *b, const o_bsdf_rec *r)
{
    v3 wi = r->wi, wo = r->wo;
    if (b->two_sided && !(wi.z > 0.f)) { wi.z = -r->wi.z; wo.z = -r->wo.z; }
    return o_bsdf_eval1(b, wi, wo);
}
float o_bsdf_pdf(const rt_bsdf_desc *b, const o_bsdf_rec *r)
{
    v3 wi = r->wi, wo = r->wo;
    if (b->two_sided && !(wi.z > 0.f)) { wi.z = -r->wi.z; wo.z = -r->wo.z; }
    return o_bsdf_pdf1(b, wi, wo);
}
c3 o_bsdf_sample(const rt_bsdf_desc *b, o_bsdf_rec *r, v2 s, uint64_t aux_key)
{
    if (b->two_sided && !(r->wi.z > 0.f)) {
        r->wi.z = -r->wi.z;
        c3 res = o_bsdf_sample1(b, r, s, aux_key);
        r->wi.z = -r->wi.z;
        r->wo.z = -r->wo.z;
        return res;
    }
    return o_bsdf_sample1(b, r, s, aux_key);
}

/* ===================== shapes used by lights ===================== */
static void o_tri_verts(const rt_scene_desc *d, int tri, v3 *p0, v3 *p1, v3 *p2)
{
    const int32_t *ix = d->indices + 3 * (size_t)tri;
    *p0 = v3_from(d->vertices + 3 * (size_t)ix[0]);
    *p1 = v3_from(d->vertices + 3 * (size_t)ix[1]);
    *p2 = v3_from(d->vertices + 3 * (size_t)ix[2]);
}

/* Mesh::sample (geometricShape/Mesh.cpp:38-68) + Triangle::sample (Triangle.cpp:251-273) */
static void o_mesh_sample(const o_scene *sc, int mesh, v2 s, v3 *pt, v3 *n)
{
    const rt_scene_desc *d = sc->d;
    float ux = s.x;
    int index = o_cdf_sample_reuse(&sc->mesh[mesh].cdf, &ux);
    v2 s2 = mk2(ux, s.y);
    int tri = d->meshes[mesh].first_tri + index;
    v3 p0, p1, p2;
    o_tri_verts(d, tri, &p0, &p1, &p2);
    v3 b = o_square_to_triangle(s2);
    *pt = v3_add(v3_add(v3_muls(p0, b.x), v3_muls(p1, b.y)), v3_muls(p2, b.z));
    if (d->normals && !isnan(d->normals[3 * (size_t)d->indices[3 * (size_t)tri]])) {
        const int32_t *ix = d->indices + 3 * (size_t)tri;
        v3 n0 = v3_from(d->normals + 3 * (size_t)ix[0]);
        v3 n1 = v3_from(d->normals + 3 * (size_t)ix[1]);
        v3 n2 = v3_from(d->normals + 3 * (size_t)ix[2]);
        *n = v3_normalized(v3_add(v3_add(v3_smul(b.x, n0), v3_smul(b.y, n1)), v3_smul(b.z, n2)));
    } else {
        *n = v3_normalized(v3_cross(v3_sub(p1, p0), v3_sub(p2, p0)));
        *n = v3_normalized(*n);
    }
}
/* Mesh::pdf (Mesh.cpp:70-93) */
static float o_mesh_pdf(const o_scene *sc, int mesh, v3 p, v3 sampled, v3 n)
{
    v3 l = v3_sub(p, sampled);
    float dist = v3_norm(l);
    l = v3_normalized(l);
    float c = v3_dot(n, l);
    if (c > 0) return dist * dist / (sc->mesh[mesh].area * c);
    return 0.f;
}
/* Sphere::normal (Sphere.cpp:27-34) */
static v3 o_sphere_normal(const rt_sphere_desc *s, v3 p)
{
    v3 lp = xf_point(s->to_object, p);
    return v3_normalized(v3_sub(lp, mk3(0, 0, 0)));
}
static float o_sphere_area(const rt_sphere_desc *s) { return 4.f * O_PI * s->radius * s->radius * s->radius; }
/* Plane::Plane (geometricShape/Plane.cpp:7-18): the product of the lengths of
   the two transformed edges from the (-1,-1,0) corner */
float o_plane_area(const rt_sphere_desc *s)
{
    v3 mn = xf_point(s->to_world, mk3(-1.f, -1.f, 0.f));
    v3 s1 = v3_sub(xf_point(s->to_world, mk3(-1.f, 1.f, 0.f)), mn);
    v3 s2 = v3_sub(xf_point(s->to_world, mk3(1.f, -1.f, 0.f)), mn);
    return v3_norm(s1) * v3_norm(s2);
}
/* Plane::normal / getDifferentialGeometry (Plane.cpp:47-50,82-92): +z as a
   normal (inverse transpose), normalised */
v3 o_plane_normal(const rt_sphere_desc *s)
{
    return v3_normalized(xf_normal(s->to_object, mk3(0.f, 0.f, 1.f)));
}
/* Plane::sample (Plane.cpp:94-98) */
static void o_plane_sample(const rt_sphere_desc *s, v2 u, v3 *pt, v3 *n)
{
    *pt = xf_point(s->to_world, mk3(1 - 2 * u.x, 1 - 2 * u.y, 0.f));
    *n = o_plane_normal(s);
}
/* Sphere::sample (Sphere.cpp:146-173) */
static void o_sphere_sample(const rt_sphere_desc *s, v2 u, v3 *pt, v3 *n)
{
    float theta = 2.f * O_PI * u.x;
    float phi = acosf(2 * u.y - 1.f);
    float c = cosf(phi);
    float sq = sqrtf(1 - c * c);
    v3 p = mk3(sq * cosf(theta), sq * sinf(theta), c);
    p = v3_muls(p, s->radius);
    v3 nn = xf_normal(s->to_object, o_sphere_normal(s, p));
    *n = v3_normalized(nn);
    *pt = xf_point(s->to_world, p);
}
/* Sphere::pdf (Sphere.cpp:183-201) with the ISampledShape::pdf fallback (ISampledShape.cpp:17-40) */
float o_sphere_light_pdf(const rt_sphere_desc *s, v3 p, v3 sampled, v3 n)
{
    if (s->kind == RT_ANALYTIC_PLANE) {   /* ISampledShape::pdf (ISampledShape.cpp:17-40) */
        v3 l = v3_sub(p, sampled);
        float dist = v3_norm(l);
        l = v3_normalized(l);
        float c = v3_dot(n, l);
        if (c >= 0) return dist * dist / (o_plane_area(s) * c);
        return 0.f;
    }
    v3 center = xf_point(s->to_world, mk3(0.f, 0.f, 0.f));
    v3 itc = v3_sub(p, center);
    float sqd = v3_sqnorm(itc);
    if (v3_dot(n, itc) < 0.f) return 0.f;
    if (sqd - s->radius * s->radius < O_EPSILON) {
        v3 l = v3_sub(p, sampled);
        float dist = v3_norm(l);
        l = v3_normalized(l);
        float c = v3_dot(n, l);
        if (c >= 0) return dist * dist / (o_sphere_area(s) * c);
        return 0.f;
    }
    float st2 = s->radius * s->radius / sqd;
    float ct = sqrtf(smax(0.f, 1 - st2));
    return o_uniform_cone_pdf(ct);
}

/* ===================== environment light (light/EnvironmentLight.cpp) ===================== */
static c3 o_env_texel(const rt_light_desc *L, int x, int y)
{
    const float *p = L->env_rgb + 3 * ((size_t)y * L->env_width + x);
    return c3_muls(c3_from(p), L->env_scale);
}
/* EnvironmentLight.cpp:265-275 */
static void o_env_checkxy(const rt_light_desc *L, float *x, float *y)
{
    unsigned W = (unsigned)L->env_width, H = (unsigned)L->env_height;
    if (*x >= (float)W) *x = (float)((unsigned)(int)*x % W) + (*x - (float)(int)*x);
    else if (*x < 0) *x = (float)(W - (unsigned)abs((int)*x) % W) + (*x - (float)(int)*x);
    if (*y >= (float)H) *y = (float)((unsigned)(int)*y % H) + (*y - (float)(int)*y);
    else if (*y < 0) *y = (float)(H - (unsigned)abs((int)*y) % H) + (*y - (float)(int)*y);
}
static int o_clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
/* core/BasicMath.h:74-90 interp2 */
static c3 o_env_interp(const rt_light_desc *L, float x, float y)
{
    int W = L->env_width, H = L->env_height;
    float ax = x - (float)(int)x;
    float ay = y - (float)(int)y;
    int x0 = o_clampi((int)x, 0, W - 2);
    int y0 = o_clampi((int)y, 0, H - 2);
    int x1 = x0 + 1 < W ? x0 + 1 : x0; x1 = o_clampi(x1, 0, W - 1);
    int y1 = y0 + 1 < H ? y0 + 1 : y0; y1 = o_clampi(y1, 0, H - 1);
    const float *a00 = L->env_rgb + 3 * ((size_t)y0 * W + x0);
    const float *a01 = L->env_rgb + 3 * ((size_t)y1 * W + x0);
    const float *a10 = L->env_rgb + 3 * ((size_t)y0 * W + x1);
    const float *a11 = L->env_rgb + 3 * ((size_t)y1 * W + x1);
    float w00 = (1 - ax) * (1 - ay), w01 = (1 - ax) * ay, w10 = ax * (1 - ay), w11 = ax * ay;
    c3 r;
    r.r = ((w00 * a00[0] + w01 * a01[0]) + w10 * a10[0]) + w11 * a11[0];
    r.g = ((w00 * a00[1] + w01 * a01[1]) + w10 * a10[1]) + w11 * a11[1];
    r.b = ((w00 * a00[2] + w01 * a01[2]) + w10 * a10[2]) + w11 * a11[2];
    return r;
}
static void o_env_dir_to_xy(const rt_light_desc *L, v3 dir, float *fx, float *fy)
{
    *fx = (o_spherical_phi(dir) / (2 * O_PI)) * (float)L->env_width;
    *fy = (o_spherical_theta(dir) / O_PI) * (float)L->env_height;
    /* offsetU/offsetV are 0 for every scene this core accepts */
    *fx += 0.f * (float)L->env_width;
    *fy += 0.f * (float)L->env_height;
    o_env_checkxy(L, fx, fy);
}
/* EnvironmentLight.cpp:193-237 */
c3 o_env_le(const o_scene *sc, int light, v3 direction)
{
    const rt_light_desc *L = &sc->d->lights[light];
    v3 dir = v3_normalized(xf_vector(L->env_to_light, direction));
    float fx, fy;
    o_env_dir_to_xy(L, dir, &fx, &fy);
    return c3_muls(o_env_interp(L, fx, fy), L->env_scale);
}
static float o_env_norm(const o_scene *sc, int light, int row)
{
    const rt_light_desc *L = &sc->d->lights[light];
    const o_env_rt *E = &sc->env[light];
    float den = E->marginal.sum * (2 * O_PI / (float)L->env_width);
    den = den * (O_PI / (float)L->env_height);
    return E->weight[row] / den;
}
/* EnvironmentLight.cpp:85-146 */
static void o_env_sample(const o_scene *sc, int light, v3 p, v2 s, o_light_rec *out)
{
    const rt_light_desc *L = &sc->d->lights[light];
    const o_env_rt *E = &sc->env[light];
    float pr, pc;
    int row = o_cdf_sample_pdf(&E->marginal, s.x, &pr);
    int col = o_cdf_sample_pdf(&E->row[row], s.y, &pc);
    float rcol = (float)col + 0.f * (float)L->env_width;
    float rrow = (float)row + 0.f * (float)L->env_height;
    o_env_checkxy(L, &rcol, &rrow);
    row = (int)rrow;
    col = (int)rcol;
    float theta = O_PI * (float)row / (float)L->env_height;
    float phi = 2 * O_PI * (float)col / (float)L->env_width;
    float st = sinf(theta);
    v3 dir = o_cartesian_from_spherical(theta, phi);
    dir = xf_vector(L->env_to_world, dir);
    out->distance = E->sphere_radius;
    dir = v3_normalized(dir);
    out->to_light = dir;
    out->point = v3_add(p, v3_smul(E->sphere_radius, dir));
    out->normal = mk3(0, 0, 0);
    out->intensity = o_env_texel(L, o_clampi(col, 0, L->env_width - 1), o_clampi(row, 0, L->env_height - 1));
    float pdf = c3_lum(out->intensity) * E->weight[row];
    float den = E->marginal.sum * (2 * O_PI / (float)L->env_width);
    den = den * (O_PI / (float)L->env_height);
    pdf = pdf / den;
    pdf /= smax(fabsf(st), O_EPSILON);
    out->pdf = pdf;
}
/* EnvironmentLight.cpp:148-191 (sin of the pixel coordinate, as the reference does) */
static float o_env_pdf(const o_scene *sc, int light, v3 to_light)
{
    const rt_light_desc *L = &sc->d->lights[light];
    v3 dir = v3_normalized(xf_vector(L->env_to_light, to_light));
    float fx, fy;
    o_env_dir_to_xy(L, dir, &fx, &fy);
    float st = sinf(fy);
    /* a NaN direction (degenerate sample) must not index outside the table */
    float nf = o_env_norm(sc, light, isnan(fy) ? 0 : (int)fy);
    float lum = c3_lum(c3_muls(o_env_interp(L, fx, fy), L->env_scale));
    float pdf = lum * nf;
    pdf /= smax(fabsf(st), O_EPSILON);
    return pdf;
}

/* ===================== delta lights ===================== */
/* PointLight::sample (light/PointLight.cpp:20-33); SpotLight::sample and
   SpotLight::falloff (light/SpotLight.cpp:19-44).  The spot's cosine is the z
   of the inverse-toWorld image of -interToLight, without renormalising. */
static void o_delta_sample(const rt_light_desc *L, v3 p, o_light_rec *out)
{
    v3 pos = mk3(L->position[0], L->position[1], L->position[2]);
    out->to_light = v3_sub(pos, p);
    out->distance = v3_norm(out->to_light);
    float inv = 1.f / out->distance;
    out->to_light = v3_smul(inv, out->to_light);
    c3 I = c3_from(L->intensity);
    if (L->type == RT_LIGHT_SPOT) {
        v3 ld = xf_vector(L->spot_to_light, v3_neg(out->to_light));
        float ct = ld.z, f;
        if (ct < L->cos_total_width) f = 0.f;
        else if (ct > L->cos_falloff_start) f = 1.f;
        else {
            float dl = (ct - L->cos_total_width) / (L->cos_falloff_start - L->cos_total_width);
            f = (dl * dl) * (dl * dl);
        }
        I = c3_muls(I, f);
    }
    out->intensity = c3_muls(c3_muls(I, inv), inv);
    out->point = pos;
    out->normal = mk3(0.f, 0.f, 0.f);
    out->pdf = 1.f;
}

int o_light_is_delta(const o_scene *sc, int light)
{
    int t = sc->d->lights[light].type;
    return t == RT_LIGHT_POINT || t == RT_LIGHT_SPOT;
}

/* ===================== light dispatch ===================== */
void o_light_sample(const o_scene *sc, int light, v3 p, v2 s, o_light_rec *out)
{
    const rt_light_desc *L = &sc->d->lights[light];
    out->light = light;
    out->pdf = 0.f;
    out->distance = 0.f;
    out->intensity = cfill(0.f);
    if (L->type == RT_LIGHT_ENV) { o_env_sample(sc, light, p, s, out); return; }
    if (o_light_is_delta(sc, light)) { o_delta_sample(L, p, out); return; }
    v3 pt, n;
    if (L->shape_kind == RT_SHAPE_MESH) o_mesh_sample(sc, L->shape, s, &pt, &n);
    else if (sc->d->spheres[L->shape].kind == RT_ANALYTIC_PLANE) o_plane_sample(&sc->d->spheres[L->shape], s, &pt, &n);
    else o_sphere_sample(&sc->d->spheres[L->shape], s, &pt, &n);
    out->point = pt;
    out->normal = n;
    out->to_light = v3_sub(pt, p);
    out->distance = v3_norm(out->to_light);
    out->to_light = v3_divs(out->to_light, out->distance);
    float c = v3_dot(n, v3_neg(out->to_light));
    if (L->mesh_light && L->shape_kind == RT_SHAPE_MESH) {
        /* MeshLight.cpp:42-61 */
        if (c <= 0) { out->intensity = cfill(0.f); out->pdf = 0.f; }
        else {
            out->intensity = c3_from(L->radiance);
            out->pdf = out->distance * out->distance / (sc->mesh[L->shape].area * c);
        }
    } else {
        /* AreaLight.cpp:41-52 */
        if (c < 0) { out->intensity = cfill(0.f); out->pdf = 0.f; }
        else {
            out->intensity = c3_from(L->radiance);
            out->pdf = o_light_pdf(sc, light, p, out);
        }
    }
}

float o_light_pdf(const o_scene *sc, int light, v3 p, const o_light_rec *rec)
{
    const rt_light_desc *L = &sc->d->lights[light];
    if (o_light_is_delta(sc, light)) return 0.f;   /* PointLight / SpotLight::pdf */
    if (L->type == RT_LIGHT_ENV) return o_env_pdf(sc, light, rec->to_light);
    if (L->shape_kind == RT_SHAPE_MESH) return o_mesh_pdf(sc, L->shape, p, rec->point, rec->normal);
    return o_sphere_light_pdf(&sc->d->spheres[L->shape], p, rec->point, rec->normal);
}

/* ===================== camera (camera/NoriPerspective.cpp:80-118) ===================== */
o_ray o_ray_make(v3 o, v3 d, float mint, float maxt)
{
    o_ray r;
    r.o = o; r.d = d; r.mint = mint; r.maxt = maxt;
    r.inv = mk3(1.f / d.x, 1.f / d.y, 1.f / d.z);
    return r;
}

o_ray o_camera_ray(const rt_camera_desc *c, float px, float py, v2 lens)
{
    float invw = 1.f / (float)c->width, invh = 1.f / (float)c->height;
    v3 nearP = xf_point(c->sample_to_camera, mk3(px * invw, py * invh, 0.0f));
    v3 d = v3_normalized(nearP);
    float invZ = 1.0f / d.z;
    v3 o = mk3(0.f, 0.f, 0.f);
    if (c->aperture_radius > 0.f) {
        v2 s = o_square_to_concentric_disk(lens);
        s.x *= c->aperture_radius; s.y *= c->aperture_radius;
        o = mk3(s.x, s.y, 0.f);
        float tdist = c->focal_plane * invZ;
        v3 fp = v3_smul(tdist, d);
        d = v3_normalized(v3_sub(fp, o));
    }
    v3 wo = xf_point(c->camera_to_world, o);
    v3 wd = xf_vector(c->camera_to_world, d);
    return o_ray_make(wo, wd, c->near_clip * invZ, c->far_clip * invZ);
}

/* ===================== phase functions ===================== */
/* HGPhaseFunction.cpp:53-57 / IsotropicPhaseFunction */
float o_phase_eval(const rt_medium_desc *m, v3 wi, v3 wo)
{
    if (m->phase == RT_PHASE_ISOTROPIC) return O_INV_FOUR_PI;
    float g = m->g;
    float c = v3_dot(v3_neg(wi), wo);
    return O_INV_FOUR_PI * (1 - g * g) / powf(1 + g * g - 2 * g * c, 1.5f);
}
/* HGPhaseFunction.cpp:27-42 (world-frame direction, as the reference does) */
float o_phase_sample(const rt_medium_desc *m, v3 wi, v2 u, v3 *wo, float *pdf)
{
    if (m->phase == RT_PHASE_ISOTROPIC) {
        *wo = o_square_to_uniform_sphere(u);
        *pdf = O_INV_FOUR_PI;
        return 1.f;
    }
    float g = m->g;
    float ct;
    if (g < O_EPSILON) ct = 1.f - 2.f * u.x;
    else ct = (1 + g * g - ((1 - g * g) * (1 - g * g) / (1 - g + 2 * g * u.x))) / (2 * g);
    float theta = acosf(ct);
    float phi = 2 * O_PI * u.y;
    *wo = o_cartesian_from_spherical(theta, phi);
    *pdf = o_phase_eval(m, wi, *wo);
    return 1.f;
}

/* ===================== media ===================== */
/* Homogeneous (medium/Homogeneous.cpp:6-78) */
static c3 o_homog_sigma_t(const rt_medium_desc *m)
{
    c3 sa = c3_from(m->sigma_a), ss = c3_from(m->sigma_s);
    if (m->scale != 1.f) { sa = c3_muls(sa, m->scale); ss = c3_muls(ss, m->scale); }
    return c3_add(sa, ss);
}
static c3 o_homog_sigma_s(const rt_medium_desc *m)
{
    c3 ss = c3_from(m->sigma_s);
    if (m->scale != 1.f) ss = c3_muls(ss, m->scale);
    return ss;
}
static c3 o_homog_tr(const rt_medium_desc *m, float mint, float maxt)
{
    float t = maxt - mint;
    c3 st = o_homog_sigma_t(m);
    return mkc(expf(-st.r * t), expf(-st.g * t), expf(-st.b * t));
}

/* GridVolume::lookupSigmaT (volume/GridVolume.cpp:118-149) * scale */
static float o_grid_lookup(const rt_medium_desc *m, v3 pa)
{
    float px = pa.x * (float)m->res[0], py = pa.y * (float)m->res[1], pz = pa.z * (float)m->res[2];
    float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    if (ix < 0 || iy < 0 || iz < 0) return 0.0f * m->scale;
    if (ix >= m->res[0] - 1 || iy >= m->res[1] - 1 || iz >= m->res[2] - 1) return 0.0f * m->scale;
    size_t row = (size_t)m->res[0], slab = row * (size_t)m->res[1];
    size_t off = (size_t)iz * slab + (size_t)iy * row + (size_t)ix;
    const float *D = m->density;
    float d000 = D[off], d001 = D[off + 1], d010 = D[off + row], d011 = D[off + row + 1];
    float d100 = D[off + slab], d101 = D[off + slab + 1], d110 = D[off + slab + row], d111 = D[off + slab + row + 1];
    float w1x = px - fx, w1y = py - fy, w1z = pz - fz;
    float w0x = 1 - w1x, w0y = 1 - w1y, w0z = 1 - w1z;
    float v = ((d000 * w0x + d001 * w1x) * w0y + (d010 * w0x + d011 * w1x) * w1y) * w0z +
              ((d100 * w0x + d101 * w1x) * w0y + (d110 * w0x + d111 * w1x) * w1y) * w1z;
    return v * m->scale;
}

/* BoundingBox::intersection (core/BoundingBox.h:154-183) */
static int o_box_hit(const float *bmin, const float *bmax, const o_ray *r, float *nearT, float *farT)
{
    *nearT = -O_MAX_REAL;
    *farT = O_MAX_REAL;
    for (int i = 0; i < 3; i++) {
        float o = v3_get(r->o, i), dd = v3_get(r->d, i), inv = v3_get(r->inv, i);
        float mn = bmin[i], mx = bmax[i];
        if (dd == 0) {
            if (o < mn || o > mx) return 0;
        } else {
            float t1 = (mn - o) * inv;
            float t2 = (mx - o) * inv;
            if (t1 > t2) { float t = t1; t1 = t2; t2 = t; }
            *nearT = smax(t1, *nearT);
            *farT = smin(t2, *farT);
            if (!(*nearT <= *farT)) return 0;
        }
    }
    return (r->mint <= *farT && r->maxt >= *nearT);
}

static o_ray o_ray_xf(const float *m, const o_ray *r)
{
    return o_ray_make(xf_point(m, r->o), xf_vector(m, r->d), r->mint, r->maxt);
}

/* Heterogeneous::transmittance (medium/Heterogeneous.cpp:419-489) */
static c3 o_hetero_tr(const o_scene *sc, int mi, const o_ray *wr, o_sampler *s)
{
    const rt_medium_desc *m = &sc->d->media[mi];
    const o_medium_rt *M = &sc->med[mi];
    o_ray ray = o_ray_xf(M->world_to_array, wr);
    float tmax = ray.maxt - ray.mint;
    float tr = 1.f;
    float st = 0.f;
    int breaker = 0;
    float nearT, farT;
    static const float bmin[3] = {0.f, 0.f, 0.f}, bmax[3] = {1.f, 1.f, 1.f};
    if (!o_box_hit(bmin, bmax, &ray, &nearT, &farT)) return cfill(1.f);
    tmax = smin(tmax, farT);
    st = smax(nearT, ray.mint);
    for (;;) {
        st += -logf(1.f - o_next1d(s)) / M->max_sigma_t;
        v3 pa = v3_add(ray.o, v3_smul(st, ray.d));
        float proba = o_grid_lookup(m, pa);
        if (st >= tmax) return cfill(tr);
        tr *= 1 - smax(0.f, proba / M->max_sigma_t);
        const float threshold = .1f;
        if (tr < threshold) {
            float q = smax(.05f, 1 - tr);
            if (o_next1d(s) < q) return cfill(0.f);
            tr /= 1 - q;
        }
        if (breaker > 1024) return cfill(0.f);
        breaker++;
    }
}

/* Heterogeneous::sampleDistance (medium/Heterogeneous.cpp:491-546) */
static int o_hetero_sample(const o_scene *sc, int mi, const o_ray *wr, o_sampler *s,
                           float *t, c3 *weight, c3 *emission)
{
    const rt_medium_desc *m = &sc->d->media[mi];
    const o_medium_rt *M = &sc->med[mi];
    o_ray ray = o_ray_xf(M->world_to_array, wr);
    *t = ray.mint;
    float cur = 0.f;
    float nearT, farT;
    if (!o_box_hit(M->wbox_min, M->wbox_max, wr, &nearT, &farT)) {
        *weight = cfill(1.f); *emission = cfill(0.f); *t = ray.maxt;
        return 0;
    }
    float tmax = smin(ray.maxt, farT);
    for (;;) {
        *t += -logf(1.f - o_next1d(s)) / M->max_sigma_t;
        if (*t > tmax) {
            *weight = cfill(1.f); *emission = cfill(0.f); *t = tmax;
            return 0;
        }
        v3 pw = v3_add(wr->o, v3_smul(*t, wr->d));
        cur = o_grid_lookup(m, xf_point(M->world_to_array, pw));
        float proba = cur / M->max_sigma_t;
        if (o_next1d(s) < proba) break;
    }
    if (cur != 0.f) { *weight = c3_from(m->albedo); *emission = cfill(0.f); }
    else { *weight = cfill(0.f); *emission = cfill(0.f); }
    return 1;
}

int o_medium_sample_distance(const o_scene *sc, int mi, const o_ray *ray, o_sampler *s,
                             float *t, c3 *weight, c3 *emission)
{
    const rt_medium_desc *m = &sc->d->media[mi];
    if (m->type == RT_MEDIUM_HETEROGENEOUS) return o_hetero_sample(sc, mi, ray, s, t, weight, emission);
    /* Homogeneous::sampleDistance (Homogeneous.cpp:37-78) */
    c3 st = o_homog_sigma_t(m);
    int channel = (int)(o_next1d(s) * 3);
    float ext = channel == 0 ? st.r : (channel == 1 ? st.g : st.b);
    ext += O_EPSILON;
    *t = -logf(1.f - o_next1d(s)) / ext;
    if (*t > ray->maxt) {
        *t = ray->maxt;
        c3 e = mkc(expf(-st.r * *t), expf(-st.g * *t), expf(-st.b * *t));
        float pdf = c3_avg(e);
        *weight = c3_divs(o_homog_tr(m, ray->mint, ray->maxt), pdf);
        *emission = cfill(0.f);
        return 0;
    }
    c3 e = mkc(st.r * expf(-st.r * *t), st.g * expf(-st.g * *t), st.b * expf(-st.b * *t));
    float pdf = c3_avg(e);
    *t += ray->mint;
    *weight = c3_divs(c3_mul(o_homog_sigma_s(m), o_homog_tr(m, ray->mint, *t)), pdf);
    *emission = c3_div(cfill(0.f), st);
    return 1;
}

c3 o_medium_transmittance(const o_scene *sc, int mi, const o_ray *ray, o_sampler *s)
{
    const rt_medium_desc *m = &sc->d->media[mi];
    if (m->type == RT_MEDIUM_HETEROGENEOUS) return o_hetero_tr(sc, mi, ray, s);
    return o_homog_tr(m, ray->mint, ray->maxt);
}

/* ===================== pin hooks =====================
 * Direct entry points over the restated Fresnel, warp, microfacet and phase
 * functions, so that each can be compared one to one with the reference's
 * own function on the same inputs (tests/test_oracle_pins.py).  Test
 * infrastructure, like the rest of this file. */

/* op 0: fresnelConductor for one channel (Fresnel.h:30-49), in (eta, k, cosI);
 * op 1: fresnelDielectric (Fresnel.h:51-63), in (etaI, etaT, cosI, cosT);
 * op 2: estimateDielectric (Fresnel.h:83-114), in (etaExt, etaInt, cosI),
 *       out (reflectance, etaI, etaT, relativeEta, cosThetaT).
 * Each query reads 4 floats and writes 5. */
int32_t oracle_fresnel_query(int32_t op, const float *in, int32_t n, float *out)
{
    for (int i = 0; i < n; i++) {
        const float *a = in + 4 * i;
        float *o = out + 5 * i;
        o[0] = o[1] = o[2] = o[3] = o[4] = 0.f;
        if (op == 0) o[0] = o_fresnel_conductor1(a[0], a[1], a[2]);
        else if (op == 1) o[0] = o_fresnel_dielectric(a[0], a[1], a[2], a[3]);
        else if (op == 2) {
            float f = o_estimate_dielectric(a[0], a[1], a[2], &o[1], &o[2], &o[3], &o[4]);
            o[0] = f;
        } else return RT_ERR_INVALID;
    }
    return RT_OK;
}

/* Warps of core/Mapping.h for 2-D samples u (2 floats each), 3 floats out:
 * op 0 squareToConcentricDisk (x, y, 0), 1 squareToCosineWeightedHemisphere,
 * 2 squareToTriangle (barycentrics), 3 squareToUniformSphere. */
int32_t oracle_mapping_query(int32_t op, const float *u, int32_t n, float *out)
{
    for (int i = 0; i < n; i++) {
        v2 s = mk2(u[2 * i], u[2 * i + 1]);
        v3 r;
        if (op == 0) { v2 d = o_square_to_concentric_disk(s); r = mk3(d.x, d.y, 0.f); }
        else if (op == 1) r = o_square_to_cosine_hemisphere(s);
        else if (op == 2) r = o_square_to_triangle(s);
        else if (op == 3) r = o_square_to_uniform_sphere(s);
        else return RT_ERR_INVALID;
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
    return RT_OK;
}

/* MicrofacetDistribution (bsdf/MicrofacetDistribution.cpp) of `type` at
 * `alpha`, 9 floats in and 3 out per query: op 0 D(wh) (in wh), op 1
 * G(wi, wo, wh) (in wi, wo, wh), op 2 sampleNormal(u) (in u). */
int32_t oracle_microfacet_query(int32_t type, int32_t op, float alpha, const float *in, int32_t n, float *out)
{
    for (int i = 0; i < n; i++) {
        const float *a = in + 9 * i;
        float *o = out + 3 * i;
        o[0] = o[1] = o[2] = 0.f;
        if (op == 0) o[0] = o_mf_D(type, mk3(a[0], a[1], a[2]), alpha);
        else if (op == 1) o[0] = o_mf_G(type, mk3(a[0], a[1], a[2]), mk3(a[3], a[4], a[5]), mk3(a[6], a[7], a[8]), alpha);
        else if (op == 2) {
            v3 m = o_mf_sample_normal(type, mk2(a[0], a[1]), alpha);
            o[0] = m.x; o[1] = m.y; o[2] = m.z;
        } else return RT_ERR_INVALID;
    }
    return RT_OK;
}

/* Henyey-Greenstein phase function (medium/HGPhaseFunction.cpp) with
 * asymmetry g, 6 floats in and 5 out per query: op 0 eval (in wi, wo; out
 * value), op 1 sample (in wi, u; out wo, pdf, weight). */
int32_t oracle_phase_query(float g, int32_t op, const float *in, int32_t n, float *out)
{
    rt_medium_desc m;
    memset(&m, 0, sizeof(m));
    m.phase = RT_PHASE_HG;
    m.g = g;
    for (int i = 0; i < n; i++) {
        const float *a = in + 6 * i;
        float *o = out + 5 * i;
        o[0] = o[1] = o[2] = o[3] = o[4] = 0.f;
        v3 wi = mk3(a[0], a[1], a[2]);
        if (op == 0) o[0] = o_phase_eval(&m, wi, mk3(a[3], a[4], a[5]));
        else if (op == 1) {
            v3 wo;
            float pdf;
            float w = o_phase_sample(&m, wi, mk2(a[3], a[4]), &wo, &pdf);
            o[0] = wo.x; o[1] = wo.y; o[2] = wo.z; o[3] = pdf; o[4] = w;
        } else return RT_ERR_INVALID;
    }
    return RT_OK;
}
