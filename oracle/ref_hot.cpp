/*
 * C entry points over the reference renderer's own hot-path code
 * (RaytracerNew2/src: Triangle, Sphere, Mesh, MeshLight/AreaLight,
 * EnvironmentLight, Diffuse, RoughConductor, RoughDielectric,
 * SmoothLayeredBSDF, MicrofacetDistribution, Fresnel, Mapping,
 * HGPhaseFunction, Homogeneous, Heterogeneous + GridVolume), compiled in
 * place by oracle/build_oracle.py against the Eigen-subset shim in
 * oracle/ref_include.  Each entry point takes the same query records as the
 * CPU oracle's matching hook, so the two can be compared on identical inputs
 * (tests/golden/make_golden.py, tests/test_oracle_pins.py).
 * TEST INFRASTRUCTURE ONLY: nothing in the library links this.
 *
 * Objects are built directly from Parameters, as the reference's factories
 * would build them from a scene file.  ref_scene_create assembles a whole
 * reference Scene from an rt_scene_desc (the description the GPU path and
 * the CPU oracle take) the way MeshFactory / GeometricShapeFactory and the
 * scene loader do, and ref_render_paths runs the reference's own
 * integrator (PathTracingMIS::li or VolPathTracing::li) on per-path sample
 * streams, as SampleJob::run does.  Two pieces of the reference that read
 * files are fed from memory instead: ImageLoader::load (the environment map,
 * defined below) and the GridVolume's .vol file (written to a temporary file
 * in the reference's own format).
 */
#include "accelStruct/Bvh.h"
#include "bsdf/Diffuse.h"
#include "camera/NoriPerspective.h"
#include "core/Primitive.h"
#include "core/Scene.h"
#include "core/XMLLoader.h"
#include "integrator/PathTracingMIS.h"
#include "integrator/VolPathTracing.h"
#include "bsdf/MicrofacetDistribution.h"
#include "bsdf/RoughConductor.h"
#include "bsdf/RoughDielectric.h"
#include "bsdf/SmoothLayeredBSDF.h"
#include "core/Fresnel.h"
#include "core/Mapping.h"
#include "core/Parameters.h"
#include "core/Transform.h"
#include "geometricShape/Mesh.h"
#include "geometricShape/Sphere.h"
#include "geometricShape/Triangle.h"
#include "io/ImageLoader.h"
#include "light/AreaLight.h"
#include "light/EnvironmentLight.h"
#include "light/MeshLight.h"
#include "medium/HGPhaseFunction.h"
#include "medium/Heterogeneous.h"
#include "medium/Homogeneous.h"
#include "texture/ConstantTexture.h"
#include "tools/Rng.h"
#include "volume/GridVolume.h"

#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <unistd.h>

extern "C" {
#include "rtgpu.h"
}

namespace {

// ------------------------------------------------------------------ helpers
Point3d P3(const float *v) { return Point3d(v[0], v[1], v[2]); }
Vector3d V3(const float *v) { return Vector3d(v[0], v[1], v[2]); }
Color C3(const float *v) { return Color(v[0], v[1], v[2]); }
void put3(float *o, const Eigen::Matrix<real, 3, 1> &v) { o[0] = v.x(); o[1] = v.y(); o[2] = v.z(); }
void put3c(float *o, const Color &c) { o[0] = c(0); o[1] = c(1); o[2] = c(2); }

Transform::ptr xform(const float *m16)
{
    real v[16];
    for (int i = 0; i < 16; i++) v[i] = m16[i];
    return Transform::ptr(new Transform(v));
}

const char *dist_name(int d) { return d == RT_DIST_GGX ? "ggx" : d == RT_DIST_PHONG ? "phong" : "beckmann"; }

// The per-path sample stream of the GPU path and the CPU oracle: PCG32
// (the reference's own tools/Rng.h) seeded with
// (splitmix64((seed << 32) ^ pixel), sample index); a 2-D sample draws its
// x before its y.
class PathStreamSampler : public Sampler {
public:
    Rng rng;
    Point2d getNextSample2D() override
    {
        real a = rng.nextReal();
        real b = rng.nextReal();
        return Point2d(a, b);
    }
    real getNextSample1D() override { return rng.nextReal(); }
    Sampler::ptr clone() override { return Sampler::ptr(new PathStreamSampler()); }
    void seed(uint64_t s, uint64_t l) override { rng.seed(s, l); }
};

uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

BSDF::ptr make_bsdf(const rt_bsdf_desc *b)
{
    Parameters p;
    switch (b->type) {
    case RT_BSDF_DIFFUSE:
        p.addColor("albedo", C3(b->albedo));
        return BSDF::ptr(new Diffuse(p));
    case RT_BSDF_ROUGH_CONDUCTOR:
        p.addTexture("reflectanceTexture", Texture::ptr(new ConstantTexture(C3(b->reflectance))));
        p.addReal("alpha", b->alpha);
        p.addColor("eta", C3(b->eta));
        p.addColor("absorption", C3(b->k));
        p.addString("distribution", dist_name(b->distribution));
        return BSDF::ptr(new RoughConductor(p));
    case RT_BSDF_ROUGH_DIELECTRIC:
        p.addTexture("reflectanceTexture", Texture::ptr(new ConstantTexture(C3(b->reflectance))));
        p.addTexture("transmittedTexture", Texture::ptr(new ConstantTexture(C3(b->transmittance))));
        p.addReal("alpha", b->alpha);
        p.addReal("etaInt", b->eta_int);
        p.addReal("etaExt", b->eta_ext);
        p.addString("distribution", dist_name(b->distribution));
        return BSDF::ptr(new RoughDielectric(p));
    case RT_BSDF_SMOOTH_LAYERED: {
        Parameters base;
        base.addColor("albedo", C3(b->albedo));
        p.addReal("etaInt", b->eta_int);
        p.addReal("etaExt", b->eta_ext);
        p.addReal("thickness", b->thickness);
        p.addColor("absorbance", C3(b->absorbance));
        p.addBSDF("baseBSDF", BSDF::ptr(new Diffuse(base)));
        return BSDF::ptr(new SmoothLayeredBSDF(p));
    }
    default:
        return BSDF::ptr();
    }
}

// The environment map handed to EnvironmentLight's constructor through the
// ImageLoader stand-in below.
std::shared_ptr<Array2D<Color3>> g_next_image;

// EnvironmentLight with access to the two members Scene-based
// initialisation sets (EnvironmentLight::initialize reads the scene box).
class EnvLight : public EnvironmentLight {
public:
    explicit EnvLight(const Parameters &p) : EnvironmentLight(p) {}
    void set_sphere(const Point3d &c, real r)
    {
        myCenter = c;
        mySphereRadius = r;
    }
};

// The grid of a heterogeneous medium in the .vol layout the reference reads
// (GridVolume.cpp:22-59), in a temporary file; "" on failure.
std::string write_grid(const rt_medium_desc *m)
{
    char tmpl[] = "/tmp/rt_pin_grid_XXXXXX";
    int fd = mkstemp(tmpl);
    if (fd < 0) return "";
    FILE *f = fdopen(fd, "wb");
    const char hdr[4] = {'V', 'O', 'L', 3};
    int32_t type = 1, channels = 1;
    fwrite(hdr, 1, 4, f);
    fwrite(&type, 4, 1, f);
    fwrite(m->res, 4, 3, f);
    fwrite(&channels, 4, 1, f);
    fwrite(m->grid_min, 4, 3, f);
    fwrite(m->grid_max, 4, 3, f);
    const char skipped[4] = {0, 0, 0, 0};   // GridVolume.cpp:51-54 skips 4 bytes before the data
    fwrite(skipped, 1, 4, f);
    fwrite(m->density, 4, (size_t)m->res[0] * m->res[1] * m->res[2], f);
    fclose(f);
    return tmpl;
}

// Medium of an rt_medium_desc (its phase function: HG or isotropic).
Medium::ptr make_medium(const rt_medium_desc *m, std::string &grid_path)
{
    Parameters p;
    if (m->phase == RT_PHASE_HG) {
        Parameters hp;
        hp.addReal("g", m->g);
        p.addPhaseFunction("phaseFunction", PhaseFunction::ptr(new HGPhaseFunction(hp)));
    }
    if (m->type == RT_MEDIUM_HOMOGENEOUS) {
        p.addColor("sigmaA", C3(m->sigma_a));
        p.addColor("sigmaS", C3(m->sigma_s));
        p.addReal("scale", m->scale);
        return Medium::ptr(new Homogeneous(p));
    }
    grid_path = write_grid(m);
    if (grid_path.empty()) return Medium::ptr();
    Parameters vp;
    vp.addString("path", grid_path);
    p.addVolume("volume", Volume::ptr(new GridVolume(vp)));
    p.addColor("albedo", C3(m->albedo));
    p.addReal("scale", m->scale);
    p.addBool("centered", m->centered != 0);
    p.addTransform("toWorld", xform(m->to_world));
    return Medium::ptr(new Heterogeneous(p));
}

// NoriPerspective with the two matrices of an rt_camera_desc (the sample ->
// camera and camera -> world transforms its constructor and the scene
// loader would compute).
class PinCamera : public NoriPerspective {
public:
    PinCamera(const Parameters &p, const rt_camera_desc &c) : NoriPerspective(p)
    {
        real v[16];
        for (int i = 0; i < 16; i++) v[i] = c.sample_to_camera[i];
        mySampleToCamera = Transform(v);
        myWorldTransform = xform(c.camera_to_world);
    }
};

void fill_light(rt_light_r &r, Light &L, const Point3d &p, const LightSamplingInfos &li)
{
    memset(&r, 0, sizeof(r));
    put3c(r.intensity, li.intensity);
    r.pdf = li.pdf;
    put3(r.to_light, li.interToLight);
    r.distance = li.distance;
    put3(r.point, li.sampledPoint);
    put3(r.normal, li.normal);
    r.pdf_eval = L.pdf(p, li);
}

}  // namespace

// Scene-file loader stand-in: Scene::loadScene (core/Scene.cpp:63-70) names
// it, but the pins assemble scenes from descriptions (ref_scene_create) and
// never load a file.
namespace xml {
XMLLoader::XMLLoader() {}
XMLLoader::~XMLLoader() {}
bool XMLLoader::loadScene(Scene &, const std::string &) { return false; }
}  // namespace xml

// ImageLoader::load stand-in: the image the caller put in g_next_image.
std::shared_ptr<Array2D<Color3>> ImageLoader::load(const std::string &, Channel, real, real)
{
    return g_next_image;
}

extern "C" {

/* Triangle::intersection (Triangle.cpp:46-88) of each ray against one
 * triangle (9 floats), with the ray's own [mint, maxt]. */
int32_t ref_tri_query(const float *tri_v, const rt_ray *rays, int32_t n, rt_hit *hits)
{
    std::vector<Point3d, Eigen::aligned_allocator<Point3d>> v = {P3(tri_v), P3(tri_v + 3), P3(tri_v + 6)};
    Mesh::ptr mesh(new Mesh("pin", v, {}, {}, {0, 1, 2}));
    Triangle tri(Parameters(), mesh, 0);
    for (int i = 0; i < n; i++) {
        Ray ray(P3(rays[i].o), V3(rays[i].d), rays[i].mint, rays[i].maxt);
        real t = 0;
        Point2d uv;
        memset(&hits[i], 0, sizeof(hits[i]));
        hits[i].prim = -1;
        if (tri.intersection(ray, t, uv)) {
            hits[i].t = t;
            hits[i].u = uv.x();
            hits[i].v = uv.y();
            hits[i].prim = 0;
        }
    }
    return RT_OK;
}

/* BSDF::eval / pdf / sample in the local frame (bsdf/BSDF.h), queries and
 * results as rt_bsdf_query. */
int32_t ref_bsdf_query(const rt_bsdf_desc *b, int32_t op, const rt_bsdf_q *q, int32_t n, rt_bsdf_r *r)
{
    BSDF::ptr bsdf = make_bsdf(b);
    if (!bsdf) return RT_ERR_UNSUPPORTED;
    for (int i = 0; i < n; i++) {
        memset(&r[i], 0, sizeof(r[i]));
        if (op == RT_BSDF_OP_EVAL || op == RT_BSDF_OP_PDF) {
            BSDFSamplingInfos infos(V3(q[i].wi), V3(q[i].wo));
            if (op == RT_BSDF_OP_EVAL) put3c(r[i].value, bsdf->eval(infos));
            else r[i].pdf = bsdf->pdf(infos);
        } else {
            BSDFSamplingInfos infos(V3(q[i].wi));
            Color w = bsdf->sample(infos, Point2d(q[i].u[0], q[i].u[1]));
            put3c(r[i].value, w);
            r[i].pdf = infos.pdf;
            put3(r[i].wo, infos.wo);
            r[i].relative_eta = infos.relativeEta;
            r[i].sampled_type = (int32_t)infos.sampledType;
        }
    }
    return RT_OK;
}

/* core/Fresnel.h, same layout as oracle_fresnel_query: op 0 conductor
 * (eta, k, cosI) through the Color form with that value on every channel,
 * op 1 dielectric (etaI, etaT, cosI, cosT), op 2 estimateDielectric
 * (etaExt, etaInt, cosI) -> (reflectance, etaI, etaT, relativeEta, cosT). */
int32_t ref_fresnel_query(int32_t op, const float *in, int32_t n, float *out)
{
    for (int i = 0; i < n; i++) {
        const float *a = in + 4 * i;
        float *o = out + 5 * i;
        o[0] = o[1] = o[2] = o[3] = o[4] = 0.f;
        if (op == 0) {
            Color f = fresnel::fresnelConductor(Color(a[0]), Color(a[1]), a[2]);
            o[0] = f(0);
        } else if (op == 1) {
            o[0] = fresnel::fresnelDielectric(a[0], a[1], a[2], a[3]);
        } else if (op == 2) {
            real etaI = 0, etaT = 0, rel = 0, cosT = 0;
            Color f = fresnel::estimateDielectric(a[0], a[1], a[2], etaI, etaT, rel, cosT);
            o[0] = f(0); o[1] = etaI; o[2] = etaT; o[3] = rel; o[4] = cosT;
        } else {
            return RT_ERR_INVALID;
        }
    }
    return RT_OK;
}

/* core/Mapping.h warps, same layout as oracle_mapping_query. */
int32_t ref_mapping_query(int32_t op, const float *u, int32_t n, float *out)
{
    for (int i = 0; i < n; i++) {
        Point2d s(u[2 * i], u[2 * i + 1]);
        float *o = out + 3 * i;
        if (op == 0) {
            Point2d d = Mapping::squareToConcentricDisk(s);
            o[0] = d.x(); o[1] = d.y(); o[2] = 0.f;
        } else if (op == 1) {
            put3(o, Mapping::squareToCosineWeightedHemisphere(s));
        } else if (op == 2) {
            put3(o, Mapping::squareToTriangle(s));
        } else if (op == 3) {
            put3(o, Mapping::squareToUniformSphere(s));
        } else {
            return RT_ERR_INVALID;
        }
    }
    return RT_OK;
}

/* MicrofacetDistribution, same layout as oracle_microfacet_query. */
int32_t ref_microfacet_query(int32_t type, int32_t op, float alpha, const float *in, int32_t n, float *out)
{
    MicrofacetDistribution d(dist_name(type));
    for (int i = 0; i < n; i++) {
        const float *a = in + 9 * i;
        float *o = out + 3 * i;
        o[0] = o[1] = o[2] = 0.f;
        if (op == 0) o[0] = d.D(V3(a), alpha);
        else if (op == 1) o[0] = d.G(V3(a), V3(a + 3), V3(a + 6), alpha);
        else if (op == 2) put3(o, d.sampleNormal(Point2d(a[0], a[1]), alpha));
        else return RT_ERR_INVALID;
    }
    return RT_OK;
}

/* HGPhaseFunction, same layout as oracle_phase_query. */
int32_t ref_phase_query(float g, int32_t op, const float *in, int32_t n, float *out)
{
    Parameters p;
    p.addReal("g", g);
    HGPhaseFunction hg(p);
    for (int i = 0; i < n; i++) {
        const float *a = in + 6 * i;
        float *o = out + 5 * i;
        o[0] = o[1] = o[2] = o[3] = o[4] = 0.f;
        if (op == 0) {
            PhaseFunctionSamplingInfos infos(V3(a), V3(a + 3));
            o[0] = hg.eval(infos);
        } else if (op == 1) {
            PhaseFunctionSamplingInfos infos(V3(a));
            real w = hg.sample(infos, Point2d(a[3], a[4]));
            put3(o, infos.wo);
            o[3] = infos.pdf;
            o[4] = w;
        } else {
            return RT_ERR_INVALID;
        }
    }
    return RT_OK;
}

/* A mesh light (MeshLight over a Mesh: MeshLight.cpp:32-64, Mesh.cpp:38-93)
 * of nt triangles (indices into 3-float vertices) and radiance; samples
 * from each query point with its 2-D sample; pdf_eval = AreaLight::pdf. */
int32_t ref_mesh_light_query(const float *verts, int32_t nv, const int32_t *idx, int32_t nt, const float *radiance,
                             const rt_light_q *q, int32_t n, rt_light_r *r)
{
    std::vector<Point3d, Eigen::aligned_allocator<Point3d>> v;
    for (int i = 0; i < nv; i++) v.push_back(P3(verts + 3 * i));
    std::vector<int> ix(idx, idx + 3 * nt);
    Mesh::ptr mesh(new Mesh("light", v, {}, {}, ix));
    mesh->initialize();
    Parameters p;
    p.addColor("radiance", C3(radiance));
    MeshLight L(p);
    L.setShape(mesh);
    for (int i = 0; i < n; i++) {
        Point3d from = P3(q[i].p);
        LightSamplingInfos li = L.sample(from, Point2d(q[i].u[0], q[i].u[1]));
        fill_light(r[i], L, from, li);
    }
    return RT_OK;
}

/* An AreaLight on a Sphere (Sphere.cpp:146-201, AreaLight.cpp:23-61) of
 * `radius` placed by to_world (row-major 4x4). */
int32_t ref_sphere_light_query(const float *to_world, float radius, const float *radiance, const rt_light_q *q,
                               int32_t n, rt_light_r *r)
{
    Parameters sp;
    sp.addReal("radius", radius);
    sp.addTransform("toWorld", xform(to_world));
    std::shared_ptr<Sphere> sphere(new Sphere(sp));
    Parameters p;
    p.addColor("radiance", C3(radiance));
    AreaLight L(p);
    L.setShape(sphere);
    for (int i = 0; i < n; i++) {
        Point3d from = P3(q[i].p);
        LightSamplingInfos li = L.sample(from, Point2d(q[i].u[0], q[i].u[1]));
        fill_light(r[i], L, from, li);
    }
    return RT_OK;
}

/* EnvironmentLight (EnvironmentLight.cpp:8-275) over a width x height RGB
 * image (top row first), with its scale, toWorld and the bounding sphere
 * that Scene-based initialisation would set. */
int32_t ref_env_light_query(const float *rgb, int32_t w, int32_t h, float scale, const float *to_world,
                            const float *center, float sphere_radius, const rt_light_q *q, int32_t n, rt_light_r *r)
{
    auto img = std::make_shared<Array2D<Color3>>(w, h);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const float *c = rgb + 3 * ((size_t)y * w + x);
            (*img)(x, y) = Color3(c[0], c[1], c[2]);
        }
    g_next_image = img;
    Parameters p;
    p.addString("path", "in-memory");
    p.addReal("scale", scale);
    p.addTransform("toWorld", xform(to_world));
    EnvLight L(p);
    g_next_image.reset();
    L.set_sphere(P3(center), sphere_radius);
    for (int i = 0; i < n; i++) {
        Point3d from = P3(q[i].p);
        LightSamplingInfos li = L.sample(from, Point2d(q[i].u[0], q[i].u[1]));
        fill_light(r[i], L, from, li);
    }
    return RT_OK;
}

/* Homogeneous (Homogeneous.cpp:30-78) or Heterogeneous over a GridVolume
 * (Heterogeneous.cpp:281-546, GridVolume.cpp:7-149) described by an
 * rt_medium_desc, owned by the box [owner_min, owner_max]; sampleDistance
 * or transmittance of each ray segment drawing from the query's path stream.
 * Results as rt_medium_query. */
int32_t ref_medium_query(const rt_medium_desc *m, const float *owner_min, const float *owner_max, int32_t op,
                         const rt_medium_q *q, int32_t n, rt_medium_r *r)
{
    Parameters p;
    Medium::ptr med;
    std::string path;
    if (m->type == RT_MEDIUM_HOMOGENEOUS) {
        p.addColor("sigmaA", C3(m->sigma_a));
        p.addColor("sigmaS", C3(m->sigma_s));
        p.addReal("scale", m->scale);
        med = Medium::ptr(new Homogeneous(p));
    } else {
        path = write_grid(m);
        if (path.empty()) return RT_ERR_INVALID;
        Parameters vp;
        vp.addString("path", path);
        Volume::ptr vol(new GridVolume(vp));
        p.addVolume("volume", vol);
        p.addColor("albedo", C3(m->albedo));
        p.addReal("scale", m->scale);
        p.addBool("centered", m->centered != 0);
        p.addTransform("toWorld", xform(m->to_world));
        med = Medium::ptr(new Heterogeneous(p));
        med->setOwnerBBox(BoundingBox(P3(owner_min), P3(owner_max)));
    }
    std::shared_ptr<PathStreamSampler> s(new PathStreamSampler());
    for (int i = 0; i < n; i++) {
        s->seed(mix64((q[i].seed << 32) ^ (uint64_t)q[i].pixel), (uint64_t)q[i].sample);
        Ray ray(P3(q[i].o), V3(q[i].d), q[i].mint, q[i].maxt);
        memset(&r[i], 0, sizeof(r[i]));
        if (op == RT_MEDIUM_OP_SAMPLE) {
            real t = 0;
            Color w, em;
            r[i].scattered = med->sampleDistance(ray, s, t, w, em) ? 1 : 0;
            r[i].t = t;
            put3c(r[i].weight, w);
        } else {
            put3c(r[i].weight, med->transmittance(ray, s));
        }
    }
    if (!path.empty()) unlink(path.c_str());
    return RT_OK;
}

/* ------------------------------------------------------------------ whole renders */
struct ref_scene {
    Scene scene;
    std::shared_ptr<Camera> camera;
    std::vector<std::string> grids;
    int width = 0, height = 0;
    ~ref_scene()
    {
        for (auto &g : grids) unlink(g.c_str());
    }
};

/* A reference Scene assembled from an rt_scene_desc: BSDFs (Diffuse,
 * RoughConductor, RoughDielectric, SmoothLayeredBSDF), media, area, mesh and
 * environment lights in the description's order, one Mesh (Triangles under a
 * per-mesh Bvh, MeshFactory.h:39-139) per mesh, Spheres
 * (GeometricShapeFactory.h), the camera, and the integrator of `rd`; then
 * Scene::initialize (the reference's own BVH build, light and integrator
 * initialisation).  Returns null for a description with parts the pin build
 * does not assemble (textures, planes, point and spot lights, the smooth
 * BSDFs). */
ref_scene *ref_scene_create(const rt_scene_desc *d, const rt_render_desc *rd)
{
    if (d->n_textures > 0) return nullptr;
    std::unique_ptr<ref_scene> R(new ref_scene());
    std::vector<BSDF::ptr> bsdfs;
    for (int i = 0; i < d->n_bsdfs; i++) {
        if (d->bsdfs[i].two_sided) return nullptr;
        bsdfs.push_back(make_bsdf(&d->bsdfs[i]));
        if (!bsdfs.back()) return nullptr;
    }
    std::vector<Medium::ptr> media;
    for (int i = 0; i < d->n_media; i++) {
        std::string g;
        media.push_back(make_medium(&d->media[i], g));
        if (!g.empty()) R->grids.push_back(g);
        if (!media.back()) return nullptr;
    }
    std::vector<Light::ptr> lights;
    for (int i = 0; i < d->n_lights; i++) {
        const rt_light_desc &L = d->lights[i];
        Parameters p;
        if (L.type == RT_LIGHT_AREA) {
            p.addColor("radiance", C3(L.radiance));
            if (L.mesh_light) lights.push_back(Light::ptr(new MeshLight(p)));
            else lights.push_back(Light::ptr(new AreaLight(p)));
        } else if (L.type == RT_LIGHT_ENV) {
            auto img = std::make_shared<Array2D<Color3>>(L.env_width, L.env_height);
            for (int y = 0; y < L.env_height; y++)
                for (int x = 0; x < L.env_width; x++) {
                    const float *c = L.env_rgb + 3 * ((size_t)y * L.env_width + x);
                    (*img)(x, y) = Color3(c[0], c[1], c[2]);
                }
            g_next_image = img;
            p.addString("path", "in-memory");
            p.addReal("scale", L.env_scale);
            p.addTransform("toWorld", xform(L.env_to_world));
            lights.push_back(Light::ptr(new EnvironmentLight(p)));
            g_next_image.reset();
        } else {
            return nullptr;
        }
    }
    auto med = [&](int i) { return i >= 0 ? media[i] : Medium::ptr(); };
    auto bsdf = [&](int i) { return i >= 0 ? bsdfs[i] : BSDF::ptr(); };
    for (int m = 0; m < d->n_meshes; m++) {
        const rt_mesh_desc &M = d->meshes[m];
        if (M.n_tris == 0) continue;
        // the mesh's own vertex list, in order of first use
        std::vector<Point3d, Eigen::aligned_allocator<Point3d>> verts;
        std::vector<Normal3d, Eigen::aligned_allocator<Normal3d>> normals;
        std::vector<Point2d, Eigen::aligned_allocator<Point2d>> uvs;
        std::vector<int> idx;
        std::map<int, int> remap;
        bool has_n = d->normals != nullptr, has_uv = d->uvs != nullptr;
        for (int t = M.first_tri; t < M.first_tri + M.n_tris; t++)
            for (int k = 0; k < 3; k++) {
                int v = d->indices[3 * t + k];
                if (has_n && std::isnan(d->normals[3 * v])) has_n = false;
                if (has_uv && std::isnan(d->uvs[2 * v])) has_uv = false;
            }
        for (int t = M.first_tri; t < M.first_tri + M.n_tris; t++)
            for (int k = 0; k < 3; k++) {
                int v = d->indices[3 * t + k];
                auto it = remap.find(v);
                if (it == remap.end()) {
                    it = remap.emplace(v, (int)verts.size()).first;
                    verts.push_back(P3(d->vertices + 3 * v));
                    if (has_n) normals.push_back(Normal3d(d->normals[3 * v], d->normals[3 * v + 1], d->normals[3 * v + 2]));
                    if (has_uv) uvs.push_back(Point2d(d->uvs[2 * v], d->uvs[2 * v + 1]));
                }
                idx.push_back(it->second);
            }
        Mesh::ptr mesh(new Mesh("", verts, normals, uvs, idx));
        Light::ptr light = M.light >= 0 ? lights[M.light] : Light::ptr();
        if (light) ((AreaLight *)light.get())->setShape(mesh);
        std::vector<IPrimitive::ptr> tris;
        for (unsigned i = 0; i < idx.size(); i += 3) {
            GeometricShape::ptr shape(new Triangle(Parameters(), mesh, (int)i));
            IPrimitive::ptr prim(std::make_shared<SimplePrimitive>(shape, bsdf(M.bsdf), BSSRDF::ptr(), med(M.interior),
                                                                   med(M.exterior)));
            if (light) {
                mesh->addLightTriangle(shape);
                prim->addLight(light);
            }
            tris.push_back(prim);
        }
        mesh->initialize();
        IPrimitive::ptr prim = std::make_shared<Bvh>(tris);
        if (light) prim->addLight(light);
        if (M.interior >= 0) media[M.interior]->setOwnerBBox(prim->getWorldBoundingBox());
        if (M.exterior >= 0) media[M.exterior]->setOwnerBBox(prim->getWorldBoundingBox());
        R->scene.addPrimitive(prim);
    }
    for (int i = 0; i < d->n_spheres; i++) {
        const rt_sphere_desc &S = d->spheres[i];
        if (S.kind != RT_ANALYTIC_SPHERE) return nullptr;
        Parameters sp;
        sp.addReal("radius", S.radius);
        sp.addTransform("toWorld", xform(S.to_world));
        GeometricShape::ptr shape(new Sphere(sp));
        IPrimitive::ptr prim(std::make_shared<SimplePrimitive>(shape, bsdf(S.bsdf), BSSRDF::ptr(), med(S.interior),
                                                               med(S.exterior)));
        if (S.light >= 0) {
            ((AreaLight *)lights[S.light].get())->setShape(std::dynamic_pointer_cast<ISampledShape>(shape));
            prim->addLight(lights[S.light]);
        }
        if (S.interior >= 0) media[S.interior]->setOwnerBBox(prim->getWorldBoundingBox());
        if (S.exterior >= 0) media[S.exterior]->setOwnerBBox(prim->getWorldBoundingBox());
        R->scene.addPrimitive(prim);
    }
    for (int i = 0; i < d->n_lights; i++) {
        R->scene.addLight(lights[i]);
        if (d->lights[i].type == RT_LIGHT_ENV) R->scene.setEnvironementLight(lights[i]);
    }
    const rt_camera_desc &c = d->camera;
    if (c.filter != RT_FILTER_BOX || c.filter_radius[0] != 0.5f || c.filter_radius[1] != 0.5f) return nullptr;
    Parameters cp;
    cp.addInt("sizeX", c.width);
    cp.addInt("sizeY", c.height);
    cp.addReal("nearClip", c.near_clip);
    cp.addReal("farClip", c.far_clip);
    cp.addReal("apertureRadius", c.aperture_radius);
    cp.addReal("focalPlane", c.focal_plane);
    R->camera = std::make_shared<PinCamera>(cp, c);
    R->scene.setCamera(R->camera);
    if (c.medium >= 0) R->scene.setCameraMedium(media[c.medium]);
    Parameters ip;
    ip.addInt("maxDepth", rd->max_depth);
    ip.addInt("minDepth", rd->min_depth);
    ip.addString("strategy", rd->strategy == RT_STRATEGY_ONE_LIGHT_WEIGHTED ? "one_light_weighted"
                             : rd->strategy == RT_STRATEGY_ALL_LIGHTS     ? "all_lights"
                                                                           : "one_light_uniform");
    if (rd->integrator == RT_INTEGRATOR_VOLPATH) R->scene.addIntegrator(Integrator::ptr(new VolPathTracing(ip)));
    else R->scene.addIntegrator(Integrator::ptr(new PathTracingMIS(ip)));
    R->scene.initialize();
    R->width = c.width;
    R->height = c.height;
    return R.release();
}

void ref_scene_destroy(ref_scene *s) { delete s; }

/* Radiance of path samples (pixel y * width + x, sample index) as
 * SampleJob::run computes them (core/SampleJob.cpp:46-61): the sampler on
 * the path's stream, the 2-D pixel jitter, a lens sample when the camera has
 * an aperture, Camera::getRay, Integrator::li.  rad: 3 floats per path;
 * jit: the sample's film position (2 floats per path), may be null. */
int32_t ref_render_paths(ref_scene *s, uint64_t seed, const int32_t *pixels, const int32_t *samples, int32_t n,
                         float *rad, float *jit)
{
    std::shared_ptr<PathStreamSampler> sampler(new PathStreamSampler());
    Integrator *integ = s->scene.getIntegrator().get();
    for (int i = 0; i < n; i++) {
        int x = pixels[i] % s->width, y = pixels[i] / s->width;
        sampler->seed(mix64((seed << 32) ^ (uint64_t)(uint32_t)pixels[i]), (uint64_t)(uint32_t)samples[i]);
        Point2d sample = sampler->getNextSample2D();
        real xx = (real)x + sample.x();
        real yy = (real)y + sample.y();
        Point2d lens;
        if (s->camera->needsDoFSample()) lens = sampler->getNextSample2D();
        Ray ray = s->camera->getRay(xx, yy, lens);
        Color col = integ->li(s->scene, sampler, ray);
        rad[3 * i] = col(0);
        rad[3 * i + 1] = col(1);
        rad[3 * i + 2] = col(2);
        if (jit) {
            jit[2 * i] = xx;
            jit[2 * i + 1] = yy;
        }
    }
    return RT_OK;
}

}  // extern "C"
