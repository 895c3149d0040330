/*
 * CPU oracle, part 2: the reference's binary SAH BVH and ray casting.
 * TEST INFRASTRUCTURE ONLY -- see oracle.h.
 *
 * Restates accelStruct/Bvh.cpp (build 51-79, sweep SAH 83-246, binned SAH
 * 611-771, flatten 587-607, traversal 392-481), the two-level arrangement of
 * factory/MeshFactory.h:123 + core/Scene.cpp:117, Triangle::intersection
 * (geometricShape/Triangle.cpp:46-88), Triangle::getDifferentialGeometry
 * (Triangle.cpp:130-215), Sphere::intersection/getDifferentialGeometry
 * (geometricShape/Sphere.cpp:38-139) and DifferentialGeometry::coordinateSystem
 * (core/DifferentialGeometry.h:36-50).
 */
#include <math.h>
#include "oracle.h"

#include <stdlib.h>
#include <string.h>

typedef struct { float mn[3], mx[3]; } o_box;

static o_box box_empty(void)
{
    o_box b;
    for (int i = 0; i < 3; i++) { b.mn[i] = O_MAX_REAL; b.mx[i] = -O_MAX_REAL; }
    return b;
}
/* BoundingBox::unionBox (core/BoundingBox.h:122-135) */
static o_box box_union(o_box a, o_box b)
{
    o_box r;
    for (int i = 0; i < 3; i++) { r.mn[i] = smin(a.mn[i], b.mn[i]); r.mx[i] = smax(a.mx[i], b.mx[i]); }
    return r;
}
static o_box box_union_pt(o_box a, v3 p)
{
    o_box r = a;
    r.mn[0] = smin(a.mn[0], p.x); r.mn[1] = smin(a.mn[1], p.y); r.mn[2] = smin(a.mn[2], p.z);
    r.mx[0] = smax(a.mx[0], p.x); r.mx[1] = smax(a.mx[1], p.y); r.mx[2] = smax(a.mx[2], p.z);
    return r;
}
/* BoundingBox.h:48-53 */
static float box_sa(o_box b)
{
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    return 2.f * (dx * dy + dy * dz + dx * dz);
}
static float box_centroid(o_box b, int a) { return 0.5f * (b.mx[a] + b.mn[a]); }

typedef struct { o_box box; int axis, first, count, right; } o_lnode;

enum { P_TRI = 0, P_SPHERE = 1, P_MESH = 2 };
typedef struct { int kind, id; } o_pref;

struct o_bvh {
    o_lnode *nodes; int n_nodes, cap_nodes;
    o_pref *prims; int n_prims;
    o_bvh **sub; int n_sub;  /* top level: mesh BVHs by mesh index */
};

/* build-time record */
typedef struct { o_pref ref; o_box box; float cen[3]; float bcen[3]; } o_bprim;

typedef struct o_bnode {
    o_box box;
    int axis, first, count;
    struct o_bnode *c[2];
} o_bnode;

typedef struct { o_bprim *p; int n; int nodes; } o_build;

static o_bnode *bnode_new(void)
{
    o_bnode *n = (o_bnode *)calloc(1, sizeof(o_bnode));
    n->box = box_empty();
    return n;
}
static void bnode_free(o_bnode *n)
{
    if (!n) return;
    bnode_free(n->c[0]); bnode_free(n->c[1]);
    free(n);
}

/* deterministic stable sort of p[start,end) by box centroid on an axis
 * (sortAxis, accelStruct/Bvh.h:225-240, strict less-than) */
static int g_sort_axis;
static int cmp_bprim(const void *a, const void *b)
{
    const o_bprim *x = (const o_bprim *)a, *y = (const o_bprim *)b;
    float ka = x->bcen[g_sort_axis], kb = y->bcen[g_sort_axis];
    if (ka < kb) return -1;
    if (kb < ka) return 1;
    return 0;
}
static void stable_sort_axis(o_bprim *p, int n, int axis)
{
    /* insertion sort for small ranges keeps equal keys in order */
    if (n <= 48) {
        for (int i = 1; i < n; i++) {
            o_bprim t = p[i];
            int j = i - 1;
            while (j >= 0 && t.bcen[axis] < p[j].bcen[axis]) { p[j + 1] = p[j]; j--; }
            p[j + 1] = t;
        }
        return;
    }
    /* merge sort */
    o_bprim *tmp = (o_bprim *)malloc(sizeof(o_bprim) * (size_t)n);
    int h = n / 2;
    stable_sort_axis(p, h, axis);
    stable_sort_axis(p + h, n - h, axis);
    int i = 0, j = h, k = 0;
    while (i < h && j < n) {
        if (p[j].bcen[axis] < p[i].bcen[axis]) tmp[k++] = p[j++];
        else tmp[k++] = p[i++];
    }
    while (i < h) tmp[k++] = p[i++];
    while (j < n) tmp[k++] = p[j++];
    memcpy(p, tmp, sizeof(o_bprim) * (size_t)n);
    free(tmp);
    (void)cmp_bprim;
}

/* Bvh::buildNode, SAH case (Bvh.cpp:172-246) */
static void build_node(o_build *B, int start, int end, o_bnode *node)
{
    B->nodes++;
    int number = end - start;
    float *surf = (float *)malloc(sizeof(float) * (size_t)(number > 0 ? number : 1));
    float minCost = 1.f * (float)number;
    int bestIndex = -1, bestAxis = -1;
    for (int axis = 0; axis < 3; axis++) {
        stable_sort_axis(B->p + start, number, axis);
        o_box box = box_empty();
        for (int i = start, c = 0; i < end; i++, c++) {
            box = box_union(box, B->p[i].box);
            surf[c] = box_sa(box);
        }
        if (axis == 0) node->box = box;
        float factor = 1.f / box_sa(node->box);
        o_box rb = box_empty();
        for (int j = number - 1; j >= 1; j--) {
            int index = start + j;
            rb = box_union(rb, B->p[index].box);
            float la = surf[j - 1];
            float ra = box_sa(rb);
            float ln = (float)j, rn = (float)(number - j);
            float cost = 2 * 1.f + factor * (ln * la + rn * ra);
            if (cost < minCost) { minCost = cost; bestIndex = index; bestAxis = axis; }
        }
    }
    free(surf);
    if (bestIndex == -1) {
        node->first = start;
        node->count = number;
        return;
    }
    stable_sort_axis(B->p + start, number, bestAxis);
    node->c[0] = bnode_new();
    node->c[1] = bnode_new();
    build_node(B, start, bestIndex, node->c[0]);
    build_node(B, bestIndex, end, node->c[1]);
}

/* Bvh::getLargestAxisExtent (Bvh.cpp:373-381) */
static int largest_axis(o_box b)
{
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    if (dx > dy && dx > dz) return 0;
    if (dz > dx && dz > dy) return 2;
    return 1;
}

#define O_BINS 16
/* Bvh::buildBinNode (Bvh.cpp:611-771) */
static void build_bin_node(o_build *B, int start, int end, o_bnode *node)
{
    int number = end - start;
    if (number < 32) { build_node(B, start, end, node); return; }
    B->nodes++;
    int axis = largest_axis(node->box);
    float mn = node->box.mn[axis], mx = node->box.mx[axis];
    float binc = (float)O_BINS / (mx - mn);
    node->axis = axis;
    o_box bb[O_BINS]; int bc[O_BINS];
    for (int i = 0; i < O_BINS; i++) { bb[i] = box_empty(); bc[i] = 0; }
    for (int i = start; i < end; i++) {
        int idx = imin(imax((int)((B->p[i].cen[axis] - mn) * binc), 0), O_BINS - 1);
        bb[idx] = box_union(bb[idx], B->p[i].box);
        bc[idx]++;
    }
    float minCost = 1.f * (float)number;
    int best = -1;
    o_box lb[O_BINS];
    lb[0] = bb[0];
    for (int i = 1; i < O_BINS; i++) { bc[i] += bc[i - 1]; lb[i] = box_union(lb[i - 1], bb[i]); }
    float factor = 1.f / box_sa(node->box);
    o_box rb = bb[O_BINS - 1], bestR = box_empty();
    for (int i = O_BINS - 2; i >= 0; i--) {
        float ln = (float)bc[i], rn = (float)(number - bc[i]);
        float cost = 2 * 1.f + factor * (ln * box_sa(lb[i]) + rn * box_sa(rb));
        if (cost < minCost) { minCost = cost; best = i; bestR = rb; }
        rb = box_union(rb, bb[i]);
    }
    if (best == -1) { B->nodes--; build_node(B, start, end, node); return; }
    int leftCount = bc[best];
    o_bprim *tmp = (o_bprim *)malloc(sizeof(o_bprim) * (size_t)number);
    int tl = 0, tr = leftCount;
    for (int i = start; i < end; i++) {
        int idx = imin(imax((int)((B->p[i].cen[axis] - mn) * binc), 0), O_BINS - 1);
        if (idx <= best) tmp[tl++] = B->p[i]; else tmp[tr++] = B->p[i];
    }
    memcpy(B->p + start, tmp, sizeof(o_bprim) * (size_t)number);
    free(tmp);
    node->c[0] = bnode_new(); node->c[0]->box = lb[best];
    node->c[1] = bnode_new(); node->c[1]->box = bestR;
    build_bin_node(B, start, start + leftCount, node->c[0]);
    build_bin_node(B, start + leftCount, end, node->c[1]);
}

/* Bvh::flatten (Bvh.cpp:587-607), pre-order */
static int flatten(o_bvh *b, o_bnode *n)
{
    if (b->n_nodes == b->cap_nodes) {
        b->cap_nodes = b->cap_nodes ? b->cap_nodes * 2 : 64;
        b->nodes = (o_lnode *)realloc(b->nodes, sizeof(o_lnode) * (size_t)b->cap_nodes);
    }
    int off = b->n_nodes++;
    o_lnode *ln = &b->nodes[off];
    ln->box = n->box; ln->axis = 0; ln->first = 0; ln->count = 0; ln->right = -1;
    if (!n->c[0] && !n->c[1]) {
        ln->first = n->first; ln->count = n->count;
    } else {
        b->nodes[off].axis = n->axis;
        flatten(b, n->c[0]);
        int r = flatten(b, n->c[1]);
        b->nodes[off].right = r;
    }
    return off;
}

/* Bvh::build (Bvh.cpp:51-79) */
static o_bvh *build_bvh(o_bprim *p, int n)
{
    o_bvh *b = (o_bvh *)calloc(1, sizeof(o_bvh));
    if (n == 0) return b;
    o_build B; B.p = p; B.n = n; B.nodes = 0;
    o_box root = box_empty();
    for (int i = 0; i < n; i++) root = box_union(root, p[i].box);
    o_bnode *r = bnode_new();
    r->box = root;
    build_bin_node(&B, 0, n, r);
    flatten(b, r);
    bnode_free(r);
    b->n_prims = n;
    b->prims = (o_pref *)malloc(sizeof(o_pref) * (size_t)n);
    for (int i = 0; i < n; i++) b->prims[i] = p[i].ref;
    return b;
}

static void tri_verts(const rt_scene_desc *d, int tri, v3 *p0, v3 *p1, v3 *p2)
{
    const int32_t *ix = d->indices + 3 * (size_t)tri;
    *p0 = v3_from(d->vertices + 3 * (size_t)ix[0]);
    *p1 = v3_from(d->vertices + 3 * (size_t)ix[1]);
    *p2 = v3_from(d->vertices + 3 * (size_t)ix[2]);
}

/* Sphere world box: GeometricShape::getWorldBoundingBox via Transform::transform(BoundingBox)
 * (core/Transform.h:145-158) */
static o_box sphere_box(const rt_sphere_desc *s)
{
    float r = s->radius;
    float mn[3] = {-r, -r, -r}, mx[3] = {r, r, r};
    if (s->kind == RT_ANALYTIC_PLANE) {   /* Plane::getLocalBoundingBox (Plane.cpp:28-42) */
        mn[0] = -1.f; mn[1] = -1.f; mn[2] = 0.f;
        mx[0] = 1.f; mx[1] = 1.f; mx[2] = 0.f;
    }
    const float cx[8][3] = {
        {mn[0], mn[1], mn[2]}, {mn[0], mn[1], mx[2]}, {mn[0], mx[1], mx[2]}, {mx[0], mx[1], mx[2]},
        {mx[0], mn[1], mn[2]}, {mx[0], mx[1], mn[2]}, {mx[0], mn[1], mx[2]}, {mn[0], mx[1], mn[2]}};
    o_box b = box_empty();
    for (int i = 0; i < 8; i++) b = box_union_pt(b, xf_point(s->to_world, mk3(cx[i][0], cx[i][1], cx[i][2])));
    return b;
}

void o_bvh_free(o_bvh *b)
{
    if (!b) return;
    for (int i = 0; i < b->n_sub; i++) o_bvh_free(b->sub[i]);
    free(b->sub); free(b->nodes); free(b->prims); free(b);
}

/* Bvh::getWorldBoundingBox (accelStruct/Bvh.h:166-169): the root box */
void o_bvh_root_box(const o_bvh *b, float *out6)
{
    for (int i = 0; i < 3; i++) { out6[i] = O_MAX_REAL; out6[3 + i] = -O_MAX_REAL; }
    if (!b || b->n_nodes == 0) return;
    for (int i = 0; i < 3; i++) { out6[i] = b->nodes[0].box.mn[i]; out6[3 + i] = b->nodes[0].box.mx[i]; }
}

int o_bvh_node_count(const o_bvh *b)
{
    int n = b->n_nodes;
    for (int i = 0; i < b->n_sub; i++) if (b->sub[i]) n += b->sub[i]->n_nodes;
    return n;
}

o_bvh *o_bvh_build_scene(const o_scene *sc)
{
    const rt_scene_desc *d = sc->d;
    o_bvh **sub = (o_bvh **)calloc((size_t)(d->n_meshes > 0 ? d->n_meshes : 1), sizeof(o_bvh *));
    int nobj = d->n_meshes + d->n_spheres;
    o_bprim *top = (o_bprim *)malloc(sizeof(o_bprim) * (size_t)(nobj > 0 ? nobj : 1));
    int ntop = 0;
    for (int m = 0; m < d->n_meshes; m++) {
        const rt_mesh_desc *M = &d->meshes[m];
        o_bprim *p = (o_bprim *)malloc(sizeof(o_bprim) * (size_t)(M->n_tris > 0 ? M->n_tris : 1));
        for (int i = 0; i < M->n_tris; i++) {
            int tri = M->first_tri + i;
            v3 p0, p1, p2;
            tri_verts(d, tri, &p0, &p1, &p2);
            /* Triangle::getWorldBoundingBox (Triangle.h:65-87) */
            o_box b;
            b.mn[0] = p0.x; b.mn[1] = p0.y; b.mn[2] = p0.z;
            b.mx[0] = p0.x; b.mx[1] = p0.y; b.mx[2] = p0.z;
            v3 q[2] = {p1, p2};
            for (int k = 0; k < 2; k++) {
                b.mn[0] = smin(q[k].x, b.mn[0]); b.mn[1] = smin(q[k].y, b.mn[1]); b.mn[2] = smin(q[k].z, b.mn[2]);
                b.mx[0] = smax(q[k].x, b.mx[0]); b.mx[1] = smax(q[k].y, b.mx[1]); b.mx[2] = smax(q[k].z, b.mx[2]);
            }
            p[i].box = b;
            p[i].ref.kind = P_TRI; p[i].ref.id = tri;
            /* Triangle::getCentroid (Triangle.h:92-99) */
            v3 c = v3_smul(1.f / 3, v3_add(v3_add(p0, p1), p2));
            p[i].cen[0] = c.x; p[i].cen[1] = c.y; p[i].cen[2] = c.z;
            for (int a = 0; a < 3; a++) p[i].bcen[a] = box_centroid(b, a);
        }
        sub[m] = build_bvh(p, M->n_tris);
        free(p);
        o_box rb = box_empty();
        if (sub[m]->n_nodes > 0) rb = sub[m]->nodes[0].box;
        top[ntop].box = rb;
        top[ntop].ref.kind = P_MESH; top[ntop].ref.id = m;
        for (int a = 0; a < 3; a++) { top[ntop].cen[a] = box_centroid(rb, a); top[ntop].bcen[a] = top[ntop].cen[a]; }
        ntop++;
    }
    for (int s = 0; s < d->n_spheres; s++) {
        o_box b = sphere_box(&d->spheres[s]);
        top[ntop].box = b;
        top[ntop].ref.kind = P_SPHERE; top[ntop].ref.id = s;
        v3 c = xf_point(d->spheres[s].to_world, mk3(0.f, 0.f, 0.f));
        top[ntop].cen[0] = c.x; top[ntop].cen[1] = c.y; top[ntop].cen[2] = c.z;
        for (int a = 0; a < 3; a++) top[ntop].bcen[a] = box_centroid(b, a);
        ntop++;
    }
    o_bvh *t = build_bvh(top, ntop);
    free(top);
    t->sub = sub;
    t->n_sub = d->n_meshes;
    return t;
}

/* ---------------- export (test infrastructure for rt_scene_create_bvh) ----
 * The two-level tree of o_bvh_build_scene as one binary tree over the
 * scene's triangles, the form a plugin hands to rt_scene_create_bvh: every
 * top-level mesh leaf replaced by that mesh's tree, spheres and planes left
 * out (the device tests them after the tree), a top-level leaf of several
 * meshes joined into a chain.  Nodes are numbered in post-order and the root
 * is then swapped to index 0. */
typedef struct { rt_bvh_node *nodes; int n, cap; int32_t *prims; int np, capp; int err; } o_exp;

static int exp_new(o_exp *E)
{
    if (E->n >= E->cap) { E->err = 1; return -1; }
    int k = E->n++;
    E->nodes[k].left = E->nodes[k].right = -1;
    E->nodes[k].first = E->nodes[k].count = 0;
    return k;
}
static int exp_join(o_exp *E, int l, int r)
{
    if (l < 0) return r;
    if (r < 0) return l;
    int k = exp_new(E);
    if (k < 0) return -1;
    E->nodes[k].left = l;
    E->nodes[k].right = r;
    return k;
}
static int exp_mesh(o_exp *E, const o_bvh *b, int i)
{
    const o_lnode *ln = &b->nodes[i];
    if (ln->right < 0) {   /* leaf */
        if (ln->count <= 0) return -1;
        int k = exp_new(E);
        if (k < 0) return -1;
        E->nodes[k].first = E->np;
        E->nodes[k].count = ln->count;
        for (int j = 0; j < ln->count; j++) {
            if (E->np >= E->capp) { E->err = 1; return -1; }
            E->prims[E->np++] = b->prims[ln->first + j].id;
        }
        return k;
    }
    int l = exp_mesh(E, b, i + 1);
    int r = exp_mesh(E, b, ln->right);
    return exp_join(E, l, r);
}
static int exp_top(o_exp *E, const o_bvh *t, int i)
{
    const o_lnode *ln = &t->nodes[i];
    if (ln->right < 0) {
        int acc = -1;
        for (int j = 0; j < ln->count; j++) {
            o_pref p = t->prims[ln->first + j];
            if (p.kind != P_MESH) continue;
            const o_bvh *s = t->sub[p.id];
            if (s && s->n_nodes > 0) acc = exp_join(E, acc, exp_mesh(E, s, 0));
        }
        return acc;
    }
    int l = exp_top(E, t, i + 1);
    int r = exp_top(E, t, ln->right);
    return exp_join(E, l, r);
}
int32_t oracle_export_bvh(const o_scene *sc, rt_bvh_node *nodes, int32_t cap_nodes, int32_t *prims, int32_t cap_prims,
                          int32_t *n_nodes, int32_t *n_prims)
{
    o_exp E = {nodes, 0, cap_nodes, prims, 0, cap_prims, 0};
    int root = (sc->top && sc->top->n_nodes > 0) ? exp_top(&E, sc->top, 0) : -1;
    if (E.err) return 1;
    if (root > 0) {
        rt_bvh_node tmp = E.nodes[0];
        E.nodes[0] = E.nodes[root];
        E.nodes[root] = tmp;
        for (int k = 0; k < E.n; k++) {
            if (E.nodes[k].count != 0) continue;
            if (E.nodes[k].left == 0) E.nodes[k].left = root;
            else if (E.nodes[k].left == root) E.nodes[k].left = 0;
            if (E.nodes[k].right == 0) E.nodes[k].right = root;
            else if (E.nodes[k].right == root) E.nodes[k].right = 0;
        }
    }
    *n_nodes = E.n;
    *n_prims = E.np;
    return 0;
}

/* ---------------- intersection ---------------- */
typedef struct { float t, u, v; int prim; v3 p; } o_rec;

/* Triangle::intersection (Triangle.cpp:46-88) */
static int tri_hit_p(v3 p0, v3 p1, v3 p2, const o_ray *r, float *t, float *u, float *v)
{
    v3 e1 = v3_sub(p1, p0), e2 = v3_sub(p2, p0), s = v3_sub(r->o, p0);
    v3 s1 = v3_cross(r->d, e2), s2 = v3_cross(s, e1);
    float det = v3_dot(s1, e1);
    if ((double)fabsf(det) < 1e-8) return 0;
    float inv = 1 / det;
    float b1 = inv * v3_dot(s1, s);
    if (b1 < 0.f || b1 > 1.f) return 0;
    float b2 = inv * v3_dot(s2, r->d);
    if (b2 < 0.f || b1 + b2 > 1.f) return 0;
    float tt = inv * v3_dot(s2, e2);
    if (tt < r->mint || tt > r->maxt) return 0;
    *t = tt; *u = b1; *v = b2;
    return 1;
}
static int tri_hit(const rt_scene_desc *d, int tri, const o_ray *r, float *t, float *u, float *v)
{
    v3 p0, p1, p2;
    tri_verts(d, tri, &p0, &p1, &p2);
    return tri_hit_p(p0, p1, p2, r, t, u, v);
}

/* Pin hook: Triangle::intersection of each ray against the triangle tri_v
 * (9 floats), with the ray's own [mint, maxt] (no adaptive epsilon: that is
 * the BVH's, Bvh.cpp:411-413).  hits: t, u, v, prim 0 on a hit, -1 else. */
int32_t oracle_tri_query(const float *tri_v, const rt_ray *rays, int32_t n, rt_hit *hits)
{
    v3 p0 = mk3(tri_v[0], tri_v[1], tri_v[2]), p1 = mk3(tri_v[3], tri_v[4], tri_v[5]);
    v3 p2 = mk3(tri_v[6], tri_v[7], tri_v[8]);
    for (int i = 0; i < n; i++) {
        o_ray r;
        r.o = mk3(rays[i].o[0], rays[i].o[1], rays[i].o[2]);
        r.d = mk3(rays[i].d[0], rays[i].d[1], rays[i].d[2]);
        r.mint = rays[i].mint;
        r.maxt = rays[i].maxt;
        float t = 0, u = 0, v = 0;
        memset(&hits[i], 0, sizeof(hits[i]));
        hits[i].prim = -1;
        if (tri_hit_p(p0, p1, p2, &r, &t, &u, &v)) {
            hits[i].t = t; hits[i].u = u; hits[i].v = v; hits[i].prim = 0;
        }
    }
    return RT_OK;
}

/* Sphere::intersection (Sphere.cpp:38-111) */
static int sphere_hit(const rt_sphere_desc *sp, const o_ray *r, float *t)
{
    v3 lo = xf_point(sp->to_object, r->o);
    v3 ld = xf_vector(sp->to_object, r->d);
    v3 sto = v3_sub(lo, mk3(0.f, 0.f, 0.f));
    float a = 1;
    float b = 2 * v3_dot(ld, sto);
    float c = v3_dot(sto, sto) - sp->radius * sp->radius;
    float delta = b * b - 4 * a * c;
    if (delta < 0) return 0;
    float t1 = (-b + sqrtf(delta)) / (2 * a);
    float t2 = (-b - sqrtf(delta)) / (2 * a);
    float tn = t1, tf = t2;
    if (tn > tf) { float q = tn; tn = tf; tf = q; }
    if (tn <= r->mint) {
        if (tf > r->mint && tf < r->maxt) { *t = tf; return 1; }
        return 0;
    } else if (tn > r->mint && tn < r->maxt) { *t = tn; return 1; }
    return 0;
}

/* Plane::intersection (Plane.cpp:63-79).  A ray lying in the plane gives
 * t = NaN, which the reference's range test lets through as a hit; here it is
 * a miss. */
static int plane_hit(const rt_sphere_desc *sp, const o_ray *r, float *t)
{
    v3 lo = xf_point(sp->to_object, r->o);
    v3 ld = xf_vector(sp->to_object, r->d);
    float tt = -lo.z / ld.z;
    if (!(tt >= r->mint && tt <= r->maxt)) return 0;
    v3 q = v3_add(lo, v3_smul(tt, ld));
    if (q.x < -1.f || q.x > 1.f || q.y < -1.f || q.y > 1.f) return 0;
    *t = tt;
    return 1;
}

static int box_hit(const o_box *b, const o_ray *r)
{
    float nearT = -O_MAX_REAL, farT = O_MAX_REAL;
    for (int i = 0; i < 3; i++) {
        float o = v3_get(r->o, i), dd = v3_get(r->d, i), inv = v3_get(r->inv, i);
        float mn = b->mn[i], mx = b->mx[i];
        if (dd == 0) {
            if (o < mn || o > mx) return 0;
        } else {
            float t1 = (mn - o) * inv, t2 = (mx - o) * inv;
            if (t1 > t2) { float q = t1; t1 = t2; t2 = q; }
            nearT = smax(t1, nearT);
            farT = smin(t2, farT);
            if (!(nearT <= farT)) return 0;
        }
    }
    return (r->mint <= farT && r->maxt >= nearT);
}

static int bvh_isect(const o_scene *sc, const o_bvh *b, const o_ray *in, o_rec *rec, int shadow);

/* SimplePrimitive / nested Bvh leaf dispatch (core/Primitive.cpp:19-39) */
static int prim_isect(const o_scene *sc, const o_bvh *b, o_pref p, const o_ray *ray, o_rec *rec, int shadow)
{
    const rt_scene_desc *d = sc->d;
    if (p.kind == P_MESH) return bvh_isect(sc, b->sub[p.id], ray, rec, shadow);
    float t, u = 0.f, v = 0.f;
    int hit;
    if (p.kind == P_TRI) hit = tri_hit(d, p.id, ray, &t, &u, &v);
    else if (d->spheres[p.id].kind == RT_ANALYTIC_PLANE) hit = plane_hit(&d->spheres[p.id], ray, &t);
    else hit = sphere_hit(&d->spheres[p.id], ray, &t);
    if (!hit) return 0;
    rec->p = v3_add(ray->o, v3_smul(t, ray->d));
    rec->t = t; rec->u = u; rec->v = v;
    rec->prim = p.kind == P_TRI ? p.id : -p.id - 2;
    return 1;
}

/* Bvh::intersection (Bvh.cpp:392-481) */
static int bvh_isect(const o_scene *sc, const o_bvh *b, const o_ray *in, o_rec *rec, int shadow)
{
    int stack[64];
    int cur = 0, sp = 0;
    int neg[3] = {in->inv.x < 0, in->inv.y < 0, in->inv.z < 0};
    o_ray ray = *in;
    if (ray.mint == O_EPSILON) {
        float m = smax(smax(fabsf(ray.o.x), fabsf(ray.o.y)), fabsf(ray.o.z));
        ray.mint = smax(ray.mint, ray.mint * m);
    }
    if (b->n_nodes == 0 || ray.maxt < ray.mint) return 0;
    int has = 0;
    for (;;) {
        const o_lnode *n = &b->nodes[cur];
        if (!box_hit(&n->box, &ray)) {
            if (sp == 0) break;
            cur = stack[--sp];
            continue;
        }
        if (n->right != -1) {
            if (neg[n->axis]) { stack[sp++] = cur + 1; cur = n->right; }
            else { stack[sp++] = n->right; cur++; }
            if (sp >= 64) return has; /* bound (Bvh.cpp:446 asserts) */
        } else {
            for (int i = n->first; i < n->first + n->count; i++) {
                if (prim_isect(sc, b, b->prims[i], &ray, rec, shadow)) {
                    if (shadow) return 1;
                    ray.maxt = rec->t;
                    has = 1;
                }
            }
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
    return has;
}

/* DifferentialGeometry::coordinateSystem (core/DifferentialGeometry.h:36-50) */
static void frame_from(v3 n, v3 *s, v3 *t)
{
    v3 c;
    if (fabsf(n.x) > fabsf(n.y)) {
        float il = 1.0f / sqrtf(n.x * n.x + n.z * n.z);
        c = mk3(n.z * il, 0.0f, -n.x * il);
    } else {
        float il = 1.0f / sqrtf(n.y * n.y + n.z * n.z);
        c = mk3(0.0f, n.z * il, -n.y * il);
    }
    *t = c;
    *s = v3_cross(c, n);
}

/* Scene::computeIntersection (core/Scene.cpp:106-113): closest hit plus the
 * differential geometry of the hit, or any hit for shadow rays. */
int o_intersect(const o_scene *sc, const o_ray *ray, o_hit *hit, int shadow)
{
    o_rec rec;
    rec.prim = -1; rec.t = O_MAX_REAL;
    int h = bvh_isect(sc, sc->top, ray, &rec, shadow);
    if (!h) return 0;
    hit->t = rec.t; hit->u = rec.u; hit->v = rec.v; hit->prim = rec.prim;
    if (shadow) return 1;
    const rt_scene_desc *d = sc->d;
    if (rec.prim >= 0) {
        int tri = rec.prim;
        v3 p0, p1, p2;
        tri_verts(d, tri, &p0, &p1, &p2);
        float sum = rec.u + rec.v;
        float bx = 1 - sum, by = rec.u, bz = rec.v;
        hit->p = v3_add(v3_add(v3_smul(bx, p0), v3_smul(by, p1)), v3_smul(bz, p2));
        v3 ng = v3_normalized(v3_cross(v3_sub(p1, p0), v3_sub(p2, p0)));
        hit->ng = ng;
        v3 ns = ng;
        if (d->normals && !isnan(d->normals[3 * (size_t)d->indices[3 * (size_t)tri]])) {
            const int32_t *ix = d->indices + 3 * (size_t)tri;
            v3 n0 = v3_from(d->normals + 3 * (size_t)ix[0]);
            v3 n1 = v3_from(d->normals + 3 * (size_t)ix[1]);
            v3 n2 = v3_from(d->normals + 3 * (size_t)ix[2]);
            ns = v3_normalized(v3_add(v3_add(v3_smul(bx, n0), v3_smul(by, n1)), v3_smul(bz, n2)));
        }
        hit->n = ns;
        frame_from(ns, &hit->s, &hit->tt);
        /* texture coordinates (Triangle.cpp:155-170): the vertex uvs with the
         * barycentrics, or the barycentrics themselves for a mesh without */
        hit->uv = mk2(rec.u, rec.v);
        if (d->uvs && !isnan(d->uvs[2 * (size_t)d->indices[3 * (size_t)tri]])) {
            const int32_t *ix = d->indices + 3 * (size_t)tri;
            const float *u0 = d->uvs + 2 * (size_t)ix[0], *u1 = d->uvs + 2 * (size_t)ix[1], *u2 = d->uvs + 2 * (size_t)ix[2];
            hit->uv = mk2((bx * u0[0] + by * u1[0]) + bz * u2[0], (bx * u0[1] + by * u1[1]) + bz * u2[1]);
        }
    } else {
        const rt_sphere_desc *sp = &d->spheres[-rec.prim - 2];
        hit->uv = o_sphere_uv(sp, ray, rec.t);
        hit->p = rec.p;
        v3 n;
        if (sp->kind == RT_ANALYTIC_PLANE) n = o_plane_normal(sp);
        else {
            v3 nl = v3_normalized(v3_sub(xf_point(sp->to_object, rec.p), mk3(0, 0, 0)));
            n = v3_normalized(xf_normal(sp->to_object, nl));
        }
        hit->ng = n;
        hit->n = n;
        frame_from(n, &hit->s, &hit->tt);
    }
    return 1;
}
