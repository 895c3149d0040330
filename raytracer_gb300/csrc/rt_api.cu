// rt_api.cu -- kernels of the GB300 light-transport core and its C ABI.
//
// Render structure (one rt_render call):
//   for each batch of whole reference tiles (all samples of their pixels):
//     k_camera          camera rays of every path (SampleJob.cpp:46-59)
//     repeat per path vertex (PathTracingMIS):
//       k_trace<closest> BSDF-sampled / primary rays      (Bvh.cpp:392-481)
//       k_trace<any>     light-sample shadow rays         (Integrator.cpp:228-232)
//       k_pt_shade       resolve the previous vertex, shade the new one
//                        (PathTracingMIS.cpp:54-259), compact survivors
//     or, for VolPathTracing, k_volpath: one persistent kernel that takes
//     paths from a work counter and runs VolPathTracing::li to completion
//     k_film            per-pixel reduction in the reference's sample order
//                       (Screen::addSample with the box filter, Screen::merge)
#include "rt_kernels.cuh"
#include "rt_bvh.h"
#include "../../include/rtgpu.h"

#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <algorithm>

#include "rt_internal.h"

using namespace rtgpu;

// =====================================================================
// error handling
// =====================================================================
static thread_local std::string g_err;
static rt_status fail(rt_status st, const std::string &msg)
{
    g_err = msg;
    return st;
}
// RT_ERR_LIMIT message naming the caps whose bits a render read back
static std::string limit_message(int bits)
{
    std::string m = "a device loop reached its iteration cap:";
    if (bits & RT_LIM_STACK2) m += " BVH2 traversal stack;";
    if (bits & RT_LIM_STACK4) m += " 4-wide traversal stack;";
    if (bits & RT_LIM_STACK8) m += " 8-wide group stack;";
    if (bits & RT_LIM_VOLPATH) m += " VolPathTracing loop cap;";
    return m;
}
#define CK(call)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail(RT_ERR_CUDA, std::string(#call " -> ") + cudaGetErrorString(e_)); \
    } while (0)

// =====================================================================
// kernels
// =====================================================================
__device__ __forceinline__ float4 f4(V3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ float4 f4c(C3 c, float w) { return make_float4(c.r, c.g, c.b, w); }
__device__ __forceinline__ V3 xyz(float4 a) { return v3(a.x, a.y, a.z); }
__device__ __forceinline__ C3 rgb(float4 a) { return c3(a.x, a.y, a.z); }

// warp-aggregated append to a queue
__device__ __forceinline__ void q_push(int *queue, int *count, int value, bool pred)
{
    unsigned mask = __ballot_sync(__activemask(), pred);
    if (!pred) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(mask, base, leader);
    queue[base + __popc(mask & ((1u << lane) - 1))] = value;
}

// Film footprint of a sample inside its tile: Screen::addSample with the
// box filter of radius 0.5 (Screen.cpp:52-66).  Returns the code
// (sx - lx + 1) | (ex - lx + 1) << 2 | (sy - ly + 1) << 4 | (ey - ly + 1) << 6,
// 0x55 being the usual "own pixel only".
__device__ __forceinline__ uint8_t splat_code(float xx, float yy, int ox, int oy, int lx, int ly, int tw, int th)
{
    float fx = xx - 0.5f - (float)(ox - 0);
    float fy = yy - 0.5f - (float)(oy - 0);
    int sx = (int)ceilf(fx - 0.5f), ex = (int)floorf(fx + 0.5f);
    int sy = (int)ceilf(fy - 0.5f), ey = (int)floorf(fy + 0.5f);
    sx = imax(0, sx); ex = imin(tw - 1, ex);
    sy = imax(0, sy); ey = imin(th - 1, ey);
    // ranges are within [lx-1, lx+1]; an empty range encodes as start > end
    int a = imin(imax(sx - lx + 1, 0), 3), b = imin(imax(ex - lx + 1, -1), 2);
    int c = imin(imax(sy - ly + 1, 0), 3), d = imin(imax(ey - ly + 1, -1), 2);
    if (b < 0 || d < 0 || a > b || c > d) return 0xFF;  // contributes nowhere
    return (uint8_t)(a | (b << 2) | (c << 4) | (d << 6));
}
__device__ __forceinline__ bool splat_covers(uint8_t code, int dx, int dy)
{
    // dx, dy: target offset from the source pixel, in [-1, 1]
    if (code == 0xFF) return false;
    int a = (code & 3) - 1, b = ((code >> 2) & 3) - 1, c = ((code >> 4) & 3) - 1, d = ((code >> 6) & 3) - 1;
    return dx >= a && dx <= b && dy >= c && dy <= d;
}

struct RenderParams {
    DevScene S;
    Wave W;
    int4 *tileorder;   // g -> (x, y, lx | ly << 16, tw | th << 16)
    int g0;            // first tile-order index of the batch
    int npix, spp, sample_begin, n_paths;
    uint64_t seed;
    int max_depth, min_depth;
    int *limit_flag;
    unsigned long long *stats;  // [0] closest rays, [1] shadow rays, [2] nan samples
    // graph-launched rounds: the round index lives in device memory (the
    // round loop is a conditional node; k_round_next advances it); null when
    // the host passes the round as a kernel argument
    int *round_dev;
    // rounds with fewer closest-hit rays than this are not sorted by
    // material: their hits go to one queue shaded by k_pt_shade<RT_QUEUE_MIXED>
    int sort_threshold;
    // PathTracingMIS with the all-lights strategy: every light sampled at
    // every vertex, its shadow ray traced in the shading kernel (the
    // k_pt_shade<..., ALL> kernels)
    int all_lights;
    // multi-scene batches: the scene table (one entry per job, indexed by
    // W.sid), the batch's work items and their count; null otherwise
    const DevScene *scenes;
    const MultiItem *items;
    int n_items;
    // rt_render_paths: slot i renders (pixel path_list[i].x, absolute sample
    // index path_list[i].y) and is not reduced into a film; null otherwise
    const int2 *path_list;
};

__device__ __forceinline__ int cur_round(const RenderParams &P, int round)
{
    return P.round_dev ? __ldcg(P.round_dev) : round;
}

// ---------------------------------------------------------------- camera
__global__ void k_camera(RenderParams P)
{
    const DevCamera &cam = P.S.cam;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < P.n_paths; slot += gridDim.x * blockDim.x) {
        int q = 0, x, y, lx = 0, ly = 0, tw = 1, th = 1, smp;
        if (P.path_list) {
            const int2 pl = P.path_list[slot];
            x = pl.x % cam.width;
            y = pl.x / cam.width;
            smp = pl.y;
        } else {
            q = slot % P.npix;
            int s = slot / P.npix;
            int4 to = P.tileorder[P.g0 + q];
            x = to.x; y = to.y;
            lx = to.z & 0xffff; ly = to.z >> 16; tw = to.w & 0xffff; th = to.w >> 16;
            smp = P.sample_begin + s;
        }
        Pcg32 rng;
        path_stream_seed(rng, P.seed, (uint32_t)(y * cam.width + x), (uint32_t)smp);
        V2 j = next2d(rng);
        float xx = (float)x + j.x, yy = (float)y + j.y;
        V2 lens = v2(0.f, 0.f);
        if (cam.aperture_radius > 0.f) lens = next2d(rng);
        Ray r = camera_ray(cam, xx, yy, lens);
        if (!P.path_list) {
            uint8_t code = splat_code(xx, yy, x - lx, y - ly, lx, ly, tw, th);
            P.W.splat[slot] = code;
            if (code != 0x55) P.W.pix_irregular[q] = 1;
        }
        P.W.rng[slot] = rng;
        P.W.ray_o[slot] = f4(r.o, r.mint);
        P.W.ray_d[slot] = f4(r.d, r.maxt);
        P.W.tp[slot] = make_float4(1.f, 1.f, 1.f, 1.f);
        P.W.rad[slot] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
        P.W.flags[slot] = F_FIRST;
        P.W.q_closest[slot] = slot;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.W.cnt[0].closest = P.n_paths;
        P.W.cnt[0].shadow = 0;
    }
}

// Camera rays of a multi-scene batch: the work item of each slot (binary
// search over the items' first slots), then exactly what k_camera does for
// that item's job: its camera, tile order and seed.  The slot's scene-table
// index is recorded for the kernels that follow.
__device__ __forceinline__ int item_of_slot(const MultiItem *items, int n_items, int slot)
{
    int lo = 0, hi = n_items - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (items[mid].path0 <= slot) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__global__ void k_camera_multi(RenderParams P)
{
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < P.n_paths; slot += gridDim.x * blockDim.x) {
        const MultiItem &it = P.items[item_of_slot(P.items, P.n_items, slot)];
        const DevCamera &cam = P.scenes[it.job].cam;
        const int local = slot - it.path0;
        const int q = local % it.npix;
        const int s = local / it.npix;
        int4 to = it.tileorder[it.g0 + q];
        int x = to.x, y = to.y;
        int lx = to.z & 0xffff, ly = to.z >> 16, tw = to.w & 0xffff, th = to.w >> 16;
        Pcg32 rng;
        path_stream_seed(rng, it.seed, (uint32_t)(y * cam.width + x), (uint32_t)(it.sample_begin + s));
        V2 j = next2d(rng);
        float xx = (float)x + j.x, yy = (float)y + j.y;
        V2 lens = v2(0.f, 0.f);
        if (cam.aperture_radius > 0.f) lens = next2d(rng);
        Ray r = camera_ray(cam, xx, yy, lens);
        uint8_t code = splat_code(xx, yy, x - lx, y - ly, lx, ly, tw, th);
        P.W.splat[slot] = code;
        if (code != 0x55) P.W.pix_irregular[it.pix0 + q] = 1;
        P.W.sid[slot] = it.job;
        P.W.rng[slot] = rng;
        P.W.ray_o[slot] = f4(r.o, r.mint);
        P.W.ray_d[slot] = f4(r.d, r.maxt);
        P.W.tp[slot] = make_float4(1.f, 1.f, 1.f, 1.f);
        P.W.rad[slot] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
        P.W.flags[slot] = F_FIRST;
        P.W.q_closest[slot] = slot;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.W.cnt[0].closest = P.n_paths;
        P.W.cnt[0].shadow = 0;
    }
}

// Sort a traced path by what its ray hit: the shading queue of the hit
// surface's BSDF type, or the finish queue for a miss or a surface without a
// BSDF.  Called by the lanes that just finished a closest-hit ray.
// `n` is the round's closest-hit ray count: below P.sort_threshold the hits
// are not sorted by material (one queue, one generic shading kernel).
__device__ __forceinline__ void classify_hit(const RenderParams &P, const DevScene &S, RoundCounters *C, int slot,
                                             int prim, int n)
{
    const int t = prim == -1 ? -1 : prim_type(S, prim);
    if (n < P.sort_threshold) {
        q_push(P.W.q_mixed, &C->mixed, slot, t >= 0);
    } else {
#pragma unroll
        for (int k = 0; k < RT_NBSDF; k++) q_push(P.W.q_mat[k], &C->mat[k], slot, t == k);
        if (S.has_mixed) q_push(P.W.q_mixed, &C->mixed, slot, t == RT_QUEUE_MIXED);
    }
    q_push(P.W.q_fin, &C->fin, slot, t < 0);
}

// ---------------------------------------------------------------- ray reordering
// Before a trace, the queued rays can be regrouped by a key made of the
// direction octant and the Morton code of the origin on a 32^3 grid over the
// scene bounds (a counting sort: key counts, exclusive scan, scatter), so
// that a warp traces rays that start close together and head the same way.
// Every ray still gets its own result; only the order in which rays are
// taken from the queue changes.
#define RT_SORT_GRID_BITS 5
#define RT_SORT_BINS (8 << (3 * RT_SORT_GRID_BITS))

__device__ __forceinline__ unsigned spread3(unsigned v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ unsigned ray_sort_key(const DevScene &S, float4 o, float4 d)
{
    const float G = (float)(1 << RT_SORT_GRID_BITS);
    unsigned c[3];
    const float oo[3] = {o.x, o.y, o.z};
    for (int a = 0; a < 3; a++) {
        float ext = S.bmax[a] - S.bmin[a];
        float f = ext > 0.f ? (oo[a] - S.bmin[a]) / ext * G : 0.f;
        int q = (int)f;
        c[a] = (unsigned)imin(imax(q, 0), (1 << RT_SORT_GRID_BITS) - 1);
    }
    unsigned oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
    unsigned m = spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
    return (oct << (3 * RT_SORT_GRID_BITS)) | m;
}
__global__ void k_sort_count(RenderParams P, int round, int shadow)
{
    const RoundCounters *C = &P.W.cnt[round];
    const int n = shadow ? C->shadow : C->closest;
    const int *queue = shadow ? P.W.q_shadow : P.W.q_closest;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int slot = queue[i];
        float4 o = shadow ? P.W.sh_o[slot] : P.W.ray_o[slot];
        float4 d = shadow ? P.W.sh_d[slot] : P.W.ray_d[slot];
        unsigned k = ray_sort_key(P.S, o, d);
        P.W.sort_keys[i] = k;
        atomicAdd(&P.W.sort_hist[k], 1u);
    }
}
// exclusive scan of the key counts, one block of 1024 threads
__global__ void __launch_bounds__(1024) k_sort_scan(RenderParams P)
{
    __shared__ unsigned part[1024];
    const int per = RT_SORT_BINS / 1024;
    unsigned *h = P.W.sort_hist + threadIdx.x * per;
    unsigned s = 0;
    for (int i = 0; i < per; i++) s += h[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        unsigned v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned run = part[threadIdx.x] - s;
    for (int i = 0; i < per; i++) {
        unsigned c = h[i];
        h[i] = run;
        run += c;
    }
}
__global__ void k_sort_scatter(RenderParams P, int round, int shadow)
{
    const RoundCounters *C = &P.W.cnt[round];
    const int n = shadow ? C->shadow : C->closest;
    const int *queue = shadow ? P.W.q_shadow : P.W.q_closest;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned pos = atomicAdd(&P.W.sort_hist[P.W.sort_keys[i]], 1u);
        P.W.sort_tmp[pos] = queue[i];
    }
}
__global__ void k_sort_copy(RenderParams P, int round, int shadow)
{
    const RoundCounters *C = &P.W.cnt[round];
    const int n = shadow ? C->shadow : C->closest;
    int *queue = shadow ? P.W.q_shadow : P.W.q_closest;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) queue[i] = P.W.sort_tmp[i];
}

// ---------------------------------------------------------------- traversal
// Persistent while-while traversal with per-lane dynamic ray fetch.  Lanes
// that finish a ray fetch a new one as soon as enough lanes of the warp are
// idle; inner nodes and leaves are processed in separate loops, and each
// lane postpones the first leaf it reaches until every lane of the warp has
// one, which keeps the warp converged.  COUNT adds BVH node / triangle-slot
// fetch counts to stats[3..6].
#define RT_SENT 0x76543210
#ifndef RT_FETCH_THRESHOLD
#define RT_FETCH_THRESHOLD 28
#endif

#ifndef RT_TRACE_MINB
#define RT_TRACE_MINB 10
#endif
#ifndef RT_TRACE_SSTACK
#define RT_TRACE_SSTACK 0
#endif
// BVH2 build: leaf size limit, SAH bins, node-visit cost (in triangle tests)
#ifndef RT_BVH_LEAF
#define RT_BVH_LEAF 4
#endif
#ifndef RT_BVH_BINS
#define RT_BVH_BINS 32
#endif
#ifndef RT_BVH_CNODE
#define RT_BVH_CNODE 1.0
#endif
// MULTI: a multi-scene batch; each ray traverses the tree of its path's
// scene (P.scenes[W.sid[slot]]), held per lane
template <bool ANY, bool COUNT, bool MULTI = false>
__global__ void __launch_bounds__(128, RT_TRACE_MINB) k_trace(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene S = P.S;
    const DevScene *ms = nullptr;                 // MULTI: the lane's scene
    const float4 *mnodes = nullptr, *mtris = nullptr;
    RoundCounters *C = &P.W.cnt[round];
    const int n = ANY ? C->shadow : C->closest;
    int *wc = ANY ? &C->wc_shadow : &C->wc_closest;
    const int *queue = ANY ? P.W.q_shadow : P.W.q_closest;
    const int lane = threadIdx.x & 31;
    int cnt[2] = {0, 0};

    // traversal stack: the bottom RT_TRACE_SSTACK entries in shared memory
    // (entry i of thread t at [i * 128 + t], conflict-free), the rest in a
    // local array
#if RT_TRACE_SSTACK > 0
    __shared__ int sstack[RT_TRACE_SSTACK * 128];
    int lstack[RT_STACK - RT_TRACE_SSTACK];
#define SPUSH(v)                                                                       \
    do {                                                                               \
        if (sp < RT_TRACE_SSTACK) sstack[sp * 128 + threadIdx.x] = (v);                \
        else lstack[sp - RT_TRACE_SSTACK] = (v);                                       \
        sp++;                                                                          \
    } while (0)
#define SPOP(dst)                                                                      \
    do {                                                                               \
        --sp;                                                                          \
        (dst) = sp < RT_TRACE_SSTACK ? sstack[sp * 128 + threadIdx.x] : lstack[sp - RT_TRACE_SSTACK]; \
    } while (0)
#else
    int stack[RT_STACK];
#define SPUSH(v) stack[sp++] = (v)
#define SPOP(dst) (dst) = stack[--sp]
#endif
    int sp = 0;
    int node = RT_SENT, leaf = 0;
    int slot = -1;
    bool has_ray = false;
    float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, idx = 0, idy = 0, idz = 0, oox = 0, ooy = 0, ooz = 0;
    float tmin = 0, hit_t = 0, hu = 0, hv = 0;
    float lx = 0, hx = 0, ly = 0, hy = 0, lz = 0, hz = 0;   // guarded plane offsets (slab_guard)
    int hprim = -1;
    bool dropped = false;   // a push found the stack full

    for (;;) {
        // ---- fetch rays for lanes whose ray is finished
        const bool terminated = (node == RT_SENT);
        const unsigned mterm = __ballot_sync(0xffffffffu, terminated);
        const int nterm = __popc(mterm);
        int base = 0;
        if (nterm) {
            const int leader = __ffs(mterm) - 1;
            if (lane == leader) base = atomicAdd(wc, nterm);
            base = __shfl_sync(0xffffffffu, base, leader);
        }
        if (terminated) {
            int q = base + __popc(mterm & ((1u << lane) - 1));
            has_ray = q < n;
            if (has_ray) {
                slot = queue[q];
                if (MULTI) {
                    ms = &P.scenes[P.W.sid[slot]];
                    mnodes = ms->nodes;
                    mtris = ms->tri_slots;
                }
                float4 o4 = ANY ? P.W.sh_o[slot] : P.W.ray_o[slot];
                float4 d4 = ANY ? P.W.sh_d[slot] : P.W.ray_d[slot];
                ox = o4.x; oy = o4.y; oz = o4.z; dx = d4.x; dy = d4.y; dz = d4.z;
                tmin = adapt_mint(v3(ox, oy, oz), o4.w);
                hit_t = d4.w;
                hprim = -1;
                const float eps = 1e-20f;
                idx = 1.0f / (fabsf(dx) > eps ? dx : copysignf(eps, dx));
                idy = 1.0f / (fabsf(dy) > eps ? dy : copysignf(eps, dy));
                idz = 1.0f / (fabsf(dz) > eps ? dz : copysignf(eps, dz));
                oox = ox * idx; ooy = oy * idy; ooz = oz * idz;
                lx = -(oox + copysignf(slab_guard(oox), idx)); hx = -(oox - copysignf(slab_guard(oox), idx));
                ly = -(ooy + copysignf(slab_guard(ooy), idy)); hy = -(ooy - copysignf(slab_guard(ooy), idy));
                lz = -(ooz + copysignf(slab_guard(ooz), idz)); hz = -(ooz - copysignf(slab_guard(ooz), idz));
                sp = 0;
                SPUSH(RT_SENT);
                leaf = 0;
                node = ((MULTI ? ms->n_nodes : S.n_nodes) > 0 && !(hit_t < tmin)) ? 0 : RT_SENT;
            }
        }
        if (!__any_sync(0xffffffffu, has_ray)) break;

        // ---- traversal
        while (node != RT_SENT) {
            while ((unsigned)node < (unsigned)RT_SENT) {
                if (COUNT) cnt[0]++;
                const float4 *N = (MULTI ? mnodes : S.nodes) + 4 * (size_t)node;
                float4 n0 = __ldg(N), n1 = __ldg(N + 1), n2 = __ldg(N + 2);
                int4 cc = __ldg(reinterpret_cast<const int4 *>(N + 3));
                float c0lox = __fmaf_rn(n0.x, idx, lx), c0hix = __fmaf_rn(n0.y, idx, hx);
                float c0loy = __fmaf_rn(n0.z, idy, ly), c0hiy = __fmaf_rn(n0.w, idy, hy);
                float c0loz = __fmaf_rn(n2.x, idz, lz), c0hiz = __fmaf_rn(n2.y, idz, hz);
                float c1lox = __fmaf_rn(n1.x, idx, lx), c1hix = __fmaf_rn(n1.y, idx, hx);
                float c1loy = __fmaf_rn(n1.z, idy, ly), c1hiy = __fmaf_rn(n1.w, idy, hy);
                float c1loz = __fmaf_rn(n2.z, idz, lz), c1hiz = __fmaf_rn(n2.w, idz, hz);
                float c0min = rt_max4(fminf(c0lox, c0hix), fminf(c0loy, c0hiy), fminf(c0loz, c0hiz), tmin);
                float c0max = rt_min4(fmaxf(c0lox, c0hix), fmaxf(c0loy, c0hiy), fmaxf(c0loz, c0hiz), hit_t);
                float c1min = rt_max4(fminf(c1lox, c1hix), fminf(c1loy, c1hiy), fminf(c1loz, c1hiz), tmin);
                float c1max = rt_min4(fmaxf(c1lox, c1hix), fmaxf(c1loy, c1hiy), fmaxf(c1loz, c1hiz), hit_t);
                bool t0 = c0min <= c0max, t1 = c1min <= c1max;
                if (!t0 && !t1) {
                    SPOP(node);
                } else {
                    node = t0 ? cc.x : cc.y;
                    if (t0 && t1) {
                        int far = cc.y;
                        if (c1min < c0min) { far = node; node = cc.y; }
                        if (sp < RT_STACK) SPUSH(far);
                        else dropped = true;   // unreachable: the build bounds the depth
                    }
                }
                // first leaf found: postpone it and keep traversing
                if (node < 0 && leaf >= 0) { leaf = node; SPOP(node); }
                if (!__any_sync(__activemask(), leaf >= 0)) break;
            }
            // ---- postponed leaves
            while (leaf < 0) {
                int v = ~leaf;
                int first = v >> 3, cl = (v & 7) + 1;
                for (int i = 0; i < cl; i++) {
                    if (COUNT) cnt[1]++;
                    const float4 *T = (MULTI ? mtris : S.tri_slots) + 3 * (size_t)(first + i);
                    float4 a = __ldg(T), b = __ldg(T + 1), c = __ldg(T + 2);
                    float t, u, w;
                    if (mt_test(a, b, c, v3(ox, oy, oz), v3(dx, dy, dz), tmin, hit_t, t, u, w)) {
                        hit_t = t; hu = u; hv = w; hprim = __float_as_int(a.w);
                        if (ANY) { node = RT_SENT; break; }
                    }
                }
                if (ANY && node == RT_SENT && hprim >= 0) { leaf = 0; break; }
                leaf = node;
                if (node < 0) SPOP(node);
            }
            if (__popc(__activemask()) < RT_FETCH_THRESHOLD) break;
        }
        // ---- finished rays: analytic spheres, then store
        if (node == RT_SENT && has_ray) {
            if (!(ANY && hprim >= 0)) {
                const int nsph = MULTI ? ms->n_spheres : S.n_spheres;
                const DevSphere *sph = MULTI ? ms->spheres : S.spheres;
                for (int si = 0; si < nsph; si++) {
                    float t;
                    if (analytic_test(sph[si], v3(ox, oy, oz), v3(dx, dy, dz), tmin, hit_t, t)) {
                        hit_t = t; hu = 0.f; hv = 0.f; hprim = -si - 2;
                        if (ANY) break;
                    }
                }
            }
            if (ANY) P.W.occl[slot] = hprim != -1 ? 1 : 0;
            else {
                P.W.hit[slot] = make_float4(hit_t, hu, hv, __int_as_float(hprim));
                if (MULTI) classify_hit(P, *ms, C, slot, hprim, n);
                else classify_hit(P, S, C, slot, hprim, n);
            }
            has_ray = false;
        }
    }
    if (COUNT) {
        for (int off = 16; off > 0; off >>= 1) {
            cnt[0] += __shfl_down_sync(0xffffffffu, cnt[0], off);
            cnt[1] += __shfl_down_sync(0xffffffffu, cnt[1], off);
        }
        if (lane == 0) {
            atomicAdd(&P.stats[ANY ? 5 : 3], (unsigned long long)cnt[0]);
            atomicAdd(&P.stats[ANY ? 6 : 4], (unsigned long long)cnt[1]);
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&P.stats[ANY ? 1 : 0], (unsigned long long)n);
    if (dropped && P.limit_flag) atomicOr(P.limit_flag, RT_LIM_STACK2);
#undef SPUSH
#undef SPOP
}

// ---------------------------------------------------------------- 4-wide traversal
// Persistent traversal of the 4-wide BVH (rt_bvh.h), built like k_trace:
// while-while node and leaf phases, postponed leaves, lanes that finish a
// ray take the next one from the queue.  A node visit tests its four child
// boxes with the BVH2's fused slab test and guards, sorts the hit children
// by entry distance (4-key network on (distance bits | slot)), descends into
// the nearest and pushes the others far to near.  Half as many dependent
// node fetches per ray as the binary tree, for about twice the arithmetic
// per fetch.  The boxes are the BVH2's, so the same triangles are tested
// against the same rays: closest hits and occlusion equal the BVH2's (a tie
// at exactly equal distance may name another triangle).
#ifndef RT_STACK4
#define RT_STACK4 96
#endif
#ifndef RT_TRACE4_MINB
#define RT_TRACE4_MINB 8
#endif

// Key of child `slot` of a 4-wide node: its near and far planes per axis
// (chosen by the ray's direction signs) through the BVH2's guarded slab
// test.  A hit child's key orders by entry distance; a miss sorts last.
__device__ __forceinline__ unsigned box4_key(float xn, float xf, float yn, float yf, float zn, float zf, unsigned slot,
                                             float idx, float idy, float idz, float nx, float fx, float ny, float fy,
                                             float nz, float fz, float tmin, float tmax)
{
    const float tn = rt_max3(__fmaf_rn(xn, idx, nx), __fmaf_rn(yn, idy, ny), fmaxf(__fmaf_rn(zn, idz, nz), tmin));
    const float tf = rt_min3(__fmaf_rn(xf, idx, fx), __fmaf_rn(yf, idy, fy), fminf(__fmaf_rn(zf, idz, fz), tmax));
    return tn <= tf ? ((__float_as_uint(tn) & ~3u) | slot) : 0xffffffffu;
}

__device__ __forceinline__ int link4(const int4 &cc, unsigned key)
{
    const unsigned s = key & 3u;
    return s == 0 ? cc.x : s == 1 ? cc.y : s == 2 ? cc.z : cc.w;
}

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(128, RT_TRACE4_MINB) k_trace4(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene S = P.S;
    RoundCounters *C = &P.W.cnt[round];
    const int n = ANY ? C->shadow : C->closest;
    int *wc = ANY ? &C->wc_shadow : &C->wc_closest;
    const int *queue = ANY ? P.W.q_shadow : P.W.q_closest;
    const int lane = threadIdx.x & 31;
    int cnt[2] = {0, 0};

    int stack[RT_STACK4];
    int sp = 0;
    int node = RT_SENT, leaf = 0;
    int slot = -1;
    bool has_ray = false;
    float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, idx = 0, idy = 0, idz = 0;
    float tmin = 0, hit_t = 0, hu = 0, hv = 0;
    float nx = 0, fx = 0, ny = 0, fy = 0, nz = 0, fz = 0;   // near / far plane offsets (slab_guard)
    int sx = 0, sy = 0, sz = 0;                             // 1: the axis's near plane is the box's upper one
    int hprim = -1;
    bool dropped = false;   // a push found the stack full

    for (;;) {
        // ---- fetch rays for lanes whose ray is finished
        const bool terminated = (node == RT_SENT);
        const unsigned mterm = __ballot_sync(0xffffffffu, terminated);
        const int nterm = __popc(mterm);
        int base = 0;
        if (nterm) {
            const int leader = __ffs(mterm) - 1;
            if (lane == leader) base = atomicAdd(wc, nterm);
            base = __shfl_sync(0xffffffffu, base, leader);
        }
        if (terminated) {
            int q = base + __popc(mterm & ((1u << lane) - 1));
            has_ray = q < n;
            if (has_ray) {
                slot = queue[q];
                float4 o4 = ANY ? P.W.sh_o[slot] : P.W.ray_o[slot];
                float4 d4 = ANY ? P.W.sh_d[slot] : P.W.ray_d[slot];
                ox = o4.x; oy = o4.y; oz = o4.z; dx = d4.x; dy = d4.y; dz = d4.z;
                tmin = adapt_mint(v3(ox, oy, oz), o4.w);
                hit_t = d4.w;
                hprim = -1;
                const float eps = 1e-20f;
                idx = 1.0f / (fabsf(dx) > eps ? dx : copysignf(eps, dx));
                idy = 1.0f / (fabsf(dy) > eps ? dy : copysignf(eps, dy));
                idz = 1.0f / (fabsf(dz) > eps ? dz : copysignf(eps, dz));
                const float oox = ox * idx, ooy = oy * idy, ooz = oz * idz;
                nx = -(oox + slab_guard(oox)); fx = -(oox - slab_guard(oox));
                ny = -(ooy + slab_guard(ooy)); fy = -(ooy - slab_guard(ooy));
                nz = -(ooz + slab_guard(ooz)); fz = -(ooz - slab_guard(ooz));
                sx = idx < 0.f; sy = idy < 0.f; sz = idz < 0.f;
                sp = 0;
                stack[sp++] = RT_SENT;
                leaf = 0;
                node = (S.n_nodes4 > 0 && !(hit_t < tmin)) ? 0 : RT_SENT;
            }
        }
        if (!__any_sync(0xffffffffu, has_ray)) break;

        // ---- traversal
        while (node != RT_SENT) {
            while ((unsigned)node < (unsigned)RT_SENT) {
                if (COUNT) cnt[0]++;
                const float4 *N = S.nodes4 + 8 * (size_t)node;
                // near / far plane rows of each axis by the ray's direction sign
                const float4 xn = __ldg(N + sx), xf = __ldg(N + 1 - sx);
                const float4 yn = __ldg(N + 2 + sy), yf = __ldg(N + 3 - sy);
                const float4 zn = __ldg(N + 4 + sz), zf = __ldg(N + 5 - sz);
                const int4 cc = __ldg(reinterpret_cast<const int4 *>(N + 6));
                unsigned k0 = box4_key(xn.x, xf.x, yn.x, yf.x, zn.x, zf.x, 0u, idx, idy, idz, nx, fx, ny, fy, nz, fz, tmin, hit_t);
                unsigned k1 = box4_key(xn.y, xf.y, yn.y, yf.y, zn.y, zf.y, 1u, idx, idy, idz, nx, fx, ny, fy, nz, fz, tmin, hit_t);
                unsigned k2 = box4_key(xn.z, xf.z, yn.z, yf.z, zn.z, zf.z, 2u, idx, idy, idz, nx, fx, ny, fy, nz, fz, tmin, hit_t);
                unsigned k3 = box4_key(xn.w, xf.w, yn.w, yf.w, zn.w, zf.w, 3u, idx, idy, idz, nx, fx, ny, fy, nz, fz, tmin, hit_t);
#define RT_CSWAP(a, b)                  \
    do {                                \
        const unsigned t_ = umin(a, b); \
        b = umax(a, b);                 \
        a = t_;                         \
    } while (0)
                RT_CSWAP(k0, k1); RT_CSWAP(k2, k3); RT_CSWAP(k0, k2); RT_CSWAP(k1, k3); RT_CSWAP(k1, k2);
#undef RT_CSWAP
                if (k0 == 0xffffffffu) {
                    node = stack[--sp];
                } else {
                    // push the farther hits, farthest first
                    if (k3 != 0xffffffffu) { if (sp < RT_STACK4) stack[sp++] = link4(cc, k3); else dropped = true; }
                    if (k2 != 0xffffffffu) { if (sp < RT_STACK4) stack[sp++] = link4(cc, k2); else dropped = true; }
                    if (k1 != 0xffffffffu) { if (sp < RT_STACK4) stack[sp++] = link4(cc, k1); else dropped = true; }
                    node = link4(cc, k0);
                }
                // first leaf found: postpone it and keep traversing
                if (node < 0 && leaf >= 0) { leaf = node; node = stack[--sp]; }
                if (!__any_sync(__activemask(), leaf >= 0)) break;
            }
            // ---- postponed leaves
            while (leaf < 0) {
                int v = ~leaf;
                int first = v >> 3, cl = (v & 7) + 1;
                for (int i = 0; i < cl; i++) {
                    if (COUNT) cnt[1]++;
                    const float4 *T = S.tri_slots + 3 * (size_t)(first + i);
                    float4 a = __ldg(T), b = __ldg(T + 1), c = __ldg(T + 2);
                    float t, u, w;
                    if (mt_test(a, b, c, v3(ox, oy, oz), v3(dx, dy, dz), tmin, hit_t, t, u, w)) {
                        hit_t = t; hu = u; hv = w; hprim = __float_as_int(a.w);
                        if (ANY) { node = RT_SENT; break; }
                    }
                }
                if (ANY && node == RT_SENT && hprim >= 0) { leaf = 0; break; }
                leaf = node;
                if (node < 0) node = stack[--sp];
            }
            if (__popc(__activemask()) < RT_FETCH_THRESHOLD) break;
        }
        // ---- finished rays: analytic spheres, then store
        if (node == RT_SENT && has_ray) {
            if (!(ANY && hprim >= 0)) {
                for (int si = 0; si < S.n_spheres; si++) {
                    float t;
                    if (analytic_test(S.spheres[si], v3(ox, oy, oz), v3(dx, dy, dz), tmin, hit_t, t)) {
                        hit_t = t; hu = 0.f; hv = 0.f; hprim = -si - 2;
                        if (ANY) break;
                    }
                }
            }
            if (ANY) P.W.occl[slot] = hprim != -1 ? 1 : 0;
            else {
                P.W.hit[slot] = make_float4(hit_t, hu, hv, __int_as_float(hprim));
                classify_hit(P, S, C, slot, hprim, n);
            }
            has_ray = false;
        }
    }
    if (COUNT) {
        for (int off = 16; off > 0; off >>= 1) {
            cnt[0] += __shfl_down_sync(0xffffffffu, cnt[0], off);
            cnt[1] += __shfl_down_sync(0xffffffffu, cnt[1], off);
        }
        if (lane == 0) {
            atomicAdd(&P.stats[ANY ? 5 : 3], (unsigned long long)cnt[0]);
            atomicAdd(&P.stats[ANY ? 6 : 4], (unsigned long long)cnt[1]);
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&P.stats[ANY ? 1 : 0], (unsigned long long)n);
    if (dropped && P.limit_flag) atomicOr(P.limit_flag, RT_LIM_STACK4);
}

// ---------------------------------------------------------------- 8-wide traversal
// Persistent traversal of the compressed 8-wide BVH with node groups: one
// node visit tests its (up to) eight quantised child boxes and keeps the hit
// children as an 8-bit mask in the ray's octant order (bit k <-> slot
// k ^ octant, the build places children so that this order is roughly front
// to back).  The lane walks the group; when it descends into an internal
// child, the rest of the group is pushed as one stack entry
// (node << 8 | mask), so the stack grows by at most one entry per level.
// Node phase and leaf phase alternate warp-wide (while-while), and lanes
// whose ray finished take a new ray from the queue as in k_trace.
#define RT_WSTACK 32

// byte j of w as an exact float: the byte is placed in the mantissa of 2^23
// (one byte permute) and 2^23 subtracted, avoiding an integer conversion
__device__ __forceinline__ float byte_f(unsigned w, int j)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (unsigned)j)) - 8388608.0f;
}

__device__ __forceinline__ unsigned meta_byte(int4 w1, unsigned slot)
{
    unsigned w = slot < 4 ? (unsigned)w1.z : (unsigned)w1.w;
    return (w >> (8 * (slot & 3))) & 0xffu;
}

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(128, 8) k_trace8(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene S = P.S;
    RoundCounters *C = &P.W.cnt[round];
    const int n = ANY ? C->shadow : C->closest;
    int *wc = ANY ? &C->wc_shadow : &C->wc_closest;
    const int *queue = ANY ? P.W.q_shadow : P.W.q_closest;
    const int lane = threadIdx.x & 31;
    int cnt[2] = {0, 0};

    int stack[RT_WSTACK];
    int sp = 0;
    int gnode = 0, vnode = -1;      // current group's node; node to visit next (-1 none)
    unsigned gmask = 0, oct = 0;    // remaining hit children (octant order); ray octant
    int4 g1 = make_int4(0, 0, 0, 0);
    bool trav = false;              // a ray is being traversed
    int slot = -1;
    float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, idx = 0, idy = 0, idz = 0;
    float tmin = 0, hit_t = 0, hu = 0, hv = 0;
    float nx_ = 0, fx_ = 0, ny_ = 0, fy_ = 0, nz_ = 0, fz_ = 0;   // near / far plane offsets (slab_guard)
    int hprim = -1;
    bool negx = false, negy = false, negz = false;
    bool dropped = false;   // a push found the group stack full

    for (;;) {
        // ---- fetch rays for lanes whose ray is finished
        const bool idle = !trav;
        const unsigned midle = __ballot_sync(0xffffffffu, idle);
        const int nidle = __popc(midle);
        int base = 0;
        bool has_ray = trav;
        if (nidle) {
            const int leader = __ffs(midle) - 1;
            if (lane == leader) base = atomicAdd(wc, nidle);
            base = __shfl_sync(0xffffffffu, base, leader);
        }
        if (idle) {
            int q = base + __popc(midle & ((1u << lane) - 1));
            has_ray = q < n;
            if (has_ray) {
                slot = queue[q];
                float4 o4 = ANY ? P.W.sh_o[slot] : P.W.ray_o[slot];
                float4 d4 = ANY ? P.W.sh_d[slot] : P.W.ray_d[slot];
                ox = o4.x; oy = o4.y; oz = o4.z; dx = d4.x; dy = d4.y; dz = d4.z;
                tmin = adapt_mint(v3(ox, oy, oz), o4.w);
                hit_t = d4.w;
                hprim = -1;
                const float eps = 1e-20f;
                idx = 1.0f / (fabsf(dx) > eps ? dx : copysignf(eps, dx));
                idy = 1.0f / (fabsf(dy) > eps ? dy : copysignf(eps, dy));
                idz = 1.0f / (fabsf(dz) > eps ? dz : copysignf(eps, dz));
                const float oox = ox * idx, ooy = oy * idy, ooz = oz * idz;
                nx_ = -(oox + slab_guard(oox)); fx_ = -(oox - slab_guard(oox));
                ny_ = -(ooy + slab_guard(ooy)); fy_ = -(ooy - slab_guard(ooy));
                nz_ = -(ooz + slab_guard(ooz)); fz_ = -(ooz - slab_guard(ooz));
                negx = idx < 0.f; negy = idy < 0.f; negz = idz < 0.f;
                oct = (negx ? 1u : 0u) | (negy ? 2u : 0u) | (negz ? 4u : 0u);
                sp = 0;
                gmask = 0;
                vnode = (S.n_wnodes > 0 && !(hit_t < tmin)) ? 0 : -1;
                trav = true;
            }
        }
        if (!__any_sync(0xffffffffu, has_ray)) break;

        while (trav) {
            // ---- node phase: visit internal nodes until the next item is a leaf
            for (;;) {
                if (vnode < 0) {
                    if (gmask == 0) {
                        if (sp == 0) { trav = false; break; }
                        const int e = stack[--sp];
                        gnode = e >> 8;
                        gmask = (unsigned)e & 0xffu;
                        g1 = __ldg(reinterpret_cast<const int4 *>(S.wnodes + 5 * (size_t)gnode + 1));
                    }
                    const unsigned m = meta_byte(g1, (unsigned)(__ffs(gmask) - 1) ^ oct);
                    if ((m >> 5) != 7u) break;             // a leaf comes next
                    gmask &= gmask - 1;
                    if (gmask) {
                        if (sp < RT_WSTACK) stack[sp++] = (gnode << 8) | (int)gmask;
                        else dropped = true;   // unreachable: deeper trees are not uploaded
                    }
                    vnode = g1.x + (int)(m & 31u);
                }
                if (COUNT) cnt[0]++;
                const float4 *N = S.wnodes + 5 * (size_t)vnode;
                float4 w0 = __ldg(N);
                int4 w1 = __ldg(reinterpret_cast<const int4 *>(N + 1));
                uint4 w2 = __ldg(reinterpret_cast<const uint4 *>(N + 2));
                uint4 w3 = __ldg(reinterpret_cast<const uint4 *>(N + 3));
                uint4 w4 = __ldg(reinterpret_cast<const uint4 *>(N + 4));
                unsigned eb = __float_as_uint(w0.w);
                float sx = __uint_as_float((eb & 0xffu) << 23);
                float sy = __uint_as_float(((eb >> 8) & 0xffu) << 23);
                float sz = __uint_as_float(((eb >> 16) & 0xffu) << 23);
                float anx = __fmaf_rn(w0.x, idx, nx_), any_ = __fmaf_rn(w0.y, idy, ny_), anz = __fmaf_rn(w0.z, idz, nz_);
                float afx = __fmaf_rn(w0.x, idx, fx_), afy = __fmaf_rn(w0.y, idy, fy_), afz = __fmaf_rn(w0.z, idz, fz_);
                float kx = sx * idx, ky = sy * idy, kz = sz * idz;
                // near/far planes per axis from the direction signs
                uint2 qxn = negx ? make_uint2(w3.z, w3.w) : make_uint2(w2.x, w2.y);
                uint2 qxf = negx ? make_uint2(w2.x, w2.y) : make_uint2(w3.z, w3.w);
                uint2 qyn = negy ? make_uint2(w4.x, w4.y) : make_uint2(w2.z, w2.w);
                uint2 qyf = negy ? make_uint2(w2.z, w2.w) : make_uint2(w4.x, w4.y);
                uint2 qzn = negz ? make_uint2(w4.z, w4.w) : make_uint2(w3.x, w3.y);
                uint2 qzf = negz ? make_uint2(w3.x, w3.y) : make_uint2(w4.z, w4.w);
                unsigned hm = 0;
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    unsigned wxn = i < 4 ? qxn.x : qxn.y, wxf = i < 4 ? qxf.x : qxf.y;
                    unsigned wyn = i < 4 ? qyn.x : qyn.y, wyf = i < 4 ? qyf.x : qyf.y;
                    unsigned wzn = i < 4 ? qzn.x : qzn.y, wzf = i < 4 ? qzf.x : qzf.y;
                    float tnx = __fmaf_rn(byte_f(wxn, i & 3), kx, anx), tfx = __fmaf_rn(byte_f(wxf, i & 3), kx, afx);
                    float tny = __fmaf_rn(byte_f(wyn, i & 3), ky, any_), tfy = __fmaf_rn(byte_f(wyf, i & 3), ky, afy);
                    float tnz = __fmaf_rn(byte_f(wzn, i & 3), kz, anz), tfz = __fmaf_rn(byte_f(wzf, i & 3), kz, afz);
                    float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
                    float tf = fminf(fminf(tfx, tfy), fminf(tfz, hit_t));
                    if (tn <= tf) hm |= 1u << i;
                }
                // empty slots hold an inverted box (lo 255, hi 0) and meta 0, a
                // leaf of no triangles, should a degenerate node still report them
                // slot order -> octant order: bit k <- bit k ^ oct
                if (oct & 1u) hm = ((hm & 0x55u) << 1) | ((hm >> 1) & 0x55u);
                if (oct & 2u) hm = ((hm & 0x33u) << 2) | ((hm >> 2) & 0x33u);
                if (oct & 4u) hm = ((hm & 0x0fu) << 4) | ((hm >> 4) & 0x0fu);
                gnode = vnode;
                gmask = hm;
                g1 = w1;
                vnode = -1;
            }
            // ---- leaf phase: test the leaves at the front of the group
            while (trav && gmask) {
                const unsigned m = meta_byte(g1, (unsigned)(__ffs(gmask) - 1) ^ oct);
                if ((m >> 5) == 7u) break;
                gmask &= gmask - 1;
                const int first = g1.y + (int)(m & 31u), cl = (int)(m >> 5);
                bool done = false;
                for (int i = 0; i < cl; i++) {
                    if (COUNT) cnt[1]++;
                    const float4 *T = S.wtri + 3 * (size_t)(first + i);
                    float4 a = __ldg(T), b = __ldg(T + 1), c = __ldg(T + 2);
                    float t, u, w;
                    if (mt_test(a, b, c, v3(ox, oy, oz), v3(dx, dy, dz), tmin, hit_t, t, u, w)) {
                        hit_t = t; hu = u; hv = w; hprim = __float_as_int(a.w);
                        if (ANY) { done = true; break; }
                    }
                }
                if (done) { gmask = 0; sp = 0; vnode = -1; trav = false; }
            }
            if (__popc(__activemask()) < RT_FETCH_THRESHOLD) break;
        }
        if (!trav && has_ray) {
            if (!(ANY && hprim >= 0)) {
                for (int si = 0; si < S.n_spheres; si++) {
                    float t;
                    if (analytic_test(S.spheres[si], v3(ox, oy, oz), v3(dx, dy, dz), tmin, hit_t, t)) {
                        hit_t = t; hu = 0.f; hv = 0.f; hprim = -si - 2;
                        if (ANY) break;
                    }
                }
            }
            if (ANY) P.W.occl[slot] = hprim != -1 ? 1 : 0;
            else {
                P.W.hit[slot] = make_float4(hit_t, hu, hv, __int_as_float(hprim));
                classify_hit(P, S, C, slot, hprim, n);
            }
            has_ray = false;
        }
    }
    if (COUNT) {
        for (int off = 16; off > 0; off >>= 1) {
            cnt[0] += __shfl_down_sync(0xffffffffu, cnt[0], off);
            cnt[1] += __shfl_down_sync(0xffffffffu, cnt[1], off);
        }
        if (lane == 0) {
            atomicAdd(&P.stats[ANY ? 5 : 3], (unsigned long long)cnt[0]);
            atomicAdd(&P.stats[ANY ? 6 : 4], (unsigned long long)cnt[1]);
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&P.stats[ANY ? 1 : 0], (unsigned long long)n);
    if (dropped && P.limit_flag) atomicOr(P.limit_flag, RT_LIM_STACK8);
}

// rays of the rt_trace test hook into the wavefront buffers, and back
__global__ void k_rays_in(const rt_ray *rays, int n, RenderParams P, int anyhit)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rt_ray r = rays[i];
    float4 o = make_float4(r.o[0], r.o[1], r.o[2], r.mint), d = make_float4(r.d[0], r.d[1], r.d[2], r.maxt);
    if (anyhit) { P.W.sh_o[i] = o; P.W.sh_d[i] = d; P.W.q_shadow[i] = i; }
    else { P.W.ray_o[i] = o; P.W.ray_d[i] = d; P.W.q_closest[i] = i; }
    if (i == 0) {
        RoundCounters c;
        memset(&c, 0, sizeof(c));
        c.closest = anyhit ? 0 : n;
        c.shadow = anyhit ? n : 0;
        P.W.cnt[0] = c;
    }
}
__global__ void k_hits_out(RenderParams P, int n, int anyhit, rt_hit *hits)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rt_hit h;
    if (anyhit) {
        h.t = 0.f; h.u = 0.f; h.v = 0.f; h.prim = P.W.occl[i] ? 0 : -1;
    } else {
        float4 v = P.W.hit[i];
        int prim = __float_as_int(v.w);
        h.prim = prim;
        h.t = prim != -1 ? v.x : 0.f;
        h.u = prim != -1 ? v.y : 0.f;
        h.v = prim != -1 ? v.z : 0.f;
    }
    hits[i] = h;
}

// ---------------------------------------------------------------- PathTracingMIS vertex
// The per-vertex loop body of PathTracingMIS::li (PathTracingMIS.cpp:54-259)
// runs as three wavefront stages after the traces of a round:
//   k_trace<closest>  sorts each traced path by what its ray hit (classify_hit);
//   k_pt_finish       ends the paths whose ray missed or hit a surface without
//                     a BSDF, and those that ended in shading with a light
//                     sample pending: light sample if unoccluded (:140), the
//                     MIS-weighted emission the BSDF-sampled ray found
//                     (:173-220);
//   k_pt_shade<T>     for paths that hit a surface of BSDF type T: first
//                     finishes the previous vertex as above, then throughput /
//                     eta update (:222-223) and Russian roulette (:225-253),
//                     then shades the new vertex: emission at depth 0
//                     (:73-74), light sample (:121-153), BSDF sample (:156-168),
//                     emitting the shadow ray and the next closest-hit ray.
__device__ __forceinline__ void pt_finish_path(const RenderParams &P, const DevScene &S, int slot)
{
    const int env = S.env_light;
    int flags = P.W.flags[slot];
    C3 L = rgb(P.W.rad[slot]);
    if (flags & F_FIRST) {
        // camera ray: the environment if it missed; a surface without a
        // BSDF ends the path (PathTracingMIS.cpp:60-70)
        float4 hv = P.W.hit[slot];
        if (__float_as_int(hv.w) == -1 && env >= 0) L = L + env_le(S.lights[env], xyz(P.W.ray_d[slot]));
    } else {
        if ((flags & F_NEE) && !P.W.occl[slot]) L = L + rgb(P.W.nee[slot]);
        if (!(flags & F_END)) {
            float4 hv = P.W.hit[slot];
            Hit h; h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_int(hv.w);
            float4 ro = P.W.ray_o[slot], rd = P.W.ray_d[slot];
            V3 o = xyz(ro), d = xyz(rd);
            int caught = -1;
            C3 Le = cfill(0.f);
            V3 pt = v3(0, 0, 0), nn = v3(0, 0, 0);
            if (h.prim != -1) {
                int nl = prim_light(S, h.prim);
                if (nl >= 0) {
                    Frame fr = hit_frame(S, h, o, d);
                    pt = fr.p; nn = fr.n;
                    caught = nl;
                    Le = area_le(S, nl, -d, fr.n);
                }
            } else if (env >= 0) {
                caught = env;
                Le = env_le(S.lights[env], d);
            }
            if (caught >= 0) {
                C3 T = rgb(P.W.tp[slot]);
                float4 bsv = P.W.bs[slot];
                float pl = (flags & F_DELTA) ? 0.f : light_pdf(S, caught, o, pt, nn, d);
                float w = power_heuristic(bsv.w, pl);
                L = L + ((T * Le) * rgb(bsv)) * w;
            }
        }
    }
    P.W.out[slot] = f4c(L, 0.f);
    P.W.flags[slot] = (flags & ~(F_FIRST | F_NEE)) | F_DONE;
}
// MULTI: a multi-scene batch, each path read against its own scene
template <bool MULTI = false>
__global__ void __launch_bounds__(128) k_pt_finish(RenderParams P, int round)
{
    round = cur_round(P, round);
    RoundCounters *C = &P.W.cnt[round];
    const int nf = C->fin, n = nf + C->end;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int slot = idx < nf ? P.W.q_fin[idx] : P.W.q_end[idx - nf];
        if (MULTI) pt_finish_path(P, P.scenes[P.W.sid[slot]], slot);
        else pt_finish_path(P, P.S, slot);
    }
}

// The BSDF functions of one shading queue (bsdf_queue), with the TwoSides
// mirroring of bsdf_eval/bsdf_pdf/bsdf_sample.  Queue RT_QUEUE_DELTA holds
// the smooth BSDFs, whose eval and pdf are zero; RT_QUEUE_MIXED holds every
// type and dispatches at run time.
template <int BT>
__device__ __forceinline__ C3 bsdf_eval_t(const DevBsdf &b, V3 wi, V3 wo)
{
    if (BT == RT_QUEUE_MIXED) return bsdf_eval(b, wi, wo);
    if (BT == RT_QUEUE_DELTA) return cfill(0.f);
    if (b.two_sided && !(wi.z > 0.f)) { wi.z = -wi.z; wo.z = -wo.z; }
    if (BT == 0) return diffuse_eval(b.albedo, wi, wo);
    if (BT == 1) return rc_eval(b, wi, wo);
    if (BT == 2) return rd_eval(b, wi, wo);
    if (BT == 3) return sl_eval(b, wi, wo);
    return ly_eval(b, wi, wo);
}
template <int BT>
__device__ __forceinline__ float bsdf_pdf_t(const DevBsdf &b, V3 wi, V3 wo)
{
    if (BT == RT_QUEUE_MIXED) return bsdf_pdf(b, wi, wo);
    if (BT == RT_QUEUE_DELTA) return 0.f;
    if (b.two_sided && !(wi.z > 0.f)) { wi.z = -wi.z; wo.z = -wo.z; }
    if (BT == 0) return diffuse_pdf(wi, wo);
    if (BT == 1) return rc_pdf(b, wi, wo);
    if (BT == 2) return rd_pdf(b, wi, wo);
    if (BT == 3) return sl_pdf(b, wi, wo);
    return ly_pdf(b, wi, wo);
}
template <int BT>
__device__ __forceinline__ C3 bsdf_sample1_t(const DevBsdf &b, BsdfRec &r, V2 s, uint64_t aux_key)
{
    if (BT == 0) return diffuse_sample(b.albedo, r, s);
    if (BT == 1) return rc_sample(b, r, s);
    if (BT == 2) return rd_sample(b, r, s);
    if (BT == 3) return sl_sample(b, r, s);
    if (BT == 4) return ly_sample(b, r, s, aux_key);
    if (b.type == RT_BSDF_DIELECTRIC) return dl_sample(b, r, s);
    if (b.type == RT_BSDF_CONDUCTOR) return cd_sample(b, r);
    if (b.type == RT_BSDF_SHEET_DIELECTRIC) return sd_sample(b, r, s);
    return mr_sample(r);
}
template <int BT>
__device__ __forceinline__ C3 bsdf_sample_t(const DevBsdf &b, BsdfRec &r, V2 s, uint64_t aux_key)
{
    if (BT == RT_QUEUE_MIXED) return bsdf_sample(b, r, s, aux_key);
    if (b.two_sided && !(r.wi.z > 0.f)) {
        r.wi.z = -r.wi.z;
        C3 res = bsdf_sample1_t<BT>(b, r, s, aux_key);
        r.wi.z = -r.wi.z;
        r.wo.z = -r.wo.z;
        return res;
    }
    return bsdf_sample1_t<BT>(b, r, s, aux_key);
}

#ifndef RT_SHADE_MINB
#define RT_SHADE_MINB 8
#endif
#ifndef RT_SHADE_GRID
#define RT_SHADE_GRID 16
#endif
// The all-lights strategy of PathTracingMIS::li (PathTracingMIS.cpp:80-117):
// one sample of every light in turn, each with its own shadow ray (traced
// here, any hit through the binary tree and the analytic shapes, as
// Integrator::sampleOneLight does) and its MIS weight against the BSDF,
// added to L in light order.  Out of line so that the shading kernels'
// registers on the one-light path stay as they are.
template <int BT>
__device__ __noinline__ C3 pt_all_lights(const DevScene &S, const DevBsdf &B, const Frame &fr, V3 d, C3 T, C3 L,
                                         Pcg32 &rng)
{
    for (int l = 0; l < S.n_lights; l++) {
        const V2 s = next2d(rng);
        LightRec li;
        light_sample(S, l, fr.p, s, li);
        C3 value = cfill(0.f);
        if (li.pdf > 0 && lum(li.intensity) > 0) {
            Hit sh;
            if (!trace_ray<true>(S, fr.p, li.to_light, RT_EPSILON, li.distance - RT_EPSILON, sh))
                value = li.intensity / li.pdf;
        }
        if (!iszero(value)) {
            V3 wi = to_local(fr, li.to_light), wo = to_local(fr, -d);
            float ct = fabsf(wi.z);
            float bp = li.delta ? 0.f : bsdf_pdf_t<BT>(B, wi, wo);
            float w = power_heuristic(li.pdf, bp);
            L = L + (((T * value) * bsdf_eval_t<BT>(B, wi, wo)) * ct) * w;
        }
    }
    return L;
}

template <int BT, bool ALL = false>
__device__ __forceinline__ void pt_shade_path(const RenderParams &P, const DevScene &S, int slot, bool &push_end,
                                              bool &push_closest, bool &push_shadow)
{
    Pcg32 rng = P.W.rng[slot];
    float4 tpv = P.W.tp[slot];
    C3 T = rgb(tpv);
    float eta = tpv.w;
    float4 radv = P.W.rad[slot];
    C3 L = rgb(radv);
    int depth = __float_as_int(radv.w);
    int flags = P.W.flags[slot];
    float4 ro = P.W.ray_o[slot], rd = P.W.ray_d[slot];
    V3 o = xyz(ro), d = xyz(rd);
    float4 hv = P.W.hit[slot];
    Hit h; h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_int(hv.w);
    Frame fr = hit_frame(S, h, o, d);
    // the mixed queue's BSDF is a copy with its textures applied at
    // the hit; the sorted queues read the scene's (untextured) BSDF
    DevBsdf Bl;
    if (BT == RT_QUEUE_MIXED) {
        Bl = S.bsdfs[prim_bsdf(S, h.prim)];
        if (Bl.textured) tex_apply(S, Bl, hit_uv(S, h, o, d));
    }
    const DevBsdf &B = BT == RT_QUEUE_MIXED ? Bl : S.bsdfs[prim_bsdf(S, h.prim)];
    bool done = false;
    // finish the previous vertex (its light sample and the emission
    // its BSDF-sampled ray found), update throughput, roulette
    if (flags & F_FIRST) {
        flags &= ~F_FIRST;
        if (depth >= P.max_depth) done = true;
    } else {
        if ((flags & F_NEE) && !P.W.occl[slot]) L = L + rgb(P.W.nee[slot]);
        flags &= ~F_NEE;
        float4 bsv = P.W.bs[slot];
        C3 f = rgb(bsv);
        int nl = prim_light(S, h.prim);
        if (nl >= 0) {
            C3 Le = area_le(S, nl, -d, fr.n);
            float pl = (flags & F_DELTA) ? 0.f : light_pdf(S, nl, o, fr.p, fr.n, d);
            float w = power_heuristic(bsv.w, pl);
            L = L + ((T * Le) * f) * w;
        }
        T = T * f;
        eta *= P.W.rel_eta[slot];
        if (depth >= P.min_depth) {
            float stop = smin(0.95f, lum(T) * eta * eta);
            if (next1d(rng) < stop) T = T / stop;
            else done = true;
        }
        if (!done) {
            depth++;
            if (depth >= P.max_depth) done = true;
        }
    }
    if (done) {
        P.W.out[slot] = f4c(L, 0.f);
        P.W.flags[slot] = flags | F_DONE;
        P.W.rng[slot] = rng;
    } else {
    // emission of a light hit by the camera ray (PathTracingMIS.cpp:73-74)
    if (depth == 0) {
        int hl = prim_light(S, h.prim);
        if (hl >= 0) L = L + T * area_le(S, hl, -d, fr.n);
    }
    // light sampling (Integrator::sampleLightDirect, Integrator.cpp:176-218)
    if (ALL) {
        L = pt_all_lights<BT>(S, B, fr, d, T, L, rng);
    } else {
    V2 s = next2d(rng);
    if (S.n_lights > 0) {
        float lw;
        int li_idx = cdf_sample_reuse(S.light_cdf, S.n_lights + 1, s.x, lw);
        LightRec li;
        light_sample(S, li_idx, fr.p, s, li);
        if (li.pdf > 0 && lum(li.intensity) > 0) {
            C3 value = (li.intensity / li.pdf) / lw;
            li.pdf *= lw;
            if (!iszero(value)) {
                V3 wi = to_local(fr, li.to_light), wo = to_local(fr, -d);
                float ct = fabsf(wi.z);
                // a delta light's sample takes a zero BSDF pdf (PathTracingMIS.cpp:136)
                float bp = li.delta ? 0.f : bsdf_pdf_t<BT>(B, wi, wo);
                float w = power_heuristic(li.pdf, bp);
                C3 contrib = (((T * value) * bsdf_eval_t<BT>(B, wi, wo)) * ct) * w;
                // The reference traces the shadow ray before it weighs the
                // sample by the BSDF (Integrator.cpp:176-218); the ray draws
                // no random numbers, so when the weighted contribution is
                // exactly zero (e.g. a light direction below an opaque
                // surface) its outcome cannot change L and it is not traced.
                if (contrib.r != 0.f || contrib.g != 0.f || contrib.b != 0.f) {
                    P.W.nee[slot] = f4c(contrib, 0.f);
                    P.W.sh_o[slot] = f4(fr.p, RT_EPSILON);
                    P.W.sh_d[slot] = f4(li.to_light, li.distance - RT_EPSILON);
                    flags |= F_NEE;
                    push_shadow = true;
                }
            }
        }
    }
    }
    // BSDF sampling
    BsdfRec r;
    r.wi = to_local(fr, -d); r.wo = v3(0, 0, 0);
    r.type = BT_ALL; r.rel_eta = 1.f; r.pdf = -1.f;
    V2 u = next2d(rng);
    C3 f = bsdf_sample_t<BT>(B, r, u, rng.state);
    if (iszero(f)) {
        if (flags & F_NEE) {
            flags |= F_END;   // the light sample still needs its shadow ray
            push_end = true;
        } else {
            flags |= F_DONE;
            P.W.out[slot] = f4c(L, 0.f);
        }
    } else {
        P.W.ray_o[slot] = f4(fr.p, RT_EPSILON);
        P.W.ray_d[slot] = f4(to_world(fr, r.wo), RT_MAX_REAL);
        P.W.bs[slot] = f4c(f, r.pdf);
        P.W.rel_eta[slot] = r.rel_eta;
        if (r.type & BT_DELTA) flags |= F_DELTA; else flags &= ~F_DELTA;
        push_closest = true;
    }
    P.W.rad[slot] = f4c(L, __int_as_float(depth));
    P.W.tp[slot] = f4c(T, eta);
    P.W.rng[slot] = rng;
    P.W.flags[slot] = flags;
    }
}
// MULTI: a multi-scene batch, each path shaded against its own scene.
// ALL: the all-lights strategy (its own instantiations, so that the
// one-light kernels are compiled as without it)
template <int BT, bool MULTI = false, bool ALL = false>
__global__ void __launch_bounds__(128, RT_SHADE_MINB) k_pt_shade(RenderParams P, int round)
{
    round = cur_round(P, round);
    RoundCounters *C = &P.W.cnt[round];
    RoundCounters *Cout = &P.W.cnt[round + 1];
    const int n = BT == RT_QUEUE_MIXED ? C->mixed : C->mat[BT];
    const int *qin = BT == RT_QUEUE_MIXED ? P.W.q_mixed : P.W.q_mat[BT];
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    int stride = gridDim.x * blockDim.x;
    int iters = (n + stride - 1) / stride;
    for (int it = 0; it < iters; it++, idx += stride) {
        bool valid = idx < n;
        int slot = valid ? qin[idx] : 0;
        bool push_end = false, push_closest = false, push_shadow = false;
        if (valid) {
            if (MULTI) pt_shade_path<BT, ALL>(P, P.scenes[P.W.sid[slot]], slot, push_end, push_closest, push_shadow);
            else pt_shade_path<BT, ALL>(P, P.S, slot, push_end, push_closest, push_shadow);
        }
        q_push(P.W.q_end, &Cout->end, slot, push_end);
        q_push(P.W.q_closest, &Cout->closest, slot, push_closest);
        q_push(P.W.q_shadow, &Cout->shadow, slot, push_shadow);
    }
}

// The shading kernels of one round for the shading queues in `types` (bit
// q: queue q in use), the all-lights instantiations for that strategy
static void launch_shades(int types, const RenderParams &P, int r, int blocks, cudaStream_t st)
{
    if (P.all_lights) {
        if (types & 1) k_pt_shade<0, false, true><<<blocks, 128, 0, st>>>(P, r);
        if (types & 2) k_pt_shade<1, false, true><<<blocks, 128, 0, st>>>(P, r);
        if (types & 4) k_pt_shade<2, false, true><<<blocks, 128, 0, st>>>(P, r);
        if (types & 8) k_pt_shade<3, false, true><<<blocks, 128, 0, st>>>(P, r);
        if (types & 16) k_pt_shade<4, false, true><<<blocks, 128, 0, st>>>(P, r);
        if (types & 32) k_pt_shade<5, false, true><<<blocks, 128, 0, st>>>(P, r);
        if (types & (1 << RT_QUEUE_MIXED)) k_pt_shade<RT_QUEUE_MIXED, false, true><<<blocks, 128, 0, st>>>(P, r);
    } else {
        if (types & 1) k_pt_shade<0><<<blocks, 128, 0, st>>>(P, r);
        if (types & 2) k_pt_shade<1><<<blocks, 128, 0, st>>>(P, r);
        if (types & 4) k_pt_shade<2><<<blocks, 128, 0, st>>>(P, r);
        if (types & 8) k_pt_shade<3><<<blocks, 128, 0, st>>>(P, r);
        if (types & 16) k_pt_shade<4><<<blocks, 128, 0, st>>>(P, r);
        if (types & 32) k_pt_shade<5><<<blocks, 128, 0, st>>>(P, r);
        if (types & (1 << RT_QUEUE_MIXED)) k_pt_shade<RT_QUEUE_MIXED><<<blocks, 128, 0, st>>>(P, r);
    }
}

// End of one graph-launched round: continue the round loop (the
// conditional node's body) while the next round has paths to trace or to
// finish, at most up to round max_rounds - 1, as the host-driven loop does.
// The loop ends after at most max_rounds bodies whatever the counters say.
__global__ void k_round_next(RenderParams P, cudaGraphConditionalHandle loop, int max_rounds)
{
    const int r = __ldcg(P.round_dev);
    const RoundCounters &nc = P.W.cnt[r + 1];
    const bool more = r + 1 < max_rounds && (__ldcg(&nc.closest) != 0 || __ldcg(&nc.end) != 0);
    if (more) P.round_dev[0] = r + 1;
    P.stats[7] += 1;   // rounds run, for the launch count
    cudaGraphSetConditional(loop, more ? 1u : 0u);
}

#include "rt_volpath.cuh"

// ---------------------------------------------------------------- film
// One thread per batch pixel: contributions in the order the reference's
// tile loop produces them (pixels row-major, samples in order), restricted
// to the 3x3 neighbourhood a box-filter splat can reach.
__global__ void k_film(RenderParams P, float4 *film, int width, int accumulate)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P.npix) return;
    int4 to = P.tileorder[P.g0 + q];
    int lx = to.z & 0xffff, ly = to.z >> 16, tw = to.w & 0xffff, th = to.w >> 16;
    float r = 0.f, g = 0.f, b = 0.f, w = 0.f;
    int nan = 0;
    for (int dy = -1; dy <= 1; dy++) {
        for (int dx = -1; dx <= 1; dx++) {
            int sx = lx + dx, sy = ly + dy;
            if (sx < 0 || sy < 0 || sx >= tw || sy >= th) continue;
            int qs = q + dy * tw + dx;
            bool self = (dx == 0 && dy == 0);
            if (!self && !P.W.pix_irregular[qs]) continue;
            for (int s = 0; s < P.spp; s++) {
                int slot = s * P.npix + qs;
                uint8_t code = P.W.splat[slot];
                if (!splat_covers(code, -dx, -dy)) continue;
                float4 L = P.W.out[slot];
                if (isnan(L.x) || isnan(L.y) || isnan(L.z)) { if (self) nan++; continue; }
                r += L.x * 1.f; g += L.y * 1.f; b += L.z * 1.f; w += 1.f;
            }
        }
    }
    float4 *px = &film[(size_t)to.y * width + to.x];
    if (accumulate) {
        float4 o = *px;
        *px = make_float4(o.x + r, o.y + g, o.z + b, o.w + w);
    } else {
        *px = make_float4(0.f + r, 0.f + g, 0.f + b, 0.f + w);
    }
    if (nan) atomicAdd(&P.stats[2], (unsigned long long)nan);
}

// k_film for a multi-scene batch: one thread per batch pixel of any item,
// reduced in the same order into the item's job film.  A pixel's neighbours
// lie in its own tile, so in its own item.
__global__ void k_film_multi(RenderParams P)
{
    int gq = blockIdx.x * blockDim.x + threadIdx.x;
    if (gq >= P.npix) return;
    int lo = 0, hi = P.n_items - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (P.items[mid].pix0 <= gq) lo = mid; else hi = mid - 1;
    }
    const MultiItem &it = P.items[lo];
    const int q = gq - it.pix0;
    int4 to = it.tileorder[it.g0 + q];
    int lx = to.z & 0xffff, ly = to.z >> 16, tw = to.w & 0xffff, th = to.w >> 16;
    float r = 0.f, g = 0.f, b = 0.f, w = 0.f;
    int nan = 0;
    for (int dy = -1; dy <= 1; dy++) {
        for (int dx = -1; dx <= 1; dx++) {
            int sx = lx + dx, sy = ly + dy;
            if (sx < 0 || sy < 0 || sx >= tw || sy >= th) continue;
            int qs = q + dy * tw + dx;
            bool self = (dx == 0 && dy == 0);
            if (!self && !P.W.pix_irregular[it.pix0 + qs]) continue;
            for (int s = 0; s < it.spp; s++) {
                int slot = it.path0 + s * it.npix + qs;
                uint8_t code = P.W.splat[slot];
                if (!splat_covers(code, -dx, -dy)) continue;
                float4 L = P.W.out[slot];
                if (isnan(L.x) || isnan(L.y) || isnan(L.z)) { if (self) nan++; continue; }
                r += L.x * 1.f; g += L.y * 1.f; b += L.z * 1.f; w += 1.f;
            }
        }
    }
    float4 *px = &it.film[(size_t)to.y * it.width + to.x];
    if (it.accumulate) {
        float4 o = *px;
        *px = make_float4(o.x + r, o.y + g, o.z + b, o.w + w);
    } else {
        *px = make_float4(0.f + r, 0.f + g, 0.f + b, 0.f + w);
    }
    if (nan) atomicAdd(&P.stats[2], (unsigned long long)nan);
}

// Film for reconstruction filters other than the box of radius 0.5
// (Screen::addSample / merge / postProcessColor, Screen.cpp:44-157).  Each
// tile's screen holds its pixels plus an overlap of ceil(r - 0.5) pixels on
// every side; samples splat value * w and w into every pixel of that screen
// within the filter radius, w read from the 32 x 32 table; screens are merged
// into the full screen in tile order.  One thread per output pixel gathers,
// tile by tile in raster order (the merge order of a single-threaded run), the
// samples of the tile's pixels that reach it, in the tile loop's pixel and
// sample order, re-deriving each sample's jitter from its path stream.  The
// output is the full screen's top-left width x height block, which is what
// the reference reads back (operator() and postProcessColor ignore the
// overlap offset, Screen.h:52, Screen.cpp:113-122).
__global__ void k_film_wide(RenderParams P, float4 *film, int t0, int t1, int tiles_x, int bx, int by)
{
    const DevCamera &cam = P.S.cam;
    const int W = cam.width, H = cam.height;
    const int ovx = cam.ov_x, ovy = cam.ov_y;
    const float rx = cam.frx, ry = cam.fry;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    const int ax = i % W, ay = i / W;   // full-screen (overlapped) coordinates
    float4 acc = film[i];
    const int ty_hi = imin((H + by - 1) / by - 1, ay / by), tx_hi = imin(tiles_x - 1, ax / bx);
    const int ty_lo = imax(0, (ay - 2 * ovy) / by - 1), tx_lo = imax(0, (ax - 2 * ovx) / bx - 1);
    const int reach_x = (int)ceilf(rx + 0.5f), reach_y = (int)ceilf(ry + 0.5f);
    for (int ty = ty_lo; ty <= ty_hi; ty++) {
        const int oy = ty * by, th = imin(by, H - oy);
        for (int tx = tx_lo; tx <= tx_hi; tx++) {
            const int t = ty * tiles_x + tx;
            if (t < t0 || t >= t1) continue;
            const int ox = tx * bx, tw = imin(bx, W - ox);
            const int lx = ax - ox, ly = ay - oy;
            if (lx < 0 || ly < 0 || lx >= tw + 2 * ovx || ly >= th + 2 * ovy) continue;
            // first batch pixel of the tile: full tile rows above, then the tiles to the left
            const int tile_first = oy * W + ox * th;
            const int qx0 = imax(ox, ax - ovx - reach_x), qx1 = imin(ox + tw - 1, ax - ovx + reach_x);
            const int qy0 = imax(oy, ay - ovy - reach_y), qy1 = imin(oy + th - 1, ay - ovy + reach_y);
            float sr = 0.f, sg = 0.f, sb = 0.f, sw = 0.f;
            for (int qy = qy0; qy <= qy1; qy++)
                for (int qx = qx0; qx <= qx1; qx++) {
                    const int q = tile_first - P.g0 + (qy - oy) * tw + (qx - ox);
                    for (int sm = 0; sm < P.spp; sm++) {
                        float4 L = P.W.out[(size_t)sm * P.npix + q];
                        if (isnan(L.x) || isnan(L.y) || isnan(L.z)) continue;
                        Pcg32 rng;
                        path_stream_seed(rng, P.seed, (uint32_t)(qy * W + qx), (uint32_t)(P.sample_begin + sm));
                        V2 j = next2d(rng);
                        float xl = ((float)qx + j.x) - 0.5f - (float)(ox - ovx);
                        float yl = ((float)qy + j.y) - 0.5f - (float)(oy - ovy);
                        int sx = imax(0, (int)ceilf(xl - rx)), ex = imin(tw + 2 * ovx - 1, (int)floorf(xl + rx));
                        int sy = imax(0, (int)ceilf(yl - ry)), ey = imin(th + 2 * ovy - 1, (int)floorf(yl + ry));
                        if (lx < sx || lx > ex || ly < sy || ly > ey) continue;
                        int ix = imin((int)((32 * fabsf((float)lx - xl)) / rx), 31);
                        int iy = imin((int)((32 * fabsf((float)ly - yl)) / ry), 31);
                        float w = __ldg(cam.filter_table + ix + iy * 32);
                        sr += L.x * w; sg += L.y * w; sb += L.z * w; sw += w;
                    }
                }
            acc = make_float4(acc.x + sr, acc.y + sg, acc.z + sb, acc.w + sw);
        }
    }
    film[i] = acc;
}

// ---------------------------------------------------------------- standalone queries
// ---------------------------------------------------------------- scene refit
// rt_scene_refit: new vertex positions into the triangle arrays, then the
// binary tree's boxes bottom-up over its unchanged topology, widened as the
// host build widens them, then the 4-wide tree's copies of them.
__global__ void k_refit_tris(const float *vtx, const float *nrm, const int32_t *idx, int nt, float *tri_v, float *tri_n)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x)
        for (int k = 0; k < 3; k++) {
            const size_t v = (size_t)idx[3 * (size_t)t + k];
            for (int a = 0; a < 3; a++) {
                tri_v[9 * (size_t)t + 3 * k + a] = vtx[3 * v + a];
                if (tri_n) tri_n[9 * (size_t)t + 3 * k + a] = nrm[3 * v + a];
            }
        }
}
// triangle slots (p0 and id, e1 = p1 - p0, e2 = p2 - p0) from the new vertices
__global__ void k_refit_slots(float4 *slots, int n_slots, const float *tri_v)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_slots; i += gridDim.x * blockDim.x) {
        const float4 a = slots[3 * (size_t)i];
        const float *P = tri_v + 9 * (size_t)__float_as_int(a.w);
        slots[3 * (size_t)i] = make_float4(P[0], P[1], P[2], a.w);
        slots[3 * (size_t)i + 1] = make_float4(P[3] - P[0], P[4] - P[1], P[5] - P[2], 0.f);
        slots[3 * (size_t)i + 2] = make_float4(P[6] - P[0], P[7] - P[1], P[8] - P[2], 0.f);
    }
}
// one level of internal nodes: the exact boxes of both children (a leaf's
// triangles, or an internal child's two boxes from the deeper level) into
// boxes[12 * node]: child 0 then child 1, each (min xyz, max xyz)
__global__ void k_refit_level(const float4 *nodes, const float4 *slots, const float *tri_v, const int32_t *order,
                              int begin, int end, float *boxes)
{
    for (int i = begin + blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
        const int nd = order[i];
        const float4 n1 = nodes[4 * (size_t)nd + 1];
        const int4 cc = reinterpret_cast<const int4 *>(nodes)[4 * (size_t)nd + 3];
        for (int k = 0; k < 2; k++) {
            float b[6] = {RT_MAX_REAL, RT_MAX_REAL, RT_MAX_REAL, -RT_MAX_REAL, -RT_MAX_REAL, -RT_MAX_REAL};
            const int link = k ? cc.y : cc.x;
            // the empty second child of a root leaf (an inverted box) stays empty
            const bool empty = k == 1 && !(n1.x <= n1.y);
            if (empty) {
                b[0] = b[1] = b[2] = INFINITY;
                b[3] = b[4] = b[5] = -INFINITY;
            } else if (link < 0) {
                const int v = ~link, first = v >> 3, cnt = (v & 7) + 1;
                for (int j = 0; j < cnt; j++) {
                    const float *P = tri_v + 9 * (size_t)__float_as_int(slots[3 * (size_t)(first + j)].w);
                    for (int c = 0; c < 3; c++)
                        for (int a = 0; a < 3; a++) {
                            b[a] = fminf(b[a], P[3 * c + a]);
                            b[3 + a] = fmaxf(b[3 + a], P[3 * c + a]);
                        }
                }
            } else {
                const float *cb = boxes + 12 * (size_t)link;
                for (int a = 0; a < 3; a++) {
                    b[a] = fminf(cb[a], cb[6 + a]);
                    b[3 + a] = fmaxf(cb[3 + a], cb[9 + a]);
                }
            }
            for (int a = 0; a < 6; a++) boxes[12 * (size_t)nd + 6 * k + a] = b[a];
        }
    }
}
// every node's two child boxes widened (pad = extent 1e-6 + magnitude 1.2e-6
// + 1e-7 of the scene's largest extent, as the host build pads) into the node
__global__ void k_refit_widen(float4 *nodes, int n_nodes, const float *boxes)
{
    float sext = 0.f;
    for (int a = 0; a < 3; a++) {
        float mn = boxes[a], mx = boxes[3 + a];
        if (boxes[6] <= boxes[9]) { mn = fminf(mn, boxes[6 + a]); mx = fmaxf(mx, boxes[9 + a]); }
        sext = fmaxf(sext, mx - mn);
    }
    const float seps = fmaxf(sext * 1e-7f, 1e-30f);
    for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < n_nodes; nd += gridDim.x * blockDim.x) {
        float w[2][6];
        for (int k = 0; k < 2; k++) {
            const float *b = boxes + 12 * (size_t)nd + 6 * k;
            for (int a = 0; a < 3; a++) {
                if (!(b[0] <= b[3])) { w[k][2 * a] = INFINITY; w[k][2 * a + 1] = -INFINITY; continue; }
                const float ext = b[3 + a] - b[a];
                const float m = fmaxf(fabsf(b[a]), fabsf(b[3 + a]));
                const float pad = ext * 1e-6f + m * 1.2e-6f + seps;
                w[k][2 * a] = b[a] - pad;
                w[k][2 * a + 1] = b[3 + a] + pad;
            }
        }
        nodes[4 * (size_t)nd] = make_float4(w[0][0], w[0][1], w[0][2], w[0][3]);
        nodes[4 * (size_t)nd + 1] = make_float4(w[1][0], w[1][1], w[1][2], w[1][3]);
        nodes[4 * (size_t)nd + 2] = make_float4(w[0][4], w[0][5], w[1][4], w[1][5]);
    }
}
// the 4-wide tree's child planes: copies of the binary tree's (src[slot])
__global__ void k_refit_bvh4(float *nodes4, int n4, const int32_t *src, const float4 *nodes2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * n4; i += gridDim.x * blockDim.x) {
        const int s = src[i];
        if (s < 0) continue;
        const int nd = s >> 1, k = s & 1, slot = i & 3;
        const float4 a = nodes2[4 * (size_t)nd + k], z = nodes2[4 * (size_t)nd + 2];
        const float pl[6] = {a.x, a.y, a.z, a.w, k ? z.z : z.x, k ? z.w : z.y};
        float *o = nodes4 + 32 * (size_t)(i >> 2);
        for (int p = 0; p < 6; p++) o[4 * p + slot] = pl[p];
    }
}

#include "rt_lbvh.cuh"

__global__ void k_trace_rays(DevScene S, const rt_ray *rays, int n, int any, rt_hit *hits)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rt_ray r = rays[i];
    Hit h;
    bool hit = any ? trace_ray<true>(S, vload(r.o), vload(r.d), r.mint, r.maxt, h)
                   : trace_ray<false>(S, vload(r.o), vload(r.d), r.mint, r.maxt, h);
    rt_hit o;
    o.t = hit && !any ? h.t : 0.f;
    o.u = hit && !any ? h.u : 0.f;
    o.v = hit && !any ? h.v : 0.f;
    o.prim = hit ? (any ? 0 : h.prim) : -1;
    hits[i] = o;
}

__global__ void k_bsdf_query(DevScene S, int bsdf, int op, const rt_bsdf_q *q, int n, rt_bsdf_r *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevBsdf &B = S.bsdfs[bsdf];
    rt_bsdf_r r;
    memset(&r, 0, sizeof(r));
    V3 wi = vload(q[i].wi), wo = vload(q[i].wo);
    if (op == RT_BSDF_OP_EVAL) {
        C3 v = bsdf_eval(B, wi, wo);
        r.value[0] = v.r; r.value[1] = v.g; r.value[2] = v.b;
    } else if (op == RT_BSDF_OP_PDF) {
        r.pdf = bsdf_pdf(B, wi, wo);
    } else {
        BsdfRec rec;
        rec.wi = wi; rec.wo = v3(0, 0, 0); rec.type = BT_ALL; rec.rel_eta = 1.f; rec.pdf = -1.f;
        // a LayeredBSDF query keys its coat-normal side stream by the sample's bits
        uint64_t key = ((uint64_t)__float_as_uint(q[i].u[0]) << 32) | __float_as_uint(q[i].u[1]);
        C3 v = bsdf_sample(B, rec, v2(q[i].u[0], q[i].u[1]), key);
        r.value[0] = v.r; r.value[1] = v.g; r.value[2] = v.b;
        r.pdf = rec.pdf;
        r.wo[0] = rec.wo.x; r.wo[1] = rec.wo.y; r.wo[2] = rec.wo.z;
        r.relative_eta = rec.rel_eta;
        r.sampled_type = rec.type;
    }
    out[i] = r;
}

__global__ void k_light_query(DevScene S, int light, const rt_light_q *q, int n, rt_light_r *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    LightRec li;
    li.point = li.to_light = li.normal = v3(0, 0, 0);
    li.intensity = cfill(0.f); li.distance = 0.f; li.pdf = 0.f;
    V3 p = vload(q[i].p);
    light_sample(S, light, p, v2(q[i].u[0], q[i].u[1]), li);
    rt_light_r r;
    r.intensity[0] = li.intensity.r; r.intensity[1] = li.intensity.g; r.intensity[2] = li.intensity.b;
    r.pdf = li.pdf;
    r.to_light[0] = li.to_light.x; r.to_light[1] = li.to_light.y; r.to_light[2] = li.to_light.z;
    r.distance = li.distance;
    r.point[0] = li.point.x; r.point[1] = li.point.y; r.point[2] = li.point.z;
    r.normal[0] = li.normal.x; r.normal[1] = li.normal.y; r.normal[2] = li.normal.z;
    r.pdf_eval = light_pdf(S, light, p, li.point, li.normal, li.to_light);
    r.pad = 0.f;
    out[i] = r;
}

__global__ void k_medium_query(DevScene S, int medium, int op, const rt_medium_q *q, int n, rt_medium_r *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Pcg32 rng;
    path_stream_seed(rng, q[i].seed, q[i].pixel, q[i].sample);
    Ray r = make_ray(vload(q[i].o), vload(q[i].d), q[i].mint, q[i].maxt);
    const DevMedium &m = S.media[medium];
    int limit = 0;
    rt_medium_r o;
    memset(&o, 0, sizeof(o));
    if (op == RT_MEDIUM_OP_SAMPLE) {
        float t = 0.f;
        C3 w, em;
        o.scattered = medium_sample(m, r, rng, t, w, em, limit) ? 1 : 0;
        o.weight[0] = w.r; o.weight[1] = w.g; o.weight[2] = w.b;
        o.t = t;
    } else {
        C3 tr = medium_tr(m, r, rng, limit);
        o.weight[0] = tr.r; o.weight[1] = tr.g; o.weight[2] = tr.b;
    }
    o.limit = limit;
    out[i] = o;
}

// =====================================================================
// host side
// =====================================================================
struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
};

struct rt_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // wavefront buffers (grown on demand)
    int capacity = 0;
    std::vector<void *> wave_allocs;
    Wave W;
    int4 *tileorder = nullptr;
    size_t tileorder_n = 0;
    int *work = nullptr;
    int *limit_flag = nullptr;
    unsigned long long *stats = nullptr;
    float *light_cdf = nullptr;
    int light_cdf_n = 0;
    float4 *film = nullptr;
    size_t film_n = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    rt_render_stats last;
    int profiling = 0;
    int bvh_width = 2;          // traversal used by renders and rt_trace: 2, 4 or 8
    int bvh_builder = 0;        // scenes created later: RT_BUILDER_HOST_SAH or RT_BUILDER_DEVICE
    int wave_paths = 1 << 26;   // target paths per wavefront batch (about 14 GB of path state)
    int ray_sort = 0;           // reorder secondary and shadow rays before tracing
    // launch shapes and the material-sort threshold (rt_ctx_set_tuning)
    int trace_bpsm = 12;        // traversal kernels: blocks per SM
    int shade_bpsm = RT_SHADE_GRID;   // finish and shading kernels: blocks per SM
    int sort_threshold = 0;     // rounds with fewer closest-hit rays shade unsorted
    int volpath_wave = 1;       // VolPathTracing as the wavefront (0: the megakernel)
    int batch_wave = 1;         // rt_batch_render: eligible jobs in one multi-scene wavefront
    std::vector<cudaEvent_t> ev_pool;
    std::vector<int> ev_kind;   // kernel kind per recorded pair
    size_t ev_used = 0;
    int tile_key[4] = {-1, -1, -1, -1};
    std::vector<int> tile_start;
    rt_lane_pool *pool = nullptr;   // worker lanes of rt_batch_render (rt_serve.cpp)
    // CUDA-graph batches (rt_ctx_set_graphs): instantiated graphs keyed by
    // the exact bytes of their launch parameters, newest last
    int graphs = 0;
    int *round_dev = nullptr;
    // graphs are captured on two streams of the context's own (the caller's
    // stream may be the legacy default stream, which cannot capture) and
    // launched on the context's stream
    cudaStream_t cap_stream = nullptr;    // captures the batch
    cudaStream_t body_stream = nullptr;   // captures the round loop's body
    struct GraphEntry {
        std::vector<unsigned char> key;
        cudaGraphExec_t exec;
    };
    std::vector<GraphEntry> gcache;
    int64_t graph_builds = 0, graph_hits = 0;
    // multi-scene batches (rt_internal_render_multi): scene table, work
    // items, concatenated tile orders and light CDFs (grown on demand)
    DevScene *m_scenes = nullptr;
    size_t m_scenes_n = 0;
    MultiItem *m_items = nullptr;
    size_t m_items_n = 0;
    int4 *m_order = nullptr;
    size_t m_order_n = 0;
    float *m_cdf = nullptr;
    size_t m_cdf_n = 0;
};

static void graph_cache_clear(rt_ctx *c)
{
    for (auto &e : c->gcache) cudaGraphExecDestroy(e.exec);
    c->gcache.clear();
}

// kinds for per-kernel timing
enum { K_CAMERA = 0, K_TRACE_C = 1, K_TRACE_A = 2, K_SHADE = 3, K_VOLPATH = 4, K_FILM = 5, K_RESOLVE = 6, K_SORT = 7,
       K_KINDS = 8 };

static void prof_begin(rt_ctx *c, int kind)
{
    if (!c->profiling) return;
    size_t need = 2 * (c->ev_used + 1);
    while (c->ev_pool.size() < need) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        c->ev_pool.push_back(e);
    }
    if (c->ev_kind.size() < c->ev_used + 1) c->ev_kind.resize(c->ev_used + 1);
    c->ev_kind[c->ev_used] = kind;
    cudaEventRecord(c->ev_pool[2 * c->ev_used], c->stream);
}
static void prof_end(rt_ctx *c)
{
    if (!c->profiling) return;
    cudaEventRecord(c->ev_pool[2 * c->ev_used + 1], c->stream);
    c->ev_used++;
}

struct rt_scene {
    rt_ctx *ctx = nullptr;
    DevScene S;
    std::vector<void *> allocs;
    int64_t bytes = 0;
    float bounds[6];
    int n_lights = 0;
    int n_bsdfs = 0;
    int n_media = 0;
    int bsdf_types = 0;   // bit q set when some BSDF uses shading queue q (bsdf_queue)
    int wide_depth = 0;
    bool wide_ok = false;  // the 8-wide BVH is uploaded (or the scene has no triangles)
    bool w4_ok = false;    // the 4-wide BVH is uploaded (or the scene has no triangles)
    std::vector<float> light_power_lum;  // per light, for the weighted strategy
    std::vector<DevLight> lights_host;
    DevLight *lights_dev = nullptr;
    // rt_scene_refit: the vertex count and device indices, the binary tree's
    // internal nodes deepest level first (level_off[l] .. level_off[l+1]),
    // the 4-wide tree's slot sources, scratch for exact boxes; refit_why is
    // empty when the scene can be refitted
    int n_vertices = 0, n_tris = 0;
    bool has_normals = false;
    const int32_t *indices_dev = nullptr;
    const int32_t *refit_order = nullptr;
    std::vector<int> level_off;
    const int32_t *bvh4_src = nullptr;
    float *refit_boxes = nullptr;
    std::string refit_why;
    float sph_bounds[6] = {RT_MAX_REAL, RT_MAX_REAL, RT_MAX_REAL, -RT_MAX_REAL, -RT_MAX_REAL, -RT_MAX_REAL};
};

// Traversal of a scene under the context's tree width (rt_ctx_set_bvh_width):
// the 8- or 4-wide tree where the scene has it uploaded, else the binary one.
static int trace_width(const rt_ctx *ctx, const rt_scene *sc);
// One closest-hit (any = false) or shadow-ray (any = true) traversal launch
// of round r; count adds the node / triangle fetch counters.
static void launch_trace(int width, const RenderParams &P, int r, bool any, bool count, int blocks, cudaStream_t st)
{
    if (width == 8) {
        if (any) { if (count) k_trace8<true, true><<<blocks, 128, 0, st>>>(P, r); else k_trace8<true, false><<<blocks, 128, 0, st>>>(P, r); }
        else { if (count) k_trace8<false, true><<<blocks, 128, 0, st>>>(P, r); else k_trace8<false, false><<<blocks, 128, 0, st>>>(P, r); }
    } else if (width == 4) {
        if (any) { if (count) k_trace4<true, true><<<blocks, 128, 0, st>>>(P, r); else k_trace4<true, false><<<blocks, 128, 0, st>>>(P, r); }
        else { if (count) k_trace4<false, true><<<blocks, 128, 0, st>>>(P, r); else k_trace4<false, false><<<blocks, 128, 0, st>>>(P, r); }
    } else {
        if (any) { if (count) k_trace<true, true><<<blocks, 128, 0, st>>>(P, r); else k_trace<true, false><<<blocks, 128, 0, st>>>(P, r); }
        else { if (count) k_trace<false, true><<<blocks, 128, 0, st>>>(P, r); else k_trace<false, false><<<blocks, 128, 0, st>>>(P, r); }
    }
}

template <typename T>
static rt_status upload(rt_scene *sc, const T *host, size_t count, const T **dev)
{
    *dev = nullptr;
    if (count == 0) return RT_OK;
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * count);
    if (e != cudaSuccess) return fail(RT_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    sc->allocs.push_back(p);
    sc->bytes += (int64_t)(sizeof(T) * count);
    e = cudaMemcpy(p, host, sizeof(T) * count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    *dev = (const T *)p;
    return RT_OK;
}

// ---------------------------------------------------------------- host math mirrors
static float h_cavg1(float v) { float s = 0.f; s += v; s += v; s += v; return s / 3.f; }
static float h_lum(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }
static float h_smin(float a, float b) { return (b < a) ? b : a; }
static float h_smax(float a, float b) { return (a < b) ? b : a; }

struct HCdf {
    std::vector<float> c{0.f};
    float sum = 0.f;
    void add(float p) { sum += p; c.push_back(sum); }
    void normalize()
    {
        if (sum != 0.f) {
            float f = 1.f / sum;
            for (size_t i = 1; i < c.size(); i++) c[i] *= f;
            c.back() = 1.f;
        }
    }
};

// ReconstructionFilter::precompute (ReconstructionFilter.cpp:27-40): the
// filter at (x rX / 32, y rY / 32), x, y = 0..31, with the Gaussian
// (GaussianFilter.cpp:28-36) and Mitchell-Netravali
// (MitchellNetravaliFilter.cpp:28-52) one-dimensional profiles; binary32 in
// the reference's operation order
static float h_gauss1(float a, float w, float v)
{
    float e1 = expf(-a * v * v), e2 = expf(-a * w * w);
    float d = e1 - e2;
    return d < 0.f ? 0.f : d;
}
static float h_mitchell1(float B, float C, float v)
{
    v = fabsf(2.f * v);
    if (v > 1.f)
        return ((((-B - 6 * C) * v * v * v + (6 * B + 30 * C) * v * v) + (-12 * B - 48 * C) * v + 8 * B) + 24 * C) *
               (1.f / 6.f);
    return ((12 - 9 * B - 6 * C) * v * v * v + (-18 + 12 * B + 6 * C) * v * v + (6 - 2 * B)) * (1.f / 6.f);
}
static void filter_table(const rt_camera_desc &c, float *t)
{
    const float rx = c.filter_radius[0], ry = c.filter_radius[1];
    for (int x = 0; x < 32; x++)
        for (int y = 0; y < 32; y++) {
            float fx = x * rx / 32, fy = y * ry / 32;
            float v = 1.f;
            if (c.filter == RT_FILTER_GAUSSIAN)
                v = h_gauss1(c.filter_param[0], c.filter_param[1], fx) * h_gauss1(c.filter_param[0], c.filter_param[1], fy);
            else if (c.filter == RT_FILTER_MITCHELL)
                v = h_mitchell1(c.filter_param[0], c.filter_param[1], fx / rx) *
                    h_mitchell1(c.filter_param[0], c.filter_param[1], fy / ry);
            t[x + y * 32] = v;
        }
}

// guide[k] = first i with c[i] >= k / G, k = 0..G (cdf_sample_guided)
static void cdf_guide(const float *c, int n, int G, int *g)
{
    int i = 0;
    for (int k = 0; k <= G; k++) {
        float t = (float)k / (float)G;
        while (i < n && c[i] < t) i++;
        g[k] = i;
    }
}
static int pow2_at_least(int n)
{
    int g = 1;
    while (g < n && g < (1 << 20)) g <<= 1;
    return g;
}

static void mat_mul4(const double *a, const double *b, double *o)
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a[i * 4 + k] * b[k * 4 + j];
            o[i * 4 + j] = s;
        }
}
static bool mat_inv4(const double *m, double *inv)
{
    double a[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 8; j++) a[i][j] = j < 4 ? m[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; c++) {
        int p = c;
        for (int r = c + 1; r < 4; r++) if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        if (a[p][c] == 0) return false;
        if (p != c) for (int j = 0; j < 8; j++) std::swap(a[p][j], a[c][j]);
        double d = a[c][c];
        for (int j = 0; j < 8; j++) a[c][j] /= d;
        for (int r = 0; r < 4; r++) {
            if (r == c) continue;
            double f = a[r][c];
            for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j];
        }
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) inv[i * 4 + j] = a[i][j + 4];
    return true;
}
static V3 h_xf_point(const float *m, V3 p) { return xf_point(m, p); }

// Heterogeneous::setOwnerBBox (medium/Heterogeneous.cpp:281-369), matrices in double
static void setup_hetero(const rt_medium_desc &m, const float *bmin, const float *bmax, DevMedium &D)
{
    double gmn[3], gmx[3], bmn[3], bmx[3];
    for (int i = 0; i < 3; i++) { gmn[i] = m.grid_min[i]; gmx[i] = m.grid_max[i]; bmn[i] = bmin[i]; bmx[i] = bmax[i]; }
    double ratio = (bmx[0] - bmn[0]) / (gmx[0] - gmn[0]);
    double ry = (bmx[1] - bmn[1]) / (gmx[1] - gmn[1]);
    if (ry < ratio) ratio = ry;
    double rz = (bmx[2] - bmn[2]) / (gmx[2] - gmn[2]);
    if (rz < ratio) ratio = rz;
    double S[16] = {0}, ext[3];
    for (int i = 0; i < 3; i++) { ext[i] = (gmx[i] - gmn[i]) * ratio; S[i * 5] = 1.0 / ext[i]; }
    S[15] = 1;
    double T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    for (int i = 0; i < 3; i++) T[i * 4 + 3] = m.centered ? -(bmn[i] + ((bmx[i] - bmn[i]) / 2.0 - ext[i] / 2.0)) : -bmn[i];
    double Wm[16], Winv[16];
    for (int i = 0; i < 16; i++) Wm[i] = m.to_world[i];
    if (!mat_inv4(Wm, Winv)) std::memcpy(Winv, Wm, sizeof(Wm));
    double ST[16], A[16], Ainv[16];
    mat_mul4(S, T, ST);
    mat_mul4(ST, Winv, A);
    mat_inv4(A, Ainv);
    float a2w[16];
    for (int i = 0; i < 16; i++) { D.world_to_array[i] = (float)A[i]; a2w[i] = (float)Ainv[i]; }
    float mn[3] = {RT_MAX_REAL, RT_MAX_REAL, RT_MAX_REAL}, mx[3] = {-RT_MAX_REAL, -RT_MAX_REAL, -RT_MAX_REAL};
    const float c[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 1, 0}};
    for (int k = 0; k < 8; k++) {
        V3 p = h_xf_point(a2w, v3(c[k][0], c[k][1], c[k][2]));
        mn[0] = h_smin(mn[0], p.x); mn[1] = h_smin(mn[1], p.y); mn[2] = h_smin(mn[2], p.z);
        mx[0] = h_smax(mx[0], p.x); mx[1] = h_smax(mx[1], p.y); mx[2] = h_smax(mx[2], p.z);
    }
    for (int i = 0; i < 3; i++) { D.wbox_min[i] = mn[i]; D.wbox_max[i] = mx[i]; }
    size_t nv = (size_t)m.res[0] * m.res[1] * m.res[2];
    float mxs = m.density[0];
    for (size_t i = 1; i < nv; i++) if (m.density[i] > mxs) mxs = m.density[i];
    D.max_sigma_t = mxs * m.scale;
}

// =====================================================================
// C ABI
// =====================================================================
extern "C" {

int32_t rt_abi_version(void) { return RTGPU_ABI_VERSION; }
const char *rt_last_error(void) { return g_err.c_str(); }
uint64_t rt_mix64(uint64_t x) { return mix64(x); }

rt_status rt_ctx_create(int32_t device, rt_ctx **out)
{
    if (!out) return fail(RT_ERR_INVALID, "rt_ctx_create: null out");
    *out = nullptr;
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(RT_ERR_INVALID, "rt_ctx_create: bad device index");
    CK(cudaSetDevice(device));
    rt_ctx *c = new rt_ctx();
    c->device = device;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) { delete c; return fail(RT_ERR_CUDA, cudaGetErrorString(e)); }
    c->sm_count = prop.multiProcessorCount;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return fail(RT_ERR_CUDA, cudaGetErrorString(e)); }
    c->own_stream = true;
    cudaMalloc(&c->work, sizeof(int) * 4);
    cudaMalloc(&c->limit_flag, sizeof(int));
    cudaMalloc(&c->stats, sizeof(unsigned long long) * 8);
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    std::memset(&c->last, 0, sizeof(c->last));
    *out = c;
    return RT_OK;
}

static void free_wave(rt_ctx *c)
{
    graph_cache_clear(c);   // the graphs hold the freed buffers' addresses
    for (void *p : c->wave_allocs) cudaFree(p);
    c->wave_allocs.clear();
    c->capacity = 0;
    c->W.vw_capacity = 0;
}

rt_status rt_ctx_destroy(rt_ctx *c)
{
    if (!c) return RT_OK;
    if (c->pool) rt_lane_pool_destroy(c->pool);
    c->pool = nullptr;
    cudaSetDevice(c->device);
    free_wave(c);
    cudaFree(c->round_dev);
    if (c->body_stream) cudaStreamDestroy(c->body_stream);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    cudaFree(c->tileorder);
    cudaFree(c->work);
    cudaFree(c->m_scenes);
    cudaFree(c->m_items);
    cudaFree(c->m_order);
    cudaFree(c->m_cdf);
    cudaFree(c->limit_flag);
    cudaFree(c->stats);
    cudaFree(c->light_cdf);
    cudaFree(c->film);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return RT_OK;
}

rt_status rt_ctx_set_profiling(rt_ctx *c, int32_t level)
{
    if (!c) return fail(RT_ERR_INVALID, "null ctx");
    if (level < 0 || level > 2) return fail(RT_ERR_INVALID, "profiling level must be 0, 1 or 2");
    c->profiling = level;
    return RT_OK;
}

rt_status rt_ctx_set_bvh_width(rt_ctx *c, int32_t width)
{
    if (!c) return fail(RT_ERR_INVALID, "null ctx");
    if (width != 2 && width != 4 && width != 8) return fail(RT_ERR_INVALID, "BVH width must be 2, 4 or 8");
    c->bvh_width = width;
    return RT_OK;
}

rt_status rt_ctx_set_bvh_builder(rt_ctx *c, int32_t builder)
{
    if (!c) return fail(RT_ERR_INVALID, "null ctx");
    if (builder != RT_BUILDER_HOST_SAH && builder != RT_BUILDER_DEVICE)
        return fail(RT_ERR_INVALID, "BVH builder must be RT_BUILDER_HOST_SAH or RT_BUILDER_DEVICE");
    c->bvh_builder = builder;
    return RT_OK;
}

rt_status rt_ctx_set_wave_paths(rt_ctx *c, int32_t paths)
{
    if (!c) return fail(RT_ERR_INVALID, "null ctx");
    if (paths < (1 << 16) || paths > (1 << 26)) return fail(RT_ERR_INVALID, "wave paths must be in [2^16, 2^26]");
    c->wave_paths = paths;
    return RT_OK;
}

rt_status rt_ctx_set_ray_sort(rt_ctx *c, int32_t on)
{
    if (!c) return fail(RT_ERR_INVALID, "null ctx");
    c->ray_sort = on ? 1 : 0;
    return RT_OK;
}

rt_status rt_ctx_set_graphs(rt_ctx *c, int32_t on)
{
    if (!c) return fail(RT_ERR_INVALID, "null ctx");
    c->graphs = on ? 1 : 0;
    if (!c->graphs) {
        cudaSetDevice(c->device);
        graph_cache_clear(c);
    }
    return RT_OK;
}

rt_status rt_ctx_set_stream(rt_ctx *c, void *stream)
{
    if (!c) return fail(RT_ERR_INVALID, "null ctx");
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
    return RT_OK;
}

rt_status rt_scene_destroy(rt_scene *sc)
{
    if (!sc) return RT_OK;
    for (void *p : sc->allocs) cudaFree(p);
    cudaFree(sc->refit_boxes);
    delete sc;
    return RT_OK;
}

static rt_status validate(const rt_scene_desc *d)
{
    if (!d) return fail(RT_ERR_INVALID, "null scene desc");
    if (d->n_triangles < 0 || d->n_vertices < 0 || d->n_meshes < 0 || d->n_spheres < 0 || d->n_bsdfs < 0 ||
        d->n_lights < 0 || d->n_media < 0)
        return fail(RT_ERR_INVALID, "negative count in scene desc");
    if (d->n_triangles > (1 << 27)) return fail(RT_ERR_LIMIT, "more than 2^27 triangles");
    if (d->n_triangles > 0 && (!d->vertices || !d->indices)) return fail(RT_ERR_INVALID, "missing geometry arrays");
    for (int i = 0; i < 3 * d->n_triangles; i++)
        if (d->indices[i] < 0 || d->indices[i] >= d->n_vertices) return fail(RT_ERR_INVALID, "vertex index out of range");
    int64_t covered = 0;
    for (int m = 0; m < d->n_meshes; m++) {
        const rt_mesh_desc &M = d->meshes[m];
        if (M.first_tri < 0 || M.n_tris < 0 || (int64_t)M.first_tri + M.n_tris > d->n_triangles)
            return fail(RT_ERR_INVALID, "mesh triangle range out of bounds");
        if (M.bsdf >= d->n_bsdfs || M.light >= d->n_lights || M.interior >= d->n_media || M.exterior >= d->n_media)
            return fail(RT_ERR_INVALID, "mesh references a missing component");
        covered += M.n_tris;
    }
    if (covered != d->n_triangles) return fail(RT_ERR_INVALID, "meshes must cover every triangle exactly once");
    for (int s = 0; s < d->n_spheres; s++) {
        const rt_sphere_desc &S = d->spheres[s];
        if (S.bsdf >= d->n_bsdfs || S.light >= d->n_lights || S.interior >= d->n_media || S.exterior >= d->n_media)
            return fail(RT_ERR_INVALID, "sphere references a missing component");
        if (S.kind != RT_ANALYTIC_SPHERE && S.kind != RT_ANALYTIC_PLANE)
            return fail(RT_ERR_INVALID, "analytic shape of unknown kind");
    }
    for (int l = 0; l < d->n_lights; l++) {
        const rt_light_desc &L = d->lights[l];
        if (L.type == RT_LIGHT_ENV) {
            if (L.env_width < 2 || L.env_height < 2 || !L.env_rgb) return fail(RT_ERR_INVALID, "bad environment map");
        } else if (L.type == RT_LIGHT_AREA) {
            if (L.shape_kind == RT_SHAPE_MESH ? (L.shape < 0 || L.shape >= d->n_meshes || d->meshes[L.shape].n_tris == 0)
                                              : (L.shape < 0 || L.shape >= d->n_spheres))
                return fail(RT_ERR_INVALID, "area light without a valid shape");
        } else if (L.type == RT_LIGHT_POINT || L.type == RT_LIGHT_SPOT) {
            for (int i = 0; i < 3; i++)
                if (!std::isfinite(L.position[i]) || !std::isfinite(L.intensity[i]))
                    return fail(RT_ERR_INVALID, "point or spot light with a non-finite position or intensity");
        } else {
            return fail(RT_ERR_UNSUPPORTED, "light type not supported");
        }
    }
    if (d->n_textures < 0 || (d->n_textures > 0 && !d->textures)) return fail(RT_ERR_INVALID, "bad texture table");
    for (int i = 0; i < d->n_textures; i++) {
        const rt_texture_desc &T = d->textures[i];
        if (T.width < 1 || T.height < 1 || !T.rgb || (int64_t)T.width * T.height > (1 << 28) || !(T.scale >= 0.f) ||
            !(T.scale < 1e30f))
            return fail(RT_ERR_INVALID, "texture without texels, too large, or with a bad scale");
    }
    for (int b = 0; b < d->n_bsdfs; b++) {
        const rt_bsdf_desc &B = d->bsdfs[b];
        if (B.type < 0 || B.type > RT_BSDF_MICROFACET) return fail(RT_ERR_UNSUPPORTED, "BSDF type not supported");
        const int32_t tx[4] = {B.tex_albedo, B.tex_reflectance, B.tex_transmittance, B.tex_alpha};
        for (int k = 0; k < 4; k++)
            if (tx[k] < 0 || tx[k] > d->n_textures) return fail(RT_ERR_INVALID, "BSDF texture index out of range");
        // the parameters each BSDF reads through a texture in the reference
        const int t = B.type;
        const bool ok = (!B.tex_albedo || t == RT_BSDF_DIFFUSE || t == RT_BSDF_MICROFACET) &&
                        (!B.tex_reflectance || t == RT_BSDF_ROUGH_CONDUCTOR || t == RT_BSDF_ROUGH_DIELECTRIC ||
                         t == RT_BSDF_DIELECTRIC || t == RT_BSDF_CONDUCTOR || t == RT_BSDF_SHEET_DIELECTRIC) &&
                        (!B.tex_transmittance || t == RT_BSDF_ROUGH_DIELECTRIC || t == RT_BSDF_DIELECTRIC ||
                         t == RT_BSDF_SHEET_DIELECTRIC) &&
                        (!B.tex_alpha || t == RT_BSDF_ROUGH_CONDUCTOR || t == RT_BSDF_ROUGH_DIELECTRIC);
        if (!ok) return fail(RT_ERR_UNSUPPORTED, "a texture on a parameter this BSDF type does not texture");
    }
    for (int m = 0; m < d->n_media; m++) {
        const rt_medium_desc &M = d->media[m];
        if (M.type == RT_MEDIUM_HETEROGENEOUS && (!M.density || M.res[0] < 2 || M.res[1] < 2 || M.res[2] < 2))
            return fail(RT_ERR_INVALID, "heterogeneous medium without a grid");
    }
    if (d->env_light >= d->n_lights) return fail(RT_ERR_INVALID, "env_light index out of range");
    if (d->camera.width <= 0 || d->camera.height <= 0 || d->camera.width > 32768 || d->camera.height > 32768)
        return fail(RT_ERR_INVALID, "bad film size");
    if (d->camera.medium >= d->n_media) return fail(RT_ERR_INVALID, "camera medium out of range");
    if (d->camera.filter < RT_FILTER_BOX || d->camera.filter > RT_FILTER_MITCHELL)
        return fail(RT_ERR_UNSUPPORTED, "reconstruction filter type not supported");
    for (int k = 0; k < 2; k++)
        if (!(d->camera.filter_radius[k] > 0.f) || d->camera.filter_radius[k] > 16.f)
            return fail(RT_ERR_INVALID, "filter radius must be in (0, 16]");
    return RT_OK;
}

static rt_status launch_check(const char *what);

// The binary tree built on the device (rt_lbvh.cuh) over the scene's
// triangles, already on the device in S.tri_v: the node image and the
// triangle slots, in memory the scene owns.  RT_ERR_LIMIT when the tree is
// deeper than the traversal stacks (the caller then builds on the host).
static rt_status device_tree(rt_ctx *ctx, rt_scene *sc, int nt)
{
    DevScene &S = sc->S;
    cudaStream_t st = ctx->stream;
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    auto grid = [&](int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm * 32)); };
    const int tiles = (nt + RT_RSORT_TILE - 1) / RT_RSORT_TILE;
    // temporaries in one allocation: codes and ids twice, digit counts,
    // parents, arrival counters, exact boxes, the depth
    const size_t n = (size_t)nt;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~(size_t)255; return o; };
    const size_t o_code0 = take(4 * n), o_code1 = take(4 * n), o_id0 = take(4 * n), o_id1 = take(4 * n);
    const size_t o_hist = take(4 * 256 * (size_t)tiles), o_ipar = take(4 * n), o_lpar = take(4 * n);
    const size_t o_arr = take(4 * n), o_box = take(48 * n), o_depth = take(4);
    char *tmp = nullptr;
    if (cudaMalloc((void **)&tmp, off) != cudaSuccess) return fail(RT_ERR_NOMEM, "device tree: scratch allocation failed");
    unsigned *code[2] = {(unsigned *)(tmp + o_code0), (unsigned *)(tmp + o_code1)};
    int *id[2] = {(int *)(tmp + o_id0), (int *)(tmp + o_id1)};
    int *hist = (int *)(tmp + o_hist), *ipar = (int *)(tmp + o_ipar), *lpar = (int *)(tmp + o_lpar);
    int *arr = (int *)(tmp + o_arr), *depth = (int *)(tmp + o_depth);
    float *boxes = (float *)(tmp + o_box);
    float4 *nodes = nullptr, *slots = nullptr;
    rt_status s = RT_OK;
    auto done = [&](rt_status r) { cudaFree(tmp); return r; };
    if (cudaMalloc((void **)&nodes, sizeof(float4) * 4 * (n - 1)) != cudaSuccess) return done(fail(RT_ERR_NOMEM, "device tree: node allocation failed"));
    sc->allocs.push_back(nodes);
    if (cudaMalloc((void **)&slots, sizeof(float4) * 3 * n) != cudaSuccess) return done(fail(RT_ERR_NOMEM, "device tree: slot allocation failed"));
    sc->allocs.push_back(slots);
    sc->bytes += (int64_t)(sizeof(float4) * (4 * (n - 1) + 3 * n));
    // Morton codes over the scene box
    float scale[3];
    for (int a = 0; a < 3; a++) {
        const float ext = sc->bounds[3 + a] - sc->bounds[a];
        scale[a] = ext > 0.f ? 1024.f / ext : 0.f;
    }
    k_lbvh_codes<<<grid(nt), 256, 0, st>>>(S.tri_v, nt, sc->bounds[0], sc->bounds[1], sc->bounds[2], scale[0], scale[1],
                                          scale[2], code[0], id[0]);
    int cur = 0;
    for (int shift = 0; shift < 30; shift += 8) {
        k_rsort_hist<<<tiles, RT_RSORT_THREADS, 0, st>>>(code[cur], nt, shift, tiles, hist);
        k_rsort_scan<<<1, 1024, 0, st>>>(hist, 256 * tiles);
        k_rsort_scatter<<<tiles, RT_RSORT_THREADS, 0, st>>>(code[cur], id[cur], nt, shift, tiles, hist, code[1 - cur],
                                                            id[1 - cur]);
        cur = 1 - cur;
    }
    k_lbvh_nodes<<<grid(nt - 1), 256, 0, st>>>(code[cur], nt, nodes, ipar, lpar);
    if (cudaMemsetAsync(arr, 0, 4 * n, st) != cudaSuccess || cudaMemsetAsync(depth, 0, 4, st) != cudaSuccess)
        return done(fail(RT_ERR_CUDA, "device tree: memset failed"));
    k_lbvh_boxes<<<grid(nt), 256, 0, st>>>(S.tri_v, id[cur], nt, ipar, lpar, arr, boxes, depth);
    k_refit_widen<<<grid(nt - 1), 256, 0, st>>>(nodes, nt - 1, boxes);
    k_lbvh_slots<<<grid(nt), 256, 0, st>>>(S.tri_v, id[cur], nt, slots);
    if ((s = launch_check("device tree kernels")) != RT_OK) return done(s);
    int maxd = 0;
    if (cudaMemcpyAsync(&maxd, depth, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
        return done(fail(RT_ERR_CUDA, "device tree: readback failed"));
    if (maxd + 1 > RT_STACK) {
        // too deep for the stacks: give the memory back; the caller builds on the host
        sc->allocs.pop_back();
        sc->allocs.pop_back();
        cudaFree(nodes);
        cudaFree(slots);
        sc->bytes -= (int64_t)(sizeof(float4) * (4 * (n - 1) + 3 * n));
        return done(fail(RT_ERR_LIMIT, "device tree: deeper than the traversal stack"));
    }
    S.nodes = nodes;
    S.tri_slots = slots;
    S.n_nodes = nt - 1;
    return done(RT_OK);
}

// a caller-built binary tree (rt_scene_create_bvh)
struct ExtTree {
    const rt_bvh_node *nodes;
    int n_nodes;
    const int32_t *prims;
    int n_prims;
};
static_assert(sizeof(rt_bvh_node) == sizeof(ExtNode), "rt_bvh_node and ExtNode share one layout");

static rt_status scene_create(rt_ctx *ctx, const rt_scene_desc *d, const ExtTree *ext, rt_scene **out)
{
    if (!ctx || !out) return fail(RT_ERR_INVALID, "rt_scene_create: null argument");
    *out = nullptr;
    rt_status st = validate(d);
    if (st != RT_OK) return st;
    CK(cudaSetDevice(ctx->device));
    rt_scene *sc = new rt_scene();
    sc->ctx = ctx;
    DevScene &S = sc->S;
    std::memset(&S, 0, sizeof(S));
    const int nt = d->n_triangles;
    // per-triangle original vertices / normals / mesh id
    std::vector<float> tri_v(9 * (size_t)nt), tri_n;
    std::vector<int> tri_mesh(nt, 0);
    for (int t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++)
            for (int a = 0; a < 3; a++) tri_v[9 * (size_t)t + 3 * k + a] = d->vertices[3 * (size_t)d->indices[3 * (size_t)t + k] + a];
    if (d->normals) {
        tri_n.resize(9 * (size_t)nt);
        for (int t = 0; t < nt; t++)
            for (int k = 0; k < 3; k++)
                for (int a = 0; a < 3; a++) tri_n[9 * (size_t)t + 3 * k + a] = d->normals[3 * (size_t)d->indices[3 * (size_t)t + k] + a];
    }
    std::vector<float> tri_uv;   // 6 floats per triangle; NaN u: mesh without uvs
    if (d->uvs) {
        tri_uv.resize(6 * (size_t)nt);
        for (int t = 0; t < nt; t++)
            for (int k = 0; k < 3; k++)
                for (int a = 0; a < 2; a++) tri_uv[6 * (size_t)t + 2 * k + a] = d->uvs[2 * (size_t)d->indices[3 * (size_t)t + k] + a];
    }
    // meshes: area CDF (Mesh.cpp:19-31) and owner boxes
    std::vector<DevMesh> meshes(d->n_meshes);
    std::vector<float> mesh_cdf;
    std::vector<float> mbox(6 * (size_t)std::max(1, d->n_meshes));
    float bmin[3] = {RT_MAX_REAL, RT_MAX_REAL, RT_MAX_REAL}, bmax[3] = {-RT_MAX_REAL, -RT_MAX_REAL, -RT_MAX_REAL};
    for (int m = 0; m < d->n_meshes; m++) {
        const rt_mesh_desc &M = d->meshes[m];
        DevMesh &D = meshes[m];
        D.first_tri = M.first_tri; D.n_tris = M.n_tris; D.bsdf = M.bsdf; D.light = M.light;
        D.interior = M.interior; D.exterior = M.exterior;
        D.cdf_off = (int)mesh_cdf.size();
        HCdf c;
        float area = 0.f;
        float *mb = &mbox[6 * (size_t)m];
        for (int i = 0; i < 3; i++) { mb[i] = RT_MAX_REAL; mb[3 + i] = -RT_MAX_REAL; }
        for (int i = 0; i < M.n_tris; i++) {
            int t = M.first_tri + i;
            tri_mesh[t] = m;
            const float *P = &tri_v[9 * (size_t)t];
            V3 p0 = vload(P), p1 = vload(P + 3), p2 = vload(P + 6);
            float a = 0.5f * norm(cross(p1 - p0, p2 - p0));
            c.add(a);
            area += a;
            for (int k = 0; k < 3; k++)
                for (int ax = 0; ax < 3; ax++) {
                    mb[ax] = h_smin(mb[ax], P[3 * k + ax]);
                    mb[3 + ax] = h_smax(mb[3 + ax], P[3 * k + ax]);
                }
        }
        c.normalize();
        D.area = area;
        mesh_cdf.insert(mesh_cdf.end(), c.c.begin(), c.c.end());
        for (int ax = 0; ax < 3; ax++) { bmin[ax] = h_smin(bmin[ax], mb[ax]); bmax[ax] = h_smax(bmax[ax], mb[3 + ax]); }
    }
    // spheres
    std::vector<DevSphere> spheres(d->n_spheres);
    for (int s = 0; s < d->n_spheres; s++) {
        const rt_sphere_desc &Sd = d->spheres[s];
        DevSphere &D = spheres[s];
        D.radius = Sd.radius;
        std::memcpy(D.to_world, Sd.to_world, sizeof(D.to_world));
        std::memcpy(D.to_object, Sd.to_object, sizeof(D.to_object));
        D.bsdf = Sd.bsdf; D.light = Sd.light; D.interior = Sd.interior; D.exterior = Sd.exterior;
        D.kind = Sd.kind;
        D.area = 0.f;
        float r = Sd.radius;
        float lo[3] = {-r, -r, -r}, hi[3] = {r, r, r};
        if (Sd.kind == RT_ANALYTIC_PLANE) {
            // Plane::getLocalBoundingBox (Plane.cpp:28-42) and the surface area
            // of Plane::Plane (Plane.cpp:13-17)
            lo[0] = -1.f; lo[1] = -1.f; lo[2] = 0.f;
            hi[0] = 1.f; hi[1] = 1.f; hi[2] = 0.f;
            V3 mn = h_xf_point(Sd.to_world, v3(-1.f, -1.f, 0.f));
            V3 s1 = h_xf_point(Sd.to_world, v3(-1.f, 1.f, 0.f)) - mn;
            V3 s2 = h_xf_point(Sd.to_world, v3(1.f, -1.f, 0.f)) - mn;
            D.area = sqrtf(dot(s1, s1)) * sqrtf(dot(s2, s2));
        }
        const float cx[8][3] = {{lo[0], lo[1], lo[2]}, {lo[0], lo[1], hi[2]}, {lo[0], hi[1], hi[2]}, {hi[0], hi[1], hi[2]},
                                {hi[0], lo[1], lo[2]}, {hi[0], hi[1], lo[2]}, {hi[0], lo[1], hi[2]}, {lo[0], hi[1], lo[2]}};
        for (int k = 0; k < 8; k++) {
            V3 p = h_xf_point(Sd.to_world, v3(cx[k][0], cx[k][1], cx[k][2]));
            bmin[0] = h_smin(bmin[0], p.x); bmin[1] = h_smin(bmin[1], p.y); bmin[2] = h_smin(bmin[2], p.z);
            bmax[0] = h_smax(bmax[0], p.x); bmax[1] = h_smax(bmax[1], p.y); bmax[2] = h_smax(bmax[2], p.z);
            const float pc[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; a++) {
                sc->sph_bounds[a] = h_smin(sc->sph_bounds[a], pc[a]);
                sc->sph_bounds[3 + a] = h_smax(sc->sph_bounds[3 + a], pc[a]);
            }
        }
    }
    for (int i = 0; i < 3; i++) { sc->bounds[i] = bmin[i]; sc->bounds[3 + i] = bmax[i]; S.bmin[i] = bmin[i]; S.bmax[i] = bmax[i]; }
    // BSDFs
    std::vector<DevBsdf> bsdfs(d->n_bsdfs);
    for (int b = 0; b < d->n_bsdfs; b++) {
        const rt_bsdf_desc &B = d->bsdfs[b];
        DevBsdf &D = bsdfs[b];
        D.type = B.type; D.distribution = B.distribution;
        for (int i = 0; i < 3; i++) {
            D.albedo[i] = B.albedo[i]; D.reflectance[i] = B.reflectance[i]; D.transmittance[i] = B.transmittance[i];
            D.eta[i] = B.eta[i]; D.k[i] = B.k[i]; D.absorbance[i] = B.absorbance[i];
        }
        D.alpha = B.alpha;
        D.alpha_avg = h_cavg1(B.alpha);
        D.dist_base = B.distribution_base;
        D.alpha_base_avg = h_cavg1(B.alpha_base);
        D.eta_int = B.eta_int; D.eta_ext = B.eta_ext; D.thickness = B.thickness;
        D.two_sided = B.two_sided != 0;
        D.tex[TEX_ALBEDO] = B.tex_albedo - 1;
        D.tex[TEX_REFLECTANCE] = B.tex_reflectance - 1;
        D.tex[TEX_TRANSMITTANCE] = B.tex_transmittance - 1;
        D.tex[TEX_ALPHA] = B.tex_alpha - 1;
        D.textured = (B.tex_albedo | B.tex_reflectance | B.tex_transmittance | B.tex_alpha) != 0;
        D.ks = B.ks;
    }
    // media
    std::vector<DevMedium> media(d->n_media);
    for (int m = 0; m < d->n_media; m++) {
        const rt_medium_desc &M = d->media[m];
        DevMedium &D = media[m];
        std::memset(&D, 0, sizeof(D));
        D.type = M.type; D.phase = M.phase; D.g = M.g; D.scale = M.scale;
        float sa[3], ss[3];
        for (int i = 0; i < 3; i++) { sa[i] = M.sigma_a[i]; ss[i] = M.sigma_s[i]; D.albedo[i] = M.albedo[i]; }
        if (M.scale != 1.f) for (int i = 0; i < 3; i++) { sa[i] *= M.scale; ss[i] *= M.scale; }
        for (int i = 0; i < 3; i++) { D.sigma_t[i] = sa[i] + ss[i]; D.sigma_s[i] = ss[i]; D.res[i] = M.res[i]; }
    }
    // Heterogeneous owner boxes, in mesh order, interior then exterior (MeshFactory.h:133-136)
    for (int m = 0; m < d->n_meshes; m++) {
        const rt_mesh_desc &M = d->meshes[m];
        if (M.n_tris == 0) continue;
        const float *mb = &mbox[6 * (size_t)m];
        if (M.interior >= 0 && d->media[M.interior].type == RT_MEDIUM_HETEROGENEOUS)
            setup_hetero(d->media[M.interior], mb, mb + 3, media[M.interior]);
        if (M.exterior >= 0 && d->media[M.exterior].type == RT_MEDIUM_HETEROGENEOUS)
            setup_hetero(d->media[M.exterior], mb, mb + 3, media[M.exterior]);
    }
    // lights
    std::vector<DevLight> lights(d->n_lights);
    sc->light_power_lum.assign(d->n_lights, 0.f);
    for (int l = 0; l < d->n_lights; l++) {
        const rt_light_desc &L = d->lights[l];
        DevLight &D = lights[l];
        std::memset(&D, 0, sizeof(D));
        D.type = L.type; D.mesh_light = L.mesh_light; D.shape_kind = L.shape_kind; D.shape = L.shape;
        for (int i = 0; i < 3; i++) D.radiance[i] = L.radiance[i];
        std::memcpy(D.env_to_world, L.env_to_world, sizeof(D.env_to_world));
        std::memcpy(D.env_to_light, L.env_to_light, sizeof(D.env_to_light));
        if (L.type == RT_LIGHT_POINT || L.type == RT_LIGHT_SPOT) {
            for (int i = 0; i < 3; i++) { D.position[i] = L.position[i]; D.intensity[i] = L.intensity[i]; }
            std::memcpy(D.spot_to_light, L.spot_to_light, sizeof(D.spot_to_light));
            D.cos_falloff_start = L.cos_falloff_start;
            D.cos_total_width = L.cos_total_width;
            // Light::power (PointLight.h, SpotLight.h) for the weighted light CDF
            float k = 4 * RT_PI, f = 1.f;
            if (L.type == RT_LIGHT_SPOT) { k = 2 * RT_PI; f = 1.f - 0.5f * (L.cos_falloff_start + L.cos_total_width); }
            sc->light_power_lum[l] = h_lum((L.intensity[0] * k) * f, (L.intensity[1] * k) * f, (L.intensity[2] * k) * f);
        } else if (L.type == RT_LIGHT_ENV) {
            int Wd = L.env_width, H = L.env_height;
            D.env_w = Wd; D.env_h = H; D.env_scale = L.env_scale;
            std::vector<float> rows((size_t)H * (Wd + 1)), weight(H);
            HCdf marg;
            for (int i = 0; i < H; i++) {
                float w = sinf(RT_PI * ((float)i + 0.5f) / (float)H);
                HCdf row;
                for (int j = 0; j < Wd; j++) {
                    const float *p = L.env_rgb + 3 * ((size_t)i * Wd + j);
                    row.add(h_lum(p[0] * L.env_scale, p[1] * L.env_scale, p[2] * L.env_scale));
                }
                weight[i] = w;
                marg.add(row.sum * w);
                row.normalize();
                std::copy(row.c.begin(), row.c.end(), rows.begin() + (size_t)i * (Wd + 1));
            }
            marg.normalize();
            D.env_marginal_sum = marg.sum;
            V3 bmn = vload(bmin), bmx = vload(bmax);
            V3 c = 0.5f * (bmx + bmn);
            D.env_radius = 2 * h_smax(norm(bmn - c), norm(bmx - c));
            const float *dp;
            if ((st = upload(sc, L.env_rgb, 3 * (size_t)Wd * H, &dp)) != RT_OK) { rt_scene_destroy(sc); return st; }
            D.env_rgb = dp;
            if ((st = upload(sc, rows.data(), rows.size(), &dp)) != RT_OK) { rt_scene_destroy(sc); return st; }
            D.env_row_cdf = dp;
            if ((st = upload(sc, marg.c.data(), marg.c.size(), &dp)) != RT_OK) { rt_scene_destroy(sc); return st; }
            D.env_marginal = dp;
            if ((st = upload(sc, weight.data(), weight.size(), &dp)) != RT_OK) { rt_scene_destroy(sc); return st; }
            D.env_weight = dp;
            // guide tables for the marginal and row CDF searches
            D.env_gm = pow2_at_least(H);
            D.env_gr = pow2_at_least(Wd);
            std::vector<int> gm(D.env_gm + 1), gr((size_t)H * (D.env_gr + 1));
            cdf_guide(marg.c.data(), H + 1, D.env_gm, gm.data());
            for (int i = 0; i < H; i++)
                cdf_guide(rows.data() + (size_t)i * (Wd + 1), Wd + 1, D.env_gr, gr.data() + (size_t)i * (D.env_gr + 1));
            const int *ip;
            if ((st = upload(sc, gm.data(), gm.size(), &ip)) != RT_OK) { rt_scene_destroy(sc); return st; }
            D.env_marg_guide = ip;
            if ((st = upload(sc, gr.data(), gr.size(), &ip)) != RT_OK) { rt_scene_destroy(sc); return st; }
            D.env_row_guide = ip;
            float R = D.env_radius;
            float pw = 4 * RT_PI * R * R;
            sc->light_power_lum[l] = h_lum(1.f * pw, 1.f * pw, 1.f * pw);
        } else {
            float area;
            if (L.shape_kind == RT_SHAPE_MESH) area = meshes[L.shape].area;
            else if (d->spheres[L.shape].kind == RT_ANALYTIC_PLANE) area = spheres[L.shape].area;
            else { float r = d->spheres[L.shape].radius; area = 4.f * RT_PI * r * r * r; }
            sc->light_power_lum[l] = h_lum(RT_PI * L.radiance[0] * area, RT_PI * L.radiance[1] * area,
                                           RT_PI * L.radiance[2] * area);
        }
    }
    // medium grids
    for (int m = 0; m < d->n_media; m++) {
        const rt_medium_desc &M = d->media[m];
        if (M.type != RT_MEDIUM_HETEROGENEOUS) continue;
        const float *dp;
        if ((st = upload(sc, M.density, (size_t)M.res[0] * M.res[1] * M.res[2], &dp)) != RT_OK) { rt_scene_destroy(sc); return st; }
        media[m].density = dp;
    }
    const float *fp;
    const int *ip;
    if ((st = upload(sc, tri_v.data(), tri_v.size(), &fp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.tri_v = fp;
    // BVH: built on the device when the context asks for it (a tree too deep
    // for the stacks falls back to the host build), else on the host
    bool dev_tree = false;
    if (!ext && ctx->bvh_builder == RT_BUILDER_DEVICE && nt >= 2 && nt < (1 << 28)) {
        if ((st = device_tree(ctx, sc, nt)) == RT_OK) dev_tree = true;
        else if (st != RT_ERR_LIMIT) { rt_scene_destroy(sc); return st; }
    }
    if (dev_tree) {
        // one triangle per leaf; no wide trees, no refit table
        S.n_nodes4 = 0; sc->w4_ok = false;
        S.n_wnodes = 0; sc->wide_ok = false;
        sc->refit_why = "a tree built on the device";
    } else {
    BvhImage img;
    if (ext) {
        std::string why;
        if (!import_bvh2(tri_v.data(), nt, reinterpret_cast<const ExtNode *>(ext->nodes), ext->n_nodes, ext->prims,
                         ext->n_prims, img, &why)) {
            rt_scene_destroy(sc);
            return fail(RT_ERR_INVALID, "rt_scene_create_bvh: " + why);
        }
    } else {
        build_bvh2(tri_v.data(), nt, img, RT_BVH_LEAF, RT_BVH_BINS, RT_BVH_CNODE);
    }
    // the traversal stacks hold a sentinel plus one entry per level; the
    // builder (and the import) bound the depth (RT_BVH_DEPTH_CAP), so this
    // only guards it
    if (img.max_depth + 1 > RT_STACK) {
        rt_scene_destroy(sc);
        return fail(RT_ERR_LIMIT, "rt_scene_create: BVH depth " + std::to_string(img.max_depth) +
                                      " exceeds the traversal stack (" + std::to_string(RT_STACK) + " entries)");
    }
    const float4 *np = nullptr, *tp = nullptr;
    if ((st = upload(sc, reinterpret_cast<const float4 *>(img.nodes.data()), (size_t)img.n_nodes * 4, &np)) != RT_OK) { rt_scene_destroy(sc); return st; }
    if ((st = upload(sc, reinterpret_cast<const float4 *>(img.tri_slots.data()), (size_t)img.n_slots * 3, &tp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.nodes = np; S.tri_slots = tp; S.n_nodes = img.n_nodes;
    if (nt > 0) {
        // refit data: internal nodes by depth (children before parents when
        // taken deepest level first), the indices, what refit cannot redo
        std::vector<int> depth(img.n_nodes, 0), order;
        std::vector<std::vector<int>> by_level(1, std::vector<int>{0});
        for (size_t l = 0; l < by_level.size(); l++)
            for (int nd : by_level[l])
                for (int k = 0; k < 2; k++) {
                    int32_t link;
                    std::memcpy(&link, &img.nodes[16 * (size_t)nd + 12 + k], 4);
                    if (link < 0 || link == nd) continue;
                    if (l + 1 >= by_level.size()) by_level.emplace_back();
                    by_level[l + 1].push_back(link);
                }
        sc->level_off.assign(1, 0);
        for (size_t l = by_level.size(); l-- > 0;) {
            order.insert(order.end(), by_level[l].begin(), by_level[l].end());
            sc->level_off.push_back((int)order.size());
        }
        if ((st = upload(sc, order.data(), order.size(), &sc->refit_order)) != RT_OK) { rt_scene_destroy(sc); return st; }
        if ((st = upload(sc, d->indices, 3 * (size_t)nt, &sc->indices_dev)) != RT_OK) { rt_scene_destroy(sc); return st; }
        sc->n_vertices = d->n_vertices;
        sc->n_tris = nt;
        sc->has_normals = d->normals != nullptr;
        for (int m = 0; m < d->n_meshes && sc->refit_why.empty(); m++) {
            const rt_mesh_desc &M = d->meshes[m];
            if (M.n_tris == 0) continue;
            if (M.light >= 0) sc->refit_why = "an emissive mesh (its area CDF would change)";
            const bool owner = (M.interior >= 0 && d->media[M.interior].type == RT_MEDIUM_HETEROGENEOUS) ||
                               (M.exterior >= 0 && d->media[M.exterior].type == RT_MEDIUM_HETEROGENEOUS);
            if (owner) sc->refit_why = "a mesh that bounds a grid medium (the medium's box would change)";
        }
        if (sc->refit_why.empty())
            for (int l = 0; l < d->n_lights; l++)
                if (d->lights[l].type != RT_LIGHT_ENV && d->lights[l].type != RT_LIGHT_POINT &&
                    d->lights[l].type != RT_LIGHT_SPOT && d->lights[l].shape_kind == RT_SHAPE_MESH)
                    sc->refit_why = "a mesh light";
    }
    {
        // the 4-wide traversal pushes up to three children per level; a tree
        // too deep for its stack is not uploaded and renders use the BVH2
        Bvh4Image w4;
        build_bvh4(img, w4);
        if (nt > 0 && 3 * (w4.max_depth + 1) + 1 > RT_STACK4) w4 = Bvh4Image();
        const float4 *n4 = nullptr;
        if ((st = upload(sc, reinterpret_cast<const float4 *>(w4.nodes.data()), (size_t)w4.n_nodes * 8, &n4)) != RT_OK) { rt_scene_destroy(sc); return st; }
        S.nodes4 = n4; S.n_nodes4 = w4.n_nodes;
        if ((st = upload(sc, w4.src.data(), w4.src.size(), &sc->bvh4_src)) != RT_OK) { rt_scene_destroy(sc); return st; }
        sc->w4_ok = nt == 0 || w4.n_nodes > 0;
    }
    {
        WideBvhImage wimg;
        build_wbvh8(tri_v.data(), nt, wimg, 32);
        // the group stack holds one entry per level and node indices < 2^23;
        // a tree outside either limit is not uploaded and renders use the BVH2
        if (nt > 0 && (wimg.max_depth + 1 > RT_WSTACK || wimg.n_nodes >= (1 << 23))) wimg = WideBvhImage();
        const float4 *wn = nullptr, *wt = nullptr;
        if ((st = upload(sc, reinterpret_cast<const float4 *>(wimg.nodes.data()), (size_t)(nt > 0 ? wimg.n_nodes : 0) * 5, &wn)) != RT_OK) { rt_scene_destroy(sc); return st; }
        if ((st = upload(sc, reinterpret_cast<const float4 *>(wimg.tri_slots.data()), (size_t)wimg.n_slots * 3, &wt)) != RT_OK) { rt_scene_destroy(sc); return st; }
        S.wnodes = wn; S.wtri = wt; S.n_wnodes = nt > 0 ? wimg.n_nodes : 0;
        sc->wide_depth = wimg.max_depth;
        sc->wide_ok = nt == 0 || wimg.n_nodes > 0;
    }
    }   // host-built tree
    if (!tri_n.empty()) { if ((st = upload(sc, tri_n.data(), tri_n.size(), &fp)) != RT_OK) { rt_scene_destroy(sc); return st; } S.tri_n = fp; }
    if (!tri_uv.empty()) { if ((st = upload(sc, tri_uv.data(), tri_uv.size(), &fp)) != RT_OK) { rt_scene_destroy(sc); return st; } S.tri_uv = fp; }
    // textures: all texels in one buffer, one DevTexture each
    if (d->n_textures > 0) {
        size_t total = 0;
        for (int i = 0; i < d->n_textures; i++) total += 3 * (size_t)d->textures[i].width * d->textures[i].height;
        std::vector<float> texels(total);
        std::vector<size_t> off(d->n_textures);
        size_t o = 0;
        for (int i = 0; i < d->n_textures; i++) {
            const rt_texture_desc &T = d->textures[i];
            off[i] = o;
            std::memcpy(texels.data() + o, T.rgb, sizeof(float) * 3 * (size_t)T.width * T.height);
            o += 3 * (size_t)T.width * T.height;
        }
        if ((st = upload(sc, texels.data(), texels.size(), &fp)) != RT_OK) { rt_scene_destroy(sc); return st; }
        std::vector<DevTexture> tex(d->n_textures);
        for (int i = 0; i < d->n_textures; i++) {
            const rt_texture_desc &T = d->textures[i];
            tex[i].w = T.width; tex[i].h = T.height; tex[i].rgb = fp + off[i];
            tex[i].scale = T.scale; tex[i].invert_x = T.invert_x != 0; tex[i].invert_y = T.invert_y != 0;
        }
        const DevTexture *tp;
        if ((st = upload(sc, tex.data(), tex.size(), &tp)) != RT_OK) { rt_scene_destroy(sc); return st; }
        S.textures = tp;
        S.n_textures = d->n_textures;
    }
    for (const DevBsdf &b : bsdfs) {
        S.has_textured |= b.textured;
        S.has_mixed |= bsdf_queue_of(b) == RT_QUEUE_MIXED;
    }
    if ((st = upload(sc, tri_mesh.data(), tri_mesh.size(), &ip)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.tri_mesh = ip;
    {
        // BSDF type per triangle: the closest-hit trace sorts hits by it
        std::vector<uint8_t> tri_type(nt, 255);
        for (int t = 0; t < nt; t++) {
            int b = d->meshes[tri_mesh[t]].bsdf;
            if (b >= 0) tri_type[t] = (uint8_t)bsdf_queue_of(bsdfs[b]);
        }
        const uint8_t *tp8;
        if ((st = upload(sc, tri_type.data(), tri_type.size(), &tp8)) != RT_OK) { rt_scene_destroy(sc); return st; }
        S.tri_type = tp8;
    }
    const DevMesh *mp;
    if ((st = upload(sc, meshes.data(), meshes.size(), &mp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.meshes = mp; S.n_meshes = d->n_meshes;
    if ((st = upload(sc, mesh_cdf.data(), mesh_cdf.size(), &fp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.mesh_cdf = fp;
    const DevSphere *spp;
    if ((st = upload(sc, spheres.data(), spheres.size(), &spp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.spheres = spp; S.n_spheres = d->n_spheres;
    const DevBsdf *bp;
    if ((st = upload(sc, bsdfs.data(), bsdfs.size(), &bp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.bsdfs = bp;
    const DevLight *lp;
    if ((st = upload(sc, lights.data(), lights.size(), &lp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.lights = lp; S.n_lights = d->n_lights; S.env_light = d->env_light;
    const DevMedium *mdp;
    if ((st = upload(sc, media.data(), media.size(), &mdp)) != RT_OK) { rt_scene_destroy(sc); return st; }
    S.media = mdp;
    // camera
    const rt_camera_desc &cd = d->camera;
    S.cam.width = cd.width; S.cam.height = cd.height;
    std::memcpy(S.cam.sample_to_camera, cd.sample_to_camera, sizeof(S.cam.sample_to_camera));
    std::memcpy(S.cam.camera_to_world, cd.camera_to_world, sizeof(S.cam.camera_to_world));
    S.cam.near_clip = cd.near_clip; S.cam.far_clip = cd.far_clip;
    S.cam.aperture_radius = cd.aperture_radius; S.cam.focal_plane = cd.focal_plane;
    S.cam.inv_w = 1.f / (float)cd.width; S.cam.inv_h = 1.f / (float)cd.height;
    S.cam.medium = cd.medium;
    {
        S.cam.filter = cd.filter;
        S.cam.frx = cd.filter_radius[0];
        S.cam.fry = cd.filter_radius[1];
        S.cam.ov_x = (int)ceilf(cd.filter_radius[0] - 0.5f);
        S.cam.ov_y = (int)ceilf(cd.filter_radius[1] - 0.5f);
        float tab[1024];
        filter_table(cd, tab);
        const float *tp;
        if ((st = upload(sc, tab, 1024, &tp)) != RT_OK) { rt_scene_destroy(sc); return st; }
        S.cam.filter_table = tp;
    }
    sc->n_lights = d->n_lights;
    sc->n_bsdfs = d->n_bsdfs;
    sc->n_media = d->n_media;
    for (int b = 0; b < d->n_bsdfs; b++) sc->bsdf_types |= 1 << bsdf_queue_of(bsdfs[b]);
    *out = sc;
    return RT_OK;
}

rt_status rt_scene_create(rt_ctx *ctx, const rt_scene_desc *d, rt_scene **out)
{
    return scene_create(ctx, d, nullptr, out);
}

rt_status rt_scene_create_bvh(rt_ctx *ctx, const rt_scene_desc *d, const rt_bvh_node *nodes, int32_t n_nodes,
                              const int32_t *prims, int32_t n_prims, rt_scene **out)
{
    if (n_nodes < 0 || n_prims < 0 || (n_nodes > 0 && !nodes) || (n_prims > 0 && !prims))
        return fail(RT_ERR_INVALID, "rt_scene_create_bvh: bad tree arguments");
    ExtTree t{nodes, n_nodes, prims, n_prims};
    return scene_create(ctx, d, &t, out);
}

rt_status rt_bvh_import_check(const float *tri_v, int32_t n, const rt_bvh_node *nodes, int32_t n_nodes,
                              const int32_t *prims, int32_t n_prims, int32_t *max_depth, int32_t *n_device_nodes)
{
    if (n < 0 || (n > 0 && !tri_v) || n_nodes < 0 || n_prims < 0 || (n_nodes > 0 && !nodes) || (n_prims > 0 && !prims))
        return fail(RT_ERR_INVALID, "rt_bvh_import_check: bad argument");
    BvhImage img;
    std::string why;
    if (!import_bvh2(tri_v, n, reinterpret_cast<const ExtNode *>(nodes), n_nodes, prims, n_prims, img, &why))
        return fail(RT_ERR_INVALID, "rt_bvh_import_check: " + why);
    int walked = 0;
    if (n > 0 && !check_bvh2(img, tri_v, n, &walked, &why))
        return fail(RT_ERR_INVALID, "rt_bvh_import_check: malformed image: " + why);
    if (max_depth) *max_depth = img.max_depth;
    if (n_device_nodes) *n_device_nodes = img.n_nodes;
    return RT_OK;
}

rt_status rt_bvh_stats(const float *tri_v, int32_t n, int32_t width, int32_t depth_cap, int32_t *max_depth,
                       int32_t *n_nodes)
{
    if (n < 0 || (n > 0 && !tri_v) || (width != 2 && width != 4 && width != 8) || depth_cap > RT_BVH_DEPTH_CAP)
        return fail(RT_ERR_INVALID, "rt_bvh_stats: bad argument");
    if (depth_cap <= 0) depth_cap = RT_BVH_DEPTH_CAP;
    if (n > 0 && (int64_t(1) << std::min(depth_cap, 62)) < (int64_t)n)
        return fail(RT_ERR_INVALID, "rt_bvh_stats: depth_cap below log2 of the triangle count");
    int d = 0, nn = 0;
    if (width == 2) {
        BvhImage img;
        build_bvh2(tri_v, n, img, RT_BVH_LEAF, RT_BVH_BINS, RT_BVH_CNODE, depth_cap);
        std::string why;
        int walked = 0;
        if (!check_bvh2(img, tri_v, n, &walked, &why)) return fail(RT_ERR_INVALID, "rt_bvh_stats: malformed tree: " + why);
        d = img.max_depth; nn = img.n_nodes;
    } else if (width == 4) {
        BvhImage img;
        build_bvh2(tri_v, n, img, RT_BVH_LEAF, RT_BVH_BINS, RT_BVH_CNODE, depth_cap);
        std::string why;
        int walked = 0;
        if (!check_bvh2(img, tri_v, n, &walked, &why)) return fail(RT_ERR_INVALID, "rt_bvh_stats: malformed tree: " + why);
        Bvh4Image w4;
        build_bvh4(img, w4);
        if (!check_bvh4(w4, img, &why)) return fail(RT_ERR_INVALID, "rt_bvh_stats: malformed 4-wide tree: " + why);
        d = w4.max_depth; nn = w4.n_nodes;
    } else {
        WideBvhImage img;
        build_wbvh8(tri_v, n, img, 32, depth_cap);
        d = img.max_depth; nn = img.n_nodes;
    }
    if (max_depth) *max_depth = d;
    if (n_nodes) *n_nodes = nn;
    return RT_OK;
}

static rt_status launch_check(const char *what);

rt_status rt_scene_refit(rt_ctx *ctx, rt_scene *sc, const float *vertices, const float *normals, int32_t on_device)
{
    if (!ctx || !sc || !vertices) return fail(RT_ERR_INVALID, "rt_scene_refit: null argument");
    if (sc->ctx != ctx) return fail(RT_ERR_INVALID, "rt_scene_refit: the scene belongs to another context");
    if (!sc->indices_dev || sc->n_tris == 0) return RT_OK;   // no triangles: nothing to refit
    if (!sc->refit_why.empty()) return fail(RT_ERR_UNSUPPORTED, "rt_scene_refit: the scene has " + sc->refit_why);
    if ((normals != nullptr) != sc->has_normals)
        return fail(RT_ERR_INVALID, sc->has_normals ? "rt_scene_refit: the scene has vertex normals: pass new ones"
                                                    : "rt_scene_refit: the scene has no vertex normals");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t nv = (size_t)sc->n_vertices;
    const int n_tris = sc->n_tris;
    // the new positions (and normals) on the device
    const float *vd = vertices, *nd_ = normals;
    void *tmp = nullptr;
    if (!on_device) {
        CK(cudaMalloc(&tmp, 3 * nv * sizeof(float) * (normals ? 2 : 1)));
        CK(cudaMemcpyAsync(tmp, vertices, 3 * nv * sizeof(float), cudaMemcpyHostToDevice, st));
        vd = (const float *)tmp;
        if (normals) {
            CK(cudaMemcpyAsync((float *)tmp + 3 * nv, normals, 3 * nv * sizeof(float), cudaMemcpyHostToDevice, st));
            nd_ = (const float *)tmp + 3 * nv;
        }
    }
    rt_status s = RT_OK;
    if (!sc->refit_boxes && cudaMalloc((void **)&sc->refit_boxes, 12 * sizeof(float) * (size_t)sc->S.n_nodes) != cudaSuccess) {
        cudaFree(tmp);
        return fail(RT_ERR_NOMEM, "rt_scene_refit: box scratch allocation failed");
    }
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    auto grid = [&](int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm * 16)); };
    k_refit_tris<<<grid(n_tris), 256, 0, st>>>(vd, nd_, sc->indices_dev, n_tris, const_cast<float *>(sc->S.tri_v),
                                               const_cast<float *>(sc->S.tri_n));
    k_refit_slots<<<grid(n_tris), 256, 0, st>>>(const_cast<float4 *>(sc->S.tri_slots), n_tris, sc->S.tri_v);
    for (size_t l = 0; l + 1 < sc->level_off.size(); l++) {
        const int b = sc->level_off[l], e = sc->level_off[l + 1];
        k_refit_level<<<grid(e - b), 256, 0, st>>>(sc->S.nodes, sc->S.tri_slots, sc->S.tri_v, sc->refit_order, b, e,
                                                    sc->refit_boxes);
    }
    k_refit_widen<<<grid(sc->S.n_nodes), 256, 0, st>>>(const_cast<float4 *>(sc->S.nodes), sc->S.n_nodes, sc->refit_boxes);
    if (sc->S.n_nodes4 > 0)
        k_refit_bvh4<<<grid(4 * (int64_t)sc->S.n_nodes4), 256, 0, st>>>(const_cast<float *>(reinterpret_cast<const float *>(sc->S.nodes4)),
                                                                        sc->S.n_nodes4, sc->bvh4_src, sc->S.nodes);
    if ((s = launch_check("refit kernels")) != RT_OK) { cudaFree(tmp); return s; }
    // the scene box: the tree's root box and the analytic shapes'
    float root[12];
    cudaError_t e = cudaMemcpyAsync(root, sc->refit_boxes, sizeof(root), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("rt_scene_refit: ") + cudaGetErrorString(e));
    for (int a = 0; a < 3; a++) {
        float mn = root[a], mx = root[3 + a];
        if (root[6] <= root[9]) { mn = std::min(mn, root[6 + a]); mx = std::max(mx, root[9 + a]); }
        mn = std::min(mn, sc->sph_bounds[a]);
        mx = std::max(mx, sc->sph_bounds[3 + a]);
        sc->bounds[a] = sc->S.bmin[a] = mn;
        sc->bounds[3 + a] = sc->S.bmax[a] = mx;
    }
    // the compressed 8-wide tree is not refitted: renders at width 8 use the binary tree
    sc->S.n_wnodes = 0;
    sc->wide_ok = false;
    return RT_OK;
}

rt_status rt_scene_info(const rt_scene *sc, float bounds[6], int64_t *device_bytes, int32_t *bvh_nodes)
{
    if (!sc) return fail(RT_ERR_INVALID, "null scene");
    if (bounds) std::memcpy(bounds, sc->bounds, sizeof(sc->bounds));
    if (device_bytes) *device_bytes = sc->bytes;
    if (bvh_nodes) *bvh_nodes = sc->S.n_nodes;
    return RT_OK;
}

// ---------------------------------------------------------------- wavefront buffers
static rt_status ensure_wave(rt_ctx *c, int capacity, int max_rounds);
// the VolPath wavefront's extra path state (after ensure_wave, which frees it
// when it reallocates)
static rt_status ensure_vw(rt_ctx *c, int capacity)
{
    if (c->W.vw_capacity >= capacity) return RT_OK;
    Wave &W = c->W;
    const size_t P = (size_t)capacity;
    float4 **arr[6] = {&W.v_seg, &W.v_p, &W.v_li0, &W.v_li1, &W.v_li2, &W.v_val};
    for (float4 **a : arr) {
        void *p = nullptr;
        if (cudaMalloc(&p, P * sizeof(float4)) != cudaSuccess) {
            cudaGetLastError();
            return fail(RT_ERR_NOMEM, "VolPath wavefront buffer allocation failed");
        }
        c->wave_allocs.push_back(p);
        *a = (float4 *)p;
    }
    W.vw_capacity = capacity;
    return RT_OK;
}

// the per-slot allocations of ensure_wave and (VolPathTracing) ensure_vw
extern "C" int64_t rt_path_state_bytes(int32_t integrator)
{
    if (integrator != RT_INTEGRATOR_PATH_MIS && integrator != RT_INTEGRATOR_VOLPATH) return 0;
    const bool volpath = integrator == RT_INTEGRATOR_VOLPATH;
    const int64_t wave = sizeof(Pcg32) +
                         10 * sizeof(float4) +                 // tp rad ray_o ray_d hit bs nee sh_o sh_d out
                         3 * sizeof(int) +                     // rel_eta flags occl
                         2 +                                   // splat pix_irregular
                         (4 + RT_NBSDF + 1) * sizeof(int) +    // fin end closest shadow, material, mixed queues
                         3 * sizeof(int);                      // sid, sort keys and scratch
    return wave + (volpath ? 6 * (int64_t)sizeof(float4) : 0);   // v_seg v_p v_li0 v_li1 v_li2 v_val
}

static rt_status ensure_wave(rt_ctx *c, int capacity, int max_rounds)
{
    if (c->capacity >= capacity && c->W.max_rounds >= max_rounds) return RT_OK;
    free_wave(c);
    Wave &W = c->W;
    size_t P = (size_t)capacity;
    auto alloc = [&](void **p, size_t bytes) -> bool {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) return false;
        c->wave_allocs.push_back(*p);
        return true;
    };
    bool ok = true;
    ok &= alloc((void **)&W.rng, P * sizeof(Pcg32));
    ok &= alloc((void **)&W.tp, P * sizeof(float4));
    ok &= alloc((void **)&W.rad, P * sizeof(float4));
    ok &= alloc((void **)&W.ray_o, P * sizeof(float4));
    ok &= alloc((void **)&W.ray_d, P * sizeof(float4));
    ok &= alloc((void **)&W.hit, P * sizeof(float4));
    ok &= alloc((void **)&W.bs, P * sizeof(float4));
    ok &= alloc((void **)&W.rel_eta, P * sizeof(float));
    ok &= alloc((void **)&W.flags, P * sizeof(int));
    ok &= alloc((void **)&W.nee, P * sizeof(float4));
    ok &= alloc((void **)&W.sh_o, P * sizeof(float4));
    ok &= alloc((void **)&W.sh_d, P * sizeof(float4));
    ok &= alloc((void **)&W.occl, P * sizeof(int));
    ok &= alloc((void **)&W.out, P * sizeof(float4));
    ok &= alloc((void **)&W.splat, P);
    ok &= alloc((void **)&W.pix_irregular, P);
    ok &= alloc((void **)&W.q_fin, P * sizeof(int));
    ok &= alloc((void **)&W.q_end, P * sizeof(int));
    ok &= alloc((void **)&W.q_closest, P * sizeof(int));
    ok &= alloc((void **)&W.q_shadow, P * sizeof(int));
    for (int t = 0; t < RT_NBSDF; t++) ok &= alloc((void **)&W.q_mat[t], P * sizeof(int));
    ok &= alloc((void **)&W.q_mixed, P * sizeof(int));
    ok &= alloc((void **)&W.cnt, (size_t)(max_rounds + 2) * sizeof(RoundCounters));
    ok &= alloc((void **)&W.sid, P * sizeof(int));
    ok &= alloc((void **)&W.sort_keys, P * sizeof(unsigned));
    ok &= alloc((void **)&W.sort_tmp, P * sizeof(int));
    ok &= alloc((void **)&W.sort_hist, (size_t)RT_SORT_BINS * sizeof(unsigned));
    if (!ok) { free_wave(c); return fail(RT_ERR_NOMEM, "wavefront buffer allocation failed"); }
    W.capacity = capacity;
    W.max_rounds = max_rounds;
    c->capacity = capacity;
    return RT_OK;
}

static rt_status launch_check(const char *what);
// reorder the round's closest-hit (shadow = 0) or shadow (shadow = 1) queue
static rt_status sort_rays(rt_ctx *ctx, const RenderParams &P, int round, int shadow, int64_t &launches)
{
    cudaStream_t st = ctx->stream;
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    CK(cudaMemsetAsync(ctx->W.sort_hist, 0, (size_t)RT_SORT_BINS * sizeof(unsigned), st));
    k_sort_count<<<sm * 8, 256, 0, st>>>(P, round, shadow);
    k_sort_scan<<<1, 1024, 0, st>>>(P);
    k_sort_scatter<<<sm * 8, 256, 0, st>>>(P, round, shadow);
    k_sort_copy<<<sm * 8, 256, 0, st>>>(P, round, shadow);
    launches += 4;
    return launch_check("ray reordering");
}

static rt_status launch_check(const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return RT_OK;
}

// One wavefront batch as a CUDA graph: reset the batch's counters and the
// device round index, camera rays, then a conditional WHILE node whose body
// is one round (PathTracingMIS: closest-hit trace, shadow trace, finish,
// shading; VolPath: its five kernels; then k_round_next), then the film
// reduction.  The graph is built once
// per distinct set of launch parameters and kept; the conditional handle it
// owns is only ever set by its own k_round_next.
static rt_status pt_batch_graph(rt_ctx *ctx, rt_scene *sc, const RenderParams &P, float4 *film, bool box_film,
                                int accumulate, int Wd, int t0, int t1, int tiles_x, int bx, int by, int max_rounds,
                                int round_buf, bool vw)
{
    cudaStream_t st = ctx->cap_stream;   // capture; the graph runs on ctx->stream
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const int cam_blocks = std::min((P.n_paths + 255) / 256, sm * 16);
    const int trace_blocks = sm * ctx->trace_bpsm, shade_blocks = sm * ctx->shade_bpsm;
    const int width = trace_width(ctx, sc);
    const int types = sc->bsdf_types | (P.sort_threshold > 0 ? 1 << RT_QUEUE_MIXED : 0);
    const size_t npix_all = (size_t)Wd * sc->S.cam.height;
    struct Tail {
        const void *film;
        int box, accumulate, wd, t0, t1, tiles_x, bx, by, max_rounds, round_buf, cam_blocks, trace_blocks,
            shade_blocks, width, types, vw;
    } tail;
    std::memset(&tail, 0, sizeof(tail));
    tail.film = film; tail.box = box_film; tail.accumulate = accumulate; tail.wd = Wd; tail.t0 = t0; tail.t1 = t1;
    tail.tiles_x = tiles_x; tail.bx = bx; tail.by = by; tail.max_rounds = max_rounds; tail.round_buf = round_buf;
    tail.cam_blocks = cam_blocks; tail.trace_blocks = trace_blocks; tail.shade_blocks = shade_blocks;
    tail.width = width; tail.types = types; tail.vw = vw;
    std::vector<unsigned char> key(sizeof(RenderParams) + sizeof(Tail));
    std::memcpy(key.data(), &P, sizeof(RenderParams));
    std::memcpy(key.data() + sizeof(RenderParams), &tail, sizeof(Tail));
    cudaGraphExec_t exec = nullptr;
    for (auto &e : ctx->gcache)
        if (e.key == key) { exec = e.exec; break; }
    if (exec) {
        ctx->graph_hits++;
    } else {
        cudaGraph_t g = nullptr;
        bool body_capturing = false;
        const char *what = nullptr;
        auto bad = [&](cudaError_t e, const char *w) {
            if (e != cudaSuccess && !what) what = w;
            return e != cudaSuccess;
        };
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        do {
            if (bad(cudaMemsetAsync(P.W.pix_irregular, 0, (size_t)P.npix, st), "memset")) break;
            if (bad(cudaMemsetAsync(P.W.cnt, 0, sizeof(RoundCounters) * (size_t)(round_buf + 2), st), "memset")) break;
            if (bad(cudaMemsetAsync(P.round_dev, 0, sizeof(int), st), "memset")) break;
            k_camera<<<cam_blocks, 256, 0, st>>>(P);
            if (bad(cudaGetLastError(), "k_camera")) break;
            cudaStreamCaptureStatus cst;
            cudaGraph_t cg = nullptr;
            const cudaGraphNode_t *deps = nullptr;
            size_t nd = 0;
            if (bad(cudaStreamGetCaptureInfo(st, &cst, nullptr, &cg, &deps, nullptr, &nd), "capture info")) break;
            cudaGraphConditionalHandle loop;
            if (bad(cudaGraphConditionalHandleCreate(&loop, cg, 1, cudaGraphCondAssignDefault), "conditional handle"))
                break;
            cudaGraphNodeParams cp = {};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = loop;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t cn;
            if (bad(cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &cp), "conditional node")) break;
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            cudaStream_t bs = ctx->body_stream;
            if (bad(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                    "body capture"))
                break;
            body_capturing = true;
            if (vw) {
                // one VolPath round (the next round's trace queue is its
                // counters' closest, which k_round_next tests)
                k_vw_trace_step<<<sm * RT_VW_MINB_STEP, 128, 0, bs>>>(P, 0);
                k_vw_shadow<<<sm * RT_VW_MINB_SHADOW, 128, 0, bs>>>(P, 0);
                k_vw_scatter<<<sm * RT_VW_MINB_TRSAMP, 128, 0, bs>>>(P, 0);
                k_vw_sample_surface<<<sm * RT_VW_MINB_SAMPLE, 128, 0, bs>>>(P, 0);
                k_vw_trsamp_finish<<<sm * RT_VW_MINB_TRSAMP, 128, 0, bs>>>(P, 0);
            } else {
                launch_trace(width, P, 0, false, false, trace_blocks, bs);
                launch_trace(width, P, 0, true, false, trace_blocks, bs);
                k_pt_finish<<<shade_blocks, 128, 0, bs>>>(P, 0);
                launch_shades(types, P, 0, shade_blocks, bs);
            }
            k_round_next<<<1, 1, 0, bs>>>(P, loop, max_rounds);
            if (bad(cudaGetLastError(), "round kernels")) break;
            body_capturing = false;
            if (bad(cudaStreamEndCapture(bs, &body), "body capture end")) break;
            if (bad(cudaStreamUpdateCaptureDependencies(st, &cn, nullptr, 1, cudaStreamSetCaptureDependencies),
                    "capture dependencies"))
                break;
            if (box_film) k_film<<<(P.npix + 127) / 128, 128, 0, st>>>(P, film, Wd, accumulate);
            else k_film_wide<<<(int)((npix_all + 127) / 128), 128, 0, st>>>(P, film, t0, t1, tiles_x, bx, by);
            if (bad(cudaGetLastError(), "film kernel")) break;
        } while (0);
        if (body_capturing) {
            cudaGraph_t bg = nullptr;
            cudaStreamEndCapture(ctx->body_stream, &bg);
        }
        cudaError_t ee = cudaStreamEndCapture(st, &g);
        if (!what && ee != cudaSuccess) what = "capture end";
        if (!what && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) what = "instantiate";
        if (g) cudaGraphDestroy(g);
        if (what) {
            cudaGetLastError();
            if (exec) cudaGraphExecDestroy(exec);
            return fail(RT_ERR_CUDA, std::string("render graph: ") + what + " failed");
        }
        if (ctx->gcache.size() >= 8) {
            cudaGraphExecDestroy(ctx->gcache.front().exec);
            ctx->gcache.erase(ctx->gcache.begin());
        }
        ctx->gcache.push_back({std::move(key), exec});
        ctx->graph_builds++;
    }
    CK(cudaGraphLaunch(exec, ctx->stream));
    return RT_OK;
}

rt_status rt_render(rt_ctx *ctx, rt_scene *sc, const rt_render_desc *rd, float *film_rgbw, int32_t on_device)
{
    if (!ctx || !sc || !rd || !film_rgbw) return fail(RT_ERR_INVALID, "rt_render: null argument");
    if (rd->spp <= 0 || rd->sample_begin < 0) return fail(RT_ERR_INVALID, "rt_render: bad sample range");
    if (rd->integrator != RT_INTEGRATOR_PATH_MIS && rd->integrator != RT_INTEGRATOR_VOLPATH)
        return fail(RT_ERR_UNSUPPORTED, "rt_render: unknown integrator");
    if (rd->max_depth < 0 || rd->min_depth < 0) return fail(RT_ERR_INVALID, "rt_render: negative depth");
    if (rd->flags & ~RT_RENDER_ACCUMULATE) return fail(RT_ERR_INVALID, "rt_render: unknown flags");
    const int accumulate = (rd->flags & RT_RENDER_ACCUMULATE) ? 1 : 0;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const DevCamera &cam = sc->S.cam;
    const int Wd = cam.width, H = cam.height;
    const int bx = rd->block_x > 0 ? rd->block_x : 32, by = rd->block_y > 0 ? rd->block_y : 32;
    if (bx > 0xffff || by > 0xffff) return fail(RT_ERR_INVALID, "block size too large");
    const int tiles_x = (Wd + bx - 1) / bx, tiles_y = (H + by - 1) / by;
    const size_t npix_all = (size_t)Wd * H;
    // tile-order table (Scene.cpp:83-95 job grid, SampleJob.cpp:40-44 pixel
    // loops); uploaded once per film size / block size
    bool same_tiles = ctx->tile_key[0] == Wd && ctx->tile_key[1] == H && ctx->tile_key[2] == bx && ctx->tile_key[3] == by;
    if (!same_tiles) {
        std::vector<int4> order(npix_all);
        ctx->tile_start.assign(tiles_x * tiles_y + 1, 0);
        size_t g = 0;
        for (int ty = 0; ty < tiles_y; ty++)
            for (int tx = 0; tx < tiles_x; tx++) {
                ctx->tile_start[ty * tiles_x + tx] = (int)g;
                int ox = tx * bx, oy = ty * by;
                int tw = std::min(Wd, ox + bx) - ox, th = std::min(H, oy + by) - oy;
                for (int y = 0; y < th; y++)
                    for (int x = 0; x < tw; x++) order[g++] = make_int4(ox + x, oy + y, x | (y << 16), tw | (th << 16));
            }
        ctx->tile_start[tiles_x * tiles_y] = (int)g;
        if (ctx->tileorder_n < npix_all) {
            cudaFree(ctx->tileorder);
            ctx->tileorder = nullptr;
            CK(cudaMalloc(&ctx->tileorder, npix_all * sizeof(int4)));
            ctx->tileorder_n = npix_all;
        }
        CK(cudaMemcpy(ctx->tileorder, order.data(), npix_all * sizeof(int4), cudaMemcpyHostToDevice));
        ctx->tile_key[0] = Wd; ctx->tile_key[1] = H; ctx->tile_key[2] = bx; ctx->tile_key[3] = by;
    }
    const std::vector<int> &tile_start = ctx->tile_start;
    // light selection CDF (Integrator::initialize, Integrator.cpp:24-38)
    {
        HCdf c;
        int n = sc->n_lights;
        float pu = (float)1. / (float)n;
        for (int l = 0; l < n; l++) c.add(rd->strategy == RT_STRATEGY_ONE_LIGHT_WEIGHTED ? sc->light_power_lum[l] : pu);
        c.normalize();
        if (ctx->light_cdf_n < (int)c.c.size()) {
            cudaFree(ctx->light_cdf);
            ctx->light_cdf = nullptr;
            CK(cudaMalloc(&ctx->light_cdf, c.c.size() * sizeof(float) + 64));
            ctx->light_cdf_n = (int)c.c.size();
        }
        CK(cudaMemcpyAsync(ctx->light_cdf, c.c.data(), c.c.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
    }
    // film target
    float4 *film = nullptr;
    if (on_device) film = reinterpret_cast<float4 *>(film_rgbw);
    else {
        if (ctx->film_n < npix_all) {
            cudaFree(ctx->film);
            ctx->film = nullptr;
            CK(cudaMalloc(&ctx->film, npix_all * sizeof(float4)));
            ctx->film_n = npix_all;
        }
        film = ctx->film;
        if (accumulate)
            CK(cudaMemcpyAsync(film, film_rgbw, npix_all * sizeof(float4), cudaMemcpyHostToDevice, st));
    }
    // the box filter of radius 0.5 reduces per batch pixel (k_film); any other
    // filter gathers into a zeroed (or, accumulating, the given) film
    const bool box_film = cam.filter == RT_FILTER_BOX && cam.frx == 0.5f && cam.fry == 0.5f;
    if (!box_film && !accumulate) CK(cudaMemsetAsync(film, 0, npix_all * sizeof(float4), st));
    // batch capacity: whole tiles, all samples of their pixels, up to
    // ctx->wave_paths paths (fewer, longer-tailed batches cost more: the last
    // rounds of a batch hold few paths and run at the traversal latency floor)
    const int cap_target = ctx->wave_paths;
    const int ntiles = tiles_x * tiles_y;
    int tile_pix = bx * by;
    if ((int64_t)tile_pix * rd->spp > (1 << 26)) return fail(RT_ERR_LIMIT, "one tile's samples exceed the path capacity");
    int tiles_per_batch = std::max(1, cap_target / std::max(1, tile_pix * rd->spp));
    int capacity = std::min(tiles_per_batch, ntiles) * tile_pix * rd->spp;
    if (rd->integrator == RT_INTEGRATOR_PATH_MIS && rd->max_depth > (1 << 16))
        return fail(RT_ERR_LIMIT, "rt_render: max_depth above 65536 is not provided by the device path");
    // rounds: PathTracingMIS, a bounce each; the VolPath wavefront, a
    // vol_step each, capped like the megakernel's 2^16 steps per path
    const bool vw = rd->integrator == RT_INTEGRATOR_VOLPATH && ctx->volpath_wave;
    int max_rounds = rd->integrator == RT_INTEGRATOR_PATH_MIS ? rd->max_depth + 3 : vw ? (1 << 16) + 2 : 1;
    int round_buf = max_rounds;
    rt_status s = ensure_wave(ctx, capacity, round_buf);
    if (s != RT_OK) return s;
    if (vw && (s = ensure_vw(ctx, capacity)) != RT_OK) return s;
    CK(cudaMemsetAsync(ctx->stats, 0, sizeof(unsigned long long) * 8, st));
    CK(cudaMemsetAsync(ctx->limit_flag, 0, sizeof(int), st));
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.S = sc->S;
    P.S.limit_flag = ctx->limit_flag;
    P.S.light_cdf = ctx->light_cdf;
    P.W = ctx->W;
    P.tileorder = ctx->tileorder;
    P.seed = rd->seed;
    P.max_depth = rd->max_depth;
    P.min_depth = rd->min_depth;
    P.limit_flag = ctx->limit_flag;
    P.stats = ctx->stats;
    P.spp = rd->spp;
    P.sample_begin = rd->sample_begin;
    P.sort_threshold = ctx->sort_threshold;
    P.all_lights = rd->integrator == RT_INTEGRATOR_PATH_MIS && rd->strategy == RT_STRATEGY_ALL_LIGHTS;
    // shading queues in use: the scene's (textured BSDFs in the mixed one),
    // and the mixed one for bounces below the sort threshold
    const int types = sc->bsdf_types | (P.sort_threshold > 0 ? 1 << RT_QUEUE_MIXED : 0);
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    int64_t launches = 0, trace_c_launches = 0, trace_a_launches = 0;
    int64_t total_paths = 0;
    // one CUDA graph per PathTracingMIS or VolPath-wavefront batch (rt_ctx_set_graphs)
    const bool use_graph = ctx->graphs && !ctx->profiling && !ctx->ray_sort &&
                           (rd->integrator == RT_INTEGRATOR_PATH_MIS || vw);
    int graph_batches = 0;
    if (use_graph) {
        if (!ctx->round_dev) CK(cudaMalloc(&ctx->round_dev, sizeof(int)));
        if (!ctx->body_stream) CK(cudaStreamCreateWithFlags(&ctx->body_stream, cudaStreamNonBlocking));
        if (!ctx->cap_stream) CK(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
        P.round_dev = ctx->round_dev;
    }
    ctx->ev_used = 0;
    CK(cudaEventRecord(ctx->ev0, st));
    for (int t0 = 0; t0 < ntiles; t0 += tiles_per_batch) {
        int t1 = std::min(ntiles, t0 + tiles_per_batch);
        P.g0 = tile_start[t0];
        P.npix = tile_start[t1] - tile_start[t0];
        P.n_paths = P.npix * rd->spp;
        total_paths += P.n_paths;
        if (use_graph) {
            if ((s = pt_batch_graph(ctx, sc, P, film, box_film, accumulate, Wd, t0, t1, tiles_x, bx, by, max_rounds,
                                    round_buf, vw)) != RT_OK)
                return s;
            graph_batches++;
            continue;
        }
        CK(cudaMemsetAsync(ctx->W.pix_irregular, 0, (size_t)P.npix, st));
        CK(cudaMemsetAsync(ctx->W.cnt, 0, sizeof(RoundCounters) * (size_t)(round_buf + 2), st));
        int cam_blocks = std::min((P.n_paths + 255) / 256, sm * 16);
        prof_begin(ctx, K_CAMERA);
        k_camera<<<cam_blocks, 256, 0, st>>>(P);
        prof_end(ctx);
        launches++;
        if ((s = launch_check("k_camera")) != RT_OK) return s;
        if (rd->integrator == RT_INTEGRATOR_VOLPATH && ctx->volpath_wave) {
            // one round = one vol_step of every live path (five kernels)
            prof_begin(ctx, K_VOLPATH);
            for (int r = 0; r < max_rounds; r++) {
                k_vw_trace_step<<<sm * RT_VW_MINB_STEP, 128, 0, st>>>(P, r);
                k_vw_shadow<<<sm * RT_VW_MINB_SHADOW, 128, 0, st>>>(P, r);
                k_vw_scatter<<<sm * RT_VW_MINB_TRSAMP, 128, 0, st>>>(P, r);
                k_vw_sample_surface<<<sm * RT_VW_MINB_SAMPLE, 128, 0, st>>>(P, r);
                k_vw_trsamp_finish<<<sm * RT_VW_MINB_TRSAMP, 128, 0, st>>>(P, r);
                launches += 5;
                if ((s = launch_check("VolPath round")) != RT_OK) return s;
                if ((r & 3) == 3 && r + 1 < max_rounds) {
                    int nq = 0;
                    CK(cudaMemcpyAsync(&nq, &ctx->W.cnt[r + 1].closest, sizeof(int), cudaMemcpyDeviceToHost, st));
                    CK(cudaStreamSynchronize(st));
                    if (nq == 0) break;
                }
            }
            prof_end(ctx);
        } else if (rd->integrator == RT_INTEGRATOR_VOLPATH) {
            CK(cudaMemsetAsync(ctx->work, 0, sizeof(int), st));
            prof_begin(ctx, K_VOLPATH);
            k_volpath<<<sm * RT_VOLPATH_GRID, 128, 0, st>>>(P, ctx->work);
            prof_end(ctx);
            launches++;
            if ((s = launch_check("k_volpath")) != RT_OK) return s;
        } else {
            int trace_blocks = sm * ctx->trace_bpsm;
            int shade_blocks = sm * ctx->shade_bpsm;
            for (int r = 0; r < max_rounds; r++) {
                int ri = r;
                const bool cnt2 = ctx->profiling >= 2;
                const int width = trace_width(ctx, sc);
                if (ctx->ray_sort && ri > 0) {
                    prof_begin(ctx, K_SORT);
                    if ((s = sort_rays(ctx, P, ri, 0, launches)) != RT_OK) return s;
                    if ((s = sort_rays(ctx, P, ri, 1, launches)) != RT_OK) return s;
                    prof_end(ctx);
                }
                prof_begin(ctx, K_TRACE_C);
                launch_trace(width, P, ri, false, cnt2, trace_blocks, st);
                prof_end(ctx);
                prof_begin(ctx, K_TRACE_A);
                launch_trace(width, P, ri, true, cnt2, trace_blocks, st);
                prof_end(ctx);
                prof_begin(ctx, K_RESOLVE);
                k_pt_finish<<<shade_blocks, 128, 0, st>>>(P, ri);
                prof_end(ctx);
                prof_begin(ctx, K_SHADE);
                launch_shades(types, P, ri, shade_blocks, st);
                prof_end(ctx);
                launches += 3 + __builtin_popcount(types);
                trace_c_launches++;
                trace_a_launches++;
                if ((s = launch_check("pt round")) != RT_OK) return s;
                // cheap early exit: peek at the survivor counts every 4 rounds
                if ((r & 3) == 3 && r + 1 < max_rounds) {
                    RoundCounters nc;
                    CK(cudaMemcpyAsync(&nc, &ctx->W.cnt[ri + 1], sizeof(nc), cudaMemcpyDeviceToHost, st));
                    CK(cudaStreamSynchronize(st));
                    if (nc.closest == 0 && nc.end == 0) break;
                }
            }
        }
        prof_begin(ctx, K_FILM);
        if (box_film) {
            int fb = (P.npix + 127) / 128;
            k_film<<<fb, 128, 0, st>>>(P, film, Wd, accumulate);
        } else {
            k_film_wide<<<(int)((npix_all + 127) / 128), 128, 0, st>>>(P, film, t0, t1, tiles_x, bx, by);
        }
        prof_end(ctx);
        launches++;
        if ((s = launch_check("k_film")) != RT_OK) return s;
    }
    CK(cudaEventRecord(ctx->ev1, st));
    if (!on_device)
        CK(cudaMemcpyAsync(film_rgbw, film, npix_all * sizeof(float4), cudaMemcpyDeviceToHost, st));
    unsigned long long stats[8];
    int limit = 0;
    CK(cudaMemcpyAsync(stats, ctx->stats, sizeof(stats), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&limit, ctx->limit_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    std::memset(&ctx->last, 0, sizeof(ctx->last));
    ctx->last.kernel_ms = ms;
    double kt[K_KINDS] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t i = 0; i < ctx->ev_used; i++) {
        float e = 0.f;
        cudaEventElapsedTime(&e, ctx->ev_pool[2 * i], ctx->ev_pool[2 * i + 1]);
        kt[ctx->ev_kind[i]] += e;
    }
    ctx->last.camera_ms = kt[K_CAMERA];
    ctx->last.trace_closest_ms = kt[K_TRACE_C];
    ctx->last.trace_any_ms = kt[K_TRACE_A];
    ctx->last.shade_ms = kt[K_SHADE] + kt[K_RESOLVE];
    ctx->last.resolve_ms = kt[K_RESOLVE];
    ctx->last.sort_ms = kt[K_SORT];
    ctx->last.volpath_ms = kt[K_VOLPATH];
    ctx->last.film_ms = kt[K_FILM];
    ctx->last.trace_closest_launches = trace_c_launches;
    ctx->last.trace_any_launches = trace_a_launches;
    ctx->last.nodes_closest = (int64_t)stats[3];
    ctx->last.tris_closest = (int64_t)stats[4];
    ctx->last.nodes_any = (int64_t)stats[5];
    ctx->last.tris_any = (int64_t)stats[6];
    ctx->last.paths = total_paths;
    ctx->last.closest_rays = (int64_t)stats[0];
    ctx->last.shadow_rays = (int64_t)stats[1];
    ctx->last.nan_samples = (int64_t)stats[2];
    if (graph_batches) {
        // camera and film per batch, the rounds' kernels and k_round_next
        const int64_t rounds = (int64_t)stats[7];
        const int per_round = vw ? 5 + 1 : 3 + __builtin_popcount(types) + 1;
        launches += 2 * (int64_t)graph_batches + rounds * per_round;
        trace_c_launches += rounds;
        trace_a_launches += rounds;
    }
    ctx->last.launches = launches;
    ctx->last.limit_hits = limit;
    if (limit) return fail(RT_ERR_LIMIT, limit_message(limit));
    return RT_OK;
}

}  // extern "C"

// Grow a device buffer of a context to hold at least `count` elements.
template <typename T>
static rt_status grow_buf(T *&buf, size_t &have, size_t count, const char *what)
{
    if (have >= count && buf) return RT_OK;
    cudaFree(buf);
    buf = nullptr;
    have = 0;
    size_t n = std::max<size_t>(count, 16);
    if (cudaMalloc(&buf, n * sizeof(T)) != cudaSuccess) return fail(RT_ERR_NOMEM, std::string(what) + " allocation failed");
    have = n;
    return RT_OK;
}

// Many PathTracingMIS jobs (scene, render desc, device film) in one
// wavefront: the path slots of a batch belong to several jobs, each path
// carries its job's scene-table index, and every kernel reads the path's own
// scene.  A job's tiles are cut into work items of whole tiles with all
// their samples; items of all jobs are packed into batches of at most
// ctx->wave_paths paths.  Each path computes exactly what it computes in
// rt_render, and each pixel's samples are reduced in order within one
// batch, so every film equals rt_render's for that job alone.  All jobs
// share max_depth and min_depth; each has its own seed, sample range,
// light-selection strategy, block size and film.
rt_status rt_internal_render_multi(rt_ctx *ctx, rt_scene *const *scenes, const rt_render_desc *descs, int n,
                                   float *const *films, int32_t on_device)
{
    if (!ctx || n <= 0 || !scenes || !descs || !films) return fail(RT_ERR_INVALID, "render_multi: bad argument");
    const int max_depth = descs[0].max_depth, min_depth = descs[0].min_depth;
    for (int j = 0; j < n; j++) {
        const rt_render_desc &rd = descs[j];
        if (!scenes[j] || !films[j]) return fail(RT_ERR_INVALID, "render_multi: null scene or film");
        if (rd.spp <= 0 || rd.sample_begin < 0) return fail(RT_ERR_INVALID, "render_multi: bad sample range");
        if (rd.integrator != RT_INTEGRATOR_PATH_MIS || rd.strategy == RT_STRATEGY_ALL_LIGHTS)
            return fail(RT_ERR_UNSUPPORTED, "render_multi: PathTracingMIS jobs only (one light per vertex)");
        if (rd.max_depth != max_depth || rd.min_depth != min_depth)
            return fail(RT_ERR_UNSUPPORTED, "render_multi: jobs must share max_depth and min_depth");
        if (rd.max_depth < 0 || rd.min_depth < 0 || rd.max_depth > (1 << 16))
            return fail(RT_ERR_INVALID, "render_multi: bad depth");
        if (rd.flags & ~RT_RENDER_ACCUMULATE) return fail(RT_ERR_INVALID, "render_multi: unknown flags");
        const DevCamera &cam = scenes[j]->S.cam;
        if (!(cam.filter == RT_FILTER_BOX && cam.frx == 0.5f && cam.fry == 0.5f))
            return fail(RT_ERR_UNSUPPORTED, "render_multi: box filter of radius 0.5 only");
        const int bx = rd.block_x > 0 ? rd.block_x : 32, by = rd.block_y > 0 ? rd.block_y : 32;
        if (bx > 0xffff || by > 0xffff) return fail(RT_ERR_INVALID, "block size too large");
        if ((int64_t)bx * by * rd.spp > ctx->wave_paths)
            return fail(RT_ERR_LIMIT, "render_multi: one tile's samples exceed the path capacity");
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int cap = ctx->wave_paths;
    // per job: tile order (Scene.cpp:83-95 job grid) and light-selection CDF
    std::vector<int4> orders;
    std::vector<size_t> order_off(n);
    std::vector<std::vector<int>> tile_start(n);
    std::vector<float> cdfs;
    std::vector<size_t> cdf_off(n);
    for (int j = 0; j < n; j++) {
        const rt_render_desc &rd = descs[j];
        const DevCamera &cam = scenes[j]->S.cam;
        const int Wd = cam.width, H = cam.height;
        const int bx = rd.block_x > 0 ? rd.block_x : 32, by = rd.block_y > 0 ? rd.block_y : 32;
        const int tiles_x = (Wd + bx - 1) / bx, tiles_y = (H + by - 1) / by;
        order_off[j] = orders.size();
        tile_start[j].assign(tiles_x * tiles_y + 1, 0);
        int g = 0;
        for (int ty = 0; ty < tiles_y; ty++)
            for (int tx = 0; tx < tiles_x; tx++) {
                tile_start[j][ty * tiles_x + tx] = g;
                int ox = tx * bx, oy = ty * by;
                int tw = std::min(Wd, ox + bx) - ox, th = std::min(H, oy + by) - oy;
                for (int y = 0; y < th; y++)
                    for (int x = 0; x < tw; x++, g++) orders.push_back(make_int4(ox + x, oy + y, x | (y << 16), tw | (th << 16)));
            }
        tile_start[j][tiles_x * tiles_y] = g;
        HCdf c;
        rt_scene *sc = scenes[j];
        float pu = (float)1. / (float)sc->n_lights;
        for (int l = 0; l < sc->n_lights; l++)
            c.add(rd.strategy == RT_STRATEGY_ONE_LIGHT_WEIGHTED ? sc->light_power_lum[l] : pu);
        c.normalize();
        cdf_off[j] = cdfs.size();
        cdfs.insert(cdfs.end(), c.c.begin(), c.c.end());
        while (cdfs.size() % 16) cdfs.push_back(0.f);
    }
    rt_status s;
    if ((s = grow_buf(ctx->m_order, ctx->m_order_n, orders.size(), "tile order")) != RT_OK) return s;
    if ((s = grow_buf(ctx->m_cdf, ctx->m_cdf_n, cdfs.size(), "light CDF")) != RT_OK) return s;
    if ((s = grow_buf(ctx->m_scenes, ctx->m_scenes_n, (size_t)n, "scene table")) != RT_OK) return s;
    CK(cudaMemcpyAsync(ctx->m_order, orders.data(), orders.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->m_cdf, cdfs.data(), cdfs.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    std::vector<DevScene> table(n);
    int types = ctx->sort_threshold > 0 ? 1 << RT_QUEUE_MIXED : 0;
    for (int j = 0; j < n; j++) {
        table[j] = scenes[j]->S;
        table[j].light_cdf = ctx->m_cdf + cdf_off[j];
        table[j].limit_flag = ctx->limit_flag;
        types |= scenes[j]->bsdf_types;
    }
    CK(cudaMemcpyAsync(ctx->m_scenes, table.data(), (size_t)n * sizeof(DevScene), cudaMemcpyHostToDevice, st));
    // device films: the caller's, or staging films for host memory
    std::vector<float4 *> dfilm(n, nullptr);
    std::vector<void *> staging;
    auto release = [&]() { for (void *p : staging) cudaFree(p); };
    for (int j = 0; j < n; j++) {
        if (on_device) { dfilm[j] = reinterpret_cast<float4 *>(films[j]); continue; }
        const size_t npix = (size_t)scenes[j]->S.cam.width * scenes[j]->S.cam.height;
        void *p = nullptr;
        if (cudaMalloc(&p, npix * sizeof(float4)) != cudaSuccess) { release(); return fail(RT_ERR_NOMEM, "film allocation failed"); }
        staging.push_back(p);
        dfilm[j] = (float4 *)p;
        if (descs[j].flags & RT_RENDER_ACCUMULATE) {
            cudaError_t e = cudaMemcpyAsync(p, films[j], npix * sizeof(float4), cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) { release(); return fail(RT_ERR_CUDA, cudaGetErrorString(e)); }
        }
    }
    // work items: per job, runs of whole tiles of at most `cap` paths
    struct Item { MultiItem m; int paths; };
    std::vector<Item> items;
    for (int j = 0; j < n; j++) {
        const rt_render_desc &rd = descs[j];
        const int bx = rd.block_x > 0 ? rd.block_x : 32, by = rd.block_y > 0 ? rd.block_y : 32;
        const int ntiles = (int)tile_start[j].size() - 1;
        const int per = std::max(1, cap / std::max(1, bx * by * rd.spp));
        for (int t0 = 0; t0 < ntiles; t0 += per) {
            int t1 = std::min(ntiles, t0 + per);
            Item it;
            std::memset(&it.m, 0, sizeof(it.m));
            it.m.job = j;
            it.m.npix = tile_start[j][t1] - tile_start[j][t0];
            it.m.spp = rd.spp;
            it.m.sample_begin = rd.sample_begin;
            it.m.g0 = tile_start[j][t0];
            it.m.width = scenes[j]->S.cam.width;
            it.m.accumulate = (rd.flags & RT_RENDER_ACCUMULATE) ? 1 : 0;
            it.m.tileorder = ctx->m_order + order_off[j];
            it.m.film = dfilm[j];
            it.m.seed = rd.seed;
            it.paths = it.m.npix * rd.spp;
            items.push_back(it);
        }
    }
    // batches: items in job order, each batch up to `cap` paths
    std::vector<std::vector<MultiItem>> batches;
    std::vector<int> batch_paths, batch_pix;
    int capacity = 0;
    for (size_t i = 0; i < items.size();) {
        std::vector<MultiItem> b;
        int paths = 0, pix = 0;
        while (i < items.size() && (b.empty() || paths + items[i].paths <= cap)) {
            MultiItem m = items[i].m;
            m.path0 = paths;
            m.pix0 = pix;
            paths += items[i].paths;
            pix += m.npix;
            b.push_back(m);
            i++;
        }
        capacity = std::max(capacity, paths);
        batches.push_back(std::move(b));
        batch_paths.push_back(paths);
        batch_pix.push_back(pix);
    }
    const int max_rounds = max_depth + 3;
    if ((s = ensure_wave(ctx, capacity, max_rounds)) != RT_OK) { release(); return s; }
    size_t max_items = 0;
    for (auto &b : batches) max_items = std::max(max_items, b.size());
    if ((s = grow_buf(ctx->m_items, ctx->m_items_n, max_items, "work items")) != RT_OK) { release(); return s; }
    CK(cudaMemsetAsync(ctx->stats, 0, sizeof(unsigned long long) * 8, st));
    CK(cudaMemsetAsync(ctx->limit_flag, 0, sizeof(int), st));
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.S = scenes[0]->S;
    P.W = ctx->W;
    P.max_depth = max_depth;
    P.min_depth = min_depth;
    P.limit_flag = ctx->limit_flag;
    P.stats = ctx->stats;
    P.sort_threshold = ctx->sort_threshold;
    P.scenes = ctx->m_scenes;
    P.items = ctx->m_items;
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const int trace_blocks = sm * ctx->trace_bpsm, shade_blocks = sm * ctx->shade_bpsm;
    int64_t launches = 0, rounds_run = 0, total_paths = 0;
    ctx->ev_used = 0;
    CK(cudaEventRecord(ctx->ev0, st));
    for (size_t bi = 0; bi < batches.size(); bi++) {
        const std::vector<MultiItem> &b = batches[bi];
        CK(cudaMemcpyAsync(ctx->m_items, b.data(), b.size() * sizeof(MultiItem), cudaMemcpyHostToDevice, st));
        P.n_items = (int)b.size();
        P.n_paths = batch_paths[bi];
        P.npix = batch_pix[bi];
        total_paths += P.n_paths;
        CK(cudaMemsetAsync(ctx->W.pix_irregular, 0, (size_t)P.npix, st));
        CK(cudaMemsetAsync(ctx->W.cnt, 0, sizeof(RoundCounters) * (size_t)(max_rounds + 2), st));
        prof_begin(ctx, K_CAMERA);
        k_camera_multi<<<std::min((P.n_paths + 255) / 256, sm * 16), 256, 0, st>>>(P);
        prof_end(ctx);
        launches++;
        if ((s = launch_check("k_camera_multi")) != RT_OK) { release(); return s; }
        for (int r = 0; r < max_rounds; r++) {
            prof_begin(ctx, K_TRACE_C);
            k_trace<false, false, true><<<trace_blocks, 128, 0, st>>>(P, r);
            prof_end(ctx);
            prof_begin(ctx, K_TRACE_A);
            k_trace<true, false, true><<<trace_blocks, 128, 0, st>>>(P, r);
            prof_end(ctx);
            prof_begin(ctx, K_RESOLVE);
            k_pt_finish<true><<<shade_blocks, 128, 0, st>>>(P, r);
            prof_end(ctx);
            prof_begin(ctx, K_SHADE);
            if (types & 1) k_pt_shade<0, true><<<shade_blocks, 128, 0, st>>>(P, r);
            if (types & 2) k_pt_shade<1, true><<<shade_blocks, 128, 0, st>>>(P, r);
            if (types & 4) k_pt_shade<2, true><<<shade_blocks, 128, 0, st>>>(P, r);
            if (types & 8) k_pt_shade<3, true><<<shade_blocks, 128, 0, st>>>(P, r);
            if (types & 16) k_pt_shade<4, true><<<shade_blocks, 128, 0, st>>>(P, r);
            if (types & 32) k_pt_shade<5, true><<<shade_blocks, 128, 0, st>>>(P, r);
            if (types & (1 << RT_QUEUE_MIXED)) k_pt_shade<RT_QUEUE_MIXED, true><<<shade_blocks, 128, 0, st>>>(P, r);
            prof_end(ctx);
            launches += 3 + __builtin_popcount(types);
            rounds_run++;
            if ((s = launch_check("multi-scene round")) != RT_OK) { release(); return s; }
            if ((r & 3) == 3 && r + 1 < max_rounds) {
                RoundCounters nc;
                CK(cudaMemcpyAsync(&nc, &ctx->W.cnt[r + 1], sizeof(nc), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (nc.closest == 0 && nc.end == 0) break;
            }
        }
        prof_begin(ctx, K_FILM);
        k_film_multi<<<(P.npix + 127) / 128, 128, 0, st>>>(P);
        prof_end(ctx);
        launches++;
        if ((s = launch_check("k_film_multi")) != RT_OK) { release(); return s; }
    }
    CK(cudaEventRecord(ctx->ev1, st));
    for (int j = 0; j < n && !on_device; j++) {
        const size_t npix = (size_t)scenes[j]->S.cam.width * scenes[j]->S.cam.height;
        cudaError_t e = cudaMemcpyAsync(films[j], dfilm[j], npix * sizeof(float4), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) { release(); return fail(RT_ERR_CUDA, cudaGetErrorString(e)); }
    }
    unsigned long long stats[8];
    int limit = 0;
    CK(cudaMemcpyAsync(stats, ctx->stats, sizeof(stats), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&limit, ctx->limit_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    release();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    std::memset(&ctx->last, 0, sizeof(ctx->last));
    ctx->last.kernel_ms = ms;
    double kt[K_KINDS] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t i = 0; i < ctx->ev_used; i++) {
        float e = 0.f;
        cudaEventElapsedTime(&e, ctx->ev_pool[2 * i], ctx->ev_pool[2 * i + 1]);
        kt[ctx->ev_kind[i]] += e;
    }
    ctx->last.camera_ms = kt[K_CAMERA];
    ctx->last.trace_closest_ms = kt[K_TRACE_C];
    ctx->last.trace_any_ms = kt[K_TRACE_A];
    ctx->last.shade_ms = kt[K_SHADE] + kt[K_RESOLVE];
    ctx->last.resolve_ms = kt[K_RESOLVE];
    ctx->last.film_ms = kt[K_FILM];
    ctx->last.trace_closest_launches = rounds_run;
    ctx->last.trace_any_launches = rounds_run;
    ctx->last.paths = total_paths;
    ctx->last.closest_rays = (int64_t)stats[0];
    ctx->last.shadow_rays = (int64_t)stats[1];
    ctx->last.nan_samples = (int64_t)stats[2];
    ctx->last.launches = launches;
    ctx->last.limit_hits = limit;
    if (limit) return fail(RT_ERR_LIMIT, limit_message(limit));
    return RT_OK;
}

extern "C" {

rt_status rt_render_paths(rt_ctx *ctx, rt_scene *sc, const rt_render_desc *rd, const int32_t *pixels,
                          const int32_t *samples, int32_t n, float *rgb)
{
    if (!ctx || !sc || !rd || n < 0 || (n > 0 && (!pixels || !samples || !rgb)))
        return fail(RT_ERR_INVALID, "rt_render_paths: bad argument");
    if (n == 0) return RT_OK;
    if (rd->integrator != RT_INTEGRATOR_PATH_MIS && rd->integrator != RT_INTEGRATOR_VOLPATH)
        return fail(RT_ERR_UNSUPPORTED, "rt_render_paths: unknown integrator");
    if (rd->max_depth < 0 || rd->min_depth < 0 || rd->max_depth > (1 << 16))
        return fail(RT_ERR_INVALID, "rt_render_paths: bad depth");
    const DevCamera &cam = sc->S.cam;
    const int64_t npix = (int64_t)cam.width * cam.height;
    std::vector<int2> list(n);
    for (int i = 0; i < n; i++) {
        if (pixels[i] < 0 || pixels[i] >= npix || samples[i] < 0)
            return fail(RT_ERR_INVALID, "rt_render_paths: pixel or sample index out of range");
        list[i] = make_int2(pixels[i], samples[i]);
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    HCdf c;
    {
        float pu = (float)1. / (float)sc->n_lights;
        for (int l = 0; l < sc->n_lights; l++)
            c.add(rd->strategy == RT_STRATEGY_ONE_LIGHT_WEIGHTED ? sc->light_power_lum[l] : pu);
        c.normalize();
    }
    const bool vw = rd->integrator == RT_INTEGRATOR_VOLPATH && ctx->volpath_wave;
    const int max_rounds = rd->integrator == RT_INTEGRATOR_PATH_MIS ? rd->max_depth + 3 : vw ? (1 << 16) + 2 : 1;
    rt_status s = ensure_wave(ctx, n, max_rounds);
    if (s != RT_OK) return s;
    if (vw && (s = ensure_vw(ctx, n)) != RT_OK) return s;
    // the list and the light CDF in one temporary buffer
    void *tmp = nullptr;
    const size_t list_bytes = (size_t)n * sizeof(int2), cdf_off = (list_bytes + 255) & ~(size_t)255;
    CK(cudaMalloc(&tmp, cdf_off + c.c.size() * sizeof(float)));
    std::vector<float4> out(n);
    auto run = [&]() -> rt_status {
        CK(cudaMemcpyAsync(tmp, list.data(), list_bytes, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync((char *)tmp + cdf_off, c.c.data(), c.c.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(ctx->limit_flag, 0, sizeof(int), st));
        CK(cudaMemsetAsync(ctx->W.cnt, 0, sizeof(RoundCounters) * (size_t)(max_rounds + 2), st));
        RenderParams P;
        std::memset(&P, 0, sizeof(P));
        P.S = sc->S;
        P.S.limit_flag = ctx->limit_flag;
        P.S.light_cdf = (const float *)((char *)tmp + cdf_off);
        P.W = ctx->W;
        P.seed = rd->seed;
        P.max_depth = rd->max_depth;
        P.min_depth = rd->min_depth;
        P.limit_flag = ctx->limit_flag;
        P.stats = ctx->stats;
        P.n_paths = n;
        P.npix = n;
        P.sort_threshold = ctx->sort_threshold;
        P.all_lights = rd->integrator == RT_INTEGRATOR_PATH_MIS && rd->strategy == RT_STRATEGY_ALL_LIGHTS;
        P.path_list = (const int2 *)tmp;
        const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
        rt_status e;
        k_camera<<<std::min((n + 255) / 256, sm * 16), 256, 0, st>>>(P);
        if ((e = launch_check("k_camera (paths)")) != RT_OK) return e;
        if (vw) {
            for (int r = 0; r < max_rounds; r++) {
                k_vw_trace_step<<<sm * RT_VW_MINB_STEP, 128, 0, st>>>(P, r);
                k_vw_shadow<<<sm * RT_VW_MINB_SHADOW, 128, 0, st>>>(P, r);
                k_vw_scatter<<<sm * RT_VW_MINB_TRSAMP, 128, 0, st>>>(P, r);
                k_vw_sample_surface<<<sm * RT_VW_MINB_SAMPLE, 128, 0, st>>>(P, r);
                k_vw_trsamp_finish<<<sm * RT_VW_MINB_TRSAMP, 128, 0, st>>>(P, r);
                if ((e = launch_check("VolPath round (paths)")) != RT_OK) return e;
                int nq = 0;
                CK(cudaMemcpyAsync(&nq, &ctx->W.cnt[r + 1].closest, sizeof(int), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (nq == 0) break;
            }
        } else if (rd->integrator == RT_INTEGRATOR_VOLPATH) {
            CK(cudaMemsetAsync(ctx->work, 0, sizeof(int), st));
            k_volpath<<<sm * RT_VOLPATH_GRID, 128, 0, st>>>(P, ctx->work);
            if ((e = launch_check("k_volpath (paths)")) != RT_OK) return e;
        } else {
            const int types = sc->bsdf_types | (P.sort_threshold > 0 ? 1 << RT_QUEUE_MIXED : 0);
            const int tb = sm * ctx->trace_bpsm, sb = sm * ctx->shade_bpsm;
            const int width = trace_width(ctx, sc);
            for (int r = 0; r < max_rounds; r++) {
                launch_trace(width, P, r, false, false, tb, st);
                launch_trace(width, P, r, true, false, tb, st);
                k_pt_finish<<<sb, 128, 0, st>>>(P, r);
                launch_shades(types, P, r, sb, st);
                if ((e = launch_check("pt round (paths)")) != RT_OK) return e;
                RoundCounters nc;
                CK(cudaMemcpyAsync(&nc, &ctx->W.cnt[r + 1], sizeof(nc), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (nc.closest == 0 && nc.end == 0) break;
            }
        }
        CK(cudaMemcpyAsync(out.data(), ctx->W.out, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost, st));
        int limit = 0;
        CK(cudaMemcpyAsync(&limit, ctx->limit_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (limit) return fail(RT_ERR_LIMIT, limit_message(limit));
        return RT_OK;
    };
    s = run();
    cudaFree(tmp);
    if (s != RT_OK) return s;
    for (int i = 0; i < n; i++) {
        rgb[3 * i] = out[i].x;
        rgb[3 * i + 1] = out[i].y;
        rgb[3 * i + 2] = out[i].z;
    }
    return RT_OK;
}

rt_status rt_render_stats_get(const rt_ctx *ctx, rt_render_stats *out)
{
    if (!ctx || !out) return fail(RT_ERR_INVALID, "null argument");
    *out = ctx->last;
    return RT_OK;
}

rt_status rt_trace(rt_ctx *ctx, rt_scene *sc, const rt_ray *rays, int32_t n, int32_t anyhit, rt_hit *hits, int32_t on_device)
{
    if (!ctx || !sc || (!rays && n) || (!hits && n) || n < 0) return fail(RT_ERR_INVALID, "rt_trace: bad argument");
    if (n == 0) return RT_OK;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    // the rays go through the same persistent traversal kernels a render uses
    rt_status s = ensure_wave(ctx, n, std::max(1, ctx->W.max_rounds));
    if (s != RT_OK) return s;
    const rt_ray *dr = rays;
    rt_hit *dh = hits;
    void *tmp_r = nullptr, *tmp_h = nullptr;
    if (!on_device) {
        CK(cudaMalloc(&tmp_r, sizeof(rt_ray) * (size_t)n));
        CK(cudaMalloc(&tmp_h, sizeof(rt_hit) * (size_t)n));
        CK(cudaMemcpyAsync(tmp_r, rays, sizeof(rt_ray) * (size_t)n, cudaMemcpyHostToDevice, st));
        dr = (const rt_ray *)tmp_r;
        dh = (rt_hit *)tmp_h;
    }
    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    P.S = sc->S;
    P.S.limit_flag = ctx->limit_flag;
    P.W = ctx->W;
    P.stats = ctx->stats;
    P.limit_flag = ctx->limit_flag;
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    CK(cudaMemsetAsync(ctx->limit_flag, 0, sizeof(int), st));
    k_rays_in<<<(n + 127) / 128, 128, 0, st>>>(dr, n, P, anyhit ? 1 : 0);
    launch_trace(trace_width(ctx, sc), P, 0, anyhit != 0, false, sm * 12, st);
    k_hits_out<<<(n + 127) / 128, 128, 0, st>>>(P, n, anyhit ? 1 : 0, dh);
    s = launch_check("rt_trace kernels");
    if (s == RT_OK && !on_device) {
        cudaError_t e = cudaMemcpyAsync(hits, tmp_h, sizeof(rt_hit) * (size_t)n, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) s = fail(RT_ERR_CUDA, cudaGetErrorString(e));
    }
    int limit = 0;
    if (s == RT_OK) {
        cudaError_t e = cudaMemcpyAsync(&limit, ctx->limit_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) s = fail(RT_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (s == RT_OK && e != cudaSuccess) s = fail(RT_ERR_CUDA, cudaGetErrorString(e));
    if (s == RT_OK && limit) s = fail(RT_ERR_LIMIT, "rt_trace: " + limit_message(limit));
    if (tmp_r) cudaFree(tmp_r);
    if (tmp_h) cudaFree(tmp_h);
    return s;
}

rt_status rt_bsdf_query(rt_ctx *ctx, rt_scene *sc, int32_t bsdf, int32_t op, const rt_bsdf_q *q, int32_t n, rt_bsdf_r *r)
{
    if (!ctx || !sc || n < 0 || (n && (!q || !r))) return fail(RT_ERR_INVALID, "rt_bsdf_query: bad argument");
    if (op < 0 || op > 2) return fail(RT_ERR_INVALID, "rt_bsdf_query: bad op");
    if (bsdf < 0 || bsdf >= sc->n_bsdfs) return fail(RT_ERR_INVALID, "rt_bsdf_query: bad bsdf index");
    if (n == 0) return RT_OK;
    CK(cudaSetDevice(ctx->device));
    void *dq = nullptr, *dr = nullptr;
    CK(cudaMalloc(&dq, sizeof(rt_bsdf_q) * (size_t)n));
    CK(cudaMalloc(&dr, sizeof(rt_bsdf_r) * (size_t)n));
    CK(cudaMemcpy(dq, q, sizeof(rt_bsdf_q) * (size_t)n, cudaMemcpyHostToDevice));
    k_bsdf_query<<<(n + 127) / 128, 128, 0, ctx->stream>>>(sc->S, bsdf, op, (const rt_bsdf_q *)dq, n, (rt_bsdf_r *)dr);
    rt_status s = launch_check("k_bsdf_query");
    cudaStreamSynchronize(ctx->stream);
    if (s == RT_OK) {
        cudaError_t e = cudaMemcpy(r, dr, sizeof(rt_bsdf_r) * (size_t)n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) s = fail(RT_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(dq);
    cudaFree(dr);
    return s;
}

rt_status rt_light_query(rt_ctx *ctx, rt_scene *sc, int32_t light, const rt_light_q *q, int32_t n, rt_light_r *r)
{
    if (!ctx || !sc || n < 0 || (n && (!q || !r))) return fail(RT_ERR_INVALID, "rt_light_query: bad argument");
    if (light < 0 || light >= sc->n_lights) return fail(RT_ERR_INVALID, "rt_light_query: bad light");
    if (n == 0) return RT_OK;
    CK(cudaSetDevice(ctx->device));
    void *dq = nullptr, *dr = nullptr;
    CK(cudaMalloc(&dq, sizeof(rt_light_q) * (size_t)n));
    CK(cudaMalloc(&dr, sizeof(rt_light_r) * (size_t)n));
    CK(cudaMemcpy(dq, q, sizeof(rt_light_q) * (size_t)n, cudaMemcpyHostToDevice));
    k_light_query<<<(n + 127) / 128, 128, 0, ctx->stream>>>(sc->S, light, (const rt_light_q *)dq, n, (rt_light_r *)dr);
    rt_status s = launch_check("k_light_query");
    cudaStreamSynchronize(ctx->stream);
    if (s == RT_OK) {
        cudaError_t e = cudaMemcpy(r, dr, sizeof(rt_light_r) * (size_t)n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) s = fail(RT_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(dq);
    cudaFree(dr);
    return s;
}

rt_status rt_medium_query(rt_ctx *ctx, rt_scene *sc, int32_t medium, int32_t op, const rt_medium_q *q, int32_t n,
                          rt_medium_r *r)
{
    if (!ctx || !sc || n < 0 || (n && (!q || !r))) return fail(RT_ERR_INVALID, "rt_medium_query: bad argument");
    if (medium < 0 || medium >= sc->n_media) return fail(RT_ERR_INVALID, "rt_medium_query: bad medium");
    if (op != RT_MEDIUM_OP_SAMPLE && op != RT_MEDIUM_OP_TRANSMITTANCE)
        return fail(RT_ERR_INVALID, "rt_medium_query: bad op");
    if (n == 0) return RT_OK;
    CK(cudaSetDevice(ctx->device));
    void *dq = nullptr, *dr = nullptr;
    CK(cudaMalloc(&dq, sizeof(rt_medium_q) * (size_t)n));
    CK(cudaMalloc(&dr, sizeof(rt_medium_r) * (size_t)n));
    CK(cudaMemcpy(dq, q, sizeof(rt_medium_q) * (size_t)n, cudaMemcpyHostToDevice));
    k_medium_query<<<(n + 127) / 128, 128, 0, ctx->stream>>>(sc->S, medium, op, (const rt_medium_q *)dq, n,
                                                              (rt_medium_r *)dr);
    rt_status s = launch_check("k_medium_query");
    cudaStreamSynchronize(ctx->stream);
    if (s == RT_OK) {
        cudaError_t e = cudaMemcpy(r, dr, sizeof(rt_medium_r) * (size_t)n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) s = fail(RT_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(dq);
    cudaFree(dr);
    return s;
}

}  // extern "C"

// =====================================================================
// Allocation-free tile render (rt_render_tile_static)
// =====================================================================
// Some callers cannot call cudaMalloc while they render: renderer plugins
// that run inside a host application whose device memory is owned by that
// application's own pool allocator under a hard budget, real-time loops that
// forbid device allocation after start-up (cudaMalloc/cudaFree can
// synchronise the device and stall the frame), and code that issues work
// while another component is capturing the stream.  For them this entry point
// renders one tile of the reference job grid with no allocation at all: the
// wavefront path state lives in the file-scope array below, which every GPU
// that loads the library holds until the process exits.  The scene (created
// earlier by rt_scene_create) and the film are the caller's inputs and output.
#define RT_STATIC_SCRATCH_BYTES (32u << 20)   // 32 MiB per device
#define RT_STATIC_MAX_DEVICES 64
#define RT_STATIC_MAX_LIGHTS 256
#define RT_STATIC_MAX_DEPTH 1024

static __device__ __align__(256) unsigned char g_static_scratch[RT_STATIC_SCRATCH_BYTES];

#include <mutex>
static std::mutex g_static_mu;
static unsigned char *g_static_ptr[RT_STATIC_MAX_DEVICES];

// Device address of g_static_scratch for the current device, looked up once
// per device (the host-side name of a __device__ array is not a device
// address).
static rt_status static_scratch(int device, unsigned char **out)
{
    if (device < 0 || device >= RT_STATIC_MAX_DEVICES) return fail(RT_ERR_LIMIT, "device index above the static scratch table");
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess)
            return fail(RT_ERR_CUDA, std::string("cudaGetSymbolAddress(g_static_scratch) -> ") + cudaGetErrorString(e));
        g_static_ptr[device] = (unsigned char *)p;
    }
    *out = g_static_ptr[device];
    return RT_OK;
}

__global__ void k_tile_order(int4 *out, int ox, int oy, int tw, int th)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tw * th) return;
    int x = i % tw, y = i / tw;
    out[i] = make_int4(ox + x, oy + y, x | (y << 16), tw | (th << 16));
}

extern "C" rt_status rt_render_tile_static(rt_ctx *ctx, rt_scene *sc, const rt_render_desc *rd, int32_t tile_x,
                                           int32_t tile_y, float *film_rgbw_device)
{
    if (!ctx || !sc || !rd || !film_rgbw_device) return fail(RT_ERR_INVALID, "rt_render_tile_static: null argument");
    if (rd->spp <= 0 || rd->sample_begin < 0) return fail(RT_ERR_INVALID, "rt_render_tile_static: bad sample range");
    if (rd->integrator != RT_INTEGRATOR_PATH_MIS && rd->integrator != RT_INTEGRATOR_VOLPATH)
        return fail(RT_ERR_UNSUPPORTED, "rt_render_tile_static: unknown integrator");
    if (rd->max_depth < 0 || rd->min_depth < 0) return fail(RT_ERR_INVALID, "rt_render_tile_static: negative depth");
    // PathTracingMIS keeps one round counter per bounce in the scratch;
    // VolPathTracing runs as one persistent kernel and needs one
    if (rd->integrator == RT_INTEGRATOR_PATH_MIS && rd->max_depth > RT_STATIC_MAX_DEPTH)
        return fail(RT_ERR_LIMIT, "rt_render_tile_static: max_depth above 1024 (the static round-counter table)");
    // every path needs well over 64 bytes of state: a larger request cannot
    // fit, and refusing it here keeps the size arithmetic below far from
    // overflow
    if (rd->spp > (int)(RT_STATIC_SCRATCH_BYTES / 64))
        return fail(RT_ERR_LIMIT, "rt_render_tile_static: spp beyond what the static scratch can hold");
    if (sc->n_lights > RT_STATIC_MAX_LIGHTS) return fail(RT_ERR_LIMIT, "rt_render_tile_static: more than 256 lights");
    const DevCamera &cam = sc->S.cam;
    if (!(cam.filter == RT_FILTER_BOX && cam.frx == 0.5f && cam.fry == 0.5f))
        return fail(RT_ERR_UNSUPPORTED, "rt_render_tile_static: only the box filter of radius 0.5");
    const int Wd = cam.width, H = cam.height;
    const int bx = rd->block_x > 0 ? rd->block_x : 32, by = rd->block_y > 0 ? rd->block_y : 32;
    if (bx > 0xffff || by > 0xffff) return fail(RT_ERR_INVALID, "block size too large");
    const int tiles_x = (Wd + bx - 1) / bx, tiles_y = (H + by - 1) / by;
    if (tile_x < 0 || tile_y < 0 || tile_x >= tiles_x || tile_y >= tiles_y)
        return fail(RT_ERR_INVALID, "rt_render_tile_static: tile index outside the job grid");
    const int ox = tile_x * bx, oy = tile_y * by;
    const int tw = std::min(Wd, ox + bx) - ox, th = std::min(H, oy + by) - oy;
    const int64_t npix = (int64_t)tw * th, paths = npix * rd->spp;
    if (paths > (int64_t)(RT_STATIC_SCRATCH_BYTES / 64)) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "rt_render_tile_static: a %dx%d tile at %d spp is %lld path samples; the static scratch holds "
                 "fewer than %u (reduce spp or the block size)", tw, th, rd->spp, (long long)paths,
                 (unsigned)(RT_STATIC_SCRATCH_BYTES / 64));
        return fail(RT_ERR_LIMIT, msg);
    }
    CK(cudaSetDevice(ctx->device));
    // The call waits on its stream (round counters, the limit flag) and
    // copies the light CDF from host memory: neither can be recorded into a
    // graph, so a stream under capture is refused before anything is queued.
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(ctx->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(RT_ERR_UNSUPPORTED, "rt_render_tile_static: the context's stream is being captured; "
                                            "the call synchronises its stream and must run outside a capture");
    }
    unsigned char *base = nullptr;
    rt_status s = static_scratch(ctx->device, &base);
    if (s != RT_OK) return s;
    // carve the scratch: every array 256-byte aligned
    const int rounds = rd->integrator == RT_INTEGRATOR_PATH_MIS ? rd->max_depth + 3 : 1;
    size_t off = 0;
    auto take = [&](size_t bytes) -> unsigned char * {
        size_t o = (off + 255) & ~(size_t)255;
        off = o + bytes;
        return base + o;
    };
    Wave W;
    std::memset(&W, 0, sizeof(W));
    const size_t P = (size_t)paths;
    W.rng = (Pcg32 *)take(P * sizeof(Pcg32));
    W.tp = (float4 *)take(P * sizeof(float4));
    W.rad = (float4 *)take(P * sizeof(float4));
    W.ray_o = (float4 *)take(P * sizeof(float4));
    W.ray_d = (float4 *)take(P * sizeof(float4));
    W.hit = (float4 *)take(P * sizeof(float4));
    W.bs = (float4 *)take(P * sizeof(float4));
    W.rel_eta = (float *)take(P * sizeof(float));
    W.flags = (int *)take(P * sizeof(int));
    W.nee = (float4 *)take(P * sizeof(float4));
    W.sh_o = (float4 *)take(P * sizeof(float4));
    W.sh_d = (float4 *)take(P * sizeof(float4));
    W.occl = (int *)take(P * sizeof(int));
    W.out = (float4 *)take(P * sizeof(float4));
    W.splat = (uint8_t *)take(P);
    W.pix_irregular = (uint8_t *)take((size_t)npix);
    W.q_fin = (int *)take(P * sizeof(int));
    W.q_end = (int *)take(P * sizeof(int));
    W.q_closest = (int *)take(P * sizeof(int));
    W.q_shadow = (int *)take(P * sizeof(int));
    for (int t = 0; t < RT_NBSDF; t++) W.q_mat[t] = (int *)take(P * sizeof(int));
    // textured and Microfacet BSDFs shade from the mixed queue
    if (sc->S.has_mixed) W.q_mixed = (int *)take(P * sizeof(int));
    W.cnt = (RoundCounters *)take((size_t)(rounds + 2) * sizeof(RoundCounters));
    W.capacity = (int)P;
    W.max_rounds = rounds;
    int4 *tileorder = (int4 *)take((size_t)npix * sizeof(int4));
    float *light_cdf = (float *)take((size_t)(RT_STATIC_MAX_LIGHTS + 1) * sizeof(float));
    unsigned long long *stats = (unsigned long long *)take(8 * sizeof(unsigned long long));
    int *limit_flag = (int *)take(sizeof(int));
    int *work = (int *)take(sizeof(int));
    if (off > RT_STATIC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "rt_render_tile_static: a %dx%d tile at %d spp needs %zu bytes of path state; the static scratch "
                 "holds %u (reduce spp or the block size)", tw, th, rd->spp, off, (unsigned)RT_STATIC_SCRATCH_BYTES);
        return fail(RT_ERR_LIMIT, msg);
    }
    cudaStream_t st = ctx->stream;
    // light selection CDF (Integrator::initialize) in a fixed host array
    float cdf[RT_STATIC_MAX_LIGHTS + 1];
    {
        int n = sc->n_lights;
        float pu = (float)1. / (float)n, sum = 0.f;
        cdf[0] = 0.f;
        for (int l = 0; l < n; l++) {
            sum += rd->strategy == RT_STRATEGY_ONE_LIGHT_WEIGHTED ? sc->light_power_lum[l] : pu;
            cdf[l + 1] = sum;
        }
        if (sum != 0.f) {
            float f = 1.f / sum;
            for (int i = 1; i <= n; i++) cdf[i] *= f;
            cdf[n] = 1.f;
        }
        CK(cudaMemcpyAsync(light_cdf, cdf, sizeof(float) * (size_t)(n + 1), cudaMemcpyHostToDevice, st));
    }
    // the scratch keeps the previous call's contents: clear what counts from zero
    CK(cudaMemsetAsync(W.cnt, 0, sizeof(RoundCounters) * (size_t)(rounds + 2), st));
    CK(cudaMemsetAsync(W.pix_irregular, 0, (size_t)npix, st));
    CK(cudaMemsetAsync(stats, 0, 8 * sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(limit_flag, 0, sizeof(int), st));
    CK(cudaMemsetAsync(work, 0, sizeof(int), st));
    k_tile_order<<<(int)((npix + 127) / 128), 128, 0, st>>>(tileorder, ox, oy, tw, th);
    if ((s = launch_check("k_tile_order")) != RT_OK) return s;
    RenderParams Pm;
    std::memset(&Pm, 0, sizeof(Pm));
    Pm.S = sc->S;
    Pm.S.light_cdf = light_cdf;
    Pm.S.limit_flag = limit_flag;
    Pm.W = W;
    Pm.tileorder = tileorder;
    Pm.g0 = 0;
    Pm.npix = (int)npix;
    Pm.spp = rd->spp;
    Pm.sample_begin = rd->sample_begin;
    Pm.n_paths = (int)paths;
    Pm.seed = rd->seed;
    Pm.max_depth = rd->max_depth;
    Pm.all_lights = rd->integrator == RT_INTEGRATOR_PATH_MIS && rd->strategy == RT_STRATEGY_ALL_LIGHTS;
    Pm.min_depth = rd->min_depth;
    Pm.limit_flag = limit_flag;
    Pm.stats = stats;
    const int sm = ctx->sm_count > 0 ? ctx->sm_count : 1;
    k_camera<<<std::min((int)((paths + 255) / 256), sm * 16), 256, 0, st>>>(Pm);
    if ((s = launch_check("k_camera")) != RT_OK) return s;
    if (rd->integrator == RT_INTEGRATOR_VOLPATH) {
        k_volpath<<<sm * RT_VOLPATH_GRID, 128, 0, st>>>(Pm, work);
        if ((s = launch_check("k_volpath")) != RT_OK) return s;
    } else {
        const int blocks = sm * 8;
        for (int r = 0; r < rounds; r++) {
            launch_trace(trace_width(ctx, sc), Pm, r, false, false, sm * 12, st);
            launch_trace(trace_width(ctx, sc), Pm, r, true, false, sm * 12, st);
            k_pt_finish<<<blocks, 128, 0, st>>>(Pm, r);
            launch_shades(sc->bsdf_types, Pm, r, blocks, st);
            if ((s = launch_check("pt round (static)")) != RT_OK) return s;
            if ((r & 3) == 3 && r + 1 < rounds) {
                RoundCounters nc;
                CK(cudaMemcpyAsync(&nc, &W.cnt[r + 1], sizeof(nc), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (nc.closest == 0 && nc.end == 0) break;
            }
        }
    }
    k_film<<<(int)((npix + 127) / 128), 128, 0, st>>>(Pm, reinterpret_cast<float4 *>(film_rgbw_device), Wd,
                                                      (rd->flags & RT_RENDER_ACCUMULATE) ? 1 : 0);
    if ((s = launch_check("k_film (static)")) != RT_OK) return s;
    int limit = 0;
    CK(cudaMemcpyAsync(&limit, limit_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (limit) return fail(RT_ERR_LIMIT, limit_message(limit));
    return RT_OK;
}

// =====================================================================
// internal hooks for the batch and server layer (rt_serve.cpp)
// =====================================================================
rt_status rt_internal_error(rt_status st, const char *msg) { return fail(st, msg ? msg : ""); }
int rt_internal_device(const rt_ctx *c) { return c->device; }
int rt_internal_bvh_width(const rt_ctx *c) { return c->bvh_width; }
static int trace_width(const rt_ctx *ctx, const rt_scene *sc)
{
    if (ctx->bvh_width == 8 && sc->wide_ok) return 8;
    if (ctx->bvh_width == 4 && sc->w4_ok) return 4;
    return 2;
}
int rt_internal_graphs(const rt_ctx *c) { return c->graphs; }
int rt_internal_volpath_wave(const rt_ctx *c) { return c->volpath_wave; }
int rt_internal_batch_wave(const rt_ctx *c) { return c->batch_wave; }
void rt_internal_set_batch_wave(rt_ctx *c, int on) { c->batch_wave = on ? 1 : 0; }
bool rt_internal_multi_ok(const rt_scene *sc, const rt_render_desc *rd)
{
    const DevCamera &cam = sc->S.cam;
    return rd->integrator == RT_INTEGRATOR_PATH_MIS && rd->strategy != RT_STRATEGY_ALL_LIGHTS && rd->spp > 0 &&
           rd->sample_begin >= 0 && rd->max_depth >= 0 && rd->min_depth >= 0 && rd->max_depth <= (1 << 16) &&
           !(rd->flags & ~RT_RENDER_ACCUMULATE) && cam.filter == RT_FILTER_BOX && cam.frx == 0.5f &&
           cam.fry == 0.5f;
}
void rt_internal_set_volpath_wave(rt_ctx *c, int on) { c->volpath_wave = on ? 1 : 0; }
void rt_internal_get_shape(const rt_ctx *c, int *wave_paths, int *trace_bpsm, int *shade_bpsm, int *sort_threshold)
{
    *wave_paths = c->wave_paths;
    *trace_bpsm = c->trace_bpsm;
    *shade_bpsm = c->shade_bpsm;
    *sort_threshold = c->sort_threshold;
}
rt_status rt_internal_set_shape(rt_ctx *c, int trace_bpsm, int shade_bpsm, int sort_threshold)
{
    if (trace_bpsm < 1 || trace_bpsm > 64 || shade_bpsm < 1 || shade_bpsm > 64 || sort_threshold < 0)
        return fail(RT_ERR_INVALID, "tuning: blocks per SM must be in 1..64 and the sort threshold >= 0");
    c->trace_bpsm = trace_bpsm;
    c->shade_bpsm = shade_bpsm;
    c->sort_threshold = sort_threshold;
    return RT_OK;
}
void *rt_internal_stream(const rt_ctx *c) { return (void *)c->stream; }
rt_lane_pool *&rt_internal_pool(rt_ctx *c) { return c->pool; }
void rt_internal_set_stats(rt_ctx *c, const rt_render_stats &s) { c->last = s; }
void rt_internal_film_size(const rt_scene *sc, int *w, int *h)
{
    *w = sc->S.cam.width;
    *h = sc->S.cam.height;
}

// partial sums of (a.rgb/a.w - b.rgb/b.w)^2 over pixels with weight in both
__device__ __forceinline__ double film_mean(float v, float w, int clip)
{
    const double m = (double)v / w;
    return clip ? fmin(fmax(m, 0.0), 1.0) : m;
}
__global__ void k_film_sqdiff(const float4 *a, const float4 *b, size_t npix, int clip, double *partial)
{
    __shared__ double sh[256];
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x) {
        float4 x = a[i], y = b[i];
        if (x.w > 0.f && y.w > 0.f) {
            double dr = film_mean(x.x, x.w, clip) - film_mean(y.x, y.w, clip);
            double dg = film_mean(x.y, x.w, clip) - film_mean(y.y, y.w, clip);
            double db = film_mean(x.z, x.w, clip) - film_mean(y.z, y.w, clip);
            acc += dr * dr + dg * dg + db * db;
        }
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_film_add(float4 *dst, const float4 *src, size_t npix)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x) {
        float4 d = dst[i], s = src[i];
        dst[i] = make_float4(d.x + s.x, d.y + s.y, d.z + s.z, d.w + s.w);
    }
}

rt_status rt_internal_film_sqdiff(rt_ctx *c, const float *a, const float *b, size_t npix, int clip,
                                  double *mean_sq)
{
    CK(cudaSetDevice(c->device));
    const int blocks = 256;
    double *part = nullptr;
    CK(cudaMalloc(&part, blocks * sizeof(double)));
    k_film_sqdiff<<<blocks, 256, 0, c->stream>>>(reinterpret_cast<const float4 *>(a), reinterpret_cast<const float4 *>(b),
                                                  npix, clip, part);
    double h[blocks];
    cudaError_t e = cudaMemcpyAsync(h, part, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(part);
    if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("film comparison: ") + cudaGetErrorString(e));
    double s = 0.0;
    for (int i = 0; i < blocks; i++) s += h[i];
    *mean_sq = npix ? s / (3.0 * (double)npix) : 0.0;
    return RT_OK;
}

rt_status rt_internal_film_add(rt_ctx *c, float *dst, const float *src, size_t npix)
{
    CK(cudaSetDevice(c->device));
    k_film_add<<<std::max(1, std::min((int)((npix + 255) / 256), 1024)), 256, 0, c->stream>>>(
        reinterpret_cast<float4 *>(dst), reinterpret_cast<const float4 *>(src), npix);
    return launch_check("k_film_add");
}
