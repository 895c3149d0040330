// rt_volpath.cuh -- VolPathTracing on the device: the persistent kernel
// (k_volpath, one vol_step pass of the reference's bounce loop per call) and
// the wavefront of six kernels over path queues (k_vw_*).  Textually part of
// rt_api.cu (included there after the PathTracingMIS kernels), which holds
// RenderParams, the queue helpers and the BSDF dispatch these use.
#pragma once

// ---------------------------------------------------------------- VolPathTracing
// Integrator::evalTransmittance (Integrator.cpp:81-133)
// Out-of-line copies of the helpers the VolPath code calls from many sites.
// Inlined, every call site carried its own BVH traversal, tracking loop and
// BSDF switch; the resulting kernel missed the instruction cache on most
// issues.  One out-of-line copy each keeps the hot code small.
__device__ __noinline__ bool vp_trace(const DevScene &S, V3 o, V3 d, float mint, float maxt, Hit &h)
{
    return trace_ray<false>(S, o, d, mint, maxt, h);
}
__device__ __noinline__ Frame vp_frame(const DevScene &S, const Hit &h, V3 o, V3 d) { return hit_frame(S, h, o, d); }
// the frame of a hit that may be shaded, with its texture coordinates when
// the scene has textured BSDFs (a sphere's need the ray that found the hit)
__device__ __noinline__ Frame vp_frame_uv(const DevScene &S, const Hit &h, V3 o, V3 d, V2 &uv)
{
    if (S.has_textured) uv = hit_uv(S, h, o, d);
    return hit_frame(S, h, o, d);
}
__device__ __noinline__ C3 vp_medium_tr(const DevMedium &m, Ray r, Pcg32 &rng, int &limit)
{
    return medium_tr(m, r, rng, limit);
}
__device__ __noinline__ bool vp_medium_sample(const DevMedium &m, Ray r, Pcg32 &rng, float &t, C3 &w, C3 &em, int &limit)
{
    return medium_sample(m, r, rng, t, w, em, limit);
}
__device__ __noinline__ C3 vp_bsdf_sample(const DevBsdf &b, BsdfRec &r, V2 u, uint64_t aux_key)
{
    return bsdf_sample(b, r, u, aux_key);
}
__device__ __noinline__ C3 vp_bsdf_eval(const DevBsdf &b, V3 wi, V3 wo) { return bsdf_eval(b, wi, wo); }
__device__ __noinline__ float vp_bsdf_pdf(const DevBsdf &b, V3 wi, V3 wo) { return bsdf_pdf(b, wi, wo); }
__device__ __noinline__ void vp_light_sample(const DevScene &S, int idx, V3 p, V2 u, LightRec &li)
{
    light_sample(S, idx, p, u, li);
}
__device__ __noinline__ float vp_light_pdf(const DevScene &S, int l, V3 p, V3 lp, V3 ln, V3 dir)
{
    return light_pdf(S, l, p, lp, ln, dir);
}

__device__ __noinline__ C3 eval_transmittance(const DevScene &S, Ray ray, int medium, Pcg32 &rng, int &limit)
{
    Ray tr = ray;
    C3 T = cfill(1.f);
    float dist = ray.maxt;
    bool first = true;
    for (int guard = 0; guard < 4096; guard++) {
        Hit h;
        bool inter = vp_trace(S, tr.o, tr.d, tr.mint, tr.maxt, h);
        if (inter && prim_bsdf(S, h.prim) >= 0) return cfill(0.f);
        if (inter) dist -= h.t;
        if (medium >= 0)
            T = T * vp_medium_tr(S.media[medium], make_ray(tr.o, tr.d, first ? tr.mint : 0.f, inter ? h.t : dist), rng, limit);
        first = false;
        if (!inter || iszero(T)) return T;
        V3 np = tr.o + h.t * tr.d;
        Frame f = vp_frame(S, h, tr.o, tr.d);
        tr = make_ray(np, tr.d, RT_EPSILON, dist);
        if (prim_interior(S, h.prim) != prim_exterior(S, h.prim))
            medium = dot(f.n, tr.d) < 0.f ? prim_interior(S, h.prim) : prim_exterior(S, h.prim);
    }
    limit = 1;
    return cfill(0.f);
}

// VolPathTracing::evalTransmittanceFromSampledBSDF (VolPathTracing.cpp:369-424)
__device__ __noinline__ C3 eval_tr_sampled(const DevScene &S, Ray ray, Pcg32 &rng, int medium, Hit &h, Frame &fr, V2 &uv,
                              bool &was, int &newm, int &limit)
{
    Ray tr = ray;
    C3 T = cfill(1.f);
    bool first = true;
    was = false;
    for (int guard = 0; guard < 4096; guard++) {
        Hit nh;
        was = vp_trace(S, tr.o, tr.d, tr.mint, tr.maxt, nh);
        if (was) { h = nh; fr = vp_frame_uv(S, h, tr.o, tr.d, uv); }
        if (medium >= 0)
            T = T * vp_medium_tr(S.media[medium], make_ray(tr.o, tr.d, first ? tr.mint : 0.f, was ? h.t : tr.maxt), rng, limit);
        if (was && prim_bsdf(S, h.prim) >= 0) return T;
        first = false;
        if (!was || iszero(T)) return T;
        V3 np = tr.o + h.t * tr.d;
        tr = make_ray(np, tr.d, RT_EPSILON, tr.maxt);
        if (prim_interior(S, h.prim) != prim_exterior(S, h.prim)) {
            medium = dot(fr.n, tr.d) < 0.f ? prim_interior(S, h.prim) : prim_exterior(S, h.prim);
            newm = medium;
        }
    }
    limit = 1;
    return T;
}

// Integrator::sampleAttenuatedLightDirect (Integrator.cpp:137-172)
__device__ __noinline__ C3 sample_attenuated_light(const DevScene &S, V3 p, Pcg32 &rng, LightRec &li, int medium, int &limit)
{
    C3 value = cfill(0.f);
    if (S.n_lights == 0) return value;
    V2 u = next2d(rng);
    float lw;
    int idx = cdf_sample_reuse(S.light_cdf, S.n_lights + 1, u.x, lw);
    vp_light_sample(S, idx, p, u, li);
    if (li.pdf > 0 && lum(li.intensity) > 0) {
        C3 tr = eval_transmittance(S, make_ray(p, li.to_light, RT_EPSILON, li.distance - RT_EPSILON), medium, rng, limit);
        li.pdf *= lw;
        value = (tr * li.intensity) / li.pdf;
    }
    return value;
}

// VolPathTracing::li (VolPathTracing.cpp:25-367)
// One VolPathTracing path as a resumable state: vol_start traces the camera
// ray, each vol_step runs one pass of the bounce loop of
// VolPathTracing::li (VolPathTracing.cpp:25-367) and returns false once the
// path has finished (its radiance is then in L).  The draws from the path's
// sample stream come in the same order as one uninterrupted loop.
struct VolState {
    C3 L, T;
    V2 uv;            // texture coordinates of h (scenes with textured BSDFs)
    float eta;
    int depth, medium, guard;
    bool emission, was;
    Ray ray;
    Hit h;
    Frame fr;
};

__device__ __forceinline__ void vol_start(const DevScene &S, VolState &st, Ray ray)
{
    st.L = cfill(0.f); st.T = cfill(1.f);
    st.eta = 1.f;
    st.depth = 0;
    st.emission = true;
    st.h.t = RT_MAX_REAL; st.h.u = st.h.v = 0.f; st.h.prim = -1;
    st.fr.p = v3(0, 0, 0); st.fr.n = st.fr.s = st.fr.t = v3(0, 0, 0);
    st.ray = ray;
    Hit nh;
    st.was = vp_trace(S, ray.o, ray.d, ray.mint, ray.maxt, nh);
    st.uv = v2(0.f, 0.f);
    if (st.was) { st.h = nh; st.fr = vp_frame_uv(S, nh, ray.o, ray.d, st.uv); }
    st.medium = S.cam.medium;
    st.guard = 0;
}

__device__ bool vol_step(const DevScene &S, VolState &st, Pcg32 &rng, int max_depth, int min_depth, int &limit)
{
    if (st.depth >= max_depth) return false;
    if (++st.guard > (1 << 16)) { limit = 1; return false; }
    const int env = S.env_light;
    Ray &ray = st.ray;
    Hit &h = st.h;
    Frame &fr = st.fr;
    C3 &L = st.L, &T = st.T;
    bool &was = st.was;
    int &medium = st.medium;
    Hit nh;
    float t = 0.f;
    C3 wm = cfill(0.f), em = cfill(0.f);
    bool scattered = false;
    if (medium >= 0) scattered = vp_medium_sample(S.media[medium], make_ray(ray.o, ray.d, ray.mint, h.t), rng, t, wm, em, limit);
    if (scattered) {
        const DevMedium &M = S.media[medium];
        L = L + T * em;
        T = T * wm;
        fr.p = ray.o + t * ray.d;
        LightRec li;
        li.point = li.to_light = li.normal = v3(0, 0, 0);
        li.intensity = cfill(0.f); li.distance = 0.f; li.pdf = 0.f; li.delta = 0;
        C3 value = sample_attenuated_light(S, fr.p, rng, li, medium, limit);
        if (!iszero(value)) {
            // a delta light's sample takes a zero phase pdf (VolPathTracing.cpp:86)
            float pf = li.delta ? 0.f : phase_eval(M, li.to_light, -ray.d);
            float w = power_heuristic(li.pdf, pf);
            float ev = phase_eval(M, li.to_light, -ray.d);
            L = L + ((T * value) * ev) * w;
        }
        V3 wo; float pfpdf;
        float pfw = phase_sample(M, -ray.d, next2d(rng), wo, pfpdf);
        ray = make_ray(fr.p, wo, 0.f, ray.maxt);
        int newm = -1;
        C3 tr = eval_tr_sampled(S, ray, rng, medium, h, fr, st.uv, was, newm, limit);
        T = T * pfw;
        if (was) {
            int hl = prim_light(S, h.prim);
            if (hl >= 0) {
                C3 Le = area_le(S, hl, -ray.d, fr.n);
                float pl = vp_light_pdf(S, hl, fr.p, li.point, li.normal, li.to_light);
                float w = power_heuristic(pfpdf, pl);
                L = L + ((T * Le) * tr) * w;
            }
        }
    } else {
        if (medium >= 0) {
            L = L + T * em;
            T = T * wm;
        }
        if (!was) {
            if (st.emission && env >= 0) L = L + T * env_le(S.lights[env], ray.d);
            return false;
        }
        int b = prim_bsdf(S, h.prim);
        if (b < 0) {
            // null boundary: pass through without a bounce (no depth, no RR)
            ray = make_ray(fr.p, ray.d, RT_EPSILON, RT_MAX_REAL);
            if (prim_interior(S, h.prim) != prim_exterior(S, h.prim))
                medium = dot(fr.n, ray.d) < 0.f ? prim_interior(S, h.prim) : prim_exterior(S, h.prim);
            was = vp_trace(S, ray.o, ray.d, ray.mint, ray.maxt, nh);
            if (was) { h = nh; fr = vp_frame_uv(S, h, ray.o, ray.d, st.uv); }
            return true;
        }
        // a textured BSDF: a copy with its textures applied at the hit
        const DevBsdf *Bp = &S.bsdfs[b];
        DevBsdf Bl;
        if (Bp->textured) {
            Bl = *Bp;
            tex_apply(S, Bl, st.uv);
            Bp = &Bl;
        }
        const DevBsdf &B = *Bp;
        int hl = prim_light(S, h.prim);
        if (st.emission && hl >= 0) L = L + T * area_le(S, hl, -ray.d, fr.n);
        LightRec li;
        li.point = li.to_light = li.normal = v3(0, 0, 0);
        li.intensity = cfill(0.f); li.distance = 0.f; li.pdf = 0.f; li.delta = 0;
        C3 value = sample_attenuated_light(S, fr.p, rng, li, medium, limit);
        if (!iszero(value)) {
            V3 wi = to_local(fr, li.to_light), wo = to_local(fr, -ray.d);
            float ct = fabsf(wi.z);
            float bp = li.delta ? 0.f : vp_bsdf_pdf(B, wi, wo);   // VolPathTracing.cpp:222
            float w = power_heuristic(li.pdf, bp);
            L = L + (((T * value) * vp_bsdf_eval(B, wi, wo)) * ct) * w;
        }
        BsdfRec r;
        r.wi = to_local(fr, -ray.d); r.wo = v3(0, 0, 0);
        r.type = BT_ALL; r.rel_eta = 1.f; r.pdf = -1.f;
        V2 bu = next2d(rng);
        C3 f = vp_bsdf_sample(B, r, bu, rng.state);
        if (iszero(f)) return false;
        V3 pfrom = fr.p;
        ray = make_ray(fr.p, to_world(fr, r.wo), RT_EPSILON, RT_MAX_REAL);
        if (prim_interior(S, h.prim) != prim_exterior(S, h.prim))
            medium = dot(fr.n, ray.d) < 0.f ? prim_interior(S, h.prim) : prim_exterior(S, h.prim);
        int caught = -1;
        bool isenv = false;
        C3 Le = cfill(0.f);
        int newm = -1;
        C3 tr = eval_tr_sampled(S, ray, rng, medium, h, fr, st.uv, was, newm, limit);
        if (was) {
            int nl = prim_light(S, h.prim);
            if (nl >= 0) { caught = nl; Le = area_le(S, nl, -ray.d, fr.n); }
        } else if (newm < 0) {
            if (env >= 0) { caught = env; isenv = true; Le = env_le(S.lights[env], ray.d); }
        }
        if (caught >= 0) {
            float pl = (r.type & BT_DELTA) ? 0.f : vp_light_pdf(S, caught, pfrom, fr.p, fr.n, ray.d);
            float w = power_heuristic(r.pdf, pl);
            L = L + (((T * Le) * f) * tr) * w;
            if (isenv && medium < 0) return false;
        }
        T = T * f;
        st.eta *= r.rel_eta;
    }
    if (st.depth >= min_depth) {
        float stop = smin(0.95f, cmax(T) * st.eta * st.eta);
        if (next1d(rng) < stop) T = T / stop;
        else return false;
    }
    was = vp_trace(S, ray.o, ray.d, ray.mint, ray.maxt, nh);
    if (was) { h = nh; fr = vp_frame_uv(S, h, ray.o, ray.d, st.uv); }
    st.emission = false;
    st.depth++;
    return true;
}

// Persistent VolPath kernel with per-lane path regeneration: a lane whose
// path finished takes the next path of the batch (warp-aggregated atomic),
// so the lanes of a warp stay busy however long each path runs.
// The kernel waits on memory (grid lookups, traversal) far more than it
// computes: full occupancy (16 blocks of 128 threads per SM, 32 registers,
// the rest spilled to L1-resident local memory) ran it 1.8x faster than the
// 114-register version at 4 blocks per SM.
#ifndef RT_VOLPATH_MINB
#define RT_VOLPATH_MINB 16
#endif
#ifndef RT_VOLPATH_GRID
#define RT_VOLPATH_GRID 32
#endif
__global__ void __launch_bounds__(128, RT_VOLPATH_MINB) k_volpath(RenderParams P, int *work)
{
    const int lane = threadIdx.x & 31;
    int limit = 0;
    VolState st;
    Pcg32 rng;
    rng.state = rng.inc = 0;
    int slot = -1;
    bool active = false, more = true;
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !active && more);
        if (need) {
            int base = 0;
            const int leader = __ffs(need) - 1;
            if (lane == leader) base = atomicAdd(work, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active && more) {
                int q = base + __popc(need & ((1u << lane) - 1));
                if (q < P.n_paths) {
                    slot = q;
                    rng = P.W.rng[slot];
                    float4 ro = P.W.ray_o[slot], rd = P.W.ray_d[slot];
                    vol_start(P.S, st, make_ray(xyz(ro), xyz(rd), ro.w, rd.w));
                    active = true;
                } else {
                    more = false;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active && !vol_step(P.S, st, rng, P.max_depth, P.min_depth, limit)) {
            P.W.out[slot] = f4c(st.L, 0.f);
            active = false;
        }
    }
    if (limit) atomicOr(P.limit_flag, RT_LIM_VOLPATH);
}

// ---------------------------------------------------------------- VolPathTracing wavefront
// The same bounce loop as vol_step, split at its loops into kernels, each
// over a queue of paths in HBM.  One round runs one vol_step of every live
// path (a bounce, or a null-boundary crossing, which the reference also
// runs as one pass of its loop):
//   k_vw_trace_step [trace queue]  closest hit of the path's ray (the trace
//                                  that ends vol_step / vol_start / a null
//                                  crossing), then depth and guard, delta
//                                  tracking through the medium, then either
//                                  the scatter point or the surface
//                                  (emission, null boundary, env miss), and
//                                  the light pick and sample of
//                                  sampleAttenuatedLightDirect
//   k_vw_shadow  [shadow queue]    the light sample's transmittance
//                                  (evalTransmittance: traces through null
//                                  boundaries, ratio tracking in media)
//   k_vw_sample_surface [surface sample queue]  the light sample's MIS
//                                  contribution, the BSDF sample and the new
//                                  ray
//   k_vw_trsamp_finish [trsamp queue]  evalTransmittanceFromSampledBSDF
//                                  along it, then emission MIS of what the
//                                  sampled ray found, throughput, Russian
//                                  roulette
//   k_vw_scatter [medium sample queue]  the same three steps for scatter
//                                  points in media (phase function), in
//                                  one kernel
// Each path's draws come in the order of one uninterrupted vol_step, so a
// path's radiance is the megakernel's.  The hit frame is not stored: it is
// rebuilt from the hit, the origin of the ray segment that found it and the
// path's direction (hit_frame), which is what the megakernel holds.  Queue
// counts live in the round's RoundCounters: trace = closest (queue
// q_closest in even rounds, q_mat[0] in odd ones), shadow = shadow, sample =
// mat[1] (medium vertices) and mat[4] (surface vertices), trsamp = mat[2];
// the next round's trace queue is the next counters' closest.
enum { VF_FIRST = F_FIRST, VF_EMISSION = 2, VF_WAS = 4, VF_SCAT = 8, VF_NULLX = 16, VF_DELTA = 32, VF_NEWM = 64,
       VF_HASVAL = 128, VF_GUARD_SHIFT = 8 };

// Integrator::sampleAttenuatedLightDirect (Integrator.cpp:137-172) up to its
// shadow ray: the light pick and sample.  Returns whether the shadow ray's
// transmittance is needed; li is zero without lights.
__device__ __forceinline__ bool vw_light_pick(const DevScene &S, V3 p, Pcg32 &rng, LightRec &li, float &lw)
{
    li.point = li.to_light = li.normal = v3(0, 0, 0);
    li.intensity = cfill(0.f); li.distance = 0.f; li.pdf = 0.f; li.delta = 0;
    lw = 0.f;
    if (S.n_lights == 0) return false;
    V2 u = next2d(rng);
    int idx = cdf_sample_reuse(S.light_cdf, S.n_lights + 1, u.x, lw);
    vp_light_sample(S, idx, p, u, li);
    return li.pdf > 0 && lum(li.intensity) > 0;
}
__device__ __forceinline__ void vw_store_light(const RenderParams &P, int slot, const LightRec &li, V3 p, float lw)
{
    P.W.v_p[slot] = f4(p, lw);
    P.W.v_li0[slot] = f4(li.to_light, li.distance);
    P.W.v_li1[slot] = f4(li.point, li.pdf);
    P.W.v_li2[slot] = f4(li.normal, li.delta ? 1.f : 0.f);
    P.W.v_val[slot] = f4c(li.intensity, 0.f);
}
__device__ __forceinline__ void vw_done(const RenderParams &P, int slot, C3 L) { P.W.out[slot] = f4c(L, 0.f); }

// evalTransmittanceFromSampledBSDF (VolPathTracing.cpp:369-424), as
// eval_tr_sampled, reporting the segment origin of the hit instead of its frame
__device__ __noinline__ C3 vw_tr_sampled(const DevScene &S, Ray ray, Pcg32 &rng, int medium, Hit &h, V3 &seg, bool &was,
                                         int &newm, int &limit)
{
    Ray tr = ray;
    C3 T = cfill(1.f);
    bool first = true;
    was = false;
    for (int guard = 0; guard < 4096; guard++) {
        Hit nh;
        was = vp_trace(S, tr.o, tr.d, tr.mint, tr.maxt, nh);
        if (was) { h = nh; seg = tr.o; }
        if (medium >= 0)
            T = T * vp_medium_tr(S.media[medium], make_ray(tr.o, tr.d, first ? tr.mint : 0.f, was ? h.t : tr.maxt), rng, limit);
        if (was && prim_bsdf(S, h.prim) >= 0) return T;
        first = false;
        if (!was || iszero(T)) return T;
        V3 np = tr.o + h.t * tr.d;
        const V3 seg_o = tr.o;
        tr = make_ray(np, tr.d, RT_EPSILON, tr.maxt);
        if (prim_interior(S, h.prim) != prim_exterior(S, h.prim)) {
            Frame f = vp_frame(S, h, seg_o, tr.d);
            medium = dot(f.n, tr.d) < 0.f ? prim_interior(S, h.prim) : prim_exterior(S, h.prim);
            newm = medium;
        }
    }
    limit = 1;
    return T;
}

// resident 128-thread blocks per SM of each wavefront kernel (its launch
// bound and its grid); the tracking loops of shadow and trsamp wait on memory
#ifndef RT_VW_MINB
#define RT_VW_MINB 8
#endif
#ifndef RT_VW_MINB_STEP
#define RT_VW_MINB_STEP RT_VW_MINB
#endif
#ifndef RT_VW_MINB_SHADOW
#define RT_VW_MINB_SHADOW RT_VW_MINB
#endif
#ifndef RT_VW_MINB_SAMPLE
#define RT_VW_MINB_SAMPLE RT_VW_MINB
#endif
#ifndef RT_VW_MINB_TRSAMP
#define RT_VW_MINB_TRSAMP RT_VW_MINB
#endif
#define VW_LOOP(COUNT, QUEUE)                                                                      \
    const int n_ = (COUNT);                                                                        \
    const int *qin_ = (QUEUE);                                                                     \
    for (int i_ = blockIdx.x * blockDim.x + threadIdx.x; i_ < n_; i_ += gridDim.x * blockDim.x)

// The trace queue of a round: rounds alternate between two arrays, since
// the kernel that reads round r's queue also appends to round r + 1's.
__device__ __forceinline__ int *vw_trace_queue(const RenderParams &P, int round)
{
    return (round & 1) ? P.W.q_mat[0] : P.W.q_closest;
}

// k_vw_trace_step: the closest hit of the path's ray (the trace that ends
// vol_step, vol_start or a null crossing), then the step over that hit:
// depth and guard, delta tracking through the medium, then the scatter point
// or the surface (emission, null boundary, env miss), and the light pick and
// sample of sampleAttenuatedLightDirect.  The trace's hit, segment origin,
// flags and depth stay in registers for the step; the hit is stored for the
// kernels after it.
__global__ void __launch_bounds__(128, RT_VW_MINB_STEP) k_vw_trace_step(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene &S = P.S;
    RoundCounters *C = &P.W.cnt[round];
    RoundCounters *Cn = &P.W.cnt[round + 1];
    int *next_q = vw_trace_queue(P, round + 1);
    int limit = 0;
    VW_LOOP(C->closest, vw_trace_queue(P, round))
    {
        const int slot = qin_[i_];
        // ---- the trace (k_vw_trace)
        int flags = P.W.flags[slot];
        const float4 ro = P.W.ray_o[slot], rd = P.W.ray_d[slot];
        float4 radv = P.W.rad[slot];
        float4 seg;
        Hit h;
        if (flags & VF_FIRST) {
            h.t = RT_MAX_REAL; h.u = h.v = 0.f; h.prim = -1;
            seg = make_float4(0.f, 0.f, 0.f, __int_as_float(S.cam.medium));
            flags = VF_EMISSION;
        } else {
            const float4 hv = P.W.hit[slot];
            h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_int(hv.w);
            seg = P.W.v_seg[slot];
            if (!(flags & VF_NULLX)) {   // the trace that ends a bounce
                flags &= ~VF_EMISSION;
                radv.w = __int_as_float(__float_as_int(radv.w) + 1);
            }
        }
        {
            Hit nh;
            const bool was = vp_trace(S, xyz(ro), xyz(rd), ro.w, rd.w, nh);
            if (was) {
                h = nh;
                seg = make_float4(ro.x, ro.y, ro.z, seg.w);
            }
            flags = (flags & ~(VF_NULLX | VF_WAS)) | (was ? VF_WAS : 0);
        }
        P.W.hit[slot] = make_float4(h.t, h.u, h.v, __int_as_float(h.prim));
        // ---- the step (k_vw_step)
        const float4 tpv = P.W.tp[slot];
        C3 L = rgb(radv), T = rgb(tpv);
        const int depth = __float_as_int(radv.w);
        bool push_shadow = false, push_sample = false, push_trace = false;
        int guard = (flags >> VF_GUARD_SHIFT) + 1;
        if (depth >= P.max_depth) {
            vw_done(P, slot, L);
        } else if (guard > (1 << 16)) {
            limit = 1;
            vw_done(P, slot, L);
        } else {
            Pcg32 rng = P.W.rng[slot];
            Ray ray = make_ray(xyz(ro), xyz(rd), ro.w, rd.w);
            int medium = __float_as_int(seg.w);
            float t = 0.f;
            C3 wm = cfill(0.f), em = cfill(0.f);
            bool scattered = false;
            if (medium >= 0)
                scattered = vp_medium_sample(S.media[medium], make_ray(ray.o, ray.d, ray.mint, h.t), rng, t, wm, em, limit);
            bool done = false;
            if (scattered) {
                L = L + T * em;
                T = T * wm;
                V3 p = ray.o + t * ray.d;
                LightRec li;
                float lw;
                const bool shadow = vw_light_pick(S, p, rng, li, lw);
                vw_store_light(P, slot, li, p, lw);
                flags |= VF_SCAT;
                flags &= ~VF_HASVAL;
                push_shadow = shadow;
                push_sample = !shadow;
            } else {
                flags &= ~VF_SCAT;
                if (medium >= 0) {
                    L = L + T * em;
                    T = T * wm;
                }
                if (!(flags & VF_WAS)) {
                    if ((flags & VF_EMISSION) && S.env_light >= 0) L = L + T * env_le(S.lights[S.env_light], ray.d);
                    done = true;
                } else {
                    Frame fr = vp_frame(S, h, xyz(seg), ray.d);
                    if (prim_bsdf(S, h.prim) < 0) {
                        // null boundary: through, without a bounce
                        ray = make_ray(fr.p, ray.d, RT_EPSILON, RT_MAX_REAL);
                        if (prim_interior(S, h.prim) != prim_exterior(S, h.prim))
                            medium = dot(fr.n, ray.d) < 0.f ? prim_interior(S, h.prim) : prim_exterior(S, h.prim);
                        P.W.ray_o[slot] = f4(ray.o, ray.mint);
                        P.W.ray_d[slot] = f4(ray.d, ray.maxt);
                        flags |= VF_NULLX;
                        push_trace = true;
                    } else {
                        int hl = prim_light(S, h.prim);
                        if ((flags & VF_EMISSION) && hl >= 0) L = L + T * area_le(S, hl, -ray.d, fr.n);
                        LightRec li;
                        float lw;
                        const bool shadow = vw_light_pick(S, fr.p, rng, li, lw);
                        vw_store_light(P, slot, li, fr.p, lw);
                        flags &= ~VF_HASVAL;
                        push_shadow = shadow;
                        push_sample = !shadow;
                    }
                }
            }
            if (done) {
                vw_done(P, slot, L);
            } else {
                P.W.rng[slot] = rng;
                P.W.rad[slot] = f4c(L, __int_as_float(depth));
                P.W.tp[slot] = f4c(T, tpv.w);
                P.W.v_seg[slot] = make_float4(seg.x, seg.y, seg.z, __int_as_float(medium));
                P.W.flags[slot] = (flags & ((1 << VF_GUARD_SHIFT) - 1)) | (guard << VF_GUARD_SHIFT);
            }
        }
        const bool scat = (flags & VF_SCAT) != 0;
        q_push(P.W.q_shadow, &C->shadow, slot, push_shadow);
        q_push(P.W.q_mat[1], &C->mat[1], slot, push_sample && scat);
        q_push(P.W.q_mat[4], &C->mat[4], slot, push_sample && !scat);
        q_push(next_q, &Cn->closest, slot, push_trace);
    }
    if (limit) atomicOr(P.limit_flag, RT_LIM_VOLPATH);
}

__global__ void __launch_bounds__(128, RT_VW_MINB_SHADOW) k_vw_shadow(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene &S = P.S;
    RoundCounters *C = &P.W.cnt[round];
    int limit = 0;
    VW_LOOP(C->shadow, P.W.q_shadow)
    {
        const int slot = qin_[i_];
        Pcg32 rng = P.W.rng[slot];
        float4 pv = P.W.v_p[slot], l0 = P.W.v_li0[slot], l1 = P.W.v_li1[slot], iv = P.W.v_val[slot];
        const int medium = __float_as_int(P.W.v_seg[slot].w);
        C3 tr = eval_transmittance(S, make_ray(xyz(pv), xyz(l0), RT_EPSILON, l0.w - RT_EPSILON), medium, rng, limit);
        float pdf = l1.w * pv.w;
        C3 value = (tr * rgb(iv)) / pdf;
        P.W.v_li1[slot] = make_float4(l1.x, l1.y, l1.z, pdf);
        P.W.v_val[slot] = f4c(value, 0.f);
        P.W.rng[slot] = rng;
        const int flags = P.W.flags[slot] | VF_HASVAL;
        P.W.flags[slot] = flags;
        q_push(P.W.q_mat[1], &C->mat[1], slot, (flags & VF_SCAT) != 0);
        q_push(P.W.q_mat[4], &C->mat[4], slot, (flags & VF_SCAT) == 0);
    }
    if (limit) atomicOr(P.limit_flag, RT_LIM_VOLPATH);
}

// k_vw_sample_surface: the paths whose vertex is on a surface (sample queue
// mat[4]): the light sample's MIS with the BSDF (textures applied), the BSDF
// sample and the new ray.  Scatter points in media (mat[1]) go through
// k_vw_scatter, which continues into the sampled ray's transmittance.
__global__ void __launch_bounds__(128, RT_VW_MINB_SAMPLE) k_vw_sample_surface(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene &S = P.S;
    RoundCounters *C = &P.W.cnt[round];
    VW_LOOP(C->mat[4], P.W.q_mat[4])
    {
        const int slot = qin_[i_];
        int flags = P.W.flags[slot];
        Pcg32 rng = P.W.rng[slot];
        float4 radv = P.W.rad[slot], tpv = P.W.tp[slot];
        C3 L = rgb(radv), T = rgb(tpv);
        float4 ro = P.W.ray_o[slot], rd = P.W.ray_d[slot];
        Ray ray = make_ray(xyz(ro), xyz(rd), ro.w, rd.w);
        float4 seg = P.W.v_seg[slot];
        int medium = __float_as_int(seg.w);
        const bool hasval = flags & VF_HASVAL;
        C3 value = hasval ? rgb(P.W.v_val[slot]) : cfill(0.f);
        bool push = true;
        {
            float4 hv = P.W.hit[slot];
            Hit h; h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_int(hv.w);
            Frame fr = vp_frame(S, h, xyz(seg), ray.d);
            const DevBsdf *Bp = &S.bsdfs[prim_bsdf(S, h.prim)];
            DevBsdf Bl;
            if (Bp->textured) {
                Bl = *Bp;
                tex_apply(S, Bl, hit_uv(S, h, xyz(seg), ray.d));
                Bp = &Bl;
            }
            const DevBsdf &B = *Bp;
            if (!iszero(value)) {
                V3 to_light = xyz(P.W.v_li0[slot]);
                float lpdf = P.W.v_li1[slot].w;
                V3 wi = to_local(fr, to_light), wo = to_local(fr, -ray.d);
                float ct = fabsf(wi.z);
                float bp = P.W.v_li2[slot].w != 0.f ? 0.f : vp_bsdf_pdf(B, wi, wo);
                float w = power_heuristic(lpdf, bp);
                L = L + (((T * value) * vp_bsdf_eval(B, wi, wo)) * ct) * w;
            }
            BsdfRec r;
            r.wi = to_local(fr, -ray.d); r.wo = v3(0, 0, 0);
            r.type = BT_ALL; r.rel_eta = 1.f; r.pdf = -1.f;
            V2 bu = next2d(rng);
            C3 f = vp_bsdf_sample(B, r, bu, rng.state);
            if (iszero(f)) {
                vw_done(P, slot, L);
                push = false;
            } else {
                ray = make_ray(fr.p, to_world(fr, r.wo), RT_EPSILON, RT_MAX_REAL);
                if (prim_interior(S, h.prim) != prim_exterior(S, h.prim))
                    medium = dot(fr.n, ray.d) < 0.f ? prim_interior(S, h.prim) : prim_exterior(S, h.prim);
                P.W.bs[slot] = f4c(f, r.pdf);
                P.W.rel_eta[slot] = r.rel_eta;
                flags = (r.type & BT_DELTA) ? (flags | VF_DELTA) : (flags & ~VF_DELTA);
            }
        }
        if (push) {
            P.W.rng[slot] = rng;
            P.W.rad[slot] = f4c(L, radv.w);
            P.W.ray_o[slot] = f4(ray.o, ray.mint);
            P.W.ray_d[slot] = f4(ray.d, ray.maxt);
            P.W.v_seg[slot] = make_float4(seg.x, seg.y, seg.z, __int_as_float(medium));
            P.W.flags[slot] = flags;
        }
        q_push(P.W.q_mat[2], &C->mat[2], slot, push);
    }
}

// The end of a pass once the sampled ray's transmittance is known: emission
// MIS of what the ray found, throughput, Russian roulette
// (VolPathTracing.cpp:300-367).  ro, rd: the sampled ray; h, seg, was,
// flags: what evalTransmittanceFromSampledBSDF reported; L: the radiance with
// this vertex's light-sample MIS.  Survivors go to the next round's trace
// queue with their sampled ray.
__device__ __forceinline__ void vw_finish_one(const RenderParams &P, const DevScene &S, RoundCounters *Cn,
                                              int *next_q, int slot, int flags, Pcg32 rng, float4 ro, float4 rd,
                                              float4 seg, const Hit &h, bool was, C3 tr, C3 L, int depth,
                                              float4 tpv, float4 bsv)
{
    C3 T = rgb(tpv);
    float eta = tpv.w;
    const V3 d = xyz(rd);
    const int medium = __float_as_int(seg.w);
    bool done = false;
    if (flags & VF_SCAT) {
        T = T * rgb(bsv);
        if (was) {
            int hl = prim_light(S, h.prim);
            if (hl >= 0) {
                Frame fr = vp_frame(S, h, xyz(seg), d);
                C3 Le = area_le(S, hl, -d, fr.n);
                float pl = vp_light_pdf(S, hl, fr.p, xyz(P.W.v_li1[slot]), xyz(P.W.v_li2[slot]),
                                        xyz(P.W.v_li0[slot]));
                float w = power_heuristic(bsv.w, pl);
                L = L + ((T * Le) * tr) * w;
            }
        }
    } else {
        const C3 f = rgb(bsv);
        int caught = -1;
        bool isenv = false;
        C3 Le = cfill(0.f);
        Frame fr;
        fr.p = fr.n = v3(0, 0, 0);
        if (was) {
            int nl = prim_light(S, h.prim);
            if (nl >= 0) {
                caught = nl;
                fr = vp_frame(S, h, xyz(seg), d);
                Le = area_le(S, nl, -d, fr.n);
            }
        } else if (!(flags & VF_NEWM)) {
            // a miss: the environment (its pdf depends on the direction only)
            if (S.env_light >= 0) { caught = S.env_light; isenv = true; Le = env_le(S.lights[S.env_light], d); }
        }
        if (caught >= 0) {
            float pl = (flags & VF_DELTA) ? 0.f : vp_light_pdf(S, caught, xyz(P.W.v_p[slot]), fr.p, fr.n, d);
            float w = power_heuristic(bsv.w, pl);
            L = L + (((T * Le) * f) * tr) * w;
            if (isenv && medium < 0) done = true;
        }
        if (!done) {
            T = T * f;
            eta *= P.W.rel_eta[slot];
        }
    }
    if (!done && depth >= P.min_depth) {
        float stop = smin(0.95f, cmax(T) * eta * eta);
        if (next1d(rng) < stop) T = T / stop;
        else done = true;
    }
    if (done) {
        vw_done(P, slot, L);
    } else {
        P.W.rng[slot] = rng;
        P.W.ray_o[slot] = ro;
        P.W.ray_d[slot] = rd;
        P.W.hit[slot] = make_float4(h.t, h.u, h.v, __int_as_float(h.prim));
        P.W.v_seg[slot] = seg;
        P.W.flags[slot] = flags;
        P.W.rad[slot] = f4c(L, __int_as_float(depth));
        P.W.tp[slot] = f4c(T, eta);
    }
    q_push(next_q, &Cn->closest, slot, !done);
}

// k_vw_trsamp_finish: evalTransmittanceFromSampledBSDF along the ray that
// k_vw_sample_surface sampled at a surface vertex, then vw_finish_one
__global__ void __launch_bounds__(128, RT_VW_MINB_TRSAMP) k_vw_trsamp_finish(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene &S = P.S;
    RoundCounters *C = &P.W.cnt[round];
    RoundCounters *Cn = &P.W.cnt[round + 1];
    int *next_q = vw_trace_queue(P, round + 1);
    int limit = 0;
    VW_LOOP(C->mat[2], P.W.q_mat[2])
    {
        const int slot = qin_[i_];
        int flags = P.W.flags[slot];
        Pcg32 rng = P.W.rng[slot];
        const float4 ro = P.W.ray_o[slot], rd = P.W.ray_d[slot];
        const float4 hv = P.W.hit[slot];
        Hit h; h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_int(hv.w);
        float4 seg = P.W.v_seg[slot];
        V3 so = xyz(seg);
        bool was;
        int newm = -1;
        const C3 tr = vw_tr_sampled(S, make_ray(xyz(ro), xyz(rd), ro.w, rd.w), rng, __float_as_int(seg.w), h, so,
                                    was, newm, limit);
        flags = (flags & ~(VF_WAS | VF_NEWM)) | (was ? VF_WAS : 0) | (newm >= 0 ? VF_NEWM : 0);
        seg = make_float4(so.x, so.y, so.z, seg.w);
        const float4 radv = P.W.rad[slot];
        vw_finish_one(P, S, Cn, next_q, slot, flags, rng, ro, rd, seg, h, was, tr, rgb(radv),
                      __float_as_int(radv.w), P.W.tp[slot], P.W.bs[slot]);
    }
    if (limit) atomicOr(P.limit_flag, RT_LIM_VOLPATH);
}

// k_vw_scatter: a scatter point in a medium (sample queue mat[1]) through the
// rest of its pass in one kernel: the phase sample and the new ray
// (the phase function's), the transmittance along it, then the light
// sample's MIS with the phase function (no draws, so its place after the
// transmittance leaves the path's stream as it was) and vw_finish_one
__global__ void __launch_bounds__(128, RT_VW_MINB_TRSAMP) k_vw_scatter(RenderParams P, int round)
{
    round = cur_round(P, round);
    const DevScene &S = P.S;
    RoundCounters *C = &P.W.cnt[round];
    RoundCounters *Cn = &P.W.cnt[round + 1];
    int *next_q = vw_trace_queue(P, round + 1);
    int limit = 0;
    VW_LOOP(C->mat[1], P.W.q_mat[1])
    {
        const int slot = qin_[i_];
        int flags = P.W.flags[slot];
        Pcg32 rng = P.W.rng[slot];
        float4 seg = P.W.v_seg[slot];
        const int medium = __float_as_int(seg.w);
        float4 rd = P.W.ray_d[slot];
        V3 wo;
        float pfpdf;
        const float pfw = phase_sample(S.media[medium], -xyz(rd), next2d(rng), wo, pfpdf);
        const float4 ro = f4(xyz(P.W.v_p[slot]), 0.f);
        rd = f4(wo, rd.w);
        const float4 hv = P.W.hit[slot];
        Hit h; h.t = hv.x; h.u = hv.y; h.v = hv.z; h.prim = __float_as_int(hv.w);
        V3 so = xyz(seg);
        bool was;
        int newm = -1;
        const C3 tr = vw_tr_sampled(S, make_ray(xyz(ro), wo, 0.f, rd.w), rng, medium, h, so, was, newm, limit);
        flags = (flags & ~(VF_WAS | VF_NEWM)) | (was ? VF_WAS : 0) | (newm >= 0 ? VF_NEWM : 0);
        seg = make_float4(so.x, so.y, so.z, seg.w);
        // the light sample's MIS at the scatter point
        const float4 radv = P.W.rad[slot], tpv = P.W.tp[slot];
        C3 L = rgb(radv);
        if (flags & VF_HASVAL) {
            const C3 value = rgb(P.W.v_val[slot]);
            if (!iszero(value)) {
                const DevMedium &M = S.media[medium];
                const V3 din = xyz(P.W.ray_d[slot]);
                const V3 to_light = xyz(P.W.v_li0[slot]);
                const float lpdf = P.W.v_li1[slot].w;
                const float pf = P.W.v_li2[slot].w != 0.f ? 0.f : phase_eval(M, to_light, -din);
                const float w = power_heuristic(lpdf, pf);
                const float ev = phase_eval(M, to_light, -din);
                L = L + ((rgb(tpv) * value) * ev) * w;
            }
        }
        vw_finish_one(P, S, Cn, next_q, slot, flags, rng, ro, rd, seg, h, was, tr, L, __float_as_int(radv.w), tpv,
                      f4c(cfill(pfw), pfpdf));
    }
    if (limit) atomicOr(P.limit_flag, RT_LIM_VOLPATH);
}
