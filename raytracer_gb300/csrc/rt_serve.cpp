// rt_serve.cpp -- batched and served rendering over the C ABI.
//
// The reference renders one scene per process: main() loads a scene file,
// Scene::compute splits the film into tiles and a JobManager runs them on a
// thread pool (core/main.cpp:439-447, core/Scene.cpp:83-101,
// core/JobManager.cpp:41-58).  Many small jobs leave a 152-SM GPU mostly
// idle when they run one after another: each render has a short wavefront
// and a host round trip every few bounces.  Both entry points here keep
// several renders in flight instead.
//
//   rt_batch_render  a list of (scene, render desc, film) jobs, largest
//                    first, on `lanes` worker contexts: one CUDA stream,
//                    wavefront buffers and host thread each.  Every film is
//                    the one rt_render produces for that job alone.
//   rt_server_*      continuous batching: PathTracingMIS jobs are admitted
//                    by a device-memory budget and rendered chunk by chunk,
//                    all resident jobs' chunks together in one multi-scene
//                    wavefront per step; other jobs run on lanes.  A job
//                    either renders its sample count in one chunk or, with
//                    a target RMSE, renders progressively into two films of
//                    interleaved sample ranges until the RMSE estimated
//                    from their difference meets the target.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rt_internal.h"

namespace {

double now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct LaneSet {
    int device = 0;
    // lanes overlap several renders; smaller batches than a lone render's
    // bound their memory (rt_path_state_bytes per path each)
    int wave_paths = 1 << 24;
    std::vector<rt_ctx *> lanes;

    // lanes take the owning context's traversal width, graph setting, launch
    // shape and sort threshold
    rt_status grow(int k, const rt_ctx *owner)
    {
        while ((int)lanes.size() < k) {
            rt_ctx *c = nullptr;
            rt_status s = rt_ctx_create(device, &c);
            if (s != RT_OK) return s;
            lanes.push_back(c);
        }
        int wave, tb, sb, thr;
        rt_internal_get_shape(owner, &wave, &tb, &sb, &thr);
        for (rt_ctx *c : lanes) {
            rt_ctx_set_bvh_width(c, rt_internal_bvh_width(owner));
            rt_ctx_set_graphs(c, rt_internal_graphs(owner));
            rt_internal_set_volpath_wave(c, rt_internal_volpath_wave(owner));
            rt_ctx_set_wave_paths(c, wave_paths);
            rt_status s = rt_internal_set_shape(c, tb, sb, thr);
            if (s != RT_OK) return s;
        }
        return RT_OK;
    }
    void clear()
    {
        for (rt_ctx *c : lanes) rt_ctx_destroy(c);
        lanes.clear();
    }
};

// first failure of a group of jobs run on several threads
struct FirstError {
    std::mutex mu;
    rt_status status = RT_OK;
    std::string msg;
    void set(rt_status s)
    {
        std::lock_guard<std::mutex> g(mu);
        if (status == RT_OK) {
            status = s;
            msg = rt_last_error();
        }
    }
};

void add_stats(rt_render_stats &a, const rt_render_stats &b)
{
    a.camera_ms += b.camera_ms;
    a.trace_closest_ms += b.trace_closest_ms;
    a.trace_any_ms += b.trace_any_ms;
    a.shade_ms += b.shade_ms;
    a.volpath_ms += b.volpath_ms;
    a.film_ms += b.film_ms;
    a.paths += b.paths;
    a.closest_rays += b.closest_rays;
    a.shadow_rays += b.shadow_rays;
    a.launches += b.launches;
    a.trace_closest_launches += b.trace_closest_launches;
    a.trace_any_launches += b.trace_any_launches;
    a.nodes_closest += b.nodes_closest;
    a.tris_closest += b.tris_closest;
    a.nodes_any += b.nodes_any;
    a.tris_any += b.tris_any;
    a.limit_hits += b.limit_hits;
    a.nan_samples += b.nan_samples;
    a.resolve_ms += b.resolve_ms;
    a.sort_ms += b.sort_ms;
}

}  // namespace

struct rt_lane_pool {
    int want = 4;
    LaneSet set;
};

void rt_lane_pool_destroy(rt_lane_pool *p)
{
    if (!p) return;
    p->set.clear();
    delete p;
}

static rt_lane_pool *pool_of(rt_ctx *ctx)
{
    rt_lane_pool *&p = rt_internal_pool(ctx);
    if (!p) {
        p = new rt_lane_pool();
        p->set.device = rt_internal_device(ctx);
    }
    return p;
}

extern "C" rt_status rt_ctx_set_lanes(rt_ctx *ctx, int32_t lanes)
{
    if (!ctx) return rt_internal_error(RT_ERR_INVALID, "null ctx");
    if (lanes < 1 || lanes > 16) return rt_internal_error(RT_ERR_INVALID, "lanes must be in 1..16");
    pool_of(ctx)->want = lanes;
    return RT_OK;
}

extern "C" rt_status rt_ctx_get_tuning(rt_ctx *ctx, rt_tuning *out)
{
    if (!ctx || !out) return rt_internal_error(RT_ERR_INVALID, "rt_ctx_get_tuning: null argument");
    rt_lane_pool *pool = pool_of(ctx);
    int wave, tb, sb, thr;
    rt_internal_get_shape(ctx, &wave, &tb, &sb, &thr);
    out->wave_paths = wave;
    out->lane_wave_paths = pool->set.wave_paths;
    out->trace_blocks_per_sm = tb;
    out->shade_blocks_per_sm = sb;
    out->sort_threshold = thr;
    out->lanes = pool->want;
    out->graphs = rt_internal_graphs(ctx);
    out->volpath_wavefront = rt_internal_volpath_wave(ctx);
    out->batch_wavefront = rt_internal_batch_wave(ctx);
    return RT_OK;
}

extern "C" rt_status rt_ctx_set_tuning(rt_ctx *ctx, const rt_tuning *t)
{
    if (!ctx || !t) return rt_internal_error(RT_ERR_INVALID, "rt_ctx_set_tuning: null argument");
    if (t->lane_wave_paths < (1 << 16) || t->lane_wave_paths > (1 << 26))
        return rt_internal_error(RT_ERR_INVALID, "tuning: lane wave paths must be in [2^16, 2^26]");
    if (t->graphs != 0 && t->graphs != 1) return rt_internal_error(RT_ERR_INVALID, "tuning: graphs must be 0 or 1");
    if (t->volpath_wavefront != 0 && t->volpath_wavefront != 1)
        return rt_internal_error(RT_ERR_INVALID, "tuning: volpath_wavefront must be 0 or 1");
    if (t->batch_wavefront != 0 && t->batch_wavefront != 1)
        return rt_internal_error(RT_ERR_INVALID, "tuning: batch_wavefront must be 0 or 1");
    rt_status s = rt_ctx_set_wave_paths(ctx, t->wave_paths);
    if (s == RT_OK) s = rt_internal_set_shape(ctx, t->trace_blocks_per_sm, t->shade_blocks_per_sm, t->sort_threshold);
    if (s == RT_OK) s = rt_ctx_set_lanes(ctx, t->lanes);
    if (s != RT_OK) return s;
    rt_ctx_set_graphs(ctx, t->graphs);
    rt_internal_set_volpath_wave(ctx, t->volpath_wavefront);
    rt_internal_set_batch_wave(ctx, t->batch_wavefront);
    pool_of(ctx)->set.wave_paths = t->lane_wave_paths;
    return RT_OK;
}

extern "C" rt_status rt_batch_render(rt_ctx *ctx, rt_scene *const *scenes, const rt_render_desc *descs, int32_t n,
                                     float *const *films, int32_t on_device)
{
    if (!ctx || n < 0 || (n > 0 && (!scenes || !descs || !films)))
        return rt_internal_error(RT_ERR_INVALID, "rt_batch_render: bad argument");
    for (int i = 0; i < n; i++)
        if (!scenes[i] || !films[i]) return rt_internal_error(RT_ERR_INVALID, "rt_batch_render: null scene or film");
    if (n == 0) return RT_OK;
    if (cudaSetDevice(rt_internal_device(ctx)) != cudaSuccess)
        return rt_internal_error(RT_ERR_CUDA, "rt_batch_render: cudaSetDevice failed");
    // work queued by the caller on the context's stream (e.g. clearing the
    // films) completes before the lanes start on their own streams
    if (cudaStreamSynchronize((cudaStream_t)rt_internal_stream(ctx)) != cudaSuccess)
        return rt_internal_error(RT_ERR_CUDA, "rt_batch_render: stream synchronize failed");
    // with batch_wavefront: the eligible jobs in one multi-scene wavefront
    // per (max_depth, min_depth) group on the calling context, the rest on
    // the lanes at the same time.  A job of at least a quarter of the
    // wavefront capacity fills the device by itself: it renders alone on a
    // lane, with the single-scene kernels (no per-path scene lookups).
    int wave_paths = 0, tb = 0, sb = 0, thr = 0;
    rt_internal_get_shape(ctx, &wave_paths, &tb, &sb, &thr);
    std::vector<int> lane_jobs;
    std::vector<std::vector<int>> groups;
    for (int i = 0; i < n; i++) {
        int fw = 0, fh = 0;
        rt_internal_film_size(scenes[i], &fw, &fh);
        const bool alone = (double)fw * fh * std::max(1, descs[i].spp) >= 0.25 * wave_paths;
        if (!rt_internal_batch_wave(ctx) || alone || !rt_internal_multi_ok(scenes[i], &descs[i])) {
            lane_jobs.push_back(i);
            continue;
        }
        bool placed = false;
        for (auto &g : groups)
            if (descs[g[0]].max_depth == descs[i].max_depth && descs[g[0]].min_depth == descs[i].min_depth) {
                g.push_back(i);
                placed = true;
                break;
            }
        if (!placed) groups.push_back({i});
    }
    rt_lane_pool *pool = pool_of(ctx);
    const int nl = (int)lane_jobs.size();
    const int k = std::min(pool->want, nl);
    if (k > 0) {
        rt_status s = pool->set.grow(k, ctx);
        if (s != RT_OK) return s;
    }
    // largest job first, so that the long ones do not start last
    std::vector<int> order(lane_jobs);
    std::vector<double> work(n);
    for (int i = 0; i < n; i++) {
        int w = 0, h = 0;
        rt_internal_film_size(scenes[i], &w, &h);
        work[i] = (double)w * h * std::max(1, descs[i].spp) * std::max(1, std::min(descs[i].max_depth, 64));
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
    std::atomic<int> next(0);
    FirstError err;
    std::vector<rt_render_stats> lane_stats(std::max(k, 1));
    const double t0 = now_ms();
    auto worker = [&](int li) {
        rt_ctx *lane = pool->set.lanes[li];
        std::memset(&lane_stats[li], 0, sizeof(rt_render_stats));
        for (;;) {
            int j = next.fetch_add(1);
            if (j >= nl) break;
            int i = order[j];
            rt_status st = rt_render(lane, scenes[i], &descs[i], films[i], on_device);
            if (st != RT_OK) { err.set(st); continue; }
            rt_render_stats one;
            rt_render_stats_get(lane, &one);
            add_stats(lane_stats[li], one);
        }
    };
    std::vector<std::thread> th;
    for (int li = 0; li < k; li++) th.emplace_back(worker, li);
    rt_render_stats multi_stats;
    std::memset(&multi_stats, 0, sizeof(multi_stats));
    for (auto &g : groups) {
        std::vector<rt_scene *> gs;
        std::vector<rt_render_desc> gd;
        std::vector<float *> gf;
        for (int i : g) {
            gs.push_back(scenes[i]);
            gd.push_back(descs[i]);
            gf.push_back(films[i]);
        }
        rt_status st = rt_internal_render_multi(ctx, gs.data(), gd.data(), (int)g.size(), gf.data(), on_device);
        if (st != RT_OK) { err.set(st); continue; }
        rt_render_stats one;
        rt_render_stats_get(ctx, &one);
        add_stats(multi_stats, one);
    }
    for (auto &t : th) t.join();
    rt_render_stats tot;
    std::memset(&tot, 0, sizeof(tot));
    for (int li = 0; li < k; li++) add_stats(tot, lane_stats[li]);
    add_stats(tot, multi_stats);
    tot.kernel_ms = (float)(now_ms() - t0);   // wall time of the whole batch
    rt_internal_set_stats(ctx, tot);
    if (err.status != RT_OK) return rt_internal_error(err.status, err.msg.c_str());
    return RT_OK;
}

// =====================================================================
// server
// =====================================================================
namespace {

struct Job {
    rt_job_id id = 0;
    rt_scene *scene = nullptr;
    rt_render_desc desc;
    float target = 0.f;
    int clip = 0;            // target RMSE over pixel means clipped to [0, 1] (rt_server_opts.rmse_display)
    int w = 0, h = 0;
    int64_t bytes = 0;       // device bytes held while resident: scene + films
    int state = RT_JOB_QUEUED;
    int spp_done = 0;
    float rmse = -1.f;
    double t_submit = 0, t_start = 0, t_end = 0;
    std::vector<float> film;
    std::string error;
    // continuous batching: device films (progressive: A and B, plain: A),
    // the next chunk size and the estimate so far
    bool batched = false;
    float *A = nullptr, *B = nullptr;
    int k = 0;
    double est = -1.0;
};

}  // namespace

struct rt_server {
    rt_ctx *parent = nullptr;
    LaneSet set;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job *> queue;        // waiting for a lane (jobs the wavefront cannot take)
    std::deque<Job *> bqueue;       // waiting for admission to the wavefront
    std::vector<Job *> resident;    // admitted to the wavefront, owned by the scheduler
    std::unordered_map<rt_job_id, Job *> jobs;
    bool stopping = false;
    rt_job_id next_id = 1;
    int max_queue = 4096;
    int64_t budget = 0, in_flight = 0, fixed = 0;
    bool wavefront = true;
    int rmse_display = 0;          // rt_server_opts.rmse_display
    rt_ctx *sched = nullptr;        // the wavefront's context
    std::thread scheduler;
};

// One job on one lane.  Plain jobs are a single rt_render.  Progressive
// jobs render chunks of k samples alternately into films A and B (A takes
// samples [s, s+k), B [s+k, s+2k)), so A and B are independent estimates of
// the same image; with equal counts the error of their average is
// |A - B| / 2 per pixel in expectation, and the next chunk is sized from
// the ratio of that estimate to the target.
static int next_chunk(const Job *J, int done, double est)
{
    const int cap = std::max(2, J->desc.spp);
    double need = done * (est / J->target) * (est / J->target) * 1.1;
    int nk = (int)std::ceil((need - done) * 0.5);
    return std::max(1, std::min(nk, (cap - done) / 2));
}
static int first_chunk(const Job *J) { return std::max(1, std::min(std::max(2, J->desc.spp) / 2, 4)); }

static rt_status run_job(rt_ctx *lane, Job *J)
{
    const size_t npix = (size_t)J->w * J->h;
    J->film.assign(npix * 4, 0.f);
    if (!(J->target > 0.f)) {
        rt_status s = rt_render(lane, J->scene, &J->desc, J->film.data(), 0);
        if (s == RT_OK) J->spp_done = J->desc.spp;
        return s;
    }
    float *A = nullptr, *B = nullptr;
    if (cudaMalloc((void **)&A, npix * 16) != cudaSuccess || cudaMalloc((void **)&B, npix * 16) != cudaSuccess) {
        cudaFree(A);
        return rt_internal_error(RT_ERR_NOMEM, "server: film allocation failed");
    }
    cudaStream_t st = (cudaStream_t)rt_internal_stream(lane);
    rt_status s = RT_OK;
    if (cudaMemsetAsync(A, 0, npix * 16, st) != cudaSuccess || cudaMemsetAsync(B, 0, npix * 16, st) != cudaSuccess)
        s = rt_internal_error(RT_ERR_CUDA, "server: film clear failed");
    const int cap = std::max(2, J->desc.spp);
    int done = 0, k = first_chunk(J);
    double est = -1.0;
    while (s == RT_OK) {
        rt_render_desc d = J->desc;
        d.flags |= RT_RENDER_ACCUMULATE;
        d.spp = k;
        d.sample_begin = J->desc.sample_begin + done;
        if ((s = rt_render(lane, J->scene, &d, A, 1)) != RT_OK) break;
        d.sample_begin += k;
        if ((s = rt_render(lane, J->scene, &d, B, 1)) != RT_OK) break;
        done += 2 * k;
        double msq = 0.0;
        if ((s = rt_internal_film_sqdiff(lane, A, B, npix, J->clip, &msq)) != RT_OK) break;
        est = std::sqrt(msq) * 0.5;
        if (est <= J->target || cap - done < 2) break;
        k = next_chunk(J, done, est);
    }
    if (s == RT_OK) s = rt_internal_film_add(lane, A, B, npix);
    if (s == RT_OK && cudaMemcpyAsync(J->film.data(), A, npix * 16, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        s = rt_internal_error(RT_ERR_CUDA, "server: film copy failed");
    if (s == RT_OK && cudaStreamSynchronize(st) != cudaSuccess)
        s = rt_internal_error(RT_ERR_CUDA, "server: stream synchronize failed");
    cudaFree(A);
    cudaFree(B);
    J->spp_done = done;
    J->rmse = (float)est;
    return s;
}

static bool admit_ok(const rt_server *S, const Job *J)
{
    return S->budget <= 0 || S->in_flight == 0 || S->fixed + S->in_flight + J->bytes <= S->budget;
}

static void serve(rt_server *S, int li)
{
    rt_ctx *lane = S->set.lanes[li];
    cudaSetDevice(S->set.device);
    for (;;) {
        Job *J = nullptr;
        {
            std::unique_lock<std::mutex> g(S->mu);
            S->cv_work.wait(g, [&] {
                if (S->stopping) return true;
                if (S->queue.empty()) return false;
                return admit_ok(S, S->queue.front());
            });
            if (S->stopping) return;
            J = S->queue.front();
            S->queue.pop_front();
            J->state = RT_JOB_RUNNING;
            J->t_start = now_ms();
            S->in_flight += J->bytes;
        }
        rt_status s = run_job(lane, J);
        {
            std::lock_guard<std::mutex> g(S->mu);
            J->t_end = now_ms();
            J->state = s == RT_OK ? RT_JOB_DONE : RT_JOB_FAILED;
            if (s != RT_OK) J->error = rt_last_error();
            S->in_flight -= J->bytes;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
}

// The wavefront's scheduler: continuous batching.  Every step admits the
// queued jobs that fit the device budget (their scene and films stay
// resident until they finish), then renders the next chunk of every
// resident job in one multi-scene wavefront per (max_depth, min_depth)
// group: a plain job all its samples into its film, a progressive job k
// samples into film A and the next k into film B (accumulating).  After the
// step each progressive job re-estimates its RMSE from |A - B| and sizes its
// next chunk, exactly as on a lane; a job whose estimate meets its target
// or whose samples are spent leaves with A + B.  A job's chunks depend on
// its own films only, so its film is the same alone and in any mix.
static void finish_batched(rt_server *S, Job *J, rt_status s)
{
    const size_t npix = (size_t)J->w * J->h;
    cudaStream_t st = (cudaStream_t)rt_internal_stream(S->sched);
    if (s == RT_OK && J->target > 0.f) s = rt_internal_film_add(S->sched, J->A, J->B, npix);
    if (s == RT_OK) {
        J->film.assign(npix * 4, 0.f);
        if (cudaMemcpyAsync(J->film.data(), J->A, npix * 16, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            s = rt_internal_error(RT_ERR_CUDA, "server: film copy failed");
    }
    cudaFree(J->A);
    cudaFree(J->B);
    J->A = J->B = nullptr;
    std::lock_guard<std::mutex> g(S->mu);
    J->t_end = now_ms();
    J->state = s == RT_OK ? RT_JOB_DONE : RT_JOB_FAILED;
    if (s != RT_OK) J->error = rt_last_error();
    S->in_flight -= J->bytes;
}

// Paths of a job's next step: both half chunks of a progressive job, all
// samples of a plain one.
static double step_paths(const Job *J, int k)
{
    return (double)J->w * J->h * (J->target > 0.f ? 2.0 * k : (double)J->desc.spp);
}

static void schedule(rt_server *S)
{
    cudaSetDevice(S->set.device);
    cudaStream_t st = (cudaStream_t)rt_internal_stream(S->sched);
    int wave = 0, tb = 0, sb = 0, thr = 0;
    rt_internal_get_shape(S->sched, &wave, &tb, &sb, &thr);
    for (;;) {
        std::vector<Job *> fresh;
        {
            std::unique_lock<std::mutex> g(S->mu);
            S->cv_work.wait(g, [&] { return S->stopping || !S->resident.empty() || !S->bqueue.empty(); });
            if (S->stopping) return;
            // Admission in arrival order while the budget allows and the
            // step still fits one wavefront batch: beyond that, more resident
            // jobs only share the device more finely (every job finishes
            // later), so later arrivals wait for the earlier ones.
            double step = 0.0;
            for (const Job *J : S->resident) step += step_paths(J, J->k);
            while (!S->bqueue.empty() && admit_ok(S, S->bqueue.front()) &&
                   ((S->resident.empty() && fresh.empty()) ||
                    step + step_paths(S->bqueue.front(), first_chunk(S->bqueue.front())) <= (double)wave)) {
                step += step_paths(S->bqueue.front(), first_chunk(S->bqueue.front()));
                Job *J = S->bqueue.front();
                S->bqueue.pop_front();
                J->state = RT_JOB_RUNNING;
                J->t_start = now_ms();
                S->in_flight += J->bytes;
                fresh.push_back(J);
            }
        }
        for (Job *J : fresh) {
            const size_t npix = (size_t)J->w * J->h;
            rt_status s = RT_OK;
            if (cudaMalloc((void **)&J->A, npix * 16) != cudaSuccess ||
                (J->target > 0.f && cudaMalloc((void **)&J->B, npix * 16) != cudaSuccess))
                s = rt_internal_error(RT_ERR_NOMEM, "server: film allocation failed");
            if (s == RT_OK && (cudaMemsetAsync(J->A, 0, npix * 16, st) != cudaSuccess ||
                               (J->B && cudaMemsetAsync(J->B, 0, npix * 16, st) != cudaSuccess)))
                s = rt_internal_error(RT_ERR_CUDA, "server: film clear failed");
            if (s != RT_OK) { finish_batched(S, J, s); S->cv_done.notify_all(); continue; }
            J->k = J->target > 0.f ? first_chunk(J) : J->desc.spp;
            S->resident.push_back(J);
        }
        if (S->resident.empty()) continue;
        // one step: the next chunk of every resident job
        std::vector<std::vector<int>> groups;
        for (int i = 0; i < (int)S->resident.size(); i++) {
            const rt_render_desc &d = S->resident[i]->desc;
            bool placed = false;
            for (auto &gr : groups)
                if (S->resident[gr[0]]->desc.max_depth == d.max_depth &&
                    S->resident[gr[0]]->desc.min_depth == d.min_depth) { gr.push_back(i); placed = true; break; }
            if (!placed) groups.push_back({i});
        }
        std::vector<rt_status> result(S->resident.size(), RT_OK);
        for (auto &gr : groups) {
            std::vector<rt_scene *> sc;
            std::vector<rt_render_desc> ds;
            std::vector<float *> fs;
            for (int i : gr) {
                Job *J = S->resident[i];
                rt_render_desc d = J->desc;
                if (J->target > 0.f) {
                    d.flags |= RT_RENDER_ACCUMULATE;
                    d.spp = J->k;
                    d.sample_begin = J->desc.sample_begin + J->spp_done;
                    sc.push_back(J->scene); ds.push_back(d); fs.push_back(J->A);
                    d.sample_begin += J->k;
                    sc.push_back(J->scene); ds.push_back(d); fs.push_back(J->B);
                } else {
                    sc.push_back(J->scene); ds.push_back(d); fs.push_back(J->A);
                }
            }
            rt_status s = rt_internal_render_multi(S->sched, sc.data(), ds.data(), (int)sc.size(), fs.data(), 1);
            for (int i : gr) result[i] = s;
        }
        std::vector<Job *> keep;
        for (size_t i = 0; i < S->resident.size(); i++) {
            Job *J = S->resident[i];
            rt_status s = result[i];
            bool done = s != RT_OK;
            if (s == RT_OK && J->target > 0.f) {
                J->spp_done += 2 * J->k;
                double msq = 0.0;
                s = rt_internal_film_sqdiff(S->sched, J->A, J->B, (size_t)J->w * J->h, J->clip, &msq);
                J->est = std::sqrt(msq) * 0.5;
                J->rmse = (float)J->est;
                const int cap = std::max(2, J->desc.spp);
                if (s != RT_OK || J->est <= J->target || cap - J->spp_done < 2) done = true;
                else J->k = next_chunk(J, J->spp_done, J->est);
            } else if (s == RT_OK) {
                J->spp_done = J->desc.spp;
                done = true;
            }
            if (done) {
                finish_batched(S, J, s);
                S->cv_done.notify_all();
                S->cv_work.notify_all();
            } else {
                keep.push_back(J);
            }
        }
        S->resident.swap(keep);
    }
}

extern "C" rt_status rt_server_start(rt_ctx *ctx, const rt_server_opts *opts, rt_server **out)
{
    if (!ctx || !out) return rt_internal_error(RT_ERR_INVALID, "rt_server_start: null argument");
    *out = nullptr;
    int lanes = opts && opts->lanes > 0 ? opts->lanes : 4;
    if (lanes > 16) return rt_internal_error(RT_ERR_INVALID, "rt_server_start: lanes must be in 1..16");
    if (opts && opts->lanes_only != 0 && opts->lanes_only != 1)
        return rt_internal_error(RT_ERR_INVALID, "rt_server_start: lanes_only must be 0 or 1");
    if (opts && opts->rmse_display != 0 && opts->rmse_display != 1)
        return rt_internal_error(RT_ERR_INVALID, "rt_server_start: rmse_display must be 0 or 1");
    rt_server *S = new rt_server();
    S->parent = ctx;
    S->set.device = rt_internal_device(ctx);
    S->max_queue = opts && opts->max_queue > 0 ? opts->max_queue : 4096;
    S->budget = opts ? opts->device_budget_bytes : 0;
    S->wavefront = !opts || opts->lanes_only == 0;
    S->rmse_display = opts ? opts->rmse_display : 0;
    S->set.wave_paths = pool_of(ctx)->set.wave_paths;
    rt_status s = S->set.grow(lanes, ctx);
    if (s == RT_OK && S->wavefront) {
        s = rt_ctx_create(S->set.device, &S->sched);
        int wave = 0, tb = 0, sb = 0, thr = 0;
        rt_internal_get_shape(ctx, &wave, &tb, &sb, &thr);
        if (s == RT_OK) s = rt_ctx_set_wave_paths(S->sched, wave);
        if (s == RT_OK) s = rt_internal_set_shape(S->sched, tb, sb, thr);
        // the wavefront's path state at its capacity (PathTracingMIS jobs)
        // counts against the budget from the start
        S->fixed = rt_path_state_bytes(RT_INTEGRATOR_PATH_MIS) * wave;
    }
    // and so does the lanes' (any job: VolPathTracing's state included)
    S->fixed += rt_path_state_bytes(RT_INTEGRATOR_VOLPATH) * S->set.wave_paths * lanes;
    if (s != RT_OK) {
        if (S->sched) rt_ctx_destroy(S->sched);
        S->set.clear();
        delete S;
        return s;
    }
    for (int li = 0; li < lanes; li++) S->threads.emplace_back(serve, S, li);
    if (S->wavefront) S->scheduler = std::thread(schedule, S);
    *out = S;
    return RT_OK;
}

extern "C" rt_status rt_job_submit(rt_server *S, rt_scene *scene, const rt_render_desc *desc, float target_rmse,
                                   rt_job_id *id)
{
    if (!S || !scene || !desc || !id) return rt_internal_error(RT_ERR_INVALID, "rt_job_submit: null argument");
    if (desc->spp <= 0) return rt_internal_error(RT_ERR_INVALID, "rt_job_submit: spp must be positive");
    if (desc->flags & RT_RENDER_ACCUMULATE)
        return rt_internal_error(RT_ERR_INVALID, "rt_job_submit: jobs render into their own film");
    Job *J = new Job();
    J->scene = scene;
    J->desc = *desc;
    J->target = target_rmse;
    J->clip = S->rmse_display;
    rt_internal_film_size(scene, &J->w, &J->h);
    int64_t scene_bytes = 0;
    float bounds[6];
    rt_scene_info(scene, bounds, &scene_bytes, nullptr);
    J->bytes = scene_bytes + (int64_t)J->w * J->h * 16 * (target_rmse > 0.f ? 3 : 1);
    J->batched = S->wavefront && rt_internal_multi_ok(scene, desc);
    std::lock_guard<std::mutex> g(S->mu);
    if (S->stopping) { delete J; return rt_internal_error(RT_ERR_INVALID, "rt_job_submit: server is stopping"); }
    if (S->budget > 0 && S->fixed + J->bytes > S->budget) {
        delete J;
        return rt_internal_error(RT_ERR_LIMIT, "rt_job_submit: the job's scene and films exceed the device budget");
    }
    if ((int)(S->queue.size() + S->bqueue.size()) >= S->max_queue) {
        delete J;
        return rt_internal_error(RT_ERR_LIMIT, "rt_job_submit: queue full");
    }
    J->id = S->next_id++;
    J->t_submit = now_ms();
    S->jobs[J->id] = J;
    if (J->batched) S->bqueue.push_back(J);
    else S->queue.push_back(J);
    *id = J->id;
    S->cv_work.notify_all();
    return RT_OK;
}

// fills info; with a film pointer and a finished job, copies the film out
// and forgets the job (caller holds S->mu)
static rt_status report(rt_server *S, Job *J, rt_job_info *info, float *film)
{
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->state = J->state;
        info->spp_done = J->spp_done;
        info->rmse_estimate = J->rmse;
        double t = now_ms();
        double start = J->t_start > 0 ? J->t_start : t;
        info->queue_ms = (float)(start - J->t_submit);
        info->run_ms = J->t_start > 0 ? (float)((J->t_end > 0 ? J->t_end : t) - J->t_start) : 0.f;
        std::strncpy(info->error, J->error.c_str(), sizeof(info->error) - 1);
    }
    if (film && (J->state == RT_JOB_DONE || J->state == RT_JOB_FAILED)) {
        if (J->state == RT_JOB_DONE) std::memcpy(film, J->film.data(), J->film.size() * sizeof(float));
        S->jobs.erase(J->id);
        delete J;
    }
    return RT_OK;
}

extern "C" rt_status rt_job_poll(rt_server *S, rt_job_id id, rt_job_info *info, float *film)
{
    if (!S) return rt_internal_error(RT_ERR_INVALID, "rt_job_poll: null server");
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->jobs.find(id);
    if (it == S->jobs.end()) return rt_internal_error(RT_ERR_INVALID, "rt_job_poll: unknown job");
    return report(S, it->second, info, film);
}

extern "C" rt_status rt_job_wait(rt_server *S, rt_job_id id, int32_t timeout_ms, rt_job_info *info, float *film)
{
    if (!S) return rt_internal_error(RT_ERR_INVALID, "rt_job_wait: null server");
    std::unique_lock<std::mutex> g(S->mu);
    auto it = S->jobs.find(id);
    if (it == S->jobs.end()) return rt_internal_error(RT_ERR_INVALID, "rt_job_wait: unknown job");
    Job *J = it->second;
    auto finished = [&] { return J->state == RT_JOB_DONE || J->state == RT_JOB_FAILED; };
    if (timeout_ms < 0) S->cv_done.wait(g, finished);
    else S->cv_done.wait_for(g, std::chrono::milliseconds(timeout_ms), finished);
    return report(S, J, info, film);
}

extern "C" rt_status rt_server_stop(rt_server *S)
{
    if (!S) return RT_OK;
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stopping = true;
    }
    S->cv_work.notify_all();
    for (auto &t : S->threads) t.join();
    if (S->scheduler.joinable()) S->scheduler.join();
    // lanes finish their running jobs; the wavefront stops between steps;
    // queued and resident jobs are dropped
    for (Job *J : S->resident) {
        cudaFree(J->A);
        cudaFree(J->B);
    }
    S->resident.clear();
    for (auto &kv : S->jobs) delete kv.second;
    S->jobs.clear();
    S->set.clear();
    if (S->sched) rt_ctx_destroy(S->sched);
    delete S;
    return RT_OK;
}
