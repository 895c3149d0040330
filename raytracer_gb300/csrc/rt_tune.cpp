// rt_tune.cpp -- the autotuner (rt_autotune).
//
// It chooses the rt_tuning of a context for a workload by timing
// rt_batch_render on a sample of the workload's jobs.  The search is
// coordinate descent over a fixed grid of candidates: one knob at a time,
// every candidate value tried with the others held at the best so far, a
// candidate kept if it is at least 2% faster and stays so when it and the
// incumbent are measured again, two passes over the knobs or until
// max_trials timed trials.  Every knob leaves the films unchanged (queue
// capacity, grid sizes, the material-sort threshold, lanes, the multi-scene
// wavefront and CUDA graphs), so the choice only trades speed.
//
// The knobs and their candidates:
//   batch_wavefront      1, 0 (jobs in one multi-scene wavefront, or lanes;
//                        samples of more than one job)
//   graphs               0, 1
//   volpath_wavefront    1, 0 (VolPath as a wavefront or one persistent kernel)
//   lanes                1, 2, 4, 8 (samples of 32 jobs or more)
//   sort_threshold       0, 2^12, 2^14, 2^16, 2^18 closest-hit rays
//   shade blocks per SM  4, 8, 16, 24
//   trace blocks per SM  8, 10, 12, 16
//   wave paths           2^20, 2^22, 2^24, 2^26 (a single render's and the
//                        multi-scene wavefront's batch capacity)
//   lane wave paths      2^20, 2^22, 2^24, 2^25 (samples of more than one job)
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "rt_internal.h"

namespace {

double wall_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Knob {
    int32_t rt_tuning::*field;
    std::vector<int32_t> values;
};

}  // namespace

extern "C" rt_status rt_autotune(rt_ctx *ctx, rt_scene *const *scenes, const rt_render_desc *descs, int32_t n,
                                 int32_t max_trials, rt_tuning *best, double *samples_per_s)
{
    if (!ctx || !scenes || !descs || !best || n <= 0 || max_trials < 1)
        return rt_internal_error(RT_ERR_INVALID, "rt_autotune: bad argument");
    for (int i = 0; i < n; i++)
        if (!scenes[i]) return rt_internal_error(RT_ERR_INVALID, "rt_autotune: null scene");
    if (cudaSetDevice(rt_internal_device(ctx)) != cudaSuccess)
        return rt_internal_error(RT_ERR_CUDA, "rt_autotune: cudaSetDevice failed");
    // scratch device films
    std::vector<float *> films(n, nullptr);
    double paths = 0;
    rt_status st = RT_OK;
    for (int i = 0; i < n && st == RT_OK; i++) {
        int w = 0, h = 0;
        rt_internal_film_size(scenes[i], &w, &h);
        paths += (double)w * h * std::max(0, descs[i].spp);
        if (cudaMalloc(&films[i], (size_t)w * h * 4 * sizeof(float)) != cudaSuccess)
            st = rt_internal_error(RT_ERR_NOMEM, "rt_autotune: scratch film allocation failed");
    }
    rt_tuning start;
    if (st == RT_OK) st = rt_ctx_get_tuning(ctx, &start);
    rt_tuning cur = start;
    double cur_s = 0;
    int trials = 0;
    // one trial: set the tuning, one untimed run (allocations, graph builds),
    // then the best of two timed runs
    auto measure = [&](const rt_tuning &t, double &sec) -> rt_status {
        rt_status s = rt_ctx_set_tuning(ctx, &t);
        if (s != RT_OK) return s;
        s = rt_batch_render(ctx, scenes, descs, n, films.data(), 1);
        if (s != RT_OK) return s;
        sec = 1e30;
        for (int r = 0; r < 2; r++) {
            double t0 = wall_s();
            s = rt_batch_render(ctx, scenes, descs, n, films.data(), 1);
            if (s != RT_OK) return s;
            sec = std::min(sec, wall_s() - t0);
        }
        trials++;
        return RT_OK;
    };
    if (st == RT_OK) st = measure(cur, cur_s);
    std::vector<Knob> knobs;
    if (n > 1) knobs.push_back({&rt_tuning::batch_wavefront, {1, 0}});
    knobs.push_back({&rt_tuning::graphs, {0, 1}});
    knobs.push_back({&rt_tuning::volpath_wavefront, {1, 0}});
    // lanes pay off across many jobs: a sample of fewer than 32 cannot show
    // it, and the caller's lane count stays
    if (n >= 32) knobs.push_back({&rt_tuning::lanes, {1, 2, 4, 8}});
    knobs.push_back({&rt_tuning::sort_threshold, {0, 1 << 12, 1 << 14, 1 << 16, 1 << 18}});
    knobs.push_back({&rt_tuning::shade_blocks_per_sm, {4, 8, 16, 24}});
    knobs.push_back({&rt_tuning::trace_blocks_per_sm, {8, 10, 12, 16}});
    if (n > 1) knobs.push_back({&rt_tuning::lane_wave_paths, {1 << 20, 1 << 22, 1 << 24, 1 << 25}});
    knobs.push_back({&rt_tuning::wave_paths, {1 << 20, 1 << 22, 1 << 24, 1 << 26}});
    for (int pass = 0; pass < 2 && st == RT_OK && trials < max_trials; pass++) {
        bool changed = false;
        for (const Knob &k : knobs) {
            for (int32_t v : k.values) {
                if (st != RT_OK || trials >= max_trials) break;
                if (cur.*(k.field) == v) continue;
                rt_tuning t = cur;
                t.*(k.field) = v;
                double s = 0;
                st = measure(t, s);
                if (st == RT_OK && s < cur_s * 0.98) {
                    // confirm against a fresh measurement of both: run-to-run
                    // noise must not move the tuning
                    double s_inc = 0, s_new = 0;
                    st = measure(cur, s_inc);
                    if (st == RT_OK) st = measure(t, s_new);
                    if (st != RT_OK) break;
                    const double inc = std::min(cur_s, s_inc), cand = std::min(s, s_new);
                    if (cand < inc * 0.98) {
                        cur = t;
                        cur_s = cand;
                        changed = true;
                    } else {
                        cur_s = inc;
                    }
                }
            }
        }
        if (!changed) break;
    }
    for (float *f : films) cudaFree(f);
    if (st != RT_OK) {
        rt_ctx_set_tuning(ctx, &start);
        return st;
    }
    st = rt_ctx_set_tuning(ctx, &cur);
    if (st != RT_OK) return st;
    *best = cur;
    if (samples_per_s) *samples_per_s = paths / std::max(cur_s, 1e-12);
    return RT_OK;
}
