// rt_internal.h -- hooks shared by the translation units of librtgpu.
//
// rt_api.cu owns contexts, scenes and kernels; rt_serve.cpp builds batched
// and served rendering on top of the public C ABI and needs a few more
// facts about a context.  Nothing here is exported.
#pragma once
#include <cstddef>

#include "rtgpu.h"

#define RT_HIDDEN __attribute__((visibility("hidden")))

struct rt_lane_pool;   // worker lanes of rt_batch_render, owned by a context

RT_HIDDEN rt_status rt_internal_error(rt_status st, const char *msg);   // sets rt_last_error()
RT_HIDDEN int rt_internal_device(const rt_ctx *c);
RT_HIDDEN int rt_internal_bvh_width(const rt_ctx *c);
RT_HIDDEN int rt_internal_graphs(const rt_ctx *c);
// launch shape and sort threshold of a context's renders (rt_tuning fields)
RT_HIDDEN void rt_internal_get_shape(const rt_ctx *c, int *wave_paths, int *trace_bpsm, int *shade_bpsm,
                                     int *sort_threshold);
RT_HIDDEN rt_status rt_internal_set_shape(rt_ctx *c, int trace_bpsm, int shade_bpsm, int sort_threshold);
RT_HIDDEN int rt_internal_volpath_wave(const rt_ctx *c);
RT_HIDDEN int rt_internal_batch_wave(const rt_ctx *c);
RT_HIDDEN void rt_internal_set_batch_wave(rt_ctx *c, int on);
// a job rt_internal_render_multi can take: PathTracingMIS, one light per
// vertex, the box filter of radius 0.5
RT_HIDDEN bool rt_internal_multi_ok(const rt_scene *sc, const rt_render_desc *rd);
RT_HIDDEN void rt_internal_set_volpath_wave(rt_ctx *c, int on);
RT_HIDDEN void *rt_internal_stream(const rt_ctx *c);
RT_HIDDEN rt_lane_pool *&rt_internal_pool(rt_ctx *c);
RT_HIDDEN void rt_internal_set_stats(rt_ctx *c, const rt_render_stats &s);
RT_HIDDEN void rt_internal_film_size(const rt_scene *sc, int *w, int *h);
// mean over pixels and channels of (a.rgb / a.w - b.rgb / b.w)^2 for two
// device films (pixels with zero weight in either are skipped); with clip,
// each mean is clipped to [0, 1] first; synchronous
RT_HIDDEN rt_status rt_internal_film_sqdiff(rt_ctx *c, const float *a, const float *b, size_t npix, int clip,
                                            double *mean_sq);
// dst += src for two device films, queued on the context's stream
RT_HIDDEN rt_status rt_internal_film_add(rt_ctx *c, float *dst, const float *src, size_t npix);

// many PathTracingMIS jobs in one wavefront (rt_api.cu): films as
// rt_render writes them for each job alone; jobs share max/min depth
RT_HIDDEN rt_status rt_internal_render_multi(rt_ctx *ctx, rt_scene *const *scenes, const rt_render_desc *descs, int n,
                                             float *const *films, int32_t on_device);

RT_HIDDEN void rt_lane_pool_destroy(rt_lane_pool *p);   // rt_serve.cpp
