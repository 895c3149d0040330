// rt_kernels.cuh -- wavefront state, kernels and launch helpers shared by
// rt_api.cu.  One batch renders complete reference tiles (block_x x block_y
// pixels, all samples of each pixel), so the film can be reduced per pixel in
// the reference's own summation order without atomics.
#pragma once
#include "rt_device.cuh"

namespace rtgpu {

// path flags
enum { F_FIRST = 1, F_DELTA = 2, F_NEE = 4, F_END = 8, F_DONE = 16 };

#define RT_NBSDF 6        // sorted shading queues (bsdf_queue): types 0-4, then the delta types;
                          // RT_QUEUE_MIXED (rt_device.cuh) is one more: textured BSDFs, and
                          // every BSDF in bounces below the sort threshold

struct RoundCounters {   // one per wavefront round, zeroed per batch
    int closest, shadow, wc_closest, wc_shadow;
    int mat[RT_NBSDF];   // paths to shade per shading queue (material-sorted)
    int fin;             // paths whose traced ray missed or hit a surface without a BSDF
    int end;             // paths that ended in shading with a light sample pending
    int mixed;           // paths to shade, not sorted by material (round below the sort threshold)
    int pad[3];
};

struct Wave {
    // per path slot
    Pcg32 *rng;
    float4 *tp;        // throughput rgb, eta
    float4 *rad;       // radiance rgb, depth (int bits)
    float4 *ray_o;     // origin, mint
    float4 *ray_d;     // direction, maxt
    float4 *hit;       // t, u, v, prim (int bits)
    float4 *bs;        // pending BSDF sample value rgb, pdf
    float *rel_eta;
    int *flags;
    float4 *nee;       // pending light-sample contribution rgb
    float4 *sh_o, *sh_d;
    int *occl;
    float4 *out;       // final radiance rgb, nan flag
    uint8_t *splat;    // film footprint code of the sample
    uint8_t *pix_irregular;  // per batch pixel: some sample splats off its pixel
    // queues of the current round
    int *q_closest, *q_shadow;
    int *q_mat[RT_NBSDF];  // shading queues (bsdf_queue), filled by the closest-hit trace
    int *q_mixed;          // the unsorted shading queue (RT_QUEUE_MIXED)
    int *q_fin;        // rays that missed or hit a surface without a BSDF (to finish)
    int *q_end;        // paths whose BSDF sample was zero, light sample pending
    // ray reordering (optional): per-ray keys, the reordered queue, key counts
    unsigned *sort_keys;
    int *sort_tmp;
    unsigned *sort_hist;
    RoundCounters *cnt;
    int *sid;          // multi-scene batches: scene-table index of the path's job
    int capacity;
    int max_rounds;
    // VolPathTracing wavefront (allocated only for it, vw_capacity paths)
    float4 *v_seg;     // origin of the ray segment that found `hit` (its direction is the path's), medium
    float4 *v_p;       // vertex position (scatter point or surface point), light-selection weight
    float4 *v_li0;     // light sample: direction to the light, distance
    float4 *v_li1;     // light sample: point on the light, pdf
    float4 *v_li2;     // light sample: normal at the point
    float4 *v_val;     // light sample intensity, then the attenuated light-sample value
    int vw_capacity;
};

// One work item of a multi-scene batch (rt_internal_render_multi): whole
// tiles of one job with every sample of their pixels.  The batch's path
// slots are the items' slots one after another; within an item, slot
// path0 + s * npix + q is sample s of the item's pixel q, as in a
// single-scene batch.
struct MultiItem {
    int job;             // scene-table index
    int path0;           // first path slot of the item
    int pix0;            // first batch pixel of the item (film threads, pix_irregular)
    int npix;            // pixels of the item's tiles
    int spp, sample_begin;
    int g0;              // first entry of the item's tiles in its job's tile order
    int width;           // film width of the job
    int accumulate;      // add to the film instead of writing it
    int pad;
    const int4 *tileorder;   // the job's tile-order table
    float4 *film;            // the job's film (device memory)
    uint64_t seed;
};

// batch geometry: tiles [tile0, tile0 + ntiles) of the reference job grid
struct Batch {
    int tile0, ntiles;      // tiles in raster order of the job grid
    int tiles_x;            // job grid width in tiles
    int bx, by;             // block size
    int npix;               // pixels in the batch
    int spp, sample_begin;
    int n_paths;            // npix * spp
    int *pix_of;            // batch pixel -> image pixel (y * W + x)
    int *tile_of;           // batch pixel -> (local x | local y << 16)
};

}  // namespace rtgpu
