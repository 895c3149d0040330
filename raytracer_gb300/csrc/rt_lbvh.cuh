// rt_lbvh.cuh -- the binary tree built on the device (rt_ctx_set_bvh_builder
// RT_BUILDER_DEVICE): a linear BVH over 30-bit Morton codes of the triangle
// centroids (Karras, "Maximizing parallelism in the construction of BVHs,
// octrees, and k-d trees", HPG 2012).  Textually part of rt_api.cu.
//
//   k_lbvh_codes     Morton code of every triangle's centroid in the scene box
//   k_rsort_*        stable least-significant-digit radix sort of the codes,
//                    8 bits per pass (the triangle index rides along; equal
//                    codes keep index order)
//   k_lbvh_nodes     the radix tree: every internal node finds its range and
//                    split from the sorted codes (ties broken by position)
//   k_lbvh_boxes     leaf-to-root box propagation: the second thread to
//                    reach a node computes its box (atomic arrival counter)
//   k_lbvh_slots     the triangle slots in sorted order, as the host build
//                    lays them out (p0 and id, e1, e2)
// k_refit_widen then widens the exact child boxes into the node image.
// Subtrees of at most RT_LBVH_LEAF triangles are linked as one leaf over
// their (contiguous) range.  The tree is built in milliseconds where the
// host SAH build takes about a second for 1.3M triangles, and it is slower
// to traverse.
#pragma once

// Subtrees of at most RT_LBVH_LEAF triangles (<= 8) become one leaf.  On the
// 1.31M-triangle frame, 1 (one triangle per leaf) renders fastest: 94 ms,
// against 96-97 ms for 2, 4 and 8 (fewer node visits, more triangle tests).
#ifndef RT_LBVH_LEAF
#define RT_LBVH_LEAF 1
#endif
#define RT_RSORT_THREADS 256
#define RT_RSORT_ITEMS 8
#define RT_RSORT_TILE (RT_RSORT_THREADS * RT_RSORT_ITEMS)

__device__ __forceinline__ unsigned lbvh_expand10(unsigned v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_lbvh_codes(const float *tri_v, int n, float bx0, float by0, float bz0, float sx, float sy, float sz,
                             unsigned *codes, int *ids)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const float *P = tri_v + 9 * (size_t)t;
        const float c[3] = {(P[0] + P[3] + P[6]) * (1.f / 3.f), (P[1] + P[4] + P[7]) * (1.f / 3.f),
                            (P[2] + P[5] + P[8]) * (1.f / 3.f)};
        const float o[3] = {bx0, by0, bz0}, sc[3] = {sx, sy, sz};
        unsigned q[3];
        for (int a = 0; a < 3; a++) {
            float f = (c[a] - o[a]) * sc[a];
            f = fminf(fmaxf(f, 0.f), 1023.f);   // a NaN centroid lands in cell 0
            q[a] = f == f ? (unsigned)f : 0u;
        }
        codes[t] = (lbvh_expand10(q[0]) << 2) | (lbvh_expand10(q[1]) << 1) | lbvh_expand10(q[2]);
        ids[t] = t;
    }
}

// digit counts of one tile: hist[digit * n_tiles + tile]
__global__ void __launch_bounds__(RT_RSORT_THREADS) k_rsort_hist(const unsigned *keys, int n, int shift, int n_tiles,
                                                                 int *hist)
{
    __shared__ int cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RT_RSORT_TILE;
    for (int j = 0; j < RT_RSORT_ITEMS; j++) {
        const int i = base + j * RT_RSORT_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xffu], 1);
    }
    __syncthreads();
    hist[threadIdx.x * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive scan of the m counts in place (one block of 1024 threads)
__global__ void __launch_bounds__(1024) k_rsort_scan(int *hist, int m)
{
    __shared__ int part[1024];
    const int per = (m + 1023) / 1024;
    const int b = threadIdx.x * per, e = min(m, b + per);
    int sum = 0;
    for (int i = b; i < e; i++) sum += hist[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - sum;
    for (int i = b; i < e; i++) {
        const int c = hist[i];
        hist[i] = run;
        run += c;
    }
}

// stable scatter of one tile: keys in the order (item j, thread) go to their
// digit's next positions
__global__ void __launch_bounds__(RT_RSORT_THREADS) k_rsort_scatter(const unsigned *keys, const int *vals, int n,
                                                                    int shift, int n_tiles, const int *hist,
                                                                    unsigned *keys_out, int *vals_out)
{
    constexpr int W = RT_RSORT_THREADS / 32;
    __shared__ int run[256];
    __shared__ int wcnt[W][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    run[threadIdx.x] = hist[threadIdx.x * n_tiles + blockIdx.x];
    const int base = blockIdx.x * RT_RSORT_TILE;
    for (int j = 0; j < RT_RSORT_ITEMS; j++) {
        for (int w = 0; w < W; w++) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const int i = base + j * RT_RSORT_THREADS + threadIdx.x;
        const bool valid = i < n;
        const unsigned k = valid ? keys[i] : 0u;
        const int d = valid ? (int)((k >> shift) & 0xffu) : 256;   // 256: no digit
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1));
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int pos = run[d] + rank;
            for (int w = 0; w < warp; w++) pos += wcnt[w][d];
            keys_out[pos] = k;
            vals_out[pos] = vals[i];
        }
        __syncthreads();
        int add = 0;
        for (int w = 0; w < W; w++) add += wcnt[w][threadIdx.x];
        run[threadIdx.x] += add;
        __syncthreads();
    }
}

// common prefix length of sorted positions i and j (-1 outside [0, n));
// equal codes are told apart by their positions
__device__ __forceinline__ int lbvh_delta(const unsigned *codes, int n, int i, long long j)
{
    if (j < 0 || j >= n) return -1;
    const unsigned a = codes[i], b = codes[(int)j];
    return a == b ? 32 + __clz((unsigned)i ^ (unsigned)j) : __clz(a ^ b);
}

// internal node i of the n - 1: its children (links in the device node
// layout: an internal index, or a leaf ~(first slot << 3 | count - 1)) and
// the parents of the children (parent * 2 + side)
__global__ void k_lbvh_nodes(const unsigned *codes, int n, float4 *nodes, int *iparent, int *lparent)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        const int d = (lbvh_delta(codes, n, i, (long long)i + 1) - lbvh_delta(codes, n, i, (long long)i - 1)) >= 0 ? 1 : -1;
        const int dmin = lbvh_delta(codes, n, i, (long long)i - d);
        long long lmax = 2;
        while (lbvh_delta(codes, n, i, (long long)i + lmax * d) > dmin) lmax *= 2;
        long long l = 0;
        for (long long t = lmax / 2; t >= 1; t /= 2)
            if (lbvh_delta(codes, n, i, (long long)i + (l + t) * d) > dmin) l += t;
        const long long j = (long long)i + l * d;
        const int dnode = lbvh_delta(codes, n, i, j);
        long long s = 0;
        for (long long div = 2;; div *= 2) {
            const long long t = (l + div - 1) / div;
            if (lbvh_delta(codes, n, i, (long long)i + (s + t) * d) > dnode) s += t;
            if (t <= 1) break;
        }
        const int gamma = (int)((long long)i + s * d + (d < 0 ? -1 : 0));
        const int lo = (int)(j < i ? j : i), hi = (int)(j < i ? i : j);
        int links[2];
        for (int side = 0; side < 2; side++) {
            const int c = gamma + side;
            const bool leaf = side == 0 ? lo == gamma : hi == gamma + 1;
            // the child's range of sorted triangles
            const int start = side == 0 ? lo : gamma + 1, size = side == 0 ? gamma - lo + 1 : hi - gamma;
            if (leaf) {
                links[side] = ~(c << 3);
                lparent[c] = 2 * i + side;
            } else {
                // a subtree of at most RT_LBVH_LEAF triangles becomes one leaf
                // over its range; its nodes still carry the boxes up to here
                links[side] = size <= RT_LBVH_LEAF ? ~((start << 3) | (size - 1)) : c;
                iparent[c] = 2 * i + side;
            }
        }
        reinterpret_cast<int4 *>(nodes)[4 * (size_t)i + 3] = make_int4(links[0], links[1], 0, 0);
    }
}

// boxes from the leaves up: every leaf writes its triangle's box into its
// parent's child slot; the second arrival at a node unites the two and goes on
__global__ void k_lbvh_boxes(const float *tri_v, const int *ids, int n, const int *iparent, const int *lparent,
                             int *arrivals, float *boxes, int *max_depth)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const float *P = tri_v + 9 * (size_t)ids[s];
        float b[6];
        for (int a = 0; a < 3; a++) {
            b[a] = fminf(fminf(P[a], P[3 + a]), P[6 + a]);
            b[3 + a] = fmaxf(fmaxf(P[a], P[3 + a]), P[6 + a]);
        }
        int up = lparent[s], depth = 1;
        for (;;) {
            const int node = up >> 1, side = up & 1;
            float *slot = boxes + 12 * (size_t)node + 6 * side;
            for (int a = 0; a < 6; a++) slot[a] = b[a];
            __threadfence();
            if (atomicAdd(&arrivals[node], 1) == 0) break;   // the sibling is not done yet
            __threadfence();
            const float *o = boxes + 12 * (size_t)node + 6 * (1 - side);
            for (int a = 0; a < 3; a++) {
                b[a] = fminf(b[a], __ldcg(o + a));
                b[3 + a] = fmaxf(b[3 + a], __ldcg(o + 3 + a));
            }
            if (node == 0) break;
            up = iparent[node];
            depth++;
            if (depth > n) break;   // a malformed tree cannot loop forever
        }
        // the leaf's depth (its internal ancestors), for the stack check
        int dd = 0;
        for (int u = lparent[s]; dd <= 64; dd++) {
            const int node = u >> 1;
            if (node == 0) break;
            u = iparent[node];
        }
        atomicMax(max_depth, dd + 1);
    }
}

// triangle slots in sorted order: (p0, id), (p1 - p0), (p2 - p0)
__global__ void k_lbvh_slots(const float *tri_v, const int *ids, int n, float4 *slots)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int id = ids[s];
        const float *P = tri_v + 9 * (size_t)id;
        slots[3 * (size_t)s] = make_float4(P[0], P[1], P[2], __int_as_float(id));
        slots[3 * (size_t)s + 1] = make_float4(P[3] - P[0], P[4] - P[1], P[5] - P[2], 0.f);
        slots[3 * (size_t)s + 2] = make_float4(P[6] - P[0], P[7] - P[1], P[8] - P[2], 0.f);
    }
}
