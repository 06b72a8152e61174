// bh.cu -- Barnes-Hut gravity on the GPU: the astro2 (octree) and astro
// (quadtree) elements, astro/src/transformers.rs:31-69,122-160, over the
// reference's tree semantics (astro/src/octree.rs, astro/src/quadtree.rs).
//
// Pipeline, all on the device (no host round trip, so it can be captured):
//   1. extent    X = max_i max(|x_i|,|y_i|,|z_i|) in f64 (transformers.rs:126-131);
//                the root cell is centred at the origin with half-width X.
//   2. keys      per axis the cell index q at the finest level D, with the
//                reference's octant rule (p > centre goes high, ties low,
//                octree.rs:160-165), interleaved x-lowest into a Morton key:
//                octree 21 levels x 3 bits = 63 bits, quadtree 31 x 2 = 62.
//                Bodies within a rounding margin of a cell boundary re-derive
//                q by replaying the reference's f64 centre arithmetic.
//   3. sort      stable LSD radix sort of (key, body) pairs, 8-bit digits.
//   4. tree      level-by-level, not path-compressed (as the reference's
//                pointer tree): a cell with more than leaf_size bodies that
//                are not all at one key splits into its non-empty children;
//                children are contiguous, levels are contiguous, and node
//                order is deterministic (per-level scans, no atomics).
//                Geometric centres are computed exactly as the reference does
//                (child = parent +- extent/2, octree.rs:167-215).
//   5. moments   mass and centre of mass of every cell from f64 prefix sums
//                over the sorted bodies.
//   6. traversal one warp per 32 consecutive sorted bodies, DFS with a shared
//                stack, the reference's opening rule extent/|x - centre| < theta
//                (octree.rs:137-144).  EXACT: every body keeps its own
//                interaction list (the reference's); WARP: a cell is accepted
//                only if all 32 bodies accept it, and the common list is
//                batched through shared memory.  Pair law in FP32 with one
//                MUFU.RSQ per pair and compensated per-body sums.
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include "common.cuh"
#include "engine.h"
#include "plugin_state.h"

namespace pg {

namespace {

constexpr int kRadixBits = 8;
constexpr int kRadixBuckets = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per block
constexpr int kSortWarps = kSortThreads / 32;

constexpr int kBuildThreads = 256;
constexpr int kMaxLevels = 31;

constexpr int kTravWarps = 4;
constexpr int kStack = 192;
constexpr int kBuf = 128;

// flags[0]: node capacity exceeded (tree truncated; results stay exact)
// flags[1]: traversal stack overflow (results of the affected warp invalid)
constexpr int kFlagNodes = 0;
constexpr int kFlagStack = 1;

struct LevelInfo {
    int32_t begin[kMaxLevels + 2];
    int32_t count[kMaxLevels + 2];
    int32_t total;  // nodes in the tree
};

__host__ __device__ inline int tree_levels(int nchild) { return nchild == 8 ? 21 : 31; }
__host__ __device__ inline int level_bits(int nchild) { return nchild == 8 ? 3 : 2; }

// ---------------------------------------------------------------------------
// 1. extent
// ---------------------------------------------------------------------------
__global__ void extent_kernel(const double *__restrict__ x, const double *__restrict__ y,
                              const double *__restrict__ z, int n,
                              unsigned long long *__restrict__ out_bits)
{
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        m = fmax(m, fabs(x[i]));
        m = fmax(m, fabs(y[i]));
        m = fmax(m, fabs(z[i]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double wm[32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        // non-negative doubles order like their bit patterns
        if (threadIdx.x == 0) atomicMax(out_bits, (unsigned long long)__double_as_longlong(m));
    }
}

// ---------------------------------------------------------------------------
// 2. keys
// ---------------------------------------------------------------------------
// Cell index of coordinate p at the finest level D: the reference descends
// from centre 0 / half-width X deciding `p > centre` at every level.
__device__ __forceinline__ uint32_t axis_cell(double p, double X, double scale, int D,
                                              double margin)
{
    const int lim = (int)((1u << D) - 1u);
    const double u = __dmul_rn(__dadd_rn(p, X), scale);  // (p + X) / (2X) * 2^D
    const double fl = trunc(u);
    const double frac = u - fl;  // exact
    if (!(u == u)) return 0;
    if (frac >= margin && frac <= 1.0 - margin) {
        // u is not within `margin` of a cell boundary: ceil(u) - 1 = floor(u)
        return (uint32_t)min(max((int)fl, 0), lim);
    }
    // Close to a boundary: replay the reference's centre arithmetic.
    double c = 0.0, ext = X;
    uint32_t q = 0;
    for (int d = 0; d < D; ++d) {
        const bool hi = p > c;
        const double h = __ddiv_rn(ext, 2.0);
        c = hi ? __dadd_rn(c, h) : __dsub_rn(c, h);
        ext = h;
        q = (q << 1) | (hi ? 1u : 0u);
    }
    return q;
}

__device__ __forceinline__ uint64_t spread3(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__device__ __forceinline__ uint64_t spread2(uint32_t v)
{
    uint64_t x = v & 0x7fffffffu;
    x = (x | x << 16) & 0x0000ffff0000ffffull;
    x = (x | x << 8) & 0x00ff00ff00ff00ffull;
    x = (x | x << 4) & 0x0f0f0f0f0f0f0f0full;
    x = (x | x << 2) & 0x3333333333333333ull;
    x = (x | x << 1) & 0x5555555555555555ull;
    return x;
}

__global__ void keys_kernel(const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, int n, int nchild,
                            const unsigned long long *__restrict__ extent_bits,
                            uint64_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
    __shared__ double s_scale;
    const double X = __longlong_as_double((long long)*extent_bits);
    const int D = tree_levels(nchild);
    if (threadIdx.x == 0) s_scale = X > 0.0 ? __ddiv_rn(ldexp(1.0, D - 1), X) : 0.0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double scale = s_scale;
    const double margin = ldexp(1.0, D - 40);
    uint64_t key = 0;
    if (X > 0.0) {
        const uint32_t qx = axis_cell(x[i], X, scale, D, margin);
        const uint32_t qy = axis_cell(y[i], X, scale, D, margin);
        if (nchild == 8) {
            const uint32_t qz = axis_cell(z[i], X, scale, D, margin);
            key = spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
        } else {
            key = spread2(qx) | (spread2(qy) << 1);
        }
    }
    keys[i] = key;
    vals[i] = (uint32_t)i;
}

// ---------------------------------------------------------------------------
// 3. radix sort (stable, LSD, 8-bit digits)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__global__ void __launch_bounds__(kSortThreads)
radix_hist_kernel(const uint64_t *__restrict__ keys, int n, int shift, uint32_t *__restrict__ hist,
                  int n_tiles)
{
    __shared__ uint32_t h[kSortWarps][kRadixBuckets];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < kSortWarps * kRadixBuckets; k += kSortThreads)
        (&h[0][0])[k] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile + warp * (kSortItems * 32);
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        const uint32_t d = valid ? (uint32_t)(keys[idx] >> shift) & (kRadixBuckets - 1) : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (valid && (peers & lanemask_lt()) == 0) h[warp][d] += __popc(peers);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixBuckets; d += kSortThreads) {
        uint32_t s = 0;
        for (int w = 0; w < kSortWarps; ++w) s += h[w][d];
        hist[(size_t)d * n_tiles + blockIdx.x] = s;
    }
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums,
                                                         uint32_t &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? warp_sums[lane] : 0;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) warp_sums[lane] = wi - w;
        if (lane == 31) warp_sums[32] = wi;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + incl - v;
    total = warp_sums[32];
    __syncthreads();
    return r;
}

// Per digit (one block each), the exclusive prefix over tiles of that
// digit's counts, in place; the digit's total goes to totals[digit].
__global__ void __launch_bounds__(kSortThreads)
radix_digit_scan_kernel(uint32_t *__restrict__ hist, int n_tiles, uint32_t *__restrict__ totals)
{
    __shared__ uint32_t ws[33];
    uint32_t *row = hist + (size_t)blockIdx.x * n_tiles;
    uint32_t carry = 0;
    for (int t0 = 0; t0 < n_tiles; t0 += blockDim.x) {
        const int t = t0 + threadIdx.x;
        const uint32_t v = t < n_tiles ? row[t] : 0;
        uint32_t total;
        const uint32_t ex = block_exclusive_scan(v, ws, total);
        if (t < n_tiles) row[t] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads)
radix_scatter_kernel(const uint64_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                     uint64_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int n,
                     int shift, const uint32_t *__restrict__ offsets, int n_tiles,
                     const uint32_t *__restrict__ totals)
{
    static_assert(kSortThreads == kRadixBuckets, "one thread per digit");
    __shared__ uint32_t h[kSortWarps][kRadixBuckets];
    __shared__ uint32_t digit_base[kRadixBuckets];
    __shared__ uint32_t ws[33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < kSortWarps * kRadixBuckets; k += kSortThreads)
        (&h[0][0])[k] = 0;
    {
        uint32_t total;
        digit_base[threadIdx.x] = block_exclusive_scan(totals[threadIdx.x], ws, total);
    }
    __syncthreads();
    const int base = blockIdx.x * kSortTile + warp * (kSortItems * 32);
    uint64_t kk[kSortItems];
    uint32_t vv[kSortItems];
    uint32_t rank[kSortItems];
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        kk[r] = valid ? keys_in[idx] : 0;
        vv[r] = valid ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0;
        const uint32_t d = valid ? (uint32_t)(kk[r] >> shift) & (kRadixBuckets - 1) : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = __popc(peers & lanemask_lt());
        uint32_t cur = 0;
        if (valid) cur = h[warp][d];
        __syncwarp();
        if (valid && before == 0) h[warp][d] = cur + __popc(peers);
        __syncwarp();
        rank[r] = cur + before;
    }
    __syncthreads();
    // exclusive prefix over warps, per digit, plus the global offset
    for (int d = threadIdx.x; d < kRadixBuckets; d += kSortThreads) {
        uint32_t run = digit_base[d] + offsets[(size_t)d * n_tiles + blockIdx.x];
        for (int w = 0; w < kSortWarps; ++w) {
            uint32_t c = h[w][d];
            h[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        if (idx >= n) continue;
        const uint32_t d = (uint32_t)(kk[r] >> shift) & (kRadixBuckets - 1);
        const uint32_t pos = h[warp][d] + rank[r];
        keys_out[pos] = kk[r];
        vals_out[pos] = vv[r];
    }
}

// ---------------------------------------------------------------------------
// gather of sorted bodies
// ---------------------------------------------------------------------------
__global__ void gather_kernel(const uint32_t *__restrict__ order, int n,
                              const float4 *__restrict__ body4, const double *__restrict__ x,
                              const double *__restrict__ y, const double *__restrict__ z,
                              const double *__restrict__ m, float4 *__restrict__ sbody,
                              double *__restrict__ spos, double *__restrict__ smass)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t i = order[k];
    sbody[k] = body4[i];
    spos[k] = x[i];
    spos[n + k] = y[i];
    spos[2 * (size_t)n + k] = z[i];
    smass[k] = m[i];
}

// ---------------------------------------------------------------------------
// 4. tree build
// ---------------------------------------------------------------------------
struct NodeArrays {
    int32_t *begin, *count, *child;
    uint8_t *nchild, *level;
    double *c64;   // 4 x cap: cx, cy, cz, extent
    float4 *geo;   // cx, cy, cz, extent (f32)
    float4 *com;   // x, y, z, mass (f32)
    int4 *meta;    // (id | nchild << 28, first child, first body, body count)
    int cap;
};

__global__ void root_kernel(NodeArrays nd, LevelInfo *lv, int n,
                            const unsigned long long *__restrict__ extent_bits)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double X = __longlong_as_double((long long)*extent_bits);
    for (int d = 0; d < kMaxLevels + 2; ++d) {
        lv->begin[d] = 0;
        lv->count[d] = 0;
    }
    lv->total = n > 0 ? 1 : 0;
    lv->count[0] = n > 0 ? 1 : 0;
    lv->begin[1] = 1;
    nd.begin[0] = 0;
    nd.count[0] = n;
    nd.child[0] = -1;
    nd.nchild[0] = 0;
    nd.level[0] = 0;
    nd.c64[0] = 0.0;
    nd.c64[nd.cap] = 0.0;
    nd.c64[2 * (size_t)nd.cap] = 0.0;
    nd.c64[3 * (size_t)nd.cap] = X;
}

// The top levels hold few, large nodes whose child ranges would take long
// binary searches.  For levels <= kTop, child ranges come from a table of
// cell starts at level kTop instead: top[p] = first sorted index whose
// level-kTop prefix is >= p (so empty cells point at the next cell), top[cells] = n.
__host__ __device__ inline int top_levels(int nchild) { return nchild == 8 ? 5 : 7; }

__global__ void top_mark_kernel(const uint64_t *__restrict__ keys, int n, int shift,
                                int32_t *__restrict__ top)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint64_t p = keys[k] >> shift;
    if (k == 0 || (keys[k - 1] >> shift) != p) top[p] = k;
}

// Suffix minimum over the marks (-1 = empty cell) fills empty cells with the
// start of the next non-empty one.  Two passes over blocks of 1024 cells
// (cells is a power of two >= 1024): per-block minima, then per-block
// suffix minima plus the minimum of all later blocks.
__device__ __forceinline__ int32_t mark_value(int32_t v, int n) { return v >= 0 ? v : n; }

__global__ void __launch_bounds__(1024) top_blockmin_kernel(const int32_t *__restrict__ top, int n,
                                                            int32_t *__restrict__ blockmin)
{
    __shared__ int32_t wm[32];
    int32_t m = mark_value(top[blockIdx.x * 1024 + threadIdx.x], n);
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = wm[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) blockmin[blockIdx.x] = m;
    }
}

__global__ void __launch_bounds__(1024) top_fill_kernel(int32_t *__restrict__ top, int cells, int n,
                                                        const int32_t *__restrict__ blockmin)
{
    __shared__ int32_t wm[32];
    __shared__ int32_t later;
    const int nb = cells / 1024;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        int32_t m = n;
        for (int b = (int)blockIdx.x + 1 + lane; b < nb; b += 32) m = min(m, blockmin[b]);
        for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) later = m;
    }
    const int p = blockIdx.x * 1024 + threadIdx.x;
    int32_t v = mark_value(top[p], n);
    // inclusive suffix min within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o < 32) v = min(v, t);
    }
    if (lane == 0) wm[warp] = v;  // minimum of the whole warp
    __syncthreads();
    int32_t r = later;
    for (int w = warp + 1; w < 32; ++w) r = min(r, wm[w]);
    top[p] = min(v, r);
    if (blockIdx.x == 0 && threadIdx.x == 0) top[cells] = n;
}

// Child ranges of a node at `level` covering [b, e): bounds[c] = first sorted
// index in [b, e) whose digit at `shift` is >= c; bounds[nchild] = e.
__device__ __forceinline__ void child_bounds(const uint64_t *__restrict__ keys, int b, int e,
                                             int shift, int nchild, int *bounds,
                                             const int32_t *__restrict__ top, int level, int D,
                                             int bits)
{
    const int K = top_levels(nchild);
    if (level < K) {
        const uint64_t prefix = keys[b] >> (bits * (D - level));
        for (int c = 0; c < nchild; ++c)
            bounds[c] = top[((prefix << bits) | (uint64_t)c) << (bits * (K - level - 1))];
        bounds[0] = b;
        bounds[nchild] = e;
        return;
    }
    const uint32_t mask = nchild - 1;
    bounds[0] = b;
    for (int c = 1; c < nchild; ++c) {
        int lo = bounds[c - 1], hi = e;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (((uint32_t)(keys[mid] >> shift) & mask) < (uint32_t)c)
                lo = mid + 1;
            else
                hi = mid;
        }
        bounds[c] = lo;
    }
    bounds[nchild] = e;
}

__device__ __forceinline__ bool node_splits(const uint64_t *__restrict__ keys, int b, int cnt,
                                            int leaf, int level, int D)
{
    return level < D && cnt > leaf && keys[b] != keys[b + cnt - 1];
}

__device__ int node_child_count(const uint64_t *__restrict__ keys, const NodeArrays &nd, int node,
                                int leaf, int level, int D, int bits, int nchild,
                                const int32_t *__restrict__ top)
{
    const int b = nd.begin[node], cnt = nd.count[node];
    if (!node_splits(keys, b, cnt, leaf, level, D)) return 0;
    int bounds[9];
    child_bounds(keys, b, b + cnt, bits * (D - level - 1), nchild, bounds, top, level, D, bits);
    int k = 0;
    for (int c = 0; c < nchild; ++c) k += bounds[c + 1] > bounds[c];
    return k;
}

// Per-block sums of child counts over the level's nodes (block b takes a
// contiguous chunk).  The last block to finish (atomic ticket after a
// memory fence; nothing waits) turns the block sums into exclusive offsets
// and sizes the next level, leaving it empty (the level's nodes stay
// leaves: exact, slower) if the node arrays would overflow.
__global__ void __launch_bounds__(kBuildThreads)
level_count_kernel(const uint64_t *__restrict__ keys, NodeArrays nd, LevelInfo *lv, int level,
                   int leaf, int nchild, const int32_t *__restrict__ top, int32_t *__restrict__ bsum,
                   unsigned int *__restrict__ ticket, uint32_t *__restrict__ flags)
{
    const int D = tree_levels(nchild), bits = level_bits(nchild);
    const int cnt = lv->count[level], first = lv->begin[level];
    if (cnt == 0) {  // empty level: the tree is complete
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            lv->begin[level + 1] = first;
            lv->count[level + 1] = 0;
        }
        return;
    }
    const int chunk = (cnt + gridDim.x - 1) / gridDim.x;
    const int cb = blockIdx.x * chunk, ce = min(cb + chunk, cnt);
    int s = 0;
    for (int k = cb + threadIdx.x; k < ce; k += blockDim.x)
        s += node_child_count(keys, nd, first + k, leaf, level, D, bits, nchild, top);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ int ws[kBuildThreads / 32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kBuildThreads / 32; ++w) t += ws[w];
        bsum[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x == 0) {
        int32_t run = 0;
        for (int b = 0; b < (int)gridDim.x; ++b) {
            const int32_t v = ((volatile int32_t *)bsum)[b];
            bsum[b] = run;
            run += v;
        }
        const int32_t next_begin = first + cnt;
        const bool fits = (long long)next_begin + run <= (long long)nd.cap;
        lv->begin[level + 1] = next_begin;
        lv->count[level + 1] = fits ? run : 0;
        lv->total = next_begin + (fits ? run : 0);
        if (!fits) atomicOr(&flags[kFlagNodes], 1u);
        *ticket = 0;
    }
}

// Writes the children of the level's nodes at the offsets level_count_kernel
// produced.
__global__ void __launch_bounds__(kBuildThreads)
level_write_kernel(const uint64_t *__restrict__ keys, NodeArrays nd, const LevelInfo *__restrict__ lv,
                   int level, int leaf, int nchild, const int32_t *__restrict__ top,
                   const int32_t *__restrict__ boff)
{
    const int D = tree_levels(nchild), bits = level_bits(nchild);
    const int cnt = lv->count[level], first = lv->begin[level];
    if (cnt == 0 || lv->count[level + 1] == 0) return;
    __shared__ int32_t ws[kBuildThreads / 32];
    __shared__ int32_t carry;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) carry = boff[blockIdx.x];
    __syncthreads();
    const int child_base = lv->begin[level + 1];
    const int chunk = (cnt + gridDim.x - 1) / gridDim.x;
    const int cb = blockIdx.x * chunk, ce = min(cb + chunk, cnt);
    for (int k0 = cb; k0 < ce; k0 += blockDim.x) {
        const int k = k0 + threadIdx.x;
        const int node = first + k;
        int bounds[9];
        int nc = 0;
        bool split = false;
        if (k < ce) {
            const int b = nd.begin[node], c = nd.count[node];
            split = node_splits(keys, b, c, leaf, level, D);
            if (split) {
                child_bounds(keys, b, b + c, bits * (D - level - 1), nchild, bounds, top, level, D,
                             bits);
                for (int q = 0; q < nchild; ++q) nc += bounds[q + 1] > bounds[q];
            }
        }
        // block-wide exclusive scan of nc
        int incl = nc;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        int wbase = 0;
        for (int w = 0; w < warp; ++w) wbase += ws[w];
        const int excl = carry + wbase + incl - nc;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + nc;
        if (k < ce) {
            if (split) {
                const int fc = child_base + excl;
                nd.child[node] = fc;
                nd.nchild[node] = (uint8_t)nc;
                const size_t cap = nd.cap;
                const double pcx = nd.c64[node], pcy = nd.c64[cap + node];
                const double pcz = nd.c64[2 * cap + node], pext = nd.c64[3 * cap + node];
                const double h = __ddiv_rn(pext, 2.0);
                int w = 0;
                for (int q = 0; q < nchild; ++q) {
                    if (bounds[q + 1] <= bounds[q]) continue;
                    const int ci = fc + w++;
                    nd.begin[ci] = bounds[q];
                    nd.count[ci] = bounds[q + 1] - bounds[q];
                    nd.child[ci] = -1;
                    nd.nchild[ci] = 0;
                    nd.level[ci] = (uint8_t)(level + 1);
                    nd.c64[ci] = (q & 1) ? __dadd_rn(pcx, h) : __dsub_rn(pcx, h);
                    nd.c64[cap + ci] = (q & 2) ? __dadd_rn(pcy, h) : __dsub_rn(pcy, h);
                    nd.c64[2 * cap + ci] =
                        nchild == 8 ? ((q & 4) ? __dadd_rn(pcz, h) : __dsub_rn(pcz, h)) : pcz;
                    nd.c64[3 * cap + ci] = h;
                }
            } else {
                nd.child[node] = -1;
                nd.nchild[node] = 0;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// 5. moments: exclusive prefix sums of m, m x, m y, m z over sorted bodies
// ---------------------------------------------------------------------------
constexpr int kMomThreads = 256;

__global__ void __launch_bounds__(kMomThreads)
moment_partial_kernel(const double *__restrict__ spos, const double *__restrict__ smass, int n,
                      double *__restrict__ bsum)
{
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int cb = blockIdx.x * chunk, ce = min(cb + chunk, n);
    double s[4] = {0, 0, 0, 0};
    for (int k = cb + threadIdx.x; k < ce; k += blockDim.x) {
        const double m = smass[k];
        s[0] += m;
        s[1] += m * spos[k];
        s[2] += m * spos[n + k];
        s[3] += m * spos[2 * (size_t)n + k];
    }
    __shared__ double red[4][kMomThreads];
    for (int c = 0; c < 4; ++c) red[c][threadIdx.x] = s[c];
    __syncthreads();
    for (int off = kMomThreads / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int c = 0; c < 4; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x < 4) bsum[threadIdx.x * gridDim.x + blockIdx.x] = red[threadIdx.x][0];
}

// Exclusive scan of the per-block sums, one warp per component.
__global__ void __launch_bounds__(128) moment_blockscan_kernel(double *__restrict__ bsum, int nblocks)
{
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *v = bsum + (size_t)c * nblocks;
    const int per = (nblocks + 31) / 32;
    const int b = lane * per, e = min(b + per, nblocks);
    double s = 0.0;
    for (int k = b; k < e; ++k) s += v[k];
    double incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    double run = incl - s;
    for (int k = b; k < e; ++k) {
        const double t = v[k];
        v[k] = run;
        run += t;
    }
}

constexpr int kMomItems = 4;

// Exclusive prefix sums pref[c][k] of (m, m x, m y, m z) over the sorted
// bodies.  Block b covers a contiguous chunk starting from its block offset;
// each thread takes kMomItems consecutive bodies per tile.
__global__ void __launch_bounds__(kMomThreads)
moment_scan_kernel(const double *__restrict__ spos, const double *__restrict__ smass, int n,
                   const double *__restrict__ boff, double *__restrict__ pref)
{
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int cb = blockIdx.x * chunk, ce = min(cb + chunk, n);
    const size_t stride = (size_t)n + 1;
    __shared__ double carry[4];
    __shared__ double ws[4][kMomThreads / 32];
    if (threadIdx.x < 4) carry[threadIdx.x] = boff[threadIdx.x * gridDim.x + blockIdx.x];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kTile = kMomThreads * kMomItems;
    for (int t0 = cb; t0 < ce; t0 += kTile) {
        const int k0 = t0 + threadIdx.x * kMomItems;
        double v[kMomItems][4];
        double tot[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int j = 0; j < kMomItems; ++j) {
            const int k = k0 + j;
            double m = 0.0, px = 0.0, py = 0.0, pz = 0.0;
            if (k < ce) {
                m = smass[k];
                px = spos[k];
                py = spos[n + k];
                pz = spos[2 * (size_t)n + k];
            }
            v[j][0] = m;
            v[j][1] = m * px;
            v[j][2] = m * py;
            v[j][3] = m * pz;
#pragma unroll
            for (int c = 0; c < 4; ++c) tot[c] += v[j][c];
        }
        double incl[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            incl[c] = tot[c];
            for (int o = 1; o < 32; o <<= 1) {
                const double t = __shfl_up_sync(0xffffffffu, incl[c], o);
                if (lane >= o) incl[c] += t;
            }
            if (lane == 31) ws[c][warp] = incl[c];
        }
        __syncthreads();
        double run[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double wb = 0.0;
            for (int w = 0; w < warp; ++w) wb += ws[c][w];
            run[c] = carry[c] + wb + incl[c] - tot[c];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kMomItems; ++j) {
            const int k = k0 + j;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (k < ce) pref[c * stride + k] = run[c];
                run[c] += v[j][c];
            }
        }
        if (threadIdx.x == kMomThreads - 1)
#pragma unroll
            for (int c = 0; c < 4; ++c) carry[c] = run[c];
        __syncthreads();
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
        for (int c = 0; c < 4; ++c) pref[c * stride + n] = carry[c];
}

__global__ void node_finish_kernel(NodeArrays nd, const LevelInfo *__restrict__ lv,
                                   const double *__restrict__ pref, int n,
                                   const float4 *__restrict__ sbody, const double *__restrict__ spos)
{
    const int total = lv->total;
    const size_t stride = (size_t)n + 1;
    const size_t cap = nd.cap;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int b = nd.begin[i], e = b + nd.count[i];
        nd.geo[i] = make_float4((float)nd.c64[i], (float)nd.c64[cap + i], (float)nd.c64[2 * cap + i],
                                (float)nd.c64[3 * cap + i]);
        float4 com;
        const bool same_pos = spos[b] == spos[e - 1] && spos[n + b] == spos[n + e - 1] &&
                              spos[2 * (size_t)n + b] == spos[2 * (size_t)n + e - 1];
        const double M = pref[e] - pref[b];
        if (e - b == 1) {
            // a single body: the body itself, so it cancels against itself in
            // the pair law as the reference's equal-centre skip does
            com = sbody[b];
        } else if (same_pos) {
            com = sbody[b];
            com.w = (float)M;
        } else if (M != 0.0) {
            com = make_float4((float)((pref[stride + e] - pref[stride + b]) / M),
                              (float)((pref[2 * stride + e] - pref[2 * stride + b]) / M),
                              (float)((pref[3 * stride + e] - pref[3 * stride + b]) / M), (float)M);
        } else {
            com = make_float4((float)nd.c64[i], (float)nd.c64[cap + i], (float)nd.c64[2 * cap + i],
                              0.f);
        }
        nd.com[i] = com;
        nd.meta[i] = make_int4(i | ((int)nd.nchild[i] << 28), nd.child[i], b, e - b);
    }
}

// ---------------------------------------------------------------------------
// 6. traversal
// ---------------------------------------------------------------------------
struct TravArgs {
    NodeArrays nd;
    const float4 *sbody;
    const double *spos;
    const uint32_t *order;
    const LevelInfo *lv;
    int n;
    float theta, e;
    double theta64;
    float extent;  // root half-width X (set on the device before the traversal)
    uint32_t *flags;
    double *partial;
    const unsigned long long *extent_bits;
    unsigned long long *stats;  // [0] node visits, [1] pair interactions (lanes)
};

__device__ __forceinline__ float load_extent(const TravArgs &a)
{
    return (float)__longlong_as_double((long long)*a.extent_bits);
}

// The reference's opening rule `extent / r < theta` (octree.rs:137-144):
// FP32, re-evaluated in f64 with the reference's arithmetic near the edge.
__device__ __forceinline__ bool accept_cell(const TravArgs &a, int node, float4 geo, float qx,
                                            float qy, float qz, int k)
{
    const float dx = qx - geo.x, dy = qy - geo.y, dz = qz - geo.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float inv = rsqrt_approx(r2);
    const float ratio = geo.w * inv;
    // Bound on the relative error of `ratio` against the reference's f64
    // value: rounding positions and centres (|.| <= X) to f32 perturbs each
    // difference by <= 3 * 2^-24 * X, i.e. r by <= 3.1e-7 X; rsqrt.approx and
    // the f32 extent add ~3e-7.  Decisions inside twice that band are redone
    // in f64 with the reference's operations.
    const float band = fabsf(a.theta) * (6.4e-7f * a.extent * inv + 1e-6f) + 1e-30f;
    if (fabsf(ratio - a.theta) > band && ratio == ratio && r2 > 1e-30f)
        return ratio < a.theta;
    const size_t cap = a.nd.cap;
    const double d0 = a.spos[k] - a.nd.c64[node];
    const double d1 = a.spos[a.n + k] - a.nd.c64[cap + node];
    const double d2 = a.spos[2 * (size_t)a.n + k] - a.nd.c64[2 * cap + node];
    const double r64 = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    return a.nd.c64[3 * cap + node] / r64 < a.theta64;
}

__device__ __forceinline__ void pair_acc(float qx, float qy, float qz, float4 b, float e,
                                         float &ax, float &ay, float &az)
{
    const float dx = b.x - qx, dy = b.y - qy, dz = b.z - qz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float w = r2 + e;
    const float q = fmaf(r2, w * w, kPairGuard);
    const float s = b.w * rsqrt_approx(q);
    ax = fmaf(dx, s, ax);
    ay = fmaf(dy, s, ay);
    az = fmaf(dz, s, az);
}

__device__ __forceinline__ void fold(float &hi, float &lo, float &t)
{
    float s, err;
    two_sum(hi, t, s, err);
    hi = s;
    lo += err;
    t = 0.f;
}

struct StackEntry {
    int32_t node;
    uint32_t mask;
};

__global__ void __launch_bounds__(kTravWarps * 32)
traverse_exact_kernel(TravArgs a_in)
{
    __shared__ StackEntry stack[kTravWarps][kStack];
    TravArgs a = a_in;
    a.extent = load_extent(a_in);
    unsigned long long visits = 0, pairs = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k0 = (blockIdx.x * kTravWarps + warp) * 32;
    if (k0 >= a.n) return;
    const int k = k0 + lane;
    const bool valid = k < a.n;
    const uint32_t active = __ballot_sync(0xffffffffu, valid);
    const float4 q = valid ? a.sbody[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    float ax = 0.f, ay = 0.f, az = 0.f, hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
    int sp = 0;
    if (lane == 0) stack[warp][0] = {0, active};
    sp = 1;
    int since_fold = 0;
    __syncwarp();
    while (sp > 0) {
        const StackEntry top = stack[warp][sp - 1];
        --sp;
        __syncwarp();
        const int node = top.node;
        const bool in = (top.mask >> lane) & 1u;
        const float4 geo = a.nd.geo[node];
        const int child = a.nd.child[node];
        bool acc = false;
        if (in) acc = accept_cell(a, node, geo, q.x, q.y, q.z, k);
        const uint32_t open = top.mask & ~__ballot_sync(0xffffffffu, acc);
        ++visits;
        if (acc) {
            pair_acc(q.x, q.y, q.z, a.nd.com[node], a.e, ax, ay, az);
            ++pairs;
        }
        ++since_fold;
        if (child < 0) {
            if (open) {
                const int b = a.nd.begin[node], c = a.nd.count[node];
                const bool mine = (open >> lane) & 1u;
                for (int j = b; j < b + c; ++j) {
                    const float4 bj = a.sbody[j];
                    if (mine) pair_acc(q.x, q.y, q.z, bj, a.e, ax, ay, az);
                }
                if (mine) pairs += c;
                since_fold += c;
            }
        } else if (open) {
            const int nc = a.nd.nchild[node];
            if (sp + nc > kStack) {
                if (lane == 0) atomicOr(&a.flags[kFlagStack], 1u);
                break;
            }
            // push children 0..nc-1 so the last child is popped first, the
            // reference's pop order (octree.rs:152-154)
            if (lane < nc) stack[warp][sp + lane] = {child + lane, open};
            sp += nc;
            __syncwarp();
        }
        if (since_fold >= 64) {
            fold(hx, lx, ax);
            fold(hy, ly, ay);
            fold(hz, lz, az);
            since_fold = 0;
        }
    }
    fold(hx, lx, ax);
    fold(hy, ly, ay);
    fold(hz, lz, az);
    for (int o = 16; o > 0; o >>= 1) pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    if (lane == 0) {
        atomicAdd(&a.stats[0], visits);
        atomicAdd(&a.stats[1], pairs);
    }
    if (valid) {
        const uint32_t i = a.order[k];
        a.partial[i] = (double)hx + (double)lx;
        a.partial[a.n + i] = (double)hy + (double)ly;
        a.partial[2 * (size_t)a.n + i] = (double)hz + (double)lz;
    }
}

// Warp traversal: the 32 bodies of a warp (consecutive in Morton order) walk
// the tree together, and the lanes work on different cells.  Each iteration
// takes up to 32 pending cells from the top of a shared stack, one per lane,
// and tests each against the warp's bounding box: a cell is accepted when
//     extent * (1 + 2e-6) < theta * (r_min - 6e-7 X),
// r_min = distance from the cell centre to the box.  Every body of the warp
// is at least r_min (less f32 rounding of positions and centres, <= 2.1e-7 X)
// from the centre, so an accepted cell passes every body's own f64 reference
// test extent / r < theta; cells that some body would open are opened.
// Accepted cells and the bodies of opened leaves are queued (>= 0 body,
// < 0 cell) and gathered 32 at a time into shared memory, where all lanes
// evaluate them against their own body.
constexpr int kGStack = 1024;                 // pending cells per warp
constexpr int kGWide = kGStack - 256 - 8 * 22;  // above this, pop one cell at a time
constexpr int kGQueue = 640;                  // queued interactions per warp

__device__ __forceinline__ int warp_exclusive_scan(int v, int lane, int &total)
{
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

__global__ void __launch_bounds__(kTravWarps * 32)
traverse_warp_kernel(TravArgs a_in)
{
    __shared__ int32_t gstack[kTravWarps][kGStack];
    __shared__ int32_t queue[kTravWarps][kGQueue];
    __shared__ float4 tile[kTravWarps][32];
    TravArgs a = a_in;
    a.extent = load_extent(a_in);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k0 = (blockIdx.x * kTravWarps + warp) * 32;
    if (k0 >= a.n) return;
    const int k = k0 + lane;
    const bool valid = k < a.n;
    const int nvalid = __popc(__ballot_sync(0xffffffffu, valid));
    const float4 q = valid ? a.sbody[k] : a.sbody[k0];
    float lo_x = q.x, hi_x = q.x, lo_y = q.y, hi_y = q.y, lo_z = q.z, hi_z = q.z;
    for (int o = 16; o > 0; o >>= 1) {
        lo_x = fminf(lo_x, __shfl_xor_sync(0xffffffffu, lo_x, o));
        hi_x = fmaxf(hi_x, __shfl_xor_sync(0xffffffffu, hi_x, o));
        lo_y = fminf(lo_y, __shfl_xor_sync(0xffffffffu, lo_y, o));
        hi_y = fmaxf(hi_y, __shfl_xor_sync(0xffffffffu, hi_y, o));
        lo_z = fminf(lo_z, __shfl_xor_sync(0xffffffffu, lo_z, o));
        hi_z = fmaxf(hi_z, __shfl_xor_sync(0xffffffffu, hi_z, o));
    }
    // largest coordinate magnitude in the box: bounds the f32 rounding of the
    // warp's positions
    const float bmax = fmaxf(fmaxf(fmaxf(fabsf(lo_x), fabsf(hi_x)), fmaxf(fabsf(lo_y), fabsf(hi_y))),
                             fmaxf(fabsf(lo_z), fabsf(hi_z)));
    const float pmax = fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fabsf(q.z));
    const float theta = a.theta;
    float ax = 0.f, ay = 0.f, az = 0.f, hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
    unsigned long long visits = 0, pairs = 0;
    int nq = 0;
    int sp = 1;
    if (lane == 0) gstack[warp][0] = 0;
    __syncwarp();
    auto flush = [&]() {
        for (int j0 = 0; j0 < nq; j0 += 32) {
            const int m = min(32, nq - j0);
            __syncwarp();
            if (lane < m) {
                const int r = queue[warp][j0 + lane];
                tile[warp][lane] = r >= 0 ? a.sbody[r] : a.nd.com[-r - 1];
            }
            __syncwarp();
            for (int j = 0; j < m; ++j) pair_acc(q.x, q.y, q.z, tile[warp][j], a.e, ax, ay, az);
        }
        pairs += nq;
        fold(hx, lx, ax);
        fold(hy, ly, ay);
        fold(hz, lz, az);
        nq = 0;
        __syncwarp();
    };
    bool overflow = false;
    while (sp > 0) {
        const int m = sp > kGWide ? 1 : min(32, sp);
        int cell = 0;
        if (lane < m) cell = gstack[warp][sp - m + lane];
        __syncwarp();
        sp -= m;
        visits += m;
        int qref = 0, qcnt = 0, nchild = 0, first_child = 0;
        float4 geo = make_float4(0.f, 0.f, 0.f, 0.f);
        bool acc = false, maybe = false;
        if (lane < m) {
            geo = a.nd.geo[cell];
            const int4 meta = a.nd.meta[cell];
            const float cmax = fmaxf(fmaxf(fabsf(geo.x), fabsf(geo.y)), fabsf(geo.z));
            const float dx = fmaxf(fmaxf(lo_x - geo.x, geo.x - hi_x), 0.f);
            const float dy = fmaxf(fmaxf(lo_y - geo.y, geo.y - hi_y), 0.f);
            const float dz = fmaxf(fmaxf(lo_z - geo.z, geo.z - hi_z), 0.f);
            const float r = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
            // f32 rounding of positions and centre moves r by at most
            // 1.1e-7 (|p| + |c|) + 3.5e-7 r against the reference's f64 value
            const float rmin = r - (2e-7f * (bmax + cmax) + 5e-7f * r);
            acc = theta > 0.f && rmin > 0.f && geo.w * (1.f + 2e-6f) < theta * rmin;
            if (acc) {
                qref = -cell - 1;
                qcnt = 1;
            } else if (meta.y < 0) {
                qref = meta.z;  // first body of the leaf
                qcnt = meta.w;
            } else {
                nchild = (int)((uint32_t)meta.x >> 28);
                first_child = meta.y;
                maybe = theta > 0.f;
            }
        }
        // Internal cells the box test rejects: accept them if every body of
        // the warp passes its own test (with the same rounding margin).
        uint32_t pend = __ballot_sync(0xffffffffu, maybe);
        while (pend) {
            const int src = __ffs(pend) - 1;
            pend &= pend - 1;
            const float gx = __shfl_sync(0xffffffffu, geo.x, src);
            const float gy = __shfl_sync(0xffffffffu, geo.y, src);
            const float gz = __shfl_sync(0xffffffffu, geo.z, src);
            const float gw = __shfl_sync(0xffffffffu, geo.w, src);
            const float ddx = q.x - gx, ddy = q.y - gy, ddz = q.z - gz;
            const float r2 = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz));
            const float r = r2 * rsqrt_approx(r2);
            const float cm = fmaxf(fmaxf(fabsf(gx), fabsf(gy)), fabsf(gz));
            const float rl = r - (2e-7f * (pmax + cm) + 5e-7f * r);
            const bool ok = !valid || (rl > 0.f && gw * (1.f + 2e-6f) < theta * rl);
            if (__all_sync(0xffffffffu, ok) && lane == src) {
                qref = -cell - 1;
                qcnt = 1;
                nchild = 0;
            }
        }
        // push the children of opened cells
        int ctotal;
        const int coff = warp_exclusive_scan(nchild, lane, ctotal);
        if (sp + ctotal > kGStack) {
            overflow = true;
            break;
        }
        for (int c = 0; c < nchild; ++c) gstack[warp][sp + coff + c] = first_child + c;
        sp += ctotal;
        // queue cells and leaf bodies, at most 16 entries per lane per round
        while (__any_sync(0xffffffffu, qcnt > 0)) {
            const int take = min(qcnt, 16);
            int qtotal;
            const int qoff = warp_exclusive_scan(take, lane, qtotal);
            if (nq + qtotal > kGQueue) flush();
            if (qref < 0) {
                if (take) queue[warp][nq + qoff] = qref;
            } else {
                for (int j = 0; j < take; ++j) queue[warp][nq + qoff + j] = qref + j;
                qref += take;
            }
            qcnt -= take;
            nq += qtotal;
        }
        __syncwarp();
        if (nq >= 256) flush();
    }
    flush();
    if (lane == 0) {
        if (overflow) atomicOr(&a.flags[kFlagStack], 1u);
        atomicAdd(&a.stats[0], visits);
        atomicAdd(&a.stats[1], pairs * (unsigned long long)nvalid);
    }
    if (valid) {
        const uint32_t i = a.order[k];
        a.partial[i] = (double)hx + (double)lx;
        a.partial[a.n + i] = (double)hy + (double)ly;
        a.partial[2 * (size_t)a.n + i] = (double)hz + (double)lz;
    }
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
// workspace + host driver
// ---------------------------------------------------------------------------
struct BhWorkspace {
    int device = 0;
    size_t cap_n = 0;
    int grid_build = 0;  // blocks of the per-level build kernels
    int grid_mom = 0;
    uint64_t *keys[2] = {nullptr, nullptr};
    uint32_t *vals[2] = {nullptr, nullptr};
    uint32_t *hist = nullptr;
    uint32_t *digit_totals = nullptr;
    float4 *sbody = nullptr;
    double *spos = nullptr, *smass = nullptr, *pref = nullptr, *mom_bsum = nullptr;
    NodeArrays nd = {};
    LevelInfo *lv = nullptr;
    int32_t *bsum = nullptr;
    unsigned long long *extent_bits = nullptr;
    unsigned long long *stats = nullptr;  // node visits, pair interactions of the last traversal
    unsigned int *ticket = nullptr;       // last-block ticket of level_count_kernel (kept at 0)
    int32_t *top = nullptr;               // cell starts of the top tree level (see top_levels)
    int32_t *top_blockmin = nullptr;      // per-1024-cell minima while filling `top`
    uint32_t *flags = nullptr;
    int launches = 0;
    // which key/val buffer holds the sorted result
    int sorted = 0;
    int leaf_min = 1;  // smallest leaf size the node capacity was sized for
    // optional events around the traversal kernel (recorded into graphs too)
    bool profiling = false;
    cudaEvent_t trav_ev[2] = {nullptr, nullptr};
};

static void ws_release(BhWorkspace *ws)
{
    void *p[] = {ws->keys[0],  ws->keys[1],   ws->vals[0],       ws->vals[1],     ws->hist,
                 ws->digit_totals,
                 ws->sbody,    ws->spos,      ws->smass,         ws->pref,        ws->mom_bsum,
                 ws->nd.begin, ws->nd.count,  ws->nd.child,      ws->nd.nchild,   ws->nd.level,
                 ws->nd.c64,   ws->nd.geo,    ws->nd.com,        ws->lv,          ws->bsum,
                 ws->extent_bits, ws->flags, ws->nd.meta, ws->stats, ws->ticket,
                 ws->top, ws->top_blockmin};
    for (void *q : p)
        if (q) cudaFree(q);
}

template <typename T>
static int wsalloc(T *&p, size_t count)
{
    PG_CUDA(cudaMalloc((void **)&p, (count ? count : 1) * sizeof(T)));
    return PHYSIM_OK;
}

int bh_reserve(BhWorkspace *&ws, size_t n, int device, int leaf)
{
    leaf = leaf < 1 ? 1 : leaf;
    if (ws && n <= ws->cap_n && leaf >= ws->leaf_min) return PHYSIM_OK;
    if (ws) {
        ws_release(ws);
        delete ws;
        ws = nullptr;
    }
    BhWorkspace *w = new (std::nothrow) BhWorkspace();
    PG_CHECK(w, PHYSIM_ERR_MEMORY, "out of host memory");
    w->device = device;
    const size_t cap = n < 64 ? 64 : n;
    w->cap_n = cap;
    const int sms = device_sm_count(device);
    w->grid_build = sms * 2;
    w->grid_mom = sms * 2;
    const int tiles = cdiv((long long)cap, kSortTile);
    // Node capacity: leaves hold about leaf/4 bodies on average, so 8N/leaf
    // (at most 4N) nodes hold every non-degenerate distribution; deeper
    // chains only leave levels unsplit (exact, slower) and raise a flag.
    const size_t ncap = std::min<size_t>(4 * cap, 8 * cap / (size_t)leaf) + 4096 + 64 * kMaxLevels;
    w->leaf_min = leaf;
    int rc = PHYSIM_OK;
#define PG_WA(ptr, cnt)                                                                     \
    if (rc == PHYSIM_OK) rc = wsalloc(ptr, cnt)
    PG_WA(w->keys[0], cap);
    PG_WA(w->keys[1], cap);
    PG_WA(w->vals[0], cap);
    PG_WA(w->vals[1], cap);
    PG_WA(w->hist, (size_t)kRadixBuckets * tiles);
    PG_WA(w->digit_totals, kRadixBuckets);
    PG_WA(w->sbody, cap);
    PG_WA(w->spos, 3 * cap);
    PG_WA(w->smass, cap);
    PG_WA(w->pref, 4 * (cap + 1));
    PG_WA(w->mom_bsum, 4 * (size_t)w->grid_mom);
    PG_WA(w->nd.begin, ncap);
    PG_WA(w->nd.count, ncap);
    PG_WA(w->nd.child, ncap);
    PG_WA(w->nd.nchild, ncap);
    PG_WA(w->nd.level, ncap);
    PG_WA(w->nd.c64, 4 * ncap);
    PG_WA(w->nd.geo, ncap);
    PG_WA(w->nd.com, ncap);
    PG_WA(w->nd.meta, ncap);
    PG_WA(w->stats, 4);
    PG_WA(w->ticket, 1);
    PG_WA(w->top, (size_t)(1 << 15) + 1);
    PG_WA(w->top_blockmin, 32);
    PG_WA(w->lv, 1);
    PG_WA(w->bsum, (size_t)w->grid_build);
    PG_WA(w->extent_bits, 1);
    PG_WA(w->flags, 4);
#undef PG_WA
    w->nd.cap = (int)ncap;
    if (rc == PHYSIM_OK && (cudaMemset(w->flags, 0, 4 * sizeof(uint32_t)) != cudaSuccess ||
                            cudaMemset(w->ticket, 0, sizeof(unsigned int)) != cudaSuccess))
        rc = PHYSIM_ERR_CUDA;
    if (rc != PHYSIM_OK) {
        ws_release(w);
        delete w;
        return rc;
    }
    ws = w;
    return PHYSIM_OK;
}

void bh_free(BhWorkspace *ws)
{
    if (!ws) return;
    for (cudaEvent_t e : ws->trav_ev)
        if (e) cudaEventDestroy(e);
    ws_release(ws);
    delete ws;
}

int bh_set_profiling(BhWorkspace *ws, bool enable)
{
    PG_CHECK(ws, PHYSIM_ERR_ARGUMENT, "null workspace");
    if (enable && !ws->trav_ev[0])
        for (cudaEvent_t &e : ws->trav_ev) PG_CUDA(cudaEventCreate(&e));
    ws->profiling = enable;
    return PHYSIM_OK;
}

int bh_traversal_ms(BhWorkspace *ws, double *ms)
{
    PG_CHECK(ws && ms && ws->profiling, PHYSIM_ERR_ARGUMENT, "profiling is off");
    PG_CUDA(cudaEventSynchronize(ws->trav_ev[1]));
    float t = 0.f;
    PG_CUDA(cudaEventElapsedTime(&t, ws->trav_ev[0], ws->trav_ev[1]));
    *ms = t;
    return PHYSIM_OK;
}

int bh_launches(const BhWorkspace *ws) { return ws ? ws->launches : 0; }

int bh_stats(BhWorkspace *ws, cudaStream_t st, uint64_t out[2])
{
    PG_CHECK(ws && out, PHYSIM_ERR_ARGUMENT, "null argument");
    unsigned long long h[2] = {0, 0};
    PG_CUDA(cudaMemcpyAsync(h, ws->stats, sizeof h, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    out[0] = h[0];
    out[1] = h[1];
    return PHYSIM_OK;
}

static int bh_build(BhWorkspace *ws, const DeviceBodies &b, const BhParams &p, cudaStream_t st)
{
    const int n = (int)b.n;
    int launches = 0;
    PG_CUDA(cudaMemsetAsync(ws->extent_bits, 0, sizeof(unsigned long long), st));
    const int sms = device_sm_count(ws->device);
    extent_kernel<<<sms * 2, 256, 0, st>>>(b.x, b.y, b.z, n, ws->extent_bits);
    keys_kernel<<<cdiv(n, 256), 256, 0, st>>>(b.x, b.y, b.z, n, p.nchild, ws->extent_bits,
                                              ws->keys[0], ws->vals[0]);
    launches += 2;
    // radix sort
    const int tiles = cdiv(n, kSortTile);
    const int key_bits = tree_levels(p.nchild) * level_bits(p.nchild);
    int cur = 0;
    for (int shift = 0; shift < key_bits; shift += kRadixBits) {
        radix_hist_kernel<<<tiles, kSortThreads, 0, st>>>(ws->keys[cur], n, shift, ws->hist, tiles);
        radix_digit_scan_kernel<<<kRadixBuckets, kSortThreads, 0, st>>>(ws->hist, tiles,
                                                                        ws->digit_totals);
        radix_scatter_kernel<<<tiles, kSortThreads, 0, st>>>(
            ws->keys[cur], shift == 0 ? nullptr : ws->vals[cur], ws->keys[cur ^ 1],
            ws->vals[cur ^ 1], n, shift, ws->hist, tiles, ws->digit_totals);
        cur ^= 1;
        launches += 3;
    }
    ws->sorted = cur;
    gather_kernel<<<cdiv(n, 256), 256, 0, st>>>(ws->vals[cur], n, b.body4, b.x, b.y, b.z, b.m,
                                                ws->sbody, ws->spos, ws->smass);
    root_kernel<<<1, 32, 0, st>>>(ws->nd, ws->lv, n, ws->extent_bits);
    launches += 2;
    const int D = tree_levels(p.nchild);
    const int K = top_levels(p.nchild);
    const int top_cells = 1 << (level_bits(p.nchild) * K);
    PG_CUDA(cudaMemsetAsync(ws->top, 0xff, top_cells * sizeof(int32_t), st));
    top_mark_kernel<<<cdiv(n, 256), 256, 0, st>>>(ws->keys[cur], n, level_bits(p.nchild) * (D - K),
                                                  ws->top);
    top_blockmin_kernel<<<top_cells / 1024, 1024, 0, st>>>(ws->top, n, ws->top_blockmin);
    top_fill_kernel<<<top_cells / 1024, 1024, 0, st>>>(ws->top, top_cells, n, ws->top_blockmin);
    launches += 3;
    for (int level = 0; level < D; ++level) {
        level_count_kernel<<<ws->grid_build, kBuildThreads, 0, st>>>(
            ws->keys[cur], ws->nd, ws->lv, level, p.leaf_size, p.nchild, ws->top, ws->bsum,
            ws->ticket, ws->flags);
        level_write_kernel<<<ws->grid_build, kBuildThreads, 0, st>>>(
            ws->keys[cur], ws->nd, ws->lv, level, p.leaf_size, p.nchild, ws->top, ws->bsum);
        launches += 2;
    }
    moment_partial_kernel<<<ws->grid_mom, kMomThreads, 0, st>>>(ws->spos, ws->smass, n,
                                                                ws->mom_bsum);
    moment_blockscan_kernel<<<1, 128, 0, st>>>(ws->mom_bsum, ws->grid_mom);
    moment_scan_kernel<<<ws->grid_mom, kMomThreads, 0, st>>>(ws->spos, ws->smass, n, ws->mom_bsum,
                                                             ws->pref);
    node_finish_kernel<<<sms * 4, 256, 0, st>>>(ws->nd, ws->lv, ws->pref, n, ws->sbody, ws->spos);
    launches += 4;
    PG_CUDA(cudaGetLastError());
    ws->launches = launches;
    return PHYSIM_OK;
}

int bh_accelerations(BhWorkspace *ws, const DeviceBodies &b, const BhParams &p, double *partial,
                     cudaStream_t st)
{
    PG_CHECK(ws && b.x, PHYSIM_ERR_ARGUMENT, "Barnes-Hut needs the f64 body state");
    PG_CHECK(p.nchild == 8 || p.nchild == 4, PHYSIM_ERR_ARGUMENT, "nchild must be 8 or 4");
    PG_CHECK(b.n <= ws->cap_n, PHYSIM_ERR_ARGUMENT, "workspace too small");
    const int n = (int)b.n;
    if (n == 0) return PHYSIM_OK;
    PG_TRY(bh_build(ws, b, p, st));
    TravArgs a;
    a.nd = ws->nd;
    a.sbody = ws->sbody;
    a.spos = ws->spos;
    a.order = ws->vals[ws->sorted];
    a.lv = ws->lv;
    a.n = n;
    a.theta = (float)p.theta;
    a.theta64 = p.theta;
    a.e = (float)p.e;
    a.flags = ws->flags;
    a.partial = partial;
    a.extent = 0.f;  // read on the device from extent_bits
    a.extent_bits = ws->extent_bits;
    a.stats = ws->stats;
    PG_CUDA(cudaMemsetAsync(ws->stats, 0, 2 * sizeof(unsigned long long), st));
    const int blocks = cdiv(cdiv(n, 32), kTravWarps);
    // external records, so they also time the kernel when replayed from a graph
    if (ws->profiling)
        PG_CUDA(cudaEventRecordWithFlags(ws->trav_ev[0], st, cudaEventRecordExternal));
    if (p.traversal == PHYSIM_TRAVERSAL_WARP)
        traverse_warp_kernel<<<blocks, kTravWarps * 32, 0, st>>>(a);
    else
        traverse_exact_kernel<<<blocks, kTravWarps * 32, 0, st>>>(a);
    PG_CUDA(cudaGetLastError());
    if (ws->profiling)
        PG_CUDA(cudaEventRecordWithFlags(ws->trav_ev[1], st, cudaEventRecordExternal));
    ws->launches += 1;
    return PHYSIM_OK;
}

// Copies the tree of the last build to host arrays (tests / diagnostics).
int bh_snapshot(BhWorkspace *ws, size_t n, cudaStream_t st, PhysimTreeSnapshot *out)
{
    PG_CHECK(ws && out, PHYSIM_ERR_ARGUMENT, "null argument");
    LevelInfo lv;
    uint32_t flags[4];
    unsigned long long xb = 0;
    PG_CUDA(cudaMemcpyAsync(&lv, ws->lv, sizeof lv, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(flags, ws->flags, sizeof flags, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(&xb, ws->extent_bits, sizeof xb, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    double X;
    memcpy(&X, &xb, sizeof X);
    out->extent = X;
    out->n_bodies = n;
    out->n_nodes = (size_t)lv.total;
    out->flags = flags[kFlagNodes] | (flags[kFlagStack] << 1);
    const size_t nn = out->n_nodes < out->cap_nodes ? out->n_nodes : out->cap_nodes;
    auto cp = [&](void *dst, const void *src, size_t bytes) -> int {
        if (dst && bytes) PG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
        return PHYSIM_OK;
    };
    PG_TRY(cp(out->keys, ws->keys[ws->sorted], n * sizeof(uint64_t)));
    PG_TRY(cp(out->order, ws->vals[ws->sorted], n * sizeof(uint32_t)));
    PG_TRY(cp(out->node_begin, ws->nd.begin, nn * sizeof(int32_t)));
    PG_TRY(cp(out->node_count, ws->nd.count, nn * sizeof(int32_t)));
    PG_TRY(cp(out->node_child, ws->nd.child, nn * sizeof(int32_t)));
    PG_TRY(cp(out->node_nchild, ws->nd.nchild, nn));
    PG_TRY(cp(out->node_level, ws->nd.level, nn));
    if (out->node_centre)
        for (int c = 0; c < 4; ++c)
            PG_TRY(cp(out->node_centre + c * nn, ws->nd.c64 + (size_t)c * ws->nd.cap,
                      nn * sizeof(double)));
    PG_TRY(cp(out->node_com, ws->nd.com, nn * sizeof(float4)));
    PG_CUDA(cudaStreamSynchronize(st));
    return PHYSIM_OK;
}

}  // namespace pg
