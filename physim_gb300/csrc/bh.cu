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
//   3. sort      stable LSD radix sort of (key, body) pairs, 9-bit digits.
//   4. tree      not path-compressed (as the reference's pointer tree): a
//                cell with more than leaf_size bodies that are not all at
//                one key splits into its non-empty children; breadth-first
//                layout (levels contiguous, children contiguous in key
//                order), built flat for all levels at once from the
//                key-prefix boundaries (section 4).  Geometric centres are
//                computed exactly as the reference does (child = parent +-
//                extent/2, octree.rs:167-215).
//   5. moments   mass, centre of mass (double-float sums) and optionally
//                second moments (f32) of every cell, bottom up in one launch.
//   6. traversal one warp per 32 consecutive sorted bodies, DFS with a shared
//                stack, the reference's opening rule extent/|x - centre| < theta
//                (octree.rs:137-144).  EXACT: every body keeps its own
//                interaction list (the reference's); WARP: a cell is accepted
//                only if all 32 bodies accept it, and the common list is
//                batched through shared memory.  Pair law in FP32 with one
//                MUFU.RSQ per pair and compensated per-body sums.
#include <stdio.h>
#include <string.h>

#include <cuda/atomic>

#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "engine.h"
#include "plugin_state.h"

namespace pg {

namespace {

constexpr int kRadixBits = 9;
constexpr int kRadixBuckets = 1 << kRadixBits;
// 8,192 keys per tile: few tiles keep the look-back chains of a pass short
// (all tiles of a 1M-key sort are resident at once, so a pass's time is set
// by how far an inclusive prefix must travel from tile 0)
constexpr int kSortThreads = 512;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / 32;
constexpr size_t kSortSmem = (size_t)kSortTile * (sizeof(uint64_t) + sizeof(uint32_t));  // staged tile

constexpr int kMaxLevels = 31;

constexpr int kTravWarps = 4;
constexpr int kStack = 192;

// flags[0]: node capacity exceeded (tree truncated; results stay exact)
// flags[1]: traversal stack overflow (results of the affected warp invalid)
// flags[2]: a radix-sort look-back wait gave up (sort order invalid)
constexpr int kFlagNodes = 0;
constexpr int kFlagStack = 1;
constexpr int kFlagSort = 2;

// Radix sort of the 63-bit (62-bit) keys: 7 passes of 9-bit digits (512
// digits: one look-back thread each in a 512-thread tile).
constexpr int kSortPasses = 7;
// Look-back spin limit per digit (each spin is one L2 load, ~0.5 us worst
// case), far above any wait of a running predecessor tile; the default of
// physim_gpu_set_wait_limit.
constexpr int kLookbackSpins = 1 << 20;
// Predecessor tiles a look-back reads per round trip.
constexpr int kLookbackWindow = 8;

struct LevelInfo {
    int32_t begin[kMaxLevels + 2];  // first node of each level
    int32_t count[kMaxLevels + 2];  // nodes of each level
    int32_t total;                  // nodes in the tree
    int32_t max_level;              // deepest level built (below D only if capacity ran out)
};

__host__ __device__ inline int tree_levels(int nchild) { return nchild == 8 ? 21 : 31; }
__host__ __device__ inline int level_bits(int nchild) { return nchild == 8 ? 3 : 2; }

// ---------------------------------------------------------------------------
// 1. extent
// ---------------------------------------------------------------------------
// |coordinate| maxima on the f64 bit patterns: non-negative doubles order like
// their bit patterns, so integer maxima replace f64 ones (GB300 issues f64
// instructions at a small fraction of its integer rate).  NaN coordinates are
// skipped, as f64::max skips a NaN operand.
__device__ __forceinline__ unsigned long long abs_bits(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return b > 0x7ff0000000000000ull ? 0ull : b;
}

__global__ void extent_kernel(const double *__restrict__ x, const double *__restrict__ y,
                              const double *__restrict__ z, int n,
                              unsigned long long *__restrict__ out_bits)
{
    unsigned long long m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        m = max(m, abs_bits(x[i]));
        m = max(m, abs_bits(y[i]));
        m = max(m, abs_bits(z[i]));
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ unsigned long long wm[32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : 0ull;
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) atomicMax(out_bits, m);
    }
}

// ---------------------------------------------------------------------------
// 2. keys
// ---------------------------------------------------------------------------
// Cell index of coordinate p at the finest level D: the reference descends
// from centre 0 / half-width X deciding `p > centre` at every level.
// u = (p + X) * 2^(D-1) / X is the position in finest-cell units; unless u is
// within 2^-mbits (mbits = 40 - D) of a cell boundary, the cell is floor(u),
// read off u's bits with integer instructions (two f64 operations per axis).
// Close to a boundary, or for u < 1, the reference's centre arithmetic is
// replayed in f64.
__device__ __forceinline__ uint32_t axis_cell(double p, double X, double scale, int D, int mbits)
{
    const uint32_t lim = (1u << D) - 1u;
    const double u = __dmul_rn(__dadd_rn(p, X), scale);
    const unsigned long long bits = (unsigned long long)__double_as_longlong(u);
    const int ex = (int)((bits >> 52) & 0x7ff) - 1023;
    if (ex == 1024) return 0;  // NaN (or infinite) coordinate
    if (ex >= 0 && ex <= 52 - mbits) {
        const unsigned long long mant = (bits & 0xfffffffffffffull) | (1ull << 52);
        const int fb = 52 - ex;  // fraction bits of u
        const unsigned long long ip = mant >> fb;
        const unsigned long long top = (mant >> (fb - mbits)) & ((1ull << mbits) - 1ull);
        if (top != 0ull && top != (1ull << mbits) - 1ull)
            return ip > lim ? lim : (uint32_t)ip;
    }
    double c = 0.0, ext = X;
    uint32_t q = 0;
    for (int d = 0; d < D; ++d) {
        const bool hi = p > c;
        const double h = __dmul_rn(ext, 0.5);  // ext / 2, exact
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

// Keys, plus the histograms of all 7 radix digits of all keys (block-local in
// shared memory, then one global atomic per non-empty bucket), for the
// one-sweep sort.  ghist [7][512] must be zero on entry.  Block 0 also resets
// the sort's tile counters and grid barrier and advances its epoch (see
// radix_pass_kernel).
__global__ void __launch_bounds__(256)
keys_kernel(const double *__restrict__ x, const double *__restrict__ y,
            const double *__restrict__ z, int n, int nchild,
            const unsigned long long *__restrict__ extent_bits, uint64_t *__restrict__ keys,
            uint32_t *__restrict__ vals, uint32_t *__restrict__ ghist,
            uint32_t *__restrict__ tile_ctr, uint32_t *__restrict__ epoch,
            uint32_t *__restrict__ sort_bar)
{
    __shared__ double s_scale;
    __shared__ uint32_t h[kSortPasses][kRadixBuckets];
    const double X = __longlong_as_double((long long)*extent_bits);
    const int D = tree_levels(nchild);
    for (int k = threadIdx.x; k < kSortPasses * kRadixBuckets; k += blockDim.x) (&h[0][0])[k] = 0;
    if (threadIdx.x == 0) s_scale = X > 0.0 ? __ddiv_rn(ldexp(1.0, D - 1), X) : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int p = 0; p < kSortPasses; ++p) tile_ctr[p] = 0;
        *sort_bar = 0;
        *epoch += 1u;
    }
    __syncthreads();
    const double scale = s_scale;
    const int mbits = 40 - D;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t key = 0;
        if (X > 0.0) {
            const uint32_t qx = axis_cell(x[i], X, scale, D, mbits);
            const uint32_t qy = axis_cell(y[i], X, scale, D, mbits);
            if (nchild == 8) {
                const uint32_t qz = axis_cell(z[i], X, scale, D, mbits);
                key = spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
            } else {
                key = spread2(qx) | (spread2(qy) << 1);
            }
        }
        keys[i] = key;
        vals[i] = (uint32_t)i;
#pragma unroll
        for (int p = 0; p < kSortPasses; ++p)
            atomicAdd(&h[p][(uint32_t)(key >> (kRadixBits * p)) & (kRadixBuckets - 1)], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kSortPasses * kRadixBuckets; k += blockDim.x) {
        const uint32_t c = (&h[0][0])[k];
        if (c) atomicAdd(&ghist[k], c);
    }
}

// ---------------------------------------------------------------------------
// 3. radix sort (stable, LSD, 9-bit digits)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
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

// One tile of one pass of the radix sort (the body shared by the per-pass
// kernel and the single-launch sort): ranks the tile's keys by digit,
// publishes and looks back, and scatters through shared memory.  digit_base
// is this thread's digit's first place in the output (the scan of the
// pass's global histogram); h must be zero on entry.  The key and value
// pointers carry no __restrict__: in the single-launch sort a pass reads what
// other blocks of the same launch wrote, which the read-only cache path may
// not serve.
__device__ __forceinline__ void sort_tile(
    const uint64_t *keys_in, const uint32_t *vals_in, uint64_t *keys_out, uint32_t *vals_out,
    int n, int pass, int tile,
    uint32_t digit_base, unsigned long long *__restrict__ status,
    const uint32_t *__restrict__ epoch_ptr, uint32_t *__restrict__ flags, int spin_limit,
    int stall_tile, uint32_t (*h)[kRadixBuckets], uint32_t *digit_off, uint32_t *local_start,
    uint32_t *ws)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int shift = kRadixBits * pass;
    const int base = tile * kSortTile + warp * (kSortItems * 32);
    uint64_t kk[kSortItems];
    uint32_t vv[kSortItems];
    uint32_t rank[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        kk[r] = valid ? keys_in[idx] : 0;
        vv[r] = valid ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0;
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        // lanes with this lane's digit: one vote per digit bit (MATCH.ANY is
        // several times slower here)
        const uint32_t d = valid ? (uint32_t)(kk[r] >> shift) & (kRadixBuckets - 1) : 0u;
        uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int b = 0; b < kRadixBits; ++b) {
            const uint32_t bit = (d >> b) & 1u;
            const uint32_t vote = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? vote : ~vote;
        }
        const uint32_t before = __popc(peers & lanemask_lt());
        uint32_t cur = 0;
        if (valid) cur = h[warp][d];
        __syncwarp();
        if (valid && before == 0) h[warp][d] = cur + __popc(peers);
        __syncwarp();
        rank[r] = cur + before;
    }
    __syncthreads();
    // this tile's count of digit d, and the warps' exclusive offsets within it
    // (threads 0..255, one digit each)
    const int d = threadIdx.x;
    if (d < kRadixBuckets) {
        uint32_t count = 0;
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = h[w][d];
            h[w][d] = count;
            count += c;
        }
        {
            uint32_t total;
            local_start[d] = block_exclusive_scan(count, ws, total);
        }
        // tag base of this sort and pass: the passes share the status array
        const unsigned long long ep =
            ((unsigned long long)(*epoch_ptr & 0x03ffffffu) * kSortPasses + (unsigned)pass) * 4ull;
        volatile unsigned long long *st = status;
        uint32_t excl = 0;
        if (tile == 0) {
            st[d] = ((ep + 2ull) << 32) | count;
        } else {
            st[(size_t)tile * kRadixBuckets + d] = ((ep + 1ull) << 32) | count;
            // walk back kLookbackWindow tiles per round trip: the window's words
            // are loaded together, then summed up to the first inclusive prefix
            int t = tile - 1;
            int spins = 0;
            const bool stall = tile == stall_tile;
            for (;;) {
                unsigned long long w[kLookbackWindow];
#pragma unroll
                for (int j = 0; j < kLookbackWindow; ++j)
                    w[j] = t - j >= 0 && !stall ? st[(size_t)(t - j) * kRadixBuckets + d] : 0ull;
                int used = 0;
                bool done = false;
#pragma unroll
                for (int j = 0; j < kLookbackWindow; ++j) {
                    if (done || used != j) continue;
                    const unsigned long long tag = w[j] >> 32;
                    if (tag == ep + 2ull) {
                        excl += (uint32_t)w[j];
                        done = true;
                    } else if (tag == ep + 1ull) {
                        excl += (uint32_t)w[j];
                        ++used;  // t - j > 0 here: tile 0 publishes its inclusive prefix at once
                    }
                }
                if (done) break;
                t -= used;
                if (used == 0 && ++spins > spin_limit) {
                    atomicOr(&flags[kFlagSort], 1u);
                    break;
                }
            }
            st[(size_t)tile * kRadixBuckets + d] = ((ep + 2ull) << 32) | (excl + count);
        }
        digit_off[d] = digit_base + excl;
    }
    __syncthreads();
    // the tile in digit order in shared memory, then each digit's run written
    // to its place in one contiguous stretch (scattered 8-byte stores cost
    // a third of the pass)
    extern __shared__ uint64_t skeys[];  // kSortTile keys, then kSortTile values
    uint32_t *svals = reinterpret_cast<uint32_t *>(skeys + kSortTile);
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        if (idx >= n) continue;
        const uint32_t dg = (uint32_t)(kk[r] >> shift) & (kRadixBuckets - 1);
        const uint32_t lp = local_start[dg] + h[warp][dg] + rank[r];
        skeys[lp] = kk[r];
        svals[lp] = vv[r];
    }
    __syncthreads();
    const int cnt = min(kSortTile, n - tile * kSortTile);
    for (int j = threadIdx.x; j < cnt; j += kSortThreads) {
        const uint64_t key = skeys[j];
        const uint32_t dg = (uint32_t)(key >> shift) & (kRadixBuckets - 1);
        const uint32_t pos = digit_off[dg] + (uint32_t)j - local_start[dg];
        keys_out[pos] = key;
        vals_out[pos] = svals[j];
    }
}

// One stable counting pass of the one-sweep LSD radix sort (single-pass
// chained scan with decoupled look-back, after Merrill & Garland 2016 and
// Adinets & Merrill 2022).  Tiles of kSortTile keys are claimed in launch
// order from an atomic counter, so every tile a block looks back at is held
// by a block that is already running.  Each block ranks its keys by digit
// (warp by warp, stable, lanes of equal digit found by one ballot per digit
// bit), publishes its per-digit counts, then walks back over the preceding
// tiles' published words until it meets an inclusive prefix, publishes its
// own inclusive prefix, and scatters: the tile is first put in digit order
// in shared memory, so each digit's keys leave in one contiguous run.  A status word is
// (epoch * 4 + flag) << 32 | count, flag 1 = tile count, 2 = inclusive
// prefix, and epoch counts (sort, pass) pairs; words of earlier passes and
// sorts carry older epochs and read as not ready, so the status array needs
// no clearing.  A wait that exceeds
// the wait limit (kLookbackSpins unless physim_gpu_set_wait_limit set one)
// sets flags[kFlagSort] and gives up: the tile still scatters, at positions no
// higher than the right ones (its prefix is a partial sum), so every write
// stays in bounds; every later kernel of the build and the traversal see the
// flag and return at once, so nothing reads the invalid order or an unbuilt
// tree, and the host reports PHYSIM_ERR_TIMEOUT.  stall_tile >= 0
// (physim_gpu_test_stall_sort) makes that tile's look-back see no
// predecessor word, so the limit is reached for sure.
__global__ void __launch_bounds__(kSortThreads)
radix_pass_kernel(const uint64_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                  uint64_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int n,
                  int pass, const uint32_t *__restrict__ ghist, uint32_t *__restrict__ tile_ctr,
                  unsigned long long *__restrict__ status, const uint32_t *__restrict__ epoch_ptr,
                  uint32_t *__restrict__ flags, int spin_limit, int stall_tile)
{
    static_assert(kSortThreads >= kRadixBuckets, "one thread per digit");
    __shared__ uint32_t h[kSortWarps][kRadixBuckets];
    __shared__ uint32_t digit_off[kRadixBuckets];
    __shared__ uint32_t local_start[kRadixBuckets];  // the digit's first key in the staged tile
    __shared__ uint32_t ws[33];
    __shared__ int s_tile, s_stop;
    // an earlier wait failed: the whole block leaves (one read, shared, since
    // another block of this launch may raise the flag meanwhile)
    if (threadIdx.x == 0) {
        s_stop = *(volatile const uint32_t *)&flags[kFlagSort] != 0u;
        s_tile = (int)atomicAdd(&tile_ctr[pass], 1u);
    }
    __syncthreads();
    if (s_stop) return;
    for (int k = threadIdx.x; k < kSortWarps * kRadixBuckets; k += kSortThreads)
        (&h[0][0])[k] = 0;
    uint32_t digit_base;
    {
        uint32_t total;
        const uint32_t c = threadIdx.x < kRadixBuckets ? ghist[pass * kRadixBuckets + threadIdx.x]
                                                       : 0u;
        digit_base = block_exclusive_scan(c, ws, total);
    }
    sort_tile(keys_in, vals_in, keys_out, vals_out, n, pass, s_tile, digit_base, status,
              epoch_ptr, flags, spin_limit, stall_tile, h, digit_off, local_start, ws);
}

// All seven passes in one cooperative launch (every block resident, up to
// one per SM): each block takes tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// of every pass, and a grid barrier separates the passes (a pass reads keys
// that every tile of the previous one wrote).  Every tile a look-back waits on
// is lower-numbered, so it is held by a resident block that reaches it after
// lower tiles only: the waits end.  The barrier is a counter each block adds
// to once per pass (reset by keys_kernel); its wait gives up after the wait
// limit, or at once when the sort's error flag is up, raising the flag, so no
// block waits for one that has left.  Against one launch per pass this saves
// six launch gaps and the tail of each pass.
__device__ __forceinline__ bool sort_grid_barrier(uint32_t *bar, uint32_t target,
                                                  uint32_t *flags, int spin_limit, int *s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        int spins = 0;
        while (*(volatile uint32_t *)bar < target) {
            if (*(volatile uint32_t *)&flags[kFlagSort] != 0u) break;
            if (++spins > spin_limit) {
                atomicOr(&flags[kFlagSort], 1u);
                break;
            }
        }
        __threadfence();
        *s_ok = *(volatile uint32_t *)&flags[kFlagSort] == 0u;
    }
    __syncthreads();
    return *s_ok != 0;
}

__global__ void __launch_bounds__(kSortThreads, 1)
radix_sort_kernel(uint64_t *k0, uint32_t *v0, uint64_t *k1, uint32_t *v1, int n,
                  const uint32_t *__restrict__ ghist, unsigned long long *__restrict__ status,
                  const uint32_t *__restrict__ epoch_ptr, uint32_t *__restrict__ flags,
                  int spin_limit, int stall_tile, uint32_t *bar)
{
    static_assert(kSortThreads == kRadixBuckets, "one thread per digit");
    __shared__ uint32_t h[kSortWarps][kRadixBuckets];
    __shared__ uint32_t digit_off[kRadixBuckets];
    __shared__ uint32_t local_start[kRadixBuckets];
    __shared__ uint32_t ws[33];
    __shared__ int s_ok;
    if (threadIdx.x == 0) s_ok = *(volatile const uint32_t *)&flags[kFlagSort] == 0u;
    __syncthreads();
    if (!s_ok) return;
    const int tiles = (n + kSortTile - 1) / kSortTile;
    for (int pass = 0; pass < kSortPasses; ++pass) {
        const uint64_t *keys_in = (pass & 1) ? k1 : k0;
        const uint32_t *vals_in = pass == 0 ? nullptr : ((pass & 1) ? v1 : v0);
        uint64_t *keys_out = (pass & 1) ? k0 : k1;
        uint32_t *vals_out = (pass & 1) ? v0 : v1;
        uint32_t digit_base;
        {
            uint32_t total;
            digit_base = block_exclusive_scan(ghist[pass * kRadixBuckets + threadIdx.x], ws, total);
        }
        for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
            for (int k = threadIdx.x; k < kSortWarps * kRadixBuckets; k += kSortThreads)
                (&h[0][0])[k] = 0;
            __syncthreads();
            sort_tile(keys_in, vals_in, keys_out, vals_out, n, pass, tile, digit_base, status,
                      epoch_ptr, flags, spin_limit, stall_tile, h, digit_off, local_start, ws);
            __syncthreads();  // the staged tile, h and the offsets serve the next tile
        }
        if (pass + 1 < kSortPasses &&
            !sort_grid_barrier(bar, (uint32_t)(pass + 1) * gridDim.x, flags, spin_limit, &s_ok))
            return;
    }
}

// ---------------------------------------------------------------------------
// node arrays
// ---------------------------------------------------------------------------
struct NodeArrays {
    int32_t *begin, *count, *child;
    uint8_t *nchild, *level;
    double *c64;   // 4 x cap: cx, cy, cz, extent
    float4 *geo;   // cx, cy, cz, extent (f32)
    float4 *com;   // x, y, z, mass (f32)
    int4 *meta;    // (id | nchild << 28, first child, first body, body count)
    int32_t *parent;   // parent node, -1 for the root
    float4 *msum_hi;   // mass and mass-weighted position sums (M, Mx, My, Mz) as
    float4 *msum_lo;   //   double-float pairs (hi + lo)
    float4 *quad_a;    // second moments about the centre of mass: Sxx, Syy, Szz, trace
    float4 *quad_b;    // Sxy, Sxz, Syz, 0
    uint32_t *arrivals;  // children finished, for the bottom-up moment pass (kept at 0)
    int cap;
};

// ---------------------------------------------------------------------------
// 4. tree build (flat: a few launches for all levels)
// ---------------------------------------------------------------------------
// The tree is the reference's non-path-compressed one over the sorted keys: a
// node at level l is a maximal run of bodies sharing the first l digits of
// their keys, and it exists iff l = 0 or the run one level up (its parent)
// splits, i.e. holds more than leaf_size bodies whose keys are not all equal,
// at a level below D.  Node numbering is breadth first: levels one after the
// other, each in key order, so a node's children are contiguous and in
// octant order, as a level-by-level serial build lays them out.
//
// With L(i) the number of leading digits keys[i-1] and keys[i] share, a run
// at level l starts at body i iff i = 0 or L(i) < l, and everything about
// the runs starting at i follows from L near i:
//   * the run at level l starting at i has more than `leaf` bodies iff
//     L(i+1..i+leaf) are all >= l (those bodies exist);
//   * it is not uniform iff the first body after i with a different key,
//     u(i), has L(u(i)) >= l;
//   * so it splits iff l <= c(i) = min(m(i), L(u(i)), D - 1), m(i) the
//     minimum of L over the next leaf boundaries;
//   * a run at level l > L(i) + 1 starting at i exists iff its parent (the
//     run at l - 1 starting at i) splits, i.e. l <= c(i) + 1;
//   * the run at level L(i) + 1 exists iff the run at level L(i) containing
//     i - 1 and i (not uniform: those keys differ) has more than leaf
//     bodies, which a scan of L over leaf boundaries either side decides.
// Each body's existing runs form a bit mask over levels; a node's index is
// the start of its level plus the count of set bits of that level before its
// body (block counts, one scan over blocks, warp ballots within a block).
// The deepest run a body starts is a leaf; its end (the next boundary below
// its level) is read off the same shared tile of L.

constexpr int kTreeBlock = 1024;   // bodies per block of the mask and node kernels
constexpr int kTreeHalo = 72;      // boundaries read either side (> the largest leaf + 1)
constexpr int kMaxLeaf = 64;
constexpr uint8_t kLongLeaf = 255;  // leaf count marker: longer than the shared tile reaches

__device__ __forceinline__ bool sort_failed(const uint32_t *flags)
{
    return *(volatile const uint32_t *)&flags[kFlagSort] != 0u;
}

// L(k) for k >= 1 (the number of leading digits keys[k-1] and keys[k] share,
// D for equal keys), and the sorted f32 bodies.
__global__ void boundary_kernel(const uint64_t *__restrict__ keys,
                                const uint32_t *__restrict__ order, int n, int nchild,
                                const float4 *__restrict__ body4, float4 *__restrict__ sbody,
                                uint8_t *__restrict__ lcp, const uint32_t *__restrict__ flags)
{
    if (sort_failed(flags)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int D = tree_levels(nchild), B = level_bits(nchild);
    sbody[k] = body4[order[k]];
    int L = 0;
    if (k > 0) {
        const uint64_t x = keys[k - 1] ^ keys[k];
        // keys use the low B * D bits: 64 - B * D leading bits are always 0
        L = x == 0 ? D : (__clzll((long long)x) - (64 - B * D)) / B;
    }
    lcp[k] = (uint8_t)L;
}

// First index j in [lo, n) with keys[j] != keys[i] (keys sorted), or n.
__device__ __forceinline__ int next_key_change(const uint64_t *__restrict__ keys, int i, int lo,
                                               int n)
{
    const uint64_t ki = keys[i];
    int hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] == ki)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Level masks of the bodies (bit l: a node at level l starts at this body),
// per-block counts of every level (blk_cnt[l * nblk + block]) and the body
// count of the leaf starting at each body (the deepest run it starts; 0: no
// node starts here, kLongLeaf: longer than the shared tile reaches); also
// zeroes the child counters.  The questions about L near a body (the minimum
// over the next `leaf` boundaries; how many consecutive boundaries either side,
// or after the body, are at or below a level) are answered from tables of
// window minima over 1, 2, 4, ..., 64 boundaries of the block's tile: the
// minimum over any window of up to 64 from two overlapping entries, a run
// length by binary lifting (the longest run is the sum of the powers of two
// whose windows, taken largest first, stay at or below the level), so every
// body takes the same few steps instead of a loop of data-dependent length.
constexpr int kTreeTile = kTreeBlock + 2 * kTreeHalo;
constexpr int kMinTables = 7;  // windows of 2^0 .. 2^6 boundaries
static_assert(kMaxLeaf <= (1 << (kMinTables - 1)) && kMaxLeaf + 1 < kTreeHalo,
              "leaf windows fit the tables and the halo");

__global__ void __launch_bounds__(kTreeBlock)
mask_kernel(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ lcp, int n,
            int nchild, int leaf, uint32_t *__restrict__ mask, uint32_t *__restrict__ blk_cnt,
            int nblk, uint8_t *__restrict__ leafcnt, uint32_t *__restrict__ nchild32, int cap,
            const uint32_t *__restrict__ flags)
{
    if (sort_failed(flags)) return;
    // sM[p][t]: minimum of L over boundaries t .. t + 2^p - 1 of the tile
    // (clipped at the tile's end; every query below stays inside it)
    __shared__ int8_t sM[kMinTables][kTreeTile];
    __shared__ uint32_t cnt[32];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cap; k += gridDim.x * blockDim.x)
        nchild32[k] = 0u;
    const int D = tree_levels(nchild);
    const int base = blockIdx.x * kTreeBlock;
    // boundaries base - halo .. base + block + halo; -1 marks "no boundary
    // beyond here" (index 0 starts every run, indices >= n end them)
    for (int t = threadIdx.x; t < kTreeTile; t += blockDim.x) {
        const int j = base - kTreeHalo + t;
        sM[0][t] = (j >= 1 && j < n) ? (int8_t)lcp[j] : (int8_t)-1;
    }
    if (threadIdx.x < 32) cnt[threadIdx.x] = 0u;
    __syncthreads();
    for (int q = 1; q < kMinTables; ++q) {
        const int h = 1 << (q - 1);
        for (int t = threadIdx.x; t < kTreeTile; t += blockDim.x) {
            const int a = sM[q - 1][t];
            sM[q][t] = (int8_t)(t + h < kTreeTile ? min(a, (int)sM[q - 1][t + h]) : a);
        }
        __syncthreads();
    }
    const int8_t *sL = sM[0];
    const int i = base + threadIdx.x;
    uint32_t m = 0u;
    if (i < n) {
        const int s = threadIdx.x + kTreeHalo;  // i's slot in the tile
        const int Li = i == 0 ? -1 : sL[s];
        // m(i): min of L over the next leaf boundaries, -1 if fewer remain
        int mi = -1;
        if (i + leaf <= n - 1) {
            const int q = 31 - __clz(leaf);
            mi = min((int)sM[q][s + 1], (int)sM[q][s + leaf + 1 - (1 << q)]);
        }
        // u(i): the next body with another key; L(u(i)), -1 if none
        int Lu = -1;
        {
            int j = i + 1, t = s + 1;
            while (j < n && t < kTreeTile && sL[t] == D) {
                ++j;
                ++t;
            }
            if (j < n && t >= kTreeTile) j = next_key_change(keys, i, j, n);
            if (j < n) Lu = lcp[j];
        }
        const int c = min(min(mi, Lu), D - 1);
        if (i == 0) {
            m = 1u;  // the root
            for (int l = 1; l <= c + 1; ++l) m |= 1u << l;
        } else if (Li < D) {
            // the run at level Li containing i - 1 and i: more than leaf bodies?
            // (lft, rgt: consecutive boundaries at or below Li before and
            // after i, up to leaf each)
            int lft = 0, rgt = 0;
#pragma unroll
            for (int q = kMinTables - 1; q >= 0; --q) {
                const int k = 1 << q;
                if (lft + k <= leaf && sM[q][s - lft - k] >= Li) lft += k;
                if (rgt + k <= leaf && sM[q][s + rgt + 1] >= Li) rgt += k;
            }
            if (lft + rgt + 2 > leaf) {
                m |= 1u << (Li + 1);
                for (int l = Li + 2; l <= c + 1; ++l) m |= 1u << l;
            }
        }
        mask[i] = m;
        // the leaf starting here (the deepest run; unless the capacity stops
        // the tree above it) runs to the next boundary below its level
        uint8_t lc = 0;
        if (m != 0u) {
            const int lf = 31 - __clz(m);
            const int room = kTreeTile - 1 - s;  // boundaries after i in the tile
            int run = 0;
            while (run + 64 <= room && sM[6][s + 1 + run] >= lf) run += 64;
#pragma unroll
            for (int q = kMinTables - 2; q >= 0; --q) {
                const int k = 1 << q;
                if (run + k <= room && sM[q][s + 1 + run] >= lf) run += k;
            }
            const int e = i + 1 + run, t = s + 1 + run;
            lc = (e < n && t >= kTreeTile) || e - i >= (int)kLongLeaf ? kLongLeaf
                                                                      : (uint8_t)(e - i);
        }
        leafcnt[i] = lc;
    }
    // per-level counts: only the levels some lane of the warp starts
    uint32_t present = __reduce_or_sync(0xffffffffu, m);
    while (present) {
        const int l = __ffs(present) - 1;
        present &= present - 1u;
        const uint32_t b = __ballot_sync(0xffffffffu, (m >> l) & 1u);
        if ((threadIdx.x & 31) == 0) atomicAdd(&cnt[l], (uint32_t)__popc(b));
    }
    __syncthreads();
    if (threadIdx.x < 32) blk_cnt[(size_t)threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

// One block: per level, the exclusive scan of the block counts (blk_off,
// same layout as blk_cnt) and the level's first node.  Warp l scans row l,
// 32 blocks per step.  If the nodes do not fit the node arrays, the tree
// stops at the deepest level that fits (its nodes become leaves: results
// stay exact, slower) and flags[kFlagNodes] is raised.
__global__ void __launch_bounds__(1024)
level_scan_kernel(const uint32_t *__restrict__ blk_cnt, int nblk, int nchild,
                  uint32_t *__restrict__ blk_off, LevelInfo *lv, int cap,
                  uint32_t *__restrict__ flags)
{
    if (sort_failed(flags)) return;
    __shared__ uint32_t total_of[32];
    const int D = tree_levels(nchild);
    const int l = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t *row = blk_cnt + (size_t)l * nblk;
    uint32_t *orow = blk_off + (size_t)l * nblk;
    uint32_t carry = 0;
    constexpr int kAhead = 4;  // row chunks loaded before they are scanned
    for (int c0 = 0; c0 < nblk; c0 += 32 * kAhead) {
        uint32_t v[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            const int b = c0 + u * 32 + lane;
            v[u] = b < nblk ? row[b] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            uint32_t incl = v[u];
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int b = c0 + u * 32 + lane;
            if (b < nblk) orow[b] = carry + incl - v[u];
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
    if (lane == 0) total_of[l] = carry;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long at = 0;
        int max_level = D;
        for (int q = 0; q <= D; ++q) {
            const long long c = total_of[q];
            if (at + c > cap) {
                max_level = q - 1;
                atomicOr(&flags[kFlagNodes], 1u);
                break;
            }
            at += c;
        }
        at = 0;
        for (int q = 0; q < kMaxLevels + 2; ++q) {
            const int c = q <= max_level ? (int)total_of[q] : 0;
            lv->begin[q] = (int32_t)at;
            lv->count[q] = c;
            at += c;
        }
        lv->total = (int32_t)at;
        lv->max_level = max_level;
    }
}

// Node records: per body, one node per set bit of its mask.  Leaves get
// their body count here; an internal node's count, its child count and its
// traversal metadata are completed by the moment pass (children counted into
// nchild32 here); the centres by centre_kernel.
__global__ void __launch_bounds__(kTreeBlock)
node_kernel(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ leafcnt,
            const uint32_t *__restrict__ mask, const uint32_t *__restrict__ blk_off, int nblk,
            int n, int nchild, NodeArrays nd, const LevelInfo *__restrict__ lv,
            uint32_t *__restrict__ nchild32, const uint32_t *__restrict__ flags)
{
    if (sort_failed(flags)) return;
    __shared__ uint32_t sbal[kTreeBlock / 32][32];  // per warp and level: lanes with that bit
    __shared__ uint32_t woff[kTreeBlock / 32][32];  // ... and the level's nodes before the warp
    __shared__ int32_t lbeg[kMaxLevels + 2];
    const int D = tree_levels(nchild), B = level_bits(nchild);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * kTreeBlock + threadIdx.x;
    const uint32_t m = i < n ? mask[i] : 0u;
    for (int l = 0; l < 32; ++l) {
        const uint32_t b = __ballot_sync(0xffffffffu, (m >> l) & 1u);
        if (lane == 0) {
            sbal[warp][l] = b;
            woff[warp][l] = (uint32_t)__popc(b);
        }
    }
    if (threadIdx.x < kMaxLevels + 2) lbeg[threadIdx.x] = lv->begin[threadIdx.x];
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t run = blk_off[(size_t)threadIdx.x * nblk + blockIdx.x];
        for (int w = 0; w < kTreeBlock / 32; ++w) {
            const uint32_t v = woff[w][threadIdx.x];
            woff[w][threadIdx.x] = run;
            run += v;
        }
    }
    __syncthreads();
    if (m == 0u) return;
    const int max_level = lv->max_level;
    const uint32_t lt = (1u << lane) - 1u, le = lt | (1u << lane);
    const int top = min(31 - __clz(m), max_level);
    for (int l = __ffs(m) - 1; l <= top; ++l) {
        if (!((m >> l) & 1u)) continue;
        const int x = lbeg[l] + (int)woff[warp][l] + __popc(sbal[warp][l] & lt);
        int parent = -1;
        if (l > 0) {
            // the last node of level l - 1 starting at or before body i
            parent = lbeg[l - 1] + (int)woff[warp][l - 1] + __popc(sbal[warp][l - 1] & le) - 1;
            atomicAdd(&nchild32[parent], 1u);
        }
        const bool splits = l + 1 <= max_level && ((m >> (l + 1)) & 1u);
        const int first_child =
            splits ? lbeg[l + 1] + (int)woff[warp][l + 1] + __popc(sbal[warp][l + 1] & lt) : -1;
        nd.begin[x] = i;
        nd.level[x] = (uint8_t)l;
        nd.parent[x] = parent;
        nd.child[x] = first_child;
        if (!splits) {
            // a leaf: its bodies run to the next boundary below level l
            int cnt = leafcnt[i];
            if (cnt == kLongLeaf || l != 31 - __clz(m)) {
                // a long run (equal keys, or a node the capacity kept from
                // splitting): the end of its level-l key prefix
                const int sh = B * (D - l);
                const uint64_t p = keys[i] >> sh;
                int lo = i + 1, hi = n;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if ((keys[mid] >> sh) == p)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                cnt = lo - i;
            }
            nd.count[x] = cnt;
            nd.nchild[x] = 0;
            nd.meta[x] = make_int4(x, -1, i, cnt);
        }
    }
}

// Geometric centres and half-widths of the nodes.  For the exact traversal
// (exact != 0) the f64 centres follow the reference's arithmetic from the
// root down (child = parent +- half-width / 2 per level, octree.rs:167-215,
// quadtree.rs:167-194; the traversal re-decides near-threshold openings with
// them): thread x follows the digits of its node's first key.  The warp
// traversal needs only the f32 geometry: X (2q + 1 - 2^l) / 2^l from the
// cell index q, one f64 product per axis rounded to f32 (within an f32 ulp
// of the f64 chain's value; the traversal's margins allow 3).  Node-parallel,
// so consecutive threads hold nodes of one level (equal chain lengths).
__device__ __forceinline__ uint32_t compact3(uint64_t x)
{
    x &= 0x1249249249249249ull;
    x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ull;
    x = (x ^ (x >> 4)) & 0x100f00f00f00f00full;
    x = (x ^ (x >> 8)) & 0x1f0000ff0000ffull;
    x = (x ^ (x >> 16)) & 0x1f00000000ffffull;
    x = (x ^ (x >> 32)) & 0x1fffffull;
    return (uint32_t)x;
}

__device__ __forceinline__ uint32_t compact2(uint64_t x)
{
    x &= 0x5555555555555555ull;
    x = (x | (x >> 1)) & 0x3333333333333333ull;
    x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
    x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
    x = (x | (x >> 16)) & 0x00000000ffffffffull;
    return (uint32_t)x;
}

__global__ void centre_kernel(const uint64_t *__restrict__ keys, NodeArrays nd,
                              const LevelInfo *__restrict__ lv, int nchild, int exact,
                              const unsigned long long *__restrict__ extent_bits,
                              const uint32_t *__restrict__ flags)
{
    if (sort_failed(flags)) return;
    const int total = lv->total;
    const int D = tree_levels(nchild), B = level_bits(nchild);
    const uint32_t dmask = (uint32_t)nchild - 1u;
    const double X = __longlong_as_double((long long)*extent_bits);
    const size_t cap = nd.cap;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < total; x += gridDim.x * blockDim.x) {
        const int l = nd.level[x];
        const uint64_t key = keys[nd.begin[x]];
        if (exact) {
            double cx = 0.0, cy = 0.0, cz = 0.0, ext = X;
            for (int j = 1; j <= l; ++j) {
                const uint32_t q = (uint32_t)(key >> (B * (D - j))) & dmask;
                const double h = __dmul_rn(ext, 0.5);  // ext / 2, exact
                cx = (q & 1) ? __dadd_rn(cx, h) : __dsub_rn(cx, h);
                cy = (q & 2) ? __dadd_rn(cy, h) : __dsub_rn(cy, h);
                if (nchild == 8) cz = (q & 4) ? __dadd_rn(cz, h) : __dsub_rn(cz, h);
                ext = h;
            }
            nd.c64[x] = cx;
            nd.c64[cap + x] = cy;
            nd.c64[2 * cap + x] = cz;
            nd.c64[3 * cap + x] = ext;
            nd.geo[x] = make_float4((float)cx, (float)cy, (float)cz, (float)ext);
        } else {
            const uint64_t pre = l == 0 ? 0ull : key >> (B * (D - l));
            const double h = X * pow2d(-l);  // the half-width, exact
            const long long span = 1ll << l;
            const uint32_t qx = nchild == 8 ? compact3(pre) : compact2(pre);
            const uint32_t qy = nchild == 8 ? compact3(pre >> 1) : compact2(pre >> 1);
            const float gx = (float)(h * (double)(2ll * qx + 1 - span));
            const float gy = (float)(h * (double)(2ll * qy + 1 - span));
            const float gz =
                nchild == 8 ? (float)(h * (double)(2ll * compact3(pre >> 2) + 1 - span)) : 0.f;
            nd.geo[x] = make_float4(gx, gy, gz, (float)h);
        }
    }
}

// ---------------------------------------------------------------------------
// 5. moments: mass, centre of mass and (optionally) second moments of every
//    cell, bottom up in one launch
// ---------------------------------------------------------------------------
// Each leaf sums its own bodies: mass and mass-weighted positions as
// double-float (hi + lo f32) pairs, each product m x taken exactly (TwoProduct
// by FMA) -- FP32 arithmetic only, as GB300 issues f64 instructions at a small
// fraction of its f32 rate.  A parent is finished by the thread of its last
// child to arrive (an acquire-release count of arrivals; nothing waits),
// which adds the children's pairs in child order -- so results do not depend
// on the arrival order -- and continues upwards; it also completes the
// parent's body count, child count and traversal metadata.  The f32 centre
// of mass c = S / M is the double-float quotient rounded once.  A leaf whose
// bodies all sit at one position keeps that exact position, so a body there
// cancels against it as the reference's equal-centre skip does; a massless
// cell sits at its geometric centre.  Second moments (quad) are f32,
// combined with the parallel-axis rule S = sum_c [S_c + M_c (c_c - c)(c_c - c)^T].
__device__ __forceinline__ void store_quad(const NodeArrays &nd, int i, const float s[6])
{
    nd.quad_a[i] = make_float4(s[0], s[1], s[2], s[0] + s[1] + s[2]);
    nd.quad_b[i] = make_float4(s[3], s[4], s[5], 0.f);
}

// (ah, al) + (bh, bl) as a normalised double-float pair.
__device__ __forceinline__ void df_add(float &ah, float &al, float bh, float bl)
{
    float s, e;
    two_sum(ah, bh, s, e);
    e += al + bl;
    ah = s + e;
    al = e - (ah - s);
}

// f32 rounding of (sh + sl) / (mh + ml): an f32 quotient corrected once with
// its exact residual (TwoProduct by FMA).
__device__ __forceinline__ float df_div(float sh, float sl, float mh, float ml)
{
    const float q = sh / mh;
    const float p = q * mh;
    const float pe = fmaf(q, mh, -p);
    const float r = fmaf(-q, ml, ((sh - p) - pe) + sl);
    return q + r / mh;
}

__device__ __forceinline__ float4 df_com(const float4 h, const float4 l, float4 geo)
{
    if (h.x == 0.f && l.x == 0.f) return make_float4(geo.x, geo.y, geo.z, 0.f);
    return make_float4(df_div(h.y, l.y, h.x, l.x), df_div(h.z, l.z, h.x, l.x),
                       df_div(h.w, l.w, h.x, l.x), h.x + l.x);
}

// m * p added exactly-rounded into the double-float (hi, lo)
__device__ __forceinline__ void df_add_prod(float &hi, float &lo, float m, float p)
{
    const float pr = m * p;
    const float pe = fmaf(m, p, -pr);
    df_add(hi, lo, pr, pe);
}

__global__ void moments_kernel(NodeArrays nd, const LevelInfo *__restrict__ lv,
                               const float4 *__restrict__ sbody, int quad,
                               const uint32_t *__restrict__ nchild32,
                               const uint32_t *__restrict__ flags)
{
    if (sort_failed(flags)) return;
    const int total = lv->total;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (nd.child[i] >= 0) continue;
        const int b = nd.begin[i], e = b + nd.count[i];
        const float4 p0 = sbody[b];
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        bool same = true;
        for (int j = b; j < e; ++j) {
            const float4 p = sbody[j];
            df_add(h.x, l.x, p.w, 0.f);
            df_add_prod(h.y, l.y, p.w, p.x);
            df_add_prod(h.z, l.z, p.w, p.y);
            df_add_prod(h.w, l.w, p.w, p.z);
            same = same && p.x == p0.x && p.y == p0.y && p.z == p0.z;
        }
        nd.msum_hi[i] = h;
        nd.msum_lo[i] = l;
        const float4 com = same ? make_float4(p0.x, p0.y, p0.z, h.x + l.x)
                                : df_com(h, l, nd.geo[i]);
        nd.com[i] = com;
        if (quad) {
            float q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (!same)
                for (int j = b; j < e; ++j) {
                    const float4 p = sbody[j];
                    const float dx = p.x - com.x, dy = p.y - com.y, dz = p.z - com.z;
                    q[0] = fmaf(p.w * dx, dx, q[0]);
                    q[1] = fmaf(p.w * dy, dy, q[1]);
                    q[2] = fmaf(p.w * dz, dz, q[2]);
                    q[3] = fmaf(p.w * dx, dy, q[3]);
                    q[4] = fmaf(p.w * dx, dz, q[4]);
                    q[5] = fmaf(p.w * dy, dz, q[5]);
                }
            store_quad(nd, i, q);
        }
        int node = i;
        for (;;) {
            const int par = nd.parent[node];
            if (par < 0) break;
            const int nc = (int)nchild32[par];
            // release: this child's sums are visible before its arrival
            // counts; acquire: the last arriver sees every sibling's
            cuda::atomic_ref<uint32_t, cuda::thread_scope_device> arrivals(nd.arrivals[par]);
            const uint32_t arrived = arrivals.fetch_add(1u, cuda::memory_order_acq_rel);
            if (arrived + 1u != (uint32_t)nc) break;
            nd.arrivals[par] = 0u;  // ready for the next build
            const int fc = nd.child[par];
            float4 ph = __ldcg(&nd.msum_hi[fc]), pl = __ldcg(&nd.msum_lo[fc]);
            int count = __ldcg(&nd.count[fc]);
            for (int k = fc + 1; k < fc + nc; ++k) {
                const float4 ch = __ldcg(&nd.msum_hi[k]), cl = __ldcg(&nd.msum_lo[k]);
                df_add(ph.x, pl.x, ch.x, cl.x);
                df_add(ph.y, pl.y, ch.y, cl.y);
                df_add(ph.z, pl.z, ch.z, cl.z);
                df_add(ph.w, pl.w, ch.w, cl.w);
                count += __ldcg(&nd.count[k]);
            }
            nd.msum_hi[par] = ph;
            nd.msum_lo[par] = pl;
            nd.count[par] = count;
            nd.nchild[par] = (uint8_t)nc;
            nd.meta[par] = make_int4(par | (nc << 28), fc, nd.begin[par], count);
            const float4 cp = df_com(ph, pl, nd.geo[par]);
            nd.com[par] = cp;
            if (quad) {
                float t[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                for (int k = fc; k < fc + nc; ++k) {
                    const float4 cc = __ldcg(&nd.com[k]);
                    const float4 qa = __ldcg(&nd.quad_a[k]);
                    const float4 qb = __ldcg(&nd.quad_b[k]);
                    const float dx = cc.x - cp.x, dy = cc.y - cp.y, dz = cc.z - cp.z;
                    t[0] += fmaf(cc.w * dx, dx, qa.x);
                    t[1] += fmaf(cc.w * dy, dy, qa.y);
                    t[2] += fmaf(cc.w * dz, dz, qa.z);
                    t[3] += fmaf(cc.w * dx, dy, qb.x);
                    t[4] += fmaf(cc.w * dx, dz, qb.y);
                    t[5] += fmaf(cc.w * dy, dz, qb.z);
                }
                store_quad(nd, par, t);
            }
            node = par;
        }
    }
}

// ---------------------------------------------------------------------------
// 6. traversal
// ---------------------------------------------------------------------------
struct TravArgs {
    NodeArrays nd;
    const float4 *sbody;
    const double *bx, *by, *bz;  // the f64 state, unsorted (body order[k] is sorted body k)
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
    // accuracy options (not reference behaviour): quadrupole correction of
    // accepted cells, and a centre-of-mass guard that also requires
    // b_max < com_theta * |x - c| (b_max = sqrt(3) extent + |c - centre|
    // bounds the distance of the cell's bodies from c); 0 disables it.
    int quad;
    float com_theta;
    // pair-law scale (PairScale in engine.h), set on the device from the root
    // half-width X and the total mass M (the largest cell): bodies and cells
    // enter pair_acc / quad_acc at p 2^-sk with mass m 2^-skm, second moments
    // as S 2^-(2sk + skm), the easing as e 2^-2sk (es), and the sums leave
    // multiplied by 2^(skm - 2sk); opening tests use unscaled positions
    int sk, skm;
    float sc, msc, es;
};

__device__ __forceinline__ float load_extent(const TravArgs &a)
{
    return (float)__longlong_as_double((long long)*a.extent_bits);
}

__device__ __forceinline__ void set_pair_scale(TravArgs &a)
{
    a.sk = pair_scale_exp(a.extent, a.e);
    a.skm = mass_scale_exp(a.n > 0 ? a.nd.com[0].w : 0.f);  // root: the total mass
    a.sc = pow2f(-a.sk);
    a.msc = pow2f(-a.skm);
    a.es = a.e * pow2f(-2 * a.sk);
}

// (x, y, z, m) scaled by sc and msc
__device__ __forceinline__ float4 scaled(float4 p, float sc, float msc)
{
    return make_float4(p.x * sc, p.y * sc, p.z * sc, p.w * msc);
}

// second moments scaled by f = sc^2 msc
__device__ __forceinline__ float4 scaled2(float4 q, float f)
{
    return make_float4(q.x * f, q.y * f, q.z * f, q.w * f);
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
    const uint32_t i = a.order[k];
    const double d0 = a.bx[i] - a.nd.c64[node];
    const double d1 = a.by[i] - a.nd.c64[cap + node];
    const double d2 = a.bz[i] - a.nd.c64[2 * cap + node];
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

// Quadrupole correction of a cell with centre of mass c and second moments S
// (about c) for the reference's law a = sum m d / (|d| (|d|^2 + e)):
// expanding d g(|d|), g(r) = 1/(r (r^2 + e)), to second order about c gives
//   a_2 = h S D + (h tr S + h' / r  D.S.D) D / 2,  D = c - x,
// h = g'(r)/r = -A / (r u^2), h'/r = (-6 + A (1/r^2 + 2 A / (u r))) / (r u^2),
// u = r (r^2 + e), A = 3 r^2 + e (e = 0 gives the Newtonian -3/r^5, 15/r^7).
__device__ __forceinline__ void quad_acc(float qx, float qy, float qz, float4 c, float4 qa,
                                         float4 qb, float e, float &ax, float &ay, float &az)
{
    const float dx = c.x - qx, dy = c.y - qy, dz = c.z - qz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (!(r2 > 1e-30f)) return;
    const float ir = rsqrt_approx(r2);
    const float iu = ir * __fdividef(1.f, r2 + e);
    const float A = fmaf(3.f, r2, e);
    const float base = ir * iu * iu;
    const float h = -A * base;
    const float hp = base * fmaf(A, fmaf(2.f * A, iu * ir, ir * ir), -6.f);
    const float sdx = fmaf(qa.x, dx, fmaf(qb.x, dy, qb.y * dz));
    const float sdy = fmaf(qb.x, dx, fmaf(qa.y, dy, qb.z * dz));
    const float sdz = fmaf(qb.y, dx, fmaf(qb.z, dy, qa.z * dz));
    const float dsd = fmaf(dx, sdx, fmaf(dy, sdy, dz * sdz));
    const float k = 0.5f * fmaf(h, qa.w, hp * dsd);
    ax = fmaf(h, sdx, fmaf(k, dx, ax));
    ay = fmaf(h, sdy, fmaf(k, dy, ay));
    az = fmaf(h, sdz, fmaf(k, dz, az));
}

// Monopole + quadrupole terms of two accepted cells for one body (nq =
// -position), the cells' (x, y, z, m) and second moments given as float2
// planes, through packed FP32 instructions.  Per lane the monopole and the
// quadrupole share one reciprocal square root: 1/sqrt(r^2 (r^2 + e)^2) = 1/u
// and 1/r = (r^2 + e)/u; the quadrupole term is that of quad_acc.
__device__ __forceinline__ void cell_quad_acc2(float2 nqx, float2 nqy, float2 nqz, float2 cx,
                                               float2 cy, float2 cz, float2 cm, float2 qax,
                                               float2 qay, float2 qaz, float2 qaw, float2 qbx,
                                               float2 qby, float2 qbz, float2 e2, float2 &ax,
                                               float2 &ay, float2 &az)
{
    const float2 dx = add2(cx, nqx), dy = add2(cy, nqy), dz = add2(cz, nqz);
    float2 r2 = mul2(dz, dz);
    r2 = fma2(dy, dy, r2);
    r2 = fma2(dx, dx, r2);
    const float2 w = add2(r2, e2);
    const float2 arg = fma2(r2, mul2(w, w), make_float2(kPairGuard, kPairGuard));
    const float2 iu = make_float2(rsqrt_approx(arg.x), rsqrt_approx(arg.y));
    const float2 s = mul2(cm, iu);
    float2 ir = mul2(iu, w);
    ir.x = r2.x > 1e-30f ? ir.x : 0.f;  // no quadrupole term at r = 0
    ir.y = r2.y > 1e-30f ? ir.y : 0.f;
    const float2 A = fma2(make_float2(3.f, 3.f), r2, e2);
    const float2 base = mul2(mul2(ir, iu), iu);
    const float2 h = mul2(make_float2(-A.x, -A.y), base);
    const float2 hp =
        mul2(base, fma2(A, fma2(mul2(make_float2(2.f, 2.f), A), mul2(iu, ir), mul2(ir, ir)),
                        make_float2(-6.f, -6.f)));
    const float2 sdx = fma2(qax, dx, fma2(qbx, dy, mul2(qby, dz)));
    const float2 sdy = fma2(qbx, dx, fma2(qay, dy, mul2(qbz, dz)));
    const float2 sdz = fma2(qby, dx, fma2(qbz, dy, mul2(qaz, dz)));
    const float2 dsd = fma2(dx, sdx, fma2(dy, sdy, mul2(dz, sdz)));
    const float2 k = fma2(make_float2(0.5f, 0.5f), fma2(h, qaw, mul2(hp, dsd)), s);
    ax = fma2(h, sdx, fma2(k, dx, ax));
    ay = fma2(h, sdy, fma2(k, dy, ay));
    az = fma2(h, sdz, fma2(k, dz, az));
}

// The centre-of-mass guard for one body: b_max < com_theta |x - c|.
__device__ __forceinline__ bool com_guard(const TravArgs &a, float4 geo, float4 c, float qx,
                                          float qy, float qz)
{
    if (a.com_theta <= 0.f) return true;
    const float ox = c.x - geo.x, oy = c.y - geo.y, oz = c.z - geo.z;
    const float bmax = fmaf(1.7320509f, geo.w, sqrtf(fmaf(ox, ox, fmaf(oy, oy, oz * oz))));
    const float dx = c.x - qx, dy = c.y - qy, dz = c.z - qz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    return bmax * bmax < a.com_theta * a.com_theta * r2;
}

// Two interactions of one body (nq = -position, both lanes) with sources
// (x, y, z, m) given as float2 planes, through packed FP32 instructions; the
// arithmetic of each lane is that of pair_acc.
__device__ __forceinline__ void pair_acc2(float2 nqx, float2 nqy, float2 nqz, float2 x, float2 y,
                                          float2 z, float2 m, float2 e2, float2 &ax, float2 &ay,
                                          float2 &az)
{
    const float2 dx = add2(x, nqx), dy = add2(y, nqy), dz = add2(z, nqz);
    float2 r2 = mul2(dz, dz);
    r2 = fma2(dy, dy, r2);
    r2 = fma2(dx, dx, r2);
    const float2 w = add2(r2, e2);
    const float2 q = fma2(r2, mul2(w, w), make_float2(kPairGuard, kPairGuard));
    const float2 s = mul2(m, make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y)));
    ax = fma2(dx, s, ax);
    ay = fma2(dy, s, ay);
    az = fma2(dz, s, az);
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
    __shared__ float4 child_geo[kTravWarps][8];  // the children being tested
    __shared__ int4 child_meta[kTravWarps][8];
    // a failed sort left no tree to walk (the node arrays may hold anything)
    if (sort_failed(a_in.flags)) return;
    TravArgs a = a_in;
    a.extent = load_extent(a_in);
    set_pair_scale(a);
    const float sc2 = a.sc * a.sc * a.msc;
    unsigned long long visits = 0, pairs = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k0 = (blockIdx.x * kTravWarps + warp) * 32;
    if (k0 >= a.n) return;
    const int k = k0 + lane;
    const bool valid = k < a.n;
    const uint32_t active = __ballot_sync(0xffffffffu, valid);
    const float4 q = valid ? a.sbody[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 qs = scaled(q, a.sc, a.msc);
    float ax = 0.f, ay = 0.f, az = 0.f, hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
    int sp = 0;
    int since_fold = 0;
    bool overflow = false;
    // Tests cell `node` (geometry `geo`, record `meta`) for the lanes of
    // `mask`, each with the reference's own opening rule for its body:
    // accepted lanes take the cell's monopole (and quadrupole); the lanes that
    // open a leaf take its bodies here; an internal cell opened by any lane
    // goes on the stack with those lanes, to have its children tested.
    auto visit = [&](int node, uint32_t mask, float4 geo, int4 meta) {
        const bool in = (mask >> lane) & 1u;
        bool acc = false;
        if (in) {
            acc = accept_cell(a, node, geo, q.x, q.y, q.z, k);
            if (acc && a.com_theta > 0.f) acc = com_guard(a, geo, a.nd.com[node], q.x, q.y, q.z);
        }
        const uint32_t open = mask & ~__ballot_sync(0xffffffffu, acc);
        ++visits;
        if (acc) {
            const float4 cm = scaled(a.nd.com[node], a.sc, a.msc);
            pair_acc(qs.x, qs.y, qs.z, cm, a.es, ax, ay, az);
            if (a.quad)
                quad_acc(qs.x, qs.y, qs.z, cm, scaled2(a.nd.quad_a[node], sc2),
                         scaled2(a.nd.quad_b[node], sc2), a.es, ax, ay, az);
            ++pairs;
        }
        ++since_fold;
        if (!open) return;
        if (meta.y < 0) {
            const int b = meta.z, c = meta.w;
            const bool mine = (open >> lane) & 1u;
            for (int j = b; j < b + c; ++j) {
                const float4 bj = scaled(a.sbody[j], a.sc, a.msc);
                if (mine) pair_acc(qs.x, qs.y, qs.z, bj, a.es, ax, ay, az);
            }
            if (mine) pairs += c;
            since_fold += c;
        } else if (sp < kStack) {
            if (lane == 0) stack[warp][sp] = {node, open};
            ++sp;
        } else {
            overflow = true;
        }
        if (since_fold >= 64) {
            fold(hx, lx, ax);
            fold(hy, ly, ay);
            fold(hz, lz, az);
            since_fold = 0;
        }
    };
    visit(0, active, a.nd.geo[0], a.nd.meta[0]);
    while (sp > 0 && !overflow) {
        __syncwarp();
        const StackEntry top = stack[warp][sp - 1];
        --sp;
        __syncwarp();
        const int4 pm = a.nd.meta[top.node];
        const int fc = pm.y, nc = (int)((uint32_t)pm.x >> 28);
        // the children's records, one lane each, loaded together
        if (lane < nc) {
            child_geo[warp][lane] = a.nd.geo[fc + lane];
            child_meta[warp][lane] = a.nd.meta[fc + lane];
        }
        __syncwarp();
        // last child first, as the reference pops them (octree.rs:152-154)
#pragma unroll 1
        for (int c = nc - 1; c >= 0; --c)
            visit(fc + c, top.mask, child_geo[warp][c], child_meta[warp][c]);
    }
    if (overflow && lane == 0) atomicOr(&a.flags[kFlagStack], 1u);
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
        const double unsc = pow2d(a.skm - 2 * a.sk);
        a.partial[i] = ((double)hx + (double)lx) * unsc;
        a.partial[a.n + i] = ((double)hy + (double)ly) * unsc;
        a.partial[2 * (size_t)a.n + i] = ((double)hz + (double)lz) * unsc;
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

// kQuad: quadrupole corrections of accepted cells (the quadrupole tiles are
// only sized in that instantiation, so the monopole kernel keeps its
// registers and occupancy).
template <bool kQuad>
__global__ void __launch_bounds__(kTravWarps * 32)
traverse_warp_kernel(TravArgs a_in)
{
    __shared__ int32_t gstack[kTravWarps][kGStack];
    __shared__ int32_t queue[kTravWarps][kGQueue];
    __shared__ float4 tile[kTravWarps][32];
    __shared__ float4 tqa[kQuad ? kTravWarps : 1][32];
    __shared__ float4 tqb[kQuad ? kTravWarps : 1][32];
    // a failed sort left no tree to walk (the node arrays may hold anything)
    if (sort_failed(a_in.flags)) return;
    TravArgs a = a_in;
    a.extent = load_extent(a_in);
    set_pair_scale(a);
    const float sc = a.sc, msc = a.msc, sc2 = a.sc * a.sc * a.msc;
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
    // Bodies are queued from the front of the queue, accepted cells from the
    // back, so each is evaluated by its own loop: plain pairs for bodies,
    // pair + quadrupole (kQuad) for cells.
    int nc = 0;  // queued cells
    const float2 nqx = make_float2(-q.x * sc, -q.x * sc), nqy = make_float2(-q.y * sc, -q.y * sc);
    const float2 nqz = make_float2(-q.z * sc, -q.z * sc), e2 = make_float2(a.es, a.es);
    // Evaluates `count` queued interactions whose (x, y, z, m) load(t) gives:
    // entries 2k and 2k + 1 are staged interleaved as (x, x', y, y')(z, z', m, m'),
    // so two 128-bit loads give the float2 operands of two interactions, which go
    // through packed FADD2/FMUL2/FFMA2 (an odd count is padded with a massless
    // entry, which adds exactly zero); the next tile is loaded while the current
    // one is evaluated.
    auto eval_packed = [&](int count, auto load) {
        float4 nb = make_float4(0.f, 0.f, 0.f, 0.f);
        if (lane < count) nb = load(lane);
        for (int j0 = 0; j0 < count; j0 += 32) {
            const int m = min(32, count - j0);
            __syncwarp();
            const float4 bj = nb;
            nb = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j0 + 32 + lane < count) nb = load(j0 + 32 + lane);
            float *pl = reinterpret_cast<float *>(&tile[warp][lane & ~1]) + (lane & 1);
            pl[0] = bj.x * sc;
            pl[2] = bj.y * sc;
            pl[4] = bj.z * sc;
            pl[6] = bj.w * msc;
            __syncwarp();
            float2 sx = make_float2(0.f, 0.f), sy = sx, sz = sx;
            for (int jj = 0; jj < (m + 1) >> 1; ++jj) {
                const float4 A = tile[warp][2 * jj], B = tile[warp][2 * jj + 1];
                pair_acc2(nqx, nqy, nqz, make_float2(A.x, A.y), make_float2(A.z, A.w),
                          make_float2(B.x, B.y), make_float2(B.z, B.w), e2, sx, sy, sz);
            }
            ax += sx.x + sx.y;
            ay += sy.x + sy.y;
            az += sz.x + sz.y;
        }
    };
    auto flush = [&]() {
        // leaf bodies, then accepted cells (monopoles packed like bodies;
        // with quadrupoles one cell per lane step)
        eval_packed(nq, [&](int t) { return a.sbody[queue[warp][t]]; });
        if (!kQuad) {
            eval_packed(nc, [&](int t) { return a.nd.com[-queue[warp][kGQueue - 1 - t] - 1]; });
        } else {
            // cells with quadrupoles, two per packed instruction: centre of
            // mass and both moment vectors staged interleaved like bodies
            for (int j0 = 0; j0 < nc; j0 += 32) {
                const int m = min(32, nc - j0);
                __syncwarp();
                float4 c4 = make_float4(0.f, 0.f, 0.f, 0.f), qa = c4, qb = c4;
                if (lane < m) {
                    const int c = -queue[warp][kGQueue - 1 - (j0 + lane)] - 1;
                    c4 = scaled(a.nd.com[c], sc, msc);
                    qa = scaled2(a.nd.quad_a[c], sc2);
                    qb = scaled2(a.nd.quad_b[c], sc2);
                }
                const int slot = lane & ~1, half = lane & 1;
                float *pc = reinterpret_cast<float *>(&tile[warp][slot]) + half;
                float *pa = reinterpret_cast<float *>(&tqa[warp][slot]) + half;
                float *pb = reinterpret_cast<float *>(&tqb[warp][slot]) + half;
                pc[0] = c4.x; pc[2] = c4.y; pc[4] = c4.z; pc[6] = c4.w;
                pa[0] = qa.x; pa[2] = qa.y; pa[4] = qa.z; pa[6] = qa.w;
                pb[0] = qb.x; pb[2] = qb.y; pb[4] = qb.z; pb[6] = qb.w;
                __syncwarp();
                float2 sx = make_float2(0.f, 0.f), sy = sx, sz = sx;
                for (int jj = 0; jj < (m + 1) >> 1; ++jj) {
                    const float4 C0 = tile[warp][2 * jj], C1 = tile[warp][2 * jj + 1];
                    const float4 A0 = tqa[warp][2 * jj], A1 = tqa[warp][2 * jj + 1];
                    const float4 B0 = tqb[warp][2 * jj], B1 = tqb[warp][2 * jj + 1];
                    cell_quad_acc2(nqx, nqy, nqz, make_float2(C0.x, C0.y), make_float2(C0.z, C0.w),
                                   make_float2(C1.x, C1.y), make_float2(C1.z, C1.w),
                                   make_float2(A0.x, A0.y), make_float2(A0.z, A0.w),
                                   make_float2(A1.x, A1.y), make_float2(A1.z, A1.w),
                                   make_float2(B0.x, B0.y), make_float2(B0.z, B0.w),
                                   make_float2(B1.x, B1.y), e2, sx, sy, sz);
                }
                ax += sx.x + sx.y;
                ay += sy.x + sy.y;
                az += sz.x + sz.y;
            }
        }
        pairs += nq + nc;
        fold(hx, lx, ax);
        fold(hy, ly, ay);
        fold(hz, lz, az);
        nq = 0;
        nc = 0;
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
            if (acc && a.com_theta > 0.f) {
                // centre-of-mass guard against the whole box (distance from c
                // to the box is a lower bound of every body's |x - c|)
                const float4 cm = a.nd.com[cell];
                const float ox = cm.x - geo.x, oy = cm.y - geo.y, oz = cm.z - geo.z;
                const float bmax =
                    fmaf(1.7320509f, geo.w, sqrtf(fmaf(ox, ox, fmaf(oy, oy, oz * oz))));
                const float ex = fmaxf(fmaxf(lo_x - cm.x, cm.x - hi_x), 0.f);
                const float ey = fmaxf(fmaxf(lo_y - cm.y, cm.y - hi_y), 0.f);
                const float ez = fmaxf(fmaxf(lo_z - cm.z, cm.z - hi_z), 0.f);
                const float rc2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                acc = bmax * bmax < a.com_theta * a.com_theta * rc2;
            }
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
            bool ok = !valid || (rl > 0.f && gw * (1.f + 2e-6f) < theta * rl);
            if (a.com_theta > 0.f) {
                const int src_cell = __shfl_sync(0xffffffffu, cell, src);
                const float4 c4 = a.nd.com[src_cell];
                ok = ok && (!valid || com_guard(a, make_float4(gx, gy, gz, gw), c4, q.x, q.y, q.z));
            }
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
        // queue leaf bodies (front) and cells (back), at most 16 entries per
        // lane per round
        while (__any_sync(0xffffffffu, qcnt > 0)) {
            const int take = min(qcnt, 16);
            const bool is_cell = qref < 0;
            int btotal, ctotal;
            const int boff = warp_exclusive_scan(is_cell ? 0 : take, lane, btotal);
            const int coff = warp_exclusive_scan(is_cell ? take : 0, lane, ctotal);
            if (nq + nc + btotal + ctotal > kGQueue) flush();
            if (is_cell) {
                if (take) queue[warp][kGQueue - 1 - (nc + coff)] = qref;
            } else {
                for (int j = 0; j < take; ++j) queue[warp][nq + boff + j] = qref + j;
                qref += take;
            }
            qcnt -= take;
            nq += btotal;
            nc += ctotal;
        }
        __syncwarp();
        if (nq + nc >= 256) flush();
    }
    flush();
    if (lane == 0) {
        if (overflow) atomicOr(&a.flags[kFlagStack], 1u);
        atomicAdd(&a.stats[0], visits);
        atomicAdd(&a.stats[1], pairs * (unsigned long long)nvalid);
    }
    if (valid) {
        const uint32_t i = a.order[k];
        const double unsc = pow2d(a.skm - 2 * a.sk);
        a.partial[i] = ((double)hx + (double)lx) * unsc;
        a.partial[a.n + i] = ((double)hy + (double)ly) * unsc;
        a.partial[2 * (size_t)a.n + i] = ((double)hz + (double)lz) * unsc;
    }
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
// workspace + host driver
// ---------------------------------------------------------------------------
namespace {
// per device: the sort's kernel attributes are set, and how many blocks of the
// single-launch sort an SM holds (0 = one launch per pass)
std::atomic<bool> g_sort_ready[64];
std::atomic<int> g_sort_coop_per_sm[64];
}  // namespace

struct BhWorkspace {
    int device = 0;
    cudaStream_t stream = nullptr;  // allocations and frees are ordered on it
    size_t cap_n = 0;
    uint64_t *keys[2] = {nullptr, nullptr};
    uint32_t *vals[2] = {nullptr, nullptr};
    // sort_meta: digit histograms of the passes, then the passes' tile
    // counters, the epoch and the single-launch sort's grid barrier;
    // sort_status: look-back words, tiles x digits
    uint32_t *sort_meta = nullptr;
    unsigned long long *sort_status = nullptr;
    float4 *sbody = nullptr;
    uint8_t *lcp = nullptr;        // L(k): leading digits keys[k-1] and keys[k] share
    uint32_t *mask = nullptr;      // level mask of each sorted body
    uint8_t *leafcnt = nullptr;    // bodies of the leaf starting at each sorted body
    uint32_t *blk_cnt = nullptr;   // per level and tree block: nodes starting in it
    uint32_t *blk_off = nullptr;   // ... and the level's nodes before the block
    uint32_t *nchild32 = nullptr;  // children of each node (counted by the node kernel)
    NodeArrays nd = {};
    LevelInfo *lv = nullptr;
    unsigned long long *extent_bits = nullptr;
    unsigned long long *stats = nullptr;  // node visits, pair interactions of the last traversal
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
    void *p[] = {ws->keys[0],     ws->keys[1],    ws->vals[0],    ws->vals[1],
                 ws->sort_meta,   ws->sort_status, ws->sbody,     ws->lcp,
                 ws->mask,        ws->leafcnt,    ws->blk_cnt,    ws->blk_off,
                 ws->nchild32,    ws->nd.msum_hi, ws->nd.msum_lo, ws->nd.begin,
                 ws->nd.count,    ws->nd.child,   ws->nd.nchild,  ws->nd.level,
                 ws->nd.c64,      ws->nd.geo,     ws->nd.com,     ws->lv,
                 ws->extent_bits, ws->flags,      ws->nd.meta,    ws->stats,
                 ws->nd.parent,   ws->nd.quad_a,  ws->nd.quad_b,  ws->nd.arrivals};
    for (void *q : p) dev_free(q, ws->stream);
}

template <typename T>
static int wsalloc(T *&p, size_t count, cudaStream_t st)
{
    return dev_alloc(p, count, st);
}

int bh_reserve(BhWorkspace *&ws, size_t n, int device, int leaf, cudaStream_t stream)
{
    leaf = leaf < 1 ? 1 : leaf;
    if (ws && n <= ws->cap_n && leaf >= ws->leaf_min) return PHYSIM_OK;
    if (ws) {
        ws_release(ws);
        delete ws;
        ws = nullptr;
    }
    // the radix sort stages its tile in 96 KB of dynamic shared memory; set
    // once per device, here (never inside a stream capture), with the number
    // of single-launch sort blocks an SM holds (0: no cooperative launch)
    if (device >= 0 && device < 64 && !g_sort_ready[device].load()) {
        PG_CUDA(cudaFuncSetAttribute(radix_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSortSmem));
        PG_CUDA(cudaFuncSetAttribute(radix_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSortSmem));
        int coop = 0, per_sm = 0;
        PG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
        if (coop)
            PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, radix_sort_kernel,
                                                                  kSortThreads, kSortSmem));
        g_sort_coop_per_sm[device].store(per_sm);
        g_sort_ready[device].store(true);
    }
    BhWorkspace *w = new (std::nothrow) BhWorkspace();
    PG_CHECK(w, PHYSIM_ERR_MEMORY, "out of host memory");
    w->device = device;
    w->stream = stream;
    const size_t cap = n < 64 ? 64 : n;
    w->cap_n = cap;
    const int tiles = cdiv((long long)cap, kSortTile);
    const size_t tree_blocks = (size_t)cdiv((long long)cap, kTreeBlock);
    // Node capacity: leaves hold about leaf/4 bodies on average, so 8N/leaf
    // (at most 4N) nodes hold every non-degenerate distribution; deeper
    // chains only leave levels unsplit (exact, slower) and raise a flag.
    const size_t ncap = std::min<size_t>(4 * cap, 8 * cap / (size_t)leaf) + 4096 + 64 * kMaxLevels;
    w->leaf_min = leaf;
    int rc = PHYSIM_OK;
#define PG_WA(ptr, cnt)                                                                     \
    if (rc == PHYSIM_OK) rc = wsalloc(ptr, cnt, stream)
    PG_WA(w->keys[0], cap);
    PG_WA(w->keys[1], cap);
    PG_WA(w->vals[0], cap);
    PG_WA(w->vals[1], cap);
    PG_WA(w->sort_meta, (size_t)kSortPasses * kRadixBuckets + kSortPasses + 2);
    PG_WA(w->sort_status, (size_t)kRadixBuckets * tiles);
    PG_WA(w->sbody, cap);
    PG_WA(w->lcp, cap);
    PG_WA(w->mask, cap);
    PG_WA(w->leafcnt, cap);
    PG_WA(w->blk_cnt, 32 * tree_blocks);
    PG_WA(w->blk_off, 32 * tree_blocks);
    PG_WA(w->nchild32, ncap);
    PG_WA(w->nd.begin, ncap);
    PG_WA(w->nd.count, ncap);
    PG_WA(w->nd.child, ncap);
    PG_WA(w->nd.nchild, ncap);
    PG_WA(w->nd.level, ncap);
    PG_WA(w->nd.c64, 4 * ncap);
    PG_WA(w->nd.geo, ncap);
    PG_WA(w->nd.com, ncap);
    PG_WA(w->nd.meta, ncap);
    PG_WA(w->nd.parent, ncap);
    PG_WA(w->nd.msum_hi, ncap);
    PG_WA(w->nd.msum_lo, ncap);
    PG_WA(w->nd.quad_a, ncap);
    PG_WA(w->nd.quad_b, ncap);
    PG_WA(w->nd.arrivals, ncap);
    PG_WA(w->stats, 4);
    PG_WA(w->lv, 1);
    PG_WA(w->extent_bits, 1);
    PG_WA(w->flags, 4);
#undef PG_WA
    w->nd.cap = (int)ncap;
    if (rc == PHYSIM_OK &&
        (cudaMemsetAsync(w->flags, 0, 4 * sizeof(uint32_t), stream) != cudaSuccess ||
         cudaMemsetAsync(w->nd.arrivals, 0, ncap * sizeof(uint32_t), stream) != cudaSuccess ||
         cudaMemsetAsync(w->lv, 0, sizeof(LevelInfo), stream) != cudaSuccess ||
         cudaMemsetAsync(w->sort_meta, 0,
                         ((size_t)kSortPasses * kRadixBuckets + kSortPasses + 2) * sizeof(uint32_t),
                         stream) != cudaSuccess ||
         cudaMemsetAsync(w->sort_status, 0,
                         (size_t)kRadixBuckets * tiles * sizeof(unsigned long long),
                         stream) != cudaSuccess))
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

int bh_check(BhWorkspace *ws, cudaStream_t st)
{
    if (!ws) return PHYSIM_OK;
    uint32_t f[4];
    PG_CUDA(cudaMemcpyAsync(f, ws->flags, sizeof f, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    if (f[kFlagStack] == 0 && f[kFlagSort] == 0) return PHYSIM_OK;
    PG_CUDA(cudaMemsetAsync(ws->flags + kFlagStack, 0, 2 * sizeof(uint32_t), st));
    PG_CUDA(cudaStreamSynchronize(st));
    if (f[kFlagSort]) {
        set_error("Barnes-Hut build: a bounded wait (radix sort look-back or pass barrier, "
                  "or tree level) gave up; "
                  "results are invalid");
        return PHYSIM_ERR_TIMEOUT;
    }
    set_error("Barnes-Hut traversal stack overflow; results are invalid");
    return PHYSIM_ERR_TREE;
}

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

namespace {
std::atomic<uint32_t> g_wait_limit{0};  // 0: kLookbackSpins
std::atomic<int32_t> g_stall_tile{-1};
std::atomic<int> g_sort_single{1};
int wait_limit()
{
    const uint32_t v = g_wait_limit.load();
    return v == 0u ? kLookbackSpins : (int)std::min<uint32_t>(v, (uint32_t)INT32_MAX);
}
}  // namespace

static int bh_build(BhWorkspace *ws, const DeviceBodies &b, const BhParams &p, cudaStream_t st)
{
    const int n = (int)b.n;
    int launches = 0;
    PG_CUDA(cudaMemsetAsync(ws->extent_bits, 0, sizeof(unsigned long long), st));
    const int sms = device_sm_count(ws->device);
    extent_kernel<<<sms * 2, 256, 0, st>>>(b.x, b.y, b.z, n, ws->extent_bits);
    uint32_t *ghist = ws->sort_meta;
    uint32_t *tile_ctr = ws->sort_meta + kSortPasses * kRadixBuckets;
    uint32_t *epoch = tile_ctr + kSortPasses;
    uint32_t *sort_bar = epoch + 1;
    PG_CUDA(cudaMemsetAsync(ghist, 0, kSortPasses * kRadixBuckets * sizeof(uint32_t), st));
    keys_kernel<<<std::min(cdiv(n, 256), sms * 8), 256, 0, st>>>(
        b.x, b.y, b.z, n, p.nchild, ws->extent_bits, ws->keys[0], ws->vals[0], ghist, tile_ctr,
        epoch, sort_bar);
    launches += 2;
    // one-sweep radix sort over 9-bit digits: all passes in one cooperative
    // launch where the device allows it, else one launch per pass
    const int tiles = cdiv(n, kSortTile);
    const int per_sm = ws->device >= 0 && ws->device < 64 ? g_sort_coop_per_sm[ws->device].load() : 0;
    int cur = 0;
    if (g_sort_single.load() && per_sm > 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)std::min(tiles, per_sm * sms));
        cfg.blockDim = dim3(kSortThreads);
        cfg.dynamicSmemBytes = kSortSmem;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        PG_CUDA(cudaLaunchKernelEx(&cfg, radix_sort_kernel, ws->keys[0], ws->vals[0], ws->keys[1],
                                   ws->vals[1], n, (const uint32_t *)ghist, ws->sort_status,
                                   (const uint32_t *)epoch, ws->flags, wait_limit(),
                                   (int)g_stall_tile.load(), sort_bar));
        cur = kSortPasses & 1;
        launches += 1;
    } else {
        for (int pass = 0; pass < kSortPasses; ++pass) {
            radix_pass_kernel<<<tiles, kSortThreads, kSortSmem, st>>>(
                ws->keys[cur], pass == 0 ? nullptr : ws->vals[cur], ws->keys[cur ^ 1],
                ws->vals[cur ^ 1], n, pass, ghist, tile_ctr, ws->sort_status, epoch, ws->flags,
                wait_limit(), g_stall_tile.load());
            cur ^= 1;
            launches += 1;
        }
    }
    ws->sorted = cur;
    // the tree: boundaries (+ sorted f32 bodies), level masks, one scan, node
    // records, centres, moments
    boundary_kernel<<<cdiv(n, 256), 256, 0, st>>>(ws->keys[cur], ws->vals[cur], n, p.nchild,
                                                  b.body4, ws->sbody, ws->lcp, ws->flags);
    const int tree_blocks = cdiv(n, kTreeBlock);
    PG_CHECK(p.leaf_size >= 1 && p.leaf_size <= kMaxLeaf, PHYSIM_ERR_ARGUMENT,
             "leaf size %d outside 1..%d", p.leaf_size, kMaxLeaf);
    mask_kernel<<<tree_blocks, kTreeBlock, 0, st>>>(ws->keys[cur], ws->lcp, n, p.nchild,
                                                    p.leaf_size, ws->mask, ws->blk_cnt,
                                                    tree_blocks, ws->leafcnt, ws->nchild32,
                                                    ws->nd.cap, ws->flags);
    level_scan_kernel<<<1, 1024, 0, st>>>(ws->blk_cnt, tree_blocks, p.nchild, ws->blk_off, ws->lv,
                                          ws->nd.cap, ws->flags);
    node_kernel<<<tree_blocks, kTreeBlock, 0, st>>>(ws->keys[cur], ws->leafcnt, ws->mask,
                                                    ws->blk_off, tree_blocks, n, p.nchild, ws->nd,
                                                    ws->lv, ws->nchild32, ws->flags);
    centre_kernel<<<sms * 8, 256, 0, st>>>(ws->keys[cur], ws->nd, ws->lv, p.nchild,
                                           p.traversal == PHYSIM_TRAVERSAL_EXACT ? 1 : 0,
                                           ws->extent_bits, ws->flags);
    // one thread per node (the capacity bounds the count): a grid-stride loop
    // would queue a second leaf's climb behind the first's on one thread
    moments_kernel<<<cdiv(ws->nd.cap, 256), 256, 0, st>>>(
        ws->nd, ws->lv, ws->sbody, p.multipole == kMultipoleQuadrupole ? 1 : 0, ws->nchild32,
        ws->flags);
    launches += 6;
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
    a.bx = b.x;
    a.by = b.y;
    a.bz = b.z;
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
    a.quad = p.multipole == kMultipoleQuadrupole ? 1 : 0;
    a.com_theta = (float)p.com_theta;
    a.sk = a.skm = 0;  // set on the device (extent, total mass)
    a.sc = a.msc = 1.f;
    a.es = a.e;
    PG_CUDA(cudaMemsetAsync(ws->stats, 0, 2 * sizeof(unsigned long long), st));
    const int blocks = cdiv(cdiv(n, 32), kTravWarps);
    // external records, so they also time the kernel when replayed from a graph
    if (ws->profiling)
        PG_CUDA(cudaEventRecordWithFlags(ws->trav_ev[0], st, cudaEventRecordExternal));
    if (p.traversal == PHYSIM_TRAVERSAL_WARP && a.quad)
        traverse_warp_kernel<true><<<blocks, kTravWarps * 32, 0, st>>>(a);
    else if (p.traversal == PHYSIM_TRAVERSAL_WARP)
        traverse_warp_kernel<false><<<blocks, kTravWarps * 32, 0, st>>>(a);
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
    out->flags = flags[kFlagNodes] | (flags[kFlagStack] << 1) | (flags[kFlagSort] << 2);
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
    if (out->node_quad) {
        PG_TRY(cp(out->node_quad, ws->nd.quad_a, nn * sizeof(float4)));
        PG_TRY(cp(out->node_quad + 4 * nn, ws->nd.quad_b, nn * sizeof(float4)));
    }
    PG_CUDA(cudaStreamSynchronize(st));
    return PHYSIM_OK;
}

}  // namespace pg

extern "C" int physim_gpu_set_wait_limit(uint32_t polls)
{
    pg::g_wait_limit.store(polls);
    return PHYSIM_OK;
}

extern "C" int physim_gpu_set_sort_single_launch(int32_t on)
{
    pg::g_sort_single.store(on ? 1 : 0);
    return PHYSIM_OK;
}

extern "C" int physim_gpu_test_stall_sort(int32_t tile)
{
    pg::g_stall_tile.store(tile < 0 ? -1 : tile);
    return PHYSIM_OK;
}
