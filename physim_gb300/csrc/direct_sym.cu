// direct_sym.cu -- simple_astro pair forces with every unordered pair
// evaluated once (astro/src/transformers.rs:219-244, force law
// astro/src/lib.rs:84-113).
//
// The reference's force is antisymmetric: F_ji = -F_ij.  With
//     s_ij = 1 / sqrt(r^2 (r^2 + e)^2),   d = x_j - x_i,
// body i gains  m_j s_ij d  and body j gains  -m_i s_ij d  from one
// evaluation of d, r^2 and the reciprocal square root.  Per unordered pair
// that is 17 FP32 FMA-pipe operations (3 differences, 3 for r^2, 3 for the
// argument, m_j s and the 3-term update of a_i, -m_i s and the 3-term
// update of a_j) and one MUFU.RSQ, against 2 x 13 operations and 2 MUFU when
// each ordered pair is evaluated on its own.  The FMA pipe bounds the pair
// kernels, so this is up to 1.53x the interactions per second.
//
// Schedule.  Bodies form tiles of 1,024 (the body padding unit).  A block
// holds the 1,024 bodies of one tile I in registers (2 warps, 16 per thread,
// as 8 packed FFMA2 pairs); a warp takes the bodies of a tile J 32 at a
// time, one per lane, and rotates them through its lanes with shuffles:
// after 32 steps every lane's bodies have met all 32, and each travelling
// body's accumulated reaction is back at its home lane (sym_pair_core).  The
// diagonal tile pair (I, I) evaluates all ordered pairs of the tile and
// updates a_i only.
//
// Two schedules share that core.  With few tiles (one [3][n] f32 slot per
// tile fits in kSymPairsSlotBytes) every tile pair (I, J), I <= J, is one
// block (sym_tile_pair in direct_sym_tile.cuh): tile J's contribution to tile
// I goes to slot J, tile I's to tile J to slot I, and a reduce adds each
// body's T slots.  That keeps every SM busy at any size and is the faster of
// the two, but its slots grow as 12 T n bytes (12.9 GB at 1,048,580 bodies),
// so once they would exceed kSymPairsSlotBytes (4 GiB, about 600,000 bodies)
// the cluster schedule below takes over.
//
// Blocks work in thread-block clusters of kSymCluster (8) blocks: a cluster
// takes the I tiles g*8 .. g*8+7 (one per block) and a run of kSymRun (16) J
// tiles r*16 .. r*16+15, the pairs with I <= J.  A block's a_i accumulates
// over the whole run and is written once, to slot r of its tile's i-side
// slots: after each J tile a thread folds its register sums into its bodies'
// compensated (TwoSum) sums in shared memory (high part f32, low part bf16:
// the low part only carries rounding errors), so every tile's contribution
// is compensated as when each tile pair had a slot of its own.  A block's
// two warps add their reactions to tile J into one shared buffer; the
// cluster then adds its blocks' buffers (read through distributed shared
// memory, ranks in a fixed order, TwoSum-compensated, each block summing an
// eighth of the tile) and writes them once, to slot g of tile J's j-side
// slots.  Per cluster of up to 8 x 16 tile pairs that is 8 + 16 slot writes
// of 12 KB instead of 2 per tile pair.
// The cluster barrier is split: a block arrives when its reactions to tile
// J are in shared memory and waits for the others only after it has
// evaluated tile J + 1, so a block that is behind by up to a tile holds no
// other block up.  Three reaction buffers make that safe: the buffer of tile
// J + 1 was last read (for tile J - 2) before every block arrived for tile
// J - 1, which this block waited for before starting tile J + 1.  Every
// block of a cluster takes the same arrivals and waits (its run's length
// plus one), and a last arrive-and-wait keeps each block's shared memory
// alive until the others have read it.
// Cluster schedule output.  Tile K has Rn - floor(K / 16) i-side slots (the runs r whose last
// J tile is >= K) and floor(K / 8) + 1 j-side slots (the groups g with
// 8 g <= K), each [3][1024] f32, packed tile after tile (offsets in closed
// form, sym_iside_base / sym_jside_base): 1.2 GB at 1,048,580 bodies,
// against 12.9 GB for one slot per tile pair.  A second kernel sums each
// body's slots with compensated (TwoSum) arithmetic in a fixed order (i-side
// by run, then j-side by group) into the f64 partial-sum layout the
// integrators read (one split).  The result is deterministic, and the slot
// sums act as the per-tile compensation of the one-pair kernels.
#include <math.h>

#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <atomic>

#include "common.cuh"
#include "direct_sym_tile.cuh"
#include "engine.h"

namespace pg {

namespace cg = cooperative_groups;

namespace {

// The tile-pair schedule while its slot buffer (12 B per body per tile) fits
// in 4 GiB (up to about 600,000 bodies) or the physim_gpu_set_symmetric_pairs_limit.
constexpr size_t kSymPairsSlotBytes = size_t(4) << 30;
std::atomic<uint64_t> g_pairs_limit{0};

constexpr int kSymCluster = 8;  // I tiles per thread-block cluster (a portable size)
constexpr int kSymRun = 16;     // J tiles per run

// Slots of tile K (see the file comment), in units of one [3][1024] slot.
__host__ __device__ inline long long sym_iside_count(int K, int runs)
{
    return runs - K / kSymRun;
}

__host__ __device__ inline long long sym_iside_base(int K, int runs)
{
    const long long q = K / kSymRun, rem = K - q * kSymRun;
    return (long long)K * runs - (kSymRun * q * (q - 1) / 2 + q * rem);
}

__host__ __device__ inline long long sym_jside_base(int K)
{
    const long long q = K / kSymCluster, rem = K - q * kSymCluster;
    return (long long)K + kSymCluster * q * (q - 1) / 2 + q * rem;
}

constexpr int kSlot = 3 * kSymTile;  // floats per slot

// Clusters: I group g (tiles 8g .. 8g+7) with the J runs r >= floor(8g / 16).
__host__ __device__ inline long long sym_clusters(int T)
{
    const int groups = (T + kSymCluster - 1) / kSymCluster;
    const int runs = (T + kSymRun - 1) / kSymRun;
    long long c = 0;
    for (int g = 0; g < groups; ++g) c += runs - (g * kSymCluster) / kSymRun;
    return c;
}

// Dynamic shared memory of the pair kernel: three reaction buffers
// (jacc[3][1024][3] f32), then the compensated i-side sums of the run
// (hi[3][1024] f32, lo[3][1024] bf16): 54 KB, four blocks per SM.
constexpr int kSymBufs = 3;
constexpr size_t kSymJacc = (size_t)kSymBufs * kSymTile * 3;  // floats
constexpr size_t kSymSmem =
    kSymJacc * sizeof(float) + 3 * kSymTile * (sizeof(float) + sizeof(__nv_bfloat16));

// The cluster barrier in two halves (PTX barrier.cluster): arrive publishes
// this thread's earlier shared-memory writes to the cluster, wait returns
// once every thread of the cluster has arrived and makes their writes
// visible.  Arrivals and waits alternate.
__device__ __forceinline__ void cluster_arrive()
{
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}

__device__ __forceinline__ void cluster_wait()
{
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Tile J's reactions from this cluster's I tiles (those <= J): this block
// sums bodies rank*128 .. rank*128+127 over the ranks' buffers, in rank
// order with TwoSum, and writes them to slot g of tile J's j-side slots.
__device__ __forceinline__ void sym_reduce_tile(cg::cluster_group &cluster, int rank, int g,
                                                int J, int n, const float (*jw)[3],
                                                float *__restrict__ Pj)
{
    if (g * kSymCluster > J) return;  // no I tile of this cluster reaches tile J
    constexpr int per = kSymTile / kSymCluster;
    float *dst = Pj + (sym_jside_base(J) + g) * kSlot;
    const float *own = &jw[0][0];
    for (int t = threadIdx.x; t < per * 3; t += kSymThreads) {
        const int at = rank * per * 3 + t;  // = 3 jj + c
        float v[kSymCluster];
#pragma unroll
        for (int src = 0; src < kSymCluster; ++src) v[src] = cluster.map_shared_rank(own, src)[at];
        float hi = 0.f, lo = 0.f;
#pragma unroll
        for (int src = 0; src < kSymCluster; ++src) {
            float sum, err;
            two_sum(hi, v[src], sum, err);
            hi = sum;
            lo += err;
        }
        const int jj = at / 3, c = at - 3 * jj;
        if (J * kSymTile + jj < n) dst[c * kSymTile + jj] = hi + lo;
    }
}

// 64 threads of up to 255 registers (about 245 used), 54 KB of shared
// memory: four blocks per SM.
__global__ void __cluster_dims__(kSymCluster, 1, 1) __launch_bounds__(kSymThreads, 4)
direct_sym_kernel(const float4 *__restrict__ body, int n, int T, float e,
                  const PairScale *__restrict__ scale, float *__restrict__ Pi,
                  float *__restrict__ Pj)
{
    extern __shared__ float4 smem4[];
    float *smem = reinterpret_cast<float *>(smem4);
    float (*jacc)[kSymTile][3] = reinterpret_cast<float (*)[kSymTile][3]>(smem);
    float *ihi = smem + kSymJacc;
    __nv_bfloat16 *ilo = reinterpret_cast<__nv_bfloat16 *>(ihi + 3 * kSymTile);
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int runs = (T + kSymRun - 1) / kSymRun;
    // this cluster's (g, r)
    int u = (int)(blockIdx.x / kSymCluster), g = 0;
    for (;;) {
        const int c = runs - (g * kSymCluster) / kSymRun;
        if (u < c) break;
        u -= c;
        ++g;
    }
    const int r = (g * kSymCluster) / kSymRun + u;
    const int I = g * kSymCluster + rank;
    const int J0 = r * kSymRun, nJ = min(J0 + kSymRun, T) - J0;
    const bool have_i = I < T;
    const int warp = threadIdx.x >> 5;
    const int ib = warp * 32 + (threadIdx.x & 31);  // this thread's first body of tile I
    const int sk = scale->k, skm = scale->km;
    const float sc = pow2f(-sk), msc = pow2f(-skm);
    const float es = e * pow2f(-2 * sk);
    const float2 e2 = make_float2(es, es);
    float2 nx[kSymQ], ny[kSymQ], nz[kSymQ], nm[kSymQ], ax[kSymQ], ay[kSymQ], az[kSymQ];
#pragma unroll
    for (int q = 0; q < kSymQ; ++q) {
        ax[q] = ay[q] = az[q] = make_float2(0.f, 0.f);
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ihi[c * kSymTile + ib + (2 * q + h) * kSymThreads] = 0.f;
                ilo[c * kSymTile + ib + (2 * q + h) * kSymThreads] = __float2bfloat16_rn(0.f);
            }
    }
    if (have_i) sym_load_i(body, I, sc, msc, nx, ny, nz, nm);
    for (int t = 0; t < nJ; ++t) {
        const int J = J0 + t;
        float (*jw)[3] = jacc[t % kSymBufs];
        // free: every block has read it (tile J - 3) before arriving for tile J - 2
        for (int x = threadIdx.x; x < 3 * kSymTile; x += kSymThreads) (&jw[0][0])[x] = 0.f;
        __syncthreads();
        if (have_i && I < J)
            sym_pair_core<false, true>(body, J, sc, msc, e2, nx, ny, nz, nm, ax, ay, az, jw);
        else if (have_i && I == J)
            sym_pair_core<true>(body, J, sc, msc, e2, nx, ny, nz, nm, ax, ay, az, jw);
        if (have_i && I <= J) {
            // this tile's partial sums into the compensated run sums
#pragma unroll
            for (int q = 0; q < kSymQ; ++q) {
                const float v[2][3] = {{ax[q].x, ay[q].x, az[q].x}, {ax[q].y, ay[q].y, az[q].y}};
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const int at = c * kSymTile + ib + (2 * q + h) * kSymThreads;
                        float sum, err;
                        two_sum(ihi[at], v[h][c], sum, err);
                        ihi[at] = sum;
                        ilo[at] = __float2bfloat16_rn(__bfloat162float(ilo[at]) + err);
                    }
                ax[q] = ay[q] = az[q] = make_float2(0.f, 0.f);
            }
        }
        if (t > 0) {
            cluster_wait();  // every block's reactions to tile J - 1
            sym_reduce_tile(cluster, rank, g, J - 1, n, jacc[(t - 1) % kSymBufs], Pj);
        }
        cluster_arrive();  // this block's reactions to tile J
    }
    cluster_wait();
    sym_reduce_tile(cluster, rank, g, J0 + nJ - 1, n, jacc[(nJ - 1) % kSymBufs], Pj);
    if (have_i && J0 + nJ - 1 >= I) {
        // tile I's sums over the run: i-side slot r
        float *dst = Pi + (sym_iside_base(I, runs) + (r - I / kSymRun)) * kSlot;
#pragma unroll
        for (int q = 0; q < kSymQ; ++q)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int b = ib + (2 * q + h) * kSymThreads;
                if (I * kSymTile + b < n)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const int at = c * kSymTile + b;
                        dst[at] = ihi[at] + __bfloat162float(ilo[at]);
                    }
            }
    }
    // every block's shared memory stays until the others have read it
    cluster_arrive();
    cluster_wait();
}

// out[c*n + k] = the sum of body k's slots (i-side by run, then j-side by
// group), TwoSum-compensated f32, rounded once to f64 and unscaled
// (x 2^(km - 2k)).
__global__ void sym_reduce_kernel(const float *__restrict__ Pi, const float *__restrict__ Pj,
                                  int n, int T, const PairScale *__restrict__ scale,
                                  double *__restrict__ out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3ll * n) return;
    const int c = (int)(idx / n), k = (int)(idx - (long long)c * n);
    const int K = k / kSymTile, local = k - K * kSymTile;
    const int runs = (T + kSymRun - 1) / kSymRun;
    float hi = 0.f, lo = 0.f;
    const float *p = Pi + sym_iside_base(K, runs) * kSlot + c * kSymTile + local;
    const int ni = (int)sym_iside_count(K, runs);
    for (int t = 0; t < ni; ++t) {
        const float v = __ldcs(p + (size_t)t * kSlot);
        float s, err;
        two_sum(hi, v, s, err);
        hi = s;
        lo += err;
    }
    p = Pj + sym_jside_base(K) * kSlot + c * kSymTile + local;
    const int nj = K / kSymCluster + 1;
    for (int t = 0; t < nj; ++t) {
        const float v = __ldcs(p + (size_t)t * kSlot);
        float s, err;
        two_sum(hi, v, s, err);
        hi = s;
        lo += err;
    }
    out[idx] = ((double)hi + (double)lo) * pow2d(scale->km - 2 * scale->k);
}

// The tile-pair schedule: block u takes tile pair (I, J) (unit_tiles).
__global__ void __launch_bounds__(kSymThreads, 3)
direct_sym_pairs_kernel(const float4 *__restrict__ body, int n, float e,
                        const PairScale *__restrict__ scale, float *__restrict__ P)
{
    __shared__ float jacc[kSymWarps][kSymTile][3];
    int I, J;
    unit_tiles(blockIdx.x, I, J);
    const int sk = scale->k, skm = scale->km;
    if (I == J)
        sym_tile_pair<true>(body, n, I, J, e, sk, skm, P, jacc);
    else
        sym_tile_pair<false>(body, n, I, J, e, sk, skm, P, jacc);
}

// out[idx] = the sum of entry idx of the T slots P[t][3][n], in slot order,
// TwoSum-compensated, rounded once to f64 and unscaled (x 2^(km - 2k)).
__global__ void sym_pairs_reduce_kernel(const float *__restrict__ P, long long n3, int T,
                                        const PairScale *__restrict__ scale,
                                        double *__restrict__ out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n3) return;
    float hi = 0.f, lo = 0.f;
    const float *p = P + idx;
#pragma unroll 8
    for (int t = 0; t < T; ++t) {
        const float v = __ldcs(p + (size_t)t * n3);
        float s, err;
        two_sum(hi, v, s, err);
        hi = s;
        lo += err;
    }
    out[idx] = ((double)hi + (double)lo) * pow2d(scale->km - 2 * scale->k);
}

}  // namespace

DirectPlan make_symmetric_plan(int n)
{
    // 54 KB of dynamic shared memory per block, and the largest carveout to keep four
    // resident.  Set here, when a plan is made (never inside a stream capture), per device.
    static std::atomic<bool> attrs_set[64];
    int device = 0;
    if (cudaGetDevice(&device) == cudaSuccess && device >= 0 && device < 64 &&
        !attrs_set[device].load()) {
        if (cudaFuncSetAttribute(direct_sym_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kSymSmem) == cudaSuccess)
            attrs_set[device].store(true);
        else
            (void)cudaGetLastError();  // the launch then reports the error
        if (cudaFuncSetAttribute(direct_sym_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            (void)cudaGetLastError();  // a hint only: the kernel runs without it
        if (cudaFuncSetAttribute(direct_sym_pairs_kernel,
                                 cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            (void)cudaGetLastError();
    }
    DirectPlan p;
    p.symmetric = true;
    p.block = kSymThreads;
    p.ipt = kSymIpt;
    p.n = n;
    p.compensated = true;
    p.splits = 1;
    p.tiles = (int)(pad_bodies((size_t)n) / kSymTile);
    p.n_itiles = p.tiles;
    p.n_jtiles = p.tiles;
    p.chunk_tiles = p.tiles;
    const uint64_t limit = g_pairs_limit.load();
    p.clusters = (size_t)p.tiles * 12 * (size_t)(n > 0 ? n : 1) >
                 (limit ? (size_t)limit : kSymPairsSlotBytes);
    return p;
}

// f32 floats of the symmetric plan's i-side and j-side slots
static size_t sym_slot_floats(int T, size_t *jside_at)
{
    const int runs = (T + kSymRun - 1) / kSymRun;
    const size_t ni = (size_t)sym_iside_base(T, runs) * kSlot;
    const size_t nj = (size_t)sym_jside_base(T) * kSlot;
    if (jside_at) *jside_at = ni;
    return ni + nj;
}

size_t direct_partial_doubles(const DirectPlan &p)
{
    const size_t n3 = 3 * (size_t)(p.n > 0 ? p.n : 1);
    if (!p.symmetric) return (size_t)p.splits * n3;
    // f64 sums, then the f32 slots carved after them
    if (!p.clusters) return n3 + ((size_t)p.tiles * n3 + 1) / 2;
    return n3 + (sym_slot_floats(p.tiles, nullptr) + 1) / 2;
}

int launch_direct_symmetric(const DirectPlan &plan, const float4 *body4, float e,
                            const PairScale *scale, double *partial, cudaStream_t stream,
                            cudaEvent_t pairs_done)
{
    if (plan.n <= 0) return PHYSIM_OK;
    if (!plan.clusters) {
        const long long T = plan.tiles;
        const long long units = T * (T + 1) / 2;
        PG_CHECK(units < (1ll << 31), PHYSIM_ERR_ARGUMENT, "too many bodies for one pass: %d",
                 plan.n);
        const long long n3 = 3ll * plan.n;
        float *P = (float *)(partial + n3);
        direct_sym_pairs_kernel<<<(unsigned)units, kSymThreads, 0, stream>>>(body4, plan.n, e,
                                                                            scale, P);
        PG_CUDA(cudaGetLastError());
        if (pairs_done) PG_TRY(record_event(pairs_done, stream));
        sym_pairs_reduce_kernel<<<(unsigned)((n3 + 255) / 256), 256, 0, stream>>>(
            P, n3, (int)T, scale, partial);
        PG_CUDA(cudaGetLastError());
        return PHYSIM_OK;
    }
    const int T = plan.tiles;
    const long long blocks = sym_clusters(T) * kSymCluster;
    PG_CHECK(blocks < (1ll << 31), PHYSIM_ERR_ARGUMENT, "too many bodies for one pass: %d",
             plan.n);
    const long long n3 = 3ll * plan.n;
    size_t jside_at = 0;
    sym_slot_floats(T, &jside_at);
    float *Pi = (float *)(partial + n3);
    float *Pj = Pi + jside_at;
    direct_sym_kernel<<<(unsigned)blocks, kSymThreads, kSymSmem, stream>>>(body4, plan.n, T, e,
                                                                           scale, Pi, Pj);
    PG_CUDA(cudaGetLastError());
    if (pairs_done) PG_TRY(record_event(pairs_done, stream));
    sym_reduce_kernel<<<(unsigned)((n3 + 255) / 256), 256, 0, stream>>>(Pi, Pj, plan.n, T,
                                                                         scale, partial);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg

extern "C" int physim_gpu_set_symmetric_pairs_limit(uint64_t bytes)
{
    pg::g_pairs_limit.store(bytes);
    return PHYSIM_OK;
}
