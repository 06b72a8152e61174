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
// Schedule.  Bodies form tiles of 1,024 (the body padding unit); one block
// evaluates one tile pair (I, J), I <= J, of the T(T+1)/2.  Its 4 warps hold
// the 1,024 bodies of tile I in registers (8 per thread, as 4 packed FFMA2
// pairs).  A warp takes the bodies of tile J 32 at a time, one per lane, and
// rotates them through its lanes with shuffles: after 32 steps every lane's
// 8 bodies have met all 32, and each travelling body's accumulated reaction
// (a float2: the two halves of the packed pairs) is back at its home lane.
// a_i stays in registers for the whole tile; each warp writes its a_j sums
// for the tile to its own slice of shared memory, and the block adds the 4
// slices in a fixed order.  The diagonal tile pair (I, I) evaluates all
// ordered pairs of the tile and updates a_i only (a body meets itself with
// d = 0, which contributes 0 through the r^2 guard).
//
// Output.  Tile pair (I, J) writes the contribution of tile J to the bodies
// of tile I in slot J, and that of tile I to the bodies of tile J in slot I,
// of a buffer P[T][3][n] (f32): every (slot, body) entry is written exactly
// once per pass.  A second kernel sums the T slots of each body with
// compensated (TwoSum) arithmetic in a fixed order into the f64 partial-sum
// layout the integrators read (one split).  The result is deterministic, and
// the slot sums act as the per-tile compensation of the one-pair kernels.
#include <math.h>

#include <atomic>

#include "common.cuh"
#include "engine.h"

namespace pg {

namespace {

constexpr int kSymWarps = 4;
constexpr int kSymThreads = kSymWarps * 32;
constexpr int kSymIpt = 8;                          // bodies of tile I per thread
constexpr int kSymTile = kSymThreads * kSymIpt;     // 1,024
constexpr int kSymGroups = kSymTile / 32;           // groups of 32 bodies of tile J
static_assert(kSymTile == kBodyPad, "tiles are whole units of the body padding");

// Tile pair of block u: J-major order, u = J (J + 1) / 2 + I, 0 <= I <= J.
__device__ __forceinline__ void unit_tiles(long long u, int &I, int &J)
{
    long long j = (long long)((sqrt(8.0 * (double)u + 1.0) - 1.0) * 0.5);
    while (j > 0 && j * (j + 1) / 2 > u) --j;
    while ((j + 1) * (j + 2) / 2 <= u) ++j;
    J = (int)j;
    I = (int)(u - j * (j + 1) / 2);
}

template <bool DIAG>
__device__ __forceinline__ void sym_tile_pair(const float4 *__restrict__ body, int n, int I,
                                              int J, float e, float *__restrict__ P,
                                              float (*jacc)[kSymTile][3])
{
    constexpr int Q = kSymIpt / 2;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const size_t n3 = 3 * (size_t)n;

    // bodies I*1024 + p*128 + warp*32 + lane, p = 2q (x half) and 2q+1 (y half)
    const int ib = I * kSymTile + warp * 32 + lane;
    float2 nx[Q], ny[Q], nz[Q], nm[Q], ax[Q], ay[Q], az[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float4 b0 = body[ib + (2 * q) * kSymThreads];
        const float4 b1 = body[ib + (2 * q + 1) * kSymThreads];
        nx[q] = make_float2(-b0.x, -b1.x);
        ny[q] = make_float2(-b0.y, -b1.y);
        nz[q] = make_float2(-b0.z, -b1.z);
        nm[q] = make_float2(-b0.w, -b1.w);
        ax[q] = ay[q] = az[q] = make_float2(0.f, 0.f);
    }
    const float2 e2 = make_float2(e, e);
    const float2 g2 = make_float2(kPairGuard, kPairGuard);
    const unsigned full = 0xffffffffu;
    const int src = (lane + 1) & 31;

    float4 next = body[J * kSymTile + lane];
    for (int g = 0; g < kSymGroups; ++g) {
        const float4 bj = next;
        // the next group's body is loaded while this group is evaluated
        if (g + 1 < kSymGroups) next = body[J * kSymTile + (g + 1) * 32 + lane];
        float xj = bj.x, yj = bj.y, zj = bj.z, mj = bj.w;
        float2 jx = make_float2(0.f, 0.f), jy = jx, jz = jx;
#pragma unroll 4
        for (int k = 0; k < 32; ++k) {
            const float2 xj2 = make_float2(xj, xj);
            const float2 yj2 = make_float2(yj, yj);
            const float2 zj2 = make_float2(zj, zj);
            const float2 mj2 = make_float2(mj, mj);
            // the next body's coordinates do not depend on this step
            xj = __shfl_sync(full, xj, src);
            yj = __shfl_sync(full, yj, src);
            zj = __shfl_sync(full, zj, src);
            mj = __shfl_sync(full, mj, src);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const float2 dx = add2(xj2, nx[q]);
                const float2 dy = add2(yj2, ny[q]);
                const float2 dz = add2(zj2, nz[q]);
                float2 r2 = mul2(dz, dz);
                r2 = fma2(dy, dy, r2);
                r2 = fma2(dx, dx, r2);
                const float2 w = add2(r2, e2);
                const float2 ww = mul2(w, w);
                const float2 qv = fma2(r2, ww, g2);
                const float2 inv = make_float2(rsqrt_approx(qv.x), rsqrt_approx(qv.y));
                const float2 fi = mul2(mj2, inv);
                ax[q] = fma2(dx, fi, ax[q]);
                ay[q] = fma2(dy, fi, ay[q]);
                az[q] = fma2(dz, fi, az[q]);
                if (!DIAG) {
                    const float2 fj = mul2(nm[q], inv);
                    jx = fma2(dx, fj, jx);
                    jy = fma2(dy, fj, jy);
                    jz = fma2(dz, fj, jz);
                }
            }
            if (!DIAG) {
                jx.x = __shfl_sync(full, jx.x, src);
                jx.y = __shfl_sync(full, jx.y, src);
                jy.x = __shfl_sync(full, jy.x, src);
                jy.y = __shfl_sync(full, jy.y, src);
                jz.x = __shfl_sync(full, jz.x, src);
                jz.y = __shfl_sync(full, jz.y, src);
            }
        }
        if (!DIAG) {
            // after 32 rotations lane `lane` holds body g*32 + lane's reaction again
            float *dst = jacc[warp][g * 32 + lane];
            dst[0] = jx.x + jx.y;
            dst[1] = jy.x + jy.y;
            dst[2] = jz.x + jz.y;
        }
    }

    // tile J's contribution to tile I's bodies: slot J
    float *pi = P + (size_t)J * n3;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int i0 = ib + (2 * q) * kSymThreads;
        const int i1 = i0 + kSymThreads;
        if (i0 < n) {
            pi[i0] = ax[q].x;
            pi[(size_t)n + i0] = ay[q].x;
            pi[2 * (size_t)n + i0] = az[q].x;
        }
        if (i1 < n) {
            pi[i1] = ax[q].y;
            pi[(size_t)n + i1] = ay[q].y;
            pi[2 * (size_t)n + i1] = az[q].y;
        }
    }
    if (!DIAG) {
        // tile I's contribution to tile J's bodies: slot I, warps added in order
        __syncthreads();
        float *pj = P + (size_t)I * n3;
        for (int j = threadIdx.x; j < kSymTile; j += kSymThreads) {
            const int k = J * kSymTile + j;
            if (k >= n) break;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float s = jacc[0][j][c];
#pragma unroll
                for (int w = 1; w < kSymWarps; ++w) s += jacc[w][j][c];
                pj[(size_t)c * n + k] = s;
            }
        }
    }
}

// 3 blocks per SM: room for 170 registers, which the 4-step unroll uses (measured
// 1% faster than 4 blocks of at most 128 registers)
__global__ void __launch_bounds__(kSymThreads, 3)
direct_sym_kernel(const float4 *__restrict__ body, int n, float e, float *__restrict__ P)
{
    __shared__ float jacc[kSymWarps][kSymTile][3];
    int I, J;
    unit_tiles(blockIdx.x, I, J);
    if (I == J)
        sym_tile_pair<true>(body, n, I, J, e, P, jacc);
    else
        sym_tile_pair<false>(body, n, I, J, e, P, jacc);
}

// out[c*n + k] = sum over the T slots of P[t][c][k], TwoSum-compensated f32
// in slot order, rounded once to f64.
__global__ void sym_reduce_kernel(const float *__restrict__ P, long long n3, int T,
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
    out[idx] = (double)hi + (double)lo;
}

}  // namespace

DirectPlan make_symmetric_plan(int n)
{
    // Three 48 KB blocks per SM need the largest shared-memory carveout.  Set
    // here, when a plan is made (never inside a stream capture), per device.
    static std::atomic<bool> carveout_set[64];
    int device = 0;
    if (cudaGetDevice(&device) == cudaSuccess && device >= 0 && device < 64 &&
        !carveout_set[device].load()) {
        if (cudaFuncSetAttribute(direct_sym_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess)
            carveout_set[device].store(true);
        else
            (void)cudaGetLastError();  // a hint only: the kernel runs without it
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
    return p;
}

size_t direct_partial_doubles(const DirectPlan &p)
{
    const size_t n3 = 3 * (size_t)(p.n > 0 ? p.n : 1);
    if (!p.symmetric) return (size_t)p.splits * n3;
    // f64 sums, then the f32 slot buffer P[T][3][n] carved after them
    return n3 + ((size_t)p.tiles * n3 + 1) / 2;
}

int launch_direct_symmetric(const DirectPlan &plan, const float4 *body4, float e,
                            double *partial, cudaStream_t stream, cudaEvent_t pairs_done)
{
    if (plan.n <= 0) return PHYSIM_OK;
    const long long T = plan.tiles;
    const long long units = T * (T + 1) / 2;
    PG_CHECK(units < (1ll << 31), PHYSIM_ERR_ARGUMENT, "too many bodies for one pass: %d",
             plan.n);
    const long long n3 = 3ll * plan.n;
    float *P = (float *)(partial + n3);
    direct_sym_kernel<<<(unsigned)units, kSymThreads, 0, stream>>>(body4, plan.n, e, P);
    PG_CUDA(cudaGetLastError());
    if (pairs_done) PG_TRY(record_event(pairs_done, stream));
    sym_reduce_kernel<<<(unsigned)((n3 + 255) / 256), 256, 0, stream>>>(P, n3, (int)T, partial);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg
