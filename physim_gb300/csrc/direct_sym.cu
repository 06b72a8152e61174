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
// evaluates one tile pair (I, J), I <= J, of the T(T+1)/2.  Its 2 warps hold
// the 1,024 bodies of tile I in registers (16 per thread, as 8 packed FFMA2
// pairs, so each rotation of the travelling bodies serves 16 pairs).  A warp takes the bodies of tile J 32 at a time, one per lane, and
// rotates them through its lanes with shuffles: after 32 steps every lane's
// 8 bodies have met all 32, and each travelling body's accumulated reaction
// (a float2: the two halves of the packed pairs) is back at its home lane.
// a_i stays in registers for the whole tile; each warp writes its a_j sums
// for the tile to its own slice of shared memory, and the block adds the 2
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
#include "direct_sym_tile.cuh"
#include "engine.h"

namespace pg {

namespace {

// 64 threads of up to 255 registers (about 250 used); measured on GB300 at
// 1,048,580 bodies: 274.5 ms per pass, against 300.9 ms for 4 warps of 8
// bodies per thread on the same GPU (the shuffles per pair halve)
__global__ void __launch_bounds__(kSymThreads, 3)
direct_sym_kernel(const float4 *__restrict__ body, int n, float e,
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

// out[c*n + k] = sum over the T slots of P[t][c][k], TwoSum-compensated f32
// in slot order, rounded once to f64 and unscaled (x 2^(km - 2k)).
__global__ void sym_reduce_kernel(const float *__restrict__ P, long long n3, int T,
                                  const PairScale *__restrict__ scale, double *__restrict__ out)
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
    // Blocks of 24 KB of shared memory: the largest carveout keeps them all resident.  Set
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
                            const PairScale *scale, double *partial, cudaStream_t stream,
                            cudaEvent_t pairs_done)
{
    if (plan.n <= 0) return PHYSIM_OK;
    const long long T = plan.tiles;
    const long long units = T * (T + 1) / 2;
    PG_CHECK(units < (1ll << 31), PHYSIM_ERR_ARGUMENT, "too many bodies for one pass: %d",
             plan.n);
    const long long n3 = 3ll * plan.n;
    float *P = (float *)(partial + n3);
    direct_sym_kernel<<<(unsigned)units, kSymThreads, 0, stream>>>(body4, plan.n, e, scale, P);
    PG_CUDA(cudaGetLastError());
    if (pairs_done) PG_TRY(record_event(pairs_done, stream));
    sym_reduce_kernel<<<(unsigned)((n3 + 255) / 256), 256, 0, stream>>>(P, n3, (int)T, scale,
                                                                         partial);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg
