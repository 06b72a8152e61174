// direct_sym_tile.cuh -- one tile pair of the symmetric direct sum (each
// unordered pair evaluated once, both bodies updated), shared by the
// per-simulation kernel (direct_sym.cu) and the batched ensemble kernel
// (ensemble.cu) so both evaluate bit-identical arithmetic.  The schedule and
// the slot-buffer layout are described in direct_sym.cu.
#pragma once

#include "common.cuh"
#include "engine.h"

namespace pg {

constexpr int kSymWarps = 2;
constexpr int kSymThreads = kSymWarps * 32;
constexpr int kSymIpt = 16;                         // bodies of tile I per thread
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

// Tile I's bodies in registers: positions (negated) scaled by sc, masses
// (negated) by msc (PairScale in engine.h).  Thread layout: bodies
// I*1024 + p*128 + warp*32 + lane, p = 2q (x half) and 2q+1 (y half).
constexpr int kSymQ = kSymIpt / 2;

__device__ __forceinline__ void sym_load_i(const float4 *__restrict__ body, int I, float sc,
                                           float msc, float2 (&nx)[kSymQ], float2 (&ny)[kSymQ],
                                           float2 (&nz)[kSymQ], float2 (&nm)[kSymQ])
{
    const int ib = I * kSymTile + (threadIdx.x >> 5) * 32 + (threadIdx.x & 31);
#pragma unroll
    for (int q = 0; q < kSymQ; ++q) {
        const float4 b0 = body[ib + (2 * q) * kSymThreads];
        const float4 b1 = body[ib + (2 * q + 1) * kSymThreads];
        nx[q] = make_float2(-b0.x * sc, -b1.x * sc);
        ny[q] = make_float2(-b0.y * sc, -b1.y * sc);
        nz[q] = make_float2(-b0.z * sc, -b1.z * sc);
        nm[q] = make_float2(-b0.w * msc, -b1.w * msc);
    }
}

// *p += v on a shared-memory float, atomically (PTX red.shared.add.f32).
__device__ __forceinline__ void red_shared_add(float *p, float v)
{
    asm volatile("red.shared.add.f32 [%0], %1;"
                 :
                 : "r"((unsigned)__cvta_generic_to_shared(p)), "f"(v)
                 : "memory");
}

// Tile I (in registers) against tile J: a_i += the pairs' terms (scaled, see
// sym_load_i); unless DIAG, tile J's reactions go to shared memory, jw[j][c]
// for body j of tile J: stored (this warp's own slice), or with ADD added to
// a slice that starts at zero and that both warps of the block add to (two
// terms added onto zero round the same in either order, so the sum does not
// depend on which warp comes first).  With DIAG (I == J) every ordered pair
// of the tile is evaluated for a_i only (a body meets itself with d = 0,
// which contributes 0 through the r^2 guard).
template <bool DIAG, bool ADD = false>
__device__ __forceinline__ void sym_pair_core(const float4 *__restrict__ body, int J, float sc,
                                              float msc, float2 e2, const float2 (&nx)[kSymQ],
                                              const float2 (&ny)[kSymQ],
                                              const float2 (&nz)[kSymQ],
                                              const float2 (&nm)[kSymQ], float2 (&ax)[kSymQ],
                                              float2 (&ay)[kSymQ], float2 (&az)[kSymQ],
                                              float (*jw)[3])
{
    const int lane = threadIdx.x & 31;
    const float2 g2 = make_float2(kPairGuard, kPairGuard);
    const unsigned full = 0xffffffffu;
    const int src = (lane + 1) & 31;

    float4 next = body[J * kSymTile + lane];
    for (int g = 0; g < kSymGroups; ++g) {
        const float4 bj = next;
        // the next group's body is loaded while this group is evaluated
        if (g + 1 < kSymGroups) next = body[J * kSymTile + (g + 1) * 32 + lane];
        float xj = bj.x * sc, yj = bj.y * sc, zj = bj.z * sc, mj = bj.w * msc;
        float2 jx = make_float2(0.f, 0.f), jy = jx, jz = jx;
#pragma unroll 2
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
            for (int q = 0; q < kSymQ; ++q) {
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
            float *dst = jw[g * 32 + lane];
            if (ADD) {
                red_shared_add(dst + 0, jx.x + jx.y);
                red_shared_add(dst + 1, jy.x + jy.y);
                red_shared_add(dst + 2, jz.x + jz.y);
            } else {
                dst[0] = jx.x + jx.y;
                dst[1] = jy.x + jy.y;
                dst[2] = jz.x + jz.y;
            }
        }
    }
}

// One tile pair (I, J) with its own slots (the ensemble's layout): tile J's
// contribution to tile I's bodies goes to slot J, tile I's to tile J's
// bodies to slot I, of P[T][3][n] (f32, left scaled: positions entering as
// p 2^-sk, masses as m 2^-skm; the reduction multiplies by 2^(skm - 2sk) in
// f64).
template <bool DIAG>
__device__ __forceinline__ void sym_tile_pair(const float4 *__restrict__ body, int n, int I,
                                              int J, float e, int sk, int skm,
                                              float *__restrict__ P, float (*jacc)[kSymTile][3])
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const size_t n3 = 3 * (size_t)n;
    const int ib = I * kSymTile + warp * 32 + lane;
    const float sc = pow2f(-sk), msc = pow2f(-skm);
    const float es = e * pow2f(-2 * sk);
    const float2 e2 = make_float2(es, es);
    float2 nx[kSymQ], ny[kSymQ], nz[kSymQ], nm[kSymQ], ax[kSymQ], ay[kSymQ], az[kSymQ];
    sym_load_i(body, I, sc, msc, nx, ny, nz, nm);
#pragma unroll
    for (int q = 0; q < kSymQ; ++q) ax[q] = ay[q] = az[q] = make_float2(0.f, 0.f);
    sym_pair_core<DIAG>(body, J, sc, msc, e2, nx, ny, nz, nm, ax, ay, az, jacc[warp]);

    // tile J's contribution to tile I's bodies: slot J
    float *pi = P + (size_t)J * n3;
#pragma unroll
    for (int q = 0; q < kSymQ; ++q) {
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

}  // namespace pg
