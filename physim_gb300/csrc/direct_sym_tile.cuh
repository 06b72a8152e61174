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

// The f32 slot sums are left scaled (a' of PairScale: positions entering as
// p 2^-sk, masses as m 2^-skm): the reduction multiplies by 2^(skm - 2sk) in
// f64.
template <bool DIAG>
__device__ __forceinline__ void sym_tile_pair(const float4 *__restrict__ body, int n, int I,
                                              int J, float e, int sk, int skm,
                                              float *__restrict__ P, float (*jacc)[kSymTile][3])
{
    constexpr int Q = kSymIpt / 2;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const size_t n3 = 3 * (size_t)n;

    // bodies I*1024 + p*128 + warp*32 + lane, p = 2q (x half) and 2q+1 (y half)
    const int ib = I * kSymTile + warp * 32 + lane;
    const float sc = pow2f(-sk);  // 2^-sk, exact
    const float msc = pow2f(-skm);
    float2 nx[Q], ny[Q], nz[Q], nm[Q], ax[Q], ay[Q], az[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float4 b0 = body[ib + (2 * q) * kSymThreads];
        const float4 b1 = body[ib + (2 * q + 1) * kSymThreads];
        nx[q] = make_float2(-b0.x * sc, -b1.x * sc);
        ny[q] = make_float2(-b0.y * sc, -b1.y * sc);
        nz[q] = make_float2(-b0.z * sc, -b1.z * sc);
        nm[q] = make_float2(-b0.w * msc, -b1.w * msc);
        ax[q] = ay[q] = az[q] = make_float2(0.f, 0.f);
    }
    const float es = e * pow2f(-2 * sk);
    const float2 e2 = make_float2(es, es);
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

}  // namespace pg
