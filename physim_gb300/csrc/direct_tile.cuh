// direct_tile.cuh -- the direct-sum pair loop shared by the per-simulation
// kernel (direct.cu) and the batched ensemble kernel (ensemble.cu), so both
// evaluate bit-identical pair arithmetic.
//
// Per pair (i, j) the reference (astro/src/lib.rs:84-113) computes
//     F_ij = (x_j - x_i) / r * G m_i m_j / (r^2 + e),
// and divides the sum by m_i.  The m_i cancels, so the loop accumulates
//     a_i = sum_j m_j (x_j - x_i) / sqrt(r^2 (r^2 + e)^2)
// with ONE reciprocal square root per pair.  13 FP32 FMA-pipe operations
// and one MUFU per pair, two pairs per instruction with packed FFMA2/FADD2/
// FMUL2.  j bodies are staged in shared memory as (x,x,y,y)(z,z,m,m) so one
// 128-bit broadcast load yields the float2 operands.  Per-body sums are
// compensated: each j tile is summed in plain FP32 and folded into a
// (hi, lo) pair with TwoSum once per tile.  Positions enter scaled by 2^-sk,
// masses by 2^-skm, and the sums leave multiplied by 2^(skm - 2sk)
// (PairScale in engine.h).
#pragma once

#include "common.cuh"
#include "engine.h"

namespace pg {

// One i tile of BLOCK*IPT bodies starting at i_base against the j tiles
// [t0, t1) of `body` (n bodies, padded), writing this split's partial sums to
// out[c*n + i].  `tile` is the block's shared staging buffer; sk and skm the
// pair scale exponents.
template <int BLOCK, int IPT, bool COMP>
__device__ __forceinline__ void direct_tile(const float4 *__restrict__ body, int n, int i_base,
                                            int t0, int t1, float e, int sk, int skm,
                                            double *__restrict__ out, float4 (*tile)[BLOCK][2])
{
    static_assert(IPT % 2 == 0, "bodies per thread must be even (packed pairs)");
    constexpr int P = IPT / 2;
    const int tid = threadIdx.x;
    const float sc = pow2f(-sk);      // 2^-sk, exact
    const float msc = pow2f(-skm);    // 2^-skm
    const double unsc = pow2d(skm - 2 * sk);  // back to unscaled accelerations

    float2 nx[P], ny[P], nz[P];
    float2 ax[P], ay[P], az[P];
    float2 hx[P], hy[P], hz[P], lx[P], ly[P], lz[P];
#pragma unroll
    for (int p = 0; p < P; ++p) {
        // bodies i_base + tid + k*BLOCK, k = 2p, 2p+1 (rows padded, always readable)
        float4 b0 = body[i_base + tid + (2 * p) * BLOCK];
        float4 b1 = body[i_base + tid + (2 * p + 1) * BLOCK];
        nx[p] = make_float2(-b0.x * sc, -b1.x * sc);
        ny[p] = make_float2(-b0.y * sc, -b1.y * sc);
        nz[p] = make_float2(-b0.z * sc, -b1.z * sc);
        ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
        hx[p] = hy[p] = hz[p] = make_float2(0.f, 0.f);
        lx[p] = ly[p] = lz[p] = make_float2(0.f, 0.f);
    }
    const float es = e * pow2f(-2 * sk);
    const float2 e2 = make_float2(es, es);
    const float2 g2 = make_float2(kPairGuard, kPairGuard);

    if (t0 < t1) {
        float4 nxt = body[t0 * BLOCK + tid];
        for (int t = t0; t < t1; ++t) {
            const int buf = (t - t0) & 1;
            const float sx = nxt.x * sc, sy = nxt.y * sc, sz = nxt.z * sc;
            tile[buf][tid][0] = make_float4(sx, sx, sy, sy);
            const float sm = nxt.w * msc;
            tile[buf][tid][1] = make_float4(sz, sz, sm, sm);
            __syncthreads();
            if (t + 1 < t1) nxt = body[(t + 1) * BLOCK + tid];
#pragma unroll 4
            for (int j = 0; j < BLOCK; ++j) {
                const float4 A = tile[buf][j][0];
                const float4 B = tile[buf][j][1];
                const float2 xj = make_float2(A.x, A.y);
                const float2 yj = make_float2(A.z, A.w);
                const float2 zj = make_float2(B.x, B.y);
                const float2 mj = make_float2(B.z, B.w);
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    const float2 dx = add2(xj, nx[p]);
                    const float2 dy = add2(yj, ny[p]);
                    const float2 dz = add2(zj, nz[p]);
                    float2 r2 = mul2(dz, dz);
                    r2 = fma2(dy, dy, r2);
                    r2 = fma2(dx, dx, r2);
                    const float2 w = add2(r2, e2);
                    const float2 ww = mul2(w, w);
                    const float2 q = fma2(r2, ww, g2);
                    const float2 inv = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
                    const float2 s = mul2(mj, inv);
                    ax[p] = fma2(dx, s, ax[p]);
                    ay[p] = fma2(dy, s, ay[p]);
                    az[p] = fma2(dz, s, az[p]);
                }
            }
            if (COMP) {
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    float s, err;
                    two_sum(hx[p].x, ax[p].x, s, err); hx[p].x = s; lx[p].x += err;
                    two_sum(hx[p].y, ax[p].y, s, err); hx[p].y = s; lx[p].y += err;
                    two_sum(hy[p].x, ay[p].x, s, err); hy[p].x = s; ly[p].x += err;
                    two_sum(hy[p].y, ay[p].y, s, err); hy[p].y = s; ly[p].y += err;
                    two_sum(hz[p].x, az[p].x, s, err); hz[p].x = s; lz[p].x += err;
                    two_sum(hz[p].y, az[p].y, s, err); hz[p].y = s; lz[p].y += err;
                    ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
                }
            }
        }
    }
    if (!COMP) {
#pragma unroll
        for (int p = 0; p < P; ++p) {
            hx[p] = ax[p];
            hy[p] = ay[p];
            hz[p] = az[p];
        }
    }
    double *px = out;
    double *py = out + n;
    double *pz = out + 2 * (size_t)n;
#pragma unroll
    for (int p = 0; p < P; ++p) {
        const int i0 = i_base + tid + (2 * p) * BLOCK;
        const int i1 = i0 + BLOCK;
        if (i0 < n) {
            px[i0] = ((double)hx[p].x + (double)lx[p].x) * unsc;
            py[i0] = ((double)hy[p].x + (double)ly[p].x) * unsc;
            pz[i0] = ((double)hz[p].x + (double)lz[p].x) * unsc;
        }
        if (i1 < n) {
            px[i1] = ((double)hx[p].y + (double)lx[p].y) * unsc;
            py[i1] = ((double)hy[p].y + (double)ly[p].y) * unsc;
            pz[i1] = ((double)hz[p].y + (double)lz[p].y) * unsc;
        }
    }
}

}  // namespace pg
