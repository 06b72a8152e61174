// direct.cu -- tiled FP32 direct-sum pair forces (the `simple_astro` element,
// astro/src/transformers.rs:219-244, force law astro/src/lib.rs:84-113).
//
// Per pair (i, j) the reference computes, in f64,
//     F_ij = (x_j - x_i) / r * G m_i m_j / (r^2 + e),   r = |x_j - x_i|,
// skips pairs at exactly equal positions, sums F_ij over j and divides by
// m_i.  The m_i cancels, so the kernel accumulates
//     a_i = sum_j m_j (x_j - x_i) / sqrt(r^2 (r^2 + e)^2)
// with ONE reciprocal square root per pair (MUFU.RSQ) instead of a square
// root and a reciprocal.  13 FP32 FMA-pipe operations and one MUFU per pair;
// pairs are evaluated two at a time with Blackwell's packed FFMA2/FADD2/FMUL2
// so the issue slots are not the bound.
//
// Layout: j bodies are staged through shared memory in tiles of BLOCK bodies,
// each stored as (x,x,y,y)(z,z,m,m) so one 128-bit broadcast load yields the
// float2 operands of the packed instructions.  Each thread holds IPT i bodies.
// The j range can be split over gridDim.y blocks (partial sums are combined
// by the integrator kernel), which keeps the last wave of a GPU with 152 SMs
// full.  Per-body sums are compensated: each j tile is summed in plain FP32
// and folded into a (hi, lo) pair with TwoSum once per tile.
#include <algorithm>

#include "common.cuh"
#include "engine.h"

namespace pg {

namespace {

template <int BLOCK, int IPT, bool COMP>
__global__ void __launch_bounds__(BLOCK, 2)
direct_forces_kernel(const float4 *__restrict__ body, int n, int n_jtiles, int chunk_tiles, float e,
                     double *__restrict__ partial)
{
    static_assert(IPT % 2 == 0, "bodies per thread must be even (packed pairs)");
    constexpr int P = IPT / 2;
    __shared__ float4 tile[2][BLOCK][2];

    const int tid = threadIdx.x;
    const int i_base = blockIdx.x * BLOCK * IPT;
    const int split = blockIdx.y;
    const int t0 = split * chunk_tiles;
    const int t1 = min(t0 + chunk_tiles, n_jtiles);

    float2 nx[P], ny[P], nz[P];
    float2 ax[P], ay[P], az[P];
    float2 hx[P], hy[P], hz[P], lx[P], ly[P], lz[P];
#pragma unroll
    for (int p = 0; p < P; ++p) {
        // bodies i_base + tid + k*BLOCK, k = 2p, 2p+1 (rows padded, always readable)
        float4 b0 = body[i_base + tid + (2 * p) * BLOCK];
        float4 b1 = body[i_base + tid + (2 * p + 1) * BLOCK];
        nx[p] = make_float2(-b0.x, -b1.x);
        ny[p] = make_float2(-b0.y, -b1.y);
        nz[p] = make_float2(-b0.z, -b1.z);
        ax[p] = ay[p] = az[p] = make_float2(0.f, 0.f);
        hx[p] = hy[p] = hz[p] = make_float2(0.f, 0.f);
        lx[p] = ly[p] = lz[p] = make_float2(0.f, 0.f);
    }
    const float2 e2 = make_float2(e, e);
    const float2 g2 = make_float2(kPairGuard, kPairGuard);

    if (t0 < t1) {
        float4 nxt = body[t0 * BLOCK + tid];
        for (int t = t0; t < t1; ++t) {
            const int buf = (t - t0) & 1;
            tile[buf][tid][0] = make_float4(nxt.x, nxt.x, nxt.y, nxt.y);
            tile[buf][tid][1] = make_float4(nxt.z, nxt.z, nxt.w, nxt.w);
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
    double *px = partial + (size_t)(split * 3 + 0) * n;
    double *py = partial + (size_t)(split * 3 + 1) * n;
    double *pz = partial + (size_t)(split * 3 + 2) * n;
#pragma unroll
    for (int p = 0; p < P; ++p) {
        const int i0 = i_base + tid + (2 * p) * BLOCK;
        const int i1 = i0 + BLOCK;
        if (i0 < n) {
            px[i0] = (double)hx[p].x + (double)lx[p].x;
            py[i0] = (double)hy[p].x + (double)ly[p].x;
            pz[i0] = (double)hz[p].x + (double)lz[p].x;
        }
        if (i1 < n) {
            px[i1] = (double)hx[p].y + (double)lx[p].y;
            py[i1] = (double)hy[p].y + (double)ly[p].y;
            pz[i1] = (double)hz[p].y + (double)lz[p].y;
        }
    }
}

struct Shape {
    int block, ipt;
};
constexpr Shape kShapes[] = {{256, 4}, {128, 4}, {128, 2}, {256, 2}};

template <int BLOCK, int IPT>
void *kernel_ptr(bool comp)
{
    return comp ? (void *)direct_forces_kernel<BLOCK, IPT, true>
                : (void *)direct_forces_kernel<BLOCK, IPT, false>;
}

void *shape_kernel(int block, int ipt, bool comp)
{
    if (block == 256 && ipt == 4) return kernel_ptr<256, 4>(comp);
    if (block == 128 && ipt == 4) return kernel_ptr<128, 4>(comp);
    if (block == 128 && ipt == 2) return kernel_ptr<128, 2>(comp);
    if (block == 256 && ipt == 2) return kernel_ptr<256, 2>(comp);
    return nullptr;
}

int resident_blocks(int block, int ipt, bool comp)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, shape_kernel(block, ipt, comp), block,
                                                      0) != cudaSuccess)
        return 1;
    return nb > 0 ? nb : 1;
}

DirectPlan make_plan(int n, int block, int ipt, int splits, bool comp)
{
    DirectPlan p;
    p.block = block;
    p.ipt = ipt;
    p.n = n;
    p.compensated = comp;
    p.n_itiles = (n + block * ipt - 1) / (block * ipt);
    p.n_jtiles = (n + block - 1) / block;
    splits = std::max(1, std::min(splits, std::max(1, p.n_jtiles)));
    p.chunk_tiles = (p.n_jtiles + splits - 1) / splits;
    p.splits = (p.n_jtiles + p.chunk_tiles - 1) / p.chunk_tiles;
    if (p.splits < 1) p.splits = 1;
    return p;
}

}  // namespace

int device_sm_count(int device)
{
    static int cache[64] = {0};
    if (device < 0 || device >= 64) return 1;
    if (cache[device] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
            v <= 0)
            v = 1;
        cache[device] = v;
    }
    return cache[device];
}

// Fraction of the block slots that do useful work over all waves.
static double wave_efficiency(long units, long slots)
{
    long waves = (units + slots - 1) / slots;
    return (double)units / (double)(waves * slots);
}

DirectPlan plan_direct(int n, int device, bool compensated)
{
    const int sms = device_sm_count(device);
    DirectPlan best;
    double best_score = -1.0;
    for (const Shape &s : kShapes) {
        const long slots = (long)sms * resident_blocks(s.block, s.ipt, compensated);
        const int n_itiles = (n + s.block * s.ipt - 1) / (s.block * s.ipt);
        const int n_jtiles = (n + s.block - 1) / s.block;
        for (int split = 1; split <= 32; ++split) {
            if (split > n_jtiles) break;
            DirectPlan p = make_plan(n, s.block, s.ipt, split, compensated);
            const long units = (long)n_itiles * p.splits;
            // Larger i tiles re-read j less; weigh a small bonus for them.
            double score = wave_efficiency(units, slots);
            if (units < slots) score = (double)units / slots;
            score += (s.ipt == 4 ? 0.004 : 0.0) + (s.block == 256 ? 0.002 : 0.0);
            score -= 0.0005 * p.splits;  // fewer partial sums to combine
            if (score > best_score) {
                best_score = score;
                best = p;
            }
        }
    }
    return best;
}

int direct_candidates(int n, int device, bool compensated, DirectPlan *out, int cap)
{
    const int sms = device_sm_count(device);
    int k = 0;
    for (const Shape &s : kShapes) {
        const long slots = (long)sms * resident_blocks(s.block, s.ipt, compensated);
        const int n_itiles = (n + s.block * s.ipt - 1) / (s.block * s.ipt);
        const int n_jtiles = (n + s.block - 1) / s.block;
        // the two best split counts for this shape
        int best[2] = {1, 1};
        double sc[2] = {-1.0, -1.0};
        for (int split = 1; split <= 32 && split <= n_jtiles; ++split) {
            DirectPlan p = make_plan(n, s.block, s.ipt, split, compensated);
            long units = (long)n_itiles * p.splits;
            double score = units < slots ? (double)units / slots : wave_efficiency(units, slots);
            if (score > sc[0]) {
                sc[1] = sc[0];
                best[1] = best[0];
                sc[0] = score;
                best[0] = p.splits;
            } else if (score > sc[1] && p.splits != best[0]) {
                sc[1] = score;
                best[1] = p.splits;
            }
        }
        for (int q = 0; q < 2 && k < cap; ++q) {
            if (q == 1 && best[1] == best[0]) continue;
            out[k++] = make_plan(n, s.block, s.ipt, best[q], compensated);
        }
    }
    return k;
}

int launch_direct(const DirectPlan &plan, const float4 *body4, float e, double *partial,
                  cudaStream_t stream)
{
    if (plan.n <= 0) return PHYSIM_OK;
    dim3 grid(plan.n_itiles, plan.splits);
    void *fn = shape_kernel(plan.block, plan.ipt, plan.compensated);
    PG_CHECK(fn != nullptr, PHYSIM_ERR_ARGUMENT, "no direct-sum kernel for block %d ipt %d",
             plan.block, plan.ipt);
    int n = plan.n, njt = plan.n_jtiles, ct = plan.chunk_tiles;
    void *args[] = {(void *)&body4, (void *)&n, (void *)&njt, (void *)&ct, (void *)&e,
                    (void *)&partial};
    PG_CUDA(cudaLaunchKernel(fn, grid, dim3(plan.block), args, 0, stream));
    return PHYSIM_OK;
}

}  // namespace pg
