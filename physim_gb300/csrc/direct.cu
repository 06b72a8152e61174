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
#include <math.h>

#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "direct_tile.cuh"
#include "engine.h"

namespace pg {

namespace {

template <int BLOCK, int IPT, bool COMP>
__global__ void __launch_bounds__(BLOCK, 2)
direct_forces_kernel(const float4 *__restrict__ body, int n, int n_jtiles, int chunk_tiles, float e,
                     const PairScale *__restrict__ scale, double *__restrict__ partial)
{
    __shared__ float4 tile[2][BLOCK][2];
    const int split = blockIdx.y;
    const int t0 = split * chunk_tiles;
    const int t1 = min(t0 + chunk_tiles, n_jtiles);
    direct_tile<BLOCK, IPT, COMP>(body, n, blockIdx.x * BLOCK * IPT, t0, t1, e, scale->k,
                                  scale->km, partial + (size_t)split * 3 * n, tile);
}

// Largest |coordinate| and |mass| of body4[0, n) (f32 bit patterns order
// like the non-negative values; NaN and infinities skipped), reduced by the
// last block to finish into ps->k and ps->km (see PairScale).
__device__ __forceinline__ uint32_t finite_abs_bits(float v)
{
    const uint32_t b = __float_as_uint(v) & 0x7fffffffu;
    return b < 0x7f800000u ? b : 0u;
}

__global__ void __launch_bounds__(256)
pair_scale_kernel(const float4 *__restrict__ body, int n, float e, PairScale *ps)
{
    uint32_t m = 0, w = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 b = body[i];
        m = max(m, max(finite_abs_bits(b.x), max(finite_abs_bits(b.y), finite_abs_bits(b.z))));
        w = max(w, finite_abs_bits(b.w));
    }
    for (int o = 16; o > 0; o >>= 1) {
        m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        w = max(w, __shfl_xor_sync(0xffffffffu, w, o));
    }
    __shared__ uint32_t wm[8], ww[8];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) {
        wm[threadIdx.x >> 5] = m;
        ww[threadIdx.x >> 5] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            m = max(m, wm[k]);
            w = max(w, ww[k]);
        }
        ps->blockmax[blockIdx.x] = m;
        ps->blockmass[blockIdx.x] = w;
        __threadfence();
        last = atomicAdd(&ps->arrivals, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    uint32_t t = 0, tw = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        t = max(t, __ldcg(&ps->blockmax[b]));
        tw = max(tw, __ldcg(&ps->blockmass[b]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        t = max(t, __shfl_xor_sync(0xffffffffu, t, o));
        tw = max(tw, __shfl_xor_sync(0xffffffffu, tw, o));
    }
    if ((threadIdx.x & 31) == 0) {
        wm[threadIdx.x >> 5] = t;
        ww[threadIdx.x >> 5] = tw;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            t = max(t, wm[k]);
            tw = max(tw, ww[k]);
        }
        ps->k = pair_scale_exp(__uint_as_float(t), e);
        ps->km = mass_scale_exp(__uint_as_float(tw));
        ps->arrivals = 0u;
    }
}

struct Shape {
    int block, ipt;
};
constexpr Shape kShapes[] = {{256, 4}, {128, 4}, {128, 2}, {256, 2}, {128, 8}};

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
    if (block == 128 && ipt == 8) return kernel_ptr<128, 8>(comp);
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

// Bodies from which the heuristic plan evaluates each unordered pair once.
// Measured on GB300 (best one-pair plan vs the symmetric plan, force pass):
// 8,192 bodies 0.039 vs 0.105 ms (36 tile pairs cannot fill 152 SMs),
// 16,384 0.120 vs 0.108 ms, 65,536 1.81 vs 1.20 ms, 1,048,580 428 vs 293 ms.
constexpr int kSymmetricMinBodies = 20480;
// Smallest size at which the autotuner also times the symmetric plan.
constexpr int kSymmetricCandidateBodies = 12288;

// The symmetric plan's slot buffer grows as n^2 (12 B per body and 1,024-body
// tile: 12.9 GB at 1,048,580 bodies, 51 GB at 2M).  It is planned only while
// it stays within the cap (a quarter of the device's memory unless
// physim_gpu_set_symmetric_cap set one) and within the device's free memory
// at planning time less a margin for everything else; otherwise the one-pair
// plans are used.  A plan that still fails to allocate falls back to a
// one-pair plan at the caller (element.cu, sim.cu).
static std::atomic<uint64_t> g_symmetric_cap{0};
constexpr size_t kSymmetricFreeMargin = size_t(1) << 30;

static bool symmetric_fits(int n, int device)
{
    int cur = 0;
    size_t free_b = 0, total_b = 0;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != device ||
        cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    const uint64_t cap = g_symmetric_cap.load();
    const size_t need = direct_partial_doubles(make_symmetric_plan(n)) * sizeof(double);
    return need <= (cap ? cap : total_b / 4) && need + kSymmetricFreeMargin <= free_b;
}

DirectPlan plan_direct_one_pair(int n, int device, bool compensated)
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

DirectPlan plan_direct(int n, int device, bool compensated)
{
    if (compensated && n >= kSymmetricMinBodies && symmetric_fits(n, device))
        return make_symmetric_plan(n);
    return plan_direct_one_pair(n, device, compensated);
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
    if (compensated && n >= kSymmetricCandidateBodies && k < cap && symmetric_fits(n, device))
        out[k++] = make_symmetric_plan(n);
    return k;
}

DirectPlan make_direct_plan(int n, int block, int ipt, int splits, bool compensated)
{
    return make_plan(n, block, ipt, splits, compensated);
}

bool direct_shape_supported(int block, int ipt)
{
    return shape_kernel(block, ipt, true) != nullptr;
}

int record_event(cudaEvent_t ev, cudaStream_t stream)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PG_CUDA(cudaStreamIsCapturing(stream, &cs));
    PG_CUDA(cudaEventRecordWithFlags(
        ev, stream, cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0));
    return PHYSIM_OK;
}

int launch_pair_scale(const float4 *body4, int n, float e, PairScale *ps, cudaStream_t stream)
{
    const int blocks = std::max(1, std::min(kScaleBlocks, (n + 2047) / 2048));
    pair_scale_kernel<<<blocks, 256, 0, stream>>>(body4, n, e, ps);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

float max_abs_mass(const Entity *state, size_t n)
{
    float m = 0.f;
    for (size_t i = 0; i < n; ++i) {
        const float a = fabsf((float)state[i].mass);
        if (a <= 3.4028235e38f && a > m) m = a;  // NaN and infinities skipped
    }
    return m;
}

float max_abs_coordinate(const Entity *state, size_t n)
{
    float m = 0.f;
    for (size_t i = 0; i < n; ++i) {
        const float c[3] = {(float)state[i].x, (float)state[i].y, (float)state[i].z};
        for (float v : c) {
            const float a = fabsf(v);
            if (a <= 3.4028235e38f && a > m) m = a;  // NaN and infinities skipped
        }
    }
    return m;
}

int launch_direct(const DirectPlan &plan, const float4 *body4, float e, PairScale *scale,
                  double *partial, cudaStream_t stream, cudaEvent_t pairs_done)
{
    if (plan.n <= 0) return PHYSIM_OK;
    PG_CHECK(scale, PHYSIM_ERR_ARGUMENT, "no pair-scale workspace");
    PG_TRY(launch_pair_scale(body4, plan.n, e, scale, stream));
    if (plan.symmetric)
        return launch_direct_symmetric(plan, body4, e, scale, partial, stream, pairs_done);
    dim3 grid(plan.n_itiles, plan.splits);
    void *fn = shape_kernel(plan.block, plan.ipt, plan.compensated);
    PG_CHECK(fn != nullptr, PHYSIM_ERR_ARGUMENT, "no direct-sum kernel for block %d ipt %d",
             plan.block, plan.ipt);
    int n = plan.n, njt = plan.n_jtiles, ct = plan.chunk_tiles;
    const PairScale *sc = scale;
    void *args[] = {(void *)&body4, (void *)&n, (void *)&njt, (void *)&ct, (void *)&e,
                    (void *)&sc, (void *)&partial};
    PG_CUDA(cudaLaunchKernel(fn, grid, dim3(plan.block), args, 0, stream));
    if (pairs_done) PG_TRY(record_event(pairs_done, stream));
    return PHYSIM_OK;
}

}  // namespace pg

extern "C" int physim_gpu_set_symmetric_cap(uint64_t bytes)
{
    pg::g_symmetric_cap.store(bytes);
    return PHYSIM_OK;
}
