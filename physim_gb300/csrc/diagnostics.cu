// diagnostics.cu -- whole-system diagnostics of a device-resident simulation,
// accumulated in f64: mass, centre of mass, momentum, kinetic energy and the
// potential energy that belongs to the reference's force law.
//
// The reference's pair force has magnitude G m_a m_b / (r^2 + e)
// (astro/src/lib.rs:84-113), so the potential whose gradient it is, with
// V -> 0 far away, is
//     V(r) = -G m_a m_b atan(sqrt(e) / r) / sqrt(e)      (e > 0)
//     V(r) = -G m_a m_b / r                              (e = 0)
// (physim's debug energysink computes -m_a m_b / r and keeps only the last
// pair, debug/src/energysink.rs:86; this is the consistent total).  Pairs at
// exactly equal positions are skipped, as the force loop skips them.  Pair
// separations are f64, pair terms FP32, per-body sums f64 per tile; every
// other sum is f64.
#include <string.h>

#include <new>

#include "common.cuh"
#include "engine.h"

namespace pg {
namespace {

constexpr int kDiagThreads = 256;

__global__ void moments_kernel(const double *__restrict__ x, const double *__restrict__ y,
                               const double *__restrict__ z, const double *__restrict__ vx,
                               const double *__restrict__ vy, const double *__restrict__ vz,
                               const double *__restrict__ m, int n, double *__restrict__ out)
{
    // out: mass, m x, m y, m z, m vx, m vy, m vz, kinetic
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double mi = m[i];
        s[0] += mi;
        s[1] += mi * x[i];
        s[2] += mi * y[i];
        s[3] += mi * z[i];
        s[4] += mi * vx[i];
        s[5] += mi * vy[i];
        s[6] += mi * vz[i];
        s[7] += 0.5 * mi * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
    }
    __shared__ double red[8][kDiagThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < 8; ++c) {
        double v = s[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[c][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double v = 0.0;
        for (int w = 0; w < kDiagThreads / 32; ++w) v += red[threadIdx.x][w];
        atomicAdd(&out[threadIdx.x], v);
    }
}

// Potential: thread i sums m_j phi(r_ij) over a j range.  Separations are
// taken in f64 from the f64 state and rounded to FP32 (relative error 2^-24
// of the separation itself, however close the pair); phi is evaluated in
// FP32, summed in FP32 per 256-body tile and folded into f64 per tile.
// f64 position and mass of one body (32-byte aligned: two 128-bit loads).
struct alignas(32) Pos4 {
    double x, y, z, w;
};

// 0.5 m_i * sum goes to out[8].
__global__ void __launch_bounds__(kDiagThreads)
potential_kernel(const double *__restrict__ x, const double *__restrict__ y,
                 const double *__restrict__ z, const double *__restrict__ m, int n, float e,
                 int chunk, double *__restrict__ out)
{
    __shared__ Pos4 tile[kDiagThreads];
    const int i = blockIdx.x * kDiagThreads + threadIdx.x;
    const int j0 = blockIdx.y * chunk, j1 = min(j0 + chunk, n);
    const Pos4 bi = i < n ? Pos4{x[i], y[i], z[i], m[i]} : Pos4{0.0, 0.0, 0.0, 0.0};
    const float se = sqrtf(e);
    const float inv_se = e > 0.f ? 1.f / se : 0.f;
    double acc = 0.0;
    for (int t = j0; t < j1; t += kDiagThreads) {
        __syncthreads();
        const int j = t + threadIdx.x;
        tile[threadIdx.x] = j < j1 ? Pos4{x[j], y[j], z[j], m[j]} : Pos4{0.0, 0.0, 0.0, 0.0};
        __syncthreads();
        const int cnt = min(kDiagThreads, j1 - t);
        float part = 0.f;
        for (int k = 0; k < cnt; ++k) {
            const Pos4 bj = tile[k];
            const double ddx = bj.x - bi.x, ddy = bj.y - bi.y, ddz = bj.z - bi.z;
            if (ddx == 0.0 && ddy == 0.0 && ddz == 0.0) continue;  // equal centres
            const float dx = (float)ddx, dy = (float)ddy, dz = (float)ddz;
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (r2 == 0.f) continue;  // separation below FP32 range
            const float inv_r = rsqrtf(r2);
            const float phi = e > 0.f ? atanf(se * inv_r) * inv_se : inv_r;
            part = fmaf((float)bj.w, phi, part);
        }
        acc += (double)part;
    }
    double v = i < n ? -0.5 * bi.w * acc : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ double red[kDiagThreads / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kDiagThreads / 32; ++w) s += red[w];
        atomicAdd(&out[8], s);
    }
}

}  // namespace

// out[0..8]: mass, m*x, m*y, m*z, m*vx, m*vy, m*vz, kinetic, potential (f64)
int launch_diagnostics(const DeviceBodies &b, double e, double *d_out, bool potential,
                       int device, cudaStream_t st)
{
    PG_CUDA(cudaMemsetAsync(d_out, 0, 9 * sizeof(double), st));
    if (b.n == 0) return PHYSIM_OK;
    const int n = (int)b.n;
    moments_kernel<<<2 * device_sm_count(device), kDiagThreads, 0, st>>>(b.x, b.y, b.z, b.vx, b.vy,
                                                                     b.vz, b.m, n, d_out);
    if (potential) {
        const int chunk = 16384;
        dim3 grid((n + kDiagThreads - 1) / kDiagThreads, (n + chunk - 1) / chunk);
        potential_kernel<<<grid, kDiagThreads, 0, st>>>(b.x, b.y, b.z, b.m, n, (float)e, chunk,
                                                        d_out);
    }
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg

// ---------------------------------------------------------------------------
// Diagnostics of host Entity arrays (the energysink element's computation)
// ---------------------------------------------------------------------------
struct PhysimEnergy {
    int device = 0;
    cudaStream_t stream = nullptr;
    pg::DeviceBodies b;
    double *d_out = nullptr;
};

extern "C" int physim_gpu_energy_create(int32_t device, PhysimEnergy **out)
{
    PG_CHECK(out, PHYSIM_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    PG_CUDA(cudaSetDevice(device));
    PhysimEnergy *E = new (std::nothrow) PhysimEnergy();
    PG_CHECK(E, PHYSIM_ERR_MEMORY, "out of host memory");
    E->device = device;
    if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete E;
        pg::set_error("cudaStreamCreate failed");
        return PHYSIM_ERR_CUDA;
    }
    *out = E;
    return PHYSIM_OK;
}

extern "C" int physim_gpu_energy_compute(PhysimEnergy *E, const Entity *state, size_t n,
                                         double e, int with_potential, PhysimDiagnostics *out)
{
    using namespace pg;
    PG_CHECK(E && out && (state || n == 0), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(n < (size_t)INT32_MAX, PHYSIM_ERR_ARGUMENT, "too many bodies: %zu", n);
    memset(out, 0, sizeof *out);
    if (n == 0) return PHYSIM_OK;
    PG_CUDA(cudaSetDevice(E->device));
    PG_TRY(bodies_reserve(E->b, n, true, E->stream));
    if (!E->d_out) PG_TRY(dev_alloc(E->d_out, 9, E->stream));
    PG_CUDA(cudaMemcpyAsync(E->b.aos, state, n * sizeof(Entity), cudaMemcpyHostToDevice,
                            E->stream));
    PG_TRY(launch_unpack(E->b, E->b.aos, n, true, E->stream));
    PG_TRY(launch_diagnostics(E->b, fabs(e), E->d_out, with_potential != 0, E->device,
                              E->stream));
    double h[9];
    PG_CUDA(cudaMemcpyAsync(h, E->d_out, sizeof h, cudaMemcpyDeviceToHost, E->stream));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    out->mass = h[0];
    for (int c = 0; c < 3; ++c) {
        out->centre_of_mass[c] = h[0] != 0.0 ? h[1 + c] / h[0] : 0.0;
        out->momentum[c] = h[4 + c];
    }
    out->kinetic = h[7];
    out->potential = with_potential ? h[8] : 0.0;
    out->energy = out->kinetic + out->potential;
    return PHYSIM_OK;
}

extern "C" void physim_gpu_energy_destroy(PhysimEnergy *E)
{
    if (!E) return;
    cudaSetDevice(E->device);
    pg::bodies_free(E->b, E->stream);
    pg::dev_free(E->d_out, E->stream);
    cudaStreamSynchronize(E->stream);
    cudaStreamDestroy(E->stream);
    delete E;
}
