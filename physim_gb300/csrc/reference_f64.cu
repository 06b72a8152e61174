// reference_f64.cu -- the reference's direct-sum force in f64 for a sample of
// bodies (physim_gpu_sim_accelerations_f64): the accuracy yardstick for the
// FP32 pair kernels and the Barnes-Hut traversal, evaluated where the state
// already is.
//
// Per pair the reference (astro/src/lib.rs:84-113) computes, in f64,
//     d = x_a - x_b,  r = sqrt(d.d),  w = d.d + e,
//     F = ((x_b - x_a) / r) * G * m_a * m_b / w       (G = 1, lib.rs:27)
// skipping bodies at exactly the same position (transformers.rs:145,230), and
// a_i = (sum_j F_ij) / m_i.  Every operation here is an explicitly rounded
// f64 operation in that order (no contraction), so each pair term is the
// reference's bit for bit; only the order in which a body's terms are summed
// differs (a block of 256 threads, each summing a strided subset of j, then a
// fixed-order tree), which changes the result at the level of f64 rounding.
//
// GB300 issues f64 at a small fraction of its f32 rate (one correctly rounded
// f64 division per pair term costs ~19 ps of the whole GPU), so this path is
// for samples: 16,384 bodies against 1,048,580 take about two seconds.
#include "common.cuh"
#include "engine.h"

namespace pg {

namespace {

constexpr int kRefThreads = 256;

__global__ void __launch_bounds__(kRefThreads)
f64_sample_kernel(const double *__restrict__ x, const double *__restrict__ y,
                  const double *__restrict__ z, const double *__restrict__ m,
                  const uint8_t *__restrict__ fixed, int n, double e,
                  const int64_t *__restrict__ idx, Acceleration *__restrict__ out)
{
    __shared__ double red[3][kRefThreads];
    const int64_t i = idx[blockIdx.x];
    const double ax = x[i], ay = y[i], az = z[i], am = m[i];
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    for (int j = threadIdx.x; j < n; j += kRefThreads) {
        const double bx = x[j], by = y[j], bz = z[j];
        if (ax == bx && ay == by && az == bz) continue;
        const double d0 = __dsub_rn(ax, bx), d1 = __dsub_rn(ay, by), d2 = __dsub_rn(az, bz);
        const double dd = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)),
                                    __dmul_rn(d2, d2));
        const double r = __dsqrt_rn(dd);
        const double w = __dadd_rn(dd, e);
        const double bm = m[j];
        // ((b_k - a_k) / r) * G * m_a * m_b / w, G = 1 (a product by 1.0 is exact)
        f0 = __dadd_rn(f0, __ddiv_rn(__dmul_rn(__dmul_rn(__ddiv_rn(__dsub_rn(bx, ax), r), am), bm), w));
        f1 = __dadd_rn(f1, __ddiv_rn(__dmul_rn(__dmul_rn(__ddiv_rn(__dsub_rn(by, ay), r), am), bm), w));
        f2 = __dadd_rn(f2, __ddiv_rn(__dmul_rn(__dmul_rn(__ddiv_rn(__dsub_rn(bz, az), r), am), bm), w));
    }
    red[0][threadIdx.x] = f0;
    red[1][threadIdx.x] = f1;
    red[2][threadIdx.x] = f2;
    __syncthreads();
    for (int s = kRefThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int c = 0; c < 3; ++c)
                red[c][threadIdx.x] = __dadd_rn(red[c][threadIdx.x], red[c][threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        Acceleration a = {0.0, 0.0, 0.0};
        if (!fixed[i]) {
            a.x = __ddiv_rn(red[0][0], am);
            a.y = __ddiv_rn(red[1][0], am);
            a.z = __ddiv_rn(red[2][0], am);
        }
        out[blockIdx.x] = a;
    }
}

}  // namespace

int launch_f64_sample(const DeviceBodies &b, double e, const int64_t *d_idx, size_t count,
                      Acceleration *d_out, cudaStream_t stream)
{
    if (count == 0 || b.n == 0) return PHYSIM_OK;
    PG_CHECK(b.x != nullptr, PHYSIM_ERR_ARGUMENT, "no f64 state");
    PG_CHECK(count < (1u << 31), PHYSIM_ERR_ARGUMENT, "sample too large: %zu", count);
    f64_sample_kernel<<<(unsigned)count, kRefThreads, 0, stream>>>(b.x, b.y, b.z, b.m, b.fixed,
                                                                   (int)b.n, e, d_idx, d_out);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg
