// init.cu -- the `cube` and `plummer` initial-condition elements
// (astro/src/initialisers.rs:81-106 and :286-330) generated on the device.
//
// The reference draws its uniform variates from a ChaCha8 stream (rand_chacha,
// not part of the reference source), which cannot be reproduced, so the
// variates here come from a counter-based generator: variate k of body i is
// the SplitMix64 finaliser (Steele, Lea & Flood, OOPSLA 2014) of
// seed + (3 i + k + 1) * 0x9E3779B97F4A7C15, scaled to [0, 1) with 53 bits.
// Given the variates, every formula is the reference's, in its operation
// order, in f64.  Each body is independent, so a simulation of any size is
// initialised in one launch with no host-side generation or upload.
#include <math.h>

#include "common.cuh"
#include "engine.h"

namespace pg {

namespace {

__host__ __device__ inline double uniform53(uint64_t seed, uint64_t i, int k)
{
    uint64_t z = seed + (3ull * i + (uint64_t)k + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

constexpr double kPi = 3.14159265358979311600;  // f64::consts::PI

// initialisers.rs:81-106 with Entity::random (physim-core/src/lib.rs:115-128):
// x, y uniform in [-1, 1), z in [0, 1), radius 0.02; scaled by size; spin
// velocity (y s, -x s, 0) from the scaled position; then moved to the centre.
__global__ void cube_kernel(PhysimCubeParams p, int n, Entity *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Entity e;
    memset(&e, 0, sizeof e);
    e.x = __dadd_rn(-1.0, __dmul_rn(2.0, uniform53(p.seed, (uint64_t)i, 0)));
    e.y = __dadd_rn(-1.0, __dmul_rn(2.0, uniform53(p.seed, (uint64_t)i, 1)));
    e.z = uniform53(p.seed, (uint64_t)i, 2);
    e.radius = 0.02;
    e.x = __dmul_rn(e.x, p.size);
    e.y = __dmul_rn(e.y, p.size);
    e.z = __dmul_rn(e.z, p.size);
    e.vx = __dmul_rn(e.y, p.spin);
    e.vy = __dmul_rn(-e.x, p.spin);
    e.x = __dadd_rn(e.x, p.centre[0]);
    e.y = __dadd_rn(e.y, p.centre[1]);
    e.z = __dadd_rn(e.z, p.centre[2]);
    e.mass = __ddiv_rn(p.mass, (double)n);
    e.id = (uintptr_t)p.id;
    e.fixed = false;
    out[i] = e;
}

// initialisers.rs:286-330: r = a (c0^(-2/3) - 1)^(1/2), theta = pi c2,
// phi = 2 pi c1, radius 0.01, tangential speed spin sqrt(M r^2/(r^2+a^2)^1.5)
// plus the bulk velocity v.
__global__ void plummer_kernel(PhysimPlummerParams p, int n, Entity *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double c0 = uniform53(p.seed, (uint64_t)i, 0);
    const double c1 = uniform53(p.seed, (uint64_t)i, 1);
    const double c2 = uniform53(p.seed, (uint64_t)i, 2);
    const double m = __ddiv_rn(p.mass, (double)n);
    const double r = __dmul_rn(p.a, sqrt(__dsub_rn(pow(c0, -2.0 / 3.0), 1.0)));
    const double theta = __dmul_rn(kPi, c2);
    const double phi = __dmul_rn(__dmul_rn(2.0, kPi), c1);
    const double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
    Entity e;
    memset(&e, 0, sizeof e);
    e.x = __dadd_rn(__dmul_rn(__dmul_rn(r, st), cp), p.centre[0]);
    e.y = __dadd_rn(__dmul_rn(__dmul_rn(r, st), sp), p.centre[1]);
    e.z = __dadd_rn(__dmul_rn(r, ct), p.centre[2]);
    e.mass = m;
    e.radius = 0.01;
    const double r2 = __dmul_rn(r, r);
    const double a2 = __dmul_rn(p.a, p.a);
    const double v_phi =
        __dmul_rn(p.spin, sqrt(__ddiv_rn(__dmul_rn(p.mass, r2), pow(__dadd_rn(r2, a2), 1.5))));
    e.vx = __dadd_rn(__dmul_rn(-v_phi, sp), p.v[0]);
    e.vy = __dadd_rn(__dmul_rn(v_phi, cp), p.v[1]);
    e.vz = __dadd_rn(0.0, p.v[2]);
    e.id = (uintptr_t)p.id;
    e.fixed = false;
    out[i] = e;
}

}  // namespace

int launch_generate(int kind, const void *params, Entity *d_out, size_t n, cudaStream_t stream)
{
    if (n == 0) return PHYSIM_OK;
    PG_CHECK(n < (size_t)INT32_MAX, PHYSIM_ERR_ARGUMENT, "too many bodies: %zu", n);
    const int blocks = (int)((n + 255) / 256);
    if (kind == 0)
        cube_kernel<<<blocks, 256, 0, stream>>>(*(const PhysimCubeParams *)params, (int)n, d_out);
    else
        plummer_kernel<<<blocks, 256, 0, stream>>>(*(const PhysimPlummerParams *)params, (int)n,
                                                   d_out);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg
