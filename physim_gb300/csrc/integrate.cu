// integrate.cu -- body staging and the integrators on the device: verlet
// (integrators/src/verlet.rs:24-107), euler (integrators/src/euler.rs:17-49)
// and rk4 (integrators/src/rk4.rs:24-178).
//
// The integrator runs in f64 with the reference's operation order, written
// with explicit round-to-nearest intrinsics so the compiler cannot contract
// a*b+c into an FMA (Rust does not either).  Given the same accelerations,
// new positions and velocities are therefore bit-identical to the reference.
// The same kernel combines the pair kernel's partial sums, so one launch
// does combine + kick + drift + refresh of the f32 body copy.
#include <string.h>
#include <sys/mman.h>
#include <unistd.h>

#include <atomic>

// madvise advice values of Linux 5.14+ (absent from older headers)
#ifndef MADV_POPULATE_READ
#define MADV_POPULATE_READ 22
#endif
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23
#endif

#include "common.cuh"
#include "engine.h"

namespace pg {

namespace {

constexpr int kThreads = 256;

inline int blocks_for(size_t n) { return (int)((n + kThreads - 1) / kThreads); }

// Copies `bytes` (a multiple of 8) between global memory -- HBM, or the
// caller's host array reached through the host's page tables -- and shared
// memory with every thread of the block, as consecutive 16-byte words when
// both ends are 16-byte aligned, else 8-byte words.  An array of structs read
// one struct per thread touches a 32-byte sector per 8-byte field; this moves
// whole runs instead, which is what a link to host memory needs.
__device__ __forceinline__ void block_copy(void *dst, const void *src, int bytes)
{
    if (((((uintptr_t)dst | (uintptr_t)src) & 15) == 0) && (bytes & 15) == 0) {
        const int4 *s = (const int4 *)src;
        int4 *d = (int4 *)dst;
        for (int w = threadIdx.x; w < bytes / 16; w += blockDim.x) d[w] = s[w];
    } else {
        const long long *s = (const long long *)src;
        long long *d = (long long *)dst;
        for (int w = threadIdx.x; w < bytes / 8; w += blockDim.x) d[w] = s[w];
    }
}

__global__ void unpack_kernel(const Entity *__restrict__ in, int n, int n_pad, float4 *body4,
                              uint8_t *fixed, double *x, double *y, double *z, double *vx,
                              double *vy, double *vz, double *m, double *radius, uint64_t *id)
{
    __shared__ __align__(16) Entity s_in[kThreads];
    const int base = blockIdx.x * kThreads;
    const int count = min(kThreads, n - base);  // <= 0 for blocks of the padded tail
    if (count > 0) block_copy(s_in, in + base, count * (int)sizeof(Entity));
    __syncthreads();
    const int i = base + threadIdx.x;
    if (i >= n_pad) return;
    if (i >= n) {
        body4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const Entity en = s_in[threadIdx.x];
    body4[i] = make_float4((float)en.x, (float)en.y, (float)en.z, (float)en.mass);
    fixed[i] = en.fixed ? 1 : 0;
    m[i] = en.mass;
    if (x) {
        x[i] = en.x;
        y[i] = en.y;
        z[i] = en.z;
        vx[i] = en.vx;
        vy[i] = en.vy;
        vz[i] = en.vz;
        radius[i] = en.radius;
        id[i] = (uint64_t)en.id;
    }
}

__global__ void pack_kernel(Entity *out, int n, const uint8_t *fixed, const double *x,
                            const double *y, const double *z, const double *vx, const double *vy,
                            const double *vz, const double *m, const double *radius,
                            const uint64_t *id)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Entity en;
    memset(&en, 0, sizeof en);
    en.x = x[i];
    en.y = y[i];
    en.z = z[i];
    en.vx = vx[i];
    en.vy = vy[i];
    en.vz = vz[i];
    en.radius = radius[i];
    en.mass = m[i];
    en.id = (uintptr_t)id[i];
    en.fixed = fixed[i] != 0;
    out[i] = en;
}

// a_i from the partial sums; zero for fixed bodies (never accumulated);
// NaN for a massless body, whose reference value is F/m_i = 0/0.
__device__ __forceinline__ void body_acc(const double *partial, int splits, int n, int i,
                                         bool fixed, double mass, double &ax, double &ay,
                                         double &az)
{
    ax = ay = az = 0.0;
    if (fixed) return;
    for (int s = 0; s < splits; ++s) {
        ax += partial[(size_t)(s * 3 + 0) * n + i];
        ay += partial[(size_t)(s * 3 + 1) * n + i];
        az += partial[(size_t)(s * 3 + 2) * n + i];
    }
    if (mass == 0.0) ax = ay = az = __longlong_as_double(0x7ff8000000000000LL);
}

// The block's accelerations are read and written back as one contiguous run;
// a fixed body's entry is written back with the bits it was read with.
__global__ void accumulate_aos_kernel(const double *__restrict__ mass, const uint8_t *fixed,
                                      const double *partial, int splits, int n,
                                      Acceleration *acc)
{
    __shared__ __align__(16) Acceleration s_acc[kThreads];
    const int base = blockIdx.x * kThreads;
    const int count = min(kThreads, n - base);
    block_copy(s_acc, acc + base, count * (int)sizeof(Acceleration));
    __syncthreads();
    const int i = base + threadIdx.x;
    // transformers.rs:139-141: fixed bodies are left untouched
    if (i < n && !fixed[i]) {
        double ax, ay, az;
        body_acc(partial, splits, n, i, false, mass[i], ax, ay, az);
        Acceleration a = s_acc[threadIdx.x];
        a.x = __dadd_rn(a.x, ax);
        a.y = __dadd_rn(a.y, ay);
        a.z = __dadd_rn(a.z, az);
        s_acc[threadIdx.x] = a;
    }
    __syncthreads();
    block_copy(acc + base, s_acc, count * (int)sizeof(Acceleration));
}

__global__ void combine_soa_kernel(const double *__restrict__ mass, const uint8_t *fixed,
                                   const double *partial, int splits, int n, double *acc)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double ax, ay, az;
    body_acc(partial, splits, n, i, fixed[i] != 0, mass[i], ax, ay, az);
    acc[i] = ax;
    acc[n + i] = ay;
    acc[2 * (size_t)n + i] = az;
}

// verlet.rs:33-39 (initial, Taylor step) and verlet.rs:64-70 (regular).
__device__ __forceinline__ void verlet_axis(double &x, double &v, double &p, double a, double dt,
                                            double dt2, bool initial)
{
    double xn, vn;
    if (initial) {
        // x + vx*dt + 0.5*a*dt^2 ; vx + a*dt
        xn = __dadd_rn(__dadd_rn(x, __dmul_rn(v, dt)), __dmul_rn(__dmul_rn(0.5, a), dt2));
        vn = __dadd_rn(v, __dmul_rn(a, dt));
    } else {
        // 2*x - prev + a*dt^2 ; (x' - x)/dt
        xn = __dadd_rn(__dsub_rn(__dmul_rn(2.0, x), p), __dmul_rn(a, dt2));
        vn = __ddiv_rn(__dsub_rn(xn, x), dt);
    }
    p = x;
    x = xn;
    v = vn;
}

__global__ void verlet_kernel(float4 *body4, const double *mass, const uint8_t *fixed,
                              const double *partial,
                              int splits, int n, double *x, double *y, double *z, double *vx,
                              double *vy, double *vz, double *px, double *py, double *pz,
                              double dt, int initial)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 b = body4[i];
    double ax, ay, az;
    body_acc(partial, splits, n, i, fixed[i] != 0, mass[i], ax, ay, az);
    const double dt2 = __dmul_rn(dt, dt);
    double xi = x[i], yi = y[i], zi = z[i];
    double vxi = vx[i], vyi = vy[i], vzi = vz[i];
    double pxi = px[i], pyi = py[i], pzi = pz[i];
    verlet_axis(xi, vxi, pxi, ax, dt, dt2, initial);
    verlet_axis(yi, vyi, pyi, ay, dt, dt2, initial);
    verlet_axis(zi, vzi, pzi, az, dt, dt2, initial);
    x[i] = xi; y[i] = yi; z[i] = zi;
    vx[i] = vxi; vy[i] = vyi; vz[i] = vzi;
    px[i] = pxi; py[i] = pyi; pz[i] = pzi;
    b.x = (float)xi;
    b.y = (float)yi;
    b.z = (float)zi;
    body4[i] = b;
}

__global__ void verlet_aos_kernel(const Entity *in, const Entity *prev, Entity *out, Entity *keep,
                                  const Acceleration *acc, int n, double dt, int initial)
{
    __shared__ __align__(16) Entity s_e[kThreads];
    __shared__ __align__(16) Acceleration s_a[kThreads];
    const int base = blockIdx.x * kThreads;
    const int count = min(kThreads, n - base);
    block_copy(s_e, in + base, count * (int)sizeof(Entity));
    block_copy(s_a, acc + base, count * (int)sizeof(Acceleration));
    __syncthreads();
    if (keep) block_copy(keep + base, s_e, count * (int)sizeof(Entity));
    const int i = base + threadIdx.x;
    double x = 0.0, y = 0.0, z = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
    if (i < n) {
        const Entity &en = s_e[threadIdx.x];
        x = en.x;
        y = en.y;
        z = en.z;
        vx = en.vx;
        vy = en.vy;
        vz = en.vz;
        const Acceleration a = s_a[threadIdx.x];
        const double dt2 = __dmul_rn(dt, dt);
        double px = 0.0, py = 0.0, pz = 0.0;
        if (!initial) {
            px = prev[i].x;
            py = prev[i].y;
            pz = prev[i].z;
        }
        verlet_axis(x, vx, px, a.x, dt, dt2, initial);
        verlet_axis(y, vy, py, a.y, dt, dt2, initial);
        verlet_axis(z, vz, pz, a.z, dt, dt2, initial);
    }
    __syncthreads();  // every read of s_e (the keep copy) is done
    // Only the six updated fields are rewritten: every other byte of the
    // output record, struct padding included, is the input's.
    if (i < n) {
        Entity &en = s_e[threadIdx.x];
        en.x = x;
        en.y = y;
        en.z = z;
        en.vx = vx;
        en.vy = vy;
        en.vz = vz;
    }
    __syncthreads();
    block_copy(out + base, s_e, count * (int)sizeof(Entity));
}

// euler.rs:29-37: x + vx*dt + 0.5*a*dt^2 ; vx + a*dt for every body.  A fixed
// body has a = 0 (transforms skip it) and still drifts with its velocity.
__global__ void euler_kernel(float4 *body4, const double *mass, const uint8_t *fixed,
                             const double *partial, int splits, int n, double *x, double *y,
                             double *z, double *vx, double *vy, double *vz, double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 b = body4[i];
    double ax, ay, az;
    body_acc(partial, splits, n, i, fixed[i] != 0, mass[i], ax, ay, az);
    const double dt2 = __dmul_rn(dt, dt);
    double xi = x[i], yi = y[i], zi = z[i];
    double vxi = vx[i], vyi = vy[i], vzi = vz[i];
    double unused = 0.0;
    verlet_axis(xi, vxi, unused, ax, dt, dt2, true);
    verlet_axis(yi, vyi, unused, ay, dt, dt2, true);
    verlet_axis(zi, vzi, unused, az, dt, dt2, true);
    x[i] = xi; y[i] = yi; z[i] = zi;
    vx[i] = vxi; vy[i] = vyi; vz[i] = vzi;
    b.x = (float)xi;
    b.y = (float)yi;
    b.z = (float)zi;
    body4[i] = b;
}

// One RK4 stage (rk4.rs:33-178) for body i, given the stage state q (x, y, z,
// vx, vy, vz), its acceleration a, the entity's own state e and the running
// sum S of the k's.  k = (dt v_q, dt a) (rk4.rs:40-46); S accumulates
// k1 + 2 k2 + 2 k3 + k4 left to right, as rk4.rs:160-165 evaluates it.
// Stages 1-3 return the next stage state e + k/2 (stages 1, 2) or e + k
// (stage 3); stage 4 returns the new state e + S/6, or (e, v = 0) for a fixed
// body (rk4.rs:165-171).
__device__ __forceinline__ void rk4_stage(int stage, const double q[6], const double a[3],
                                          const double e[6], double S[6], bool fixed, double dt,
                                          double out[6])
{
    double k[6];
    for (int c = 0; c < 3; ++c) {
        k[c] = __dmul_rn(dt, q[3 + c]);
        k[3 + c] = __dmul_rn(dt, a[c]);
    }
    for (int c = 0; c < 6; ++c) {
        if (stage == 1)
            S[c] = k[c];
        else if (stage == 4)
            S[c] = __dadd_rn(S[c], k[c]);
        else
            S[c] = __dadd_rn(S[c], __dmul_rn(2.0, k[c]));
    }
    if (stage < 3) {
        for (int c = 0; c < 6; ++c) out[c] = __dadd_rn(e[c], __dmul_rn(0.5, k[c]));
    } else if (stage == 3) {
        for (int c = 0; c < 6; ++c) out[c] = __dadd_rn(e[c], k[c]);
    } else if (!fixed) {
        for (int c = 0; c < 6; ++c) out[c] = __dadd_rn(e[c], __ddiv_rn(S[c], 6.0));
    } else {
        for (int c = 0; c < 3; ++c) {
            out[c] = e[c];
            out[3 + c] = 0.0;
        }
    }
}

// Device-resident RK4 stage: the stage state is in (x .. vz) and body4; the
// entity's state is saved in `save` at stage 1; S lives in `ksum`.  Writes
// the next stage state (or the new state) back to (x .. vz) and body4, so
// the next force evaluation reads it like any other state.
__global__ void rk4_stage_kernel(float4 *body4, const double *mass, const uint8_t *fixed,
                                 const double *partial, int splits, int n, double *x, double *y,
                                 double *z, double *vx, double *vy, double *vz, double *save,
                                 double *ksum, double dt, int stage)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool fx = fixed[i] != 0;
    double a[3];
    body_acc(partial, splits, n, i, fx, mass[i], a[0], a[1], a[2]);
    double *st[6] = {x, y, z, vx, vy, vz};
    double q[6], e[6], S[6], out[6];
    for (int c = 0; c < 6; ++c) q[c] = st[c][i];
    if (stage == 1) {
        for (int c = 0; c < 6; ++c) {
            e[c] = q[c];
            save[(size_t)c * n + i] = q[c];
        }
    } else {
        for (int c = 0; c < 6; ++c) {
            e[c] = save[(size_t)c * n + i];
            S[c] = ksum[(size_t)c * n + i];
        }
    }
    rk4_stage(stage, q, a, e, S, fx, dt, out);
    if (stage < 4)
        for (int c = 0; c < 6; ++c) ksum[(size_t)c * n + i] = S[c];
    for (int c = 0; c < 6; ++c) st[c][i] = out[c];
    float4 b = body4[i];
    b.x = (float)out[0];
    b.y = (float)out[1];
    b.z = (float)out[2];
    body4[i] = b;
}

__global__ void euler_aos_kernel(const Entity *in, Entity *out, const Acceleration *acc, int n,
                                 double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Entity en = in[i];
    const Acceleration a = acc[i];
    const double dt2 = __dmul_rn(dt, dt);
    double unused = 0.0;
    verlet_axis(en.x, en.vx, unused, a.x, dt, dt2, true);
    verlet_axis(en.y, en.vy, unused, a.y, dt, dt2, true);
    verlet_axis(en.z, en.vz, unused, a.z, dt, dt2, true);
    out[i] = en;
}

// RK4 stage over Entity arrays: `ent` the entities, `q` the stage state, f
// its accelerations; writes the next stage state (stages 1-3: the entity with
// x, v replaced, rk4.rs:50-62) or the new state (stage 4) to `out`, which may
// alias q.
__global__ void rk4_aos_stage_kernel(const Entity *ent, const Entity *q_in,
                                     const Acceleration *f, double *ksum, Entity *out, int n,
                                     double dt, int stage)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Entity en = ent[i];
    const Entity qe = q_in[i];
    const Acceleration fa = f[i];
    const double q[6] = {qe.x, qe.y, qe.z, qe.vx, qe.vy, qe.vz};
    const double e[6] = {en.x, en.y, en.z, en.vx, en.vy, en.vz};
    const double a[3] = {fa.x, fa.y, fa.z};
    double S[6] = {0, 0, 0, 0, 0, 0}, r[6];
    if (stage > 1)
        for (int c = 0; c < 6; ++c) S[c] = ksum[(size_t)c * n + i];
    rk4_stage(stage, q, a, e, S, en.fixed, dt, r);
    if (stage < 4)
        for (int c = 0; c < 6; ++c) ksum[(size_t)c * n + i] = S[c];
    Entity o = en;
    o.x = r[0]; o.y = r[1]; o.z = r[2];
    o.vx = r[3]; o.vy = r[4]; o.vz = r[5];
    out[i] = o;
}

}  // namespace

int dev_alloc_bytes(void **p, size_t bytes, cudaStream_t stream)
{
    *p = nullptr;
    int device = 0;
    if (cudaGetDevice(&device) == cudaSuccess && device >= 0 && device < 64) {
        // keep freed blocks in the device's default pool for reuse (a
        // setting of this process's pool only)
        static bool pool_set[64] = {false};
        if (!pool_set[device]) {
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
                uint64_t keep = ~0ull;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
            pool_set[device] = true;
        }
    }
    cudaError_t err = cudaMallocAsync(p, bytes ? bytes : 1, stream);
    if (err != cudaSuccess) {
        *p = nullptr;
        set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(err));
        return PHYSIM_ERR_MEMORY;
    }
    return PHYSIM_OK;
}

void dev_free(void *p, cudaStream_t stream)
{
    if (p) cudaFreeAsync(p, stream);
}

namespace {
std::atomic<uint32_t> g_host_access{PHYSIM_HOST_ACCESS_AUTO};
std::atomic<int> g_pageable[64];  // 0 unknown, 1 no, 2 yes
}  // namespace

int host_direct(int device, bool *direct)
{
    *direct = false;
    const uint32_t mode = g_host_access.load(std::memory_order_relaxed);
    if (mode == PHYSIM_HOST_ACCESS_COPY) return PHYSIM_OK;
    PG_CHECK(device >= 0 && device < 64, PHYSIM_ERR_ARGUMENT, "device %d out of range", device);
    int known = g_pageable[device].load(std::memory_order_relaxed);
    if (known == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                   device) != cudaSuccess)
            v = 0;
        known = v ? 2 : 1;
        g_pageable[device].store(known, std::memory_order_relaxed);
    }
    PG_CHECK(known == 2 || mode == PHYSIM_HOST_ACCESS_AUTO, PHYSIM_ERR_ARGUMENT,
             "host access DIRECT: device %d does not reach pageable host memory through the "
             "host's page tables",
             device);
    *direct = known == 2;
    return PHYSIM_OK;
}

void bodies_free(DeviceBodies &b, cudaStream_t stream)
{
    void *ptrs[] = {b.body4, b.fixed, b.x,  b.y,  b.z,      b.vx, b.vy,    b.vz,
                    b.px,    b.py,    b.pz, b.m,  b.radius, b.id, b.aos, b.scale};
    for (void *p : ptrs) dev_free(p, stream);
    b = DeviceBodies();
}

int bodies_reserve(DeviceBodies &b, size_t n, bool with_state, cudaStream_t stream)
{
    size_t need = pad_bodies(n);
    if (need <= b.cap && (!with_state || b.x)) {
        b.n = n;
        return PHYSIM_OK;
    }
    bodies_free(b, stream);
    b.cap = need;
    b.n = n;
    PG_TRY(dev_alloc(b.body4, need, stream));
    PG_TRY(dev_alloc(b.fixed, need, stream));
    PG_TRY(dev_alloc(b.aos, need, stream));
    PG_TRY(dev_alloc(b.m, need, stream));
    PG_TRY(dev_alloc(b.scale, 1, stream));
    PG_CUDA(cudaMemsetAsync(b.scale, 0, sizeof(PairScale), stream));
    if (with_state) {
        double **d[] = {&b.x, &b.y, &b.z, &b.vx, &b.vy, &b.vz, &b.px, &b.py, &b.pz, &b.radius};
        for (double **p : d) PG_TRY(dev_alloc(*p, need, stream));
        PG_TRY(dev_alloc(b.id, need, stream));
    }
    return PHYSIM_OK;
}

int launch_unpack(DeviceBodies &b, const Entity *aos, size_t n, bool full_state,
                  cudaStream_t stream)
{
    size_t n_pad = pad_bodies(n);
    if (n_pad == 0) return PHYSIM_OK;
    unpack_kernel<<<blocks_for(n_pad), kThreads, 0, stream>>>(
        aos, (int)n, (int)n_pad, b.body4, b.fixed, full_state ? b.x : nullptr, b.y, b.z, b.vx,
        b.vy, b.vz, b.m, b.radius, b.id);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_pack(DeviceBodies &b, cudaStream_t stream)
{
    if (b.n == 0) return PHYSIM_OK;
    pack_kernel<<<blocks_for(b.n), kThreads, 0, stream>>>(b.aos, (int)b.n, b.fixed, b.x, b.y,
                                                            b.z, b.vx, b.vy, b.vz, b.m,
                                                            b.radius, b.id);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_accumulate_aos(const DeviceBodies &b, const double *partial, int splits,
                          Acceleration *d_acc, cudaStream_t stream)
{
    if (b.n == 0) return PHYSIM_OK;
    accumulate_aos_kernel<<<blocks_for(b.n), kThreads, 0, stream>>>(b.m, b.fixed, partial,
                                                                      splits, (int)b.n, d_acc);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_combine_soa(const DeviceBodies &b, const double *partial, int splits,
                       double *acc_soa, cudaStream_t stream)
{
    if (b.n == 0) return PHYSIM_OK;
    combine_soa_kernel<<<blocks_for(b.n), kThreads, 0, stream>>>(b.m, b.fixed, partial,
                                                                   splits, (int)b.n, acc_soa);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_verlet(DeviceBodies &b, const double *partial, int splits, double dt, bool initial,
                  cudaStream_t stream)
{
    if (b.n == 0) return PHYSIM_OK;
    verlet_kernel<<<blocks_for(b.n), kThreads, 0, stream>>>(
        b.body4, b.m, b.fixed, partial, splits, (int)b.n, b.x, b.y, b.z, b.vx, b.vy, b.vz, b.px, b.py,
        b.pz, dt, initial ? 1 : 0);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_euler(DeviceBodies &b, const double *partial, int splits, double dt,
                 cudaStream_t stream)
{
    if (b.n == 0) return PHYSIM_OK;
    euler_kernel<<<blocks_for(b.n), kThreads, 0, stream>>>(b.body4, b.m, b.fixed, partial, splits,
                                                           (int)b.n, b.x, b.y, b.z, b.vx, b.vy,
                                                           b.vz, dt);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_rk4_stage(DeviceBodies &b, const double *partial, int splits, double dt, int stage,
                     double *save, double *ksum, cudaStream_t stream)
{
    if (b.n == 0) return PHYSIM_OK;
    PG_CHECK(stage >= 1 && stage <= 4, PHYSIM_ERR_ARGUMENT, "rk4 stage %d", stage);
    rk4_stage_kernel<<<blocks_for(b.n), kThreads, 0, stream>>>(
        b.body4, b.m, b.fixed, partial, splits, (int)b.n, b.x, b.y, b.z, b.vx, b.vy, b.vz, save,
        ksum, dt, stage);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_euler_aos(const Entity *d_in, Entity *d_out, const Acceleration *d_acc, size_t n,
                     double dt, cudaStream_t stream)
{
    if (n == 0) return PHYSIM_OK;
    euler_aos_kernel<<<blocks_for(n), kThreads, 0, stream>>>(d_in, d_out, d_acc, (int)n, dt);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_rk4_aos_stage(const Entity *d_ent, const Entity *d_q, const Acceleration *d_f,
                         double *ksum, Entity *d_out, size_t n, double dt, int stage,
                         cudaStream_t stream)
{
    if (n == 0) return PHYSIM_OK;
    PG_CHECK(stage >= 1 && stage <= 4, PHYSIM_ERR_ARGUMENT, "rk4 stage %d", stage);
    rk4_aos_stage_kernel<<<blocks_for(n), kThreads, 0, stream>>>(d_ent, d_q, d_f, ksum, d_out,
                                                                 (int)n, dt, stage);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

int launch_verlet_aos(const Entity *in, const Entity *d_prev, Entity *out, Entity *keep,
                      const Acceleration *acc, size_t n, double dt, bool initial,
                      cudaStream_t stream)
{
    if (n == 0) return PHYSIM_OK;
    verlet_aos_kernel<<<blocks_for(n), kThreads, 0, stream>>>(in, d_prev, out, keep, acc, (int)n,
                                                              dt, initial ? 1 : 0);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg

void pg::host_prefault(const void *p, size_t bytes, bool write)
{
    if (!p || !bytes) return;
    static const uintptr_t page = (uintptr_t)sysconf(_SC_PAGESIZE);
    const uintptr_t lo = (uintptr_t)p & ~(page - 1);
    const uintptr_t hi = ((uintptr_t)p + bytes + page - 1) & ~(page - 1);
    (void)madvise((void *)lo, hi - lo, write ? MADV_POPULATE_WRITE : MADV_POPULATE_READ);
}

extern "C" int physim_gpu_set_host_access(uint32_t mode)
{
    PG_CHECK(mode <= PHYSIM_HOST_ACCESS_DIRECT, PHYSIM_ERR_ARGUMENT, "unknown host access mode %u",
             mode);
    pg::g_host_access.store(mode);
    return PHYSIM_OK;
}

extern "C" int physim_gpu_host_access(int32_t device, uint32_t *mode)
{
    PG_CHECK(mode, PHYSIM_ERR_ARGUMENT, "null argument");
    bool direct = false;
    PG_TRY(pg::host_direct(device, &direct));
    *mode = direct ? PHYSIM_HOST_ACCESS_DIRECT : PHYSIM_HOST_ACCESS_COPY;
    return PHYSIM_OK;
}
