// integrate.cu -- body staging and the verlet integrator
// (integrators/src/verlet.rs:24-107) on the device.
//
// The integrator runs in f64 with the reference's operation order, written
// with explicit round-to-nearest intrinsics so the compiler cannot contract
// a*b+c into an FMA (Rust does not either).  Given the same accelerations,
// new positions and velocities are therefore bit-identical to the reference.
// The same kernel combines the pair kernel's partial sums, so one launch
// does combine + kick + drift + refresh of the f32 body copy.
#include <string.h>

#include "common.cuh"
#include "engine.h"

namespace pg {

namespace {

constexpr int kThreads = 256;

inline int blocks_for(size_t n) { return (int)((n + kThreads - 1) / kThreads); }

__global__ void unpack_kernel(const Entity *__restrict__ in, int n, int n_pad, float4 *body4,
                              uint8_t *fixed, double *x, double *y, double *z, double *vx,
                              double *vy, double *vz, double *m, double *radius, uint64_t *id)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    if (i >= n) {
        body4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const Entity en = in[i];
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

__global__ void accumulate_aos_kernel(const double *__restrict__ mass, const uint8_t *fixed,
                                      const double *partial, int splits, int n,
                                      Acceleration *acc)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (fixed[i]) return;  // transformers.rs:139-141: fixed bodies are left untouched
    double ax, ay, az;
    body_acc(partial, splits, n, i, false, mass[i], ax, ay, az);
    Acceleration a = acc[i];
    a.x = __dadd_rn(a.x, ax);
    a.y = __dadd_rn(a.y, ay);
    a.z = __dadd_rn(a.z, az);
    acc[i] = a;
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

__global__ void verlet_aos_kernel(const Entity *in, const Entity *prev, Entity *out,
                                  const Acceleration *acc, int n, double dt, int initial)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Entity en = in[i];
    const Acceleration a = acc[i];
    const double dt2 = __dmul_rn(dt, dt);
    double px = 0.0, py = 0.0, pz = 0.0;
    if (!initial) {
        px = prev[i].x;
        py = prev[i].y;
        pz = prev[i].z;
    }
    verlet_axis(en.x, en.vx, px, a.x, dt, dt2, initial);
    verlet_axis(en.y, en.vy, py, a.y, dt, dt2, initial);
    verlet_axis(en.z, en.vz, pz, a.z, dt, dt2, initial);
    out[i] = en;
}

template <typename T>
int dalloc(T **p, size_t count)
{
    if (count == 0) count = 1;
    cudaError_t err = cudaMalloc((void **)p, count * sizeof(T));
    if (err != cudaSuccess) {
        *p = nullptr;
        set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T),
                  cudaGetErrorString(err));
        return PHYSIM_ERR_MEMORY;
    }
    return PHYSIM_OK;
}

}  // namespace

void bodies_free(DeviceBodies &b)
{
    void *ptrs[] = {b.body4, b.fixed, b.x,  b.y,  b.z,      b.vx, b.vy,
                    b.vz,    b.px,    b.py, b.pz, b.m,      b.radius, b.id, b.aos};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    b = DeviceBodies();
}

int bodies_reserve(DeviceBodies &b, size_t n, bool with_state)
{
    size_t need = pad_bodies(n);
    if (need <= b.cap && (!with_state || b.x)) {
        b.n = n;
        return PHYSIM_OK;
    }
    bodies_free(b);
    b.cap = need;
    b.n = n;
    PG_TRY(dalloc(&b.body4, need));
    PG_TRY(dalloc(&b.fixed, need));
    PG_TRY(dalloc(&b.aos, need));
    PG_TRY(dalloc(&b.m, need));
    if (with_state) {
        double **d[] = {&b.x, &b.y, &b.z, &b.vx, &b.vy, &b.vz, &b.px, &b.py, &b.pz, &b.radius};
        for (double **p : d) PG_TRY(dalloc(p, need));
        PG_TRY(dalloc(&b.id, need));
    }
    return PHYSIM_OK;
}

int launch_unpack(DeviceBodies &b, const Entity *d_aos, size_t n, bool full_state,
                  cudaStream_t stream)
{
    size_t n_pad = pad_bodies(n);
    if (n_pad == 0) return PHYSIM_OK;
    unpack_kernel<<<blocks_for(n_pad), kThreads, 0, stream>>>(
        d_aos, (int)n, (int)n_pad, b.body4, b.fixed, full_state ? b.x : nullptr, b.y, b.z, b.vx,
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

int launch_verlet_aos(const Entity *d_in, const Entity *d_prev, Entity *d_out,
                      const Acceleration *d_acc, size_t n, double dt, bool initial,
                      cudaStream_t stream)
{
    if (n == 0) return PHYSIM_OK;
    verlet_aos_kernel<<<blocks_for(n), kThreads, 0, stream>>>(d_in, d_prev, d_out, d_acc, (int)n,
                                                              dt, initial ? 1 : 0);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

}  // namespace pg
