// engine.h -- internal interfaces shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "physim_gb300.h"

namespace pg {

// Bodies are padded to a multiple of this many entries (zero mass at the
// origin), so every kernel can read whole tiles without bounds checks.
constexpr int kBodyPad = 1024;

inline size_t pad_bodies(size_t n) { return (n + kBodyPad - 1) / kBodyPad * kBodyPad; }

// Guard added to r^2 (r^2 + e)^2 before the reciprocal square root.  It makes
// the contribution of a body at exactly the same position zero (dx = 0 times
// a finite factor), which is the reference's "skip equal centres" rule
// (astro/src/transformers.rs:145,230), without a per-pair branch.  It is the
// smallest normal float, so it changes no pair whose (scaled, see PairScale)
// r^2 (r^2 + e)^2 exceeds 1.2e-31 by more than 1e-7 relative.
constexpr float kPairGuard = 1.17549435e-38f;

// ------------------------------------------------------------------------
// Power-of-two scaling of the pair law
// ------------------------------------------------------------------------
// The pair kernels evaluate r^2 (r^2 + e)^2 in FP32, which spans six times
// the exponent range of the coordinates: unscaled it overflows for
// separations above ~2.6e6 and underflows (e = 0) below ~5e-7.  A pair at
// one position (a body with itself, coincident bodies) contributes
// 0 * m / sqrt(guard), which needs m / sqrt(guard) finite.  So positions
// enter the pair arithmetic as p' = p 2^-k, with k chosen per force pass so
// the largest |coordinate| of the state maps into [0.5, 1), masses as
// m' = m 2^-km, the largest mass into [0.5, 1) (for Barnes-Hut: the total
// mass, the largest cell), the easing as e' = e 2^-2k, and the accelerations
// leave as a = a' 2^(km - 2k) -- every factor a power of two, so no bits are
// lost and a state that was in range before gives the same results.  k is
// clamped so that e' <= 2^60 (r'^2 (r'^2 + e')^2 then stays finite), k and km
// to [-100, 100].  What remains: with e = 0, pairs closer than ~3e-6 of the
// largest |coordinate| lose accuracy beyond 1e-5 relative, and closer than
// ~5e-7 of it they contribute almost nothing (r'^6 underflows into the guard).
constexpr int kScaleBlocks = 256;
struct PairScale {
    int32_t k;          // coordinate scale exponent of the current state
    int32_t km;         // mass scale exponent
    uint32_t arrivals;  // blocks of a running scale pass that finished (reset by the last)
    uint32_t pad;
    uint32_t blockmax[kScaleBlocks];   // per-block max |coordinate| (f32 bit patterns)
    uint32_t blockmass[kScaleBlocks];  // per-block max |mass|
};

// Exponent of the largest |coordinate| m: m = f 2^k, f in [0.5, 1) (0 for m = 0).
__host__ __device__ inline int coord_exp(float m)
{
    int k = 0;
    if (m > 0.f && m <= 3.4028235e38f) (void)frexpf(m, &k);
    return k;
}

// The scale exponent for coordinate exponent kx and easing e: kx, raised so
// that e 2^-2k <= 2^60, within [-100, 100].
__host__ __device__ inline int pair_scale_from(int kx, float e)
{
    int k = kx;
    if (e > 0.f && e <= 3.4028235e38f) {
        int ke = 0;
        (void)frexpf(e, &ke);  // e < 2^ke
        const int kmin = (ke - 60 + 1) >> 1;  // ceil((ke - 60) / 2)
        if (k < kmin) k = kmin;
    }
    return k < -100 ? -100 : (k > 100 ? 100 : k);
}

__host__ __device__ inline int pair_scale_exp(float m, float e)
{
    return pair_scale_from(coord_exp(m), e);
}

// Mass scale exponent for the largest |mass| m, within [-100, 100].
__host__ __device__ inline int mass_scale_exp(float m)
{
    const int k = coord_exp(m);
    return k < -100 ? -100 : (k > 100 ? 100 : k);
}

// Computes ps->k and ps->km for the n bodies of body4 (max over |x|, |y|,
// |z| and over |m|; NaN and infinite values skipped) and easing e, on
// `stream`: one launch whose last block to finish reduces the per-block
// maxima.  ps->arrivals must be 0 before the first pass (it is left 0).
int launch_pair_scale(const float4 *body4, int n, float e, PairScale *ps, cudaStream_t stream);
// The coordinate pass over the members of an ensemble is done by its
// integrator kernel; host-side values for a state being uploaded:
float max_abs_coordinate(const Entity *state, size_t n);
float max_abs_mass(const Entity *state, size_t n);

// ------------------------------------------------------------------------
// Direct sum (simple_astro)
// ------------------------------------------------------------------------
struct DirectPlan {
    int block = 256;       // threads per block
    int ipt = 4;           // bodies per thread
    int splits = 1;        // j-range chunks (partial sums combined afterwards)
    int n = 0;             // bodies
    int n_itiles = 0;      // i tiles of block*ipt bodies
    int n_jtiles = 0;      // j tiles of `block` bodies
    int chunk_tiles = 0;   // j tiles per split
    bool compensated = true;
    // Every unordered pair evaluated once (direct_sym.cu): `tiles` body tiles
    // of 1,024; the partial sums come out as one split, after f32 slot sums
    // the same allocation holds.  clusters: thread-block clusters over runs of
    // tiles (3T^2/32 slots of 3 x 1,024 floats); otherwise one block per tile
    // pair (one [3][n] slot per tile).
    bool symmetric = false;
    int tiles = 0;
    bool clusters = false;
};

// Heuristic plan that fills the GPU: picks the i-tile shape and the number of
// j splits whose block count wastes least in the last wave.
DirectPlan plan_direct(int n, int device, bool compensated);
// The heuristic one-pair plan (never the symmetric one): the fallback when the
// symmetric plan's slot buffer cannot be allocated.
DirectPlan plan_direct_one_pair(int n, int device, bool compensated);
// A plan with a given shape and number of j splits (clamped to 1..j tiles).
DirectPlan make_direct_plan(int n, int block, int ipt, int splits, bool compensated);
// Enumerates the candidate plans the autotuner times for n bodies.
int direct_candidates(int n, int device, bool compensated, DirectPlan *out, int cap);

// Whether a one-pair kernel of this shape is built.
bool direct_shape_supported(int block, int ipt);
// The symmetric plan for n bodies (compensated sums only).
DirectPlan make_symmetric_plan(int n);
// Doubles the `partial` buffer of a plan must hold.
size_t direct_partial_doubles(const DirectPlan &plan);

// Launches the pair kernel.  body4: n_pad (x,y,z,m) f32 entries.  partial:
// direct_partial_doubles(plan) doubles; on return partial[(s*3+c)*n + i] for
// s < plan.splits holds the partial sums.  pairs_done (optional) is recorded
// on `stream` right after the pair kernel, before any reduction of its
// output (as an external event node when the stream is being captured).
// Before the pair kernel, launch_direct runs the scale pass of body4 into
// `scale` (see PairScale); the partial sums come out unscaled.
int launch_direct(const DirectPlan &plan, const float4 *body4, float e, PairScale *scale,
                  double *partial, cudaStream_t stream, cudaEvent_t pairs_done = nullptr);
int launch_direct_symmetric(const DirectPlan &plan, const float4 *body4, float e,
                            const PairScale *scale, double *partial, cudaStream_t stream,
                            cudaEvent_t pairs_done);
// Records `ev` on `stream`; inside a stream capture as an external event node.
int record_event(cudaEvent_t ev, cudaStream_t stream);

// ------------------------------------------------------------------------
// Body staging, integration and accumulation (integrate.cu)
// ------------------------------------------------------------------------
struct DeviceBodies {
    size_t n = 0, cap = 0;  // live bodies, allocated capacity (padded)
    float4 *body4 = nullptr;  // f32 (x,y,z,m), padded with zero-mass entries
    uint8_t *fixed = nullptr;
    double *x = nullptr, *y = nullptr, *z = nullptr;     // f64 positions
    double *vx = nullptr, *vy = nullptr, *vz = nullptr;  // f64 velocities
    double *px = nullptr, *py = nullptr, *pz = nullptr;  // verlet previous positions
    double *m = nullptr;                                  // f64 masses
    double *radius = nullptr;
    uint64_t *id = nullptr;
    Entity *aos = nullptr;  // staging for host<->device copies
    PairScale *scale = nullptr;  // pair-law scale of the direct-sum kernels
};

// Stream-ordered device memory (cudaMallocAsync / cudaFreeAsync on the
// owner's stream).  cudaMalloc and cudaFree synchronise the whole device, so
// objects created and destroyed while others run (the server's jobs) would
// stall every stream; stream-ordered allocation does not, and the device's
// default pool keeps freed memory for reuse.  count 0 allocates one element.
int dev_alloc_bytes(void **p, size_t bytes, cudaStream_t stream);
void dev_free(void *p, cudaStream_t stream);
template <typename T>
inline int dev_alloc(T *&p, size_t count, cudaStream_t stream)
{
    return dev_alloc_bytes((void **)&p, (count ? count : 1) * sizeof(T), stream);
}

// `stream` orders the allocations (and frees) with the owner's work.
int bodies_reserve(DeviceBodies &b, size_t n, bool with_state, cudaStream_t stream);
void bodies_free(DeviceBodies &b, cudaStream_t stream);

// True when calls on `device` hand the caller's host arrays to the kernels
// in place (PHYSIM_HOST_ACCESS_DIRECT, or AUTO on a device with pageable
// memory access through the host's page tables); false when they copy.
// Fails if DIRECT is requested on a device that cannot.
int host_direct(int device, bool *direct);
// Before kernels touch a host array in place: maps every page of
// [p, p + bytes) into the process (writable if `write`), without changing its
// contents, so the GPU meets no page that was never touched.  A GPU access to
// such a page (a freshly mmap'd output array) is a fault the host's kernel
// serves one page at a time, an order of magnitude slower than the same
// fault taken on the CPU.  Best effort: a range the host's kernel will not
// populate (not host memory, an older kernel) is left to the GPU's faults.
void host_prefault(const void *p, size_t bytes, bool write);

// Unpacks an Entity array into the SoA arrays.  `aos` may be device memory
// or, where host_direct() holds, the caller's host array: each block reads
// its 256 entities as one contiguous run.
int launch_unpack(DeviceBodies &b, const Entity *aos, size_t n, bool full_state,
                  cudaStream_t stream);
// Packs the SoA state back into b.aos.
int launch_pack(DeviceBodies &b, cudaStream_t stream);

// acc[i] += a_i (f64) for each non-fixed body, a_i = sum over splits of the
// partial sums; NaN for a massless body (the reference divides F by m_i).
int launch_accumulate_aos(const DeviceBodies &b, const double *partial, int splits,
                          Acceleration *d_acc, cudaStream_t stream);
// acc_soa[c*n + i] = a_i (f64).
int launch_combine_soa(const DeviceBodies &b, const double *partial, int splits,
                       double *acc_soa, cudaStream_t stream);
// Verlet step (verlet.rs:24-82) fused with the combine of the partial sums,
// updating the f64 state and the f32 body copy in place.
int launch_verlet(DeviceBodies &b, const double *partial, int splits, double dt, bool initial,
                  cudaStream_t stream);

// Euler step (euler.rs:17-49) fused with the combine of the partial sums.
int launch_euler(DeviceBodies &b, const double *partial, int splits, double dt,
                 cudaStream_t stream);
// RK4 stage 1..4 (rk4.rs:24-178) after the forces of the stage state: saves
// the entity state (stage 1, `save`: 6 x n f64), accumulates the k's (`ksum`:
// 6 x n f64) and writes the next stage state, or the new state at stage 4,
// to the f64 state and the f32 body copy.
int launch_rk4_stage(DeviceBodies &b, const double *partial, int splits, double dt, int stage,
                     double *save, double *ksum, cudaStream_t stream);
// Euler and RK4 stages over explicit Entity arrays (host-array integrators).
int launch_euler_aos(const Entity *d_in, Entity *d_out, const Acceleration *d_acc, size_t n,
                     double dt, cudaStream_t stream);
int launch_rk4_aos_stage(const Entity *d_ent, const Entity *d_q, const Acceleration *d_f,
                         double *ksum, Entity *d_out, size_t n, double dt, int stage,
                         cudaStream_t stream);

// Verlet over explicit Entity arrays (the host-array integrator path).  in,
// out and acc may be host arrays where host_direct() holds; prev and keep
// are device memory.  keep (optional) receives a copy of in, the next
// call's previous state.
int launch_verlet_aos(const Entity *in, const Entity *d_prev, Entity *out, Entity *keep,
                      const Acceleration *acc, size_t n, double dt, bool initial,
                      cudaStream_t stream);

// The reference's direct-sum accelerations in f64 (reference per-pair
// operation order) of the bodies d_idx[0..count) of b's f64 state, into
// d_out[0..count) (reference_f64.cu).  Indices must be in [0, b.n).
int launch_f64_sample(const DeviceBodies &b, double e, const int64_t *d_idx, size_t count,
                      Acceleration *d_out, cudaStream_t stream);

// Whole-system f64 diagnostics into d_out[0..8]: mass, m*x, m*y, m*z,
// m*vx, m*vy, m*vz, kinetic energy, potential energy (if `potential`).
int launch_diagnostics(const DeviceBodies &b, double e, double *d_out, bool potential,
                       int device, cudaStream_t stream);

// The cube (kind 0, PhysimCubeParams) or plummer (kind 1, PhysimPlummerParams)
// initialiser written as n Entities to d_out (init.cu).
int launch_generate(int kind, const void *params, Entity *d_out, size_t n, cudaStream_t stream);

// Device count / SM count helpers (cached).
int device_sm_count(int device);

}  // namespace pg
