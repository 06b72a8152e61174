// ensemble.cu -- many independent direct-sum simulations of uneven size in
// one persistent launch per step (physim_gpu_ensemble_*).
//
// Each member is one physim pipeline (simple_astro + verlet,
// astro/src/transformers.rs:219-244, integrators/src/verlet.rs:24-107) with
// its own bodies, easing factor, time step and step budget.  Per step:
//   1. one persistent pair kernel: blocks (SMs x resident blocks) pull work
//      units (member, i tile, j chunk) from a list sorted longest-first
//      through an atomic counter, so 256-body and 65,536-body members share
//      the GPU without a tail; the pair arithmetic is direct_tile, the same
//      code as the per-simulation kernel;
//   2. one kernel combining the partial sums and applying verlet in f64 for
//      every member with steps left, then counting the step.
// Members from a plan's size threshold up evaluate each unordered pair once
// (direct_sym_tile.cuh): a second persistent kernel pulls their 1,024-body
// tile pairs, writing per-member f32 slot sums that the verlet kernel adds
// with TwoSum; smaller members keep the one-pair units.
// One step is captured once (per work plan) into a CUDA graph and replayed
// for every step.  Members can be resized in place (a finished member's slot
// takes the next job; the work plan is rebuilt).  The autotuner times the candidate kernel shapes (threads x bodies per thread)
// and j-chunk lengths on the members' own data and keeps the fastest.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "direct_sym_tile.cuh"
#include "direct_tile.cuh"
#include "engine.h"

namespace pg {
namespace {

struct MemberInfo {
    int32_t off;          // first slot of the member in the concatenated arrays
    int32_t n;            // bodies
    int32_t n_jtiles;     // j tiles of the current shape
    int32_t chunk_tiles;  // j tiles per work unit
    int64_t poff;         // first partial sum of the member
    int32_t splits;
    float e;
    double dt;
    int32_t sym_tiles;    // > 0: tiles of the symmetric units, slot sums at soff
    int32_t pad;
    int64_t soff;         // first f32 slot sum of the member
};

struct WorkUnit {
    int32_t member, itile, split, pad;
};

// A tile pair (I, J), I <= J, of a member on the symmetric units.
struct SymUnit {
    int32_t member, I, J, pad;
};

template <int BLOCK, int IPT, bool COMP>
__global__ void __launch_bounds__(BLOCK, 2)
ensemble_forces_kernel(const float4 *__restrict__ body4, const MemberInfo *__restrict__ members,
                       const WorkUnit *__restrict__ units, int n_units,
                       const unsigned long long *__restrict__ remaining, int *__restrict__ counter,
                       const int32_t *__restrict__ member_kx, const int32_t *__restrict__ member_km,
                       double *__restrict__ partial)
{
    __shared__ float4 tile[2][BLOCK][2];
    __shared__ int next;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(counter, 1);
        __syncthreads();
        const int u = next;
        if (u >= n_units) return;
        const WorkUnit w = units[u];
        if (remaining[w.member] != 0) {
            const MemberInfo m = members[w.member];
            const int t0 = w.split * m.chunk_tiles;
            const int t1 = min(t0 + m.chunk_tiles, m.n_jtiles);
            direct_tile<BLOCK, IPT, COMP>(body4 + m.off, m.n, w.itile * BLOCK * IPT, t0, t1, m.e,
                                          pair_scale_from(member_kx[w.member], m.e),
                                          member_km[w.member],
                                          partial + m.poff + (size_t)w.split * 3 * m.n, tile);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSymThreads, 3)
ensemble_sym_kernel(const float4 *__restrict__ body4, const MemberInfo *__restrict__ members,
                    const SymUnit *__restrict__ units, int n_units,
                    const unsigned long long *__restrict__ remaining, int *__restrict__ counter,
                    const int32_t *__restrict__ member_kx, const int32_t *__restrict__ member_km,
                    float *__restrict__ slots)
{
    __shared__ float jacc[kSymWarps][kSymTile][3];
    __shared__ int next;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(counter, 1);
        __syncthreads();
        const int u = next;
        if (u >= n_units) return;
        const SymUnit w = units[u];
        if (remaining[w.member] != 0) {
            const MemberInfo m = members[w.member];
            const int sk = pair_scale_from(member_kx[w.member], m.e), skm = member_km[w.member];
            if (w.I == w.J)
                sym_tile_pair<true>(body4 + m.off, m.n, w.I, w.J, m.e, sk, skm, slots + m.soff,
                                    jacc);
            else
                sym_tile_pair<false>(body4 + m.off, m.n, w.I, w.J, m.e, sk, skm, slots + m.soff,
                                     jacc);
        }
        __syncthreads();
    }
}

// Combine + verlet for every member with steps left (verlet.rs:24-82; the
// first step after an upload is the Taylor step).  slot_member[s] < 0 marks
// padding.  Each warp also folds the largest |coordinate| of its new f32
// positions into member_ext of its member (members are padded to whole
// 1,024-slot tiles, so a warp's slots belong to one member); the count
// kernel turns it into the member's next pair scale.
__global__ void ensemble_verlet_kernel(float4 *body4, const double *__restrict__ mass,
                                       const uint8_t *__restrict__ fixed,
                                       const int32_t *__restrict__ slot_member,
                                       const MemberInfo *__restrict__ members,
                                       const unsigned long long *__restrict__ remaining,
                                       const unsigned long long *__restrict__ done,
                                       const double *__restrict__ partial,
                                       const float *__restrict__ slot_sums, int slots, double *x,
                                       double *y, double *z, double *vx, double *vy, double *vz,
                                       double *px, double *py, double *pz,
                                       const int32_t *__restrict__ member_kx,
                                       const int32_t *__restrict__ member_km,
                                       uint32_t *__restrict__ member_ext)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = s < slots ? slot_member[s] : -1;
    const bool active = k >= 0 && remaining[k] != 0;
    uint32_t ext = 0;
    if (active) {
        const MemberInfo m = members[k];
        const int i = s - m.off;
        double ax = 0.0, ay = 0.0, az = 0.0;
        if (!fixed[s]) {
            if (m.sym_tiles > 0) {
                // the member's slot sums, TwoSum-compensated in slot order, unscaled
                const size_t n3 = 3 * (size_t)m.n;
                const float *p = slot_sums + m.soff + i;
                float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
                for (int t = 0; t < m.sym_tiles; ++t)
                    for (int c = 0; c < 3; ++c) {
                        float sum, err;
                        two_sum(h[c], p[(size_t)t * n3 + (size_t)c * m.n], sum, err);
                        h[c] = sum;
                        l[c] += err;
                    }
                const double unsc =
                    pow2d(member_km[k] - 2 * pair_scale_from(member_kx[k], m.e));
                ax = ((double)h[0] + (double)l[0]) * unsc;
                ay = ((double)h[1] + (double)l[1]) * unsc;
                az = ((double)h[2] + (double)l[2]) * unsc;
            } else {
                for (int sp = 0; sp < m.splits; ++sp) {
                    const double *p = partial + m.poff + (size_t)sp * 3 * m.n;
                    ax += p[i];
                    ay += p[m.n + i];
                    az += p[2 * (size_t)m.n + i];
                }
            }
            if (mass[s] == 0.0) ax = ay = az = __longlong_as_double(0x7ff8000000000000LL);
        }
        const bool initial = done[k] == 0;
        const double dt = m.dt, dt2 = __dmul_rn(dt, dt);
        double q[3] = {x[s], y[s], z[s]}, v[3] = {vx[s], vy[s], vz[s]},
               pr[3] = {px[s], py[s], pz[s]};
        const double a[3] = {ax, ay, az};
        for (int c = 0; c < 3; ++c) {
            double xn, vn;
            if (initial) {
                xn = __dadd_rn(__dadd_rn(q[c], __dmul_rn(v[c], dt)),
                               __dmul_rn(__dmul_rn(0.5, a[c]), dt2));
                vn = __dadd_rn(v[c], __dmul_rn(a[c], dt));
            } else {
                xn = __dadd_rn(__dsub_rn(__dmul_rn(2.0, q[c]), pr[c]), __dmul_rn(a[c], dt2));
                vn = __ddiv_rn(__dsub_rn(xn, q[c]), dt);
            }
            pr[c] = q[c];
            q[c] = xn;
            v[c] = vn;
        }
        x[s] = q[0]; y[s] = q[1]; z[s] = q[2];
        vx[s] = v[0]; vy[s] = v[1]; vz[s] = v[2];
        px[s] = pr[0]; py[s] = pr[1]; pz[s] = pr[2];
        float4 b = body4[s];
        b.x = (float)q[0];
        b.y = (float)q[1];
        b.z = (float)q[2];
        body4[s] = b;
        const uint32_t ex = __float_as_uint(b.x) & 0x7fffffffu;
        const uint32_t ey = __float_as_uint(b.y) & 0x7fffffffu;
        const uint32_t ez = __float_as_uint(b.z) & 0x7fffffffu;
        ext = max(ext, ex < 0x7f800000u ? ex : 0u);  // NaN and infinities skipped
        ext = max(ext, ey < 0x7f800000u ? ey : 0u);
        ext = max(ext, ez < 0x7f800000u ? ez : 0u);
    }
    const uint32_t wext = __reduce_max_sync(0xffffffffu, ext);
    const int wk = (int)__reduce_max_sync(0xffffffffu, (uint32_t)(k + 1)) - 1;
    const bool any = __any_sync(0xffffffffu, active);
    if ((threadIdx.x & 31) == 0 && any && wk >= 0 && wext != 0) atomicMax(&member_ext[wk], wext);
}

__global__ void ensemble_count_kernel(unsigned long long *remaining, unsigned long long *done,
                                      int count, int *counter, int32_t *member_kx,
                                      uint32_t *member_ext)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) counter[0] = counter[1] = 0;  // the next step's work queues start empty
    if (k >= count || remaining[k] == 0) return;
    // the pair scale of the member's new positions (kept if all sit at the origin)
    const uint32_t ext = member_ext[k];
    if (ext != 0u) member_kx[k] = coord_exp(__uint_as_float(ext));
    member_ext[k] = 0u;
    done[k] += 1;
    if (remaining[k] != ~0ull) remaining[k] -= 1;
}

__global__ void ensemble_unpack_kernel(const Entity *__restrict__ in, int n, int off, float4 *body4,
                                       uint8_t *fixed, double *x, double *y, double *z,
                                       double *vx, double *vy, double *vz, double *m,
                                       double *radius, uint64_t *id)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Entity en = in[i];
    const int s = off + i;
    body4[s] = make_float4((float)en.x, (float)en.y, (float)en.z, (float)en.mass);
    fixed[s] = en.fixed ? 1 : 0;
    x[s] = en.x; y[s] = en.y; z[s] = en.z;
    vx[s] = en.vx; vy[s] = en.vy; vz[s] = en.vz;
    m[s] = en.mass;
    radius[s] = en.radius;
    id[s] = (uint64_t)en.id;
}

__global__ void ensemble_pack_kernel(Entity *out, int n, int off, const uint8_t *fixed,
                                     const double *x, const double *y, const double *z,
                                     const double *vx, const double *vy, const double *vz,
                                     const double *m, const double *radius, const uint64_t *id)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = off + i;
    Entity en;
    memset(&en, 0, sizeof en);
    en.x = x[s]; en.y = y[s]; en.z = z[s];
    en.vx = vx[s]; en.vy = vy[s]; en.vz = vz[s];
    en.radius = radius[s];
    en.mass = m[s];
    en.id = (uintptr_t)id[s];
    en.fixed = fixed[s] != 0;
    out[i] = en;
}

// A member's slot range [off, off + slot_len): the first n slots belong to
// member k, the rest are padding (member -1, zero mass, fixed).
__global__ void ensemble_slot_kernel(int32_t *slot_member, float4 *body4, uint8_t *fixed,
                                     double *m, int off, int slot_len, int n, int k)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slot_len) return;
    const int s = off + i;
    if (i < n) {
        slot_member[s] = k;
    } else {
        slot_member[s] = -1;
        body4[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        fixed[s] = 1;
        m[s] = 0.0;
    }
}

struct Shape {
    int block, ipt;
};
constexpr Shape kShapes[] = {{128, 2}, {128, 4}, {256, 4}, {256, 2}, {128, 8}};
constexpr int kChunks[] = {4096, 8192, 16384, 65536};
constexpr int kMinChunk = 4096;  // smallest j chunk any plan uses (sizes the partial sums)
// Default size from which members use the symmetric units, and the thresholds
// the autotuner compares (INT32_MAX: none).
constexpr int kEnsembleSymMin = 16384;
constexpr int kSymMins[] = {8192, 16384, 32768, INT32_MAX};

template <int BLOCK, int IPT>
void *ens_kernel_ptr(bool comp)
{
    return comp ? (void *)ensemble_forces_kernel<BLOCK, IPT, true>
                : (void *)ensemble_forces_kernel<BLOCK, IPT, false>;
}

void *ens_kernel(int block, int ipt, bool comp)
{
    if (block == 128 && ipt == 2) return ens_kernel_ptr<128, 2>(comp);
    if (block == 128 && ipt == 4) return ens_kernel_ptr<128, 4>(comp);
    if (block == 256 && ipt == 4) return ens_kernel_ptr<256, 4>(comp);
    if (block == 256 && ipt == 2) return ens_kernel_ptr<256, 2>(comp);
    if (block == 128 && ipt == 8) return ens_kernel_ptr<128, 8>(comp);
    return nullptr;
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace
}  // namespace pg

using namespace pg;

struct PhysimEnsemble {
    PhysimSimConfig cfg;
    int device = 0;
    bool own_stream = false;
    cudaStream_t stream = nullptr;
    std::vector<size_t> sizes;
    std::vector<size_t> caps;  // bodies each member's slot was created for
    std::vector<int32_t> offsets;
    std::vector<MemberInfo> members;
    int slots = 0;
    // device state (concatenated, every member padded to kBodyPad slots)
    float4 *body4 = nullptr;
    uint8_t *fixed = nullptr;
    double *x = nullptr, *y = nullptr, *z = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr;
    double *px = nullptr, *py = nullptr, *pz = nullptr, *m = nullptr, *radius = nullptr;
    uint64_t *id = nullptr;
    int32_t *slot_member = nullptr;
    MemberInfo *d_members = nullptr;
    WorkUnit *d_units = nullptr;
    int n_units = 0;
    size_t units_cap = 0;
    unsigned long long *remaining = nullptr, *done = nullptr;
    int *counter = nullptr;  // [0] one-pair units, [1] symmetric units
    int32_t *member_kx = nullptr;    // coordinate exponent of each member's pair scale
    int32_t *member_km = nullptr;    // mass scale exponent of each member
    uint32_t *member_ext = nullptr;  // largest |coordinate| of the new positions (f32 bits)
    double *partial = nullptr;
    SymUnit *d_sym_units = nullptr;
    int n_sym_units = 0;
    size_t sym_units_cap = 0;
    float *slot_sums = nullptr;  // f32 slot sums of the symmetric members
    size_t slot_cap = 0;
    int sym_grid = 0;
    Entity *staging = nullptr;
    size_t staging_cap = 0;
    // plan
    int block = 128, ipt = 4, chunk = 16384;
    int sym_min = kEnsembleSymMin;  // members from this many bodies use the symmetric units
    int grid = 0;
    bool tuned = false;
    double tuned_ms = 0.0;
    int candidates = 0;
    // graph of `graph_steps` steps
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    uint32_t graph_steps = 0;
};

namespace {

template <typename T>
int ealloc(PhysimEnsemble *E, T *&p, size_t count)
{
    return dev_alloc(p, count, E->stream);
}

void drop_graph(PhysimEnsemble *E)
{
    if (E->graph_exec) cudaGraphExecDestroy(E->graph_exec);
    if (E->graph) cudaGraphDestroy(E->graph);
    E->graph_exec = nullptr;
    E->graph = nullptr;
    E->graph_steps = 0;
}

// Builds member tiling and the work list for (block, ipt, chunk) and uploads them.
int plan_ensemble(PhysimEnsemble *E, int block, int ipt, int chunk, int sym_min)
{
    const int chunk_tiles = std::max(1, chunk / block);
    {
        // the members' slot sums grow as n^2 (12 B per body and 1,024-body
        // tile); above a quarter of the device's memory every member takes
        // the one-pair units
        size_t slot_bytes = 0, free_b = 0, total_b = 0;
        for (const MemberInfo &mi : E->members)
            if (mi.n >= sym_min)
                slot_bytes += (pad_bodies((size_t)mi.n) / kSymTile) * 12 * (size_t)mi.n;
        if (slot_bytes > 0 &&
            (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || slot_bytes > total_b / 4))
            sym_min = INT32_MAX;
    }
    std::vector<WorkUnit> units;
    std::vector<SymUnit> sym_units;
    std::vector<long long> cost;
    int64_t poff = 0, soff = 0;
    for (size_t k = 0; k < E->members.size(); ++k) {
        MemberInfo &mi = E->members[k];
        mi.n_jtiles = cdiv(mi.n, block);
        mi.chunk_tiles = chunk_tiles;
        mi.splits = std::max(1, cdiv(mi.n_jtiles, chunk_tiles));
        mi.poff = poff;
        mi.sym_tiles = 0;
        mi.soff = soff;
        if (mi.n >= sym_min && E->cfg.compensated != 0) {
            // each unordered pair once: all tile pairs of the member
            const int T = (int)(pad_bodies((size_t)mi.n) / kSymTile);
            mi.sym_tiles = T;
            mi.splits = 0;
            soff += (int64_t)T * 3 * mi.n;
            for (int J = 0; J < T; ++J)
                for (int I = 0; I <= J; ++I) sym_units.push_back({(int32_t)k, I, J, 0});
            continue;
        }
        poff += (int64_t)mi.splits * 3 * mi.n;
        const int n_itiles = cdiv(mi.n, block * ipt);
        for (int it = 0; it < n_itiles; ++it)
            for (int sp = 0; sp < mi.splits; ++sp) {
                const int t0 = sp * chunk_tiles, t1 = std::min(t0 + chunk_tiles, mi.n_jtiles);
                units.push_back({(int32_t)k, it, sp, 0});
                cost.push_back((long long)(t1 - t0));
            }
    }
    // longest units first (all units of one i-tile width cost ~ their j tiles)
    std::vector<int> order(units.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<WorkUnit> sorted(units.size());
    for (size_t i = 0; i < order.size(); ++i) sorted[i] = units[order[i]];
    if (sorted.size() > E->units_cap) {
        dev_free(E->d_units, E->stream);
        E->d_units = nullptr;
        PG_TRY(ealloc(E, E->d_units, sorted.size()));
        E->units_cap = sorted.size();
    }
    if (sym_units.size() > E->sym_units_cap) {
        dev_free(E->d_sym_units, E->stream);
        E->d_sym_units = nullptr;
        PG_TRY(ealloc(E, E->d_sym_units, sym_units.size()));
        E->sym_units_cap = sym_units.size();
    }
    if ((size_t)soff > E->slot_cap) {
        dev_free(E->slot_sums, E->stream);
        E->slot_sums = nullptr;
        PG_TRY(ealloc(E, E->slot_sums, (size_t)soff));
        E->slot_cap = (size_t)soff;
    }
    if (!sorted.empty())
        PG_CUDA(cudaMemcpyAsync(E->d_units, sorted.data(), sorted.size() * sizeof(WorkUnit),
                                cudaMemcpyHostToDevice, E->stream));
    if (!sym_units.empty())
        PG_CUDA(cudaMemcpyAsync(E->d_sym_units, sym_units.data(),
                                sym_units.size() * sizeof(SymUnit), cudaMemcpyHostToDevice,
                                E->stream));
    PG_CUDA(cudaMemcpyAsync(E->d_members, E->members.data(), E->members.size() * sizeof(MemberInfo),
                            cudaMemcpyHostToDevice, E->stream));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    E->n_units = (int)sorted.size();
    E->n_sym_units = (int)sym_units.size();
    E->block = block;
    E->ipt = ipt;
    E->chunk = chunk;
    E->sym_min = sym_min;
    int per_sm = 1;
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, ens_kernel(block, ipt, E->cfg.compensated != 0), block, 0));
    E->grid = std::max(1, per_sm) * device_sm_count(E->device);
    int sym_per_sm = 1;
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sym_per_sm, ensemble_sym_kernel,
                                                          kSymThreads, 0));
    E->sym_grid = std::max(1, sym_per_sm) * device_sm_count(E->device);
    drop_graph(E);
    return PHYSIM_OK;
}

int launch_forces(PhysimEnsemble *E)
{
    if (E->n_sym_units > 0) {
        ensemble_sym_kernel<<<std::min(E->sym_grid, E->n_sym_units), kSymThreads, 0, E->stream>>>(
            E->body4, E->d_members, E->d_sym_units, E->n_sym_units, E->remaining, E->counter + 1,
            E->member_kx, E->member_km, E->slot_sums);
        PG_CUDA(cudaGetLastError());
    }
    if (E->n_units == 0) return PHYSIM_OK;
    void *fn = ens_kernel(E->block, E->ipt, E->cfg.compensated != 0);
    PG_CHECK(fn, PHYSIM_ERR_ARGUMENT, "no ensemble kernel for %d x %d", E->block, E->ipt);
    void *args[] = {(void *)&E->body4, (void *)&E->d_members, (void *)&E->d_units,
                    (void *)&E->n_units, (void *)&E->remaining, (void *)&E->counter,
                    (void *)&E->member_kx, (void *)&E->member_km, (void *)&E->partial};
    PG_CUDA(cudaLaunchKernel(fn, dim3(E->grid), dim3(E->block), args, 0, E->stream));
    return PHYSIM_OK;
}

int enqueue_step(PhysimEnsemble *E)
{
    PG_TRY(launch_forces(E));
    const int t = 256;
    ensemble_verlet_kernel<<<cdiv(E->slots, t), t, 0, E->stream>>>(
        E->body4, E->m, E->fixed, E->slot_member, E->d_members, E->remaining, E->done, E->partial,
        E->slot_sums, E->slots, E->x, E->y, E->z, E->vx, E->vy, E->vz, E->px, E->py, E->pz,
        E->member_kx, E->member_km, E->member_ext);
    ensemble_count_kernel<<<cdiv((long long)E->members.size(), 256), 256, 0, E->stream>>>(
        E->remaining, E->done, (int)E->members.size(), E->counter, E->member_kx, E->member_ext);
    PG_CUDA(cudaGetLastError());
    return PHYSIM_OK;
}

void free_ensemble(PhysimEnsemble *E)
{
    drop_graph(E);
    void *p[] = {E->body4, E->fixed, E->x,  E->y,  E->z,  E->vx, E->vy, E->vz, E->px, E->py,
                 E->pz,    E->m,     E->radius, E->id, E->slot_member, E->d_members, E->d_units,
                 E->remaining, E->done, E->counter, E->partial, E->staging,
                 E->d_sym_units, E->slot_sums, E->member_kx, E->member_km, E->member_ext};
    for (void *q : p) dev_free(q, E->stream);
    if (E->stream) cudaStreamSynchronize(E->stream);
}

}  // namespace

extern "C" {

int physim_gpu_ensemble_create(const PhysimSimConfig *cfg, const size_t *sizes, size_t count,
                               PhysimEnsemble **out)
{
    PG_CHECK(cfg && out && (sizes || count == 0), PHYSIM_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    PG_CHECK(cfg->gravity == PHYSIM_GRAVITY_SIMPLE_ASTRO, PHYSIM_ERR_ARGUMENT,
             "ensembles run the simple_astro element");
    PG_CHECK(count > 0 && count < (1u << 24), PHYSIM_ERR_ARGUMENT, "member count %zu", count);
    PG_CUDA(cudaSetDevice(cfg->device));
    PhysimEnsemble *E = new (std::nothrow) PhysimEnsemble();
    PG_CHECK(E, PHYSIM_ERR_MEMORY, "out of host memory");
    E->cfg = *cfg;
    E->cfg.e = fabs(cfg->e);
    E->device = cfg->device;
    E->sizes.assign(sizes, sizes + count);
    E->caps.assign(sizes, sizes + count);
    long long slots = 0;
    long long partial_elems = 0;
    E->members.resize(count);
    for (size_t k = 0; k < count; ++k) {
        if (sizes[k] == 0 || sizes[k] >= (1u << 26)) {
            delete E;
            set_error("member %zu has %zu bodies (1 .. 2^26 allowed)", k, sizes[k]);
            return PHYSIM_ERR_ARGUMENT;
        }
        MemberInfo mi = {};
        mi.off = (int32_t)slots;
        mi.n = (int32_t)sizes[k];
        mi.e = (float)E->cfg.e;
        mi.dt = E->cfg.dt;
        E->members[k] = mi;
        slots += (long long)pad_bodies(sizes[k]);
        partial_elems += 3LL * (long long)sizes[k] * cdiv((long long)sizes[k], kMinChunk);
    }
    if (slots >= (1LL << 31)) {
        delete E;
        set_error("ensemble too large: %lld slots", slots);
        return PHYSIM_ERR_ARGUMENT;
    }
    E->slots = (int)slots;
    int rc = PHYSIM_OK;
    if (cfg->stream) {
        E->stream = (cudaStream_t)cfg->stream;
    } else if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) == cudaSuccess) {
        E->own_stream = true;
    } else {
        rc = PHYSIM_ERR_CUDA;
    }
#define EA(ptr, cnt)                                                                        \
    if (rc == PHYSIM_OK) rc = ealloc(E, ptr, cnt)
    EA(E->body4, slots);
    EA(E->fixed, slots);
    EA(E->x, slots);
    EA(E->y, slots);
    EA(E->z, slots);
    EA(E->vx, slots);
    EA(E->vy, slots);
    EA(E->vz, slots);
    EA(E->px, slots);
    EA(E->py, slots);
    EA(E->pz, slots);
    EA(E->m, slots);
    EA(E->radius, slots);
    EA(E->id, slots);
    EA(E->slot_member, slots);
    EA(E->d_members, count);
    EA(E->remaining, count);
    EA(E->done, count);
    EA(E->counter, 2);
    EA(E->member_kx, count);
    EA(E->member_km, count);
    EA(E->member_ext, count);
    EA(E->partial, partial_elems);
#undef EA
    if (rc == PHYSIM_OK) {
        // zero state (padding slots: zero mass, fixed) and the slot map
        std::vector<int32_t> map((size_t)slots, -1);
        for (size_t k = 0; k < count; ++k)
            for (size_t i = 0; i < sizes[k]; ++i) map[E->members[k].off + i] = (int32_t)k;
        std::vector<unsigned long long> rem(count, 0ull), dn(count, 0ull);
        if (cudaMemsetAsync(E->body4, 0, slots * sizeof(float4), E->stream) != cudaSuccess ||
            cudaMemsetAsync(E->fixed, 1, slots, E->stream) != cudaSuccess ||
            cudaMemsetAsync(E->m, 0, slots * sizeof(double), E->stream) != cudaSuccess ||
            cudaMemsetAsync(E->counter, 0, 2 * sizeof(int), E->stream) != cudaSuccess ||
            cudaMemsetAsync(E->member_kx, 0, count * sizeof(int32_t), E->stream) != cudaSuccess ||
            cudaMemsetAsync(E->member_km, 0, count * sizeof(int32_t), E->stream) != cudaSuccess ||
            cudaMemsetAsync(E->member_ext, 0, count * sizeof(uint32_t), E->stream) != cudaSuccess ||
            cudaMemcpyAsync(E->slot_member, map.data(), map.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice, E->stream) != cudaSuccess ||
            cudaMemcpyAsync(E->remaining, rem.data(), count * sizeof(unsigned long long),
                            cudaMemcpyHostToDevice, E->stream) != cudaSuccess ||
            cudaMemcpyAsync(E->done, dn.data(), count * sizeof(unsigned long long),
                            cudaMemcpyHostToDevice, E->stream) != cudaSuccess ||
            cudaStreamSynchronize(E->stream) != cudaSuccess) {
            set_error("ensemble initialisation failed");
            rc = PHYSIM_ERR_CUDA;
        }
    }
    if (rc == PHYSIM_OK) rc = plan_ensemble(E, 128, 4, 16384, kEnsembleSymMin);
    if (rc != PHYSIM_OK) {
        free_ensemble(E);
        if (E->own_stream) cudaStreamDestroy(E->stream);
        delete E;
        return rc;
    }
    *out = E;
    return PHYSIM_OK;
}

int physim_gpu_ensemble_upload(PhysimEnsemble *E, size_t index, const Entity *state, size_t n)
{
    PG_CHECK(E && state, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(index < E->members.size(), PHYSIM_ERR_ARGUMENT, "member %zu out of range", index);
    PG_CHECK(n == E->sizes[index], PHYSIM_ERR_ARGUMENT, "member %zu holds %zu bodies, not %zu",
             index, E->sizes[index], n);
    PG_CUDA(cudaSetDevice(E->device));
    if (n > E->staging_cap) {
        dev_free(E->staging, E->stream);
        E->staging = nullptr;
        PG_TRY(ealloc(E, E->staging, n));
        E->staging_cap = n;
    }
    PG_CUDA(cudaMemcpyAsync(E->staging, state, n * sizeof(Entity), cudaMemcpyHostToDevice,
                            E->stream));
    const int off = E->members[index].off;
    ensemble_unpack_kernel<<<cdiv((long long)n, 256), 256, 0, E->stream>>>(
        E->staging, (int)n, off, E->body4, E->fixed, E->x, E->y, E->z, E->vx, E->vy, E->vz, E->m,
        E->radius, E->id);
    PG_CUDA(cudaGetLastError());
    const unsigned long long zero = 0ull, all = ~0ull;
    // pair scale of the uploaded positions (the integrator keeps it current)
    const int32_t kx = coord_exp(max_abs_coordinate(state, n));
    const int32_t km = mass_scale_exp(max_abs_mass(state, n));  // masses do not change
    const uint32_t zero32 = 0u;
    PG_CUDA(cudaMemcpyAsync(E->member_kx + index, &kx, sizeof kx, cudaMemcpyHostToDevice,
                            E->stream));
    PG_CUDA(cudaMemcpyAsync(E->member_km + index, &km, sizeof km, cudaMemcpyHostToDevice,
                            E->stream));
    PG_CUDA(cudaMemcpyAsync(E->member_ext + index, &zero32, sizeof zero32,
                            cudaMemcpyHostToDevice, E->stream));
    PG_CUDA(cudaMemcpyAsync(E->done + index, &zero, sizeof zero, cudaMemcpyHostToDevice,
                            E->stream));
    PG_CUDA(cudaMemcpyAsync(E->remaining + index, &all, sizeof all, cudaMemcpyHostToDevice,
                            E->stream));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    return PHYSIM_OK;
}

int physim_gpu_ensemble_set_member(PhysimEnsemble *E, size_t index, double e, double dt,
                                   uint64_t steps_remaining)
{
    PG_CHECK(E, PHYSIM_ERR_ARGUMENT, "null ensemble");
    PG_CHECK(index < E->members.size(), PHYSIM_ERR_ARGUMENT, "member %zu out of range", index);
    PG_CUDA(cudaSetDevice(E->device));
    E->members[index].e = (float)fabs(e);
    E->members[index].dt = dt;
    PG_CUDA(cudaMemcpyAsync(E->d_members + index, &E->members[index], sizeof(MemberInfo),
                            cudaMemcpyHostToDevice, E->stream));
    const unsigned long long r = steps_remaining;
    PG_CUDA(cudaMemcpyAsync(E->remaining + index, &r, sizeof r, cudaMemcpyHostToDevice,
                            E->stream));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    return PHYSIM_OK;
}

int physim_gpu_ensemble_autotune(PhysimEnsemble *E, PhysimEnsembleTuning *out)
{
    PG_CHECK(E, PHYSIM_ERR_ARGUMENT, "null ensemble");
    PG_CUDA(cudaSetDevice(E->device));
    cudaEvent_t a, b;
    PG_CUDA(cudaEventCreate(&a));
    PG_CUDA(cudaEventCreate(&b));
    double best = 1e300;
    int bb = E->block, bi = E->ipt, bc = E->chunk, bs = E->sym_min, tried = 0;
    int rc = PHYSIM_OK;
    // one untimed + two timed force evaluations of a plan (the state is not advanced)
    auto time_plan = [&](int block, int ipt, int chunk, int sym_min) {
        rc = plan_ensemble(E, block, ipt, chunk, sym_min);
        float ms_total = 0.f;
        for (int rep = 0; rep < 3 && rc == PHYSIM_OK; ++rep) {
            if (cudaMemsetAsync(E->counter, 0, 2 * sizeof(int), E->stream) != cudaSuccess ||
                cudaEventRecord(a, E->stream) != cudaSuccess) {
                rc = PHYSIM_ERR_CUDA;
                break;
            }
            rc = launch_forces(E);
            if (rc != PHYSIM_OK) break;
            if (cudaEventRecord(b, E->stream) != cudaSuccess ||
                cudaEventSynchronize(b) != cudaSuccess) {
                rc = PHYSIM_ERR_CUDA;
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (rep > 0) ms_total += ms;
        }
        if (rc != PHYSIM_OK) return;
        ++tried;
        const double ms = ms_total / 2.0;
        if (ms < best) {
            best = ms;
            bb = block;
            bi = ipt;
            bc = chunk;
            bs = sym_min;
        }
    };
    // the one-pair shapes with the default threshold, then the thresholds
    // with the best shape
    for (const Shape &s : kShapes)
        for (int chunk : kChunks)
            if (rc == PHYSIM_OK) time_plan(s.block, s.ipt, chunk, kEnsembleSymMin);
    const int sb = bb, si = bi, sc = bc;
    for (int sym_min : kSymMins)
        if (rc == PHYSIM_OK && sym_min != kEnsembleSymMin) time_plan(sb, si, sc, sym_min);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc != PHYSIM_OK) {
        set_error("autotune failed: %s", last_error());
        return rc;
    }
    PG_CUDA(cudaMemsetAsync(E->counter, 0, 2 * sizeof(int), E->stream));
    PG_TRY(plan_ensemble(E, bb, bi, bc, bs));
    E->tuned = true;
    E->tuned_ms = best;
    E->candidates = tried;
    if (out) {
        out->block = (uint32_t)bb;
        out->ipt = (uint32_t)bi;
        out->chunk_bodies = (uint32_t)bc;
        out->candidates = (uint32_t)tried;
        out->symmetric_from = bs == INT32_MAX ? 0u : (uint32_t)bs;
        out->force_ms = best;
    }
    return PHYSIM_OK;
}

int physim_gpu_ensemble_resize_member(PhysimEnsemble *E, size_t index, size_t n)
{
    PG_CHECK(E, PHYSIM_ERR_ARGUMENT, "null ensemble");
    PG_CHECK(index < E->members.size(), PHYSIM_ERR_ARGUMENT, "member %zu out of range", index);
    PG_CHECK(n <= E->caps[index], PHYSIM_ERR_ARGUMENT,
             "member %zu was created for %zu bodies, not %zu", index, E->caps[index], n);
    PG_CUDA(cudaSetDevice(E->device));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    const int off = E->members[index].off;
    const int slot_len = (int)pad_bodies(E->caps[index]);
    ensemble_slot_kernel<<<cdiv(slot_len, 256), 256, 0, E->stream>>>(
        E->slot_member, E->body4, E->fixed, E->m, off, slot_len, (int)n, (int)index);
    PG_CUDA(cudaGetLastError());
    E->members[index].n = (int32_t)n;
    E->sizes[index] = n;
    const unsigned long long zero = 0ull;
    PG_CUDA(cudaMemcpyAsync(E->done + index, &zero, sizeof zero, cudaMemcpyHostToDevice,
                            E->stream));
    PG_CUDA(cudaMemcpyAsync(E->remaining + index, &zero, sizeof zero, cudaMemcpyHostToDevice,
                            E->stream));
    drop_graph(E);
    return plan_ensemble(E, E->block, E->ipt, E->chunk, E->sym_min);
}

int physim_gpu_ensemble_step(PhysimEnsemble *E, uint32_t steps)
{
    PG_CHECK(E, PHYSIM_ERR_ARGUMENT, "null ensemble");
    if (steps == 0) return PHYSIM_OK;
    PG_CUDA(cudaSetDevice(E->device));
    // one step is captured once per plan and replayed `steps` times, so the
    // step count of a call and re-plans (members resized) cost no re-capture
    // of long graphs
    if (!E->graph_exec) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        PG_CUDA(cudaStreamIsCapturing(E->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone) {  // the caller is capturing: plain launches
            for (uint32_t k = 0; k < steps; ++k) PG_TRY(enqueue_step(E));
            return PHYSIM_OK;
        }
        PG_CUDA(cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(E);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(E->stream, &g);
        if (rc != PHYSIM_OK || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (rc == PHYSIM_OK) set_error("graph capture failed: %s", cudaGetErrorString(ce));
            return rc != PHYSIM_OK ? rc : PHYSIM_ERR_CUDA;
        }
        if (cudaGraphInstantiate(&E->graph_exec, g, 0) != cudaSuccess) {
            cudaGraphDestroy(g);
            set_error("graph instantiation failed");
            return PHYSIM_ERR_CUDA;
        }
        E->graph = g;
        E->graph_steps = 1;
    }
    for (uint32_t k = 0; k < steps; ++k) PG_CUDA(cudaGraphLaunch(E->graph_exec, E->stream));
    return PHYSIM_OK;
}

int physim_gpu_ensemble_download(PhysimEnsemble *E, size_t index, Entity *state, size_t n)
{
    PG_CHECK(E && state, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(index < E->members.size(), PHYSIM_ERR_ARGUMENT, "member %zu out of range", index);
    PG_CHECK(n == E->sizes[index], PHYSIM_ERR_ARGUMENT, "member %zu holds %zu bodies, not %zu",
             index, E->sizes[index], n);
    PG_CUDA(cudaSetDevice(E->device));
    if (n > E->staging_cap) {
        dev_free(E->staging, E->stream);
        E->staging = nullptr;
        PG_TRY(ealloc(E, E->staging, n));
        E->staging_cap = n;
    }
    const int off = E->members[index].off;
    ensemble_pack_kernel<<<cdiv((long long)n, 256), 256, 0, E->stream>>>(
        E->staging, (int)n, off, E->fixed, E->x, E->y, E->z, E->vx, E->vy, E->vz, E->m, E->radius,
        E->id);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(state, E->staging, n * sizeof(Entity), cudaMemcpyDeviceToHost,
                            E->stream));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    return PHYSIM_OK;
}

int physim_gpu_ensemble_progress(PhysimEnsemble *E, uint64_t *steps_done, uint64_t *remaining)
{
    PG_CHECK(E, PHYSIM_ERR_ARGUMENT, "null ensemble");
    PG_CUDA(cudaSetDevice(E->device));
    const size_t c = E->members.size();
    if (steps_done)
        PG_CUDA(cudaMemcpyAsync(steps_done, E->done, c * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                E->stream));
    if (remaining)
        PG_CUDA(cudaMemcpyAsync(remaining, E->remaining, c * sizeof(uint64_t),
                                cudaMemcpyDeviceToHost, E->stream));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    return PHYSIM_OK;
}

int physim_gpu_ensemble_synchronize(PhysimEnsemble *E)
{
    PG_CHECK(E, PHYSIM_ERR_ARGUMENT, "null ensemble");
    PG_CUDA(cudaSetDevice(E->device));
    PG_CUDA(cudaStreamSynchronize(E->stream));
    return PHYSIM_OK;
}

void *physim_gpu_ensemble_stream(PhysimEnsemble *E) { return E ? (void *)E->stream : nullptr; }

int physim_gpu_ensemble_launches_per_step(PhysimEnsemble *E)
{
    if (!E) return 0;
    return 2 + (E->n_units > 0 ? 1 : 0) + (E->n_sym_units > 0 ? 1 : 0);
}

void physim_gpu_ensemble_destroy(PhysimEnsemble *E)
{
    if (!E) return;
    cudaSetDevice(E->device);
    if (E->stream) cudaStreamSynchronize(E->stream);
    free_ensemble(E);
    if (E->own_stream && E->stream) cudaStreamDestroy(E->stream);
    delete E;
}

}  // extern "C"
