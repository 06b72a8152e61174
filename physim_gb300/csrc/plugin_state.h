// plugin_state.h -- per-instance state of a transform element.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "engine.h"

namespace pg {

struct BhWorkspace;

constexpr int kMultipoleMonopole = 0;
constexpr int kMultipoleQuadrupole = 1;

struct ElementState {
    int kind = 0;  // 0 simple_astro, 1 astro2, 2 astro
    double theta = 1.0;
    double e = 1.0;
    int leaf_size = 1;
    int traversal = PHYSIM_TRAVERSAL_EXACT;
    int multipole = 0;       // kMultipoleMonopole / kMultipoleQuadrupole
    double com_theta = 0.0;  // centre-of-mass guard, 0 = off
    int device = 0;

    // GPU resources, created by the first transform.
    std::mutex lock;
    bool ready = false;
    cudaStream_t stream = nullptr;
    DeviceBodies bodies;
    Acceleration *d_acc = nullptr;
    size_t acc_cap = 0;
    double *partial = nullptr;
    size_t partial_cap = 0;
    DirectPlan plan;
    int plan_n = -1;
    BhWorkspace *bh = nullptr;
};

// acc[i] += a_i on host arrays (host->device copies, kernels, device->host).
int element_accumulate(ElementState *el, const Entity *state, size_t n, Acceleration *acc);
void element_destroy(ElementState *el);

// ------------------------------------------------------------------------
// Barnes-Hut (bh.cu)
// ------------------------------------------------------------------------
struct BhParams {
    int nchild = 8;  // 8 octree (astro2), 4 quadtree (astro)
    double theta = 1.0;
    double e = 1.0;
    int leaf_size = 1;
    int traversal = PHYSIM_TRAVERSAL_EXACT;
    bool compensated = true;
    // Accuracy options beyond the reference (defaults: off, the reference's
    // monopole cells and opening rule): quadrupole correction of accepted
    // cells, and the centre-of-mass guard b_max < com_theta |x - c|.
    int multipole = kMultipoleMonopole;
    double com_theta = 0.0;
};

// Allocations (and the frees of bh_free) are ordered on `stream`.
int bh_reserve(BhWorkspace *&ws, size_t n, int device, int leaf, cudaStream_t stream);
// Waits for the stream, then reports (and clears) the error flags the kernels
// raise: PHYSIM_ERR_TREE for a traversal stack overflow, PHYSIM_ERR_TIMEOUT
// for a radix-sort look-back wait that gave up.
int bh_check(BhWorkspace *ws, cudaStream_t st);
void bh_free(BhWorkspace *ws);
// Accelerations of the bodies in b (f64 positions and f32 copies must be
// current) into partial[c*n + i] (one split).
int bh_accelerations(BhWorkspace *ws, const DeviceBodies &b, const BhParams &p, double *partial,
                     cudaStream_t stream);
// Kernel launches one bh_accelerations call makes.
int bh_launches(const BhWorkspace *ws);
// Events around the traversal kernel; its last duration in milliseconds.
int bh_set_profiling(BhWorkspace *ws, bool enable);
int bh_traversal_ms(BhWorkspace *ws, double *ms);
// Node visits (per warp) and pair interactions (per body) of the last traversal.
int bh_stats(BhWorkspace *ws, cudaStream_t stream, uint64_t out[2]);
// Copies keys, sort order and tree of the last build to host arrays.
int bh_snapshot(BhWorkspace *ws, size_t n, cudaStream_t stream, PhysimTreeSnapshot *out);

}  // namespace pg
