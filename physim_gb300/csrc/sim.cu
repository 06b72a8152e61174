// sim.cu -- device-resident simulations (physim_gpu_sim_*) and the verlet
// integrator over host arrays (physim_gpu_verlet_*).
//
// A simulation restates one pipeline step of physim (pipeline.rs:137-173 with
// a single gravity transform and the verlet integrator, verlet.rs:85-107) but
// keeps the state in HBM: per step, the gravity kernels write per-body
// partial sums and one fused kernel combines them and applies the verlet
// update in f64, refreshing the f32 body copy the next step reads.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "plugin_state.h"

struct PhysimSim {
    PhysimSimConfig cfg;
    size_t n = 0;
    bool own_stream = false;
    cudaStream_t stream = nullptr;
    pg::DeviceBodies b;
    double *partial = nullptr;
    size_t partial_cap = 0;
    double *acc_soa = nullptr;
    pg::DirectPlan plan;
    pg::BhWorkspace *bh = nullptr;
    bool history = false;  // verlet previous_state is valid
    bool uploaded = false;
    // Optional per-step timing: events around the gravity kernels and the
    // integrator of the most recent step.
    bool profiling = false;
    // step start, gravity done, step done, pair kernel done (simple_astro)
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // The gravity phase of a step, captured once and replayed: the
    // Barnes-Hut build is ~100 short kernels whose launch cost would
    // otherwise dominate at small N.
    bool use_graph = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    double *diag = nullptr;  // 9 f64 diagnostics sums
    // rk4 (rk4.rs:24-178): the entity state saved at stage 1 and the running
    // sum of the k's, 6 x n f64 each
    double *rk4_save = nullptr, *rk4_ksum = nullptr;
};

struct PhysimIntegrator {
    uint32_t kind = 0;
    int device = 0;
    PhysimVerlet *verlet = nullptr;  // kind == verlet: previous_state lives here
    cudaStream_t stream = nullptr;
    Entity *d_ent = nullptr, *d_q = nullptr;  // entities, stage state
    Acceleration *d_acc = nullptr;
    double *d_ksum = nullptr;  // rk4 running sum of the k's, 6 x n
    Entity *h_q = nullptr;     // pinned host copy of the stage state for acc_fn
    Acceleration *h_acc = nullptr;
    size_t cap = 0;
};

struct PhysimVerlet {
    int device = 0;
    cudaStream_t stream = nullptr;
    Entity *d_in = nullptr, *d_prev = nullptr, *d_out = nullptr;
    Acceleration *d_acc = nullptr;
    size_t cap = 0;
    size_t prev_len = 0;  // length of previous_state (verlet.rs:102)
    bool has_prev = false;
};

namespace {

using namespace pg;

int sim_forces(PhysimSim *s, int *splits_out)
{
    const size_t n = s->n;
    const PhysimSimConfig &c = s->cfg;
    if (c.gravity == PHYSIM_GRAVITY_SIMPLE_ASTRO) {
        *splits_out = s->plan.splits;
        return launch_direct(s->plan, s->b.body4, (float)c.e, s->b.scale, s->partial, s->stream,
                             s->profiling ? s->ev[3] : nullptr);
    }
    BhParams p;
    p.nchild = c.gravity == PHYSIM_GRAVITY_ASTRO2 ? 8 : 4;
    p.theta = c.theta;
    p.e = c.e;
    p.leaf_size = (int)c.leaf_size;
    p.traversal = (int)c.traversal;
    p.compensated = c.compensated != 0;
    p.multipole = c.multipole == PHYSIM_MULTIPOLE_QUADRUPOLE ? kMultipoleQuadrupole
                                                             : kMultipoleMonopole;
    p.com_theta = c.com_theta;
    *splits_out = 1;
    (void)n;
    return bh_accelerations(s->bh, s->b, p, s->partial, s->stream);
}

// Captures the gravity phase into a graph.  If the stream cannot be captured
// (e.g. the caller is itself capturing), the simulation stays eager.
int sim_capture(PhysimSim *s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PG_CUDA(cudaStreamIsCapturing(s->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone) {
        s->use_graph = false;
        return PHYSIM_OK;
    }
    PG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int splits = 1;
    int rc = sim_forces(s, &splits);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
    if (rc != PHYSIM_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ce != cudaSuccess || !g) {
        (void)cudaGetLastError();
        s->use_graph = false;
        return PHYSIM_OK;
    }
    if (cudaGraphInstantiate(&s->graph_exec, g, 0) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaGraphDestroy(g);
        s->graph_exec = nullptr;
        s->use_graph = false;
        return PHYSIM_OK;
    }
    s->graph = g;
    return PHYSIM_OK;
}

}  // namespace

extern "C" {

void physim_gpu_sim_config_default(PhysimSimConfig *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof *cfg);
    cfg->gravity = PHYSIM_GRAVITY_SIMPLE_ASTRO;
    cfg->leaf_size = 1;
    cfg->traversal = PHYSIM_TRAVERSAL_EXACT;
    cfg->compensated = 1;
    cfg->theta = 1.0;
    cfg->e = 1.0;
    cfg->dt = 1e-6;
    cfg->stream = nullptr;
    cfg->device = 0;
    cfg->integrator = PHYSIM_INTEGRATOR_VERLET;
}

int physim_gpu_sim_create(const PhysimSimConfig *cfg, size_t n, PhysimSim **out)
{
    PG_CHECK(cfg && out, PHYSIM_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    PG_CHECK(cfg->gravity <= PHYSIM_GRAVITY_ASTRO, PHYSIM_ERR_ARGUMENT, "unknown gravity %u",
             cfg->gravity);
    PG_CHECK(cfg->leaf_size >= 1 && cfg->leaf_size <= 64, PHYSIM_ERR_ARGUMENT,
             "leaf_size %u outside 1..64", cfg->leaf_size);
    PG_CHECK(cfg->traversal <= PHYSIM_TRAVERSAL_WARP, PHYSIM_ERR_ARGUMENT, "unknown traversal");
    PG_CHECK(n < (size_t)INT32_MAX, PHYSIM_ERR_ARGUMENT, "too many bodies: %zu", n);
    PG_CHECK(cfg->integrator <= PHYSIM_INTEGRATOR_RK4, PHYSIM_ERR_ARGUMENT,
             "unknown integrator %u", cfg->integrator);
    PG_CHECK(cfg->multipole <= PHYSIM_MULTIPOLE_QUADRUPOLE, PHYSIM_ERR_ARGUMENT,
             "unknown multipole order %u", cfg->multipole);
    PG_CHECK(cfg->com_theta >= 0.f && cfg->com_theta == cfg->com_theta, PHYSIM_ERR_ARGUMENT,
             "com_theta must be >= 0");
    PG_CUDA(cudaSetDevice(cfg->device));
    PhysimSim *s = new (std::nothrow) PhysimSim();
    PG_CHECK(s, PHYSIM_ERR_MEMORY, "out of host memory");
    s->cfg = *cfg;
    s->cfg.e = fabs(cfg->e);
    s->n = n;
    int rc = PHYSIM_OK;
    if (cfg->stream) {
        s->stream = (cudaStream_t)cfg->stream;
    } else {
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
            set_error("cudaStreamCreate failed");
            delete s;
            return PHYSIM_ERR_CUDA;
        }
        s->own_stream = true;
    }
    rc = bodies_reserve(s->b, n, true, s->stream);
    size_t partial_elems = 3 * (n ? n : 1);
    if (rc == PHYSIM_OK && cfg->gravity == PHYSIM_GRAVITY_SIMPLE_ASTRO) {
        s->plan = plan_direct((int)n, cfg->device, cfg->compensated != 0);
        partial_elems = direct_partial_doubles(s->plan);
    }
    if (rc == PHYSIM_OK && cfg->gravity != PHYSIM_GRAVITY_SIMPLE_ASTRO)
        rc = bh_reserve(s->bh, n, cfg->device, (int)cfg->leaf_size, s->stream);
    if (rc == PHYSIM_OK) rc = dev_alloc(s->partial, partial_elems, s->stream);
    if (rc == PHYSIM_ERR_MEMORY && s->plan.symmetric) {
        // the symmetric plan's slot buffer did not fit: fall back to a one-pair plan
        (void)cudaGetLastError();
        s->plan = plan_direct_one_pair((int)n, cfg->device, cfg->compensated != 0);
        partial_elems = direct_partial_doubles(s->plan);
        rc = dev_alloc(s->partial, partial_elems, s->stream);
    }
    s->partial_cap = partial_elems;
    if (rc == PHYSIM_OK && cfg->integrator == PHYSIM_INTEGRATOR_RK4) {
        const size_t m = 6 * (n ? n : 1);
        rc = dev_alloc(s->rk4_save, m, s->stream);
        if (rc == PHYSIM_OK) rc = dev_alloc(s->rk4_ksum, m, s->stream);
    }
    if (rc != PHYSIM_OK) {
        physim_gpu_sim_destroy(s);
        return rc;
    }
    *out = s;
    return PHYSIM_OK;
}

int physim_gpu_sim_upload(PhysimSim *s, const Entity *state, size_t n)
{
    PG_CHECK(s && (state || n == 0), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(n == s->n, PHYSIM_ERR_ARGUMENT, "upload of %zu bodies into a simulation of %zu", n,
             s->n);
    PG_CUDA(cudaSetDevice(s->cfg.device));
    if (n) {
        PG_CUDA(cudaMemcpyAsync(s->b.aos, state, n * sizeof(Entity), cudaMemcpyHostToDevice,
                                s->stream));
        PG_TRY(launch_unpack(s->b, s->b.aos, n, true, s->stream));
    }
    s->history = false;
    s->uploaded = true;
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PHYSIM_OK;
}

namespace {

int sim_generate(PhysimSim *s, int kind, const void *params)
{
    PG_CHECK(s && params, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    if (s->n) {
        PG_TRY(launch_generate(kind, params, s->b.aos, s->n, s->stream));
        PG_TRY(launch_unpack(s->b, s->b.aos, s->n, true, s->stream));
    }
    s->history = false;
    s->uploaded = true;
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PHYSIM_OK;
}

int generate_host(int kind, const void *params, Entity *out, size_t n, int32_t device)
{
    PG_CHECK(params && (out || n == 0), PHYSIM_ERR_ARGUMENT, "null argument");
    if (n == 0) return PHYSIM_OK;
    PG_CUDA(cudaSetDevice(device));
    cudaStream_t st;
    PG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    Entity *d = nullptr;
    int rc = dev_alloc(d, n, st);
    if (rc == PHYSIM_OK) rc = launch_generate(kind, params, d, n, st);
    if (rc == PHYSIM_OK &&
        cudaMemcpyAsync(out, d, n * sizeof(Entity), cudaMemcpyDeviceToHost, st) != cudaSuccess) {
        set_error("copy of generated bodies failed");
        rc = PHYSIM_ERR_CUDA;
    }
    dev_free(d, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == PHYSIM_OK) {
        set_error("generation failed");
        rc = PHYSIM_ERR_CUDA;
    }
    cudaStreamDestroy(st);
    return rc;
}

// The gravity phase of one force evaluation: the captured graph, or the
// kernels themselves when the stream cannot be captured.
int sim_gravity(PhysimSim *s, int *splits)
{
    if (s->use_graph && !s->graph_exec) PG_TRY(sim_capture(s));
    if (s->graph_exec) {
        PG_CUDA(cudaGraphLaunch(s->graph_exec, s->stream));
        *splits = s->cfg.gravity == PHYSIM_GRAVITY_SIMPLE_ASTRO ? s->plan.splits : 1;
        return PHYSIM_OK;
    }
    return sim_forces(s, splits);
}

}  // namespace

int physim_gpu_sim_init_cube(PhysimSim *s, const PhysimCubeParams *p)
{
    return sim_generate(s, 0, p);
}

int physim_gpu_sim_init_plummer(PhysimSim *s, const PhysimPlummerParams *p)
{
    return sim_generate(s, 1, p);
}

int physim_gpu_generate_cube(const PhysimCubeParams *p, Entity *out, size_t n, int32_t device)
{
    return generate_host(0, p, out, n, device);
}

int physim_gpu_generate_plummer(const PhysimPlummerParams *p, Entity *out, size_t n,
                                int32_t device)
{
    return generate_host(1, p, out, n, device);
}

int physim_gpu_sim_step(PhysimSim *s, uint32_t steps)
{
    PG_CHECK(s, PHYSIM_ERR_ARGUMENT, "null simulation");
    PG_CHECK(s->uploaded, PHYSIM_ERR_ARGUMENT, "step before upload");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    for (uint32_t k = 0; k < steps; ++k) {
        if (s->n == 0) break;
        int splits = 1;
        if (s->profiling) PG_CUDA(cudaEventRecord(s->ev[0], s->stream));
        if (s->cfg.integrator == PHYSIM_INTEGRATOR_RK4) {
            // four force evaluations at the stage states (rk4.rs:33,57,82,108)
            for (int stage = 1; stage <= 4; ++stage) {
                PG_TRY(sim_gravity(s, &splits));
                if (stage == 4 && s->profiling) PG_CUDA(cudaEventRecord(s->ev[1], s->stream));
                PG_TRY(launch_rk4_stage(s->b, s->partial, splits, s->cfg.dt, stage, s->rk4_save,
                                        s->rk4_ksum, s->stream));
            }
        } else {
            PG_TRY(sim_gravity(s, &splits));
            if (s->profiling) PG_CUDA(cudaEventRecord(s->ev[1], s->stream));
            if (s->cfg.integrator == PHYSIM_INTEGRATOR_EULER)
                PG_TRY(launch_euler(s->b, s->partial, splits, s->cfg.dt, s->stream));
            else
                PG_TRY(launch_verlet(s->b, s->partial, splits, s->cfg.dt, !s->history,
                                     s->stream));
        }
        if (s->profiling) PG_CUDA(cudaEventRecord(s->ev[2], s->stream));
        s->history = true;
    }
    return PHYSIM_OK;
}

int physim_gpu_sim_autotune(PhysimSim *s, PhysimDirectTuning *out)
{
    PG_CHECK(s, PHYSIM_ERR_ARGUMENT, "null simulation");
    PG_CHECK(s->uploaded, PHYSIM_ERR_ARGUMENT, "autotune before upload");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    if (s->cfg.gravity != PHYSIM_GRAVITY_SIMPLE_ASTRO || s->n == 0) {
        if (out) memset(out, 0, sizeof *out);
        return PHYSIM_OK;
    }
    DirectPlan cand[16];
    const int k = direct_candidates((int)s->n, s->cfg.device, s->cfg.compensated != 0, cand, 16);
    size_t need = 3 * s->n;
    for (int c = 0; c < k; ++c) need = std::max(need, direct_partial_doubles(cand[c]));
    if (need > s->partial_cap) {
        dev_free(s->partial, s->stream);
        s->partial = nullptr;
        s->partial_cap = 0;
        PG_TRY(dev_alloc(s->partial, need, s->stream));
        s->partial_cap = need;
    }
    cudaEvent_t a, b;
    PG_CUDA(cudaEventCreate(&a));
    PG_CUDA(cudaEventCreate(&b));
    int best = -1;
    double best_ms = 1e300;
    int rc = PHYSIM_OK;
    for (int c = 0; c < k && rc == PHYSIM_OK; ++c) {
        // one untimed and two timed force passes (the state is not advanced)
        float total = 0.f;
        for (int rep = 0; rep < 3 && rc == PHYSIM_OK; ++rep) {
            if (cudaEventRecord(a, s->stream) != cudaSuccess) rc = PHYSIM_ERR_CUDA;
            if (rc == PHYSIM_OK)
                rc = launch_direct(cand[c], s->b.body4, (float)s->cfg.e, s->b.scale, s->partial,
                                   s->stream);
            if (rc == PHYSIM_OK && (cudaEventRecord(b, s->stream) != cudaSuccess ||
                                    cudaEventSynchronize(b) != cudaSuccess))
                rc = PHYSIM_ERR_CUDA;
            float ms = 0.f;
            if (rc == PHYSIM_OK) cudaEventElapsedTime(&ms, a, b);
            if (rep > 0) total += ms;
        }
        if (rc == PHYSIM_OK && total / 2.0 < best_ms) {
            best_ms = total / 2.0;
            best = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc != PHYSIM_OK) {
        if (rc == PHYSIM_ERR_CUDA) set_error("autotune: a CUDA call failed");
        return rc;
    }
    if (best >= 0) {
        s->plan = cand[best];
        // the captured gravity phase used the old plan
        if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
        if (s->graph) cudaGraphDestroy(s->graph);
        s->graph_exec = nullptr;
        s->graph = nullptr;
    }
    if (out) {
        out->block = (uint32_t)s->plan.block;
        out->ipt = (uint32_t)s->plan.ipt;
        out->splits = (uint32_t)s->plan.splits;
        out->candidates = (uint32_t)k;
        out->symmetric = s->plan.symmetric ? 1u : 0u;
        out->tiles = (uint32_t)s->plan.tiles;
        out->force_ms = best_ms;
    }
    return PHYSIM_OK;
}

int physim_gpu_sim_plan(PhysimSim *s, PhysimDirectTuning *out)
{
    PG_CHECK(s && out, PHYSIM_ERR_ARGUMENT, "null argument");
    memset(out, 0, sizeof *out);
    if (s->cfg.gravity != PHYSIM_GRAVITY_SIMPLE_ASTRO) return PHYSIM_OK;
    out->block = (uint32_t)s->plan.block;
    out->ipt = (uint32_t)s->plan.ipt;
    out->splits = (uint32_t)s->plan.splits;
    out->symmetric = s->plan.symmetric ? 1u : 0u;
    out->tiles = (uint32_t)s->plan.tiles;
    return PHYSIM_OK;
}

int physim_gpu_sim_accelerations_f64(PhysimSim *s, const int64_t *idx, size_t count,
                                     Acceleration *out)
{
    PG_CHECK(s && ((idx && out) || count == 0), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(s->uploaded, PHYSIM_ERR_ARGUMENT, "accelerations before upload");
    for (size_t k = 0; k < count; ++k)
        PG_CHECK(idx[k] >= 0 && (size_t)idx[k] < s->n, PHYSIM_ERR_ARGUMENT,
                 "sample index %lld out of range (%zu bodies)", (long long)idx[k], s->n);
    if (count == 0) return PHYSIM_OK;
    PG_CUDA(cudaSetDevice(s->cfg.device));
    int64_t *d_idx = nullptr;
    Acceleration *d_out = nullptr;
    PG_TRY(dev_alloc(d_idx, count, s->stream));
    int rc = dev_alloc(d_out, count, s->stream);
    if (rc == PHYSIM_OK &&
        cudaMemcpyAsync(d_idx, idx, count * sizeof(int64_t), cudaMemcpyHostToDevice, s->stream) !=
            cudaSuccess) {
        set_error("copy of the sample indices failed");
        rc = PHYSIM_ERR_CUDA;
    }
    if (rc == PHYSIM_OK) rc = launch_f64_sample(s->b, s->cfg.e, d_idx, count, d_out, s->stream);
    if (rc == PHYSIM_OK && (cudaMemcpyAsync(out, d_out, count * sizeof(Acceleration),
                                            cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
                            cudaStreamSynchronize(s->stream) != cudaSuccess)) {
        set_error("f64 sample accelerations failed");
        rc = PHYSIM_ERR_CUDA;
    }
    dev_free(d_idx, s->stream);
    dev_free(d_out, s->stream);
    return rc;
}

int physim_gpu_sim_set_plan(PhysimSim *s, const PhysimDirectTuning *plan)
{
    PG_CHECK(s && plan, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(s->cfg.gravity == PHYSIM_GRAVITY_SIMPLE_ASTRO, PHYSIM_ERR_ARGUMENT,
             "pair-kernel plans apply to simple_astro simulations");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    const bool comp = s->cfg.compensated != 0;
    DirectPlan p;
    if (plan->symmetric) {
        PG_CHECK(comp, PHYSIM_ERR_ARGUMENT, "the symmetric plan needs compensated sums");
        p = make_symmetric_plan((int)s->n);
    } else {
        PG_CHECK(direct_shape_supported((int)plan->block, (int)plan->ipt), PHYSIM_ERR_ARGUMENT,
                 "no pair kernel with %u threads and %u bodies per thread", plan->block,
                 plan->ipt);
        PG_CHECK(plan->splits >= 1, PHYSIM_ERR_ARGUMENT, "splits must be >= 1");
        p = make_direct_plan((int)s->n, (int)plan->block, (int)plan->ipt, (int)plan->splits, comp);
    }
    const size_t need = direct_partial_doubles(p);
    if (need > s->partial_cap) {
        dev_free(s->partial, s->stream);
        s->partial = nullptr;
        s->partial_cap = 0;
        PG_TRY(dev_alloc(s->partial, need, s->stream));
        s->partial_cap = need;
    }
    s->plan = p;
    // the captured gravity phase used the old plan
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->graph_exec = nullptr;
    s->graph = nullptr;
    return PHYSIM_OK;
}

int physim_gpu_sim_set_profiling(PhysimSim *s, int enable)
{
    PG_CHECK(s, PHYSIM_ERR_ARGUMENT, "null simulation");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    if (enable && !s->ev[0])
        for (cudaEvent_t &e : s->ev) PG_CUDA(cudaEventCreate(&e));
    s->profiling = enable != 0;
    if (s->bh) PG_TRY(bh_set_profiling(s->bh, s->profiling));
    // the captured gravity phase must be re-captured with (or without) the
    // traversal and pair-kernel events
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->graph_exec = nullptr;
    s->graph = nullptr;
    return PHYSIM_OK;
}

int physim_gpu_sim_last_pair_ms(PhysimSim *s, double *pair_ms)
{
    PG_CHECK(s && pair_ms, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(s->profiling, PHYSIM_ERR_ARGUMENT, "profiling is off");
    PG_CHECK(s->cfg.gravity == PHYSIM_GRAVITY_SIMPLE_ASTRO, PHYSIM_ERR_ARGUMENT,
             "the pair kernel is simple_astro's");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    PG_CUDA(cudaEventSynchronize(s->ev[2]));
    float a = 0.f;
    PG_CUDA(cudaEventElapsedTime(&a, s->ev[0], s->ev[3]));
    *pair_ms = a;
    return PHYSIM_OK;
}

int physim_gpu_sim_last_step_ms(PhysimSim *s, double *gravity_ms, double *integrate_ms)
{
    PG_CHECK(s && gravity_ms && integrate_ms, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(s->profiling, PHYSIM_ERR_ARGUMENT, "profiling is off");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    PG_CUDA(cudaEventSynchronize(s->ev[2]));
    float a = 0.f, b = 0.f;
    PG_CUDA(cudaEventElapsedTime(&a, s->ev[0], s->ev[1]));
    PG_CUDA(cudaEventElapsedTime(&b, s->ev[1], s->ev[2]));
    *gravity_ms = a;
    *integrate_ms = b;
    return PHYSIM_OK;
}

int physim_gpu_sim_download(PhysimSim *s, Entity *state, size_t n)
{
    PG_CHECK(s && (state || n == 0), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(n == s->n, PHYSIM_ERR_ARGUMENT, "download of %zu bodies from a simulation of %zu",
             n, s->n);
    PG_CUDA(cudaSetDevice(s->cfg.device));
    if (n) {
        PG_TRY(launch_pack(s->b, s->stream));
        PG_CUDA(cudaMemcpyAsync(state, s->b.aos, n * sizeof(Entity), cudaMemcpyDeviceToHost,
                                s->stream));
    }
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return bh_check(s->bh, s->stream);
}

int physim_gpu_sim_accelerations(PhysimSim *s, Acceleration *acc, size_t n)
{
    PG_CHECK(s && (acc || n == 0), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(n == s->n, PHYSIM_ERR_ARGUMENT, "size mismatch %zu vs %zu", n, s->n);
    PG_CHECK(s->uploaded, PHYSIM_ERR_ARGUMENT, "accelerations before upload");
    if (n == 0) return PHYSIM_OK;
    PG_CUDA(cudaSetDevice(s->cfg.device));
    if (!s->acc_soa) PG_TRY(dev_alloc(s->acc_soa, 3 * n, s->stream));
    int splits = 1;
    PG_TRY(sim_forces(s, &splits));
    PG_TRY(launch_combine_soa(s->b, s->partial, splits, s->acc_soa, s->stream));
    std::vector<double> h(3 * n);
    PG_CUDA(cudaMemcpyAsync(h.data(), s->acc_soa, 3 * n * sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    PG_TRY(bh_check(s->bh, s->stream));
    for (size_t i = 0; i < n; ++i) {
        acc[i].x = h[i];
        acc[i].y = h[n + i];
        acc[i].z = h[2 * n + i];
    }
    return PHYSIM_OK;
}

int physim_gpu_sim_tree_snapshot(PhysimSim *s, PhysimTreeSnapshot *out)
{
    PG_CHECK(s && out, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(s->cfg.gravity != PHYSIM_GRAVITY_SIMPLE_ASTRO, PHYSIM_ERR_ARGUMENT,
             "simple_astro builds no tree");
    PG_CHECK(s->uploaded, PHYSIM_ERR_ARGUMENT, "snapshot before upload");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    int splits = 1;
    if (s->n) PG_TRY(sim_forces(s, &splits));
    return bh_snapshot(s->bh, s->n, s->stream, out);
}

int physim_gpu_sim_bh_stats(PhysimSim *s, uint64_t *node_visits, uint64_t *interactions,
                            double *traversal_ms)
{
    PG_CHECK(s && node_visits && interactions, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(s->cfg.gravity != PHYSIM_GRAVITY_SIMPLE_ASTRO, PHYSIM_ERR_ARGUMENT,
             "simple_astro has no traversal");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    uint64_t v[2];
    PG_TRY(bh_stats(s->bh, s->stream, v));
    *node_visits = v[0];
    *interactions = v[1];
    if (traversal_ms) {
        *traversal_ms = -1.0;
        if (s->profiling) PG_TRY(bh_traversal_ms(s->bh, traversal_ms));
    }
    return PHYSIM_OK;
}

int physim_gpu_sim_diagnostics(PhysimSim *s, PhysimDiagnostics *out, int with_potential)
{
    PG_CHECK(s && out, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(s->uploaded, PHYSIM_ERR_ARGUMENT, "diagnostics before upload");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    if (!s->diag) PG_TRY(dev_alloc(s->diag, 9, s->stream));
    PG_TRY(launch_diagnostics(s->b, s->cfg.e, s->diag, with_potential != 0, s->cfg.device,
                              s->stream));
    double h[9];
    PG_CUDA(cudaMemcpyAsync(h, s->diag, sizeof h, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
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

int physim_gpu_sim_synchronize(PhysimSim *s)
{
    PG_CHECK(s, PHYSIM_ERR_ARGUMENT, "null simulation");
    PG_CUDA(cudaSetDevice(s->cfg.device));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return bh_check(s->bh, s->stream);
}

void *physim_gpu_sim_stream(PhysimSim *s) { return s ? (void *)s->stream : nullptr; }

int physim_gpu_sim_launches_per_step(PhysimSim *s)
{
    if (!s) return 0;
    // gravity launches + the integrator's kernel
    const int per_eval = s->cfg.gravity == PHYSIM_GRAVITY_SIMPLE_ASTRO
                             ? (s->plan.symmetric ? 2 : 1) + 1
                             : bh_launches(s->bh) + 1;
    return s->cfg.integrator == PHYSIM_INTEGRATOR_RK4 ? 4 * per_eval : per_eval;
}

void physim_gpu_sim_destroy(PhysimSim *s)
{
    if (!s) return;
    cudaSetDevice(s->cfg.device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    // the graph references the buffers: destroy it before they are freed
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    bodies_free(s->b, s->stream);
    dev_free(s->partial, s->stream);
    dev_free(s->acc_soa, s->stream);
    dev_free(s->diag, s->stream);
    dev_free(s->rk4_save, s->stream);
    dev_free(s->rk4_ksum, s->stream);
    bh_free(s->bh);
    for (cudaEvent_t e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

// ------------------------------------------------------------------------
// Verlet over host arrays
// ------------------------------------------------------------------------
int physim_gpu_verlet_create(int32_t device, PhysimVerlet **out)
{
    PG_CHECK(out, PHYSIM_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    PhysimVerlet *v = new (std::nothrow) PhysimVerlet();
    PG_CHECK(v, PHYSIM_ERR_MEMORY, "out of host memory");
    v->device = device;
    *out = v;
    return PHYSIM_OK;
}

int physim_gpu_verlet_integrate(PhysimVerlet *v, const Entity *entities, Entity *new_state,
                                size_t n, const Acceleration *acc, double dt)
{
    PG_CHECK(v, PHYSIM_ERR_ARGUMENT, "null integrator");
    PG_CHECK(n == 0 || (entities && new_state && acc), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CUDA(cudaSetDevice(v->device));
    if (!v->stream) PG_CUDA(cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking));
    if (n > v->cap) {
        Entity **bufs[] = {&v->d_in, &v->d_prev, &v->d_out};
        // Keep previous_state across a growth only if its length still matches.
        Entity *old_prev = v->d_prev;
        size_t old_cap = v->cap;
        if (v->d_in) cudaFree(v->d_in);
        if (v->d_out) cudaFree(v->d_out);
        if (v->d_acc) cudaFree(v->d_acc);
        v->d_in = v->d_out = nullptr;
        v->d_acc = nullptr;
        v->d_prev = nullptr;
        for (Entity **b : bufs) PG_CUDA(cudaMalloc((void **)b, n * sizeof(Entity)));
        PG_CUDA(cudaMalloc((void **)&v->d_acc, n * sizeof(Acceleration)));
        if (old_prev) {
            if (v->has_prev && v->prev_len <= old_cap && v->prev_len > 0)
                PG_CUDA(cudaMemcpyAsync(v->d_prev, old_prev, v->prev_len * sizeof(Entity),
                                        cudaMemcpyDeviceToDevice, v->stream));
            PG_CUDA(cudaStreamSynchronize(v->stream));
            cudaFree(old_prev);
        }
        v->cap = n;
    }
    // verlet.rs:102: a different length means the Taylor first step.
    const bool initial = !v->has_prev || v->prev_len != n;
    if (n) {
        bool direct = false;
        PG_TRY(host_direct(v->device, &direct));
        if (direct) {
            // the kernel reads entities and acc and writes new_state in host
            // memory, keeping a device copy of entities in d_in
            host_prefault(entities, n * sizeof(Entity), false);
            host_prefault(acc, n * sizeof(Acceleration), false);
            host_prefault(new_state, n * sizeof(Entity), true);
            PG_TRY(launch_verlet_aos(entities, v->d_prev, new_state, v->d_in, acc, n, dt, initial,
                                     v->stream));
        } else {
            PG_CUDA(cudaMemcpyAsync(v->d_in, entities, n * sizeof(Entity),
                                    cudaMemcpyHostToDevice, v->stream));
            PG_CUDA(cudaMemcpyAsync(v->d_acc, acc, n * sizeof(Acceleration),
                                    cudaMemcpyHostToDevice, v->stream));
            PG_TRY(launch_verlet_aos(v->d_in, v->d_prev, v->d_out, nullptr, v->d_acc, n, dt,
                                     initial, v->stream));
            PG_CUDA(cudaMemcpyAsync(new_state, v->d_out, n * sizeof(Entity),
                                    cudaMemcpyDeviceToHost, v->stream));
        }
    }
    PG_CUDA(cudaStreamSynchronize(v->stream));
    // previous_state = entities (verlet.rs:31,81)
    Entity *t = v->d_prev;
    v->d_prev = v->d_in;
    v->d_in = t;
    v->prev_len = n;
    v->has_prev = true;
    return PHYSIM_OK;
}

void physim_gpu_verlet_destroy(PhysimVerlet *v)
{
    if (!v) return;
    cudaSetDevice(v->device);
    if (v->stream) cudaStreamSynchronize(v->stream);
    if (v->d_in) cudaFree(v->d_in);
    if (v->d_prev) cudaFree(v->d_prev);
    if (v->d_out) cudaFree(v->d_out);
    if (v->d_acc) cudaFree(v->d_acc);
    if (v->stream) cudaStreamDestroy(v->stream);
    delete v;
}

// ------------------------------------------------------------------------
// verlet / euler / rk4 over host arrays with an acc_fn callback
// ------------------------------------------------------------------------
namespace {

void integrator_release(PhysimIntegrator *it)
{
    if (it->d_ent) cudaFree(it->d_ent);
    if (it->d_q) cudaFree(it->d_q);
    if (it->d_acc) cudaFree(it->d_acc);
    if (it->d_ksum) cudaFree(it->d_ksum);
    if (it->h_q) cudaFreeHost(it->h_q);
    if (it->h_acc) cudaFreeHost(it->h_acc);
    it->d_ent = it->d_q = nullptr;
    it->d_acc = nullptr;
    it->d_ksum = nullptr;
    it->h_q = nullptr;
    it->h_acc = nullptr;
    it->cap = 0;
}

int integrator_reserve(PhysimIntegrator *it, size_t n)
{
    if (n <= it->cap) return PHYSIM_OK;
    integrator_release(it);
    PG_CUDA(cudaMalloc((void **)&it->d_ent, n * sizeof(Entity)));
    PG_CUDA(cudaMalloc((void **)&it->d_q, n * sizeof(Entity)));
    PG_CUDA(cudaMalloc((void **)&it->d_acc, n * sizeof(Acceleration)));
    PG_CUDA(cudaMallocHost((void **)&it->h_acc, n * sizeof(Acceleration)));
    if (it->kind == PHYSIM_INTEGRATOR_RK4) {
        PG_CUDA(cudaMalloc((void **)&it->d_ksum, 6 * n * sizeof(double)));
        PG_CUDA(cudaMallocHost((void **)&it->h_q, n * sizeof(Entity)));
    }
    it->cap = n;
    return PHYSIM_OK;
}

// acc_fn(state) into zeroed accelerations, copied to d_acc
int integrator_eval(PhysimIntegrator *it, const Entity *state, size_t n, PhysimAccFn acc_fn,
                    void *user)
{
    memset(it->h_acc, 0, n * sizeof(Acceleration));
    acc_fn(user, state, n, it->h_acc);
    PG_CUDA(cudaMemcpyAsync(it->d_acc, it->h_acc, n * sizeof(Acceleration),
                            cudaMemcpyHostToDevice, it->stream));
    return PHYSIM_OK;
}

}  // namespace

int physim_gpu_integrator_create(uint32_t kind, int32_t device, PhysimIntegrator **out)
{
    PG_CHECK(out, PHYSIM_ERR_ARGUMENT, "null argument");
    *out = nullptr;
    PG_CHECK(kind <= PHYSIM_INTEGRATOR_RK4, PHYSIM_ERR_ARGUMENT, "unknown integrator %u", kind);
    PhysimIntegrator *it = new (std::nothrow) PhysimIntegrator();
    PG_CHECK(it, PHYSIM_ERR_MEMORY, "out of host memory");
    it->kind = kind;
    it->device = device;
    if (kind == PHYSIM_INTEGRATOR_VERLET) {
        int rc = physim_gpu_verlet_create(device, &it->verlet);
        if (rc != PHYSIM_OK) {
            delete it;
            return rc;
        }
    }
    *out = it;
    return PHYSIM_OK;
}

int physim_gpu_integrator_integrate(PhysimIntegrator *it, const Entity *entities,
                                    Entity *new_state, size_t n, PhysimAccFn acc_fn, void *user,
                                    double dt)
{
    PG_CHECK(it && acc_fn, PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(n == 0 || (entities && new_state), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CUDA(cudaSetDevice(it->device));
    if (it->kind == PHYSIM_INTEGRATOR_VERLET) {
        // verlet.rs:92-106: one acc_fn call, then the (Taylor or regular) step
        std::vector<Acceleration> acc(n ? n : 1);
        memset(acc.data(), 0, acc.size() * sizeof(Acceleration));
        acc_fn(user, entities, n, acc.data());
        return physim_gpu_verlet_integrate(it->verlet, entities, new_state, n, acc.data(), dt);
    }
    if (!it->stream) PG_CUDA(cudaStreamCreateWithFlags(&it->stream, cudaStreamNonBlocking));
    if (n == 0) {
        acc_fn(user, entities, 0, nullptr);
        return PHYSIM_OK;
    }
    PG_TRY(integrator_reserve(it, n));
    PG_CUDA(cudaMemcpyAsync(it->d_ent, entities, n * sizeof(Entity), cudaMemcpyHostToDevice,
                            it->stream));
    if (it->kind == PHYSIM_INTEGRATOR_EULER) {
        // euler.rs:25-47
        PG_TRY(integrator_eval(it, entities, n, acc_fn, user));
        PG_TRY(launch_euler_aos(it->d_ent, it->d_q, it->d_acc, n, dt, it->stream));
    } else {
        // rk4.rs:33-178: the stage states are formed on the device and handed
        // to acc_fn on the host
        const Entity *q_host = entities;
        for (int stage = 1; stage <= 4; ++stage) {
            PG_TRY(integrator_eval(it, q_host, n, acc_fn, user));
            const Entity *d_q_in = stage == 1 ? it->d_ent : it->d_q;
            PG_TRY(launch_rk4_aos_stage(it->d_ent, d_q_in, it->d_acc, it->d_ksum, it->d_q, n, dt,
                                        stage, it->stream));
            if (stage < 4) {
                PG_CUDA(cudaMemcpyAsync(it->h_q, it->d_q, n * sizeof(Entity),
                                        cudaMemcpyDeviceToHost, it->stream));
                PG_CUDA(cudaStreamSynchronize(it->stream));
                q_host = it->h_q;
            }
        }
    }
    PG_CUDA(cudaMemcpyAsync(new_state, it->d_q, n * sizeof(Entity), cudaMemcpyDeviceToHost,
                            it->stream));
    PG_CUDA(cudaStreamSynchronize(it->stream));
    return PHYSIM_OK;
}

void physim_gpu_integrator_destroy(PhysimIntegrator *it)
{
    if (!it) return;
    cudaSetDevice(it->device);
    if (it->stream) cudaStreamSynchronize(it->stream);
    integrator_release(it);
    if (it->verlet) physim_gpu_verlet_destroy(it->verlet);
    if (it->stream) cudaStreamDestroy(it->stream);
    delete it;
}

}  // extern "C"
