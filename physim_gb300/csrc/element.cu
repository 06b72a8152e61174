// element.cu -- the compute behind a transform element's transform call:
// host Entity array in, `acc[i] += a_i` out (astro/src/transformers.rs:122-160
// for astro2, :31-69 for astro, :219-244 for simple_astro).
//
// Per call: the Entity array (80 B/body) is unpacked to f32 (x,y,z,m) + f64
// state, the gravity kernels run, and the accelerations (24 B/body) are added
// to the caller's in f64.  With host access DIRECT the unpack and accumulate
// kernels read and write the caller's host arrays in place; with COPY both
// arrays are copied to the device first and the accelerations copied back.
// Fixed bodies keep their incoming value untouched.
#include "common.cuh"
#include "engine.h"
#include "plugin_state.h"

namespace pg {

static int ensure_doubles(double *&p, size_t &cap, size_t need, cudaStream_t st)
{
    if (need <= cap) return PHYSIM_OK;
    dev_free(p, st);
    p = nullptr;
    cap = 0;
    PG_TRY(dev_alloc(p, need, st));
    cap = need;
    return PHYSIM_OK;
}

static int accumulate_locked(ElementState *el, const Entity *state, size_t n, Acceleration *acc)
{
    if (n == 0) return PHYSIM_OK;
    PG_CHECK(n < (size_t)INT32_MAX, PHYSIM_ERR_ARGUMENT, "too many bodies: %zu", n);
    PG_CUDA(cudaSetDevice(el->device));
    if (!el->ready) {
        PG_CUDA(cudaStreamCreateWithFlags(&el->stream, cudaStreamNonBlocking));
        el->ready = true;
    }
    cudaStream_t st = el->stream;
    const bool tree = el->kind != 0;
    bool direct = false;
    PG_TRY(host_direct(el->device, &direct));
    PG_TRY(bodies_reserve(el->bodies, n, tree, st));
    Acceleration *acc_io = acc;  // DIRECT: the kernels read and write the caller's array
    const Entity *state_in = state;
    if (direct) {
        host_prefault(state, n * sizeof(Entity), false);
        host_prefault(acc, n * sizeof(Acceleration), true);
    } else {
        if (el->acc_cap < n) {
            dev_free(el->d_acc, st);
            el->d_acc = nullptr;
            el->acc_cap = 0;
            PG_TRY(dev_alloc(el->d_acc, n, st));
            el->acc_cap = n;
        }
        PG_CUDA(cudaMemcpyAsync(el->bodies.aos, state, n * sizeof(Entity), cudaMemcpyHostToDevice,
                                st));
        PG_CUDA(cudaMemcpyAsync(el->d_acc, acc, n * sizeof(Acceleration), cudaMemcpyHostToDevice,
                                st));
        acc_io = el->d_acc;
        state_in = el->bodies.aos;
    }
    PG_TRY(launch_unpack(el->bodies, state_in, n, tree, st));
    int splits = 1;
    if (!tree) {
        if (el->plan_n != (int)n) {
            el->plan = plan_direct((int)n, el->device, true);
            el->plan_n = (int)n;
        }
        int rc = ensure_doubles(el->partial, el->partial_cap, direct_partial_doubles(el->plan), st);
        if (rc == PHYSIM_ERR_MEMORY && el->plan.symmetric) {
            // the slot buffer did not fit after all: one-pair kernels need 3n doubles
            (void)cudaGetLastError();
            el->plan = plan_direct_one_pair((int)n, el->device, true);
            rc = ensure_doubles(el->partial, el->partial_cap, direct_partial_doubles(el->plan), st);
        }
        PG_TRY(rc);
        splits = el->plan.splits;
        PG_TRY(launch_direct(el->plan, el->bodies.body4, (float)el->e, el->bodies.scale,
                             el->partial, st));
    } else {
        PG_TRY(ensure_doubles(el->partial, el->partial_cap, 3 * n, st));
        PG_TRY(bh_reserve(el->bh, n, el->device, el->leaf_size, st));
        BhParams p;
        p.nchild = el->kind == 1 ? 8 : 4;
        p.theta = el->theta;
        p.e = el->e;
        p.leaf_size = el->leaf_size;
        p.traversal = el->traversal;
        p.multipole = el->multipole;
        p.com_theta = el->com_theta;
        PG_TRY(bh_accelerations(el->bh, el->bodies, p, el->partial, st));
    }
    PG_TRY(launch_accumulate_aos(el->bodies, el->partial, splits, acc_io, st));
    if (!direct)
        PG_CUDA(cudaMemcpyAsync(acc, el->d_acc, n * sizeof(Acceleration), cudaMemcpyDeviceToHost,
                                st));
    PG_CUDA(cudaStreamSynchronize(st));
    if (tree) PG_TRY(bh_check(el->bh, st));
    return PHYSIM_OK;
}

int element_accumulate(ElementState *el, const Entity *state, size_t n, Acceleration *acc)
{
    std::lock_guard<std::mutex> g(el->lock);
    return accumulate_locked(el, state, n, acc);
}

void element_destroy(ElementState *el)
{
    if (el->ready) {
        cudaSetDevice(el->device);
        cudaStreamSynchronize(el->stream);
        bodies_free(el->bodies, el->stream);
        dev_free(el->d_acc, el->stream);
        dev_free(el->partial, el->stream);
        bh_free(el->bh);
        cudaStreamSynchronize(el->stream);
        cudaStreamDestroy(el->stream);
    }
    delete el;
}

}  // namespace pg
