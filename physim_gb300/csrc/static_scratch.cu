// static_scratch.cu -- simple_astro accelerations without any device
// allocation (physim_gpu_simple_astro_accumulate_static).
//
// Some callers cannot allocate device memory: code running where the CUDA
// allocator is off limits (inside another framework's memory pool or arena,
// a real-time loop that must not call cudaMalloc, or a process whose device
// memory is all handed out up front).  They pass device-accessible input and
// output arrays; the scratch this computation needs (the f32 body copy, the
// masses and fixed flags, the partial sums) lives in one file-scope
// __device__ array of fixed size below, which every GPU that loads the
// library holds until the process exits.
#include <mutex>

#include "common.cuh"
#include "engine.h"

namespace pg {
namespace {

// Largest state this entry point accepts, and the j splits it may use.
constexpr size_t kStaticMaxBodies = 65536;
constexpr int kStaticMaxSplits = 4;

constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kStaticPad = (kStaticMaxBodies + kBodyPad - 1) / kBodyPad * kBodyPad;
constexpr size_t kOffBody4 = 0;
constexpr size_t kOffMass = align256(kOffBody4 + kStaticPad * sizeof(float4));
constexpr size_t kOffFixed = align256(kOffMass + kStaticPad * sizeof(double));
constexpr size_t kOffScale = align256(kOffFixed + kStaticPad);
constexpr size_t kOffPartial = align256(kOffScale + sizeof(PairScale));
constexpr size_t kStaticBytes =
    align256(kOffPartial + (size_t)kStaticMaxSplits * 3 * kStaticMaxBodies * sizeof(double));

// About 7.9 MiB per device.  Every call shares it: calls that overlap on
// the GPU (different streams, or different host threads) race on it.
__device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// Device address of g_static_scratch per device ordinal, looked up once with
// that device current (the host-side symbol is not a device address).  The
// cache lives as long as the process: after a cudaDeviceReset the module is
// loaded again and the array may sit elsewhere, so this entry point must not
// be used after a reset of a device it was called on.
std::mutex g_scratch_lock;
unsigned char *g_scratch_addr[64] = {nullptr};

int scratch_address(int device, unsigned char **out)
{
    std::lock_guard<std::mutex> g(g_scratch_lock);
    PG_CHECK(device >= 0 && device < 64, PHYSIM_ERR_ARGUMENT, "device %d out of range", device);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&p, g_static_scratch);
        if (err != cudaSuccess || !p) {
            set_error("cudaGetSymbolAddress of the static scratch failed: %s",
                      cudaGetErrorString(err));
            return PHYSIM_ERR_CUDA;
        }
        g_scratch_addr[device] = (unsigned char *)p;
    }
    *out = g_scratch_addr[device];
    return PHYSIM_OK;
}

}  // namespace
}  // namespace pg

using namespace pg;

extern "C" int physim_gpu_simple_astro_accumulate_static(const Entity *state, size_t n, double e,
                                                         Acceleration *acc, void *stream)
{
    PG_CHECK(n == 0 || (state && acc), PHYSIM_ERR_ARGUMENT, "null argument");
    PG_CHECK(n <= kStaticMaxBodies, PHYSIM_ERR_ARGUMENT,
             "%zu bodies exceed the static scratch of this entry point (at most %zu); use "
             "simple_astro_transform or a physim_gpu_sim for larger states",
             n, kStaticMaxBodies);
    if (n == 0) return PHYSIM_OK;
    int device = 0;
    PG_CUDA(cudaGetDevice(&device));
    // The arrays are read and written by kernels: host memory the GPU cannot
    // reach would fault there, so it is rejected here (pageable host memory
    // is reachable on a device with pageable memory access, as GB300's
    // NVLink-C2C host is).
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess)
        pageable = 0;
    const void *arrays[2] = {state, acc};
    for (const void *ptr : arrays) {
        cudaPointerAttributes attr;
        const cudaError_t err = cudaPointerGetAttributes(&attr, ptr);
        if (err != cudaSuccess) {
            (void)cudaGetLastError();
            set_error("cudaPointerGetAttributes(%p) failed: %s", ptr, cudaGetErrorString(err));
            return PHYSIM_ERR_ARGUMENT;
        }
        PG_CHECK(attr.type != cudaMemoryTypeUnregistered || pageable, PHYSIM_ERR_ARGUMENT,
                 "%p is pageable host memory, which device %d cannot access: pass device, "
                 "managed or registered host memory",
                 ptr, device);
        PG_CHECK(attr.type != cudaMemoryTypeDevice || attr.device == device, PHYSIM_ERR_ARGUMENT,
                 "%p is memory of device %d, not of the current device %d", ptr, attr.device,
                 device);
    }
    unsigned char *base = nullptr;
    PG_TRY(scratch_address(device, &base));
    cudaStream_t st = (cudaStream_t)stream;

    DeviceBodies view;  // a view of the static scratch; nothing is allocated
    view.n = n;
    view.cap = kStaticPad;
    view.body4 = (float4 *)(base + kOffBody4);
    view.m = (double *)(base + kOffMass);
    view.fixed = (uint8_t *)(base + kOffFixed);
    double *partial = (double *)(base + kOffPartial);
    PairScale *scale = (PairScale *)(base + kOffScale);

    // The f32 copy is rewritten for all padded slots (zero mass past n), and
    // every partial sum is overwritten by the pair kernel.  The scale pass's
    // arrival count must start at zero: it is left at zero by every completed
    // pass, and cleared here as well (a memset, not an allocation), so a call
    // after an interrupted one still starts clean.
    PG_CUDA(cudaMemsetAsync(&scale->arrivals, 0, sizeof(uint32_t), st));
    PG_TRY(launch_unpack(view, state, n, false, st));
    const int sms = device_sm_count(device);
    const int block = 128, ipt = 4;
    const int n_itiles = (int)((n + block * ipt - 1) / (block * ipt));
    int splits = (2 * sms + n_itiles - 1) / n_itiles;
    splits = splits < 1 ? 1 : (splits > kStaticMaxSplits ? kStaticMaxSplits : splits);
    const DirectPlan plan = make_direct_plan((int)n, block, ipt, splits, true);
    PG_CHECK(plan.splits <= kStaticMaxSplits, PHYSIM_ERR_ARGUMENT, "internal: %d splits",
             plan.splits);
    PG_TRY(launch_direct(plan, view.body4, (float)fabs(e), scale, partial, st));
    PG_TRY(launch_accumulate_aos(view, partial, plan.splits, acc, st));
    return PHYSIM_OK;
}
