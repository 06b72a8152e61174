// common.cuh -- shared types, error plumbing and FP32x2 helpers for the
// GB300 (sm_103a) gravity + integration library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include "physim_gb300.h"

namespace pg {

// The state layout handed over by physim (physim-core/src/lib.rs:16-37).
static_assert(sizeof(Entity) == 80, "Entity must match physim's repr(C) layout");
static_assert(sizeof(Acceleration) == 24, "Acceleration must match physim's layout");
static_assert(offsetof(Entity, mass) == 56 && offsetof(Entity, id) == 64 &&
                  offsetof(Entity, fixed) == 72,
              "Entity field offsets");

// Last error message of the calling thread (physim_gpu_last_error).
void set_error(const char *fmt, ...);
const char *last_error();

}  // namespace pg

// Evaluate a CUDA runtime call; on failure record the message and return
// PHYSIM_ERR_CUDA from the enclosing function.
#define PG_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t pg_e_ = (call);                                                    \
        if (pg_e_ != cudaSuccess) {                                                    \
            ::pg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                 \
                            cudaGetErrorString(pg_e_));                                \
            return PHYSIM_ERR_CUDA;                                                    \
        }                                                                              \
    } while (0)

#define PG_CHECK(cond, code, ...)                                                      \
    do {                                                                               \
        if (!(cond)) {                                                                 \
            ::pg::set_error(__VA_ARGS__);                                              \
            return (code);                                                             \
        }                                                                              \
    } while (0)

#define PG_TRY(expr)                                                                   \
    do {                                                                               \
        int pg_rc_ = (expr);                                                           \
        if (pg_rc_ != PHYSIM_OK) return pg_rc_;                                        \
    } while (0)

#ifdef __CUDACC__
namespace pg {

// Packed FP32 pairs: Blackwell issues one FFMA2/FADD2/FMUL2 for two lanes of
// work, which halves the issue slots the pair loop needs.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Hardware reciprocal square root (MUFU.RSQ), flush-to-zero approximate form.
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 2^k as a float (|k| <= 126) and as a double (|k| <= 1022), exact.
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }
__device__ __forceinline__ double pow2d(int k)
{
    return __longlong_as_double((long long)(1023 + k) << 52);
}

// Knuth's TwoSum: s + err == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &err)
{
    s = a + b;
    float bp = s - a;
    float ap = s - bp;
    err = (a - ap) + (b - bp);
}

}  // namespace pg
#endif
