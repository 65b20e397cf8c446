// lla_common.cuh -- shared device/host helpers of the GB300 SPD library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/lla_gb300.h"

namespace lla {

// Per-element arithmetic in two flavours.
//  Exact: one IEEE round-to-nearest operation per Rust operation -- separate
//         multiply and add (the __*_rn intrinsics are never contracted into
//         FMA), IEEE division and square root.  This reproduces the
//         reference's results bit for bit when the operation order is kept.
//  Fast : fused multiply-add.
template <typename T> struct Arith;

template <> struct Arith<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
};

template <> struct Arith<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
    static __device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
};

// Column-major element access: (i, j) of a matrix with leading dimension ld.
template <typename T>
__device__ __forceinline__ T &cm(T *p, int64_t ld, int64_t i, int64_t j) { return p[i + j * ld]; }
template <typename T>
__device__ __forceinline__ const T &cm(const T *p, int64_t ld, int64_t i, int64_t j) { return p[i + j * ld]; }

// Bounded spin limit for inter-CTA waits (polls with nanosleep back-off):
// roughly a few seconds before the kernel gives up and reports LLA_ERR_TIMEOUT.
constexpr long long kSpinLimit = 1ll << 24;

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while its predecessor in the stream still runs;
// pdl_wait() returns once the predecessor has completed and its writes are
// visible (at once for a kernel launched without the attribute).  Every
// kernel of such a chain calls pdl_wait() before its first read of the
// predecessor's output and before any exit, then pdl_trigger() to let its
// own successor start: so a kernel may read, before its wait, anything
// written two or more launches earlier.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launches `kern` on `st`, allowed to overlap the tail of the stream's
// previous kernel when `pdl` (the kernel must follow the pdl_wait rules).
template <typename... Exp, typename... Act>
inline cudaError_t launch_maybe_pdl(bool pdl, void (*kern)(Exp...), dim3 grid, dim3 block, size_t smem,
                                    cudaStream_t st, Act &&...args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Act>(args)...);
}

}  // namespace lla

// Error plumbing used by the host drivers (defined in lla_api.cpp).
extern "C" int lla__set_cuda_error(lla_error *err, cudaError_t e);
extern "C" int lla__set_status(lla_error *err, int code);

#define LLA_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t lla_e__ = (expr);                        \
        if (lla_e__ != cudaSuccess) return lla__set_cuda_error(err, lla_e__); \
    } while (0)
