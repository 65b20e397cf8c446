// lla_probe.cu -- measured arithmetic peaks used as roofline denominators for
// the kernels whose pipes have no entry in a measured peak table (the
// FP64 tensor pipe, DFMA, FFMA).  Each probe runs a register-resident loop of
// independent instructions on every SM, times it with CUDA events and returns
// TFLOP/s (best of three); every thread writes one result element, in bounds.
#include <cuda_runtime.h>

#include "../../include/lla_gb300.h"

namespace {

constexpr int kIters = 2048;

// Eight MMAs per step with two distinct A fragments and four distinct B
// fragments, as a GEMM tile issues them.  (Issuing the same operand registers
// back to back runs several times faster on GB300 -- operand reuse that no
// GEMM can exploit -- so it would not be an honest roofline denominator.)
__global__ void probe_dmma(double *out, double av, double bv) {
    double a[2][8], b[4][4], c[8][4];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int j = 0; j < 8; ++j) a[q][j] = (av + threadIdx.x + j + q) * 0.1234567891234567;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int j = 0; j < 4; ++j) b[q][j] = (bv + j + q) * 0.7654321987654321;
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) c[j][q] = 0.0;
    for (int i = 0; i < kIters / 64; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int ia = j % 2, ib = j / 2;
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
                : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
                : "d"(a[ia][0]), "d"(a[ia][1]), "d"(a[ia][2]), "d"(a[ia][3]), "d"(a[ia][4]),
                  "d"(a[ia][5]), "d"(a[ia][6]), "d"(a[ia][7]), "d"(b[ib][0]), "d"(b[ib][1]),
                  "d"(b[ib][2]), "d"(b[ib][3]));
        }
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) s += c[j][q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_dfma(double *out, double a, double b) {
    double x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = threadIdx.x + j;
    for (int i = 0; i < kIters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_ffma(double *out, float a, float b) {
    float x[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = threadIdx.x + j;
    for (int i = 0; i < kIters; ++i)
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = fmaf(x[j], a, b);
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 16; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" double lla_measure_peak_tflops(int which) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    const int threads = 256, blocks = sms * 8;
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        double flops = 0.0;
        if (which == 0) {  // FP64 tensor pipe: 8 x m16n8k16 per step
            probe_dmma<<<blocks, threads>>>(out, 0.5, 0.25);
            flops = 2.0 * 16 * 8 * 16 * 8 * (kIters / 64) * (double)(threads / 32) * blocks;
        } else if (which == 1) {
            probe_dfma<<<blocks, threads>>>(out, 0.999, 1e-3);
            flops = 2.0 * 8 * kIters * (double)threads * blocks;
        } else {
            probe_ffma<<<blocks, threads>>>(out, 0.999f, 1e-3f);
            flops = 2.0 * 16 * kIters * (double)threads * blocks;
        }
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    const bool ok = cudaGetLastError() == cudaSuccess;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return ok ? best : -1.0;
}
