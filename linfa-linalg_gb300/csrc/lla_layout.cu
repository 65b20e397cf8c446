// lla_layout.cu -- moving strided views in and out of the column-major
// working layout, triangle masking and the is_triangular predicate.
//
// Views keep ndarray's convention: element (i, j) at R[i*rs + j*cs] with
// signed element strides.  Import/export go through 32 x 32 shared-memory
// tiles so both the strided side and the column-major side are read and
// written in coalesced runs whichever way the view is laid out.
#include "lla_common.cuh"
#include "lla_kernels.h"
#include "lla_prof.h"

namespace lla {

template <typename T>
__global__ void import_kernel(const T *__restrict__ R, int64_t rs, int64_t cs, int64_t rows,
                              int64_t cols, T *__restrict__ W, int64_t ld) {
    __shared__ T tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    const bool row_major = (cs == 1);
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        // row-major source: consecutive threads walk j; otherwise walk i
        const int64_t i = row_major ? i0 + k : i0 + threadIdx.x;
        const int64_t j = row_major ? j0 + threadIdx.x : j0 + k;
        if (i < rows && j < cols) {
            const T v = R[i * rs + j * cs];
            if (row_major)
                tile[k][threadIdx.x] = v;
            else
                tile[threadIdx.x][k] = v;
        }
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, j = j0 + k;
        if (i < rows && j < cols) W[i + j * ld] = tile[threadIdx.x][k];
    }
}

__device__ __forceinline__ bool export_selected(int mode, int64_t i, int64_t j, int64_t f) {
    switch (mode) {
        case EXPORT_FULL: return true;
        case EXPORT_LOWER: return j <= i;
        case EXPORT_LOWER_ZERO_UPPER: return true;
        default: return (i < f && j <= i) || (i == f && j < f);
    }
}

template <typename T>
__global__ void export_kernel(const T *__restrict__ W, int64_t ld, T *__restrict__ R, int64_t rs,
                              int64_t cs, int64_t rows, int64_t cols, int mode, int64_t f) {
    __shared__ T tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    const bool row_major = (cs == 1);
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, j = j0 + k;
        if (i < rows && j < cols) tile[threadIdx.x][k] = W[i + j * ld];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t i = row_major ? i0 + k : i0 + threadIdx.x;
        const int64_t j = row_major ? j0 + threadIdx.x : j0 + k;
        if (i < rows && j < cols && export_selected(mode, i, j, f)) {
            const T v = row_major ? tile[k][threadIdx.x] : tile[threadIdx.x][k];
            R[i * rs + j * cs] = (mode == EXPORT_LOWER_ZERO_UPPER && j > i) ? T(0) : v;
        }
    }
}

template <typename T>
__global__ void mask_kernel(T *R, int64_t rs, int64_t cs, int64_t n, int uplo) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t j = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    // triangular_inplace (src/triangular.rs:37-53): Upper zeroes j < i, Lower zeroes j > i
    const bool zero = (uplo == LLA_UPPER) ? (j < i) : (j > i);
    if (zero) R[i * rs + j * cs] = T(0);
}

template <typename T>
__global__ void is_triangular_kernel(const T *R, int64_t rs, int64_t cs, int64_t n, int uplo,
                                     int *flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t j = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    // is_triangular (src/triangular.rs:67-90): any non-zero outside the triangle -> false
    const bool outside = (uplo == LLA_UPPER) ? (j < i) : (j > i);
    if (outside && R[i * rs + j * cs] != T(0)) *flag = 0;
}

template <typename T>
__global__ void eye_kernel(T *W, int64_t ld, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) W[i + j * ld] = (i == j) ? T(1) : T(0);
}

__global__ void fill_int_kernel(int *p, int v) { *p = v; }

int fill_int_launch(int *p, int v, cudaStream_t st) {
    LaunchScope ls(K_MISC, st);
    fill_int_kernel<<<1, 1, 0, st>>>(p, v);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

static dim3 tiles2d(int64_t rows, int64_t cols) {
    return dim3((unsigned)ceil_div(rows, 32), (unsigned)ceil_div(cols, 32));
}

template <typename T>
int import_launch(const T *R, int64_t rs, int64_t cs, int64_t rows, int64_t cols, T *W, int64_t ld,
                  cudaStream_t st) {
    if (rows == 0 || cols == 0) return 0;
    LaunchScope ls(K_LAYOUT, st);
    import_kernel<T><<<tiles2d(rows, cols), dim3(32, 8), 0, st>>>(R, rs, cs, rows, cols, W, ld);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T>
int export_launch(const T *W, int64_t ld, T *R, int64_t rs, int64_t cs, int64_t rows, int64_t cols,
                  int mode, int64_t fail_row, cudaStream_t st) {
    if (rows == 0 || cols == 0) return 0;
    LaunchScope ls(K_LAYOUT, st);
    export_kernel<T><<<tiles2d(rows, cols), dim3(32, 8), 0, st>>>(W, ld, R, rs, cs, rows, cols,
                                                                  mode, fail_row);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T>
int mask_launch(T *R, int64_t rs, int64_t cs, int64_t n, int uplo, cudaStream_t st) {
    if (n == 0) return 0;
    LaunchScope ls(K_LAYOUT, st);
    mask_kernel<T><<<tiles2d(n, n), dim3(32, 32), 0, st>>>(R, rs, cs, n, uplo);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T>
int is_triangular_launch(const T *R, int64_t rs, int64_t cs, int64_t n, int uplo, int *d_flag,
                         cudaStream_t st) {
    if (n == 0) return 0;
    LaunchScope ls(K_LAYOUT, st);
    is_triangular_kernel<T><<<tiles2d(n, n), dim3(32, 32), 0, st>>>(R, rs, cs, n, uplo, d_flag);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <typename T>
int eye_launch(T *W, int64_t ld, int64_t n, cudaStream_t st) {
    if (n == 0) return 0;
    const unsigned gy = (unsigned)std::min<int64_t>(n, 65535);
    LaunchScope ls(K_LAYOUT, st);
    eye_kernel<T><<<dim3((unsigned)ceil_div(n, 256), gy), 256, 0, st>>>(W, ld, n);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// The strict upper part from the lower one: block (I, J), I <= J, writes the
// entries i < j of output tile (I, J) from the transposed lower tile (J, I),
// staged through shared memory so both sides stay coalesced.
template <typename T>
__global__ void symmetrize_kernel(T *W, int64_t ld, int64_t n) {
    __shared__ T tile[32][33];
    const int64_t I = blockIdx.x, J = blockIdx.y;
    if (I > J) return;
    const int64_t i0 = I * 32, j0 = J * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = j0 + threadIdx.x, c = i0 + k;  // element (r, c) = (j, i) of the lower tile
        if (r < n && c < n) tile[threadIdx.x][k] = W[r + c * ld];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, j = j0 + k;
        if (i < n && j < n && i < j) W[i + j * ld] = tile[k][threadIdx.x];
    }
}

template <typename T>
int symmetrize_launch(T *W, int64_t ld, int64_t n, cudaStream_t st) {
    if (n == 0) return 0;
    LaunchScope ls(K_LAYOUT, st);
    symmetrize_kernel<T><<<tiles2d(n, n), dim3(32, 8), 0, st>>>(W, ld, n);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

#define LLA_INST(T)                                                                              \
    template int import_launch<T>(const T *, int64_t, int64_t, int64_t, int64_t, T *, int64_t,   \
                                  cudaStream_t);                                                 \
    template int export_launch<T>(const T *, int64_t, T *, int64_t, int64_t, int64_t, int64_t,   \
                                  int, int64_t, cudaStream_t);                                   \
    template int mask_launch<T>(T *, int64_t, int64_t, int64_t, int, cudaStream_t);              \
    template int is_triangular_launch<T>(const T *, int64_t, int64_t, int64_t, int, int *,       \
                                         cudaStream_t);                                          \
    template int eye_launch<T>(T *, int64_t, int64_t, cudaStream_t);                            \
    template int symmetrize_launch<T>(T *, int64_t, int64_t, cudaStream_t);
LLA_INST(double)
LLA_INST(float)

}  // namespace lla
