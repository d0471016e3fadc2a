// Device operations of the dense numeric::Matrix container
// (src/numeric/matrix.cpp, src/numeric/matrix_kernel.cu:35-631): column-major
// FP32 matrices with leading dimension ld (the reference's dataRows).
//   setEye, diag, add (scalar, matrix), scalarMultiply, elementwise
//   multiply / division (0 where the divisor is 0, matrix_kernel.cu:345-352),
//   the column reductions sum, vectorDotProduct, min and max (the result in
//   row 0 of each column, as the reference leaves it; FP64 accumulation, one
//   block per column, fixed order), and the dense product
//   C = op(A) op(B) that Matrix::multiply takes from cuBLAS (matrix.cpp:
//   298-332) as a shared-memory tiled FP32 kernel.
#include <algorithm>
#include <cfloat>

#include "mpf_internal.h"

namespace mpf {
namespace {

__global__ void k_mat_elementwise(int op, int rows, int cols, const float* __restrict__ A,
                                  const float* __restrict__ B, float* __restrict__ C, int ld, float scalar) {
    const size_t total = (size_t)rows * cols;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % rows), c = (int)(i / rows);
        const size_t o = (size_t)c * ld + r;
        switch (op) {
            case 0: C[o] = r == c ? 1.f : 0.f; break;                      // setEye
            case 1: C[o] = r == c ? A[o] : 0.f; break;                     // diag
            case 2: C[o] = A[o] + scalar; break;                           // add scalar
            case 3: C[o] = A[o] + B[o]; break;                             // add matrix
            case 4: C[o] = A[o] * scalar; break;                           // scalarMultiply
            case 5: C[o] = A[o] * B[o]; break;                             // elementwiseMultiply
            default: C[o] = B[o] != 0.f ? A[o] / B[o] : 0.f; break;        // elementwiseDivision
        }
    }
}

// result[c * ldr] = reduce_r f(A[r][c], B[r][c]); op 0 sum, 1 dot, 2 min, 3 max
__global__ void __launch_bounds__(256) k_mat_column_reduce(int op, int rows, const float* __restrict__ A,
                                                           const float* __restrict__ B, int ld,
                                                           float* __restrict__ result, int ldr) {
    const int c = blockIdx.x;
    __shared__ double red[256];
    const float* a = A + (size_t)c * ld;
    const float* b = B ? B + (size_t)c * ld : nullptr;
    double v = op == 2 ? DBL_MAX : (op == 3 ? -DBL_MAX : 0.0);
    for (int r = threadIdx.x; r < rows; r += blockDim.x) {
        const double x = (double)a[r];
        if (op == 0) v += x;
        else if (op == 1) v += x * (double)b[r];
        else if (op == 2) v = fmin(v, x);
        else v = fmax(v, x);
    }
    red[threadIdx.x] = v;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            const double o = red[threadIdx.x + h];
            double& s = red[threadIdx.x];
            s = op <= 1 ? s + o : (op == 2 ? fmin(s, o) : fmax(s, o));
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) result[(size_t)c * ldr] = (float)red[0];
}

// C (m x n) = alpha op(A) op(B) + beta C (C not read when beta == 0),
// op(X) = X or X^T; 64 x 64 tiles, 256 threads with 4 x 4 outputs each, k in
// chunks of 16 through shared memory
__global__ void __launch_bounds__(256) k_mat_gemm(int transA, int transB, int m, int n, int k, float alpha,
                                                  const float* __restrict__ A, int lda, const float* __restrict__ B,
                                                  int ldb, float beta, float* __restrict__ C, int ldc) {
    __shared__ float As[16][65], Bs[16][65];
    const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < k; k0 += 16) {
        for (int t = threadIdx.x; t < 64 * 16; t += 256) {
            const int r = t % 64, kk = t / 64;
            const int gi = i0 + r, gj = j0 + r, gk = k0 + kk;
            float a = 0.f, b = 0.f;
            if (gi < m && gk < k) a = transA ? A[(size_t)gi * lda + gk] : A[(size_t)gk * lda + gi];
            if (gj < n && gk < k) b = transB ? B[(size_t)gk * ldb + gj] : B[(size_t)gj * ldb + gk];
            As[kk][r] = a;
            Bs[kk][r] = b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                av[q] = As[kk][ty + 16 * q];
                bv[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(av[p], bv[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
            if (i < m && j < n) {
                float* c = C + (size_t)j * ldc + i;
                *c = beta == 0.f ? alpha * acc[p][q] : fmaf(alpha, acc[p][q], beta * *c);
            }
        }
}

// n scalars between FP64 and FP32 (direction 0: double -> float, 1: float ->
// double); grid-stride, one value per thread per pass
__global__ void k_convert(int direction, long long n, const void* __restrict__ src, void* __restrict__ dst) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (direction == 0) static_cast<float*>(dst)[i] = (float)static_cast<const double*>(src)[i];
        else static_cast<double*>(dst)[i] = (double)static_cast<const float*>(src)[i];
    }
}

}  // namespace

int convert_values(int direction, long long count, const void* src, void* dst, cudaStream_t s) {
    MPF_CHECK(direction == 0 || direction == 1, MPF_EINVAL, "mpf_convert_values: direction must be 0 or 1");
    MPF_CHECK(count >= 0, MPF_EINVAL, "mpf_convert_values: count < 0");
    if (count == 0) return MPF_OK;
    MPF_CHECK(src && dst, MPF_EINVAL, "mpf_convert_values: null pointer");
    const long long blocks = std::min<long long>((count + 255) / 256, 152LL * 16);
    k_convert<<<(int)blocks, 256, 0, s>>>(direction, count, src, dst);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int matrix_elementwise(int op, int rows, int cols, const float* A, const float* B, float* C, int ld, float scalar,
                       cudaStream_t s) {
    MPF_CHECK(rows >= 1 && cols >= 1 && ld >= rows && C && op >= 0 && op <= 6, MPF_EINVAL,
              "mpFlow::numeric::Matrix: bad arguments");
    MPF_CHECK(op == 0 || A, MPF_EINVAL, "mpFlow::numeric::Matrix: A == nullptr");
    MPF_CHECK((op != 3 && op != 5 && op != 6) || B, MPF_EINVAL, "mpFlow::numeric::Matrix: B == nullptr");
    const size_t total = (size_t)rows * cols;
    k_mat_elementwise<<<(int)std::min<size_t>((total + 255) / 256, 4096), 256, 0, s>>>(op, rows, cols, A, B, C, ld,
                                                                                      scalar);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int matrix_column_reduce(int op, int rows, int cols, const float* A, const float* B, int ld, float* result, int ldr,
                         cudaStream_t s) {
    MPF_CHECK(rows >= 1 && cols >= 1 && ld >= rows && A && result && op >= 0 && op <= 3 && (op != 1 || B),
              MPF_EINVAL, "mpFlow::numeric::Matrix: bad arguments");
    k_mat_column_reduce<<<cols, 256, 0, s>>>(op, rows, A, op == 1 ? B : nullptr, ld, result, ldr);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int matrix_multiply_scaled(int transA, int transB, int m, int n, int k, float alpha, const float* A, int lda,
                           const float* B, int ldb, float beta, float* C, int ldc, cudaStream_t s) {
    MPF_CHECK(m >= 1 && n >= 1 && k >= 1 && A && B && C && ldc >= m, MPF_EINVAL,
              "mpFlow::numeric::Matrix::multiply: bad arguments");
    MPF_CHECK(lda >= (transA ? k : m) && ldb >= (transB ? n : k), MPF_EINVAL,
              "mpFlow::numeric::Matrix::multiply: leading dimension too small");
    MPF_CHECK((n + 63) / 64 <= 65535, MPF_EINVAL, "mpFlow::numeric::Matrix::multiply: %d columns exceed the grid", n);
    k_mat_gemm<<<dim3((m + 63) / 64, (n + 63) / 64), 256, 0, s>>>(transA, transB, m, n, k, alpha, A, lda, B, ldb,
                                                                  beta, C, ldc);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int matrix_multiply(int transA, int transB, int m, int n, int k, const float* A, int lda, const float* B, int ldb,
                    float* C, int ldc, cudaStream_t s) {
    return matrix_multiply_scaled(transA, transB, m, n, k, 1.f, A, lda, B, ldb, 0.f, C, ldc, s);
}

}  // namespace mpf
