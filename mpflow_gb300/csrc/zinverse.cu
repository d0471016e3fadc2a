// Complex regularised inverse step, solver::Inverse<thrust::complex<float>>
// (src/solver/inverse.cpp:60-238, instantiated at :243):
//   (J^T J + (ref * factor)^2 R) dsigma = J^T (measurement - calculation)
// with the plain, unconjugated transpose (the reference's CUBLAS_OP_T gemm
// on complex data, inverse.cpp:140-150 and :195-202), for `images`
// right-hand sides and R in {I, diag(J^T J) (NOSER), L^T L (Laplacian)}.
// J^T J + mu R is complex symmetric, not Hermitian; the reference runs its
// dense CG on it.  Here it is solved exactly:
//  * R = I in the dual form dsigma = J^T (J J^T + mu I)^-1 y (the push-through
//    identity holds for the plain transpose), rowsJ x rowsJ;
//  * NOSER and Laplacian on the E x E system (E <= 6144 after padding).
// Both form the Gram in FP64 from the FP32 complex J (tiled, complex FMAs)
// and factor it as L L^T in complex FP64 without pivoting (the symmetric
// factorisation exists when every leading minor is non-zero; a zero pivot is
// reported as MPF_EBREAKDOWN).  Complex values are interleaved (re, im)
// float pairs, the memory layout of thrust::complex<float>.
#include <cmath>

#include "eit_state.h"

namespace mpf {

int laplacian_coo(mpf_eit* m);  // inverse.cu

namespace {

constexpr int ZB = 32;  // factorisation block

struct zd {
    double x, y;
};

__device__ __forceinline__ zd zsub(zd a, zd b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ zd zmul(zd a, zd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
// c + a b
__device__ __forceinline__ zd zfma(zd a, zd b, zd c) {
    return {fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))};
}
// a / b by Smith's scaling (R. L. Smith, CACM 5(8), 1962)
__device__ __forceinline__ zd zdiv(zd a, zd b) {
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
    }
    const double r = b.x / b.y, d = b.y + b.x * r;
    return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
}
// principal square root from |z|: sqrt((|z| + |x|) / 2) on the component
// that does not cancel, the other one from y / (2 t)
__device__ __forceinline__ zd zsqrt(zd z) {
    if (z.x == 0.0 && z.y == 0.0) return {0.0, 0.0};
    const double r = hypot(z.x, z.y);
    if (z.x >= 0.0) {
        const double t = sqrt(0.5 * (r + z.x));
        return {t, z.y / (2.0 * t)};
    }
    const double t = sqrt(0.5 * (r - z.x));
    return {fabs(z.y) / (2.0 * t), copysign(t, z.y)};
}
__device__ __forceinline__ zd zload(const float2* p) {
    const float2 v = *p;
    return {(double)v.x, (double)v.y};
}

// reference layout J (column-major rowsJ x E) -> row-major [rowsJ][ld], zero padding
__global__ void k_zjref_rows(int rowsJ, int E, int ld, const float2* __restrict__ Jref, float2* __restrict__ J) {
    __shared__ float2 tile[32][33];
    const int e0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int k = ty; k < 32; k += 8) {
        const int e = e0 + k, r = r0 + tx;
        tile[k][tx] = (e < E && r < rowsJ) ? Jref[(size_t)e * rowsJ + r] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int r = r0 + k, e = e0 + tx;
        if (r < rowsJ && e < ld) J[(size_t)r * ld + e] = tile[tx][k];
    }
}

// A = J J^T + shift I (no conjugation) in FP64 for J row-major [rows][ld]
// (cols used); 32 x 32 output tiles on and above the diagonal, mirrored;
// 256 threads with 2 x 2 outputs each, k in chunks of 16.
__global__ void __launch_bounds__(256) k_zgram64(int rows, int cols, const float2* __restrict__ J, int ld,
                                                 double shift, zd* __restrict__ A) {
    const int ti = blockIdx.y, tj = blockIdx.x;
    if (tj < ti) return;
    __shared__ zd As[16][33], Bs[16][33];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    zd acc[2][2] = {};
    for (int k0 = 0; k0 < cols; k0 += 16) {
        for (int t = threadIdx.x; t < 32 * 16; t += 256) {
            const int r = t / 16, k = t % 16, kk = k0 + k;
            As[k][r] = kk < cols ? zload(J + (size_t)(ti * 32 + r) * ld + kk) : zd{0.0, 0.0};
            Bs[k][r] = kk < cols ? zload(J + (size_t)(tj * 32 + r) * ld + kk) : zd{0.0, 0.0};
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < 16; ++k) {
            const zd a0 = As[k][ty], a1 = As[k][ty + 16], b0 = Bs[k][tx], b1 = Bs[k][tx + 16];
            acc[0][0] = zfma(a0, b0, acc[0][0]);
            acc[0][1] = zfma(a0, b1, acc[0][1]);
            acc[1][0] = zfma(a1, b0, acc[1][0]);
            acc[1][1] = zfma(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int r = ti * 32 + ty + 16 * i, c = tj * 32 + tx + 16 * j;
            zd v = acc[i][j];
            if (r == c) v.x += shift;
            A[(size_t)r * rows + c] = v;
            A[(size_t)c * rows + r] = v;
        }
}

// L L^T of the diagonal block k (column-major, lower triangle holds L)
__global__ void k_zpotrf_diag(int n, zd* A, int k, int* info) {
    __shared__ zd a[ZB][ZB + 1];
    __shared__ int bad;
    const int o = k * ZB;
    for (int i = threadIdx.x; i < ZB * ZB; i += blockDim.x) {
        const int r = i % ZB, c = i / ZB;
        a[r][c] = A[(size_t)(o + r) + (size_t)(o + c) * n];
    }
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < ZB; ++j) {
        if (threadIdx.x == 0) {
            const zd d = a[j][j];
            if (!(hypot(d.x, d.y) > 0.0) || !isfinite(d.x) || !isfinite(d.y)) {
                if (!bad && *info == 0) *info = o + j + 1;
                bad = 1;
                a[j][j] = {1.0, 0.0};
            } else {
                a[j][j] = zsqrt(d);
            }
        }
        __syncthreads();
        for (int i = j + 1 + threadIdx.x; i < ZB; i += blockDim.x) a[i][j] = zdiv(a[i][j], a[j][j]);
        __syncthreads();
        for (int idx = threadIdx.x; idx < ZB * ZB; idx += blockDim.x) {
            const int i = idx % ZB, l = idx / ZB;
            if (l > j && i >= l) a[i][l] = zsub(a[i][l], zmul(a[i][j], a[l][j]));
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < ZB * ZB; i += blockDim.x) {
        const int r = i % ZB, c = i / ZB;
        if (r >= c) A[(size_t)(o + r) + (size_t)(o + c) * n] = a[r][c];
    }
}

// L_ik = A_ik L_kk^-T for the block rows below block k
__global__ void k_ztrsm(int n, zd* A, int k) {
    __shared__ zd L[ZB][ZB + 1];
    __shared__ zd X[ZB][ZB + 1];
    const int o = k * ZB, ro = (k + 1 + blockIdx.x) * ZB;
    for (int i = threadIdx.x; i < ZB * ZB; i += blockDim.x) {
        const int r = i % ZB, c = i / ZB;
        L[r][c] = A[(size_t)(o + r) + (size_t)(o + c) * n];
        X[r][c] = A[(size_t)(ro + r) + (size_t)(o + c) * n];
    }
    __syncthreads();
    if (threadIdx.x < ZB) {
        const int r = threadIdx.x;
        for (int j = 0; j < ZB; ++j) {
            zd s = X[r][j];
            for (int l = 0; l < j; ++l) s = zsub(s, zmul(X[r][l], L[j][l]));
            X[r][j] = zdiv(s, L[j][j]);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ZB * ZB; i += blockDim.x) {
        const int r = i % ZB, c = i / ZB;
        A[(size_t)(ro + r) + (size_t)(o + c) * n] = X[r][c];
    }
}

// A_ij -= L_ik L_jk^T for k < j <= i
__global__ void __launch_bounds__(256) k_zsyrk(int n, zd* A, int k) {
    __shared__ zd Li[ZB][ZB + 1];
    __shared__ zd Lj[ZB][ZB + 1];
    int t = blockIdx.x, bi = 0;
    while (t > bi) {
        t -= bi + 1;
        ++bi;
    }
    const int bj = t;
    const int o = k * ZB, io = (k + 1 + bi) * ZB, jo = (k + 1 + bj) * ZB;
    for (int i = threadIdx.x; i < ZB * ZB; i += blockDim.x) {
        const int r = i % ZB, c = i / ZB;
        Li[r][c] = A[(size_t)(io + r) + (size_t)(o + c) * n];
        Lj[r][c] = A[(size_t)(jo + r) + (size_t)(o + c) * n];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < ZB * ZB; idx += blockDim.x) {
        const int r = idx % ZB, c = idx / ZB;
        zd s = {0.0, 0.0};
#pragma unroll 8
        for (int l = 0; l < ZB; ++l) s = zfma(Li[r][l], Lj[c][l], s);
        zd& d = A[(size_t)(io + r) + (size_t)(jo + c) * n];
        d = zsub(d, s);
    }
}

// L L^T x = b per right-hand side (one block of 256 threads each), in 32-row
// block steps as the real solve: right-looking forward pass, left-looking
// backward pass, diagonal blocks by one warp with shuffles.
__global__ void __launch_bounds__(256) k_zchol_solve(int n, const zd* __restrict__ L, zd* __restrict__ Ball) {
    extern __shared__ zd zx[];
    __shared__ zd D[ZB][ZB + 1];
    zd* B = Ball + (size_t)blockIdx.x * n;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int i = threadIdx.x; i < n; i += blockDim.x) zx[i] = B[i];
    const int nb = n / ZB;
    for (int bk = 0; bk < nb; ++bk) {
        const int k0 = bk * ZB;
        for (int i = threadIdx.x; i < ZB * ZB; i += blockDim.x) {
            const int r = i % ZB, c = i / ZB;
            D[r][c] = L[(size_t)(k0 + r) + (size_t)(k0 + c) * n];
        }
        __syncthreads();
        if (warp == 0) {
            zd xr = zx[k0 + lane];
            for (int j = 0; j < ZB; ++j) {
                if (lane == j) xr = zdiv(xr, D[j][j]);
                const zd xj = {__shfl_sync(0xffffffffu, xr.x, j), __shfl_sync(0xffffffffu, xr.y, j)};
                if (lane > j) xr = zsub(xr, zmul(D[lane][j], xj));
            }
            zx[k0 + lane] = xr;
        }
        __syncthreads();
        for (int r = k0 + ZB + threadIdx.x; r < n; r += blockDim.x) {
            zd s = {0.0, 0.0};
#pragma unroll 4
            for (int j = 0; j < ZB; ++j) s = zfma(L[(size_t)r + (size_t)(k0 + j) * n], zx[k0 + j], s);
            zx[r] = zsub(zx[r], s);
        }
    }
    for (int bk = nb - 1; bk >= 0; --bk) {
        const int k0 = bk * ZB, below = k0 + ZB;
        __syncthreads();
        for (int cc = warp; cc < ZB; cc += nwarps) {
            const int col = k0 + cc;
            zd s = {0.0, 0.0};
            for (int r = below + lane; r < n; r += 32) s = zfma(L[(size_t)r + (size_t)col * n], zx[r], s);
            for (int o = 16; o > 0; o >>= 1) {
                s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
                s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
            }
            if (lane == 0) zx[col] = zsub(zx[col], s);
        }
        for (int i = threadIdx.x; i < ZB * ZB; i += blockDim.x) {
            const int r = i % ZB, c = i / ZB;
            D[r][c] = L[(size_t)(k0 + r) + (size_t)(k0 + c) * n];
        }
        __syncthreads();
        if (warp == 0) {
            zd xc = zx[k0 + lane];
            for (int j = ZB - 1; j >= 0; --j) {
                if (lane == j) xc = zdiv(xc, D[j][j]);
                const zd xj = {__shfl_sync(0xffffffffu, xc.x, j), __shfl_sync(0xffffffffu, xc.y, j)};
                if (lane < j) xc = zsub(xc, zmul(D[j][lane], xj));
            }
            zx[k0 + lane] = xc;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) B[i] = zx[i];
}

// out[p][e] = sum_r J[r][e] w[p][r] (J row-major [rowsJ][ld], no conjugation)
// in FP64, as complex float (E per image) and/or complex double (ld per image)
__global__ void k_zjt_times(int rowsJ, int E, int ld, const float2* __restrict__ J, const zd* __restrict__ w,
                            float2* __restrict__ outF, zd* __restrict__ outD) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y;
    if (e >= ld) return;
    zd s = {0.0, 0.0};
    if (e < E)
        for (int r = 0; r < rowsJ; ++r) s = zfma(zload(J + (size_t)r * ld + e), w[(size_t)p * rowsJ + r], s);
    if (outF && e < E) outF[(size_t)p * E + e] = make_float2((float)s.x, (float)s.y);
    if (outD) outD[(size_t)p * ld + e] = s;
}

// y[p][row] = meas - calc in the Jacobian's row order row = m + d * MP (zero
// on padding rows); meas / calc per image column-major Mm x Md
__global__ void k_zresidual(int rowsJ, int Mm, int Md, int MP, const float2* __restrict__ meas,
                            const float2* __restrict__ calc, zd* __restrict__ y) {
    const int p = blockIdx.y;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < rowsJ; row += gridDim.x * blockDim.x) {
        const int m = row % MP, d = row / MP;
        zd v = {0.0, 0.0};
        if (m < Mm && d < Md) {
            const size_t i = (size_t)p * Mm * Md + m + (size_t)d * Mm;
            v = zsub(zload(meas + i), zload(calc + i));
        }
        y[(size_t)p * rowsJ + row] = v;
    }
}

// regulariser on the order-n system (padding rows and columns: identity)
__global__ void k_zregularise(int n, int E, int type, double mu, zd* __restrict__ A) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        zd& d = A[(size_t)i * n + i];
        if (i >= E) {
            d = {1.0, 0.0};
        } else if (type == MPF_REG_IDENTITY) {
            d.x += mu;
        } else if (type == MPF_REG_NOSER) {
            d = {d.x * (1.0 + mu), d.y * (1.0 + mu)};
        }
    }
}

__global__ void k_zadd_coo(int nnz, int n, double mu, const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                           const double* __restrict__ val, zd* __restrict__ A) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nnz; t += gridDim.x * blockDim.x)
        A[(size_t)row[t] * n + col[t]].x += mu * val[t];
}

__global__ void k_zto_float(int E, int ld, const zd* __restrict__ x, float2* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y;
    if (e < E) {
        const zd v = x[(size_t)p * ld + e];
        out[(size_t)p * E + e] = make_float2((float)v.x, (float)v.y);
    }
}

int zcholesky(int n, zd* A, int* info, cudaStream_t s) {
    MPF_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
    const int nb = n / ZB;
    for (int k = 0; k < nb; ++k) {
        k_zpotrf_diag<<<1, 256, 0, s>>>(n, A, k, info);
        const int m = nb - k - 1;
        if (m > 0) {
            k_ztrsm<<<m, 64, 0, s>>>(n, A, k);
            k_zsyrk<<<m * (m + 1) / 2, 256, 0, s>>>(n, A, k);
        }
    }
    MPF_LAUNCHED(3 * nb - 2);
    return MPF_OK;
}

int zcholesky_solve(int n, const zd* L, zd* B, int nrhs, cudaStream_t s) {
    const size_t bytes = (size_t)n * sizeof(zd);
    MPF_CHECK(bytes <= 192 * 1024, MPF_EINVAL, "complex Cholesky solve: order %d too large", n);
    if (bytes > 30 * 1024)
        MPF_CUDA(cudaFuncSetAttribute(k_zchol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    k_zchol_solve<<<nrhs, 256, bytes, s>>>(n, L, B);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

}  // namespace

int inverse_solve_complex(mpf_eit* m, int reg, double factor, int images, const float* JrefF, const float* calcF,
                          const float* measF, float* resultF, cudaStream_t s) {
    MPF_CUDA(cudaSetDevice(m->device));
    MPF_CHECK(images >= 1 && JrefF && calcF && measF && resultF, MPF_EINVAL,
              "mpFlow::solver::Inverse::solve: bad arguments");
    MPF_CHECK(reg == MPF_REG_IDENTITY || reg == MPF_REG_NOSER || reg == MPF_REG_LAPLACIAN, MPF_EINVAL,
              "mpFlow::solver::Inverse::calcRegularizationMatrix: regularization type not implemented yet");
    MPF_CHECK(images <= 65535, MPF_EINVAL, "mpf_inverse_solve_complex: %d images", images);
    const float2* Jref = reinterpret_cast<const float2*>(JrefF);
    const float2* calc = reinterpret_cast<const float2*>(calcF);
    const float2* meas = reinterpret_cast<const float2*>(measF);
    float2* result = reinterpret_cast<float2*>(resultF);
    const int rowsJ = m->rowsJ, E = m->E;
    const double mu = ((double)m->ref * factor) * ((double)m->ref * factor);
    const int MP = rowsJ / (int)data_rows((uint32_t)m->Md);
    MPF_CHECK(rowsJ % ZB == 0, MPF_EINVAL, "mpf_inverse_solve_complex: %d Jacobian rows", rowsJ);
    DevBuf<zd> y, A, b;
    DevBuf<float2> Jrow, Jt;
    DevBuf<int> info;
    MPF_TRY(y.alloc((size_t)images * rowsJ));
    MPF_TRY(info.alloc(1));
    k_zresidual<<<dim3((rowsJ + 255) / 256, images), 256, 0, s>>>(rowsJ, m->Mm, m->Md, MP, meas, calc, y.ptr);
    MPF_LAUNCHED(1);
    if (reg == MPF_REG_IDENTITY) {
        // dual: w = (J J^T + mu I)^-1 y, dsigma = J^T w
        const int ld = round_up(E, 32);
        MPF_TRY(Jrow.alloc((size_t)rowsJ * ld));
        MPF_TRY(A.alloc((size_t)rowsJ * rowsJ));
        k_zjref_rows<<<dim3(ld / 32, rowsJ / 32), dim3(32, 8), 0, s>>>(rowsJ, E, ld, Jref, Jrow.ptr);
        k_zgram64<<<dim3(rowsJ / 32, rowsJ / 32), 256, 0, s>>>(rowsJ, ld, Jrow.ptr, ld, mu, A.ptr);
        MPF_LAUNCHED(2);
        MPF_TRY(zcholesky(rowsJ, A.ptr, info.ptr, s));
        MPF_TRY(zcholesky_solve(rowsJ, A.ptr, y.ptr, images, s));
        k_zjt_times<<<dim3((ld + 255) / 256, images), 256, 0, s>>>(rowsJ, E, ld, Jrow.ptr, y.ptr, result, nullptr);
        MPF_LAUNCHED(1);
    } else {
        // primal: (J^T J + mu R) dsigma = J^T y on the E x E system
        const int n = round_up(E, 32);
        MPF_CHECK(n <= 6144, MPF_ENOTSUP,
                  "mpf_inverse_solve_complex: NOSER and Laplacian regularisation solve the E x E system; %d elements "
                  "exceed this library's limit of 6144",
                  E);
        MPF_TRY(Jrow.alloc((size_t)rowsJ * n));
        MPF_TRY(Jt.alloc((size_t)n * rowsJ));
        MPF_TRY(A.alloc((size_t)n * n));
        MPF_TRY(b.alloc((size_t)images * n));
        k_zjref_rows<<<dim3(n / 32, rowsJ / 32), dim3(32, 8), 0, s>>>(rowsJ, E, n, Jref, Jrow.ptr);
        MPF_LAUNCHED(1);
        // J^T as row-major [n][rowsJ] is the reference layout itself, zero rows below E
        MPF_CUDA(cudaMemsetAsync(Jt.ptr, 0, sizeof(float2) * (size_t)n * rowsJ, s));
        MPF_CUDA(cudaMemcpyAsync(Jt.ptr, Jref, sizeof(float2) * (size_t)E * rowsJ, cudaMemcpyDeviceToDevice, s));
        k_zgram64<<<dim3(n / 32, n / 32), 256, 0, s>>>(n, rowsJ, Jt.ptr, rowsJ, 0.0, A.ptr);
        k_zregularise<<<(n + 255) / 256, 256, 0, s>>>(n, E, reg, mu, A.ptr);
        MPF_LAUNCHED(2);
        if (reg == MPF_REG_LAPLACIAN) {
            MPF_TRY(laplacian_coo(m));
            const int nnz = (int)m->lapVal.count;
            k_zadd_coo<<<(nnz + 255) / 256, 256, 0, s>>>(nnz, n, mu, m->lapRow.ptr, m->lapCol.ptr, m->lapVal.ptr,
                                                          A.ptr);
            MPF_LAUNCHED(1);
        }
        k_zjt_times<<<dim3((n + 255) / 256, images), 256, 0, s>>>(rowsJ, E, n, Jrow.ptr, y.ptr, nullptr, b.ptr);
        MPF_LAUNCHED(1);
        MPF_TRY(zcholesky(n, A.ptr, info.ptr, s));
        MPF_TRY(zcholesky_solve(n, A.ptr, b.ptr, images, s));
        k_zto_float<<<dim3((E + 255) / 256, images), 256, 0, s>>>(E, n, b.ptr, result);
        MPF_LAUNCHED(1);
    }
    int hinfo = 0;
    MPF_CUDA(cudaMemcpyAsync(&hinfo, info.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    MPF_CUDA(cudaGetLastError());
    MPF_CHECK(hinfo == 0, MPF_EBREAKDOWN,
              "mpFlow::solver::Inverse::solve: complex symmetric system has a zero pivot at %d", hinfo);
    return MPF_OK;
}

}  // namespace mpf
