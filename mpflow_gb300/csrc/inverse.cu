// Regularised inverse step of solver::Inverse (src/solver/inverse.cpp:60-238):
//   (J^T J + (ref * factor)^2 R) dsigma = J^T (measurement - calculation)
// for `images` right-hand sides and R in {I, diag(J^T J) (NOSER), L^T L
// (Laplacian)}.  The reference assembles the E x E system with cuBLAS and
// runs an iteration-capped dense CG on it; here
//  * R = I is solved in its dual form dsigma = J^T (J J^T + mu I)^-1 y
//    (identical in exact arithmetic, rowsJ x rowsJ instead of E x E),
//  * NOSER and Laplacian, which have no dual form, build J^T J on the
//    tensor cores (split-BF16 Gram of J^T) and factor the E x E system in
//    FP64 (small meshes: E <= 6144 after padding to 128).
// Both end in an exact FP64 Cholesky solve.  The dual form refines its
// solution against the FP64 normal equations applied matrix-free with the
// FP32 J (the split-BF16 Gram carries ~1e-5 relative error, which 1/mu
// amplifies); when that refinement stalls, the Gram is rebuilt in FP64.
#include <cmath>
#include <unordered_map>

#include "eit_state.h"

namespace mpf {
namespace {

// reference layout J (column-major rowsJ x E) -> row-major [rowsJ][ld], zero padding
__global__ void k_jref_rows(int rowsJ, int E, int ld, const float* __restrict__ Jref, float* __restrict__ J) {
    __shared__ float tile[32][33];
    const int e0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int k = ty; k < 32; k += 8) {
        const int e = e0 + k, r = r0 + tx;
        tile[k][tx] = (e < E && r < rowsJ) ? Jref[(size_t)e * rowsJ + r] : 0.f;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int r = r0 + k, e = e0 + tx;
        if (r < rowsJ && e < ld) J[(size_t)r * ld + e] = tile[tx][k];
    }
}

// out[p][e] = sum_r J[r][e] w[p][r] (J row-major [rowsJ][ld]) in FP64, written
// as float (dsigma, E per image) and/or double (ld per image, zero padding)
__global__ void k_jt_times(int rowsJ, int E, int ld, const float* __restrict__ J, const double* __restrict__ w,
                           float* __restrict__ outF, double* __restrict__ outD) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y;
    if (e >= ld) return;
    double s = 0.0;
    if (e < E)
        for (int r = 0; r < rowsJ; ++r) s += (double)J[(size_t)r * ld + e] * w[(size_t)p * rowsJ + r];
    if (outF && e < E) outF[(size_t)p * E + e] = (float)s;
    if (outD) outD[(size_t)p * ld + e] = s;
}

// res[p][r] = y[p][r] - sum_e J[r][e] u[p][e] - mu w[p][r] in FP64; one block
// per (row, image), fixed-order tree reduction
__global__ void __launch_bounds__(256) k_normal_residual(int rowsJ, int ld, const float* __restrict__ J,
                                                         const double* __restrict__ u, const double* __restrict__ y,
                                                         const double* __restrict__ w, double mu,
                                                         double* __restrict__ res) {
    const int r = blockIdx.x, p = blockIdx.y;
    __shared__ double red[256];
    double s = 0.0;
    for (int e = threadIdx.x; e < ld; e += 256) s += (double)J[(size_t)r * ld + e] * u[(size_t)p * ld + e];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const size_t i = (size_t)p * rowsJ + r;
        res[i] = y[i] - red[0] - mu * w[i];
    }
}

__global__ void k_axpy64(size_t n, const double* __restrict__ d, double* __restrict__ w) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        w[i] += d[i];
}

// regulariser on the FP64 system of padded order n (padding: identity)
__global__ void k_regularise(int n, int E, int type, double mu, double* __restrict__ A) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double& d = A[(size_t)i * n + i];
        if (i >= E) {
            d = 1.0;
        } else if (type == MPF_REG_IDENTITY) {
            d += mu;
        } else if (type == MPF_REG_NOSER) {
            d += mu * d;
        }
    }
}

__global__ void k_add_coo(int nnz, int n, double mu, const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                          const double* __restrict__ val, double* __restrict__ A) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nnz; t += gridDim.x * blockDim.x)
        A[(size_t)row[t] * n + col[t]] += mu * val[t];
}

__global__ void k_to_float_rows(int images, int E, int ld, const double* __restrict__ x, float* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y;
    if (e < E) out[(size_t)p * E + e] = (float)x[(size_t)p * ld + e];
}

}  // namespace

// L^T L of the reference's edge-length Laplacian (src/solver/inverse.cpp:
// 98-113): L[edge][element] = +-length, + at the first element that visits
// the edge and - at the second, so (L^T L)[a][a] is the sum of the squared
// lengths of a's edges and (L^T L)[a][b] = -length^2 for elements sharing an
// edge.  Independent of the edge numbering.
int laplacian_coo(mpf_eit* m) {
    if (m->lapRow.ptr) return MPF_OK;
    const int E = m->E;
    std::unordered_map<unsigned long long, int> first;  // edge -> first element
    std::vector<double> diag(E, 0.0);
    std::vector<int32_t> rows, cols;
    std::vector<double> vals;
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i) {
            const int a = m->hostElements[3 * e + i], b = m->hostElements[3 * e + (i + 1) % 3];
            const double dx = m->hostNodes[2 * a] - m->hostNodes[2 * b];
            const double dy = m->hostNodes[2 * a + 1] - m->hostNodes[2 * b + 1];
            const double l2 = dx * dx + dy * dy;
            const unsigned long long key = ((unsigned long long)std::min(a, b) << 32) | (unsigned)std::max(a, b);
            diag[e] += l2;
            auto it = first.find(key);
            if (it == first.end()) {
                first.emplace(key, e);
            } else {
                rows.push_back(e);
                cols.push_back(it->second);
                vals.push_back(-l2);
                rows.push_back(it->second);
                cols.push_back(e);
                vals.push_back(-l2);
            }
        }
    for (int e = 0; e < E; ++e) {
        rows.push_back(e);
        cols.push_back(e);
        vals.push_back(diag[e]);
    }
    MPF_TRY(m->lapRow.upload(rows));
    MPF_TRY(m->lapCol.upload(cols));
    MPF_TRY(m->lapVal.upload(vals));
    return MPF_OK;
}

static bool pivot_failed(mpf_eit* m, cudaStream_t s);

// w = (J J^T + mu I)^-1 y for the images in invY (overwritten by w): the
// Cholesky solve with the factor in invA, then iterative refinement with the
// residual y - J (J^T w) - mu w in FP64 from the FP32 J in invJ.  A step
// that shrinks the residual by less than half switches to the FP64 Gram
// (once).  Stops at a relative residual of 1e-13 or after 8 steps.
static int refine_dual(mpf_eit* m, int rowsJ, int E, int ld, int images, double mu, bool exact, cudaStream_t s) {
    const size_t ny = (size_t)images * rowsJ;
    MPF_TRY(m->invYs.alloc(ny));
    MPF_TRY(m->invR.alloc(ny));
    MPF_TRY(m->invU.alloc((size_t)images * ld));
    MPF_CUDA(cudaMemcpyAsync(m->invYs.ptr, m->invY.ptr, sizeof(double) * ny, cudaMemcpyDeviceToDevice, s));
    MPF_TRY(dense_cholesky_solve_f64(1, rowsJ, m->invA.ptr, m->invY.ptr, images, s));
    std::vector<double> yh(ny), rh(ny);
    MPF_CUDA(cudaMemcpyAsync(yh.data(), m->invYs.ptr, sizeof(double) * ny, cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    std::vector<double> ynorm(images, 0.0);
    for (int p = 0; p < images; ++p)
        for (int r = 0; r < rowsJ; ++r) ynorm[p] += yh[(size_t)p * rowsJ + r] * yh[(size_t)p * rowsJ + r];
    double prev = 1e300;
    for (int step = 0; step < 8; ++step) {
        k_jt_times<<<dim3((ld + 255) / 256, images), 256, 0, s>>>(rowsJ, E, ld, m->invJ.ptr, m->invY.ptr, nullptr,
                                                                  m->invU.ptr);
        k_normal_residual<<<dim3(rowsJ, images), 256, 0, s>>>(rowsJ, ld, m->invJ.ptr, m->invU.ptr, m->invYs.ptr,
                                                               m->invY.ptr, mu, m->invR.ptr);
        MPF_LAUNCHED(2);
        MPF_CUDA(cudaMemcpyAsync(rh.data(), m->invR.ptr, sizeof(double) * ny, cudaMemcpyDeviceToHost, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        double rel = 0.0;
        for (int p = 0; p < images; ++p) {
            double rr = 0.0;
            for (int r = 0; r < rowsJ; ++r) rr += rh[(size_t)p * rowsJ + r] * rh[(size_t)p * rowsJ + r];
            if (ynorm[p] > 0.0) rel = std::max(rel, std::sqrt(rr / ynorm[p]));
        }
        if (rel <= 1e-13) break;
        if (rel > 0.5 * prev) {
            if (exact) break;
            // the split-BF16 factor is too coarse for this mu: FP64 Gram, solve again
            MPF_TRY(dense_gram_f64_exact(1, rowsJ, ld, m->invJ.ptr, ld, mu, m->invA.ptr, nullptr, s));
            MPF_TRY(dense_cholesky_f64(1, rowsJ, m->invA.ptr, m->invInfo.ptr, s));
            MPF_CUDA(cudaMemcpyAsync(m->invY.ptr, m->invYs.ptr, sizeof(double) * ny, cudaMemcpyDeviceToDevice, s));
            MPF_TRY(dense_cholesky_solve_f64(1, rowsJ, m->invA.ptr, m->invY.ptr, images, s));
            exact = true;
            prev = 1e300;
            continue;
        }
        prev = rel;
        MPF_TRY(dense_cholesky_solve_f64(1, rowsJ, m->invA.ptr, m->invR.ptr, images, s));
        k_axpy64<<<(int)std::min<size_t>((ny + 255) / 256, 1024), 256, 0, s>>>(ny, m->invR.ptr, m->invY.ptr);
        MPF_LAUNCHED(1);
    }
    return MPF_OK;
}

// true when the last Cholesky of the inverse workspace met a non-positive
// pivot (synchronises the stream)
static bool pivot_failed(mpf_eit* m, cudaStream_t s) {
    int info = 0;
    if (cudaMemcpyAsync(&info, m->invInfo.ptr, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return false;
    if (cudaStreamSynchronize(s) != cudaSuccess) return false;
    return info != 0;
}

int inverse_solve(mpf_eit* m, int reg, double factor, int images, const float* Jref, const float* calc,
                  const float* meas, float* result, cudaStream_t s) {
    MPF_CUDA(cudaSetDevice(m->device));
    MPF_CHECK(images >= 1 && Jref && calc && meas && result, MPF_EINVAL,
              "mpFlow::solver::Inverse::solve: bad arguments");
    MPF_CHECK(reg == MPF_REG_IDENTITY || reg == MPF_REG_NOSER || reg == MPF_REG_LAPLACIAN, MPF_EINVAL,
              "mpFlow::solver::Inverse::calcRegularizationMatrix: regularization type not implemented yet");
    const int rowsJ = m->rowsJ, E = m->E;
    const double mu = ((double)m->ref * factor) * ((double)m->ref * factor);
    // y = measurement - calculation in the Jacobian's row order (the per-image
    // residual norms land in invB, which the primal path reuses afterwards)
    const int n = round_up(E, 128);
    MPF_TRY(m->invY.alloc((size_t)images * rowsJ));
    MPF_TRY(m->invB.alloc((size_t)images * (reg == MPF_REG_IDENTITY ? 1 : n)));
    MPF_TRY(m->invInfo.alloc(1));
    MPF_TRY(fem_launch_residual(images, rowsJ, m->Mm, m->Md, meas, calc, m->invY.ptr, m->invB.ptr, s));
    if (reg == MPF_REG_IDENTITY) {
        // dual: w = (J J^T + mu I)^-1 y, dsigma = J^T w
        const int ld = round_up(E, kElemTile);
        MPF_TRY(m->invJ.alloc((size_t)rowsJ * ld));
        MPF_TRY(m->invHi.alloc((size_t)rowsJ * ld));
        MPF_TRY(m->invLo.alloc((size_t)rowsJ * ld));
        MPF_TRY(m->invA.alloc((size_t)rowsJ * rowsJ));
        MPF_TRY(m->invWork.alloc(dense_gram_work_floats(1, rowsJ, ld)));
        k_jref_rows<<<dim3(ld / 32, (rowsJ + 31) / 32), dim3(32, 8), 0, s>>>(rowsJ, E, ld, Jref, m->invJ.ptr);
        MPF_LAUNCHED(1);
        MPF_TRY(dense_split_bf16(1, rowsJ, ld, m->invJ.ptr, ld, m->invHi.ptr, m->invLo.ptr, s));
        MPF_TRY(dense_gram_f64_shift(1, rowsJ, ld, m->invHi.ptr, m->invLo.ptr, ld, mu, m->invA.ptr, m->invWork.ptr,
                                     m->invWork.count, s));
        MPF_TRY(dense_cholesky_f64(1, rowsJ, m->invA.ptr, m->invInfo.ptr, s));
        bool exact = false;
        if (pivot_failed(m, s)) {
            // mu below the split-BF16 Gram's error: the FP64 Gram of the FP32 J
            MPF_TRY(dense_gram_f64_exact(1, rowsJ, ld, m->invJ.ptr, ld, mu, m->invA.ptr, nullptr, s));
            MPF_TRY(dense_cholesky_f64(1, rowsJ, m->invA.ptr, m->invInfo.ptr, s));
            exact = true;
        }
        MPF_TRY(refine_dual(m, rowsJ, E, ld, images, mu, exact, s));
        k_jt_times<<<dim3((ld + 255) / 256, images), 256, 0, s>>>(rowsJ, E, ld, m->invJ.ptr, m->invY.ptr, result,
                                                                    nullptr);
        MPF_LAUNCHED(1);
    } else {
        // primal: (J^T J + mu R) dsigma = J^T y on the E x E system
        MPF_CHECK(n <= 6144, MPF_ENOTSUP,
                  "mpf_inverse_solve: NOSER and Laplacian regularisation solve the E x E system; %d elements exceed "
                  "this library's limit of 6144",
                  E);
        // J as row-major [rowsJ][n] (for J^T y) and J^T as row-major [n][rowsJ] (for the Gram)
        MPF_TRY(m->invJ.alloc((size_t)2 * rowsJ * n));
        float* Jrow = m->invJ.ptr;
        float* Jt = m->invJ.ptr + (size_t)rowsJ * n;
        MPF_TRY(m->invHi.alloc((size_t)n * rowsJ));
        MPF_TRY(m->invLo.alloc((size_t)n * rowsJ));
        MPF_TRY(m->invA.alloc((size_t)n * n));
        MPF_TRY(m->invWork.alloc(dense_gram_work_floats(1, n, rowsJ)));
        k_jref_rows<<<dim3(n / 32, (rowsJ + 31) / 32), dim3(32, 8), 0, s>>>(rowsJ, E, n, Jref, Jrow);
        MPF_LAUNCHED(1);
        MPF_CUDA(cudaMemsetAsync(Jt, 0, sizeof(float) * (size_t)n * rowsJ, s));
        MPF_CUDA(cudaMemcpyAsync(Jt, Jref, sizeof(float) * (size_t)E * rowsJ, cudaMemcpyDeviceToDevice, s));
        MPF_TRY(dense_split_bf16(1, n, rowsJ, Jt, rowsJ, m->invHi.ptr, m->invLo.ptr, s));
        auto regularise = [&]() -> int {
            k_regularise<<<(n + 255) / 256, 256, 0, s>>>(n, E, reg, mu, m->invA.ptr);
            MPF_LAUNCHED(1);
            if (reg == MPF_REG_LAPLACIAN) {
                MPF_TRY(laplacian_coo(m));
                const int nnz = (int)m->lapVal.count;
                k_add_coo<<<(nnz + 255) / 256, 256, 0, s>>>(nnz, n, mu, m->lapRow.ptr, m->lapCol.ptr, m->lapVal.ptr,
                                                             m->invA.ptr);
                MPF_LAUNCHED(1);
            }
            return MPF_OK;
        };
        MPF_TRY(dense_gram_f64_shift(1, n, rowsJ, m->invHi.ptr, m->invLo.ptr, rowsJ, 0.0, m->invA.ptr, m->invWork.ptr,
                                     m->invWork.count, s));
        MPF_TRY(regularise());
        k_jt_times<<<dim3((n + 255) / 256, images), 256, 0, s>>>(rowsJ, E, n, Jrow, m->invY.ptr, nullptr, m->invB.ptr);
        MPF_LAUNCHED(1);
        MPF_TRY(dense_cholesky_f64(1, n, m->invA.ptr, m->invInfo.ptr, s));
        if (pivot_failed(m, s)) {
            MPF_TRY(dense_gram_f64_exact(1, n, rowsJ, Jt, rowsJ, 0.0, m->invA.ptr, nullptr, s));
            MPF_TRY(regularise());
            MPF_TRY(dense_cholesky_f64(1, n, m->invA.ptr, m->invInfo.ptr, s));
        }
        MPF_TRY(dense_cholesky_solve_f64(1, n, m->invA.ptr, m->invB.ptr, images, s));
        k_to_float_rows<<<dim3((E + 255) / 256, images), 256, 0, s>>>(images, E, n, m->invB.ptr, result);
        MPF_LAUNCHED(1);
    }
    int info = 0;
    MPF_CUDA(cudaMemcpyAsync(&info, m->invInfo.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    bool aborted = false;
    MPF_TRY(dense_gram_check_abort(&aborted));
    MPF_CHECK(!aborted, MPF_ETIMEOUT, "mpf_inverse_solve: a Gram pipeline wait timed out");
    MPF_CHECK(info == 0, MPF_EBREAKDOWN, "mpFlow::solver::Inverse::solve: system not positive definite (pivot %d)",
              info);
    return MPF_OK;
}

}  // namespace mpf
