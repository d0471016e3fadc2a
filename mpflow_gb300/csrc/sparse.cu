// Standalone sparse matrix and Krylov solvers on a caller's matrix:
// numeric::SparseMatrix::multiply (src/numeric/sparse_matrix.cpp:262-288),
// numeric::ConjugateGradient::solve (src/numeric/conjugate_gradient.cpp:61-161)
// and numeric::BiCGSTAB::solve (src/numeric/bicgstab.cpp:83-193) outside the
// EIT model.
//
// The caller's matrix arrives in the reference ELL layout (dataRows x 32
// row-major values and column ids, 0xFFFFFFFF padding) and is kept in the
// slot-major layout of the EIT systems ({value, 0} slots, padding slots on
// the own row), so the batched solver kernels of cg_kernels.cu and
// bicgstab_kernels.cu run on it unchanged: the columns of b are KP
// right-hand sides of one group.  Vectors are the reference's column-major
// dataRows x cols matrices; they are transposed to and from the node-major
// layout around a solve.  dcFree solves (A + 1 1^T) x = b as the reference's
// iteration does (c' = 1, no shift).
#include <algorithm>
#include <cstring>
#include <memory>

#include "model.h"

struct mpf_sparse {
    int device = 0, rows = 0, dataRows = 0, npad = 0, nblk = 0, W = 0;
    mpf::DevBuf<int32_t> cols, diagSlot, dcFree;
    mpf::DevBuf<float2> SR;
    mpf::DevBuf<float> alpha;
    // solver workspace for right-hand-side width capKP (one group)
    int capKP = 0;
    mpf::DevBuf<float> X, Rv, Pv, Qv, B, Rhat, Zv, Tv;
    mpf::DevBuf<double> partA, partB, partC, rz, pq, bz, betaW, sumP, sumX, omegaW, rr2W, alphaX;
    mpf::DevBuf<int> conv, active, iters, pend;
    mpf::DevBuf<unsigned> counter;
    int* pinned = nullptr;
    mpf::CgGraphCache graphs;
    ~mpf_sparse() {
        mpf::cg_graphs_clear(graphs);
        if (pinned) cudaFreeHost(pinned);
    }
};

namespace mpf {
namespace {

// y[c][row] = sum_k A[row][k] x[c][col_k] for the caller's column-major
// matrices (one thread per row, coalesced over rows)
__global__ void k_ell_multiply_cm(int rows, int npad, int W, const int32_t* __restrict__ cols,
                                  const float2* __restrict__ SR, const float* __restrict__ x, int ldx,
                                  float* __restrict__ y, int ldy) {
    const int c = blockIdx.y;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < rows; row += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < W; ++k) {
            const size_t sl = (size_t)k * npad + row;
            s = fmaf(__ldg(&SR[sl]).x, __ldg(&x[(size_t)c * ldx + __ldg(&cols[sl])]), s);
        }
        y[(size_t)c * ldy + row] = s;
    }
}

// column-major (ld) <-> node-major [npad][KP], zero padding
__global__ void k_cm_to_nm(int rows, int cols, const float* __restrict__ src, int ld, int npad, int KP,
                           float* __restrict__ dst) {
    const size_t total = (size_t)npad * KP;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int row = (int)(i / KP), c = (int)(i % KP);
        dst[i] = (row < rows && c < cols) ? src[(size_t)c * ld + row] : 0.f;
    }
}
__global__ void k_nm_to_cm(int rows, int cols, const float* __restrict__ src, int KP, float* __restrict__ dst,
                           int ld) {
    const size_t total = (size_t)rows * cols;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i / rows), row = (int)(i % rows);
        dst[(size_t)c * ld + row] = src[(size_t)row * KP + c];
    }
}

int width_for(int cols) {
    for (int kp : {16, 32, 64, 128})
        if (cols <= kp) return kp;
    return 128;
}

int sparse_workspace(mpf_sparse* A, int KP) {
    if (KP <= A->capKP) return MPF_OK;
    const size_t vec = (size_t)A->npad * KP, parts = (size_t)A->nblk * KP;
    for (auto* b : {&A->X, &A->Rv, &A->Pv, &A->Qv, &A->B, &A->Rhat, &A->Zv, &A->Tv}) MPF_TRY(b->alloc(vec));
    for (auto* b : {&A->partA, &A->partB, &A->partC}) MPF_TRY(b->alloc(parts));
    for (auto* b : {&A->rz, &A->pq, &A->bz, &A->betaW, &A->sumP, &A->sumX, &A->omegaW, &A->rr2W, &A->alphaX})
        MPF_TRY(b->alloc((size_t)KP));
    MPF_TRY(A->conv.alloc((size_t)KP));
    MPF_TRY(A->active.alloc(1));
    MPF_TRY(A->iters.alloc(1));
    MPF_TRY(A->pend.alloc(1));
    MPF_TRY(A->counter.alloc(1));
    MPF_CUDA(cudaMemset(A->counter.ptr, 0, sizeof(unsigned)));
    MPF_CUDA(cudaMemset(A->pend.ptr, 0, sizeof(int)));
    if (!A->pinned) MPF_CUDA(cudaMallocHost(&A->pinned, sizeof(int) * 4));
    cg_graphs_clear(A->graphs);
    A->capKP = KP;
    return MPF_OK;
}

}  // namespace

int sparse_create(int rows, const float* values, const uint32_t* columnIds, uint32_t density, mpf_sparse** out) {
    MPF_CHECK(rows >= 1 && values && columnIds && out, MPF_EINVAL, "mpFlow::numeric::SparseMatrix: bad arguments");
    MPF_CHECK(density <= kEllWidth, MPF_EFULL, "mpFlow::numeric::SparseMatrix::setValue: sparse format full");
    auto A = new mpf_sparse();
    std::unique_ptr<mpf_sparse> guard(A);
    MPF_CUDA(cudaGetDevice(&A->device));
    A->rows = rows;
    A->dataRows = (int)data_rows((uint32_t)rows);
    A->npad = round_up(rows, kRowTile);
    A->nblk = A->npad / kRowTile;
    const size_t ell = (size_t)A->dataRows * kEllWidth;
    std::vector<float> hv(ell);
    std::vector<uint32_t> hc(ell);
    MPF_CUDA(cudaMemcpy(hv.data(), values, sizeof(float) * ell, cudaMemcpyDeviceToHost));
    MPF_CUDA(cudaMemcpy(hc.data(), columnIds, sizeof(uint32_t) * ell, cudaMemcpyDeviceToHost));
    // one extra zero slot when a full row has no diagonal entry (its Jacobi
    // inverse is then taken from that zero slot, i.e. 0)
    A->W = std::max<int>(1, (int)density);
    for (int r = 0; r < rows && A->W == (int)density && A->W < (int)kEllWidth; ++r) {
        bool hasDiag = false, full = true;
        for (int k = 0; k < (int)density; ++k) {
            const uint32_t c = hc[(size_t)r * kEllWidth + k];
            hasDiag |= c == (uint32_t)r;
            full &= c != kInvalid;
        }
        if (!hasDiag && full) A->W = (int)density + 1;
    }
    std::vector<int32_t> cols((size_t)A->W * A->npad), diag(A->npad);
    std::vector<float2> sr((size_t)A->W * A->npad, make_float2(0.f, 0.f));
    for (int r = 0; r < A->npad; ++r) {
        int d = -1, pad = -1;
        for (int k = 0; k < A->W; ++k) {
            const size_t sl = (size_t)k * A->npad + r;
            const uint32_t c = r < rows ? hc[(size_t)r * kEllWidth + k] : kInvalid;
            if (c != kInvalid) {
                MPF_CHECK((int)c < rows, MPF_EINVAL, "mpFlow::numeric::SparseMatrix: column %u of row %d out of range",
                          c, r);
                cols[sl] = (int32_t)c;
                sr[sl].x = hv[(size_t)r * kEllWidth + k];
                if ((int)c == r && d < 0) d = k;
            } else {
                cols[sl] = r;
                if (pad < 0) pad = k;
            }
        }
        // rows without a diagonal entry get a zero inverse (a padding slot)
        diag[r] = d >= 0 ? d : (pad >= 0 ? pad : 0);
    }
    MPF_TRY(A->cols.upload(cols));
    MPF_TRY(A->diagSlot.upload(diag));
    MPF_TRY(A->SR.upload(sr));
    MPF_TRY(A->alpha.upload(std::vector<float>{0.f}));
    MPF_TRY(A->dcFree.alloc(1));
    *out = guard.release();
    return MPF_OK;
}

void sparse_destroy(mpf_sparse* A) {
    if (A) cudaSetDevice(A->device);
    delete A;
}

int sparse_multiply(mpf_sparse* A, const float* x, int ldx, int cols, float* y, int ldy, cudaStream_t s) {
    MPF_CHECK(x && y && cols >= 1 && ldx >= A->rows && ldy >= A->rows, MPF_EINVAL,
              "mpFlow::numeric::SparseMatrix::multiply: bad arguments");
    MPF_CUDA(cudaSetDevice(A->device));
    const int blocks = std::min((A->rows + 255) / 256, 2048);
    k_ell_multiply_cm<<<dim3(blocks, cols), 256, 0, s>>>(A->rows, A->npad, A->W, A->cols.ptr, A->SR.ptr, x, ldx, y,
                                                          ldy);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int sparse_solve(mpf_sparse* A, int solver, const float* b, int ldb, float* x, int ldx, int cols, int maxIter,
                 double tol, int dcFree, int32_t* iterations, cudaStream_t s) {
    MPF_CHECK(b && x && cols >= 1 && ldb >= A->rows && ldx >= A->rows, MPF_EINVAL,
              "mpFlow::numeric::ConjugateGradient::solve: bad arguments");
    MPF_CUDA(cudaSetDevice(A->device));
    if (tol <= 0.0) tol = 1.1920928955078125e-07;  // the reference's stopping level: float epsilon
    if (maxIter <= 0) maxIter = 10 * A->rows;
    int total = 0, notConv = 0;
    // chunks of at most 128 right-hand sides
    for (int c0 = 0; c0 < cols; c0 += 128) {
        const int nc = std::min(128, cols - c0), KP = width_for(nc);
        MPF_TRY(sparse_workspace(A, KP));
        const int dc = dcFree ? 1 : 0;
        MPF_CUDA(cudaMemcpyAsync(A->dcFree.ptr, &dc, sizeof(int), cudaMemcpyHostToDevice, s));
        const size_t vec = (size_t)A->npad * KP;
        const int blocks = (int)std::min<size_t>((vec + 255) / 256, 4096);
        k_cm_to_nm<<<blocks, 256, 0, s>>>(A->rows, nc, b + (size_t)c0 * ldb, ldb, A->npad, KP, A->B.ptr);
        k_cm_to_nm<<<blocks, 256, 0, s>>>(A->rows, nc, x + (size_t)c0 * ldx, ldx, A->npad, KP, A->X.ptr);
        MPF_LAUNCHED(2);
        CgProblem P{};
        P.n = A->rows;
        P.npad = A->npad;
        P.W = A->W;
        P.KP = KP;
        P.G = 1;
        P.Ca = 1;
        P.nblk = A->nblk;
        P.M = 1;
        P.cols = A->cols.ptr;
        P.diagSlot = A->diagSlot.ptr;
        P.SR = A->SR.ptr;
        P.alpha = A->alpha.ptr;
        P.x = A->X.ptr;
        P.r = A->Rv.ptr;
        P.p = A->Pv.ptr;
        P.q = A->Qv.ptr;
        P.b = A->B.ptr;
        P.bPerGroup = 1;
        P.dcFree = A->dcFree.ptr;
        P.partA = A->partA.ptr;
        P.partB = A->partB.ptr;
        P.partC = A->partC.ptr;
        P.sumP = A->sumP.ptr;
        P.dcScale = 1.f;  // the reference's (A + 1 1^T)
        P.rz = A->rz.ptr;
        P.pq = A->pq.ptr;
        P.bz = A->bz.ptr;
        P.beta = A->betaW.ptr;
        P.conv = A->conv.ptr;
        P.active = A->active.ptr;
        P.iters = A->iters.ptr;
        P.counter = A->counter.ptr;
        P.alphaX = A->alphaX.ptr;
        P.pend = A->pend.ptr;
        P.tol2 = tol * tol;
        for (int k = 0; k < 3; ++k) cg_set_shape(P, k, cg_default_variant(KP));
        if (solver == 1) {
            P.solver = 1;
            P.rhat = A->Rhat.ptr;
            P.zv = A->Zv.ptr;
            P.tv = A->Tv.ptr;
            P.omega = A->omegaW.ptr;
            P.rr2 = A->rr2W.ptr;
        }
        if (dcFree) {
            MPF_TRY(cg_launch_colsum(P, A->X.ptr, nullptr, A->sumX.ptr, s));
            P.sumX0 = A->sumX.ptr;
        }
        MPF_TRY(cg_launch_init(P, false, s));
        std::vector<int> it;
        int mx = 0, nconv = 0;
        MPF_TRY(cg_run(A->graphs, A->pinned, &P, 1, maxIter, 16, s, it, &mx, &nconv));
        k_nm_to_cm<<<blocks, 256, 0, s>>>(A->rows, nc, A->X.ptr, KP, x + (size_t)c0 * ldx, ldx);
        MPF_LAUNCHED(1);
        total = std::max(total, mx);
        notConv += nconv;
    }
    MPF_CUDA(cudaStreamSynchronize(s));
    if (iterations) *iterations = total;
    return notConv ? fail(MPF_ENOCONV, "sparse solve: the iteration cap was reached") : MPF_OK;
}

}  // namespace mpf
