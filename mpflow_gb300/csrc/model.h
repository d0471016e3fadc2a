// Device-resident EIT model and the launch interfaces of its kernels.
//
// Data layout in HBM (one mesh, `frames` conductivity frames per call):
//   cols      [W][npad]            int32  slot-major ELL columns, W = density
//   SR        [F][W][npad]         float2 {stiffness, mass} slot values of each frame
//   S64, R64  [F][W][npad]         double same in FP64 (refinement residual only)
//   X         [F][Ca][npad][KP]    float  fields: node-major, the KP right-hand
//                                         sides of a node are contiguous, so one
//                                         ELL gather moves KP*4 contiguous bytes
//   J         [F][rowsJ][Epad]     float  Jacobian, element index contiguous
//   Jhi, Jlo  [F][rowsJ][Epad]     bf16   split of J for the tensor-core Gram
// A "group" g = f*Ca + ci is one (frame, active harmonic) pair; all KP
// right-hand sides of a group share one matrix S + alpha_c R.
//
// A batch of uneven meshes (batch.cu) stacks the meshes' row ranges in one
// set of arrays: each mesh owns 128-row tiles [tile0, tile0 + tiles) of
// `cols`, `SR` and every vector slice, and group g = slice * M + mesh, with
// slice = f * Ca + ci as above.  Columns are global rows, so an SpMM never
// leaves its mesh's block of the block-diagonal matrix, and every group has
// its own scalars, masks and block reductions.
#pragma once

#include <cuda_bf16.h>

#include <array>
#include <map>
#include <string>
#include <vector>

#include "mpf_internal.h"

namespace mpf {

// Per-launch view of a batched CG problem.
struct CgProblem {
    // n: real rows, npad: rows of a vector slice, nblk: 128-row tiles of the
    // largest mesh (the grid's x extent); for one mesh nblk = npad / kRowTile
    int n, npad, W, KP, G, Ca, nblk;
    // stacked meshes: M meshes per slice, seg[mesh] = {first tile, tiles,
    // end row (first row + real rows), c' of the Neumann term as float bits};
    // seg == nullptr for a single mesh (M = 1, tiles [0, nblk), rows < n)
    int M;
    const int4* seg;
    const int32_t* cols;
    const int32_t* diagSlot;
    const float2* SR;    // [F][W][npad] slot values {S, R}; columns in `cols`
    const float* alpha;  // [Ca] per active harmonic
    // vectors [G][npad][KP]
    float *x, *r, *p, *q;
    const float* b;      // right-hand side: [Ca][npad][KP] per harmonic, or [G][npad][KP]
    int bPerGroup;
    const int* dcFree;   // [Ca] 1 if the harmonic's matrix is singular (c == 0, open sources)
    // reduction state
    double* partA;       // [G][nblk][KP]
    double* partB;
    double* partC;
    double* sumP;        // [G][KP] sum(p) of Neumann groups (the 1 1^T term)
    const double* sumX0; // [G][KP] sum(x0) for a warm start, or null
    float dcScale;       // c' of the rank-one term c' 1 1^T (see model.cu); per mesh in seg
    double* rz;          // [G][KP]
    double* pq;
    double* bz;
    double* beta;
    int* conv;           // [G][KP]
    int* active;         // [G]
    int* iters;          // [G]
    unsigned* counter;   // [G] last-block-done counters (kept at zero between launches)
    double tol2;
    // launch shape of the three iteration kernels {spmm, update, direction},
    // chosen by the autotuner: variant (floats per lane x row steps in
    // flight) and 128-row tiles per block
    int variant[3];
    int tiles[3];
    // two-level preconditioner M^-1 = D^-1 + P (P^T A P)^-1 P^T over aggregates
    // of kAgg consecutive rows (coarse == 0: Jacobi only)
    int coarse;
    int nc, ncPad;        // aggregates (per mesh: from its segment), padded to a multiple of 64
    float* rc;            // [G][ncPad][KP] P^T r (restriction, written by k_update / k_init)
    float* rcB;           // [G][ncPad][KP] P^T b (k_init, for b^T M^-1 b)
    float* yc;            // [G][ncPad][KP] (P^T A P)^-1 P^T r
    const float* Binv;    // [G][ncPad][ncPad] (P^T A P)^-1, row-major, FP32
    double* rzFine;       // [G][KP] r^T D^-1 r of the last update / init
    double* bzFine;       // [G][KP] b^T D^-1 b (init)
    int first;            // k_direction: p = M^-1 r (start of an iteration)
    // halo plan of the tile-staged SpMM (k_spmm_halo; see HaloPlan): null
    // when the problem has none, and then that SpMM form is not offered
    const int32_t* halo;   // [tiles][Hpad] distinct columns outside each 128-row tile
    const int32_t* hcnt;   // [tiles] halo rows of each tile
    const uint16_t* lcol;  // [tiles][W][128] tile-local column of every slot
    int Hpad;              // halo rows reserved per tile (multiple of 8)
    int* abortFlag;        // device flag raised by a timed-out wait of a bulk-copy pipeline
    // deferred x update: k_update records alphaX = rz / pq of every
    // right-hand side and pend[g] = 1; k_direction applies x += alphaX p
    // while it still holds the old p and clears pend[g]; groups that retired
    // in k_update (k_direction skips them) get it from cg_launch_finalize
    double* alphaX;       // [G][KP]
    int* pend;            // [G]
    // solver 1: BiCGSTAB (bicgstab_kernels.cu).  Reuses x, r; p holds
    // y = K^-1 p, q holds nu = A y; rz = rho, pq = alpha, beta, bz = |b|^2.
    int solver;
    float *rhat, *zv, *tv;  // shadow residual, z = K^-1 s, t = A z (vector layout)
    double* omega;          // [G][KP]
    double* rr2;            // [G][KP] |r|^2 of the last update
    // solver 2: complex BiCGSTAB (complex_kernels.cu).  Vectors hold KP
    // complex values per node (re, im interleaved); SRz holds the complex
    // slot values {S.re, S.im, R.re, R.im}; the *I arrays are the imaginary
    // parts of rho, alpha, beta, omega and sum(.) (real parts in rz, pq,
    // beta, omega, sumP)
    const float4* SRz;
    double *rzI, *pqI, *betaI, *omegaI, *sumPI;
};

constexpr int kAgg = 64;  // rows per coarse aggregate (divides kRowTile)

// Halo plan of the tile-staged SpMM, built once per matrix structure from the
// slot-major ELL columns: for every 128-row tile t, the distinct columns
// outside the tile in ascending order (halo[t * Hpad + i], i < hcnt[t]; -1
// in the unused places up to Hpad), and
// every slot's column as an index into the tile's staged rows (lcol[(t * W +
// k) * 128 + r]: c - 128 t inside the tile, 128 + i for halo row i).  A
// tile's own rows and its halo rows are what k_spmm_halo copies into shared
// memory; on the ring meshes the halo holds 48-87 rows per tile.
struct HaloPlan {
    int Hpad = 0;
    std::vector<int32_t> halo, hcnt;
    std::vector<uint16_t> lcol;
};
void halo_plan(const std::vector<int32_t>& cols, int W, int npad, HaloPlan& out);
// the pipeline abort flag of the current device (dense_kernels.cu)
int* abort_flag_device();
// mlp_kernels.cu: split-BF16 operands and the tensor-core GEMM with an
// alpha / beta epilogue (used by the learned prior)
int split3_bf16(int rows, int rowsPad, int K, int Kp, const float* src, size_t srcRow, size_t srcCol, int order,
                __nv_bfloat16* dst, cudaStream_t s);
int tc_gemm_axpby(const __nv_bfloat16* A, int M, int lda, const __nv_bfloat16* B, int N, int ldb, int K,
                  float* out, int ldo, int rowsValid, int colsValid, float alpha, float beta, float add, int* flag,
                  cudaStream_t s);

// cg_kernels.cu
// variant v = vecIdx * 3 + rbIdx, floats per lane {4, 2, 1}[vecIdx], row steps {1, 2, 4}[rbIdx]
// (SpMM: v + 9 * form with form 0 = slots read from global memory, 1 = slots
// staged per warp with cp.async, 2 / 3 = tile-staged with 2 / 3 bulk-copy
// stages, k_spmm_halo); a launch-shape code is v % 9 + kCgVariants * ti +
// 36 * (v / 9) with 1 << ti tiles per block (4 << ti for the tile-staged SpMM)
constexpr int kCgVariants = 9;
constexpr int kCgTileChoices = 4;
constexpr int kSpmmForms = 4;
bool cg_variant_valid(int KP, int which, int v);
int cg_shape_count(int which);                      // 144 SpMM codes, 36 for the others
bool cg_shape_valid(int KP, int which, int code);
int cg_spmm_form(int code);
// cg_shape_valid and, for the tile-staged SpMM, a halo plan whose stages fit shared memory
bool cg_shape_fits(int KP, int W, int Hpad, bool haveHalo, int which, int code);
int cg_shape_code(const CgProblem& P, int which);
int cg_default_variant(int KP);
int cg_launch_init(const CgProblem& P, bool zeroGuess, cudaStream_t s);
// coarse_kernels.cu
struct CoarsePlan {
    int nc, ncPad, nnz;              // aggregates, padded count, nonzero (I, J) pairs
    const int32_t* pairI;            // [nnz]
    const int32_t* pairJ;            // [nnz]
    const int32_t* pairPtr;          // [nnz + 1] into slots
    const int32_t* slots;            // slot indices k * npad + row
    const float* aggSize;            // [nc] real rows per aggregate ([M][ncPad] for stacked meshes)
    // stacked meshes (P.seg != nullptr): the pairs of mesh j are
    // [meshPairPtr[j], meshPairPtr[j + 1]), its aggregate count meshNc[j]
    const int32_t* meshPairPtr;
    const int32_t* meshNc;
};
// Lc [G][ncPad][ncPad], LinvD [G][ncPad/32][1024]: FP32 factor scratch; Binv: the inverse (P.Binv);
// L64 [G][ncPad][ncPad]: the factor taken in FP32 arithmetic (FP64 factor in
// place of Ac64 where it breaks down; null: FP64 only); info: 2 * G ints;
// groupMask (device, [G], optional): only these groups are set up (the
// others keep their coarse space, e.g. frames left out of a solve)
int coarse_launch_setup(const CgProblem& P, const CoarsePlan& cp, double* Ac64, int* info, cudaStream_t s,
                        float* Lc, float* LinvD, float* Binv, double* L64, const int* groupMask = nullptr);
// `count`: false while recording a CUDA graph (replays are counted by the caller)
int cg_launch_coarse(const CgProblem& P, bool init, cudaStream_t s, bool count = true);
bool coarse_supported(int KP, int ncPad);
int cg_launch_iteration(const CgProblem& P, cudaStream_t s);
// kernel attributes of P's launch shapes (large dynamic shared memory), set
// before an iteration graph is recorded
int cg_prepare_launch(const CgProblem& P);
int cg_iteration_launches(const CgProblem& P);
int cg_launch_kernel(const CgProblem& P, int which /*0 spmm, 1 update, 2 direction*/, cudaStream_t s);
// x += alphaX p on the groups whose last x update is still pending (end of a CG solve)
int cg_launch_finalize(const CgProblem& P, cudaStream_t s);
int cg_launch_skip(const CgProblem& P, const int* frameSkip /*[frames] device*/, cudaStream_t s);
int cg_launch_group_mask(const CgProblem& P, const int* frameSkip, int* groupMask /*[G] device*/, cudaStream_t s);

// cg_driver.cpp: host drivers shared by single models and batches of meshes.
// Captured CUDA graphs of CG iteration chunks, keyed by the problems' bytes.
using CgGraphCache = std::map<std::string, cudaGraphExec_t>;
void cg_graphs_clear(CgGraphCache& cache);
// launch-shape code -> kernel variant and tiles per block
void cg_set_shape(CgProblem& P, int which, int code);
// Autotuner: times every valid launch shape of the three iteration kernels on
// P's own systems with CUDA events and returns the fastest shape code of each.
// It overwrites P's iteration vectors (run it before a cold solve only).
int cg_autotune(const CgProblem& P, std::array<int, 3>& best, cudaStream_t s);
// Runs CG iterations of nP problems, recorded together as CUDA graphs of
// checkEvery iterations, until every group of every problem converged or
// maxIter; pinned: host buffer of at least sum(G) + 1 ints.  iters receives the
// per-group iteration counts (problems in order), maxIters the slowest group's
// count and notConverged the groups still active.
int cg_run(CgGraphCache& cache, int* pinned, const CgProblem* Ps, int nP, int maxIter, int checkEvery,
           cudaStream_t s, std::vector<int>& iters, int* maxIters, int* notConverged);
int cg_launch_residual64(const CgProblem& P, const double* S64, const double* R64, const double* x64,
                         const double* b64, const double* sumX64, double* partR, double* partB, double* rr,
                         double* bb, cudaStream_t s);
int cg_launch_colsum(const CgProblem& P, const float* x, const double* x64, double* sums, cudaStream_t s);
int cg_launch_dc_shift(const CgProblem& P, const double* shift, float sign, cudaStream_t s);
int cg_launch_accumulate64(const CgProblem& P, double* x64, cudaStream_t s);
int cg_launch_to_float(const CgProblem& P, const double* x64, cudaStream_t s);
// bicgstab_kernels.cu (cg_launch_init / cg_launch_iteration dispatch here for solver 1)
int bicgstab_launch_init(const CgProblem& P, bool zeroGuess, cudaStream_t s);
int bicgstab_launch_iteration(const CgProblem& P, cudaStream_t s);
constexpr int kBicgstabLaunches = 5;
// complex_kernels.cu: complex admittivity (solver 2)
int zbicgstab_launch_init(const CgProblem& P, cudaStream_t s);
int zbicgstab_launch_iteration(const CgProblem& P, cudaStream_t s);
int fem_launch_zassemble(int F, int W, int npad, int E, const int32_t* cptr, const int32_t* contrib, const float* Kf,
                         const float* Mf, const float* gamma2, float ref, int logarithmic, float4* SRz, cudaStream_t s);
int cg_launch_zdc_shift(const CgProblem& P, const double* shift, float sign, cudaStream_t s);
int fem_launch_zfields_export(int F, int Ca, int C, const int32_t* compOf, int npad, int KP, int dataRows, int cols,
                              int n, const int32_t* colU, const float* colScale, const float* betaC, const float* Xz,
                              const int32_t* rowOf, float* out, cudaStream_t s);
int fem_launch_zgram_meas(int G, int KP, int npad, const int32_t* nzPtr, const int32_t* nzNode, const double* nzVal,
                          const float* Xz, double* Gmz, cudaStream_t s);
int fem_launch_zvoltages(int F, int Ca, int KP, int Mm, int Md, const double* Gmz, const float* beta,
                         const int32_t* measU, const float* measScale, const int32_t* driveU, const float* driveScale,
                         float* Vz, cudaStream_t s);

// fem_kernels.cu
int fem_launch_assemble(int F, int W, int npad, int E, const int32_t* cptr, const int32_t* contrib,
                        const float* Kf, const float* Mf, const double* Kd, const double* Md,
                        const float* gamma, float ref, int logarithmic, float2* SR, double* S64, double* R64,
                        cudaStream_t s, size_t ld = 0, size_t frameStride = 0);
// (SR of a stacked mesh: pass SR at the mesh's first row, ld = the batch's
// rows per slot, frameStride = its slots per frame; 0 = this mesh's own)
int fem_launch_export_ell(int F, int W, int npad, int n, int dataRows, const float2* SR, int component,
                          const int32_t* rowOf, float* refLayout, cudaStream_t s);
struct MeasPlan {
    int nnz;                 // nonzeros of the unique excitation columns
    const int32_t* nzNode;   // [nnz]
    const int32_t* nzCol;    // [nnz]
    const double* nzVal;     // [nnz]
    const int32_t* nzPtr;    // [KP+1] CSR by column
};
int fem_launch_gram_meas(int G, int KP, int npad, const MeasPlan& mp, const float* X, double* Gm,
                         cudaStream_t s);
int fem_launch_voltages(int F, int Ca, int KP, int Mm, int Md, const double* Gm, const float* beta,
                        const int32_t* measU, const float* measScale, const int32_t* driveU,
                        const float* driveScale, float* V, cudaStream_t s);
struct JacPlan {
    int rowsJ, Epad, E, KP, Ca;
    const int32_t* rowD;     // [rowsJ] unique column of the drive field, -1 for padding
    const int32_t* rowM;     // [rowsJ] unique column of the measurement field
    const float* rowScale;   // [rowsJ] drive scale * measurement scale
    const float* beta2;      // [Ca] harmonic weight: beta_c^2 (reference) or beta_c / h (exact)
    const float* massCoef;   // [Ca] alpha_c in exact mode, 0 in reference mode
    const int32_t* elements; // [E][3]
    const float* Kf;         // [E][9]
    const float* Mf;         // [E][9] (read only in exact mode)
    int exact;
    float ref, height;       // J *= -height (open sources)
    int logarithmic;
    const int* frameMask;    // [F] frames to compute, or null for all
    int writeF32;            // 0: only the BF16 hi/lo split (the Gauss-Newton path)
    // 1: drive row d uses field column d and measurement row m column m (for
    // every real row), so the kernel reads the staged field rows directly
    int identity;
    // > 0: every real row has this scale (rowScale is not read; with identity
    // maps the padding rows come out zero on their own)
    float uniformScale;
};
int fem_launch_jacobian(int F, const JacPlan& jp, int MP, int npad, const float* X, const float* gamma,
                        float* J, __nv_bfloat16* Jhi, __nv_bfloat16* Jlo, cudaStream_t s);
// complex_kernels.cu: Jacobian of the complex-admittivity model
int fem_launch_zjacobian(int F, const JacPlan& jp, int MP, int npad, const float* Xz, const float* gamma2, float* Jz,
                         cudaStream_t s);
int fem_launch_ztranspose_jacobian(int F, int rowsJ, int Epad, int E, const float* Jz, float* Jref, cudaStream_t s);
int fem_launch_transpose_jacobian(int F, int rowsJ, int Epad, int E, const float* J, float* Jref,
                                  cudaStream_t s);
int fem_launch_fields_export(int F, int Ca, int C, const int32_t* compOf, int npad, int KP,
                             int dataRows, int cols, int n, const int32_t* colU, const float* colScale,
                             const float* betaC, const float* X, const int32_t* rowOf, float* out,
                             cudaStream_t s);
int fem_launch_residual(int F, int rowsJ, int Mm, int Md, const float* vMeas, const float* V,
                        double* y, double* res, cudaStream_t s);
int fem_launch_fill_frames(int F, int E, const int* frameMask, float value, float* gamma, cudaStream_t s);
// bad[f] = active frame f has a non-finite or out-of-range parameter
int fem_launch_gamma_check(int F, int E, const float* gamma, const int* frameActive, bool logarithmic, int* bad,
                           cudaStream_t s);
// linear prior of the learned start: unit right-hand sides B[i] = e_{row(i)}
// (rowsJ x Mm*Md, FP64) for the Jacobian rows of the measurements, and
// Q = scale * B in FP32
int fem_launch_prior_rhs(int rowsJ, int Mm, int Md, double* B, cudaStream_t s);
int fem_launch_prior_convert(int rowsJ, int L, const double* B, double scale, float* Q, cudaStream_t s);
int fem_launch_learned_input(int F, int L, const float* vMeas, const float* V0, float invRms, float* x,
                             double* res0, cudaStream_t s);
// gamma += J^T w with J = hi + lo (the BF16 split the Gram is formed from)
int fem_launch_update_gamma(int F, int rowsJ, int Epad, int E, const __nv_bfloat16* Jhi, const __nv_bfloat16* Jlo,
                            const double* w, const int* frameActive, float* gamma, cudaStream_t s);

// dense_kernels.cu
int dense_gram_split_bf16(int batch, int rows, int cols, const __nv_bfloat16* hi, const __nv_bfloat16* lo,
                          int ld, float* C, float* work, size_t workFloats, cudaStream_t s);
size_t dense_gram_work_floats(int batch, int rows, int cols);
int dense_split_bf16(int batch, int rows, int cols, const float* A, int lda, __nv_bfloat16* hi,
                     __nv_bfloat16* lo, cudaStream_t s);
int dense_gram_f64_shift(int batch, int rows, int cols, const __nv_bfloat16* hi, const __nv_bfloat16* lo,
                         int ld, double shift, double* A64, float* work, size_t workFloats, cudaStream_t s,
                         const int* frameMask = nullptr);
int dense_gram_check_abort(bool* aborted);
int dense_profile_gram(int batch, int rows, int cols, int reps, double* msPerLaunch, cudaStream_t s);
// A64 = J J^T + shift I in FP64 from FP32 J (rows % 64 == 0, cols % 32 == 0)
int dense_gram_f64_exact(int batch, int rows, int cols, const float* J, int ld, double shift, double* A64,
                         const int* frameMask, cudaStream_t s);
int dense_gram_split_bf16_noalloc(int batch, int rows, int cols, const float* A, int lda, float* C, cudaStream_t s);
int dense_add_shift(int batch, int n, double* A, double shift, cudaStream_t s);
// frameMask: [batch] entries to process (null: all); skipped entries keep their contents
int dense_cholesky_f64(int batch, int n, double* A, int* info, cudaStream_t s, const int* frameMask = nullptr);
int dense_cholesky_solve_f64(int batch, int n, const double* L, double* B, int nrhs, cudaStream_t s,
                             const int* frameMask = nullptr);
// Cholesky in FP32 arithmetic of FP64 column-major matrices (n % 32 == 0,
// n <= 1536), a cluster of up to 4 CTAs per matrix; L may equal A (in
// place); the factor is stored in FP64; info[b] = first non-positive pivot
// (1-based) or 0
int dense_potrf32(int batch, int n, const double* A, double* L, int* info, cudaStream_t s,
                  const int* frameMask = nullptr);
// upper triangle := mirror of the lower one (the part the factors read)
int dense_mirror_lower(int batch, int n, double* A, cudaStream_t s, const int* frameMask = nullptr);
// r = y - A x (FP64, A full symmetric) with per-block partial |r|^2, |y|^2
// (n / 128 per frame, in rr / yy)
int dense_sym_residual(int batch, int n, const double* A, const double* x, const double* y, double* r, double* rr,
                       double* yy, cudaStream_t s, const int* frameMask = nullptr);
// x += d on the masked frames ([batch][n])
int dense_add_masked(int batch, int n, double* x, const double* d, cudaStream_t s, const int* frameMask = nullptr);
// X = L^-1 and XT = X^T in FP32 from the FP32 factor L (FP64 storage,
// column-major lower); L32 receives L in FP32, D the inverted 32 x 32
// diagonal blocks (batch x n / 32 x 1024); n <= 1280
int dense_trtri32(int batch, int n, const double* L, float* L32, float* D, float* X, float* XT, cudaStream_t s,
                  const int* frameMask = nullptr);
// out = tril(M) v (upper = false) or triu(M) v (upper = true), M FP32 n x n
// row-major per frame, v and out FP64
int dense_tri_rows(int batch, int n, const float* M, const double* v, double* out, bool upper, cudaStream_t s,
                   const int* frameMask = nullptr);

// matrix_ops.cu: C = alpha op(A) op(B) + beta C, column-major FP32
int matrix_multiply_scaled(int transA, int transB, int m, int n, int k, float alpha, const float* A, int lda,
                           const float* B, int ldb, float beta, float* C, int ldc, cudaStream_t s);
int convert_values(int direction, long long count, const void* src, void* dst, cudaStream_t s);
int matrix_elementwise(int op, int rows, int cols, const float* A, const float* B, float* C, int ld, float scalar,
                       cudaStream_t s);

// mlp_kernels.cu (used by the learned warm start)
void mlp_dims(const mpf_mlp* n, int* in, int* out);
int mlp_forward(mpf_mlp* n, int batch, const float* x, float* y, int ldy, cudaStream_t s);

}  // namespace mpf
