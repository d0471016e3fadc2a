// Two-level preconditioner of the batched CG:
//   M^-1 = D^-1 + P (P^T A P)^-1 P^T
// with P the piecewise-constant prolongation from aggregates of kAgg = 64
// consecutive rows.  The rows are in Morton order (model.cu), so an
// aggregate is a compact patch of the mesh and the coarse space carries the
// smooth error that Jacobi-preconditioned CG reduces slowest.  No reference
// counterpart: the reference preconditions with the diagonal only
// (src/numeric/preconditioner.cpp:59-76); the solutions are the same, the
// iteration counts are not.
//
// Setup, once per assembled matrix (k_coarse_assemble / k_coarse_fixup, the
// batched FP64 Cholesky of dense_kernels.cu, k_coarse_prep): the coarse
// matrix of every (frame, harmonic) group in FP64, its Cholesky factor, and
// an FP32 copy of the factor with inverted 32x32 diagonal blocks.
// The setup ends with the explicit inverse (P^T A P)^-1 in FP32
// (k_coarse_inverse: blocked triangular solves on identity columns), so the
// per-iteration kernel k_coarse is a dense register-tiled product
// y = (P^T A P)^-1 P^T r with no sequential dependence; it also adds
// (P^T r).y to r^T D^-1 r and updates the CG scalars and convergence masks
// of every group.
#include <algorithm>
#include <atomic>

#include <vector>

#include "model.h"

namespace mpf {
namespace {

constexpr int kCT = 256;  // threads of k_coarse

// A_c[g][I][J] = sum over the slots of rows in aggregate I whose column lies
// in aggregate J of (S + alpha R), FP64, fixed order.
// Zero the coarse matrices of the groups in groupMask.
__global__ void k_zero_groups(size_t per, double* __restrict__ Ac, const int* __restrict__ groupMask) {
    const int g = blockIdx.y;
    if (!groupMask[g]) return;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < per; t += (size_t)gridDim.x * blockDim.x)
        Ac[(size_t)g * per + t] = 0.0;
}

__global__ void k_coarse_assemble(CgProblem P, CoarsePlan cp, double* __restrict__ Ac, const int* __restrict__ groupMask) {
    const int g = blockIdx.y;
    if (groupMask && !groupMask[g]) return;
    const int slice = g / P.M, mesh = g - slice * P.M;
    const int f = slice / P.Ca, ci = slice % P.Ca;
    const double alpha = (double)P.alpha[ci];
    const float2* SR = P.SR + (size_t)f * P.W * P.npad;
    double* A = Ac + (size_t)g * cp.ncPad * cp.ncPad;
    const int t0 = cp.meshPairPtr ? cp.meshPairPtr[mesh] : 0;
    const int t1 = cp.meshPairPtr ? cp.meshPairPtr[mesh + 1] : cp.nnz;
    for (int t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = cp.pairPtr[t]; k < cp.pairPtr[t + 1]; ++k) {
            const float2 e = __ldg(&SR[cp.slots[k]]);
            s += (double)e.x + alpha * (double)e.y;
        }
        A[(size_t)cp.pairI[t] * cp.ncPad + cp.pairJ[t]] = s;
    }
}

// Neumann groups: + c' |I| |J| (the coarse image of c' 1 1^T); padding
// aggregates get an identity block.
__global__ void k_coarse_fixup(CgProblem P, CoarsePlan cp, double* __restrict__ Ac, const int* __restrict__ groupMask) {
    const int g = blockIdx.y;
    if (groupMask && !groupMask[g]) return;
    const int slice = g / P.M, mesh = g - slice * P.M;
    const bool dc = P.dcFree[slice % P.Ca] != 0;
    const int nc = cp.meshNc ? cp.meshNc[mesh] : cp.nc;
    const float* aggSize = cp.meshNc ? cp.aggSize + (size_t)mesh * cp.ncPad : cp.aggSize;
    const double dcScale = P.seg ? (double)__int_as_float(P.seg[mesh].w) : (double)P.dcScale;
    double* A = Ac + (size_t)g * cp.ncPad * cp.ncPad;
    const size_t total = (size_t)cp.ncPad * cp.ncPad;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int I = (int)(t / cp.ncPad), J = (int)(t % cp.ncPad);
        if (I < nc && J < nc) {
            if (dc) A[t] += dcScale * (double)aggSize[I] * (double)aggSize[J];
        } else if (I == J) {
            A[t] = 1.0;
        }
    }
}

// FP64 Cholesky factor (column-major lower) -> FP32 row-major lower factor
// and the inverses of its 32x32 diagonal blocks.  One warp per (block row,
// group); lane c inverts column c by forward substitution.
__global__ void __launch_bounds__(32) k_coarse_prep(int ncPad, const double* __restrict__ L64,
                                                    float* __restrict__ Lc, float* __restrict__ LinvD,
                                                    const int* __restrict__ groupMask) {
    const int bi = blockIdx.x, g = blockIdx.y, lane = threadIdx.x;
    if (groupMask && !groupMask[g]) return;
    const double* L = L64 + (size_t)g * ncPad * ncPad;
    float* Lf = Lc + (size_t)g * ncPad * ncPad;
    for (int r = 0; r < 32; ++r) {
        const int row = bi * 32 + r;
        for (int c = lane; c < ncPad; c += 32) Lf[(size_t)row * ncPad + c] = c <= row ? (float)L[row + (size_t)c * ncPad] : 0.f;
    }
    __shared__ double B[32][33];
    for (int r = 0; r < 32; ++r) B[r][lane] = lane <= r ? L[(bi * 32 + r) + (size_t)(bi * 32 + lane) * ncPad] : 0.0;
    __syncwarp();
    double x[32];
    for (int r = 0; r < 32; ++r) {
        double s = r == lane ? 1.0 : 0.0;
        for (int k = lane; k < r; ++k) s -= B[r][k] * x[k];
        x[r] = r < lane ? 0.0 : s / B[r][r];
    }
    float* D = LinvD + ((size_t)g * (ncPad / 32) + bi) * 1024;
    for (int r = 0; r < 32; ++r) D[r * 32 + lane] = (float)x[r];
}

// (L L^T) y = rhs in shared memory: y holds rhs on entry (row stride KP + 1),
// the solution on exit.  Thread (r, c0) owns row r of the current 32-row
// block and the right-hand sides c0, c0 + 8, ...
template <int KP>
__device__ void coarse_solve(const float* __restrict__ L, const float* __restrict__ Dv, int ncPad, float* y,
                             float* tmp, float (*Ls)[33]) {
    constexpr int YS = KP + 1, CPT = KP / 8;
    const int r = threadIdx.x & 31, c0 = threadIdx.x >> 5;
    const int nb = ncPad / 32;
    // forward: L z = rhs
    for (int bi = 0; bi < nb; ++bi) {
        float acc[CPT];
#pragma unroll
        for (int q = 0; q < CPT; ++q) acc[q] = 0.f;
        for (int bj = 0; bj < bi; ++bj) {
            for (int t = threadIdx.x; t < 1024; t += kCT)
                Ls[t >> 5][t & 31] = __ldg(&L[(size_t)(bi * 32 + (t >> 5)) * ncPad + bj * 32 + (t & 31)]);
            __syncthreads();
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
                const float l = Ls[r][k];
                const float* yk = y + (bj * 32 + k) * YS + c0;
#pragma unroll
                for (int q = 0; q < CPT; ++q) acc[q] = fmaf(l, yk[8 * q], acc[q]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int q = 0; q < CPT; ++q) tmp[r * YS + c0 + 8 * q] = y[(bi * 32 + r) * YS + c0 + 8 * q] - acc[q];
        for (int t = threadIdx.x; t < 1024; t += kCT) Ls[t >> 5][t & 31] = __ldg(&Dv[bi * 1024 + t]);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
            float s = 0.f;
            for (int k = 0; k <= r; ++k) s = fmaf(Ls[r][k], tmp[k * YS + c0 + 8 * q], s);
            y[(bi * 32 + r) * YS + c0 + 8 * q] = s;
        }
        __syncthreads();
    }
    // backward: L^T x = z
    for (int bi = nb - 1; bi >= 0; --bi) {
        float acc[CPT];
#pragma unroll
        for (int q = 0; q < CPT; ++q) acc[q] = 0.f;
        for (int bj = bi + 1; bj < nb; ++bj) {
            for (int t = threadIdx.x; t < 1024; t += kCT)
                Ls[t >> 5][t & 31] = __ldg(&L[(size_t)(bj * 32 + (t >> 5)) * ncPad + bi * 32 + (t & 31)]);
            __syncthreads();
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
                const float l = Ls[k][r];
                const float* yk = y + (bj * 32 + k) * YS + c0;
#pragma unroll
                for (int q = 0; q < CPT; ++q) acc[q] = fmaf(l, yk[8 * q], acc[q]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int q = 0; q < CPT; ++q) tmp[r * YS + c0 + 8 * q] = y[(bi * 32 + r) * YS + c0 + 8 * q] - acc[q];
        for (int t = threadIdx.x; t < 1024; t += kCT) Ls[t >> 5][t & 31] = __ldg(&Dv[bi * 1024 + t]);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
            float s = 0.f;
            for (int k = r; k < 32; ++k) s = fmaf(Ls[k][r], tmp[k * YS + c0 + 8 * q], s);
            y[(bi * 32 + r) * YS + c0 + 8 * q] = s;
        }
        __syncthreads();
    }
}

// Setup: columns [32 * blockIdx.x, +32) of (P^T A P)^-1 by triangular solves
// on identity columns; Binv is row-major and symmetric up to rounding.
__global__ void __launch_bounds__(kCT) k_coarse_inverse(int ncPad, const float* __restrict__ Lc,
                                                        const float* __restrict__ LinvD, float* __restrict__ Binv,
                                                        const int* __restrict__ groupMask) {
    constexpr int YS = 33;
    extern __shared__ float smc[];
    float* y = smc;
    float* tmp = y + (size_t)ncPad * YS;
    float(*Ls)[33] = reinterpret_cast<float(*)[33]>(tmp + 32 * YS);
    const int g = blockIdx.y, col0 = blockIdx.x * 32;
    if (groupMask && !groupMask[g]) return;
    for (int t = threadIdx.x; t < ncPad * 32; t += kCT) y[(t / 32) * YS + t % 32] = (t / 32 == col0 + t % 32) ? 1.f : 0.f;
    __syncthreads();
    coarse_solve<32>(Lc + (size_t)g * ncPad * ncPad, LinvD + (size_t)g * (ncPad / 32) * 1024, ncPad, y, tmp, Ls);
    float* B = Binv + (size_t)g * ncPad * ncPad;
    for (int t = threadIdx.x; t < ncPad * 32; t += kCT) B[(size_t)(t / 32) * ncPad + col0 + t % 32] = y[(t / 32) * YS + t % 32];
}

// Per iteration: y = Binv (P^T r), register-tiled.  A CTA owns 64 rows of
// one group (grid = ncPad / 64 x groups) and 32 right-hand sides at a time;
// its 128 threads each hold 4 rows x 4 columns.  Binv rows stream through
// shared memory in 32-wide k chunks (double-buffered with cp.async), P^T r
// sits in shared memory whole.  The CTA writes y for the direction kernel
// and its partial (P^T r).y; the last CTA of the group adds the partials in
// a fixed order to r^T D^-1 r and updates the CG scalars and convergence
// masks.  In the start-of-solve mode it also solves for P^T b to complete
// b^T M^-1 b.
constexpr int kCoarseRows = 64;    // rows per CTA
constexpr int kCoarseThreads = 128;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int KP>
__global__ void __launch_bounds__(kCoarseThreads) k_coarse(CgProblem P, int init) {
    constexpr int NCH = KP < 32 ? 1 : KP / 32;  // 32-column chunks
    constexpr int BS = 36;                      // Binv chunk row stride (floats, 16-byte multiple)
    const int g = blockIdx.y, r0 = blockIdx.x * kCoarseRows;
    if (!init && !P.active[g]) return;
    const int ncPad = P.ncPad;
    extern __shared__ __align__(16) float smc[];
    float* Rs = smc;                              // [ncPad][KP]
    float* Bs = smc + (size_t)ncPad * KP;         // [2][64][BS]
    __shared__ double red[16][33];
    __shared__ bool amLast;
    const float* B = P.Binv + ((size_t)g * ncPad + r0) * ncPad;
    const size_t cb = (size_t)g * ncPad * KP;
    const int rl = threadIdx.x & 15, cgp = threadIdx.x >> 4;  // rows rl + 16 i, columns 4 cgp + j
    double* part = P.partC + ((size_t)g * gridDim.x + blockIdx.x) * 2 * KP;
    auto load_chunk = [&](int buf, int k0) {
        // 64 rows x 32 floats = 512 16-byte pieces, 4 per thread
        for (int t = threadIdx.x; t < 512; t += kCoarseThreads) {
            const int row = t >> 3, piece = t & 7;
            cp_async16(Bs + ((size_t)buf * 64 + row) * BS + piece * 4, B + (size_t)row * ncPad + k0 + piece * 4);
        }
        cp_async_commit();
    };
    for (int sys = 0; sys < (init ? 2 : 1); ++sys) {
        const float* src = (sys == 0 ? P.rc : P.rcB) + cb;
        for (int t = threadIdx.x; t < ncPad * KP / 4; t += kCoarseThreads) cp_async16(Rs + 4 * t, src + 4 * t);
        cp_async_commit();
        for (int ch = 0; ch < NCH; ++ch) {
            const int col0 = ch * 32 + cgp * 4;
            float acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
            load_chunk(0, 0);
            const int nk = ncPad / 32;
            for (int kc = 0; kc < nk; ++kc) {
                if (kc + 1 < nk) {
                    load_chunk((kc + 1) & 1, (kc + 1) * 32);
                    cp_async_wait1();
                } else {
                    cp_async_wait0();
                }
                __syncthreads();
                const float* Bc = Bs + (size_t)(kc & 1) * 64 * BS;
                if (col0 < KP) {
#pragma unroll 8
                    for (int kk = 0; kk < 32; ++kk) {
                        const float4 rv = *reinterpret_cast<const float4*>(Rs + (size_t)(kc * 32 + kk) * KP + col0);
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const float bv = Bc[(rl + 16 * i) * BS + kk];
                            acc[i][0] = fmaf(bv, rv.x, acc[i][0]);
                            acc[i][1] = fmaf(bv, rv.y, acc[i][1]);
                            acc[i][2] = fmaf(bv, rv.z, acc[i][2]);
                            acc[i][3] = fmaf(bv, rv.w, acc[i][3]);
                        }
                    }
                }
                __syncthreads();
            }
            // y out and per-column partial dots over this CTA's rows
            double d[4] = {0.0, 0.0, 0.0, 0.0};
            if (col0 < KP) {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int row = r0 + rl + 16 * i;
                    const float4 rr = *reinterpret_cast<const float4*>(Rs + (size_t)row * KP + col0);
                    d[0] += (double)rr.x * acc[i][0];
                    d[1] += (double)rr.y * acc[i][1];
                    d[2] += (double)rr.z * acc[i][2];
                    d[3] += (double)rr.w * acc[i][3];
                    if (sys == 0)
                        *reinterpret_cast<float4*>(P.yc + cb + (size_t)row * KP + col0) =
                            make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) red[rl][cgp * 4 + j] = d[j];
            __syncthreads();
            if (threadIdx.x < 32 && ch * 32 + (int)threadIdx.x < KP) {
                double t = 0.0;
                for (int q = 0; q < 16; ++q) t += red[q][threadIdx.x];
                part[sys * KP + ch * 32 + threadIdx.x] = t;
            }
            __syncthreads();
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) amLast = atomicAdd(&P.counter[g], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    int notConv = 0;
    if (threadIdx.x < KP) {
        const size_t s = (size_t)g * KP + threadIdx.x;
        double c0 = 0.0, c1 = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) {
            const double* pb = P.partC + ((size_t)g * gridDim.x + b) * 2 * KP;
            c0 += __ldcg(pb + threadIdx.x);
            if (init) c1 += __ldcg(pb + KP + threadIdx.x);
        }
        if (init) {
            const double rz = P.rzFine[s] + c0, bz = P.bzFine[s] + c1;
            P.rz[s] = rz;
            P.bz[s] = bz;
            P.beta[s] = 0.0;
            const int c = rz <= P.tol2 * bz;
            P.conv[s] = c;
            notConv = !c;
        } else if (!P.conv[s]) {
            const double rzn = P.rzFine[s] + c0, rzo = P.rz[s];
            P.beta[s] = rzo != 0.0 ? rzn / rzo : 0.0;
            P.rz[s] = rzn;
            const int c = rzn <= P.tol2 * P.bz[s];
            P.conv[s] = c;
            notConv = !c;
        }
    }
    const int any = __syncthreads_or(notConv);
    if (threadIdx.x == 0) {
        P.active[g] = any;
        if (!init) P.iters[g] += 1;
        P.counter[g] = 0;
    }
}

size_t coarse_apply_smem(int ncPad, int KP) { return ((size_t)ncPad * KP + 2 * 64 * 36) * sizeof(float); }

size_t coarse_solve_smem(int ncPad) { return ((size_t)(ncPad + 32) * 33 + 32 * 33) * sizeof(float); }

template <int KP>
int launch_coarse_kp(const CgProblem& P, bool init, cudaStream_t s, bool count) {
    const size_t smem = coarse_apply_smem(P.ncPad, KP);
    // the attribute is per device: remember the size set on each
    static std::atomic<size_t> configured[64];
    int dev = 0;
    MPF_CUDA(cudaGetDevice(&dev));
    MPF_CHECK(dev >= 0 && dev < 64, MPF_EINVAL, "coarse correction: device ordinal %d out of range", dev);
    if (smem > configured[dev].load()) {
        MPF_CUDA(cudaFuncSetAttribute(k_coarse<KP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured[dev].store(smem);
    }
    k_coarse<KP><<<dim3(P.ncPad / kCoarseRows, P.G), kCoarseThreads, smem, s>>>(P, init ? 1 : 0);
    if (count) {
        MPF_LAUNCHED(1);
    } else {
        MPF_CUDA(cudaGetLastError());
    }
    return MPF_OK;
}

}  // namespace

bool coarse_supported(int KP, int ncPad) {
    return (KP == 16 || KP == 32 || KP == 64) && ncPad >= kCoarseRows && ncPad % kCoarseRows == 0 &&
           ncPad <= 1024 && coarse_apply_smem(ncPad, KP) <= 200 * 1024 && coarse_solve_smem(ncPad) <= 200 * 1024;
}

int cg_launch_coarse(const CgProblem& P, bool init, cudaStream_t s, bool count) {
    switch (P.KP) {
        case 16: return launch_coarse_kp<16>(P, init, s, count);
        case 32: return launch_coarse_kp<32>(P, init, s, count);
        case 64: return launch_coarse_kp<64>(P, init, s, count);
        default: return fail(MPF_EINVAL, "two-level preconditioner: unsupported right-hand-side width %d", P.KP);
    }
}

int coarse_launch_setup(const CgProblem& P, const CoarsePlan& cp, double* Ac64, int* info, cudaStream_t s,
                        float* Lc, float* LinvD, float* Binv, double* L64, const int* groupMask) {
    const size_t per = (size_t)cp.ncPad * cp.ncPad;
    if (!groupMask) {
        MPF_CUDA(cudaMemsetAsync(Ac64, 0, sizeof(double) * per * P.G, s));
    } else {
        k_zero_groups<<<dim3((int)std::min<size_t>((per + 255) / 256, 1024), P.G), 256, 0, s>>>(per, Ac64, groupMask);
        MPF_LAUNCHED(1);
    }
    k_coarse_assemble<<<dim3(std::min((cp.nnz + 255) / 256, 1024), P.G), 256, 0, s>>>(P, cp, Ac64, groupMask);
    k_coarse_fixup<<<dim3((int)std::min<size_t>((per + 255) / 256, 1024), P.G), 256, 0, s>>>(P, cp, Ac64,
                                                                                           groupMask);
    MPF_LAUNCHED(2);
    // The coarse operator is applied in FP32 (Binv), so its factor is taken
    // in FP32 arithmetic, one CTA per group, into L64; a group whose FP32
    // factor breaks down (a badly conditioned coarse matrix) is factored in
    // FP64 in place and its factor copied over.  A group whose coarse matrix
    // is not positive definite in FP64 either (a parameter far outside the
    // model's range) is left without the coarse correction: its Binv is zero,
    // so it iterates with Jacobi alone.
    const double* Lsrc = Ac64;
    std::vector<int> jacobiOnly;
    if (L64) {
        MPF_TRY(dense_potrf32(P.G, cp.ncPad, Ac64, L64, info, s, groupMask));
        std::vector<int> h(P.G), redo(P.G, 0);
        MPF_CUDA(cudaMemcpyAsync(h.data(), info, sizeof(int) * P.G, cudaMemcpyDeviceToHost, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        bool any = false;
        for (int g = 0; g < P.G; ++g) any |= (redo[g] = h[g] != 0) != 0;
        if (any) {
            int* mask = info + P.G;  // info has 2 * G entries: pivots, then this mask
            MPF_CUDA(cudaMemcpyAsync(mask, redo.data(), sizeof(int) * P.G, cudaMemcpyHostToDevice, s));
            MPF_TRY(dense_cholesky_f64(P.G, cp.ncPad, Ac64, info, s, mask));
            for (int g = 0; g < P.G; ++g)
                if (redo[g])
                    MPF_CUDA(cudaMemcpyAsync(L64 + per * g, Ac64 + per * g, sizeof(double) * per,
                                             cudaMemcpyDeviceToDevice, s));
            MPF_CUDA(cudaMemcpyAsync(h.data(), info, sizeof(int) * P.G, cudaMemcpyDeviceToHost, s));
            MPF_CUDA(cudaStreamSynchronize(s));
            for (int g = 0; g < P.G; ++g)
                if (redo[g] && h[g] != 0) jacobiOnly.push_back(g);
        }
        Lsrc = L64;
    } else {
        MPF_TRY(dense_cholesky_f64(P.G, cp.ncPad, Ac64, info, s, groupMask));
    }
    k_coarse_prep<<<dim3(cp.ncPad / 32, P.G), 32, 0, s>>>(cp.ncPad, Lsrc, Lc, LinvD, groupMask);
    const size_t smem = coarse_solve_smem(cp.ncPad);
    static std::atomic<size_t> configured[64];
    int dev = 0;
    MPF_CUDA(cudaGetDevice(&dev));
    MPF_CHECK(dev >= 0 && dev < 64, MPF_EINVAL, "coarse setup: device ordinal %d out of range", dev);
    if (smem > configured[dev].load()) {
        MPF_CUDA(cudaFuncSetAttribute(k_coarse_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured[dev].store(smem);
    }
    k_coarse_inverse<<<dim3(cp.ncPad / 32, P.G), kCT, smem, s>>>(cp.ncPad, Lc, LinvD, Binv, groupMask);
    MPF_LAUNCHED(2);
    for (int g : jacobiOnly) {
        MPF_CUDA(cudaMemsetAsync(Binv + per * g, 0, sizeof(float) * per, s));
        MPF_CUDA(cudaMemsetAsync(info + g, 0, sizeof(int), s));
    }
    return MPF_OK;
}

}  // namespace mpf
