// Dense kernels of the Gauss-Newton step.
//
//  * k_gram_tc   C = A A^T from split hi+lo BF16 operands on the 5th-gen tensor
//                cores: TMA (128B-swizzled tiles) -> shared memory -> tcgen05.mma
//                (kind::f16, FP32 accumulator in tensor memory) -> tcgen05.ld
//                epilogue.  Only tiles on or above the diagonal are computed
//                and the K (element) dimension is split over CTAs; a second
//                kernel reduces the splits in a fixed order and mirrors the
//                result.  hi.hi + hi.lo + lo.hi is accumulated per k-block.
//  * Cholesky    blocked right-looking FP64 factorisation (32x32 blocks:
//                diagonal factor, panel solve, trailing update) and the two
//                triangular solves, batched over frames.
// The GEMM replaces the cuBLAS J^T J of src/solver/inverse.cpp:136-156 (taken
// in dual orientation, J J^T); the factorisation replaces the dense CG of
// src/solver/inverse.cpp:213-238.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "model.h"
#include "tc_ptx.cuh"

namespace mpf {
namespace {

using namespace tc;

// ---------------------------------------------------------------------------
constexpr int kStages = 3;
constexpr int kStageBytes = 4 * kTileBytes;      // A_hi, A_lo, B_hi, B_lo
constexpr int kGramSmem = kStages * kStageBytes + 1024 /*align*/ + 256 /*barriers*/;

struct GramArgs {
    int rows;        // rows per batch entry (multiple of 128)
    int kblocks;     // K blocks (cols / 64)
    int tiles;       // upper-triangular tile count per batch entry
    int nt;          // tiles per dimension
    int splits;      // K splits
    float* work;     // [batch][splits][tiles][128][128]
    int* abortFlag;  // device flag raised by a timed-out wait
    const int* frameMask;  // [batch] entries to compute, or null for all
};

// One CTA = one (batch, upper tile, K split).  Warp 0 lane 0 issues TMA,
// warp 1 lane 0 issues the MMAs, all four warps drain TMEM.
__global__ void __launch_bounds__(128, 1) k_gram_tc(const __grid_constant__ CUtensorMap mapHi,
                                                    const __grid_constant__ CUtensorMap mapLo, GramArgs ga) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + kStages * kStageBytes);
    __shared__ uint32_t tmemBase;
    __shared__ int localAbort;
    __shared__ int issuedLoads;  // K blocks whose TMA loads the producer issued

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.z;
    if (ga.frameMask && !ga.frameMask[b]) return;
    const int split = blockIdx.y;
    // tile index -> (tm, tn) with tm <= tn
    int t = blockIdx.x, tm = 0;
    while (t >= ga.nt - tm) {
        t -= ga.nt - tm;
        ++tm;
    }
    const int tn = tm + t;
    const int kb0 = (int)((long)ga.kblocks * split / ga.splits);
    const int kb1 = (int)((long)ga.kblocks * (split + 1) / ga.splits);
    const int nk = kb1 - kb0;

    const uint32_t fullBar = smem_u32(&bars[0]);
    const uint32_t emptyBar = smem_u32(&bars[kStages]);
    const uint32_t doneBar = smem_u32(&bars[2 * kStages]);

    if (threadIdx.x == 0) {
        localAbort = 0;
        issuedLoads = 0;
        for (int s = 0; s < kStages; ++s) {
            mbar_init(fullBar + 8 * s, 1);
            mbar_init(emptyBar + 8 * s, 1);
        }
        mbar_init(doneBar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        tmem_alloc(smem_u32(&tmemBase), 128);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmemBase;
    volatile int* abortFlag = &localAbort;

    const int rowA = b * ga.rows + tm * kTile;
    const int rowB = b * ga.rows + tn * kTile;
    const uint32_t smemBase = smem_u32(smem);

    if (warp == 0 && lane == 0) {
        // producer
        for (int i = 0; i < nk; ++i) {
            const int s = i % kStages, round = i / kStages;
            if (round > 0 && !mbar_wait(emptyBar + 8 * s, (round - 1) & 1, abortFlag)) break;
            const uint32_t st = smemBase + s * kStageBytes;
            mbar_expect_tx(fullBar + 8 * s, kStageBytes);
            const int x = (kb0 + i) * kBK;
            tma_load_2d(st, &mapHi, fullBar + 8 * s, x, rowA);
            tma_load_2d(st + kTileBytes, &mapLo, fullBar + 8 * s, x, rowA);
            tma_load_2d(st + 2 * kTileBytes, &mapHi, fullBar + 8 * s, x, rowB);
            tma_load_2d(st + 3 * kTileBytes, &mapLo, fullBar + 8 * s, x, rowB);
            issuedLoads = i + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        for (int i = 0; i < nk; ++i) {
            const int s = i % kStages, round = i / kStages;
            if (!mbar_wait(fullBar + 8 * s, round & 1, abortFlag)) break;
            fence_after();
            const uint32_t st = smemBase + s * kStageBytes;
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const uint32_t off = kk * 32;
                const uint64_t aHi = sw128_desc(st + off), aLo = sw128_desc(st + kTileBytes + off);
                const uint64_t bHi = sw128_desc(st + 2 * kTileBytes + off), bLo = sw128_desc(st + 3 * kTileBytes + off);
                mma_bf16(tmem, aHi, bHi, (i > 0 || kk > 0) ? 1u : 0u);
                mma_bf16(tmem, aHi, bLo, 1u);
                mma_bf16(tmem, aLo, bHi, 1u);
            }
            mma_commit(emptyBar + 8 * s);
        }
        mma_commit(doneBar);
    }
    __syncwarp();
    // epilogue: every warp drains its 32 TMEM lanes
    const bool waited = nk > 0 && mbar_wait(doneBar, 0, abortFlag);
    const bool ok = __all_sync(0xffffffffu, waited && !*abortFlag);
    fence_after();
    const int row = warp * 32 + lane;
    float* out = ga.work + ((((size_t)b * ga.splits + split) * ga.tiles + blockIdx.x) * kTile + row) * kTile;
    if (ok) {
#pragma unroll 1
        for (int c = 0; c < kTile; c += 32) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int i = 0; i < 32; i += 4) *reinterpret_cast<float4*>(out + c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
    } else {
        for (int c = 0; c < kTile; ++c) out[c] = 0.f;
        if (threadIdx.x == 0 && nk > 0) atomicExch(ga.abortFlag, 1);
    }
    fence_before();
    if (__syncthreads_or(!ok) && nk > 0) {
        // A wait gave up: MMAs and TMA loads issued before the break may still
        // be in flight.  Before TMEM is released and the CTA exits, wait (with
        // the same limit, on a flag of its own) for the MMA issuer's final
        // commit, which covers every MMA it issued, and for the last load
        // issued into each stage (phases complete in order, and a stage's
        // round r is issued only after its round r - 1 was consumed, so the
        // parity of round r names that round).  TMEM is released even if
        // these waits give up too: a CTA that exits holding TMEM would block
        // every later allocation on its SM.  The result of a launch that
        // raised the abort flag is undefined; the host reports MPF_ETIMEOUT.
        if (threadIdx.x == 0) {
            volatile int quiet = 0;
            mbar_wait(doneBar, 0, &quiet);
            for (int s = 0; s < kStages && s < issuedLoads; ++s) {
                quiet = 0;
                mbar_wait(fullBar + 8 * s, ((issuedLoads - 1 - s) / kStages) & 1, &quiet);
            }
        }
        __syncthreads();
    }
    if (warp == 1) {
        fence_after();
        tmem_dealloc(tmem, 128);
    }
}

// Sum the K splits in order and write the full symmetric matrix, either FP32
// (C) or FP64 with a diagonal shift (A64).
__global__ void k_gram_reduce(int rows, int tiles, int nt, int splits, const float* __restrict__ work,
                              float* __restrict__ C, double* __restrict__ A64, double shift,
                              const int* __restrict__ frameMask) {
    const int b = blockIdx.z, tile = blockIdx.y;
    if (frameMask && !frameMask[b]) return;
    int t = tile, tm = 0;
    while (t >= nt - tm) {
        t -= nt - tm;
        ++tm;
    }
    const int tn = tm + t;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kTile * kTile; i += gridDim.x * blockDim.x) {
        const int r = i / kTile, c = i % kTile;
        float s = 0.f;
        for (int sp = 0; sp < splits; ++sp) s += work[(((size_t)b * splits + sp) * tiles + tile) * kTile * kTile + i];
        const int gr = tm * kTile + r, gc = tn * kTile + c;
        if (C) {
            C[(size_t)b * rows * rows + (size_t)gr * rows + gc] = s;
            C[(size_t)b * rows * rows + (size_t)gc * rows + gr] = s;
        }
        if (A64) {
            const double v = (double)s + (gr == gc ? shift : 0.0);
            A64[(size_t)b * rows * rows + (size_t)gr * rows + gc] = v;
            A64[(size_t)b * rows * rows + (size_t)gc * rows + gr] = v;
        }
    }
}

// A64[b] = J J^T + shift I in FP64 from the FP32 J (rows x ld row-major per
// frame) on the FP64 pipe: the accurate Gram for frames whose split-BF16
// J J^T + mu I is not positive definite (mu below the ~1e-5 relative error of
// the BF16 split and FP32 accumulation).  64 x 64 output tiles of the upper
// triangle, mirrored; 256 threads with 4 x 4 outputs each; K in chunks of 32
// staged in shared memory as FP64.
__global__ void __launch_bounds__(256) k_gram_f64(int rows, int cols, const float* __restrict__ J, int ld,
                                                  double shift, double* __restrict__ A64,
                                                  const int* __restrict__ frameMask) {
    const int b = blockIdx.z, ti = blockIdx.y, tj = blockIdx.x;
    if (frameMask && !frameMask[b]) return;
    if (tj < ti) return;
    __shared__ double As[32][65], Bs[32][65];
    const float* Jb = J + (size_t)b * rows * ld;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < cols; k0 += 32) {
        for (int t = threadIdx.x; t < 64 * 32; t += 256) {
            const int r = t / 32, k = t % 32;
            As[k][r] = (double)Jb[(size_t)(ti * 64 + r) * ld + k0 + k];
            Bs[k][r] = (double)Jb[(size_t)(tj * 64 + r) * ld + k0 + k];
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
            double a[4], c[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i] = As[k][ty + 16 * i];
                c[i] = Bs[k][tx + 16 * i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], c[j], acc[i][j]);
        }
        __syncthreads();
    }
    double* A = A64 + (size_t)b * rows * rows;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = ti * 64 + ty + 16 * i, c = tj * 64 + tx + 16 * j;
            const double v = acc[i][j] + (r == c ? shift : 0.0);
            A[(size_t)r * rows + c] = v;
            A[(size_t)c * rows + r] = v;
        }
}

__global__ void k_split_bf16(int batch, int rows, int cols, const float* __restrict__ A, int lda,
                             __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
    const size_t total = (size_t)batch * rows * lda;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % lda);
        const float v = c < cols ? A[i] : 0.f;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

// ---------------------------------------------------------------------------
// FP64 Cholesky, 32x32 blocks, column-major (lower triangle holds L).
constexpr int NB = 32;

__global__ void k_potrf_diag(int n, double* A, int k, int* info, const int* frameMask) {
    if (frameMask && !frameMask[blockIdx.x]) return;
    __shared__ double a[NB][NB + 1];
    __shared__ int bad;
    double* M = A + (size_t)blockIdx.x * n * n;
    const int o = k * NB;
    for (int i = threadIdx.x; i < NB * NB; i += blockDim.x) {
        const int r = i % NB, c = i / NB;
        a[r][c] = M[(size_t)(o + r) + (size_t)(o + c) * n];
    }
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < NB; ++j) {
        if (threadIdx.x == 0) {
            const double d = a[j][j];
            if (!(d > 0.0)) {
                if (!bad && info[blockIdx.x] == 0) info[blockIdx.x] = o + j + 1;
                bad = 1;
                a[j][j] = 1.0;
            } else {
                a[j][j] = sqrt(d);
            }
        }
        __syncthreads();
        for (int i = j + 1 + threadIdx.x; i < NB; i += blockDim.x) a[i][j] /= a[j][j];
        __syncthreads();
        for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
            const int i = idx % NB, l = idx / NB;
            if (l > j && i >= l) a[i][l] -= a[i][j] * a[l][j];
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < NB * NB; i += blockDim.x) {
        const int r = i % NB, c = i / NB;
        if (r >= c) M[(size_t)(o + r) + (size_t)(o + c) * n] = a[r][c];
    }
}

// ---------------------------------------------------------------------------
// Batched Cholesky in FP32 arithmetic (k_potrf32): one thread-block cluster
// of CL CTAs per matrix (CL = 1 for batches that fill the GPU on their own).
// Right-looking in 32-column steps on FP64 column-major storage:
//   (a) warp 0 of every CTA factors the diagonal block (lane r owns row r)
//       and inverts it -- the same values in every CTA;
//   (b) every CTA solves all rows of the panel below against that inverse
//       into its own shared memory (row stride 36 floats so rows can be read
//       as float4);
//   (c) the trailing lower triangle is updated in 32 x 32 tiles spread over
//       the cluster's warps: lane r owns row r of a tile, loads its targets
//       8 columns at a time, then accumulates the dot products of length 32
//       from float4 broadcasts of the panel;
//   a cluster barrier (release / acquire) ends the step, so the next step's
//   reads of the diagonal block and panel see every rank's updates;
//   (d) the step's block column (diagonal block from rank 0, each 32-row
//       panel block from one rank) is stored from shared memory after that
//       barrier, when no rank reads its input values any more.
// The factor is returned in the FP64 storage (values of FP32 precision); the
// strict upper triangle is not touched.  info[b] = the first pivot (1-based)
// that is not positive (it is replaced by 1 so that the factorisation
// finishes without NaN), as in the FP64 routine.  A CTA needs n * 36 * 4
// bytes of shared memory (n <= 1536).
constexpr int kPotrfThreads = 256;
constexpr int kPanelStride = 36;

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kPotrfThreads, 1) k_potrf32(int n, const double* __restrict__ Ain, double* __restrict__ Lall,
                                                           int* __restrict__ info, const int* __restrict__ frameMask) {
    const unsigned CL = cluster_size(), rank = cluster_rank();
    const int b = blockIdx.x / CL;
    if (frameMask && !frameMask[b]) return;  // the whole cluster leaves together
    extern __shared__ __align__(16) float panel[];  // [n][kPanelStride]
    __shared__ float D[NB][NB + 1];                // diagonal block
    __shared__ float Di[NB][NB + 1];               // its inverse
    __shared__ int bad;
    double* L = Lall + (size_t)b * n * n;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto step_sync = [&]() {
        if (CL > 1)
            cluster_sync_all();
        else
            __syncthreads();
    };
    if (Ain != Lall) {
        const double* A = Ain + (size_t)b * n * n;
        for (size_t t = rank * kPotrfThreads + threadIdx.x; t < (size_t)n * n; t += (size_t)CL * kPotrfThreads) {
            const int r = (int)(t % n), c = (int)(t / n);
            if (r >= c) L[t] = A[t];
        }
    }
    if (threadIdx.x == 0) bad = 0;
    step_sync();
    const int nb = n / NB;
    for (int k = 0; k < nb; ++k) {
        const int o = k * NB;
        // (a) diagonal block: factor and invert (warp 0 of every CTA)
        if (warp == 0) {
            for (int c = 0; c < NB; ++c) D[lane][c] = lane >= c ? (float)L[(size_t)(o + lane) + (size_t)(o + c) * n] : 0.f;
            __syncwarp();
            for (int j = 0; j < NB; ++j) {
                if (lane == 0) {
                    const float d = D[j][j];
                    if (!(d > 0.f) || !isfinite(d)) {
                        if (!bad && rank == 0) info[b] = o + j + 1;
                        bad = 1;
                        D[j][j] = 1.f;
                    } else {
                        D[j][j] = sqrtf(d);
                    }
                }
                __syncwarp();
                if (lane > j) D[lane][j] /= D[j][j];
                __syncwarp();
                if (lane > j)
                    for (int l = j + 1; l <= lane; ++l) D[lane][l] = fmaf(-D[lane][j], D[l][j], D[lane][l]);
                __syncwarp();
            }
            // column `lane` of D^-1 by forward substitution
            float x[NB];
#pragma unroll
            for (int r = 0; r < NB; ++r) {
                float v = r == lane ? 1.f : 0.f;
#pragma unroll
                for (int q = 0; q < r; ++q) v = fmaf(-D[r][q], x[q], v);
                x[r] = r < lane ? 0.f : v / D[r][r];
            }
#pragma unroll
            for (int r = 0; r < NB; ++r) Di[r][lane] = x[r];
        }
        __syncthreads();
        // (b) panel rows: L_ik = A_ik D^-T (every CTA, all rows, into shared memory)
        for (int i = o + NB + threadIdx.x; i < n; i += kPotrfThreads) {
            float a[NB];
#pragma unroll
            for (int t = 0; t < NB; ++t) a[t] = (float)L[(size_t)i + (size_t)(o + t) * n];
            float* pr = panel + (size_t)i * kPanelStride;
#pragma unroll 1
            for (int j = 0; j < NB; ++j) {
                float v = 0.f;
#pragma unroll
                for (int t = 0; t <= j; ++t) v = fmaf(a[t], Di[j][t], v);
                pr[j] = v;
            }
        }
        __syncthreads();
        // (c) trailing update A_ij -= L_ik L_jk^T on the lower tiles (bi >= bj > k)
        const int m = nb - k - 1;
        const int tiles = m * (m + 1) / 2;
        const int wpc = kPotrfThreads / 32;
#pragma unroll 1
        for (int tI = rank * wpc + warp; tI < tiles; tI += CL * wpc) {
            int bi = 0, rem = tI;
            while (rem > bi) {
                rem -= bi + 1;
                ++bi;
            }
            const int bj = rem;  // 0 <= bj <= bi < m
            const int i = o + NB + bi * NB + lane, j0 = o + NB + bj * NB;
            const int cEnd = bi != bj ? NB : lane + 1;  // diagonal tiles: the lower part only
            float4 pr[NB / 4];
            const float4* rowI = reinterpret_cast<const float4*>(panel + (size_t)i * kPanelStride);
#pragma unroll
            for (int t = 0; t < NB / 4; ++t) pr[t] = rowI[t];
            // 8 target columns at a time: their loads are issued together
#pragma unroll 1
            for (int c0 = 0; c0 < NB; c0 += 8) {
                double* rowT = L + (size_t)i + (size_t)(j0 + c0) * n;
                float tgt[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) tgt[c] = c0 + c < cEnd ? (float)rowT[(size_t)c * n] : 0.f;
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const float4* rowJ = reinterpret_cast<const float4*>(panel + (size_t)(j0 + c0 + c) * kPanelStride);
                    float v = 0.f;
#pragma unroll
                    for (int t = 0; t < NB / 4; ++t) {
                        const float4 q = rowJ[t];
                        v = fmaf(pr[t].x, q.x, v);
                        v = fmaf(pr[t].y, q.y, v);
                        v = fmaf(pr[t].z, q.z, v);
                        v = fmaf(pr[t].w, q.w, v);
                    }
                    tgt[c] -= v;
                }
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (c0 + c < cEnd) rowT[(size_t)c * n] = (double)tgt[c];
            }
        }
        step_sync();
        // (d) store block column k
        if (rank == 0 && warp == 0)
            for (int c = 0; c < NB; ++c)
                if (lane >= c) L[(size_t)(o + lane) + (size_t)(o + c) * n] = (double)D[lane][c];
        for (int i = o + NB + threadIdx.x; i < n; i += kPotrfThreads)
            if ((unsigned)((i / NB) % CL) == rank) {
                const float* pr = panel + (size_t)i * kPanelStride;
                for (int j = 0; j < NB; ++j) L[(size_t)i + (size_t)(o + j) * n] = (double)pr[j];
            }
        __syncthreads();  // the next step overwrites D, Di and the panel
    }
}

// A(j, i) = A(i, j) for i > j: the upper triangle becomes the mirror of the
// lower one, the part the Cholesky routines read (the tensor-core Gram's
// diagonal tiles are symmetric only to FP32 rounding).  32 x 32 tiles through
// shared memory; grid (n/32, n/32, batch), tiles above the diagonal exit.
__global__ void k_mirror_lower(int n, double* __restrict__ A, const int* __restrict__ frameMask) {
    const int bi = blockIdx.x, bj = blockIdx.y, b = blockIdx.z;
    if (bj > bi || (frameMask && !frameMask[b])) return;
    __shared__ double t[32][33];
    double* M = A + (size_t)b * n * n;
    const int r = threadIdx.x & 31, c0 = threadIdx.x >> 5;  // 256 threads: 8 columns per pass
    for (int c = c0; c < 32; c += 8) t[r][c] = M[(size_t)(bi * 32 + r) + (size_t)(bj * 32 + c) * n];
    __syncthreads();
    // element (bi*32 + c, bj*32 + r) of the tile goes to (bj*32 + r, bi*32 + c)
    for (int c = c0; c < 32; c += 8)
        if (bi != bj || c > r) M[(size_t)(bj * 32 + r) + (size_t)(bi * 32 + c) * n] = t[c][r];
}

// r = y - A x for the full symmetric FP64 matrices A (n x n per frame), one warp
// per row (4 rows per warp, 32 per block: every SM keeps many rows' loads in
// flight), and per block the partial sums of r.r and y.y (n / 32 per frame).
__global__ void __launch_bounds__(256) k_sym_residual(int n, const double* __restrict__ A, const double* __restrict__ x,
                                                      const double* __restrict__ y, double* __restrict__ r,
                                                      double* __restrict__ rr, double* __restrict__ yy,
                                                      const int* __restrict__ frameMask) {
    const int b = blockIdx.y;
    if (frameMask && !frameMask[b]) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double* M = A + (size_t)b * n * n;
    const double* xb = x + (size_t)b * n;
    __shared__ double red[2][8];
    double r2 = 0.0, y2 = 0.0;
    for (int q = 0; q < 4; ++q) {
        const int i = blockIdx.x * 32 + warp * 4 + q;
        const double* row = M + (size_t)i * n;
        double acc = 0.0;
#pragma unroll 4
        for (int k = lane; k < n; k += 32) acc = fma(row[k], xb[k], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            const double yi = y[(size_t)b * n + i], ri = yi - acc;
            r[(size_t)b * n + i] = ri;
            r2 += ri * ri;
            y2 += yi * yi;
        }
    }
    if (lane == 0) {
        red[0][warp] = r2;
        red[1][warp] = y2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int w = 0; w < 8; ++w) {
            s0 += red[0][w];
            s1 += red[1][w];
        }
        rr[(size_t)b * gridDim.x + blockIdx.x] = s0;
        yy[(size_t)b * gridDim.x + blockIdx.x] = s1;
    }
}

// x += d on the active frames
__global__ void k_add_masked(int n, int batch, double* __restrict__ x, const double* __restrict__ d,
                             const int* __restrict__ frameMask) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)n * batch; t += (size_t)gridDim.x * blockDim.x)
        if (!frameMask || frameMask[t / n]) x[t] += d[t];
}

// Inverse of the FP32 Cholesky factor, for refinement steps that are two
// matrix-vector products instead of two latency-bound triangular solves.
// L is the factor held in FP64 storage (values of the FP32 factor, lower
// triangle, column-major n x n per frame: L(r, c) at c n + r, as the
// triangular solves read it); the inverse X = L^-1 is computed in
// FP32 in 32 x 32 blocks (NB): first the inverse D_b of every diagonal
// block, then every block column j by forward substitution,
// X_jj = D_j, X_ij = -D_i sum_{k=j}^{i-1} L_ik X_kj (i > j).
//
// One warp per (frame, diagonal block): lane c computes column c of D_b.
__global__ void __launch_bounds__(32) k_trtri_diag(int n, const double* __restrict__ L, float* __restrict__ D,
                                                   const int* __restrict__ frameMask) {
    const int b = blockIdx.x, f = blockIdx.y;
    if (frameMask && !frameMask[f]) return;
    __shared__ float Lb[NB][NB + 1];
    const double* M = L + (size_t)f * n * n + (size_t)(b * NB) * n + b * NB;
    const int c = threadIdx.x;
    for (int k = 0; k < NB; ++k) Lb[c][k] = (float)M[(size_t)k * n + c];  // L(c, k), column k coalesced
    __syncwarp();
    float x[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        float v = i == c ? 1.f : 0.f;
#pragma unroll
        for (int k = 0; k < i; ++k) v = fmaf(-Lb[i][k], x[k], v);
        x[i] = v / Lb[i][i];
    }
    float* out = D + ((size_t)f * (n / NB) + b) * NB * NB;
#pragma unroll
    for (int i = 0; i < NB; ++i) out[i * NB + c] = x[i];
}

// L in FP32 (column-major, as the FP64 storage) for the column kernel below.
__global__ void k_to_f32(size_t count, const double* __restrict__ src, float* __restrict__ dst,
                         const int* __restrict__ frameMask, size_t per) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
        if (!frameMask || frameMask[t / per]) dst[t] = (float)src[t];
}

// One block of 256 threads per (frame, block column j): the column's blocks
// X_ij, i >= j, kept in shared memory as they are formed (the later ones
// need the earlier), written to X (row-major) and to XT = X^T (row-major, so
// that the transposed product is also a row-wise one).  X_jj = D_j,
// X_ij = -D_i sum_{k=j}^{i-1} L_ik X_kj, the L_ik staged one 32 x 32 tile at
// a time (the next tile's loads in flight while the current one is used).
// Thread t owns row t / 8 and columns 4 (t % 8) .. + 3 of the block in
// progress.  Measured alternatives, 32 frames of 1024: this order without
// the prefetch 2.8 ms; right-looking (each block column of L read once per
// step) 3.7 ms; each thread streaming its row of L from memory without
// staging 8.4 ms.
__global__ void __launch_bounds__(256) k_trtri_cols(int n, const float* __restrict__ L, const float* __restrict__ D,
                                                    float* __restrict__ X, float* __restrict__ XT,
                                                    const int* __restrict__ frameMask) {
    const int j = blockIdx.x, f = blockIdx.y, nb = n / NB;
    if (frameMask && !frameMask[f]) return;
    extern __shared__ __align__(16) float col[];  // [nb - j][NB][NB]: X_ij, i = j ..
    __shared__ float Lt[NB][NB + 1], Tt[NB][NB + 1];
    const float* Lf = L + (size_t)f * n * n;
    const float* Df = D + (size_t)f * nb * NB * NB;
    float* Xf = X + (size_t)f * n * n;
    float* XTf = XT + (size_t)f * n * n;
    const int t = threadIdx.x, r = t >> 3, c0 = (t & 7) * 4;
    for (int i = j; i < nb; ++i) {
        float* Xi = col + (size_t)(i - j) * NB * NB;
        if (i == j) {
            for (int e = t; e < NB * NB; e += 256) Xi[e] = Df[(size_t)j * NB * NB + e];
        } else {
            // T = sum_k L_ik X_kj; the next tile of L is loaded into registers
            // while the current one is used (4 elements per thread)
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            // element q of this thread: L(i NB + t % 32, k NB + t / 32 + 8 q), column-major
            const float* Lp = Lf + (size_t)(t / NB) * n + i * NB + (t % NB);
            float n0 = Lp[(size_t)(j * NB) * n], n1 = Lp[(size_t)(j * NB + 8) * n];
            float n2 = Lp[(size_t)(j * NB + 16) * n], n3 = Lp[(size_t)(j * NB + 24) * n];
            for (int k = j; k < i; ++k) {
                __syncthreads();  // Lt free
                Lt[t % NB][t / NB] = n0;
                Lt[t % NB][t / NB + 8] = n1;
                Lt[t % NB][t / NB + 16] = n2;
                Lt[t % NB][t / NB + 24] = n3;
                if (k + 1 < i) {
                    const float* Lk = Lp + (size_t)((k + 1) * NB) * n;
                    n0 = Lk[0];
                    n1 = Lk[(size_t)8 * n];
                    n2 = Lk[(size_t)16 * n];
                    n3 = Lk[(size_t)24 * n];
                }
                __syncthreads();
                const float* Xk = col + (size_t)(k - j) * NB * NB;
#pragma unroll 8
                for (int q = 0; q < NB; ++q) {
                    const float l = Lt[r][q];
                    const float4 xv = *reinterpret_cast<const float4*>(Xk + q * NB + c0);
                    acc[0] = fmaf(l, xv.x, acc[0]);
                    acc[1] = fmaf(l, xv.y, acc[1]);
                    acc[2] = fmaf(l, xv.z, acc[2]);
                    acc[3] = fmaf(l, xv.w, acc[3]);
                }
            }
            __syncthreads();  // Lt and Tt free
            for (int e = 0; e < 4; ++e) Tt[r][c0 + e] = acc[e];
            for (int e = t; e < NB * NB; e += 256) Lt[e / NB][e % NB] = Df[(size_t)i * NB * NB + e];  // D_i
            __syncthreads();
            // X_ij = -D_i T
            float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
            for (int q = 0; q < NB; ++q) {
                const float d = Lt[r][q];
#pragma unroll
                for (int e = 0; e < 4; ++e) v[e] = fmaf(d, Tt[q][c0 + e], v[e]);
            }
            for (int e = 0; e < 4; ++e) Xi[r * NB + c0 + e] = -v[e];
        }
        __syncthreads();  // X_ij complete
        for (int e = t; e < NB * NB; e += 256) {
            const int rr = e / NB, cc = e % NB;
            Xf[(size_t)(i * NB + rr) * n + j * NB + cc] = Xi[rr * NB + cc];
            XTf[(size_t)(j * NB + rr) * n + i * NB + cc] = Xi[cc * NB + rr];
        }
    }
}

// out[f][i] = sum_k M[f][i][k] v[f][k] over the lower (k <= i) or upper
// (k >= i) triangle of row i; one warp per row, FP32 products of the FP32
// matrix with v rounded to FP32, FP64 result.
__global__ void __launch_bounds__(256) k_tri_rows(int n, const float* __restrict__ M, const double* __restrict__ v,
                                                  double* __restrict__ out, int upper,
                                                  const int* __restrict__ frameMask) {
    const int f = blockIdx.y;
    if (frameMask && !frameMask[f]) return;
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= n) return;
    const float* row = M + (size_t)f * n * n + (size_t)i * n;
    const double* vf = v + (size_t)f * n;
    const int k0 = upper ? i : 0, k1 = upper ? n : i + 1;
    float acc = 0.f;
    for (int k = k0 + lane; k < k1; k += 32) acc = fmaf(row[k], (float)vf[k], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[(size_t)f * n + i] = (double)acc;
}

// L_ik = A_ik L_kk^-T for the block rows below the diagonal block k
__global__ void k_trsm(int n, double* A, int k, const int* frameMask) {
    if (frameMask && !frameMask[blockIdx.y]) return;
    __shared__ double L[NB][NB + 1];
    __shared__ double X[NB][NB + 1];
    double* M = A + (size_t)blockIdx.y * n * n;
    const int o = k * NB, ro = (k + 1 + blockIdx.x) * NB;
    for (int i = threadIdx.x; i < NB * NB; i += blockDim.x) {
        const int r = i % NB, c = i / NB;
        L[r][c] = M[(size_t)(o + r) + (size_t)(o + c) * n];
        X[r][c] = M[(size_t)(ro + r) + (size_t)(o + c) * n];
    }
    __syncthreads();
    if (threadIdx.x < NB) {
        const int r = threadIdx.x;
        for (int j = 0; j < NB; ++j) {
            double s = X[r][j];
            for (int l = 0; l < j; ++l) s -= X[r][l] * L[j][l];
            X[r][j] = s / L[j][j];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NB * NB; i += blockDim.x) {
        const int r = i % NB, c = i / NB;
        M[(size_t)(ro + r) + (size_t)(o + c) * n] = X[r][c];
    }
}

// A_ij -= L_ik L_jk^T for k < j <= i
__global__ void k_syrk(int n, double* A, int k, const int* frameMask) {
    if (frameMask && !frameMask[blockIdx.y]) return;
    __shared__ double Li[NB][NB + 1];
    __shared__ double Lj[NB][NB + 1];
    double* M = A + (size_t)blockIdx.y * n * n;
    int t = blockIdx.x, bi = 0;
    while (t > bi) {
        t -= bi + 1;
        ++bi;
    }
    const int bj = t;  // bj <= bi, both relative to k+1
    const int o = k * NB, io = (k + 1 + bi) * NB, jo = (k + 1 + bj) * NB;
    for (int i = threadIdx.x; i < NB * NB; i += blockDim.x) {
        const int r = i % NB, c = i / NB;
        Li[r][c] = M[(size_t)(io + r) + (size_t)(o + c) * n];
        Lj[r][c] = M[(size_t)(jo + r) + (size_t)(o + c) * n];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
        const int r = idx % NB, c = idx / NB;
        double s = 0.0;
#pragma unroll 8
        for (int l = 0; l < NB; ++l) s = fma(Li[r][l], Lj[c][l], s);
        M[(size_t)(io + r) + (size_t)(jo + c) * n] -= s;
    }
}

// L L^T x = b with L column-major lower, one block of 256 threads per
// (batch, right-hand side), in 32-row block steps.  Every read of L runs
// down a column (consecutive threads, consecutive rows): the forward pass
// is right-looking (after solving block k, the rows below it take
// x[r] -= L[r][k-block] x[k-block]), the backward pass left-looking (block
// k's columns take warp-reduced dots with the solved rows below).  The
// 32 x 32 diagonal block is staged in shared memory and solved by one warp
// with shuffles.
__global__ void __launch_bounds__(1024) k_chol_solve(int n, const double* __restrict__ Lall, double* __restrict__ Ball,
                                                    int nrhs, const int* __restrict__ frameMask) {
    if (frameMask && !frameMask[blockIdx.x / nrhs]) return;
    extern __shared__ double x[];
    __shared__ double D[NB][NB + 1];
    const int b = blockIdx.x / nrhs, c = blockIdx.x % nrhs;
    const double* L = Lall + (size_t)b * n * n;
    double* B = Ball + ((size_t)b * nrhs + c) * n;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = B[i];
    const int nb = n / NB;
    // forward: L z = b
    for (int bk = 0; bk < nb; ++bk) {
        const int k0 = bk * NB;
        for (int i = threadIdx.x; i < NB * NB; i += blockDim.x) {
            const int r = i % NB, cc = i / NB;
            D[r][cc] = L[(size_t)(k0 + r) + (size_t)(k0 + cc) * n];
        }
        __syncthreads();
        if (warp == 0) {
            double xr = x[k0 + lane];
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                if (lane == j) xr /= D[j][j];
                const double xj = __shfl_sync(0xffffffffu, xr, j);
                if (lane > j) xr -= D[lane][j] * xj;
            }
            x[k0 + lane] = xr;
        }
        __syncthreads();
        for (int r = k0 + NB + threadIdx.x; r < n; r += blockDim.x) {
            double s = 0.0;
#pragma unroll 8
            for (int j = 0; j < NB; ++j) s = fma(L[(size_t)r + (size_t)(k0 + j) * n], x[k0 + j], s);
            x[r] -= s;
        }
    }
    // backward: L^T x = z
    for (int bk = nb - 1; bk >= 0; --bk) {
        const int k0 = bk * NB, below = k0 + NB;
        __syncthreads();
        for (int cc = warp; cc < NB; cc += nwarps) {
            const int col = k0 + cc;
            double s = 0.0;
            for (int r = below + lane; r < n; r += 32) s = fma(L[(size_t)r + (size_t)col * n], x[r], s);
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) x[col] -= s;
        }
        for (int i = threadIdx.x; i < NB * NB; i += blockDim.x) {
            const int r = i % NB, cc = i / NB;
            D[r][cc] = L[(size_t)(k0 + r) + (size_t)(k0 + cc) * n];
        }
        __syncthreads();
        if (warp == 0) {
            double xc = x[k0 + lane];
#pragma unroll
            for (int j = NB - 1; j >= 0; --j) {
                if (lane == j) xc /= D[j][j];
                const double xj = __shfl_sync(0xffffffffu, xc, j);
                if (lane < j) xc -= D[j][lane] * xj;
            }
            x[k0 + lane] = xc;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) B[i] = x[i];
}

__global__ void k_add_shift(int n, double* A, double shift) {
    double* M = A + (size_t)blockIdx.y * n * n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) M[(size_t)i * n + i] += shift;
}

// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int get_encoder(EncodeTiledFn* out) {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    static int status = MPF_OK;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
            status = fail(MPF_ECUDA, "cuTensorMapEncodeTiled unavailable");
            return;
        }
        fn = (EncodeTiledFn)p;
    });
    *out = fn;
    return fn ? MPF_OK : status;
}

int gram_splits(int tiles, int kblocks) {
    int s = 148 / tiles;
    s = std::max(1, std::min(s, kblocks / 8));
    return std::max(1, std::min(s, kblocks));
}

// Failure-path self-test: one thread waits on an mbarrier that nothing
// arrives on, through the same bounded wait as the tensor-core kernels; the
// wait gives up after limitNs and reports through *flag.
__global__ void k_wait_selftest(int* flag, unsigned long long limitNs) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int localAbort;
    if (threadIdx.x != 0) return;
    localAbort = 0;
    mbar_init(smem_u32(&bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!mbar_wait(smem_u32(&bar), 0, &localAbort, limitNs)) atomicExch(flag, 1);
}

}  // namespace

// one pipeline abort flag per device (a kernel must not touch another
// device's memory), allocated on first use on the current device
int* abort_flag_device() {
    static std::mutex mu;
    static int* flags[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!flags[dev]) {
        int* f = nullptr;
        if (cudaMalloc(&f, sizeof(int)) != cudaSuccess) return nullptr;
        if (cudaMemset(f, 0, sizeof(int)) != cudaSuccess) {
            cudaFree(f);
            return nullptr;
        }
        flags[dev] = f;
    }
    return flags[dev];
}

int make_bf16_map(CUtensorMap* map, const __nv_bfloat16* base, int totalRows, int ld) {
    EncodeTiledFn enc;
    MPF_TRY(get_encoder(&enc));
    cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)totalRows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)kTile};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    MPF_CHECK(r == CUDA_SUCCESS, MPF_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MPF_OK;
}

int wait_selftest(int timeoutUs, cudaStream_t s) {
    MPF_CHECK(timeoutUs >= 1 && timeoutUs <= 2000000, MPF_EINVAL, "mpf_selftest_bounded_wait: timeout %d us",
              timeoutUs);
    DevBuf<int> flag;
    MPF_TRY(flag.alloc(1));
    MPF_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int), s));
    k_wait_selftest<<<1, 32, 0, s>>>(flag.ptr, (unsigned long long)timeoutUs * 1000ull);
    MPF_LAUNCHED(1);
    int h = 0;
    MPF_CUDA(cudaMemcpyAsync(&h, flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    return h ? fail(MPF_ETIMEOUT, "bounded wait ran out after %d us (self-test)", timeoutUs) : MPF_OK;
}

size_t dense_gram_work_floats(int batch, int rows, int cols) {
    const int nt = rows / kTile, tiles = nt * (nt + 1) / 2, kblocks = cols / kBK;
    return (size_t)batch * gram_splits(tiles, kblocks) * tiles * kTile * kTile;
}

static int gram_run(int batch, int rows, int cols, const __nv_bfloat16* hi, const __nv_bfloat16* lo, int ld,
                    float* C, double* A64, double shift, float* work, size_t workFloats, cudaStream_t s,
                    int* flagOverride = nullptr, const int* frameMask = nullptr) {
    MPF_CHECK(rows % kTile == 0 && cols % kBK == 0 && ld % 8 == 0 && ld >= cols, MPF_EINVAL,
              "gram: rows %% 128, cols %% 64 and ld %% 8 must be 0 (rows=%d cols=%d ld=%d)", rows, cols, ld);
    const int nt = rows / kTile, tiles = nt * (nt + 1) / 2, kblocks = cols / kBK;
    const int splits = gram_splits(tiles, kblocks);
    MPF_CHECK(workFloats >= (size_t)batch * splits * tiles * kTile * kTile, MPF_EINVAL, "gram: workspace too small");
    CUtensorMap mHi, mLo;
    MPF_TRY(make_bf16_map(&mHi, hi, batch * rows, ld));
    MPF_TRY(make_bf16_map(&mLo, lo, batch * rows, ld));
    int* flag = flagOverride ? flagOverride : abort_flag_device();
    MPF_CHECK(flag != nullptr, MPF_ENOMEM, "gram: abort flag allocation failed");
    // per device and cheap: set on every call
    MPF_CUDA(cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kGramSmem));
    GramArgs ga{rows, kblocks, tiles, nt, splits, work, flag, frameMask};
    k_gram_tc<<<dim3(tiles, splits, batch), 128, kGramSmem, s>>>(mHi, mLo, ga);
    MPF_LAUNCHED(1);
    k_gram_reduce<<<dim3(16, tiles, batch), 256, 0, s>>>(rows, tiles, nt, splits, work, C, A64, shift, frameMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_gram_split_bf16(int batch, int rows, int cols, const __nv_bfloat16* hi, const __nv_bfloat16* lo, int ld,
                          float* C, float* work, size_t workFloats, cudaStream_t s) {
    return gram_run(batch, rows, cols, hi, lo, ld, C, nullptr, 0.0, work, workFloats, s);
}

int dense_gram_f64_shift(int batch, int rows, int cols, const __nv_bfloat16* hi, const __nv_bfloat16* lo, int ld,
                         double shift, double* A64, float* work, size_t workFloats, cudaStream_t s,
                         const int* frameMask) {
    return gram_run(batch, rows, cols, hi, lo, ld, nullptr, A64, shift, work, workFloats, s, nullptr, frameMask);
}

// Measurement hook for the J J^T of the GN step: batch x (rows x cols) BF16
// hi/lo operands filled with hashed values in [-1, 1), one warm-up, then
// `reps` launches of the whole Gram (tcgen05 kernel + split-K reduction into
// FP64 with a shift) timed with CUDA events on `s`.
__global__ void k_fill_bf16_hash(size_t n, uint32_t seed, __nv_bfloat16* __restrict__ a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u ^ seed;
        h ^= h >> 16;
        h *= 0x7feb352du;
        h ^= h >> 15;
        a[i] = __float2bfloat16((float)(h & 0xffffu) * (1.f / 32768.f) - 1.f);
    }
}

int dense_profile_gram(int batch, int rows, int cols, int reps, double* msPerLaunch, cudaStream_t s) {
    MPF_CHECK(batch >= 1 && reps >= 1 && msPerLaunch, MPF_EINVAL, "mpf_profile_gram: bad arguments");
    MPF_CHECK(rows % kTile == 0 && cols % kBK == 0, MPF_EINVAL,
              "mpf_profile_gram: rows %% %d and cols %% %d must be 0 (rows=%d cols=%d)", kTile, kBK, rows, cols);
    const size_t n = (size_t)batch * rows * cols;
    DevBuf<__nv_bfloat16> hi, lo;
    DevBuf<float> work;
    DevBuf<double> A;
    MPF_TRY(hi.alloc(n));
    MPF_TRY(lo.alloc(n));
    MPF_TRY(work.alloc(dense_gram_work_floats(batch, rows, cols)));
    MPF_TRY(A.alloc((size_t)batch * rows * rows));
    k_fill_bf16_hash<<<2048, 256, 0, s>>>(n, 0x1234u, hi.ptr);
    k_fill_bf16_hash<<<2048, 256, 0, s>>>(n, 0x9876u, lo.ptr);
    MPF_LAUNCHED(2);
    MPF_TRY(gram_run(batch, rows, cols, hi.ptr, lo.ptr, cols, nullptr, A.ptr, 1.0, work.ptr, work.count, s));
    cudaEvent_t e0, e1;
    MPF_CUDA(cudaEventCreate(&e0));
    MPF_CUDA(cudaEventCreate(&e1));
    MPF_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < reps; ++r)
        MPF_TRY(gram_run(batch, rows, cols, hi.ptr, lo.ptr, cols, nullptr, A.ptr, 1.0, work.ptr, work.count, s));
    MPF_CUDA(cudaEventRecord(e1, s));
    MPF_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    MPF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    bool aborted = false;
    MPF_TRY(dense_gram_check_abort(&aborted));
    MPF_CHECK(!aborted, MPF_ETIMEOUT, "mpf_profile_gram: a pipeline wait timed out");
    *msPerLaunch = (double)ms / reps;
    return MPF_OK;
}

int dense_gram_f64_exact(int batch, int rows, int cols, const float* J, int ld, double shift, double* A64,
                         const int* frameMask, cudaStream_t s) {
    MPF_CHECK(rows % 64 == 0 && cols % 32 == 0 && ld >= cols, MPF_EINVAL,
              "FP64 Gram: rows %% 64 and cols %% 32 must be 0 (rows=%d cols=%d)", rows, cols);
    k_gram_f64<<<dim3(rows / 64, rows / 64, batch), 256, 0, s>>>(rows, cols, J, ld, shift, A64, frameMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_gram_check_abort(bool* aborted) {
    int* flag = abort_flag_device();
    int h = 0;
    MPF_CUDA(cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost));
    *aborted = h != 0;
    if (h) MPF_CUDA(cudaMemset(flag, 0, sizeof(int)));
    return MPF_OK;
}

int dense_split_bf16(int batch, int rows, int cols, const float* A, int lda, __nv_bfloat16* hi, __nv_bfloat16* lo,
                     cudaStream_t s) {
    k_split_bf16<<<2048, 256, 0, s>>>(batch, rows, cols, A, lda, hi, lo);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free Gram (mpf_gram_split_bf16_noalloc).
//
// Some callers of this library cannot allocate device memory once they are
// running: applications that size all GPU memory at start-up (a real-time
// reconstruction loop that must not stall on cudaMalloc's implicit device
// synchronisation, or a host framework whose own allocator owns the whole
// device and forbids allocations from libraries).  For them the split-BF16
// Gram has a variant whose scratch memory -- the BF16 hi/lo copies of A, the
// split-K partial sums and the pipeline abort flag -- lives in the fixed
// file-scope arrays below instead of buffers allocated per call.
//
// Limits: batch * rows * lda <= kNoAllocElems (2,097,152 elements) and the
// split-K workspace <= kNoAllocWork floats (1,048,576), i.e. 12 MB of device
// memory that every GPU loading this library keeps until the process exits.
// All calls share these arrays, which keep the contents of the last call:
// each call rewrites the parts it reads (the abort flag is cleared at the
// start of every call), and two calls that overlap on the GPU (different
// streams, no ordering between them) race on the arrays and corrupt each
// other's results.  The first call on a device resolves the arrays' device
// addresses (cudaGetSymbolAddress).  Every call copies the abort flag to the
// host and synchronises the stream, so no call can be stream-captured.
namespace {
constexpr size_t kNoAllocElems = size_t(1) << 21;
constexpr size_t kNoAllocWork = size_t(1) << 20;
static __device__ __align__(256) __nv_bfloat16 g_noallocHi[kNoAllocElems];
static __device__ __align__(256) __nv_bfloat16 g_noallocLo[kNoAllocElems];
static __device__ __align__(256) float g_noallocWork[kNoAllocWork];
static __device__ __align__(256) int g_noallocFlag[64];

struct NoAllocScratch {
    __nv_bfloat16* hi = nullptr;
    __nv_bfloat16* lo = nullptr;
    float* work = nullptr;
    int* flag = nullptr;
    bool ready = false;
};

// Device addresses of the scratch arrays, resolved once per device with that
// device current (the host-side names are stand-ins, not device addresses).
int noalloc_scratch(NoAllocScratch* out) {
    static std::mutex mu;
    static NoAllocScratch perDevice[64];
    int dev = 0;
    MPF_CUDA(cudaGetDevice(&dev));
    MPF_CHECK(dev >= 0 && dev < 64, MPF_EINVAL, "gram (no-alloc): device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    NoAllocScratch& s = perDevice[dev];
    if (!s.ready) {
        MPF_CUDA(cudaGetSymbolAddress((void**)&s.hi, g_noallocHi));
        MPF_CUDA(cudaGetSymbolAddress((void**)&s.lo, g_noallocLo));
        MPF_CUDA(cudaGetSymbolAddress((void**)&s.work, g_noallocWork));
        MPF_CUDA(cudaGetSymbolAddress((void**)&s.flag, g_noallocFlag));
        s.ready = true;
    }
    *out = s;
    return MPF_OK;
}
}  // namespace

int dense_gram_split_bf16_noalloc(int batch, int rows, int cols, const float* A, int lda, float* C, cudaStream_t s) {
    MPF_CHECK(batch >= 1 && rows % kTile == 0 && cols % kBK == 0 && lda % 8 == 0 && lda >= cols, MPF_EINVAL,
              "mpf_gram_split_bf16_noalloc: rows %% 128, cols %% 64 and lda %% 8 must be 0 (rows=%d cols=%d lda=%d)",
              rows, cols, lda);
    const size_t elems = (size_t)batch * rows * lda;
    MPF_CHECK(elems <= kNoAllocElems, MPF_EINVAL,
              "mpf_gram_split_bf16_noalloc: batch*rows*lda = %zu exceeds the fixed scratch of %zu elements", elems,
              kNoAllocElems);
    const size_t work = dense_gram_work_floats(batch, rows, cols);
    MPF_CHECK(work <= kNoAllocWork, MPF_EINVAL,
              "mpf_gram_split_bf16_noalloc: split-K workspace of %zu floats exceeds the fixed scratch of %zu floats",
              work, kNoAllocWork);
    NoAllocScratch sc;
    MPF_TRY(noalloc_scratch(&sc));
    MPF_CUDA(cudaMemsetAsync(sc.flag, 0, sizeof(int), s));
    MPF_TRY(dense_split_bf16(batch, rows, cols, A, lda, sc.hi, sc.lo, s));
    MPF_TRY(gram_run(batch, rows, cols, sc.hi, sc.lo, lda, C, nullptr, 0.0, sc.work, kNoAllocWork, s, sc.flag));
    int aborted = 0;
    MPF_CUDA(cudaMemcpyAsync(&aborted, sc.flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    MPF_CHECK(!aborted, MPF_ETIMEOUT, "mpf_gram_split_bf16_noalloc: a pipeline wait timed out");
    return MPF_OK;
}

int dense_cholesky_f64(int batch, int n, double* A, int* info, cudaStream_t s, const int* frameMask) {
    MPF_CHECK(n % NB == 0, MPF_EINVAL, "cholesky: n must be a multiple of %d (got %d)", NB, n);
    MPF_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * batch, s));
    const int nb = n / NB;
    for (int k = 0; k < nb; ++k) {
        k_potrf_diag<<<batch, 256, 0, s>>>(n, A, k, info, frameMask);
        const int m = nb - k - 1;
        if (m > 0) {
            k_trsm<<<dim3(m, batch), 64, 0, s>>>(n, A, k, frameMask);
            k_syrk<<<dim3(m * (m + 1) / 2, batch), 256, 0, s>>>(n, A, k, frameMask);
        }
    }
    MPF_LAUNCHED(3 * nb - 2);
    return MPF_OK;
}

int dense_cholesky_solve_f64(int batch, int n, const double* L, double* B, int nrhs, cudaStream_t s,
                             const int* frameMask) {
    const size_t bytes = (size_t)n * sizeof(double);
    MPF_CHECK(bytes <= 192 * 1024 && n % NB == 0, MPF_EINVAL,
              "cholesky solve: n must be a multiple of %d and at most 24576 (%d)", NB, n);
    if (bytes > 38 * 1024)
        MPF_CUDA(cudaFuncSetAttribute(k_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    // one thread per row (up to 1024): the row updates below each diagonal
    // block are latency-bound loads of L, so more threads keep more in flight
    const int threads = std::min(1024, std::max(256, n));
    k_chol_solve<<<batch * nrhs, threads, bytes, s>>>(n, L, B, nrhs, frameMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_potrf32(int batch, int n, const double* A, double* L, int* info, cudaStream_t s, const int* frameMask) {
    MPF_CHECK(n % NB == 0 && n >= NB && n <= 1536, MPF_EINVAL,
              "FP32 Cholesky: n must be a multiple of %d in [32, 1536] (got %d)", NB, n);
    // the panel plus about 8 KB of static shared memory: opt in whenever the
    // sum may pass the 48 KB default
    const size_t smem = (size_t)n * kPanelStride * sizeof(float);
    MPF_CUDA(cudaFuncSetAttribute(k_potrf32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MPF_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * batch, s));
    // large matrices in small batches: a cluster of up to 4 CTAs per matrix
    // so that the batch spreads over the SMs
    int dev = 0, sms = 0;
    MPF_CUDA(cudaGetDevice(&dev));
    MPF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int CL = 1;
    if (n >= 512)
        while (CL < 4 && (long)batch * CL * 2 <= sms) CL *= 2;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(batch * CL));
    cfg.blockDim = dim3(kPotrfThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MPF_CUDA(cudaLaunchKernelEx(&cfg, k_potrf32, n, A, L, info, frameMask));
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_mirror_lower(int batch, int n, double* A, cudaStream_t s, const int* frameMask) {
    MPF_CHECK(n % 32 == 0, MPF_EINVAL, "mirror: n must be a multiple of 32 (got %d)", n);
    k_mirror_lower<<<dim3(n / 32, n / 32, batch), 256, 0, s>>>(n, A, frameMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_sym_residual(int batch, int n, const double* A, const double* x, const double* y, double* r, double* rr,
                       double* yy, cudaStream_t s, const int* frameMask) {
    MPF_CHECK(n % 32 == 0, MPF_EINVAL, "FP64 residual: n must be a multiple of 32 (got %d)", n);
    k_sym_residual<<<dim3(n / 32, batch), 256, 0, s>>>(n, A, x, y, r, rr, yy, frameMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_add_masked(int batch, int n, double* x, const double* d, cudaStream_t s, const int* frameMask) {
    k_add_masked<<<std::min(1024, (n * batch + 255) / 256), 256, 0, s>>>(n, batch, x, d, frameMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_trtri32(int batch, int n, const double* L, float* L32, float* D, float* X, float* XT, cudaStream_t s,
                  const int* frameMask) {
    MPF_CHECK(n % NB == 0 && n >= NB && n <= 1280, MPF_EINVAL,
              "FP32 triangular inverse: n must be a multiple of %d in [32, 1280] (got %d)", NB, n);
    const int nb = n / NB;
    const size_t per = (size_t)n * n;
    k_to_f32<<<(int)std::min<size_t>((per * batch + 255) / 256, 152 * 16), 256, 0, s>>>(per * batch, L, L32,
                                                                                      frameMask, per);
    k_trtri_diag<<<dim3(nb, batch), 32, 0, s>>>(n, L, D, frameMask);
    const size_t smem = (size_t)nb * NB * NB * sizeof(float);
    MPF_CUDA(cudaFuncSetAttribute(k_trtri_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_trtri_cols<<<dim3(nb, batch), 256, smem, s>>>(n, L32, D, X, XT, frameMask);
    MPF_LAUNCHED(3);
    return MPF_OK;
}

int dense_tri_rows(int batch, int n, const float* M, const double* v, double* out, bool upper, cudaStream_t s,
                   const int* frameMask) {
    k_tri_rows<<<dim3((n + 7) / 8, batch), 256, 0, s>>>(n, M, v, out, upper ? 1 : 0, frameMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int dense_add_shift(int batch, int n, double* A, double shift, cudaStream_t s) {
    k_add_shift<<<dim3((n + 255) / 256, batch), 256, 0, s>>>(n, A, shift);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

}  // namespace mpf
