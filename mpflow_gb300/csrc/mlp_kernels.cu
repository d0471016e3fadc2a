// Learned Gauss-Newton warm start: a multilayer perceptron
//   x (in) -> GELU(W1 x + b1) (h1) -> GELU(W2 . + b2) (h2) -> W3 . + b3 (out)
// trained and evaluated with hand-written kernels.  No reference counterpart.
//
//  * k_gemm_nt  D[M][N] = sum_k A[M][k] B[N][k] with BF16 operands (both
//               K-major) on the tcgen05 tensor cores: TMA 128-byte-swizzled
//               tiles -> 3-stage mbarrier pipeline -> tcgen05.mma (FP32
//               accumulator in tensor memory) -> tcgen05.ld epilogue.  Two
//               CTAs fit on an SM, so one CTA's epilogue overlaps the other's
//               main loop.  The K range may be split over CTAs (FP32
//               partials, summed by the consumer kernel in a fixed order).
//  * k_act      sums the split partials, adds the bias and applies the
//               activation (or its derivative), writing FP32 and BF16 copies
//               in row-major and transposed layout as the next GEMMs need
//               them (every GEMM operand is K-major); the backward form also
//               writes per-32-row column sums (the bias gradient's partials).
//  * k_loss_head  the output layer of a training step: y = partials + b3
//               against the target rows (optionally gathered by index), the
//               loss partials, dY = 2 (y - t) / (batch valid) as BF16 in both
//               layouts and its per-32-row column sums, without writing y.
//  * k_bias_grad  the three bias gradients from the column-sum partials.
//  * k_adam_flat, k_adam_wt  Adam with FP32 master weights; the second, for
//               W2 and W3, also writes the BF16 copy's transpose (the operand
//               of the backward GEMMs) from the same 32 x 32 tile.
//  * k_to_bf16, k_transpose_bf16, k_init_uniform: BF16 working copies on
//               weight changes from the host side, seeded initialisation.
// Parameters live in one flat FP32 array W1 | b1 | W2 | b2 | W3 | b3 (each
// segment 64-element aligned); gradients, Adam moments and the BF16 copies
// use the same offsets.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "model.h"
#include "tc_ptx.cuh"

namespace mpf {
namespace {

using namespace tc;

constexpr int kStages = 3;
constexpr int kStageBytes = 2 * kTileBytes;  // A tile + B tile
constexpr int kGemmSmem = kStages * kStageBytes + 1024 /*align*/ + 256 /*barriers*/;
static_assert(kStages * kStageBytes >= kTile * kTile * 6,
              "the epilogues stage the FP32 tile (and the Adam form a BF16 transposed tile) in the stage buffers");

struct GemmArgs {
    int kblocks;        // K / 64
    int splits;         // K splits (grid z)
    float* out;         // out + split * splitStride + m * ldOut + n
    int ldOut;
    size_t splitStride;
    int* abortFlag;
    // ADAM form (weight gradient of a decayed M x N weight matrix, one
    // split): the epilogue applies Adam to w / m / v (ld ldOut) instead of
    // writing the gradient, and writes the BF16 copy wb (ld ldOut) and its
    // transpose wt (N x M, ld ldT)
    float* w;
    float* m;
    float* v;
    __nv_bfloat16* wb;
    __nv_bfloat16* wt;
    int ldT;
    // AXPBY form (one split): out = alpha D + beta out + add on rows <
    // rowsValid and columns < colsValid
    float alpha, beta, add;
    int rowsValid, colsValid;
};

struct AdamArgs {
    float lr, b1, b2, eps, wd, bc1, bc2;
};

// One Adam step of one parameter (decoupled weight decay when `decay`).
// Every rounding is spelled out (no contraction left to the compiler), so
// the fused GEMM epilogue and the standalone kernels give the same bits.
__device__ __forceinline__ float adam_one(float wi, float gi, float& m, float& v, bool decay, const AdamArgs& a) {
    const float mi = fmaf(a.b1, m, __fmul_rn(1.f - a.b1, gi));
    const float vi = fmaf(a.b2, v, __fmul_rn(__fmul_rn(1.f - a.b2, gi), gi));
    m = mi;
    v = vi;
    if (decay) wi = fmaf(-__fmul_rn(a.lr, a.wd), wi, wi);
    const float step = __fdiv_rn(__fmul_rn(a.lr, __fdiv_rn(mi, a.bc1)), __fadd_rn(sqrtf(__fdiv_rn(vi, a.bc2)), a.eps));
    return __fsub_rn(wi, step);
}


// One CTA = one 128x128 output tile and one K split.  Warp 0 lane 0 issues
// the TMA loads, warp 1 lane 0 the MMAs; every warp drains TMEM (four warps,
// or eight in the Adam form).
enum GemmMode { kGemmStore = 0, kGemmAdam = 1, kGemmAxpby = 2 };

template <int MODE>
__global__ void __launch_bounds__(MODE == kGemmAdam ? 256 : 128, 2) k_gemm_nt(const __grid_constant__ CUtensorMap mapA,
                                                    const __grid_constant__ CUtensorMap mapB, GemmArgs ga,
                                                    AdamArgs adam) {
    constexpr bool ADAM = MODE == kGemmAdam;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + kStages * kStageBytes);
    __shared__ uint32_t tmemBase;
    __shared__ int localAbort;
    __shared__ int issuedLoads;  // K blocks whose TMA loads the producer issued

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Plain form: row tiles fastest, so CTAs that share a B tile (the larger
    // operand of the output layer's products) run back to back and find it
    // in L2.  Adam form: column tiles fastest, so consecutive CTAs update
    // adjacent 512-byte pieces of the same 128 weight rows.
    const int tm = ADAM ? blockIdx.y : blockIdx.x, tn = ADAM ? blockIdx.x : blockIdx.y, split = blockIdx.z;
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
    if (warp == 1) tmem_alloc(smem_u32(&tmemBase), 128);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmemBase;
    volatile int* abortFlag = &localAbort;
    const uint32_t smemBase = smem_u32(smem);

    if (warp == 0 && lane == 0) {
        for (int i = 0; i < nk; ++i) {
            const int s = i % kStages, round = i / kStages;
            if (round > 0 && !mbar_wait(emptyBar + 8 * s, (round - 1) & 1, abortFlag)) break;
            const uint32_t st = smemBase + s * kStageBytes;
            mbar_expect_tx(fullBar + 8 * s, kStageBytes);
            const int x = (kb0 + i) * kBK;
            tma_load_2d(st, &mapA, fullBar + 8 * s, x, tm * kTile);
            tma_load_2d(st + kTileBytes, &mapB, fullBar + 8 * s, x, tn * kTile);
            issuedLoads = i + 1;
        }
    } else if (warp == 1 && lane == 0) {
        for (int i = 0; i < nk; ++i) {
            const int s = i % kStages, round = i / kStages;
            if (!mbar_wait(fullBar + 8 * s, round & 1, abortFlag)) break;
            fence_after();
            const uint32_t st = smemBase + s * kStageBytes;
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk)
                mma_bf16(tmem, sw128_desc(st + kk * 32), sw128_desc(st + kTileBytes + kk * 32),
                         (i > 0 || kk > 0) ? 1u : 0u);
            mma_commit(emptyBar + 8 * s);
        }
        mma_commit(doneBar);
    }
    __syncwarp();
    const bool waited = nk > 0 && mbar_wait(doneBar, 0, abortFlag);
    const bool ok = __all_sync(0xffffffffu, waited && !*abortFlag);
    fence_after();
    const bool allOk = __syncthreads_and(ok);
    float* tileOut = ga.out + split * ga.splitStride + (size_t)(tm * kTile) * ga.ldOut + tn * kTile;
    if (ADAM && allOk) {
        // Adam on the weight tile, 8 warps.  Every MMA has completed (doneBar),
        // so the stage buffers are free.  Warp w drains TMEM lanes 32 (w % 4)
        // .. + 31 (its rows), columns 64 (w / 4) .. + 63, into an FP32 tile in
        // shared memory (16-byte chunks XOR-swizzled by row), then updates the
        // same rows and columns two rows at a time with lane-consecutive
        // columns (128-byte coalesced loads and stores of w, m, v; all loads of
        // two row pairs issued before the first store), writes the BF16 copy,
        // and puts the new BF16 values into a transposed tile (4-byte words of
        // two rows, word index XOR-swizzled by column, conflict-free).  After
        // a CTA barrier every warp writes 16 rows of the transposed copy, 128
        // bytes per instruction.
        const int quarter = warp & 3, half = warp >> 2;
        float* gTile = reinterpret_cast<float*>(smem);                            // [128][128] FP32, 64 KB
        uint32_t* wTile = reinterpret_cast<uint32_t*>(smem + kTile * kTile * 4);  // [128][64] words, 32 KB
        const int r = quarter * 32 + lane;
#pragma unroll 1
        for (int c = half * 64; c < half * 64 + 64; c += 32) {
            float gv[32];
            tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, gv);
#pragma unroll
            for (int k = 0; k < 32; k += 4) {
                const int chunk = ((c + k) >> 2) ^ (r & 7);
                *reinterpret_cast<float4*>(gTile + r * kTile + chunk * 4) =
                    make_float4(gv[k], gv[k + 1], gv[k + 2], gv[k + 3]);
            }
        }
        __syncwarp();
        const size_t base = (size_t)(tm * kTile) * ga.ldOut + tn * kTile;
#pragma unroll 1
        for (int p = 0; p < 16; p += 2) {
            // rows quarter*32 + 2p .. + 3 (two pairs), columns half*64 + lane + 32 q
            float wv[4][2], mv[4][2], vv[4][2];
#pragma unroll
            for (int e = 0; e < 4; ++e)
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const size_t at = base + (size_t)(quarter * 32 + 2 * p + e) * ga.ldOut + half * 64 + lane + 32 * q;
                    wv[e][q] = ga.w[at];
                    mv[e][q] = ga.m[at];
                    vv[e][q] = ga.v[at];
                }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int jl = half * 64 + lane + 32 * q;
                float nw[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int il = quarter * 32 + 2 * p + e;
                    const float g = gTile[il * kTile + (((jl >> 2) ^ (il & 7)) << 2) + (jl & 3)];
                    nw[e] = adam_one(wv[e][q], g, mv[e][q], vv[e][q], true, adam);
                    const size_t at = base + (size_t)il * ga.ldOut + jl;
                    ga.w[at] = nw[e];
                    ga.m[at] = mv[e][q];
                    ga.v[at] = vv[e][q];
                    ga.wb[at] = __float2bfloat16_rn(nw[e]);
                }
#pragma unroll
                for (int e = 0; e < 4; e += 2) {
                    const int wi = (quarter * 32 + 2 * p + e) >> 1;  // word: rows 2 wi, 2 wi + 1
                    __nv_bfloat162 pr = __floats2bfloat162_rn(nw[e], nw[e + 1]);
                    wTile[jl * 64 + (wi ^ (jl & 31))] = *reinterpret_cast<uint32_t*>(&pr);
                }
            }
        }
        __syncthreads();
        // transposed copy: rows tn*128 + jl of wt, columns tm*128 .. + 127
#pragma unroll 2
        for (int k = 0; k < 16; ++k) {
            const int jl = warp * 16 + k;
            uint32_t* dst = reinterpret_cast<uint32_t*>(ga.wt + (size_t)(tn * kTile + jl) * ga.ldT + tm * kTile);
            dst[lane] = wTile[jl * 64 + (lane ^ (jl & 31))];
            dst[lane + 32] = wTile[jl * 64 + ((lane + 32) ^ (jl & 31))];
        }
    } else if (!ADAM && ok) {
        // Every MMA has completed (doneBar), so the stage buffers are free:
        // each warp moves its 32 accumulator rows TMEM -> registers -> shared
        // memory (16-byte chunks XOR-swizzled by row, conflict-free), then
        // writes them out one 512-byte row per instruction (the AXPBY form
        // reads the old row and writes alpha D + beta out + add in bounds).
        float* stage = reinterpret_cast<float*>(smem) + warp * 32 * kTile;
#pragma unroll 1
        for (int c = 0; c < kTile; c += 32) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int i = 0; i < 32; i += 4) {
                const int chunk = ((c + i) >> 2) ^ (lane & 7);
                *reinterpret_cast<float4*>(stage + lane * kTile + chunk * 4) =
                    make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            }
        }
        __syncwarp();
        if (MODE == kGemmStore) {
#pragma unroll 4
            for (int r = 0; r < 32; ++r) {
                const int chunk = lane ^ (r & 7);
                *reinterpret_cast<float4*>(tileOut + (size_t)(warp * 32 + r) * ga.ldOut + lane * 4) =
                    *reinterpret_cast<const float4*>(stage + r * kTile + chunk * 4);
            }
        } else {
            const int c0 = tn * kTile + lane * 4;
#pragma unroll 2
            for (int r = 0; r < 32; ++r) {
                const int gr = tm * kTile + warp * 32 + r;
                if (gr >= ga.rowsValid) break;
                const float4 d = *reinterpret_cast<const float4*>(stage + r * kTile + ((lane ^ (r & 7)) * 4));
                const float dv[4] = {d.x, d.y, d.z, d.w};
                float* o = tileOut + (size_t)(warp * 32 + r) * ga.ldOut + lane * 4;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (c0 + k < ga.colsValid)
                        o[k] = ga.beta != 0.f ? fmaf(ga.alpha, dv[k], fmaf(ga.beta, o[k], ga.add))
                                              : fmaf(ga.alpha, dv[k], ga.add);
            }
        }
    } else if (MODE == kGemmStore) {
        float* out = tileOut + (size_t)(warp * 32 + lane) * ga.ldOut;
        for (int c = 0; c < kTile; ++c) out[c] = 0.f;
    }
    if (!allOk && threadIdx.x == 0 && nk > 0) atomicExch(ga.abortFlag, 1);
    fence_before();
    __syncthreads();
    if (!allOk && nk > 0) {
        // A wait gave up: before TMEM is released and the CTA exits, wait with
        // the same limit (on a flag of its own) for the MMA issuer's final
        // commit, which covers every MMA it issued, and for the last load
        // issued into each stage (a stage's round r is issued only after round
        // r - 1 was consumed, so the parity of round r names that round).  TMEM
        // is released even if these waits give up: a CTA that exits holding
        // TMEM would block every later allocation on its SM.  The output of a
        // launch that raised the abort flag is undefined (MPF_ETIMEOUT); the
        // Adam form leaves its parameters untouched then.
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

// ---------------------------------------------------------------------------
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678f)); }
__device__ __forceinline__ float gelu_deriv(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678f)) + z * 0.39894228f * expf(-0.5f * z * z);
}

enum ActMode { kGeluFwd = 0, kLinear = 1, kGeluBwd = 2, kCast = 3 };

struct ActArgs {
    int B, N;              // rows (batch, padded) x columns
    int Bvalid;            // rows >= Bvalid are written as zeros
    int splits;
    const float* part;     // [splits][B][N] (ld N), or the FP32 input of kCast (ld ldIn)
    int ldIn;
    size_t splitStride;
    const float* bias;     // [N] or null
    const float* Zin;      // kGeluBwd: pre-activation [B][N]
    float* Zout;           // kGeluFwd: pre-activation; kLinear / kGeluBwd: FP32 result (ld ldOut)
    int ldOut;
    __nv_bfloat16* H;      // [B][N] BF16 result, or null
    __nv_bfloat16* HT;     // [N][B] BF16 result transposed, or null
    const int* rows;       // kCast: input row of each batch row (gather), or null
    float* colPart;        // kGeluBwd: [B / 32][N] column sums of the result per 32-row tile, or null
};

// One block = one 32x32 tile (32 x 8 threads); the transposed copy goes
// through shared memory so both writes are coalesced.
template <int MODE>
__global__ void __launch_bounds__(256) k_act(ActArgs a) {
    __shared__ float tile[32][33];
    const int n0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int n = n0 + tx;
    // every load of the thread's four rows is issued before the first store
    float v[4] = {0.f, 0.f, 0.f, 0.f}, z[4] = {0.f, 0.f, 0.f, 0.f};
    if (MODE == kCast) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int b = b0 + ty + 8 * k;
            if (b < a.Bvalid) v[k] = a.part[(size_t)(a.rows ? a.rows[b] : b) * a.ldIn + n];
        }
    } else {
#pragma unroll 4
        for (int s = 0; s < a.splits; ++s)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int b = b0 + ty + 8 * k;
                if (b < a.Bvalid) v[k] += a.part[s * a.splitStride + (size_t)b * a.N + n];
            }
        if (MODE == kGeluBwd)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int b = b0 + ty + 8 * k;
                if (b < a.Bvalid) z[k] = a.Zin[(size_t)b * a.N + n];
            }
        const float bias = a.bias ? a.bias[n] : 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (a.bias && b0 + ty + 8 * k < a.Bvalid) v[k] += bias;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int r = ty + 8 * k, b = b0 + r;
        float h = v[k];
        if (MODE == kGeluFwd) {
            if (a.Zout) a.Zout[(size_t)b * a.N + n] = v[k];
            h = b < a.Bvalid ? gelu(v[k]) : 0.f;
        } else if (MODE == kGeluBwd) {
            h = b < a.Bvalid ? v[k] * gelu_deriv(z[k]) : 0.f;
            if (a.Zout) a.Zout[(size_t)b * a.ldOut + n] = h;
        } else if (MODE == kLinear) {
            if (a.Zout && b < a.Bvalid) a.Zout[(size_t)b * a.ldOut + n] = v[k];
        }
        if (a.H) a.H[(size_t)b * a.N + n] = __float2bfloat16_rn(h);
        tile[r][tx] = h;
    }
    if (!a.HT && !a.colPart) return;
    __syncthreads();
    if (a.HT)
        for (int r = ty; r < 32; r += 8) a.HT[(size_t)(n0 + r) * a.B + b0 + tx] = __float2bfloat16_rn(tile[tx][r]);
    if (a.colPart && ty == 0) {
        float c = 0.f;
        for (int r = 0; r < 32; ++r) c += tile[r][tx];
        a.colPart[(size_t)blockIdx.y * a.N + n0 + tx] = c;
    }
}

struct HeadArgs {
    int B, N;              // rows (batch, padded) x outputs
    int Bvalid, Nvalid;    // rows >= Bvalid and columns >= Nvalid give d = 0
    int splits;
    const float* part;     // [splits][B][N] GEMM partials
    size_t splitStride;
    const float* bias;     // [N]
    const float* T;        // targets, row rows[b] (or b) with leading dimension ldT
    int ldT;
    const int* rows;       // gather of the target rows, or null
    float scale;           // 2 / (Bvalid Nvalid)
    __nv_bfloat16* dY;     // [B][N]
    __nv_bfloat16* dYT;    // [N][B]
    float* colPart;        // [B / 32][N] column sums of dY per 32-row tile
    double* lossPart;      // [gridDim.y][gridDim.x] sums of d^2
};

// Output layer of a training step, one 32-column x 128-row tile per block
// (32 x 8 threads): y = sum of the partials + b3 (never stored), d = y - t on
// the valid entries, dY = scale d in BF16 row-major and transposed (the A
// operands of the dW3 and dH2 products), the column sums of dY per 32-row
// tile and the block's sum of d^2.
__global__ void __launch_bounds__(256) k_loss_head(HeadArgs a) {
    __shared__ float tile[4][32][33];
    __shared__ double red[8];
    const int n0 = blockIdx.x * 32, b0 = blockIdx.y * 128;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int n = n0 + tx;
    const float bias = a.bias[n];
    const float scale = a.scale;
    // FP32 arithmetic per element (the FP64 pipe is narrow on this part):
    // each thread's 16 squares are summed in FP32, the block in FP64.  Every
    // load of the thread's 16 rows is issued before the first store.
    float y[16], t[16];
    int src[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int b = b0 + ty + 8 * k;
        y[k] = 0.f;
        src[k] = (b < a.Bvalid && n < a.Nvalid) ? (a.rows ? a.rows[b] : b) : -1;
    }
    for (int s = 0; s < a.splits; ++s)
#pragma unroll
        for (int k = 0; k < 16; ++k) y[k] += a.part[s * a.splitStride + (size_t)(b0 + ty + 8 * k) * a.N + n];
#pragma unroll
    for (int k = 0; k < 16; ++k) t[k] = src[k] >= 0 ? a.T[(size_t)src[k] * a.ldT + n] : 0.f;
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int r = ty + 8 * k;
        const float d = src[k] >= 0 ? (y[k] + bias) - t[k] : 0.f;
        acc = fmaf(d, d, acc);
        const float dy = scale * d;
        a.dY[(size_t)(b0 + r) * a.N + n] = __float2bfloat16_rn(dy);
        tile[r >> 5][r & 31][tx] = dy;
    }
    double wsum = (double)acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
    if (tx == 0) red[ty] = wsum;
    __syncthreads();
#pragma unroll
    for (int tt = 0; tt < 4; ++tt)
        for (int r = ty; r < 32; r += 8)
            a.dYT[(size_t)(n0 + r) * a.B + b0 + 32 * tt + tx] = __float2bfloat16_rn(tile[tt][tx][r]);
    if (ty < 4) {
        float c = 0.f;
        for (int r = 0; r < 32; ++r) c += tile[ty][r][tx];
        a.colPart[(size_t)(blockIdx.y * 4 + ty) * a.N + n] = c;
    }
    if (threadIdx.x == 0) {
        double l = 0.0;
        for (int w = 0; w < 8; ++w) l += red[w];
        a.lossPart[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = l;
    }
}

// Bias gradients g[off_l + j] = sum_t colPart_l[t][j] over the 32-row tiles
// in order, for the three layers at once (columns of layer 0 first).
struct BiasArgs {
    int N[3];
    const float* part[3];
    float* g[3];
    int tiles;
};
__global__ void k_bias_grad(BiasArgs a) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int l = 0; l < 3; ++l) {
        if (j < a.N[l]) {
            float c = 0.f;
            for (int t = 0; t < a.tiles; ++t) c += a.part[l][(size_t)t * a.N[l] + j];
            a.g[l][j] = c;
            return;
        }
        j -= a.N[l];
    }
}

// Adam over a flat range of `count4` groups of four parameters (the range
// starts on a 64-element segment boundary; decay per segment).
__global__ void __launch_bounds__(256) k_adam_flat(size_t count4, float4* __restrict__ w, const float4* __restrict__ g,
                                                   float4* __restrict__ m, float4* __restrict__ v,
                                                   __nv_bfloat162* __restrict__ wb, const uint8_t* __restrict__ decay,
                                                   AdamArgs a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count4; i += (size_t)gridDim.x * blockDim.x) {
        float4 wi = w[i], mi = m[i], vi = v[i];
        const float4 gi = g[i];
        const bool dec = decay[i >> 4] != 0;
        wi.x = adam_one(wi.x, gi.x, mi.x, vi.x, dec, a);
        wi.y = adam_one(wi.y, gi.y, mi.y, vi.y, dec, a);
        wi.z = adam_one(wi.z, gi.z, mi.z, vi.z, dec, a);
        wi.w = adam_one(wi.w, gi.w, mi.w, vi.w, dec, a);
        w[i] = wi;
        m[i] = mi;
        v[i] = vi;
        wb[2 * i] = __floats2bfloat162_rn(wi.x, wi.y);
        wb[2 * i + 1] = __floats2bfloat162_rn(wi.z, wi.w);
    }
}

// Adam on a weight matrix W [R][C] (row-major, decayed; R, C multiples of
// 32) that also writes the BF16 copy and its transpose WT [C][R]: one 32 x 32
// tile per block, the transpose through shared memory so both BF16 writes
// are coalesced.  Each thread loads its four rows before updating them.
__global__ void __launch_bounds__(256) k_adam_wt(int R, int C, float* __restrict__ w, const float* __restrict__ g,
                                                 float* __restrict__ m, float* __restrict__ v,
                                                 __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wt,
                                                 AdamArgs a) {
    __shared__ float tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    float wi[4], gi[4], mi[4], vi[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t idx = (size_t)(r0 + ty + 8 * k) * C + c0 + tx;
        wi[k] = w[idx];
        gi[k] = g[idx];
        mi[k] = m[idx];
        vi[k] = v[idx];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t idx = (size_t)(r0 + ty + 8 * k) * C + c0 + tx;
        const float nw = adam_one(wi[k], gi[k], mi[k], vi[k], true, a);
        w[idx] = nw;
        m[idx] = mi[k];
        v[idx] = vi[k];
        wb[idx] = __float2bfloat16_rn(nw);
        tile[ty + 8 * k][tx] = nw;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) wt[(size_t)(c0 + ty + 8 * k) * R + r0 + tx] = __float2bfloat16_rn(tile[tx][ty + 8 * k]);
}

__global__ void k_to_bf16(size_t count, const float* __restrict__ w, __nv_bfloat16* __restrict__ wb) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        wb[i] = __float2bfloat16_rn(w[i]);
}

// dst[c][r] = src[r][c], rows x cols, both multiples of 32
__global__ void __launch_bounds__(256) k_transpose_bf16(int rows, int cols, const __nv_bfloat16* __restrict__ src,
                                                        __nv_bfloat16* __restrict__ dst) {
    __shared__ __nv_bfloat16 tile[32][34];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) tile[r][tx] = src[(size_t)(r0 + r) * cols + c0 + tx];
    __syncthreads();
    for (int r = ty; r < 32; r += 8) dst[(size_t)(c0 + r) * rows + r0 + tx] = tile[tx][r];
}

// Uniform(-scale, scale) from a counter-based hash (SplitMix64 finaliser).
__global__ void k_init_uniform(size_t count, float* __restrict__ w, float scale, unsigned long long seed) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        unsigned long long z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const float u = (float)(z >> 40) * (1.f / 16777216.f);  // [0, 1)
        w[i] = scale * (2.f * u - 1.f);
    }
}

// K splits of a GEMM with `tiles` output tiles: as many as fill one wave of
// `slots` CTAs (two per SM) without starting a second, at least 4 K blocks
// per split, at most 16.
int gemm_splits(int tiles, int kblocks, int slots) {
    int s = slots / tiles;
    s = std::min(s, std::max(1, kblocks / 4));
    return std::max(1, std::min(s, 16));
}

}  // namespace
}  // namespace mpf

// ---------------------------------------------------------------------------
struct mpf_mlp {
    int in = 0, h1 = 0, h2 = 0, out = 0, device = 0;
    size_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0, P = 0;
    mpf::DevBuf<float> w, g, m, v;
    mpf::DevBuf<__nv_bfloat16> wb, W2T, W3T;
    mpf::DevBuf<uint8_t> decay;  // per 64-element segment: 1 for weights, 0 for biases
    long long step = 0;
    int slots = 0;  // GEMM CTAs in one wave (two per SM)
    // activations, grown with the batch
    int capB = 0;
    mpf::DevBuf<__nv_bfloat16> X, XT, H1, H1T, H2, H2T, dYb, dYT, dZ2, dZ2T, dZ1T;
    mpf::DevBuf<float> Z1, Z2, Y, part, colPart1, colPart2, colPart3;
    mpf::DevBuf<double> lossPart;
    std::vector<double> lossHost;
    mpf::DevBuf<int> flag;
};

namespace mpf {

int mlp_refresh(mpf_mlp* n, cudaStream_t s);

static int mlp_workspace(mpf_mlp* n, int B) {
    if (B <= n->capB) return MPF_OK;
    const size_t in = n->in, h1 = n->h1, h2 = n->h2, out = n->out;
    MPF_TRY(n->X.alloc(B * in));
    MPF_TRY(n->XT.alloc(B * in));
    MPF_TRY(n->H1.alloc(B * h1));
    MPF_TRY(n->H1T.alloc(B * h1));
    MPF_TRY(n->H2.alloc(B * h2));
    MPF_TRY(n->H2T.alloc(B * h2));
    MPF_TRY(n->dYb.alloc(B * out));
    MPF_TRY(n->dYT.alloc(B * out));
    MPF_TRY(n->dZ2.alloc(B * h2));
    MPF_TRY(n->dZ2T.alloc(B * h2));
    MPF_TRY(n->dZ1T.alloc(B * h1));
    MPF_TRY(n->Z1.alloc(B * h1));
    MPF_TRY(n->Z2.alloc(B * h2));
    MPF_TRY(n->Y.alloc(B * out));
    MPF_TRY(n->colPart1.alloc(B / 32 * h1));
    MPF_TRY(n->colPart2.alloc(B / 32 * h2));
    MPF_TRY(n->colPart3.alloc(B / 32 * out));
    MPF_TRY(n->lossPart.alloc(B / 32 * (out / 32)));
    n->lossHost.resize(B / 32 * (out / 32));
    // GEMM outputs that feed k_act: the unsplit last layer (B x out) or up to
    // 16 K-splits of a hidden-width product
    MPF_TRY(n->part.alloc((size_t)B * std::max(out, 16 * std::max(h1, h2))));
    n->capB = B;
    return MPF_OK;
}

// D = A B^T, A: M x K (ld lda), B: N x K (ld ldb), BF16, K-major.  With one
// split D goes straight to `out` (ld ldOut); otherwise the partials go to the
// network's split buffer and *splitsOut tells the consumer how many.
static int gemm(mpf_mlp* n, const __nv_bfloat16* A, int M, int lda, const __nv_bfloat16* Bm, int N, int ldb, int K,
                float* out, int ldOut, bool allowSplit, int* splitsOut, cudaStream_t s) {
    MPF_CHECK(M % kTile == 0 && N % kTile == 0 && K % kBK == 0 && lda % 8 == 0 && ldb % 8 == 0, MPF_EINVAL,
              "mlp gemm: M, N %% 128 and K %% 64 must be 0 (M=%d N=%d K=%d)", M, N, K);
    CUtensorMap mA, mB;
    MPF_TRY(make_bf16_map(&mA, A, M, lda));
    MPF_TRY(make_bf16_map(&mB, Bm, N, ldb));
    const int kblocks = K / kBK, tiles = (M / kTile) * (N / kTile);
    const int splits = allowSplit ? gemm_splits(tiles, kblocks, n->slots) : 1;
    // per device and cheap: set on every call
    MPF_CUDA(cudaFuncSetAttribute(k_gemm_nt<kGemmStore>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem));
    GemmArgs ga{kblocks, splits, splits > 1 ? n->part.ptr : out, splits > 1 ? N : ldOut, (size_t)M * N,
                n->flag.ptr};
    MPF_CHECK(splits == 1 || (size_t)splits * M * N <= n->part.count, MPF_EINVAL, "mlp gemm: split buffer too small");
    k_gemm_nt<kGemmStore><<<dim3(M / kTile, N / kTile, splits), 128, kGemmSmem, s>>>(mA, mB, ga, AdamArgs{});
    MPF_LAUNCHED(1);
    *splitsOut = splits;
    return MPF_OK;
}

// Weight gradient of the decayed weight matrix at parameter offset `off`
// (M x N, row-major) fused with its Adam step: D = A B^T is never stored;
// the epilogue updates w, m, v there and writes the BF16 copy and its
// transpose wt (N x M).  Same arithmetic as the GEMM into the gradient array
// followed by k_adam_wt.
static int gemm_adam(mpf_mlp* n, const __nv_bfloat16* A, int M, int lda, const __nv_bfloat16* Bm, int N, int ldb,
                     int K, size_t off, __nv_bfloat16* wt, const AdamArgs& adam, cudaStream_t s) {
    MPF_CHECK(M % kTile == 0 && N % kTile == 0 && K % kBK == 0 && lda % 8 == 0 && ldb % 8 == 0, MPF_EINVAL,
              "mlp gemm: M, N %% 128 and K %% 64 must be 0 (M=%d N=%d K=%d)", M, N, K);
    CUtensorMap mA, mB;
    MPF_TRY(make_bf16_map(&mA, A, M, lda));
    MPF_TRY(make_bf16_map(&mB, Bm, N, ldb));
    MPF_CUDA(cudaFuncSetAttribute(k_gemm_nt<kGemmAdam>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem));
    GemmArgs ga{K / kBK, 1, n->g.ptr + off, N, (size_t)M * N, n->flag.ptr};
    ga.w = n->w.ptr + off, ga.m = n->m.ptr + off, ga.v = n->v.ptr + off, ga.wb = n->wb.ptr + off, ga.wt = wt;
    ga.ldT = M;
    k_gemm_nt<kGemmAdam><<<dim3(N / kTile, M / kTile, 1), 256, kGemmSmem, s>>>(mA, mB, ga, adam);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

template <int MODE>
static int act(const ActArgs& a, cudaStream_t s) {
    k_act<MODE><<<dim3(a.N / 32, a.B / 32), 256, 0, s>>>(a);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

static int check_flag(mpf_mlp* n, cudaStream_t s) {
    int h = 0;
    MPF_CUDA(cudaMemcpyAsync(&h, n->flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    if (h) MPF_CUDA(cudaMemset(n->flag.ptr, 0, sizeof(int)));
    MPF_CHECK(!h, MPF_ETIMEOUT, "mlp gemm: a pipeline wait timed out");
    return MPF_OK;
}

int mlp_create(int in, int h1, int h2, int out, unsigned long long seed, int device, mpf_mlp** res) {
    MPF_CHECK(res, MPF_EINVAL, "mpf_mlp_create: out == nullptr");
    MPF_CHECK(in > 0 && h1 > 0 && h2 > 0 && out > 0 && in % 128 == 0 && h1 % 128 == 0 && h2 % 128 == 0 &&
                  out % 128 == 0,
              MPF_EINVAL, "mpf_mlp_create: layer widths must be positive multiples of 128 (%d %d %d %d)", in, h1, h2,
              out);
    MPF_CUDA(cudaSetDevice(device));
    auto n = std::make_unique<mpf_mlp>();
    n->in = in, n->h1 = h1, n->h2 = h2, n->out = out, n->device = device;
    auto seg = [](size_t& at, size_t len) {
        const size_t o = at;
        at += (len + 63) / 64 * 64;
        return o;
    };
    size_t at = 0;
    n->oW1 = seg(at, (size_t)h1 * in);
    n->ob1 = seg(at, h1);
    n->oW2 = seg(at, (size_t)h2 * h1);
    n->ob2 = seg(at, h2);
    n->oW3 = seg(at, (size_t)out * h2);
    n->ob3 = seg(at, out);
    n->P = at;
    MPF_TRY(n->w.alloc(at));
    MPF_TRY(n->g.alloc(at));
    MPF_TRY(n->m.alloc(at));
    MPF_TRY(n->v.alloc(at));
    MPF_TRY(n->wb.alloc(at));
    MPF_TRY(n->W2T.alloc((size_t)h2 * h1));
    MPF_TRY(n->W3T.alloc((size_t)out * h2));
    MPF_TRY(n->flag.alloc(1));
    int sms = 0;
    MPF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    n->slots = 2 * std::max(sms, 1);
    std::vector<uint8_t> dec(at / 64, 0);
    for (size_t i = n->oW1 / 64; i < n->ob1 / 64; ++i) dec[i] = 1;
    for (size_t i = n->oW2 / 64; i < n->ob2 / 64; ++i) dec[i] = 1;
    for (size_t i = n->oW3 / 64; i < n->ob3 / 64; ++i) dec[i] = 1;
    MPF_TRY(n->decay.alloc(dec.size()));
    MPF_CUDA(cudaMemcpy(n->decay.ptr, dec.data(), dec.size(), cudaMemcpyHostToDevice));
    MPF_CUDA(cudaMemset(n->w.ptr, 0, at * sizeof(float)));
    MPF_CUDA(cudaMemset(n->g.ptr, 0, at * sizeof(float)));
    MPF_CUDA(cudaMemset(n->m.ptr, 0, at * sizeof(float)));
    MPF_CUDA(cudaMemset(n->v.ptr, 0, at * sizeof(float)));
    MPF_CUDA(cudaMemset(n->flag.ptr, 0, sizeof(int)));
    // LeCun-uniform weights (variance 1 / fan_in), zero biases
    k_init_uniform<<<1024, 256>>>((size_t)h1 * in, n->w.ptr + n->oW1, std::sqrt(3.f / in), seed * 3 + 1);
    k_init_uniform<<<1024, 256>>>((size_t)h2 * h1, n->w.ptr + n->oW2, std::sqrt(3.f / h1), seed * 3 + 2);
    k_init_uniform<<<1024, 256>>>((size_t)out * h2, n->w.ptr + n->oW3, std::sqrt(3.f / h2), seed * 3 + 3);
    MPF_LAUNCHED(3);
    MPF_TRY(mlp_refresh(n.get(), nullptr));
    MPF_CUDA(cudaDeviceSynchronize());
    *res = n.release();
    return MPF_OK;
}

// BF16 working copies and transposes from the FP32 master weights.
int mlp_refresh(mpf_mlp* n, cudaStream_t s) {
    k_to_bf16<<<2048, 256, 0, s>>>(n->P, n->w.ptr, n->wb.ptr);
    k_transpose_bf16<<<dim3(n->h1 / 32, n->h2 / 32), 256, 0, s>>>(n->h2, n->h1, n->wb.ptr + n->oW2, n->W2T.ptr);
    k_transpose_bf16<<<dim3(n->h2 / 32, n->out / 32), 256, 0, s>>>(n->out, n->h2, n->wb.ptr + n->oW3, n->W3T.ptr);
    MPF_LAUNCHED(3);
    return MPF_OK;
}

void mlp_destroy(mpf_mlp* n) { delete n; }

size_t mlp_param_count(const mpf_mlp* n) { return n->P; }

void mlp_dims(const mpf_mlp* n, int* in, int* out) {
    *in = n->in;
    *out = n->out;
}

void mlp_layout(const mpf_mlp* n, int64_t* off) {
    off[0] = (int64_t)n->oW1, off[1] = (int64_t)n->ob1, off[2] = (int64_t)n->oW2;
    off[3] = (int64_t)n->ob2, off[4] = (int64_t)n->oW3, off[5] = (int64_t)n->ob3, off[6] = (int64_t)n->P;
}

// Forward pass on `batch` rows of x (FP32, ld ldx; row rows[b] for batch
// row b when rows is non-null); Bp = batch rounded up to 128.  Leaves X,
// Z1, H1(T), Z2, H2(T) in the workspace, and Y, unless `training`, when the
// last layer's partials are left for the loss head (*outSplits of them).
static int forward(mpf_mlp* n, int batch, const float* x, int ldx, const int* rows, bool training, int* outSplits,
                   cudaStream_t s) {
    const int Bp = round_up(batch, kTile);
    MPF_TRY(mlp_workspace(n, Bp));
    int sp = 1;
    ActArgs a{};
    a.B = Bp, a.N = n->in, a.Bvalid = batch, a.splits = 1, a.part = x, a.ldIn = ldx, a.rows = rows;
    a.H = n->X.ptr, a.HT = n->XT.ptr;
    MPF_TRY(act<kCast>(a, s));
    // layer 1
    MPF_TRY(gemm(n, n->X.ptr, Bp, n->in, n->wb.ptr + n->oW1, n->h1, n->in, n->in, n->part.ptr, n->h1, true, &sp, s));
    a = ActArgs{};
    a.B = Bp, a.N = n->h1, a.Bvalid = batch, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->h1;
    a.bias = n->w.ptr + n->ob1, a.Zout = n->Z1.ptr, a.H = n->H1.ptr, a.HT = n->H1T.ptr;
    MPF_TRY(act<kGeluFwd>(a, s));
    // layer 2
    MPF_TRY(gemm(n, n->H1.ptr, Bp, n->h1, n->wb.ptr + n->oW2, n->h2, n->h1, n->h1, n->part.ptr, n->h2, true, &sp, s));
    a = ActArgs{};
    a.B = Bp, a.N = n->h2, a.Bvalid = batch, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->h2;
    a.bias = n->w.ptr + n->ob2, a.Zout = n->Z2.ptr, a.H = n->H2.ptr, a.HT = n->H2T.ptr;
    MPF_TRY(act<kGeluFwd>(a, s));
    // layer 3 (linear)
    MPF_TRY(gemm(n, n->H2.ptr, Bp, n->h2, n->wb.ptr + n->oW3, n->out, n->h2, n->h2, n->part.ptr, n->out, true, &sp, s));
    if (outSplits) *outSplits = sp;
    if (training) return MPF_OK;
    a = ActArgs{};
    a.B = Bp, a.N = n->out, a.Bvalid = Bp, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->out;
    a.bias = n->w.ptr + n->ob3, a.Zout = n->Y.ptr, a.ldOut = n->out;
    MPF_TRY(act<kLinear>(a, s));
    return MPF_OK;
}

int mlp_forward(mpf_mlp* n, int batch, const float* x, float* y, int ldy, cudaStream_t s) {
    MPF_CHECK(n && batch >= 1 && x && y && ldy >= 1, MPF_EINVAL, "mpf_mlp_forward: bad arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    MPF_TRY(forward(n, batch, x, n->in, nullptr, false, nullptr, s));
    MPF_CUDA(cudaMemcpy2DAsync(y, (size_t)ldy * sizeof(float), n->Y.ptr, (size_t)n->out * sizeof(float),
                               (size_t)std::min(ldy, n->out) * sizeof(float), batch, cudaMemcpyDeviceToDevice, s));
    return check_flag(n, s);
}

// Forward + backward: gradients of the mean squared error against target
// rows (ld ldt, first tvalid columns compared; row rows[b] of x and of the
// target for batch row b when rows is non-null) into the gradient array.
// With `fuse` the W3 gradient is not stored: its Adam step runs in the
// epilogue of the dW3 product (after dH2 has read the old W3).
static int backward(mpf_mlp* n, int batch, const float* x, int ldx, const int* rows, const float* target, int ldt,
                    int tvalid, double* loss, const AdamArgs* fuse, cudaStream_t s) {
    int sp = 1;
    MPF_TRY(forward(n, batch, x, ldx, rows, true, &sp, s));
    const int Bp = round_up(batch, kTile);
    HeadArgs h{};
    h.B = Bp, h.N = n->out, h.Bvalid = batch, h.Nvalid = tvalid, h.splits = sp, h.part = n->part.ptr;
    h.splitStride = (size_t)Bp * n->out, h.bias = n->w.ptr + n->ob3, h.T = target, h.ldT = ldt, h.rows = rows;
    h.scale = (float)(2.0 / ((double)batch * tvalid)), h.dY = n->dYb.ptr, h.dYT = n->dYT.ptr, h.colPart = n->colPart3.ptr;
    h.lossPart = n->lossPart.ptr;
    const dim3 headGrid(n->out / 32, Bp / 128);
    k_loss_head<<<headGrid, 256, 0, s>>>(h);
    MPF_LAUNCHED(1);
    // dH2 = dY W3 -> dZ2
    MPF_TRY(gemm(n, n->dYb.ptr, Bp, n->out, n->W3T.ptr, n->h2, n->out, n->out, n->part.ptr, n->h2, true, &sp, s));
    const int spH2 = sp;
    // dW3 = dY^T H2 (or its Adam step)
    if (fuse)
        MPF_TRY(gemm_adam(n, n->dYT.ptr, n->out, Bp, n->H2T.ptr, n->h2, Bp, Bp, n->oW3, n->W3T.ptr, *fuse, s));
    else
        MPF_TRY(gemm(n, n->dYT.ptr, n->out, Bp, n->H2T.ptr, n->h2, Bp, Bp, n->g.ptr + n->oW3, n->h2, false, &sp, s));
    sp = spH2;
    ActArgs a{};
    a.B = Bp, a.N = n->h2, a.Bvalid = batch, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->h2;
    a.Zin = n->Z2.ptr, a.H = n->dZ2.ptr, a.HT = n->dZ2T.ptr, a.colPart = n->colPart2.ptr;
    MPF_TRY(act<kGeluBwd>(a, s));
    // dW2 = dZ2^T H1
    MPF_TRY(gemm(n, n->dZ2T.ptr, n->h2, Bp, n->H1T.ptr, n->h1, Bp, Bp, n->g.ptr + n->oW2, n->h1, false, &sp, s));
    // dH1 = dZ2 W2 -> dZ1
    MPF_TRY(gemm(n, n->dZ2.ptr, Bp, n->h2, n->W2T.ptr, n->h1, n->h2, n->h2, n->part.ptr, n->h1, true, &sp, s));
    a = ActArgs{};
    a.B = Bp, a.N = n->h1, a.Bvalid = batch, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->h1;
    a.Zin = n->Z1.ptr, a.HT = n->dZ1T.ptr, a.colPart = n->colPart1.ptr;
    MPF_TRY(act<kGeluBwd>(a, s));
    // dW1 = dZ1^T X
    MPF_TRY(gemm(n, n->dZ1T.ptr, n->h1, Bp, n->XT.ptr, n->in, Bp, Bp, n->g.ptr + n->oW1, n->in, false, &sp, s));
    BiasArgs ba{};
    ba.N[0] = n->h1, ba.N[1] = n->h2, ba.N[2] = n->out;
    ba.part[0] = n->colPart1.ptr, ba.part[1] = n->colPart2.ptr, ba.part[2] = n->colPart3.ptr;
    ba.g[0] = n->g.ptr + n->ob1, ba.g[1] = n->g.ptr + n->ob2, ba.g[2] = n->g.ptr + n->ob3;
    ba.tiles = Bp / 32;
    k_bias_grad<<<(n->h1 + n->h2 + n->out + 255) / 256, 256, 0, s>>>(ba);
    MPF_LAUNCHED(1);
    if (loss) {
        const size_t parts = (size_t)headGrid.x * headGrid.y;
        MPF_CUDA(cudaMemcpyAsync(n->lossHost.data(), n->lossPart.ptr, sizeof(double) * parts, cudaMemcpyDeviceToHost,
                                 s));
        MPF_TRY(check_flag(n, s));
        double t = 0.0;
        for (size_t i = 0; i < parts; ++i) t += n->lossHost[i];
        *loss = t / ((double)batch * tvalid);
    }
    return MPF_OK;
}

int mlp_backward(mpf_mlp* n, int batch, const float* x, const float* target, int ldt, int tvalid, double* loss,
                 cudaStream_t s) {
    MPF_CHECK(n && batch >= 1 && x && target && tvalid >= 1 && tvalid <= n->out && ldt >= tvalid, MPF_EINVAL,
              "mpf_mlp_backward: bad arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    return backward(n, batch, x, n->in, nullptr, target, ldt, tvalid, loss, nullptr, s);
}

// Hyperparameters of the next Adam step (advances the step count).
static AdamArgs next_adam(mpf_mlp* n, float lr, float beta1, float beta2, float eps, float weightDecay) {
    n->step += 1;
    return AdamArgs{lr, beta1, beta2, eps, weightDecay, 1.f - std::pow(beta1, (float)n->step),
                    1.f - std::pow(beta2, (float)n->step)};
}

// Adam on every parameter from the gradient array, except W3 when its step
// already ran in the dW3 product's epilogue.
static int adam(mpf_mlp* n, const AdamArgs& a, bool withW3, cudaStream_t s) {
    // flat ranges (64-aligned): W1 | b1, b2, b3; tiled with transposes: W2, W3
    auto flat = [&](size_t from, size_t to) {
        const size_t c4 = (to - from) / 4;
        const int blocks = (int)std::min<size_t>((c4 + 255) / 256, (size_t)n->slots * 8);
        k_adam_flat<<<std::max(blocks, 1), 256, 0, s>>>(
            c4, reinterpret_cast<float4*>(n->w.ptr + from), reinterpret_cast<const float4*>(n->g.ptr + from),
            reinterpret_cast<float4*>(n->m.ptr + from), reinterpret_cast<float4*>(n->v.ptr + from),
            reinterpret_cast<__nv_bfloat162*>(n->wb.ptr + from), n->decay.ptr + from / 64, a);
    };
    flat(n->oW1, n->oW2);
    flat(n->ob2, n->oW3);
    flat(n->ob3, n->P);
    k_adam_wt<<<dim3(n->h1 / 32, n->h2 / 32), 256, 0, s>>>(n->h2, n->h1, n->w.ptr + n->oW2, n->g.ptr + n->oW2,
                                                            n->m.ptr + n->oW2, n->v.ptr + n->oW2,
                                                            n->wb.ptr + n->oW2, n->W2T.ptr, a);
    MPF_LAUNCHED(4);
    if (withW3) {
        k_adam_wt<<<dim3(n->h2 / 32, n->out / 32), 256, 0, s>>>(n->out, n->h2, n->w.ptr + n->oW3, n->g.ptr + n->oW3,
                                                                 n->m.ptr + n->oW3, n->v.ptr + n->oW3,
                                                                 n->wb.ptr + n->oW3, n->W3T.ptr, a);
        MPF_LAUNCHED(1);
    }
    return MPF_OK;
}

int mlp_adam(mpf_mlp* n, float lr, float beta1, float beta2, float eps, float weightDecay, cudaStream_t s) {
    MPF_CHECK(n && lr >= 0.f && beta1 >= 0.f && beta1 < 1.f && beta2 >= 0.f && beta2 < 1.f && eps > 0.f, MPF_EINVAL,
              "mpf_mlp_adam: bad arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    return adam(n, next_adam(n, lr, beta1, beta2, eps, weightDecay), true, s);
}

int mlp_train_step(mpf_mlp* n, int batch, const float* x, int ldx, const int* rows, const float* target, int ldt,
                   int tvalid, float lr, float beta1, float beta2, float eps, float weightDecay, double* loss,
                   cudaStream_t s) {
    MPF_CHECK(n && batch >= 1 && x && target && ldx >= n->in && tvalid >= 1 && tvalid <= n->out && ldt >= tvalid,
              MPF_EINVAL, "mpf_mlp_train_step: bad arguments");
    MPF_CHECK(lr >= 0.f && beta1 >= 0.f && beta1 < 1.f && beta2 >= 0.f && beta2 < 1.f && eps > 0.f, MPF_EINVAL,
              "mpf_mlp_train_step: bad Adam arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    const AdamArgs a = next_adam(n, lr, beta1, beta2, eps, weightDecay);
    MPF_TRY(backward(n, batch, x, ldx, rows, target, ldt, tvalid, loss, &a, s));
    return adam(n, a, false, s);
}

// dst [rowsPad][3 Kp] BF16 from the rows x K FP32 matrix at src (element
// (r, k) at src[r * srcRow + k * srcCol]): row r holds three K-segments of Kp
// columns, the BF16 part hi = bf16(x) and the remainder lo = bf16(x - hi) in
// the order hi, lo, hi (order 0) or hi, hi, lo (order 1); zero outside.  A
// product of an order-0 and an order-1 matrix is hi.hi + lo.hi + hi.lo.
__global__ void k_split3(int rows, int rowsPad, int K, int Kp, const float* __restrict__ src, size_t srcRow,
                         size_t srcCol, int order, __nv_bfloat16* __restrict__ dst) {
    const size_t total = (size_t)rowsPad * Kp;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / Kp), k = (int)(i % Kp);
        const float x = (r < rows && k < K) ? src[r * srcRow + k * srcCol] : 0.f;
        const __nv_bfloat16 hi = __float2bfloat16_rn(x);
        const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
        __nv_bfloat16* d = dst + (size_t)r * 3 * Kp + k;
        d[0] = hi;
        d[Kp] = order == 0 ? lo : hi;
        d[2 * Kp] = order == 0 ? hi : lo;
    }
}

int split3_bf16(int rows, int rowsPad, int K, int Kp, const float* src, size_t srcRow, size_t srcCol, int order,
                __nv_bfloat16* dst, cudaStream_t s) {
    const size_t total = (size_t)rowsPad * Kp;
    const int blocks = (int)std::min<size_t>((total + 255) / 256, 152 * 16);
    k_split3<<<blocks, 256, 0, s>>>(rows, rowsPad, K, Kp, src, srcRow, srcCol, order, dst);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

// out (rowsValid x colsValid of ld ldo) = alpha A B^T + beta out + add with
// A: M x K and B: N x K BF16, both K-major (M, N multiples of 128, K of 64),
// FP32 accumulation on the tensor cores, no K split.  Raises `flag` if a
// pipeline wait gave up (the caller reads it).
int tc_gemm_axpby(const __nv_bfloat16* A, int M, int lda, const __nv_bfloat16* B, int N, int ldb, int K,
                  float* out, int ldo, int rowsValid, int colsValid, float alpha, float beta, float add, int* flag,
                  cudaStream_t s) {
    MPF_CHECK(M % kTile == 0 && N % kTile == 0 && K % kBK == 0 && lda % 8 == 0 && ldb % 8 == 0 &&
                  rowsValid <= M && colsValid <= N && ldo >= colsValid && flag,
              MPF_EINVAL, "tensor-core GEMM: M, N %% 128 and K %% 64 must be 0 (M=%d N=%d K=%d)", M, N, K);
    CUtensorMap mA, mB;
    MPF_TRY(make_bf16_map(&mA, A, M, lda));
    MPF_TRY(make_bf16_map(&mB, B, N, ldb));
    MPF_CUDA(cudaFuncSetAttribute(k_gemm_nt<kGemmAxpby>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem));
    GemmArgs ga{K / kBK, 1, out, ldo, 0, flag};
    ga.alpha = alpha, ga.beta = beta, ga.add = add, ga.rowsValid = rowsValid, ga.colsValid = colsValid;
    k_gemm_nt<kGemmAxpby><<<dim3(M / kTile, N / kTile, 1), 128, kGemmSmem, s>>>(mA, mB, ga, AdamArgs{});
    MPF_LAUNCHED(1);
    return MPF_OK;
}

// Copy parameters or gradients between the network and a caller device
// buffer of mlp_param_count floats.  which: 0 get weights, 1 set weights,
// 2 get gradients.
int mlp_params(mpf_mlp* n, float* buf, int which, cudaStream_t s) {
    MPF_CHECK(n && buf && which >= 0 && which <= 2, MPF_EINVAL, "mpf_mlp_params: bad arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    const size_t bytes = n->P * sizeof(float);
    if (which == 0) MPF_CUDA(cudaMemcpyAsync(buf, n->w.ptr, bytes, cudaMemcpyDeviceToDevice, s));
    if (which == 2) MPF_CUDA(cudaMemcpyAsync(buf, n->g.ptr, bytes, cudaMemcpyDeviceToDevice, s));
    if (which == 1) {
        MPF_CUDA(cudaMemcpyAsync(n->w.ptr, buf, bytes, cudaMemcpyDeviceToDevice, s));
        MPF_TRY(mlp_refresh(n, s));
        n->step = 0;
        MPF_CUDA(cudaMemsetAsync(n->m.ptr, 0, bytes, s));
        MPF_CUDA(cudaMemsetAsync(n->v.ptr, 0, bytes, s));
    }
    return MPF_OK;
}

}  // namespace mpf
