// Learned Gauss-Newton warm start: a multilayer perceptron
//   x (in) -> GELU(W1 x + b1) (h1) -> GELU(W2 . + b2) (h2) -> W3 . + b3 (out)
// trained and evaluated with hand-written kernels.  No reference counterpart.
//
//  * k_gemm_nt  D[M][N] = sum_k A[M][k] B[N][k] with BF16 operands (both
//               K-major) on the tcgen05 tensor cores: TMA 128-byte-swizzled
//               tiles -> 4-stage mbarrier pipeline -> tcgen05.mma (FP32
//               accumulator in tensor memory) -> tcgen05.ld epilogue.  The K
//               range may be split over CTAs (FP32 partials, summed by the
//               consumer kernel in a fixed order).
//  * k_act      sums the split partials, adds the bias and applies the
//               activation (or its derivative), writing FP32 and BF16 copies
//               in row-major and transposed layout as the next GEMMs need
//               them (every GEMM operand is K-major).
//  * k_mse, k_colsum, k_adam, k_transpose_bf16, k_init_uniform: loss and
//               output gradient, bias gradients, Adam with FP32 master
//               weights and BF16 working copies, weight transposes, seeded
//               initialisation.
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

constexpr int kStages = 4;
constexpr int kStageBytes = 2 * kTileBytes;  // A tile + B tile
constexpr int kGemmSmem = kStages * kStageBytes + 1024 /*align*/ + 256 /*barriers*/;

struct GemmArgs {
    int kblocks;        // K / 64
    int splits;         // K splits (grid z)
    float* out;         // out + split * splitStride + m * ldOut + n
    int ldOut;
    size_t splitStride;
    int* abortFlag;
};

// One CTA = one 128x128 output tile and one K split.  Warp 0 lane 0 issues
// the TMA loads, warp 1 lane 0 the MMAs; all four warps drain TMEM.
__global__ void __launch_bounds__(128, 1) k_gemm_nt(const __grid_constant__ CUtensorMap mapA,
                                                    const __grid_constant__ CUtensorMap mapB, GemmArgs ga) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + kStages * kStageBytes);
    __shared__ uint32_t tmemBase;
    __shared__ int localAbort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tn = blockIdx.x, tm = blockIdx.y, split = blockIdx.z;
    const int kb0 = (int)((long)ga.kblocks * split / ga.splits);
    const int kb1 = (int)((long)ga.kblocks * (split + 1) / ga.splits);
    const int nk = kb1 - kb0;

    const uint32_t fullBar = smem_u32(&bars[0]);
    const uint32_t emptyBar = smem_u32(&bars[kStages]);
    const uint32_t doneBar = smem_u32(&bars[2 * kStages]);
    if (threadIdx.x == 0) {
        localAbort = 0;
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
    const int row = warp * 32 + lane;
    float* out = ga.out + split * ga.splitStride + (size_t)(tm * kTile + row) * ga.ldOut + tn * kTile;
    if (ok) {
#pragma unroll 1
        for (int c = 0; c < kTile; c += 32) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int i = 0; i < 32; i += 4)
                *reinterpret_cast<float4*>(out + c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
    } else {
        for (int c = 0; c < kTile; ++c) out[c] = 0.f;
        if (threadIdx.x == 0 && nk > 0) atomicExch(ga.abortFlag, 1);
    }
    fence_before();
    __syncthreads();
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
};

// One block = one 32x32 tile (32 x 8 threads); the transposed copy goes
// through shared memory so both writes are coalesced.
template <int MODE>
__global__ void __launch_bounds__(256) k_act(ActArgs a) {
    __shared__ float tile[32][33];
    const int n0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) {
        const int b = b0 + r, n = n0 + tx;
        float v = 0.f;
        if (b < a.Bvalid) {
            if (MODE == kCast) {
                v = a.part[(size_t)b * a.ldIn + n];
            } else {
                for (int s = 0; s < a.splits; ++s) v += a.part[s * a.splitStride + (size_t)b * a.N + n];
                if (a.bias) v += a.bias[n];
            }
        }
        float h = v;
        if (MODE == kGeluFwd) {
            if (a.Zout) a.Zout[(size_t)b * a.N + n] = v;
            h = b < a.Bvalid ? gelu(v) : 0.f;
        } else if (MODE == kGeluBwd) {
            h = b < a.Bvalid ? v * gelu_deriv(a.Zin[(size_t)b * a.N + n]) : 0.f;
            if (a.Zout) a.Zout[(size_t)b * a.ldOut + n] = h;
        } else if (MODE == kLinear) {
            if (a.Zout && b < a.Bvalid) a.Zout[(size_t)b * a.ldOut + n] = v;
        }
        if (a.H) a.H[(size_t)b * a.N + n] = __float2bfloat16_rn(h);
        tile[r][tx] = h;
    }
    if (!a.HT) return;
    __syncthreads();
    for (int r = ty; r < 32; r += 8) a.HT[(size_t)(n0 + r) * a.B + b0 + tx] = __float2bfloat16_rn(tile[tx][r]);
}

// Mean squared error over the valid entries and its gradient
// dY = 2 (Y - T) / (Bvalid * Nvalid); one partial loss per block.
__global__ void __launch_bounds__(256) k_mse(int B, int N, int Bvalid, int Nvalid, const float* __restrict__ Y,
                                             const float* __restrict__ T, int ldT, float* __restrict__ dY,
                                             double* __restrict__ lossPart) {
    __shared__ double red[256];
    const double scale = 2.0 / ((double)Bvalid * Nvalid);
    double acc = 0.0;
    const size_t total = (size_t)B * N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(i / N), n = (int)(i % N);
        float d = 0.f;
        if (b < Bvalid && n < Nvalid) d = Y[i] - T[(size_t)b * ldT + n];
        acc += (double)d * d;
        dY[i] = (float)(scale * d);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) lossPart[blockIdx.x] = red[0];
}

// g[n] = sum_b F[b][n] (bias gradient), fixed order
__global__ void k_colsum(int B, int N, const float* __restrict__ F, float* __restrict__ g) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += F[(size_t)b * N + n];
    g[n] = s;
}

// Adam (decoupled weight decay on the weights only) over the flat arrays.
__global__ void k_adam(size_t count, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wb, const uint8_t* __restrict__ decay,
                       float lr, float b1, float b2, float eps, float wd, float bc1, float bc2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        float wi = w[i];
        if (decay[i >> 6]) wi -= lr * wd * wi;
        wi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        w[i] = wi;
        wb[i] = __float2bfloat16_rn(wi);
    }
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

int gemm_splits(int tiles, int kblocks) {
    int s = (2 * 148 + tiles - 1) / tiles;
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
    // activations, grown with the batch
    int capB = 0;
    mpf::DevBuf<__nv_bfloat16> X, XT, H1, H1T, H2, H2T, dYb, dYT, dZ2, dZ2T, dZ1T;
    mpf::DevBuf<float> Z1, Z2, Y, dY, F32, part;
    mpf::DevBuf<double> lossPart;
    mpf::DevBuf<int> flag;
};

namespace mpf {

static constexpr int kLossBlocks = 1024;
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
    MPF_TRY(n->dY.alloc(B * out));
    MPF_TRY(n->F32.alloc(B * std::max(h1, h2)));
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
    const int splits = allowSplit ? gemm_splits(tiles, kblocks) : 1;
    // per device and cheap: set on every call
    MPF_CUDA(cudaFuncSetAttribute(k_gemm_nt, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem));
    GemmArgs ga{kblocks, splits, splits > 1 ? n->part.ptr : out, splits > 1 ? N : ldOut, (size_t)M * N,
                n->flag.ptr};
    MPF_CHECK(splits == 1 || (size_t)splits * M * N <= n->part.count, MPF_EINVAL, "mlp gemm: split buffer too small");
    k_gemm_nt<<<dim3(N / kTile, M / kTile, splits), 128, kGemmSmem, s>>>(mA, mB, ga);
    MPF_LAUNCHED(1);
    *splitsOut = splits;
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
    MPF_TRY(n->lossPart.alloc(kLossBlocks));
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

// Forward pass on `batch` rows of x (FP32, ld ldx); Bp = batch rounded up to
// 128.  Leaves X, Z1, H1(T), Z2, H2(T) and Y in the workspace.
static int forward(mpf_mlp* n, int batch, const float* x, int ldx, cudaStream_t s) {
    const int Bp = round_up(batch, kTile);
    MPF_TRY(mlp_workspace(n, Bp));
    int sp = 1;
    ActArgs a{};
    a.B = Bp, a.N = n->in, a.Bvalid = batch, a.splits = 1, a.part = x, a.ldIn = ldx;
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
    a = ActArgs{};
    a.B = Bp, a.N = n->out, a.Bvalid = Bp, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->out;
    a.bias = n->w.ptr + n->ob3, a.Zout = n->Y.ptr, a.ldOut = n->out;
    MPF_TRY(act<kLinear>(a, s));
    return MPF_OK;
}

int mlp_forward(mpf_mlp* n, int batch, const float* x, float* y, int ldy, cudaStream_t s) {
    MPF_CHECK(n && batch >= 1 && x && y && ldy >= 1, MPF_EINVAL, "mpf_mlp_forward: bad arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    MPF_TRY(forward(n, batch, x, n->in, s));
    MPF_CUDA(cudaMemcpy2DAsync(y, (size_t)ldy * sizeof(float), n->Y.ptr, (size_t)n->out * sizeof(float),
                               (size_t)std::min(ldy, n->out) * sizeof(float), batch, cudaMemcpyDeviceToDevice, s));
    return check_flag(n, s);
}

// Forward + backward: gradients of the mean squared error against target
// (ld ldt, first tvalid columns compared) into the gradient array.
int mlp_backward(mpf_mlp* n, int batch, const float* x, const float* target, int ldt, int tvalid, double* loss,
                 cudaStream_t s) {
    MPF_CHECK(n && batch >= 1 && x && target && tvalid >= 1 && tvalid <= n->out && ldt >= tvalid, MPF_EINVAL,
              "mpf_mlp_backward: bad arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    MPF_TRY(forward(n, batch, x, n->in, s));
    const int Bp = round_up(batch, kTile);
    int sp = 1;
    k_mse<<<kLossBlocks, 256, 0, s>>>(Bp, n->out, batch, tvalid, n->Y.ptr, target, ldt, n->dY.ptr, n->lossPart.ptr);
    MPF_LAUNCHED(1);
    ActArgs a{};
    a.B = Bp, a.N = n->out, a.Bvalid = Bp, a.splits = 1, a.part = n->dY.ptr, a.ldIn = n->out;
    a.H = n->dYb.ptr, a.HT = n->dYT.ptr;
    MPF_TRY(act<kCast>(a, s));
    k_colsum<<<(n->out + 255) / 256, 256, 0, s>>>(Bp, n->out, n->dY.ptr, n->g.ptr + n->ob3);
    MPF_LAUNCHED(1);
    // dW3 = dY^T H2
    MPF_TRY(gemm(n, n->dYT.ptr, n->out, Bp, n->H2T.ptr, n->h2, Bp, Bp, n->g.ptr + n->oW3, n->h2, false, &sp, s));
    // dH2 = dY W3 -> dZ2
    MPF_TRY(gemm(n, n->dYb.ptr, Bp, n->out, n->W3T.ptr, n->h2, n->out, n->out, n->part.ptr, n->h2, true, &sp, s));
    a = ActArgs{};
    a.B = Bp, a.N = n->h2, a.Bvalid = batch, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->h2;
    a.Zin = n->Z2.ptr, a.Zout = n->F32.ptr, a.ldOut = n->h2, a.H = n->dZ2.ptr, a.HT = n->dZ2T.ptr;
    MPF_TRY(act<kGeluBwd>(a, s));
    k_colsum<<<(n->h2 + 255) / 256, 256, 0, s>>>(Bp, n->h2, n->F32.ptr, n->g.ptr + n->ob2);
    MPF_LAUNCHED(1);
    // dW2 = dZ2^T H1
    MPF_TRY(gemm(n, n->dZ2T.ptr, n->h2, Bp, n->H1T.ptr, n->h1, Bp, Bp, n->g.ptr + n->oW2, n->h1, false, &sp, s));
    // dH1 = dZ2 W2 -> dZ1
    MPF_TRY(gemm(n, n->dZ2.ptr, Bp, n->h2, n->W2T.ptr, n->h1, n->h2, n->h2, n->part.ptr, n->h1, true, &sp, s));
    a = ActArgs{};
    a.B = Bp, a.N = n->h1, a.Bvalid = batch, a.splits = sp, a.part = n->part.ptr, a.splitStride = (size_t)Bp * n->h1;
    a.Zin = n->Z1.ptr, a.Zout = n->F32.ptr, a.ldOut = n->h1, a.HT = n->dZ1T.ptr;
    MPF_TRY(act<kGeluBwd>(a, s));
    k_colsum<<<(n->h1 + 255) / 256, 256, 0, s>>>(Bp, n->h1, n->F32.ptr, n->g.ptr + n->ob1);
    MPF_LAUNCHED(1);
    // dW1 = dZ1^T X
    MPF_TRY(gemm(n, n->dZ1T.ptr, n->h1, Bp, n->XT.ptr, n->in, Bp, Bp, n->g.ptr + n->oW1, n->in, false, &sp, s));
    if (loss) {
        std::vector<double> lp(kLossBlocks);
        MPF_CUDA(cudaMemcpyAsync(lp.data(), n->lossPart.ptr, sizeof(double) * kLossBlocks, cudaMemcpyDeviceToHost, s));
        MPF_TRY(check_flag(n, s));
        double t = 0.0;
        for (double v : lp) t += v;
        *loss = t / ((double)batch * tvalid);
        return MPF_OK;
    }
    return MPF_OK;
}

int mlp_adam(mpf_mlp* n, float lr, float beta1, float beta2, float eps, float weightDecay, cudaStream_t s) {
    MPF_CHECK(n && lr >= 0.f && beta1 >= 0.f && beta1 < 1.f && beta2 >= 0.f && beta2 < 1.f && eps > 0.f, MPF_EINVAL,
              "mpf_mlp_adam: bad arguments");
    MPF_CUDA(cudaSetDevice(n->device));
    n->step += 1;
    const float bc1 = 1.f - std::pow(beta1, (float)n->step), bc2 = 1.f - std::pow(beta2, (float)n->step);
    k_adam<<<4096, 256, 0, s>>>(n->P, n->w.ptr, n->g.ptr, n->m.ptr, n->v.ptr, n->wb.ptr, n->decay.ptr, lr, beta1,
                                beta2, eps, weightDecay, bc1, bc2);
    MPF_LAUNCHED(1);
    k_transpose_bf16<<<dim3(n->h1 / 32, n->h2 / 32), 256, 0, s>>>(n->h2, n->h1, n->wb.ptr + n->oW2, n->W2T.ptr);
    k_transpose_bf16<<<dim3(n->h2 / 32, n->out / 32), 256, 0, s>>>(n->out, n->h2, n->wb.ptr + n->oW3, n->W3T.ptr);
    MPF_LAUNCHED(2);
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
