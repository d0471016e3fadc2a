// Device building blocks shared by the batched Krylov solvers (cg_kernels.cu,
// bicgstab_kernels.cu): lane mapping of node-major vectors, vector loads and
// stores, compensated inner-product accumulation, block reductions with a
// last-block-done counter, the mesh segment of a group, and the fused
// (S + alpha R) ELL product over a warp's rows.
#pragma once

#include "model.h"

namespace mpf {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRowsPerWarp = kRowTile / kWarps;  // 16
constexpr int kWFast = 8;                         // ELL slots unrolled at compile time

template <int KP, int VEC_>
struct Shape {
    static constexpr int VEC = VEC_;                 // floats per lane
    static constexpr int LPR = KP / VEC;             // lanes per row
    static constexpr int SUB = 32 / LPR;             // rows per warp instruction
    static constexpr int STEPS = kRowsPerWarp / SUB; // warp steps per 16 rows
    static_assert(LPR >= 1 && LPR <= 32 && 32 % LPR == 0, "invalid lane mapping");
};

template <int V>
__device__ __forceinline__ void ldv(const float* p, float (&v)[V]) {
    if constexpr (V == 1) {
        v[0] = *p;
    } else if constexpr (V == 2) {
        const float2 t = *reinterpret_cast<const float2*>(p);
        v[0] = t.x; v[1] = t.y;
    } else {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
}
template <int V>
__device__ __forceinline__ void stv(float* p, const float (&v)[V]) {
    if constexpr (V == 1) {
        *p = v[0];
    } else if constexpr (V == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    } else {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
}

// Compensated accumulation of a*b into a float pair: FMA TwoProduct gives
// the product's rounding error and Knuth's TwoSum the sum's, both collected
// in c, so value() carries about twice the float precision.
struct DotAcc {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float a, float b) {
        float p = __fmul_rn(a, b);
        float pe = __fmaf_rn(a, b, -p);
        float t = __fadd_rn(s, p);
        float z = __fsub_rn(t, s);
        float te = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
        s = t;
        c = __fadd_rn(c, __fadd_rn(te, pe));
    }
    // adds a float (e.g. a short FP32 partial sum) with Knuth's TwoSum
    __device__ __forceinline__ void addf(float x) {
        float t = __fadd_rn(s, x);
        float z = __fsub_rn(t, s);
        float te = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z));
        s = t;
        c = __fadd_rn(c, te);
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ float diag_inv(const float2* SR, const int32_t* diagSlot, int npad, int row,
                                          float alpha) {
    const int ds = __ldg(&diagSlot[row]);
    const float2 e = __ldg(&SR[(size_t)ds * npad + row]);
    const float d = e.x + alpha * e.y;
    return d != 0.f ? __frcp_rn(d) : 0.f;  // correctly rounded: the same value as 1.f / d
}

// Rows of one mesh: a single mesh covers tiles [0, nblk) and rows < n; a
// batch of stacked meshes reads its segment table (see CgProblem).
struct Seg {
    int tile0, nblk, end;
    float dcScale;
};
// aggregates of kAgg rows of a segment's mesh (the coarse space's size)
__device__ __forceinline__ int seg_aggregates(const Seg& sg) { return (sg.end - sg.tile0 * kRowTile + kAgg - 1) / kAgg; }

__device__ __forceinline__ Seg segment(const CgProblem& P, int mesh) {
    if (P.seg) {
        const int4 d = __ldg(&P.seg[mesh]);
        return {d.x, d.y, d.z, __int_as_float(d.w)};
    }
    return {0, P.nblk, P.n, P.dcScale};
}

// Block-level reduction of per-thread partials into part[g][blk][KP]; returns
// true in every thread of the block that finishes the group last (that block
// then sees all partials of the group).  nb: blocks of the group.
template <int KP, int VEC, int NDOT>
__device__ __forceinline__ bool block_partials(const DotAcc (&acc)[NDOT][VEC], double* const (&part)[NDOT], int g,
                                               unsigned* counter, int nb) {
    using Sh = Shape<KP, VEC>;
    __shared__ double red[NDOT][kWarps * Sh::SUB][KP];
    __shared__ bool amLast;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
#pragma unroll
    for (int d = 0; d < NDOT; ++d)
#pragma unroll
        for (int v = 0; v < VEC; ++v) red[d][warp * Sh::SUB + sub][j0 + v] = acc[d][v].value();
    __syncthreads();
    if (threadIdx.x < KP) {
#pragma unroll
        for (int d = 0; d < NDOT; ++d) {
            double s = 0.0;
            for (int w = 0; w < kWarps * Sh::SUB; ++w) s += red[d][w][threadIdx.x];
            part[d][((size_t)g * gridDim.x + blockIdx.x) * KP + threadIdx.x] = s;
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) amLast = atomicAdd(&counter[g], 1u) == (unsigned)(nb - 1);
    __syncthreads();
    if (amLast) __threadfence();
    return amLast;
}

// block_partials with the reduction array in caller-provided shared memory
// (red: NDOT * kWarps * SUB * KP doubles; amLast: one flag), for kernels
// whose dynamic shared memory is free again when they reduce.
template <int KP, int VEC, int NDOT>
__device__ __forceinline__ bool block_partials_in(const DotAcc (&acc)[NDOT][VEC], double* const (&part)[NDOT],
                                                  int g, unsigned* counter, int nb, double* red, int* amLast) {
    using Sh = Shape<KP, VEC>;
    constexpr int R = kWarps * Sh::SUB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
#pragma unroll
    for (int d = 0; d < NDOT; ++d)
#pragma unroll
        for (int v = 0; v < VEC; ++v) red[((size_t)d * R + warp * Sh::SUB + sub) * KP + j0 + v] = acc[d][v].value();
    __syncthreads();
    if (threadIdx.x < KP) {
#pragma unroll
        for (int d = 0; d < NDOT; ++d) {
            double s = 0.0;
            for (int w = 0; w < R; ++w) s += red[((size_t)d * R + w) * KP + threadIdx.x];
            part[d][((size_t)g * gridDim.x + blockIdx.x) * KP + threadIdx.x] = s;
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) *amLast = atomicAdd(&counter[g], 1u) == (unsigned)(nb - 1);
    __syncthreads();
    const bool last = *amLast != 0;
    if (last) __threadfence();
    return last;
}

// Fixed-order sum of the block partials of group g, right-hand side j (the
// group's nb blocks; partials are strided by the launch's x dimension).
__device__ __forceinline__ double sum_partials(const double* part, int g, int KP, int j, int nb) {
    double s = 0.0;
    const double* p = part + (size_t)g * gridDim.x * KP + j;
    for (int b = 0; b < nb; ++b) s += __ldcg(p + (size_t)b * KP);
    return s;
}

// y[i] = (S + alpha R) x over the rows row[i].  The first kWFast slots are
// unrolled in three independent batches -- all column loads, then all value
// loads and gathers -- so a warp waits for one memory latency per batch
// instead of one per slot; slots past kWFast (meshes with more than kWFast
// entries in a row) are looped.  Padding slots point at their own row with
// value 0.
template <int KP, int VEC, int RB>
__device__ __forceinline__ void spmm_rows(const int32_t* cols, const float2* SR, int W, int npad, float alpha,
                                          const float* x, int j0, const int (&row)[RB], float (&y)[RB][VEC]) {
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int v = 0; v < VEC; ++v) y[i][v] = 0.f;
    int col[kWFast][RB];
#pragma unroll
    for (int k = 0; k < kWFast; ++k)
#pragma unroll
        for (int i = 0; i < RB; ++i) col[k][i] = k < W ? __ldg(&cols[(size_t)k * npad + row[i]]) : row[i];
    float a[kWFast][RB];
#pragma unroll
    for (int k = 0; k < kWFast; ++k)
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            float2 e = make_float2(0.f, 0.f);
            if (k < W) e = __ldg(&SR[(size_t)k * npad + row[i]]);
            a[k][i] = e.x + alpha * e.y;
        }
#pragma unroll
    for (int k = 0; k < kWFast; ++k) {
        if (k < W) {
#pragma unroll
            for (int i = 0; i < RB; ++i) {
                float xv[VEC];
                ldv<VEC>(x + (size_t)col[k][i] * KP + j0, xv);
#pragma unroll
                for (int v = 0; v < VEC; ++v) y[i][v] = fmaf(a[k][i], xv[v], y[i][v]);
            }
        }
    }
    for (int k = kWFast; k < W; ++k) {
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const int c = __ldg(&cols[(size_t)k * npad + row[i]]);
            const float2 e = __ldg(&SR[(size_t)k * npad + row[i]]);
            float xv[VEC];
            ldv<VEC>(x + (size_t)c * KP + j0, xv);
            const float av = e.x + alpha * e.y;
#pragma unroll
            for (int v = 0; v < VEC; ++v) y[i][v] = fmaf(av, xv[v], y[i][v]);
        }
    }
}

}  // namespace
}  // namespace mpf
