// Batched Jacobi-preconditioned conjugate gradient for the EIT systems.
//
// Restates src/numeric/conjugate_gradient.cpp:61-161 (per-column scalars,
// Jacobi preconditioner of src/numeric/preconditioner_kernel.cu:63-83, the
// zero-denominator guards of src/numeric/conjugate_gradient_kernel.cu:77-89)
// for many independent systems at once: every (frame, harmonic) group has
// KP right-hand sides that share one matrix S + alpha_c R, and every group
// runs its own iteration with per-right-hand-side convergence masks.
//
// One CG iteration is three launches, each a single pass over the vectors:
//   k_spmm_dot   q = (S + alpha R) p,  pq = p.q
//   k_update     r -= a q, z = D^-1 r, rz' = r.z  (+ convergence)
//   k_direction  x += a p_old, p = D^-1 r + b p_old
// x is updated where the old p is read anyway (10 vector passes per
// iteration instead of 11); cg_launch_finalize applies the last update of
// groups that retired.
// Memory access: a lane moves VEC consecutive floats, so KP/VEC lanes cover
// one node's right-hand sides and one warp instruction serves 32*VEC/KP
// rows; each warp keeps RB row steps in flight, and a block walks
// P.tiles[k] consecutive 128-row tiles.  VEC and RB (template parameters)
// and the tiles per block (runtime) are chosen per model by the autotuner in
// model.cu (CUDA-event timings of every variant on the model's own systems).
// An ELL slot is a column index (int32 array) and a float2 {S, R}; the
// SpMM fuses S + alpha R (the system matrix is never materialised) and
// unrolls up to kWFast slots.  A second SpMM form stages each 128-row tile's
// slots in shared memory with cp.async, one tile ahead of the rows it
// multiplies (k_spmm_dot_staged); the autotuner picks between the two.
// Inner products: each thread accumulates its products in a compensated
// (TwoProduct/TwoSum) float pair, everything above that level is FP64; the
// per-block partials are combined by the last block of the group in a fixed
// order, so results are deterministic (helpers in cg_common.cuh).
#include "cg_common.cuh"
#include "tc_ptx.cuh"

namespace mpf {
namespace {

// Restriction P^T v of one 128-row tile for the two-level preconditioner:
// the rows of warps 0-3 form aggregate 2 * tile, those of warps 4-7
// aggregate 2 * tile + 1 (kAgg = 64).  Every thread passes its sum over the
// rows it handled; the block adds them in a fixed order and writes
// out[agg][KP].  Called by all threads of the block.
template <int KP, int VEC>
__device__ __forceinline__ void restrict_tile(const float (&part)[VEC], int tile, int nc, float* __restrict__ out,
                                              float* red) {
    using Sh = Shape<KP, VEC>;
    static_assert(kAgg * 2 == kRowTile && kRowsPerWarp * 4 == kAgg, "aggregate = 4 warps of rows");
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
#pragma unroll
    for (int v = 0; v < VEC; ++v) red[(warp * Sh::SUB + sub) * KP + j0 + v] = part[v];
    __syncthreads();
    if (threadIdx.x < 2 * KP) {
        const int half = threadIdx.x / KP, j = threadIdx.x % KP;
        float s = 0.f;
        for (int w = half * 4; w < half * 4 + 4; ++w)
            for (int u = 0; u < Sh::SUB; ++u) s += red[(w * Sh::SUB + u) * KP + j];
        const int agg = tile * 2 + half;
        if (agg < nc) out[(size_t)agg * KP + j] = s;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Neumann (dcFree) harmonics: the reference regularises the singular
// stiffness matrix as (A + 1 1^T) x = b (src/numeric/conjugate_gradient.cpp:
// 85-89,115-119).  That rank-one term puts an eigenvalue n on the constant
// vector, which in FP32 amplifies rounding in that direction ~n-fold, so the
// iteration here uses (A + c' 1 1^T) with c' = mean(diag A) / n (eigenvalue
// ~1 after Jacobi scaling); both systems have the same zero-mean solution
// and k_dc_shift adds the exact constant difference afterwards.  The
// rank-one term needs sum(p), which k_direction reduces for the next SpMM.

// r = b - A x - c' sum(x) (or r = b), z = D^-1 r, p = z, rz = r.z, bz = b.D^-1 b, sum(p)
template <int KP>
__global__ void __launch_bounds__(kThreads) k_init(CgProblem P, int zeroGuess) {
    constexpr int VEC = KP >= 32 ? 4 : 2;
    using Sh = Shape<KP, VEC>;
    constexpr int RB = Sh::STEPS < 2 ? Sh::STEPS : 2;
    const int g = blockIdx.y;
    const int slice = g / P.M;
    const Seg sg = segment(P, g - slice * P.M);
    if ((int)blockIdx.x >= sg.nblk) return;
    const int f = slice / P.Ca, ci = slice % P.Ca;
    const bool dc = P.dcFree[ci] != 0;
    const float alpha = P.alpha[ci];
    const float2* SR = P.SR + (size_t)f * P.W * P.npad;
    const size_t vb = (size_t)slice * P.npad * KP;
    const float* b = P.b + (P.bPerGroup ? vb : (size_t)ci * P.npad * KP);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    float sx[VEC] = {};
    if (dc && !zeroGuess && P.sumX0) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) sx[v] = (float)((double)sg.dcScale * P.sumX0[(size_t)g * KP + j0 + v]);
    }
    DotAcc acc[3][VEC];
    float rsum[VEC] = {}, bsum[VEC] = {};
    const int rowBase = (sg.tile0 + blockIdx.x) * kRowTile + warp * kRowsPerWarp;
    for (int st = 0; st < Sh::STEPS; st += RB) {
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) row[i] = rowBase + (st + i) * Sh::SUB + sub;
        float y[RB][VEC];
        if (!zeroGuess) {
            spmm_rows<KP, VEC, RB>(P.cols, SR, P.W, P.npad, alpha, P.x + vb, j0, row, y);
        } else {
#pragma unroll
            for (int i = 0; i < RB; ++i) {
#pragma unroll
                for (int v = 0; v < VEC; ++v) y[i][v] = 0.f;
                stv<VEC>(P.x + vb + (size_t)row[i] * KP + j0, y[i]);
            }
        }
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const bool real = row[i] < sg.end;
            float bv[VEC], rv[VEC], zv[VEC];
            ldv<VEC>(b + (size_t)row[i] * KP + j0, bv);
            const float di = diag_inv(SR, P.diagSlot, P.npad, row[i], alpha);
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                rv[v] = zeroGuess ? bv[v] : bv[v] - y[i][v] - (real ? sx[v] : 0.f);
                zv[v] = di * rv[v];
                acc[0][v].add(rv[v], zv[v]);
                acc[1][v].add(bv[v], di * bv[v]);
                if (dc && real) acc[2][v].add(zv[v], 1.f);
                rsum[v] += real ? rv[v] : 0.f;
                bsum[v] += real ? bv[v] : 0.f;
            }
            stv<VEC>(P.r + vb + (size_t)row[i] * KP + j0, rv);
            if (!P.coarse) stv<VEC>(P.p + vb + (size_t)row[i] * KP + j0, zv);
        }
    }
    if (P.coarse) {
        __shared__ float red[kWarps * 32 * VEC];
        const size_t cb = (size_t)g * P.ncPad * KP;
        restrict_tile<KP, VEC>(rsum, blockIdx.x, seg_aggregates(sg), P.rc + cb, red);
        restrict_tile<KP, VEC>(bsum, blockIdx.x, seg_aggregates(sg), P.rcB + cb, red);
    }
    double* const parts[3] = {P.partA, P.partB, P.partC};
    const int nb = sg.nblk;
    if (block_partials<KP, VEC, 3>(acc, parts, g, P.counter, nb)) {
        if (threadIdx.x < KP) P.alphaX[(size_t)g * KP + threadIdx.x] = 0.0;
        if (threadIdx.x == 0) P.pend[g] = 0;
        if (P.coarse) {
            // the coarse kernel completes r^T M^-1 r and b^T M^-1 b and sets the masks
            if (threadIdx.x < KP) {
                P.rzFine[(size_t)g * KP + threadIdx.x] = sum_partials(P.partA, g, KP, threadIdx.x, nb);
                P.bzFine[(size_t)g * KP + threadIdx.x] = sum_partials(P.partB, g, KP, threadIdx.x, nb);
            }
            if (threadIdx.x == 0) {
                P.iters[g] = 0;
                P.counter[g] = 0;
            }
            return;
        }
        int notConv = 0;
        if (threadIdx.x < KP) {
            const int j = threadIdx.x;
            double rz = sum_partials(P.partA, g, KP, j, nb);
            double bz = sum_partials(P.partB, g, KP, j, nb);
            P.sumP[(size_t)g * KP + j] = dc ? sum_partials(P.partC, g, KP, j, nb) : 0.0;
            P.rz[(size_t)g * KP + j] = rz;
            P.bz[(size_t)g * KP + j] = bz;
            P.beta[(size_t)g * KP + j] = 0.0;
            int c = rz <= P.tol2 * bz;
            P.conv[(size_t)g * KP + j] = c;
            notConv = !c;
        }
        int any = __syncthreads_or(notConv);
        if (threadIdx.x == 0) {
            P.active[g] = any;
            P.iters[g] = 0;
            P.counter[g] = 0;
        }
    }
}

// q = (S + alpha R) p (+ c' sum(p) on Neumann harmonics), pq = p.q
template <int KP, int VEC, int RB>
__global__ void __launch_bounds__(kThreads) k_spmm_dot(CgProblem P) {
    using Sh = Shape<KP, VEC>;
    const int g = blockIdx.y;
    if (!P.active[g]) return;
    const int slice = g / P.M;
    const Seg sg = segment(P, g - slice * P.M);
    const int T = P.tiles[0], nb = (sg.nblk + T - 1) / T;
    if ((int)blockIdx.x >= nb) return;
    const int f = slice / P.Ca, ci = slice % P.Ca;
    const bool dc = P.dcFree[ci] != 0;
    const float alpha = P.alpha[ci];
    const float2* SR = P.SR + (size_t)f * P.W * P.npad;
    const size_t vb = (size_t)slice * P.npad * KP;
    const float* p = P.p + vb;
    float* q = P.q + vb;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    float sp[VEC] = {};
    if (dc) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) sp[v] = (float)((double)sg.dcScale * P.sumP[(size_t)g * KP + j0 + v]);
    }
    DotAcc acc[1][VEC];
    const int tile0 = sg.tile0 + blockIdx.x * T;
    const int nsteps = (min(sg.tile0 + sg.nblk, tile0 + T) - tile0) * Sh::STEPS;
    for (int st = 0; st < nsteps; st += RB) {
        const int rowBase = (tile0 + st / Sh::STEPS) * kRowTile + warp * kRowsPerWarp +
                            (st % Sh::STEPS) * Sh::SUB + sub;
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) row[i] = rowBase + i * Sh::SUB;
        float y[RB][VEC];
        spmm_rows<KP, VEC, RB>(P.cols, SR, P.W, P.npad, alpha, p, j0, row, y);
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            if (row[i] < sg.end) {
#pragma unroll
                for (int v = 0; v < VEC; ++v) y[i][v] += sp[v];
            }
            stv<VEC>(q + (size_t)row[i] * KP + j0, y[i]);
            float pv[VEC];
            ldv<VEC>(p + (size_t)row[i] * KP + j0, pv);
#pragma unroll
            for (int v = 0; v < VEC; ++v) acc[0][v].add(pv[v], y[i][v]);
        }
    }
    double* const parts[1] = {P.partA};
    if (block_partials<KP, VEC, 1>(acc, parts, g, P.counter, nb)) {
        if (threadIdx.x < KP) P.pq[(size_t)g * KP + threadIdx.x] = sum_partials(P.partA, g, KP, threadIdx.x, nb);
        if (threadIdx.x == 0) P.counter[g] = 0;
    }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Dynamic shared memory of k_spmm_dot_staged: per warp, two buffers of its
// 16 rows' W column entries (int32) and W value entries (float2).
inline size_t staged_smem_bytes(int W) { return (size_t)2 * W * kRowTile * (sizeof(int32_t) + sizeof(float2)); }

// k_spmm_dot with the slot arrays in shared memory: every warp copies the W
// columns and values of its 16 rows of tile t + 1 (16-byte cp.async chunks:
// 64 B of columns and 128 B of values per slot, aligned because tiles start
// at multiples of 128 rows) while it multiplies tile t, so a row's only
// global latency is the gather of p; warps synchronise only with themselves.
template <int KP, int VEC, int RB>
__global__ void __launch_bounds__(kThreads) k_spmm_dot_staged(CgProblem P) {
    using Sh = Shape<KP, VEC>;
    extern __shared__ __align__(16) unsigned char stageSmem[];
    const int g = blockIdx.y;
    if (!P.active[g]) return;
    const int slice = g / P.M;
    const Seg sg = segment(P, g - slice * P.M);
    const int T = P.tiles[0], nb = (sg.nblk + T - 1) / T;
    if ((int)blockIdx.x >= nb) return;
    const int f = slice / P.Ca, ci = slice % P.Ca;
    const bool dc = P.dcFree[ci] != 0;
    const float alpha = P.alpha[ci];
    const int W = P.W;
    const float2* SR = P.SR + (size_t)f * W * P.npad;
    const size_t vb = (size_t)slice * P.npad * KP;
    const float* p = P.p + vb;
    float* q = P.q + vb;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    // this warp's buffers: [2][W][16] columns, then [2][W][16] values
    int32_t* cs = reinterpret_cast<int32_t*>(stageSmem) + (size_t)warp * 2 * W * kRowsPerWarp;
    float2* vs = reinterpret_cast<float2*>(stageSmem + (size_t)2 * W * kRowTile * sizeof(int32_t)) +
                 (size_t)warp * 2 * W * kRowsPerWarp;
    float sp[VEC] = {};
    if (dc) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) sp[v] = (float)((double)sg.dcScale * P.sumP[(size_t)g * KP + j0 + v]);
    }
    DotAcc acc[1][VEC];
    const int tile0 = sg.tile0 + blockIdx.x * T;
    const int tileEnd = min(sg.tile0 + sg.nblk, tile0 + T);
    constexpr int kColChunks = kRowsPerWarp / 4, kValChunks = kRowsPerWarp / 2;  // 16-byte chunks per slot
    auto stage = [&](int tile, int buf) {
        const size_t r0 = (size_t)tile * kRowTile + warp * kRowsPerWarp;
        for (int c = lane; c < W * (kColChunks + kValChunks); c += 32) {
            if (c < W * kColChunks) {
                const int k = c / kColChunks, o = (c % kColChunks) * 4;
                cp_async16(cs + (buf * W + k) * kRowsPerWarp + o, P.cols + (size_t)k * P.npad + r0 + o);
            } else {
                const int cv = c - W * kColChunks;
                const int k = cv / kValChunks, o = (cv % kValChunks) * 2;
                cp_async16(vs + (buf * W + k) * kRowsPerWarp + o, SR + (size_t)k * P.npad + r0 + o);
            }
        }
        cp_async_commit();
    };
    stage(tile0, 0);
    for (int t = tile0; t < tileEnd; ++t) {
        const int buf = (t - tile0) & 1;
        if (t + 1 < tileEnd) {
            stage(t + 1, buf ^ 1);
            cp_async_wait1();
        } else {
            cp_async_wait0();
        }
        __syncwarp();
        const int32_t* ct = cs + buf * W * kRowsPerWarp;
        const float2* vt = vs + buf * W * kRowsPerWarp;
        for (int st = 0; st < Sh::STEPS; st += RB) {
            int lr[RB];
#pragma unroll
            for (int i = 0; i < RB; ++i) lr[i] = (st + i) * Sh::SUB + sub;
            float y[RB][VEC];
#pragma unroll
            for (int i = 0; i < RB; ++i)
#pragma unroll
                for (int v = 0; v < VEC; ++v) y[i][v] = 0.f;
#pragma unroll
            for (int k = 0; k < kWFast; ++k) {
                if (k < W) {
#pragma unroll
                    for (int i = 0; i < RB; ++i) {
                        const int c = ct[k * kRowsPerWarp + lr[i]];
                        const float2 e = vt[k * kRowsPerWarp + lr[i]];
                        const float av = e.x + alpha * e.y;
                        float xv[VEC];
                        ldv<VEC>(p + (size_t)c * KP + j0, xv);
#pragma unroll
                        for (int v = 0; v < VEC; ++v) y[i][v] = fmaf(av, xv[v], y[i][v]);
                    }
                }
            }
            for (int k = kWFast; k < W; ++k) {
#pragma unroll
                for (int i = 0; i < RB; ++i) {
                    const int c = ct[k * kRowsPerWarp + lr[i]];
                    const float2 e = vt[k * kRowsPerWarp + lr[i]];
                    const float av = e.x + alpha * e.y;
                    float xv[VEC];
                    ldv<VEC>(p + (size_t)c * KP + j0, xv);
#pragma unroll
                    for (int v = 0; v < VEC; ++v) y[i][v] = fmaf(av, xv[v], y[i][v]);
                }
            }
#pragma unroll
            for (int i = 0; i < RB; ++i) {
                const int row = t * kRowTile + warp * kRowsPerWarp + lr[i];
                if (row < sg.end) {
#pragma unroll
                    for (int v = 0; v < VEC; ++v) y[i][v] += sp[v];
                }
                stv<VEC>(q + (size_t)row * KP + j0, y[i]);
                float pv[VEC];
                ldv<VEC>(p + (size_t)row * KP + j0, pv);
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc[0][v].add(pv[v], y[i][v]);
            }
        }
        __syncwarp();  // the next stage() overwrites this buffer
    }
    double* const parts[1] = {P.partA};
    if (block_partials<KP, VEC, 1>(acc, parts, g, P.counter, nb)) {
        if (threadIdx.x < KP) P.pq[(size_t)g * KP + threadIdx.x] = sum_partials(P.partA, g, KP, threadIdx.x, nb);
        if (threadIdx.x == 0) P.counter[g] = 0;
    }
}

// ---------------------------------------------------------------------------
// Tile-staged SpMM (k_spmm_halo).  The gathers of p are what limits the
// direct forms: each row reads W neighbour rows of KP floats through L1/L2,
// and the number of such loads a warp can keep in flight is bounded by its
// registers.  Here a block copies, per 128-row tile, everything the tile's
// products read into shared memory with bulk asynchronous copies (TMA,
// cp.async.bulk, completion counted on an mbarrier): the tile's own 128 rows
// of p (one contiguous copy), the W slot values {S, R} (one copy per slot)
// and the slots' tile-local columns; its halo rows (the distinct columns
// outside the tile) are gathered in 16-byte cp.async chunks by all threads,
// whose completion the same mbarrier counts (one bulk copy per 128-byte halo
// row was measured slower: the copy engine serialises small requests).  The
// arithmetic then reads only shared memory.  NS stages are in flight per
// block, so copies of tile t + NS - 1 overlap the products of tile t; on the
// ring meshes a tile's halo is about half its own rows, so p crosses from L2
// about 1.5 times per SpMM instead of once per slot.
constexpr int kHaloMaxSmem = 227 * 1024;
constexpr int kHaloMaxRows = 128;  // halo rows a tile may have (Hpad limit of the form)

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// A wait that ignores the abort flag, for draining copies already issued
// after another wait gave up (bounded by limitNs).
__device__ __forceinline__ bool mbar_wait_drain(uint32_t bar, uint32_t parity, uint64_t limitNs) {
    const uint64_t t0 = tc::global_timer();
    while (!tc::mbar_try_wait(bar, parity))
        if (tc::global_timer() - t0 > limitNs) return false;
    return true;
}

struct HaloLayout {
    uint32_t own, halo, sr, lc, stage;  // byte sizes of the parts of one stage
};
__host__ __device__ inline HaloLayout halo_layout(int KP, int W, int Hpad) {
    HaloLayout l;
    l.own = (uint32_t)kRowTile * KP * 4;
    l.halo = (uint32_t)Hpad * KP * 4;
    l.sr = (uint32_t)W * kRowTile * 8;
    l.lc = (uint32_t)((W * kRowTile * 2 + 15) / 16 * 16);
    l.stage = l.own + l.halo + l.sr + l.lc;
    return l;
}
inline size_t halo_smem_bytes(int KP, int W, int Hpad, int NS) {
    return (size_t)NS * halo_layout(KP, W, Hpad).stage + 16 * 8 /*mbarriers*/;
}

template <int KP, int VEC, int RB, int NS>
__global__ void __launch_bounds__(kThreads, 3) k_spmm_halo(CgProblem P) {
    using Sh = Shape<KP, VEC>;
    constexpr int kChunks = KP / 4;                                    // 16-byte chunks per row of p
    constexpr int kPer = (kHaloMaxRows * kChunks + kThreads - 1) / kThreads;  // halo chunks per thread
    extern __shared__ __align__(128) unsigned char hsm[];
    __shared__ int localAbort, amLast;
    const int g = blockIdx.y;
    if (!P.active[g]) return;
    const int slice = g / P.M;
    const Seg sg = segment(P, g - slice * P.M);
    const int T = P.tiles[0], nb = (sg.nblk + T - 1) / T;
    if ((int)blockIdx.x >= nb) return;
    const int f = slice / P.Ca, ci = slice % P.Ca;
    const bool dc = P.dcFree[ci] != 0;
    const float alpha = P.alpha[ci];
    const int W = P.W;
    const float2* SR = P.SR + (size_t)f * W * P.npad;
    const size_t vb = (size_t)slice * P.npad * KP;
    const float* p = P.p + vb;
    float* q = P.q + vb;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    const HaloLayout L = halo_layout(KP, W, P.Hpad);
    const uint32_t smem0 = tc::smem_u32(hsm);
    const uint32_t bar0 = smem0 + NS * L.stage;  // NS mbarriers, 8 bytes each
    if (threadIdx.x == 0) {
        localAbort = 0;
        for (int s = 0; s < NS; ++s) tc::mbar_init(bar0 + 8 * s, 1 + kThreads);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    float sp[VEC] = {};
    if (dc) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) sp[v] = (float)((double)sg.dcScale * P.sumP[(size_t)g * KP + j0 + v]);
    }
    const int tile0 = sg.tile0 + blockIdx.x * T;
    const int tileEnd = min(sg.tile0 + sg.nblk, tile0 + T);
    // halo row of each of this thread's chunks (-1: none), loaded one tile
    // ahead of the copies that use them so their latency is hidden
    int hrow[kPer];
    auto prefetch = [&](int t) {
        const int32_t* hl = P.halo + (size_t)t * P.Hpad;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int i = (threadIdx.x + j * kThreads) / kChunks;
            hrow[j] = i < P.Hpad ? __ldg(&hl[i]) : -1;
        }
    };
    // all threads: thread 0 arms stage s's barrier with the bulk byte count and
    // lanes 0..W+1 of warp 0 issue the bulk copies (own rows, local columns,
    // slot values); every thread copies its 16-byte chunks of the halo rows
    // with cp.async and has the barrier count their completion (one arrival
    // per thread, so the barrier's count is 1 + kThreads)
    auto issue = [&](int t, int s) {
        const uint32_t st = smem0 + s * L.stage, bar = bar0 + 8 * s;
        if (warp == 0) {
            if (lane == 0) tc::mbar_expect_tx(bar, L.own + L.sr + (uint32_t)W * kRowTile * 2);
            __syncwarp();
            if (lane == 0) bulk_g2s(st, p + (size_t)t * kRowTile * KP, L.own, bar);
            if (lane == 1)
                bulk_g2s(st + L.own + L.halo + L.sr, P.lcol + (size_t)t * W * kRowTile, W * kRowTile * 2, bar);
            if (lane >= 2 && lane < 2 + W)
                bulk_g2s(st + L.own + L.halo + (lane - 2) * kRowTile * 8,
                         SR + (size_t)(lane - 2) * P.npad + (size_t)t * kRowTile, kRowTile * 8, bar);
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int c = threadIdx.x + j * kThreads, i = c / kChunks, part = c % kChunks;
            if (hrow[j] >= 0)
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(st + L.own + (uint32_t)(i * KP + part * 4) * 4),
                             "l"(p + (size_t)hrow[j] * KP + part * 4)
                             : "memory");
        }
        asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
    };
    int issued = 0;
    for (int j = 0; j < NS - 1 && tile0 + j < tileEnd; ++j) {
        prefetch(tile0 + j);
        issue(tile0 + j, j);
        ++issued;
    }
    if (tile0 + NS - 1 < tileEnd) prefetch(tile0 + NS - 1);
    DotAcc acc[1][VEC];
    bool failed = false;
    int consumed = 0;
    for (int t = tile0; t < tileEnd; ++t, ++consumed) {
        // every warp is done with the stage the next copies overwrite (the
        // tile before this one), and all agree whether a wait gave up
        if (__syncthreads_or(failed)) break;
        if (t + NS - 1 < tileEnd) {
            issue(t + NS - 1, (consumed + NS - 1) % NS);
            ++issued;
            if (t + NS < tileEnd) prefetch(t + NS);
        }
        const int s = consumed % NS;
        failed = !tc::mbar_wait(bar0 + 8 * s, (consumed / NS) & 1, &localAbort);
        if (failed) continue;
        const unsigned char* base = hsm + (size_t)s * L.stage;
        const float* rowsS = reinterpret_cast<const float*>(base);  // own rows, then halo rows
        const float2* vt = reinterpret_cast<const float2*>(base + L.own + L.halo);
        const uint16_t* ct = reinterpret_cast<const uint16_t*>(base + L.own + L.halo + L.sr);
        float tp[VEC] = {};  // this tile's p.q terms (FP32), folded into acc once per tile
        for (int st = 0; st < Sh::STEPS; st += RB) {
            int lr[RB];
#pragma unroll
            for (int i = 0; i < RB; ++i) lr[i] = warp * kRowsPerWarp + (st + i) * Sh::SUB + sub;
            float y[RB][VEC];
#pragma unroll
            for (int i = 0; i < RB; ++i)
#pragma unroll
                for (int v = 0; v < VEC; ++v) y[i][v] = 0.f;
            // the first kWFast slots: all columns and values first, then the gathers
            int c[kWFast][RB];
            float av[kWFast][RB];
#pragma unroll
            for (int k = 0; k < kWFast; ++k)
#pragma unroll
                for (int i = 0; i < RB; ++i) {
                    c[k][i] = k < W ? (int)ct[k * kRowTile + lr[i]] : lr[i];
                    const float2 e = k < W ? vt[k * kRowTile + lr[i]] : make_float2(0.f, 0.f);
                    av[k][i] = e.x + alpha * e.y;
                }
#pragma unroll
            for (int k = 0; k < kWFast; ++k) {
                if (k < W) {
#pragma unroll
                    for (int i = 0; i < RB; ++i) {
                        float xv[VEC];
                        ldv<VEC>(rowsS + (size_t)c[k][i] * KP + j0, xv);
#pragma unroll
                        for (int v = 0; v < VEC; ++v) y[i][v] = fmaf(av[k][i], xv[v], y[i][v]);
                    }
                }
            }
            for (int k = kWFast; k < W; ++k) {
#pragma unroll
                for (int i = 0; i < RB; ++i) {
                    const int cc = ct[k * kRowTile + lr[i]];
                    const float2 e = vt[k * kRowTile + lr[i]];
                    const float a = e.x + alpha * e.y;
                    float xv[VEC];
                    ldv<VEC>(rowsS + (size_t)cc * KP + j0, xv);
#pragma unroll
                    for (int v = 0; v < VEC; ++v) y[i][v] = fmaf(a, xv[v], y[i][v]);
                }
            }
#pragma unroll
            for (int i = 0; i < RB; ++i) {
                const int row = t * kRowTile + lr[i];
                if (row < sg.end) {
#pragma unroll
                    for (int v = 0; v < VEC; ++v) y[i][v] += sp[v];
                }
                stv<VEC>(q + (size_t)row * KP + j0, y[i]);
                float pv[VEC];
                ldv<VEC>(rowsS + (size_t)lr[i] * KP + j0, pv);
#pragma unroll
                for (int v = 0; v < VEC; ++v) tp[v] = fmaf(pv[v], y[i][v], tp[v]);
            }
        }
#pragma unroll
        for (int v = 0; v < VEC; ++v) acc[0][v].addf(tp[v]);
    }
    if (__syncthreads_or(failed)) {
        // a wait gave up: let the copies this block issued land (bounded)
        // before the block exits, then report; the result is undefined
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (threadIdx.x == 0) {
            for (int j = consumed > 0 ? consumed - 1 : 0; j < issued; ++j)
                if (!mbar_wait_drain(bar0 + 8 * (j % NS), (j / NS) & 1, 1000000000ull)) break;
            if (P.abortFlag) atomicExch(P.abortFlag, 1);
        }
        __syncthreads();
        return;
    }
    // the stages are free again: reduce through their shared memory
    double* const parts[1] = {P.partA};
    if (block_partials_in<KP, VEC, 1>(acc, parts, g, P.counter, nb, reinterpret_cast<double*>(hsm), &amLast)) {
        if (threadIdx.x < KP) P.pq[(size_t)g * KP + threadIdx.x] = sum_partials(P.partA, g, KP, threadIdx.x, nb);
        if (threadIdx.x == 0) P.counter[g] = 0;
    }
}

// x += a p, r -= a q, z = D^-1 r, rz' = r.z; the last block updates the
// scalars, the convergence mask and the group's active flag.
template <int KP, int VEC, int RB>
__global__ void __launch_bounds__(kThreads) k_update(CgProblem P) {
    using Sh = Shape<KP, VEC>;
    const int g = blockIdx.y;
    if (!P.active[g]) return;
    const int slice = g / P.M;
    const Seg sg = segment(P, g - slice * P.M);
    const int T = P.tiles[1], nb = (sg.nblk + T - 1) / T;
    if ((int)blockIdx.x >= nb) return;
    const int f = slice / P.Ca, ci = slice % P.Ca;
    const float alpha = P.alpha[ci];
    const float2* SR = P.SR + (size_t)f * P.W * P.npad;
    const size_t vb = (size_t)slice * P.npad * KP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    float a[VEC];
#pragma unroll
    for (int v = 0; v < VEC; ++v) {
        const size_t s = (size_t)g * KP + j0 + v;
        const double pq = P.pq[s];
        a[v] = (!P.conv[s] && pq != 0.0) ? (float)(P.rz[s] / pq) : 0.f;
    }
    DotAcc acc[1][VEC];
    float rsum[VEC] = {};
    // r.D^-1 r: its terms are never negative, so each thread sums a tile's
    // terms in FP32 (no cancellation) and folds that sum into the
    // compensated pair once per tile
    float rz[VEC] = {};
    __shared__ float red[kWarps * 32 * VEC];
    const int tile0 = sg.tile0 + blockIdx.x * T;
    const int nsteps = (min(sg.tile0 + sg.nblk, tile0 + T) - tile0) * Sh::STEPS;
    for (int st = 0; st < nsteps; st += RB) {
        const int rowBase = (tile0 + st / Sh::STEPS) * kRowTile + warp * kRowsPerWarp +
                            (st % Sh::STEPS) * Sh::SUB + sub;
        float rv[RB][VEC], qv[RB][VEC], di[RB];
        size_t o[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const int row = rowBase + i * Sh::SUB;
            o[i] = vb + (size_t)row * KP + j0;
            ldv<VEC>(P.r + o[i], rv[i]);
            ldv<VEC>(P.q + o[i], qv[i]);
            di[i] = diag_inv(SR, P.diagSlot, P.npad, row, alpha);
        }
#pragma unroll
        for (int i = 0; i < RB; ++i) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                rv[i][v] = fmaf(-a[v], qv[i][v], rv[i][v]);
                rz[v] = fmaf(rv[i][v], di[i] * rv[i][v], rz[v]);
                rsum[v] += rv[i][v];  // padding rows keep r = 0
            }
            stv<VEC>(P.r + o[i], rv[i]);
        }
        if ((st % Sh::STEPS) + RB == Sh::STEPS) {  // end of a tile
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                acc[0][v].addf(rz[v]);
                rz[v] = 0.f;
            }
        }
        if (P.coarse && (st % Sh::STEPS) + RB == Sh::STEPS) {
            restrict_tile<KP, VEC>(rsum, tile0 - sg.tile0 + st / Sh::STEPS, seg_aggregates(sg),
                                   P.rc + (size_t)g * P.ncPad * KP, red);
#pragma unroll
            for (int v = 0; v < VEC; ++v) rsum[v] = 0.f;
        }
    }
#pragma unroll
    for (int v = 0; v < VEC; ++v) acc[0][v].addf(rz[v]);  // terms after the last tile end (if any)
    double* const parts[1] = {P.partA};
    if (block_partials<KP, VEC, 1>(acc, parts, g, P.counter, nb)) {
        // the step length of this iteration, for the deferred x update
        if (threadIdx.x < KP) {
            const size_t s = (size_t)g * KP + threadIdx.x;
            const double pq = P.pq[s];
            P.alphaX[s] = (!P.conv[s] && pq != 0.0) ? (double)(float)(P.rz[s] / pq) : 0.0;
        }
        if (threadIdx.x == 0) P.pend[g] = 1;
        if (P.coarse) {
            if (threadIdx.x < KP)
                P.rzFine[(size_t)g * KP + threadIdx.x] = sum_partials(P.partA, g, KP, threadIdx.x, nb);
            if (threadIdx.x == 0) P.counter[g] = 0;
            return;
        }
        int notConv = 0;
        if (threadIdx.x < KP) {
            const size_t s = (size_t)g * KP + threadIdx.x;
            if (!P.conv[s]) {
                const double rzn = sum_partials(P.partA, g, KP, threadIdx.x, nb);
                const double rzo = P.rz[s];
                P.beta[s] = rzo != 0.0 ? rzn / rzo : 0.0;
                P.rz[s] = rzn;
                const int c = rzn <= P.tol2 * P.bz[s];
                P.conv[s] = c;
                notConv = !c;
            }
        }
        int any = __syncthreads_or(notConv);
        if (threadIdx.x == 0) {
            P.active[g] = any;
            P.iters[g] += 1;
            P.counter[g] = 0;
        }
    }
}

// x += alphaX p_old (the step of the update just made), p = D^-1 r + beta p
// on the right-hand sides still iterating; Neumann harmonics also reduce
// sum(p) for the next SpMM.
template <int KP, int VEC, int RB>
__global__ void __launch_bounds__(kThreads) k_direction(CgProblem P) {
    using Sh = Shape<KP, VEC>;
    const int g = blockIdx.y;
    if (!P.active[g]) return;
    const int slice = g / P.M;
    const Seg sg = segment(P, g - slice * P.M);
    const int T = P.tiles[2], nb = (sg.nblk + T - 1) / T;
    if ((int)blockIdx.x >= nb) return;
    const int f = slice / P.Ca, ci = slice % P.Ca;
    const bool dc = P.dcFree[ci] != 0;
    const float alpha = P.alpha[ci];
    const float2* SR = P.SR + (size_t)f * P.W * P.npad;
    const size_t vb = (size_t)slice * P.npad * KP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    float be[VEC], ax[VEC];
    bool live[VEC];
#pragma unroll
    for (int v = 0; v < VEC; ++v) {
        const size_t s = (size_t)g * KP + j0 + v;
        live[v] = P.first || !P.conv[s];
        be[v] = P.first ? 0.f : (float)P.beta[s];
        ax[v] = P.first ? 0.f : (float)P.alphaX[s];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) P.pend[g] = 0;  // x is brought up to date below
    DotAcc acc[1][VEC];
    const int tile0 = sg.tile0 + blockIdx.x * T;
    const int nsteps = (min(sg.tile0 + sg.nblk, tile0 + T) - tile0) * Sh::STEPS;
    for (int st = 0; st < nsteps; st += RB) {
        const int rowBase = (tile0 + st / Sh::STEPS) * kRowTile + warp * kRowsPerWarp +
                            (st % Sh::STEPS) * Sh::SUB + sub;
        float rv[RB][VEC], pv[RB][VEC], di[RB], yv[VEC] = {};
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            row[i] = rowBase + i * Sh::SUB;
            const size_t o = vb + (size_t)row[i] * KP + j0;
            ldv<VEC>(P.r + o, rv[i]);
            if (P.first) {
#pragma unroll
                for (int v = 0; v < VEC; ++v) pv[i][v] = 0.f;
            } else {
                ldv<VEC>(P.p + o, pv[i]);
                float xv[VEC];
                ldv<VEC>(P.x + o, xv);
#pragma unroll
                for (int v = 0; v < VEC; ++v) xv[v] = fmaf(ax[v], pv[i][v], xv[v]);
                stv<VEC>(P.x + o, xv);
            }
            di[i] = diag_inv(SR, P.diagSlot, P.npad, row[i], alpha);
        }
        // coarse correction: all rows of a warp step lie in one aggregate
        if (P.coarse && rowBase < sg.end)
            ldv<VEC>(P.yc + ((size_t)g * P.ncPad + (rowBase - sg.tile0 * kRowTile) / kAgg) * KP + j0, yv);
#pragma unroll
        for (int i = 0; i < RB; ++i) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                const float z = fmaf(di[i], rv[i][v], row[i] < sg.end ? yv[v] : 0.f);
                pv[i][v] = live[v] ? fmaf(be[v], pv[i][v], z) : pv[i][v];
                if (dc && row[i] < sg.end) acc[0][v].add(pv[i][v], 1.f);
            }
            stv<VEC>(P.p + vb + (size_t)row[i] * KP + j0, pv[i]);
        }
    }
    if (!dc) return;
    double* const parts[1] = {P.partA};
    if (block_partials<KP, VEC, 1>(acc, parts, g, P.counter, nb)) {
        if (threadIdx.x < KP)
            P.sumP[(size_t)g * KP + threadIdx.x] = sum_partials(P.partA, g, KP, threadIdx.x, nb);
        if (threadIdx.x == 0) P.counter[g] = 0;
    }
}

// x += alphaX p on the groups whose last x update is pending (they retired
// in k_update, so k_direction skipped them); pend is cleared by the caller.
template <int KP>
__global__ void __launch_bounds__(kThreads) k_finalize_x(CgProblem P) {
    constexpr int VEC = KP >= 32 ? 4 : 2;
    using Sh = Shape<KP, VEC>;
    const int g = blockIdx.y;
    if (!P.pend[g]) return;
    const int slice = g / P.M;
    const Seg sg = segment(P, g - slice * P.M);
    if ((int)blockIdx.x >= sg.nblk) return;
    const size_t vb = (size_t)slice * P.npad * KP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    float ax[VEC];
#pragma unroll
    for (int v = 0; v < VEC; ++v) ax[v] = (float)P.alphaX[(size_t)g * KP + j0 + v];
    const int rowBase = (sg.tile0 + blockIdx.x) * kRowTile + warp * kRowsPerWarp + sub;
    for (int st = 0; st < Sh::STEPS; ++st) {
        const size_t o = vb + (size_t)(rowBase + st * Sh::SUB) * KP + j0;
        float xv[VEC], pv[VEC];
        ldv<VEC>(P.x + o, xv);
        ldv<VEC>(P.p + o, pv);
#pragma unroll
        for (int v = 0; v < VEC; ++v) xv[v] = fmaf(ax[v], pv[v], xv[v]);
        stv<VEC>(P.x + o, xv);
    }
}

// ---------------------------------------------------------------------------
// FP64 refinement: r64 = b64 - (S64 + alpha R64) x64 (- c' sum(x64) on
// Neumann harmonics), written as the float right-hand side of the next inner
// solve; rr = |r64|^2, bb = |b64|^2.
template <int KP>
__global__ void __launch_bounds__(kThreads) k_residual64(CgProblem P, const double* S64, const double* R64,
                                                         const double* x64, const double* b64,
                                                         const double* sumX64, float* rOut, double* partR,
                                                         double* partB, double* rr, double* bb) {
    constexpr int VEC = KP >= 32 ? 4 : 2;
    using Sh = Shape<KP, VEC>;
    const int g = blockIdx.y;
    const int f = g / P.Ca, ci = g % P.Ca;
    const bool dc = P.dcFree[ci] != 0;
    const double alpha = (double)P.alpha[ci];
    const double* S = S64 + (size_t)f * P.W * P.npad;
    const double* R = R64 + (size_t)f * P.W * P.npad;
    const size_t vb = (size_t)g * P.npad * KP;
    b64 += (size_t)ci * P.npad * KP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / Sh::LPR, j0 = (lane % Sh::LPR) * VEC;
    double sx[VEC] = {};
    if (dc) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) sx[v] = (double)P.dcScale * sumX64[(size_t)g * KP + j0 + v];
    }
    double accR[VEC] = {}, accB[VEC] = {};
    const int rowBase = blockIdx.x * kRowTile + warp * kRowsPerWarp;
    for (int st = 0; st < Sh::STEPS; ++st) {
        const int row = rowBase + st * Sh::SUB + sub;
        double y[VEC] = {};
        for (int k = 0; k < P.W; ++k) {
            const int col = __ldg(&P.cols[(size_t)k * P.npad + row]);
            const double a = S[(size_t)k * P.npad + row] + alpha * R[(size_t)k * P.npad + row];
#pragma unroll
            for (int v = 0; v < VEC; ++v) y[v] = fma(a, x64[vb + (size_t)col * KP + j0 + v], y[v]);
        }
        float ro[VEC];
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const double bv = b64[(size_t)row * KP + j0 + v];
            const double rv = bv - y[v] - (row < P.n ? sx[v] : 0.0);
            ro[v] = (float)rv;
            accR[v] = fma(rv, rv, accR[v]);
            accB[v] = fma(bv, bv, accB[v]);
        }
        stv<VEC>(rOut + vb + (size_t)row * KP + j0, ro);
    }
    __shared__ double red[2][kWarps * Sh::SUB][KP];
    __shared__ bool amLast;
#pragma unroll
    for (int v = 0; v < VEC; ++v) {
        red[0][warp * Sh::SUB + sub][j0 + v] = accR[v];
        red[1][warp * Sh::SUB + sub][j0 + v] = accB[v];
    }
    __syncthreads();
    if (threadIdx.x < KP) {
        double s0 = 0.0, s1 = 0.0;
        for (int w = 0; w < kWarps * Sh::SUB; ++w) {
            s0 += red[0][w][threadIdx.x];
            s1 += red[1][w][threadIdx.x];
        }
        partR[((size_t)g * P.nblk + blockIdx.x) * KP + threadIdx.x] = s0;
        partB[((size_t)g * P.nblk + blockIdx.x) * KP + threadIdx.x] = s1;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) amLast = atomicAdd(&P.counter[g], 1u) == (unsigned)(P.nblk - 1);
    __syncthreads();
    if (amLast) {
        __threadfence();
        if (threadIdx.x < KP) {
            rr[(size_t)g * KP + threadIdx.x] = sum_partials(partR, g, KP, threadIdx.x, P.nblk);
            bb[(size_t)g * KP + threadIdx.x] = sum_partials(partB, g, KP, threadIdx.x, P.nblk);
        }
        if (threadIdx.x == 0) P.counter[g] = 0;
    }
}

__global__ void k_accumulate64(size_t count, const float* x, double* x64) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        x64[i] += (double)x[i];
}

__global__ void k_to_float(size_t count, const double* x64, float* x) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        x[i] = (float)x64[i];
}

// x += sign * shift[j] on the real rows of every Neumann group: converts
// between the solution of (A + c' 1 1^T) x = b and the reference's
// (A + 1 1^T) x = b, which differ only by (sum(b) / n^2)(1 - 1/c') 1.
// shift: [M][KP], one row per stacked mesh.
__global__ void k_dc_shift(CgProblem P, const double* shift, float sign) {
    const int g = blockIdx.y;
    const int slice = g / P.M, mesh = g - slice * P.M;
    if (!P.dcFree[slice % P.Ca]) return;
    const Seg sg = segment(P, mesh);
    const size_t vb = ((size_t)slice * P.npad + (size_t)sg.tile0 * kRowTile) * P.KP;
    const size_t count = (size_t)(sg.end - sg.tile0 * kRowTile) * P.KP;
    shift += (size_t)mesh * P.KP;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        P.x[vb + i] += sign * (float)shift[i % P.KP];
}

// Column sums over the real rows of every Neumann group (0 elsewhere); one
// block per group, fixed summation order.
template <class T>
__global__ void __launch_bounds__(kThreads) k_colsum(int n, int npad, int KP, int Ca, const int* dcFree,
                                                     const T* x, double* sums) {
    const int g = blockIdx.x;
    __shared__ double red[kThreads];
    const int lanes = kThreads / KP;
    const int j = threadIdx.x % KP, r0 = threadIdx.x / KP;
    double s = 0.0;
    if (dcFree[g % Ca]) {
        const T* xg = x + (size_t)g * npad * KP;
        for (int r = r0; r < n; r += lanes) s += (double)xg[(size_t)r * KP + j];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < KP) {
        double t = 0.0;
        for (int l = 0; l < lanes; ++l) t += red[l * KP + threadIdx.x];
        sums[(size_t)g * KP + threadIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
// Variant table: variant v = vecIdx * 3 + rbIdx with VEC in {4, 2, 1} and
// RB in {1, 2, 4} (SpMM: v + 9 for the shared-memory-staged form); entries
// whose lane mapping or step count does not fit the right-hand-side width
// are null.
using CgKernel = void (*)(CgProblem);

template <int KP, int VEC, int RB>
constexpr bool valid_variant() {
    return KP / VEC <= 32 && (kRowsPerWarp / (32 / (KP / VEC))) % RB == 0 && (kRowsPerWarp / (32 / (KP / VEC))) >= RB;
}

template <int KP, int VEC, int RB>
void fill_variant(CgKernel (&t)[3][kSpmmForms * kCgVariants], int v) {
    if constexpr (KP / VEC <= 32) {
        if constexpr (valid_variant<KP, VEC, RB>()) {
            t[0][v] = k_spmm_dot<KP, VEC, RB>;
            t[0][v + kCgVariants] = k_spmm_dot_staged<KP, VEC, RB>;
            t[1][v] = k_update<KP, VEC, RB>;
            t[2][v] = k_direction<KP, VEC, RB>;
            // tile-staged form: 2 or 3 stages, right-hand-side widths up to 64
            // (a 128-wide tile needs 64 KB of own rows per stage)
            if constexpr (KP <= 64 && VEC >= 2 && RB <= 2) {
                t[0][v + 2 * kCgVariants] = k_spmm_halo<KP, VEC, RB, 2>;
                t[0][v + 3 * kCgVariants] = k_spmm_halo<KP, VEC, RB, 3>;
            }
        }
    }
}

template <int KP>
struct VariantTable {
    CgKernel k[3][kSpmmForms * kCgVariants] = {};
    VariantTable() {
        fill_variant<KP, 4, 1>(k, 0);
        fill_variant<KP, 4, 2>(k, 1);
        fill_variant<KP, 4, 4>(k, 2);
        fill_variant<KP, 2, 1>(k, 3);
        fill_variant<KP, 2, 2>(k, 4);
        fill_variant<KP, 2, 4>(k, 5);
        fill_variant<KP, 1, 1>(k, 6);
        fill_variant<KP, 1, 2>(k, 7);
        fill_variant<KP, 1, 4>(k, 8);
    }
};

CgKernel variant_kernel(int KP, int which, int v) {
    static const VariantTable<16> t16;
    static const VariantTable<32> t32;
    static const VariantTable<64> t64;
    static const VariantTable<128> t128;
    if (v < 0 || v >= kSpmmForms * kCgVariants || which < 0 || which > 2) return nullptr;
    switch (KP) {
        case 16: return t16.k[which][v];
        case 32: return t32.k[which][v];
        case 64: return t64.k[which][v];
        case 128: return t128.k[which][v];
        default: return nullptr;
    }
}

template <template <int> class Launcher, class... Args>
int dispatch_kp(int KP, Args&&... args) {
    switch (KP) {
        case 16: return Launcher<16>::run(args...);
        case 32: return Launcher<32>::run(args...);
        case 64: return Launcher<64>::run(args...);
        case 128: return Launcher<128>::run(args...);
        default: return fail(MPF_EINVAL, "unsupported right-hand-side width %d", KP);
    }
}

template <int KP>
struct InitL {
    static int run(const CgProblem& P, bool zeroGuess, cudaStream_t s) {
        k_init<KP><<<dim3(P.nblk, P.G), kThreads, 0, s>>>(P, zeroGuess ? 1 : 0);
        MPF_LAUNCHED(1);
        return MPF_OK;
    }
};
template <int KP>
struct FinalizeL {
    static int run(const CgProblem& P, cudaStream_t s) {
        k_finalize_x<KP><<<dim3(P.nblk, P.G), kThreads, 0, s>>>(P);
        MPF_LAUNCHED(1);
        MPF_CUDA(cudaMemsetAsync(P.pend, 0, sizeof(int) * P.G, s));
        return MPF_OK;
    }
};
template <int KP>
struct Res64L {
    static int run(const CgProblem& P, const double* S64, const double* R64, const double* x64,
                   const double* b64, const double* sumX64, double* partR, double* partB, double* rr,
                   double* bb, cudaStream_t s) {
        k_residual64<KP><<<dim3(P.nblk, P.G), kThreads, 0, s>>>(P, S64, R64, x64, b64, sumX64, P.r, partR,
                                                                 partB, rr, bb);
        MPF_LAUNCHED(1);
        return MPF_OK;
    }
};

}  // namespace

bool cg_variant_valid(int KP, int which, int v) { return variant_kernel(KP, which, v) != nullptr; }

int cg_shape_count(int which) {
    return which == 0 ? kSpmmForms * kCgVariants * kCgTileChoices : kCgVariants * kCgTileChoices;
}

int cg_spmm_form(int code) { return code / (kCgVariants * kCgTileChoices); }

bool cg_shape_fits(int KP, int W, int Hpad, bool haveHalo, int which, int code) {
    if (!cg_shape_valid(KP, which, code)) return false;
    if (which != 0 || cg_spmm_form(code) < 2) return true;
    const int NS = cg_spmm_form(code);
    return haveHalo && Hpad > 0 && Hpad <= kHaloMaxRows && halo_smem_bytes(KP, W, Hpad, NS) <= (size_t)kHaloMaxSmem;
}

bool cg_shape_valid(int KP, int which, int code) {
    if (code < 0 || code >= cg_shape_count(which)) return false;
    const int group = kCgVariants * kCgTileChoices;
    return cg_variant_valid(KP, which, code % kCgVariants + kCgVariants * (code / group));
}

int cg_shape_code(const CgProblem& P, int which) {
    const int v = P.variant[which];
    const int shift = (which == 0 && v >= 2 * kCgVariants) ? 2 : 0;  // see cg_set_shape
    return v % kCgVariants + kCgVariants * (31 - __builtin_clz(P.tiles[which]) - shift) +
           kCgVariants * kCgTileChoices * (v / kCgVariants);
}

int cg_default_variant(int KP) { return KP <= 64 ? 1 : 0; }  // VEC 4, RB 2 (KP 128: RB 1)

static int launch_one(const CgProblem& P, int which, cudaStream_t s, bool count);

// Start of a solve: r0, and with the two-level preconditioner the coarse
// solve and p0 = M^-1 r0 (the direction kernel with beta = 0).
int cg_launch_init(const CgProblem& P, bool zeroGuess, cudaStream_t s) {
    if (P.solver == 1) return bicgstab_launch_init(P, zeroGuess, s);
    if (P.solver == 2) {
        MPF_CHECK(zeroGuess, MPF_ENOTSUP, "complex admittivity: warm starts are not implemented");
        return zbicgstab_launch_init(P, s);
    }
    MPF_TRY(dispatch_kp<InitL>(P.KP, P, zeroGuess, s));
    if (!P.coarse) return MPF_OK;
    MPF_TRY(cg_launch_coarse(P, true, s));
    CgProblem Q = P;
    Q.first = 1;
    return launch_one(Q, 2, s, true);
}

// One CG iteration with the problem's chosen variants; `count` says whether
// the launches are real (false while recording a CUDA graph, whose replays
// are counted by the caller).
static int launch_one(const CgProblem& P, int which, cudaStream_t s, bool count) {
    const int v = P.variant[which];
    CgKernel k = variant_kernel(P.KP, which, v);
    MPF_CHECK(k != nullptr, MPF_EINVAL, "CG kernel variant %d not available for %d right-hand sides", v, P.KP);
    const int t = P.tiles[which] >= 1 ? P.tiles[which] : 1;
    size_t smem = 0;
    if (which == 0 && v >= 2 * kCgVariants) {
        const int NS = v / kCgVariants;
        MPF_CHECK(P.halo && P.hcnt && P.lcol && P.Hpad > 0, MPF_EINVAL, "tile-staged SpMM: the problem has no halo plan");
        MPF_CHECK(P.Hpad <= kHaloMaxRows, MPF_EINVAL, "tile-staged SpMM: %d halo rows per tile exceed %d", P.Hpad,
                  kHaloMaxRows);
        smem = halo_smem_bytes(P.KP, P.W, P.Hpad, NS);
        MPF_CHECK(smem <= (size_t)kHaloMaxSmem, MPF_EINVAL,
                  "tile-staged SpMM: %zu bytes of shared memory per block (%d halo rows, %d slots) exceed %d", smem,
                  P.Hpad, P.W, kHaloMaxSmem);
        // the attribute is set outside stream capture (cg_prepare_launch runs
        // before a graph of iterations is recorded)
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        MPF_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs == cudaStreamCaptureStatusNone)
            MPF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    } else if (which == 0 && v >= kCgVariants) {
        smem = staged_smem_bytes(P.W);
        MPF_CHECK(smem <= 200 * 1024, MPF_EINVAL, "staged SpMM: %d ELL slots do not fit shared memory", P.W);
        if (smem > 48 * 1024)
            MPF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    k<<<dim3((P.nblk + t - 1) / t, P.G), kThreads, smem, s>>>(P);
    if (count) {
        MPF_LAUNCHED(1);
    } else {
        MPF_CUDA(cudaGetLastError());
    }
    return MPF_OK;
}

int cg_prepare_launch(const CgProblem& P) {
    if (P.solver != 0) return MPF_OK;
    const int v = P.variant[0];
    CgKernel k = variant_kernel(P.KP, 0, v);
    MPF_CHECK(k != nullptr, MPF_EINVAL, "CG kernel variant %d not available for %d right-hand sides", v, P.KP);
    size_t smem = 0;
    if (v >= 2 * kCgVariants) {
        MPF_CHECK(P.halo && P.Hpad > 0, MPF_EINVAL, "tile-staged SpMM: the problem has no halo plan");
        smem = halo_smem_bytes(P.KP, P.W, P.Hpad, v / kCgVariants);
        MPF_CHECK(smem <= (size_t)kHaloMaxSmem, MPF_EINVAL, "tile-staged SpMM: %zu bytes of shared memory", smem);
    } else if (v >= kCgVariants) {
        smem = staged_smem_bytes(P.W);
    }
    if (smem > 48 * 1024) MPF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return MPF_OK;
}

int cg_launch_iteration(const CgProblem& P, cudaStream_t s) {
    if (P.solver == 1) return bicgstab_launch_iteration(P, s);
    if (P.solver == 2) return zbicgstab_launch_iteration(P, s);
    MPF_TRY(launch_one(P, 0, s, false));
    MPF_TRY(launch_one(P, 1, s, false));
    if (P.coarse) MPF_TRY(cg_launch_coarse(P, false, s, false));
    return launch_one(P, 2, s, false);
}

int cg_iteration_launches(const CgProblem& P) { return P.solver >= 1 ? kBicgstabLaunches : P.coarse ? 4 : 3; }

int cg_launch_kernel(const CgProblem& P, int which, cudaStream_t s) { return launch_one(P, which, s, true); }

// Groups of the frames marked in frameSkip leave the iteration before it
// starts (their x is kept as it is).  Launched after cg_launch_init.
__global__ void k_skip_frames(int G, int M, int Ca, const int* __restrict__ frameSkip, int* __restrict__ active) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < G && frameSkip[(g / M) / Ca]) active[g] = 0;
}

// groupMask[g] = 1 for the groups of frames not in frameSkip
__global__ void k_group_mask(int G, int M, int Ca, const int* __restrict__ frameSkip, int* __restrict__ groupMask) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < G) groupMask[g] = !frameSkip[(g / M) / Ca];
}

int cg_launch_group_mask(const CgProblem& P, const int* frameSkip, int* groupMask, cudaStream_t s) {
    k_group_mask<<<(P.G + 255) / 256, 256, 0, s>>>(P.G, P.M, P.Ca, frameSkip, groupMask);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int cg_launch_skip(const CgProblem& P, const int* frameSkip, cudaStream_t s) {
    k_skip_frames<<<(P.G + 255) / 256, 256, 0, s>>>(P.G, P.M, P.Ca, frameSkip, P.active);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int cg_launch_finalize(const CgProblem& P, cudaStream_t s) {
    if (P.solver != 0) return MPF_OK;
    return dispatch_kp<FinalizeL>(P.KP, P, s);
}

int cg_launch_residual64(const CgProblem& P, const double* S64, const double* R64, const double* x64,
                         const double* b64, const double* sumX64, double* partR, double* partB, double* rr,
                         double* bb, cudaStream_t s) {
    return dispatch_kp<Res64L>(P.KP, P, S64, R64, x64, b64, sumX64, partR, partB, rr, bb, s);
}

int cg_launch_accumulate64(const CgProblem& P, double* x64, cudaStream_t s) {
    size_t count = (size_t)P.G * P.npad * P.KP;
    k_accumulate64<<<1216, 256, 0, s>>>(count, P.x, x64);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int cg_launch_to_float(const CgProblem& P, const double* x64, cudaStream_t s) {
    size_t count = (size_t)P.G * P.npad * P.KP;
    k_to_float<<<1216, 256, 0, s>>>(count, x64, P.x);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int cg_launch_dc_shift(const CgProblem& P, const double* shift, float sign, cudaStream_t s) {
    k_dc_shift<<<dim3(64, P.G), 256, 0, s>>>(P, shift, sign);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int cg_launch_colsum(const CgProblem& P, const float* x, const double* x64, double* sums, cudaStream_t s) {
    if (x64)
        k_colsum<double><<<P.G, kThreads, 0, s>>>(P.n, P.npad, P.KP, P.Ca, P.dcFree, x64, sums);
    else
        k_colsum<float><<<P.G, kThreads, 0, s>>>(P.n, P.npad, P.KP, P.Ca, P.dcFree, x, sums);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

}  // namespace mpf
