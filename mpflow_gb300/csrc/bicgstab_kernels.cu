// Batched BiCGSTAB for the EIT systems.
//
// Restates numeric::BiCGSTAB::solve (src/numeric/bicgstab.cpp:83-193) for
// every (frame, harmonic[, mesh]) group and right-hand side at once, with the
// Jacobi preconditioner K^-1 = D^-1 applied on the right as the reference
// does: y = K^-1 p, nu = A y, alpha = rho / (rHat, nu), s = r - alpha nu,
// z = K^-1 s, t = A z, omega = (K^-1 t, z) / (K^-1 t, K^-1 t),
// x += alpha y + omega z, r = s - omega t, rho' = (rHat, r),
// beta = (rho' / rho)(alpha / omega), p = r + beta (p - omega nu).  The
// kernels carry y instead of p (y' = D^-1 r + beta (y - omega D^-1 nu)), so an
// SpMV never needs the preconditioner at a neighbouring row, and s is
// recomputed from r and nu where it is needed.  Each right-hand side stops on
// its own at |r| <= tol |b| (the reference tests column 0 against machine
// epsilon); a converged right-hand side keeps x and r (alpha = omega = 0).
//
// One iteration is five launches, one pass over the vectors each:
//   k_bi_direction  y = D^-1 r + beta (y - omega D^-1 nu)         (+ sum y)
//   k_bi_spmv_nu    nu = A y, (rHat, nu) -> alpha
//   k_bi_s          z = D^-1 (r - alpha nu)                        (+ sum z)
//   k_bi_spmv_t     t = A z, (z, D^-1 t), (D^-1 t, D^-1 t) -> omega
//   k_bi_update     x += alpha y + omega z, r = r - alpha nu - omega t,
//                   (rHat, r), |r|^2 -> rho, beta, masks
// On the Neumann harmonic the operator is A + c' 1 1^T, as in the CG
// (cg_kernels.cu), so both solvers return the same fields; the reference's
// BiCGSTAB ignores its dcFree argument and iterates on the singular matrix,
// whose solution differs from this one by a constant only.
#include "cg_common.cuh"

namespace mpf {
namespace {

template <int KP>
struct BiShape {
    static constexpr int VEC = KP >= 32 ? 4 : 2;
    using Sh = Shape<KP, VEC>;
    static constexpr int RB = Sh::STEPS >= 2 ? 2 : 1;
};

// Group, rows and harmonic of the calling block; false if the block has no
// rows (the largest mesh sets the grid) or its group has retired.
struct BiCtx {
    int g, slice, ci, nb, rowBase, j0;
    bool dc;
    float alpha;
    Seg sg;
    const float2* SR;
    size_t vb;
};

template <int KP>
__device__ __forceinline__ bool bi_context(const CgProblem& P, bool needActive, BiCtx& c) {
    using Sh = typename BiShape<KP>::Sh;
    c.g = blockIdx.y;
    if (needActive && !P.active[c.g]) return false;
    c.slice = c.g / P.M;
    c.sg = segment(P, c.g - c.slice * P.M);
    c.nb = c.sg.nblk;
    if ((int)blockIdx.x >= c.nb) return false;
    const int f = c.slice / P.Ca;
    c.ci = c.slice % P.Ca;
    c.dc = P.dcFree[c.ci] != 0;
    c.alpha = P.alpha[c.ci];
    c.SR = P.SR + (size_t)f * P.W * P.npad;
    c.vb = (size_t)c.slice * P.npad * KP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    c.rowBase = (c.sg.tile0 + blockIdx.x) * kRowTile + warp * kRowsPerWarp + lane / Sh::LPR;
    c.j0 = (lane % Sh::LPR) * BiShape<KP>::VEC;
    return true;
}

// r = b - (A + c' 1 1^T) x (or b), rHat = r, y = nu = 0, rho = |r|^2, |b|^2
template <int KP>
__global__ void __launch_bounds__(kThreads) k_bi_init(CgProblem P, int zeroGuess) {
    using B = BiShape<KP>;
    using Sh = typename B::Sh;
    constexpr int VEC = B::VEC, RB = B::RB;
    BiCtx c;
    if (!bi_context<KP>(P, false, c)) return;
    const float* b = P.b + (P.bPerGroup ? c.vb : (size_t)c.ci * P.npad * KP);
    float sx[VEC] = {};
    if (c.dc && !zeroGuess && P.sumX0) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) sx[v] = (float)((double)c.sg.dcScale * P.sumX0[(size_t)c.g * KP + c.j0 + v]);
    }
    DotAcc acc[2][VEC];
    for (int st = 0; st < Sh::STEPS; st += RB) {
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) row[i] = c.rowBase + (st + i) * Sh::SUB;
        float y[RB][VEC];
        if (!zeroGuess) {
            spmm_rows<KP, VEC, RB>(P.cols, c.SR, P.W, P.npad, c.alpha, P.x + c.vb, c.j0, row, y);
        } else {
#pragma unroll
            for (int i = 0; i < RB; ++i) {
#pragma unroll
                for (int v = 0; v < VEC; ++v) y[i][v] = 0.f;
                stv<VEC>(P.x + c.vb + (size_t)row[i] * KP + c.j0, y[i]);
            }
        }
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const bool real = row[i] < c.sg.end;
            const size_t o = c.vb + (size_t)row[i] * KP + c.j0;
            float bv[VEC], rv[VEC], zero[VEC];
            ldv<VEC>(b + (size_t)row[i] * KP + c.j0, bv);
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                rv[v] = zeroGuess ? bv[v] : bv[v] - y[i][v] - (real ? sx[v] : 0.f);
                zero[v] = 0.f;
                acc[0][v].add(rv[v], rv[v]);
                acc[1][v].add(bv[v], bv[v]);
            }
            stv<VEC>(P.r + o, rv);
            stv<VEC>(P.rhat + o, rv);
            stv<VEC>(P.p + o, zero);
            stv<VEC>(P.q + o, zero);
        }
    }
    double* const parts[2] = {P.partA, P.partB};
    if (block_partials<KP, VEC, 2>(acc, parts, c.g, P.counter, c.nb)) {
        int notConv = 0;
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            const double rr = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
            const double bb = sum_partials(P.partB, c.g, KP, threadIdx.x, c.nb);
            P.rz[s] = rr;  // rho = (rHat, r) with rHat = r
            P.rr2[s] = rr;
            P.bz[s] = bb;
            P.pq[s] = 0.0;
            P.omega[s] = 0.0;
            P.beta[s] = 0.0;  // first direction: y = D^-1 r
            const int cv = rr <= P.tol2 * bb;
            P.conv[s] = cv;
            notConv = !cv;
        }
        const int any = __syncthreads_or(notConv);
        if (threadIdx.x == 0) {
            P.active[c.g] = any;
            P.iters[c.g] = 0;
            P.counter[c.g] = 0;
        }
    }
}

// y = D^-1 r + beta (y - omega D^-1 nu); sum(y) on Neumann groups
template <int KP>
__global__ void __launch_bounds__(kThreads) k_bi_direction(CgProblem P) {
    using B = BiShape<KP>;
    using Sh = typename B::Sh;
    constexpr int VEC = B::VEC, RB = B::RB;
    BiCtx c;
    if (!bi_context<KP>(P, true, c)) return;
    float be[VEC], om[VEC];
    bool live[VEC];
#pragma unroll
    for (int v = 0; v < VEC; ++v) {
        const size_t s = (size_t)c.g * KP + c.j0 + v;
        live[v] = !P.conv[s];
        be[v] = (float)P.beta[s];
        om[v] = (float)P.omega[s];
    }
    DotAcc acc[1][VEC];
    for (int st = 0; st < Sh::STEPS; st += RB) {
        float rv[RB][VEC], yv[RB][VEC], nv[RB][VEC], di[RB];
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            row[i] = c.rowBase + (st + i) * Sh::SUB;
            const size_t o = c.vb + (size_t)row[i] * KP + c.j0;
            ldv<VEC>(P.r + o, rv[i]);
            ldv<VEC>(P.p + o, yv[i]);
            ldv<VEC>(P.q + o, nv[i]);
            di[i] = diag_inv(c.SR, P.diagSlot, P.npad, row[i], c.alpha);
        }
#pragma unroll
        for (int i = 0; i < RB; ++i) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                const float z = di[i] * rv[i][v];
                const float upd = be[v] != 0.f ? fmaf(be[v], fmaf(-om[v] * di[i], nv[i][v], yv[i][v]), z) : z;
                yv[i][v] = live[v] ? upd : yv[i][v];
                if (c.dc && row[i] < c.sg.end) acc[0][v].add(yv[i][v], 1.f);
            }
            stv<VEC>(P.p + c.vb + (size_t)row[i] * KP + c.j0, yv[i]);
        }
    }
    if (!c.dc) return;
    double* const parts[1] = {P.partA};
    if (block_partials<KP, VEC, 1>(acc, parts, c.g, P.counter, c.nb)) {
        if (threadIdx.x < KP) P.sumP[(size_t)c.g * KP + threadIdx.x] = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
        if (threadIdx.x == 0) P.counter[c.g] = 0;
    }
}

// out = (A + c' 1 1^T) in over the block's rows (in: y or z, sum in P.sumP)
template <int KP, int RB, int VEC>
__device__ __forceinline__ void bi_spmv(const CgProblem& P, const BiCtx& c, const float* in, const int (&row)[RB],
                                        float (&y)[RB][VEC]) {
    spmm_rows<KP, VEC, RB>(P.cols, c.SR, P.W, P.npad, c.alpha, in, c.j0, row, y);
    if (c.dc) {
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            if (row[i] < c.sg.end) {
#pragma unroll
                for (int v = 0; v < VEC; ++v)
                    y[i][v] += (float)((double)c.sg.dcScale * P.sumP[(size_t)c.g * KP + c.j0 + v]);
            }
        }
    }
}

// nu = A y; alpha = rho / (rHat, nu)
template <int KP>
__global__ void __launch_bounds__(kThreads) k_bi_spmv_nu(CgProblem P) {
    using B = BiShape<KP>;
    using Sh = typename B::Sh;
    constexpr int VEC = B::VEC, RB = B::RB;
    BiCtx c;
    if (!bi_context<KP>(P, true, c)) return;
    DotAcc acc[1][VEC];
    for (int st = 0; st < Sh::STEPS; st += RB) {
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) row[i] = c.rowBase + (st + i) * Sh::SUB;
        float y[RB][VEC];
        bi_spmv<KP, RB, VEC>(P, c, P.p + c.vb, row, y);
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const size_t o = c.vb + (size_t)row[i] * KP + c.j0;
            stv<VEC>(P.q + o, y[i]);
            float hv[VEC];
            ldv<VEC>(P.rhat + o, hv);
#pragma unroll
            for (int v = 0; v < VEC; ++v) acc[0][v].add(hv[v], y[i][v]);
        }
    }
    double* const parts[1] = {P.partA};
    if (block_partials<KP, VEC, 1>(acc, parts, c.g, P.counter, c.nb)) {
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            const double den = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
            P.pq[s] = (!P.conv[s] && den != 0.0) ? P.rz[s] / den : 0.0;
        }
        if (threadIdx.x == 0) P.counter[c.g] = 0;
    }
}

// z = D^-1 (r - alpha nu); sum(z) on Neumann groups
template <int KP>
__global__ void __launch_bounds__(kThreads) k_bi_s(CgProblem P) {
    using B = BiShape<KP>;
    using Sh = typename B::Sh;
    constexpr int VEC = B::VEC, RB = B::RB;
    BiCtx c;
    if (!bi_context<KP>(P, true, c)) return;
    float a[VEC];
#pragma unroll
    for (int v = 0; v < VEC; ++v) a[v] = (float)P.pq[(size_t)c.g * KP + c.j0 + v];
    DotAcc acc[1][VEC];
    for (int st = 0; st < Sh::STEPS; st += RB) {
        float rv[RB][VEC], nv[RB][VEC], di[RB];
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            row[i] = c.rowBase + (st + i) * Sh::SUB;
            const size_t o = c.vb + (size_t)row[i] * KP + c.j0;
            ldv<VEC>(P.r + o, rv[i]);
            ldv<VEC>(P.q + o, nv[i]);
            di[i] = diag_inv(c.SR, P.diagSlot, P.npad, row[i], c.alpha);
        }
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            float zv[VEC];
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                zv[v] = di[i] * fmaf(-a[v], nv[i][v], rv[i][v]);
                if (c.dc && row[i] < c.sg.end) acc[0][v].add(zv[v], 1.f);
            }
            stv<VEC>(P.zv + c.vb + (size_t)row[i] * KP + c.j0, zv);
        }
    }
    if (!c.dc) return;
    double* const parts[1] = {P.partA};
    if (block_partials<KP, VEC, 1>(acc, parts, c.g, P.counter, c.nb)) {
        if (threadIdx.x < KP) P.sumP[(size_t)c.g * KP + threadIdx.x] = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
        if (threadIdx.x == 0) P.counter[c.g] = 0;
    }
}

// t = A z; omega = (z, D^-1 t) / (D^-1 t, D^-1 t)
template <int KP>
__global__ void __launch_bounds__(kThreads) k_bi_spmv_t(CgProblem P) {
    using B = BiShape<KP>;
    using Sh = typename B::Sh;
    constexpr int VEC = B::VEC, RB = B::RB;
    BiCtx c;
    if (!bi_context<KP>(P, true, c)) return;
    DotAcc acc[2][VEC];
    for (int st = 0; st < Sh::STEPS; st += RB) {
        int row[RB];
#pragma unroll
        for (int i = 0; i < RB; ++i) row[i] = c.rowBase + (st + i) * Sh::SUB;
        float y[RB][VEC];
        bi_spmv<KP, RB, VEC>(P, c, P.zv + c.vb, row, y);
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const size_t o = c.vb + (size_t)row[i] * KP + c.j0;
            stv<VEC>(P.tv + o, y[i]);
            const float di = diag_inv(c.SR, P.diagSlot, P.npad, row[i], c.alpha);
            float zv[VEC];
            ldv<VEC>(P.zv + o, zv);
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                const float tk = di * y[i][v];
                acc[0][v].add(zv[v], tk);
                acc[1][v].add(tk, tk);
            }
        }
    }
    double* const parts[2] = {P.partA, P.partB};
    if (block_partials<KP, VEC, 2>(acc, parts, c.g, P.counter, c.nb)) {
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            const double zt = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
            const double tt = sum_partials(P.partB, c.g, KP, threadIdx.x, c.nb);
            P.omega[s] = (!P.conv[s] && tt > 0.0) ? zt / tt : 0.0;
        }
        if (threadIdx.x == 0) P.counter[c.g] = 0;
    }
}

// x += alpha y + omega z, r = r - alpha nu - omega t; rho' = (rHat, r),
// |r|^2, beta, convergence masks, the group's active flag
template <int KP>
__global__ void __launch_bounds__(kThreads) k_bi_update(CgProblem P) {
    using B = BiShape<KP>;
    using Sh = typename B::Sh;
    constexpr int VEC = B::VEC, RB = B::RB;
    BiCtx c;
    if (!bi_context<KP>(P, true, c)) return;
    float a[VEC], om[VEC];
#pragma unroll
    for (int v = 0; v < VEC; ++v) {
        const size_t s = (size_t)c.g * KP + c.j0 + v;
        a[v] = (float)P.pq[s];
        om[v] = (float)P.omega[s];
    }
    DotAcc acc[2][VEC];
    for (int st = 0; st < Sh::STEPS; st += RB) {
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const int row = c.rowBase + (st + i) * Sh::SUB;
            const size_t o = c.vb + (size_t)row * KP + c.j0;
            float xv[VEC], yv[VEC], zv[VEC], rv[VEC], nv[VEC], tv[VEC], hv[VEC];
            ldv<VEC>(P.x + o, xv);
            ldv<VEC>(P.p + o, yv);
            ldv<VEC>(P.zv + o, zv);
            ldv<VEC>(P.r + o, rv);
            ldv<VEC>(P.q + o, nv);
            ldv<VEC>(P.tv + o, tv);
            ldv<VEC>(P.rhat + o, hv);
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                xv[v] = fmaf(om[v], zv[v], fmaf(a[v], yv[v], xv[v]));
                rv[v] = fmaf(-om[v], tv[v], fmaf(-a[v], nv[v], rv[v]));
                acc[0][v].add(hv[v], rv[v]);
                acc[1][v].add(rv[v], rv[v]);
            }
            stv<VEC>(P.x + o, xv);
            stv<VEC>(P.r + o, rv);
        }
    }
    double* const parts[2] = {P.partA, P.partB};
    if (block_partials<KP, VEC, 2>(acc, parts, c.g, P.counter, c.nb)) {
        int notConv = 0;
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            if (!P.conv[s]) {
                const double rhoN = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
                const double rr = sum_partials(P.partB, c.g, KP, threadIdx.x, c.nb);
                const double rho = P.rz[s], al = P.pq[s], w = P.omega[s];
                P.beta[s] = (rho != 0.0 && w != 0.0) ? (rhoN / rho) * (al / w) : 0.0;
                P.rz[s] = rhoN;
                P.rr2[s] = rr;
                const int cv = rr <= P.tol2 * P.bz[s];
                P.conv[s] = cv;
                notConv = !cv;
            }
        }
        const int any = __syncthreads_or(notConv);
        if (threadIdx.x == 0) {
            P.active[c.g] = any;
            P.iters[c.g] += 1;
            P.counter[c.g] = 0;
        }
    }
}

template <int KP>
int launch_init_kp(const CgProblem& P, bool zeroGuess, cudaStream_t s) {
    k_bi_init<KP><<<dim3(P.nblk, P.G), kThreads, 0, s>>>(P, zeroGuess ? 1 : 0);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

// the five launches of one iteration (also recorded into CUDA graphs, so
// they are not counted here: the graph replays are)
template <int KP>
int launch_iteration_kp(const CgProblem& P, cudaStream_t s) {
    const dim3 grid(P.nblk, P.G);
    k_bi_direction<KP><<<grid, kThreads, 0, s>>>(P);
    k_bi_spmv_nu<KP><<<grid, kThreads, 0, s>>>(P);
    k_bi_s<KP><<<grid, kThreads, 0, s>>>(P);
    k_bi_spmv_t<KP><<<grid, kThreads, 0, s>>>(P);
    k_bi_update<KP><<<grid, kThreads, 0, s>>>(P);
    MPF_CUDA(cudaGetLastError());
    return MPF_OK;
}

}  // namespace

int bicgstab_launch_init(const CgProblem& P, bool zeroGuess, cudaStream_t s) {
    MPF_CHECK(!P.coarse, MPF_ENOTSUP, "BiCGSTAB runs with the Jacobi preconditioner only");
    switch (P.KP) {
        case 16: return launch_init_kp<16>(P, zeroGuess, s);
        case 32: return launch_init_kp<32>(P, zeroGuess, s);
        case 64: return launch_init_kp<64>(P, zeroGuess, s);
        case 128: return launch_init_kp<128>(P, zeroGuess, s);
        default: return fail(MPF_EINVAL, "BiCGSTAB: unsupported right-hand-side width %d", P.KP);
    }
}

int bicgstab_launch_iteration(const CgProblem& P, cudaStream_t s) {
    switch (P.KP) {
        case 16: return launch_iteration_kp<16>(P, s);
        case 32: return launch_iteration_kp<32>(P, s);
        case 64: return launch_iteration_kp<64>(P, s);
        case 128: return launch_iteration_kp<128>(P, s);
        default: return fail(MPF_EINVAL, "BiCGSTAB: unsupported right-hand-side width %d", P.KP);
    }
}

}  // namespace mpf
