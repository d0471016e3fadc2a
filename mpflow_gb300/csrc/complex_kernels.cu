// Complex admittivity: the EIT forward model for complex material values,
// the reference's Equation<thrust::complex<float>> instantiations
// (src/models/eit.cpp:289-304, src/fem/equation_kernel.cu:35-82).
//
//   assembly   p(gamma) = ref * gamma or ref * exp(ln(10) gamma / 10) with
//              complex gamma; S and R slot values complex (k_zassemble)
//   solve      BiCGSTAB over complex vectors with the reference's inner
//              product (a, b) = sum a * conj(b)
//              (src/numeric/matrix_kernel.cu:404-413), right-preconditioned
//              with the complex Jacobi inverse, every right-hand side
//              stopped at |r| <= tol |b|; the Neumann harmonic carries the
//              real c' 1 1^T term as the real solvers do (k_zbi_*)
//   voltages   V = sum_c beta_c Att Phi_c with complex Phi (k_zgram_meas,
//              k_zvoltages)
//   Jacobian   calcJacobianKernel's bilinear form with complex fields and
//              complex p'(gamma) (k_zjacobian), then the reference layout
// Vectors are node-major with KP complex values per node (re, im
// interleaved); a lane moves CV = 2 complex values (16 bytes).
#include "cg_common.cuh"

namespace mpf {
namespace {

constexpr int kCV = 2;  // complex values per lane

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// c + a * b
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 cinv(float2 d) {
    const float m = fmaf(d.x, d.x, d.y * d.y);
    return m != 0.f ? make_float2(d.x / m, -d.y / m) : make_float2(0.f, 0.f);
}
__device__ __forceinline__ void ldz(const float* p, float2 (&v)[kCV]) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = make_float2(t.x, t.y);
    v[1] = make_float2(t.z, t.w);
}
__device__ __forceinline__ void stz(float* p, const float2 (&v)[kCV]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
}
// acc[dr], acc[di] += a * conj(b)
__device__ __forceinline__ void zdot_add(DotAcc& re, DotAcc& im, float2 a, float2 b) {
    re.add(a.x, b.x);
    re.add(a.y, b.y);
    im.add(a.y, b.x);
    im.add(-a.x, b.y);
}
__device__ __forceinline__ double2 ddiv(double2 a, double2 b) {
    const double m = b.x * b.x + b.y * b.y;
    return m != 0.0 ? make_double2((a.x * b.x + a.y * b.y) / m, (a.y * b.x - a.x * b.y) / m) : make_double2(0.0, 0.0);
}
__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 zdiag_inv(const float4* SRz, const int32_t* diagSlot, int npad, int row, float alpha) {
    const float4 e = __ldg(&SRz[(size_t)__ldg(&diagSlot[row]) * npad + row]);
    return cinv(make_float2(fmaf(alpha, e.z, e.x), fmaf(alpha, e.w, e.y)));
}

template <int KP>
struct ZShape {
    using Sh = Shape<KP, kCV>;
};

struct ZCtx {
    int g, slice, ci, nb, rowBase, j0;
    bool dc;
    float alpha;
    Seg sg;
    const float4* SRz;
    size_t vb;  // complex offset of the group's vector slice
};

template <int KP>
__device__ __forceinline__ bool z_context(const CgProblem& P, bool needActive, ZCtx& c) {
    using Sh = typename ZShape<KP>::Sh;
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
    c.SRz = P.SRz + (size_t)f * P.W * P.npad;
    c.vb = (size_t)c.slice * P.npad * KP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    c.rowBase = (c.sg.tile0 + blockIdx.x) * kRowTile + warp * kRowsPerWarp + lane / Sh::LPR;
    c.j0 = (lane % Sh::LPR) * kCV;
    return true;
}

// float offset of (row, column j0) in a complex vector
__device__ __forceinline__ size_t zoff(const ZCtx& c, int KP, int row) { return 2 * (c.vb + (size_t)row * KP + c.j0); }

// y = (S + alpha R) x (+ c' sum(x) on real rows of Neumann groups), one row
template <int KP>
__device__ __forceinline__ void zspmv_row(const CgProblem& P, const ZCtx& c, const float* x, int row,
                                          float2 (&y)[kCV]) {
    y[0] = y[1] = make_float2(0.f, 0.f);
    for (int k = 0; k < P.W; ++k) {
        const size_t sl = (size_t)k * P.npad + row;
        const int col = __ldg(&P.cols[sl]);
        const float4 e = __ldg(&c.SRz[sl]);
        const float2 a = make_float2(fmaf(c.alpha, e.z, e.x), fmaf(c.alpha, e.w, e.y));
        float2 xv[kCV];
        ldz(x + 2 * (c.vb + (size_t)col * KP + c.j0), xv);
        y[0] = cfma(a, xv[0], y[0]);
        y[1] = cfma(a, xv[1], y[1]);
    }
    if (c.dc && row < c.sg.end) {
#pragma unroll
        for (int v = 0; v < kCV; ++v) {
            const size_t s = (size_t)c.g * KP + c.j0 + v;
            y[v].x += (float)((double)c.sg.dcScale * P.sumP[s]);
            y[v].y += (float)((double)c.sg.dcScale * P.sumPI[s]);
        }
    }
}

__global__ void k_zassemble(int W, int npad, int E, const int32_t* __restrict__ cptr,
                            const int32_t* __restrict__ contrib, const float* __restrict__ Kf,
                            const float* __restrict__ Mf, const float2* __restrict__ gamma, float ref, int logarithmic,
                            float4* __restrict__ SRz) {
    const int f = blockIdx.y;
    const size_t slots = (size_t)W * npad;
    const float2* gf = gamma + (size_t)f * E;
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < slots; s += (size_t)gridDim.x * blockDim.x) {
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int c = __ldg(&cptr[s]); c < __ldg(&cptr[s + 1]); ++c) {
            const int code = __ldg(&contrib[c]);
            const float2 g = __ldg(&gf[code / 9]);
            float2 pg;
            if (logarithmic) {
                // ref * exp(ln(10) g / 10), complex exponential
                const float a = 0.2302585093f * g.x, b = 0.2302585093f * g.y;
                float sn, cs;
                sincosf(b, &sn, &cs);
                const float m = ref * expf(a);
                pg = make_float2(m * cs, m * sn);
            } else {
                pg = make_float2(ref * g.x, ref * g.y);
            }
            const float k = __ldg(&Kf[code]), mm = __ldg(&Mf[code]);
            acc.x = fmaf(k, pg.x, acc.x);
            acc.y = fmaf(k, pg.y, acc.y);
            acc.z = fmaf(mm, pg.x, acc.z);
            acc.w = fmaf(mm, pg.y, acc.w);
        }
        SRz[(size_t)f * slots + s] = acc;
    }
}

// cold start: x = 0, r = rHat = b, y = nu = 0, rho = |b|^2
template <int KP>
__global__ void __launch_bounds__(kThreads) k_zbi_init(CgProblem P) {
    using Sh = typename ZShape<KP>::Sh;
    ZCtx c;
    if (!z_context<KP>(P, false, c)) return;
    const float* b = P.b + (P.bPerGroup ? c.vb : (size_t)c.ci * P.npad * KP);
    DotAcc acc[1][kCV];
    for (int st = 0; st < Sh::STEPS; ++st) {
        const int row = c.rowBase + st * Sh::SUB;
        float bv[kCV];
        ldv<kCV>(b + (size_t)row * KP + c.j0, bv);
        float2 rv[kCV], zero[kCV];
#pragma unroll
        for (int v = 0; v < kCV; ++v) {
            rv[v] = make_float2(bv[v], 0.f);
            zero[v] = make_float2(0.f, 0.f);
            acc[0][v].add(bv[v], bv[v]);
        }
        const size_t o = zoff(c, KP, row);
        stz(P.r + o, rv);
        stz(P.rhat + o, rv);
        stz(P.x + o, zero);
        stz(P.p + o, zero);
        stz(P.q + o, zero);
    }
    double* const parts[1] = {P.partA};
    if (block_partials<KP, kCV, 1>(acc, parts, c.g, P.counter, c.nb)) {
        int notConv = 0;
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            const double bb = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
            P.rz[s] = bb;
            P.rzI[s] = 0.0;
            P.rr2[s] = bb;
            P.bz[s] = bb;
            P.pq[s] = P.pqI[s] = 0.0;
            P.omega[s] = P.omegaI[s] = 0.0;
            P.beta[s] = P.betaI[s] = 0.0;
            const int cv = bb <= 0.0;
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

// sums of a complex vector over the real rows of a Neumann group -> sumP, sumPI
template <int KP>
__device__ __forceinline__ void zsum_finish(const CgProblem& P, const ZCtx& c, DotAcc (&acc)[2][kCV]) {
    double* const parts[2] = {P.partA, P.partB};
    if (block_partials<KP, kCV, 2>(acc, parts, c.g, P.counter, c.nb)) {
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            P.sumP[s] = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
            P.sumPI[s] = sum_partials(P.partB, c.g, KP, threadIdx.x, c.nb);
        }
        if (threadIdx.x == 0) P.counter[c.g] = 0;
    }
}

// y = D^-1 r + beta (y - omega D^-1 nu)
template <int KP>
__global__ void __launch_bounds__(kThreads) k_zbi_direction(CgProblem P) {
    using Sh = typename ZShape<KP>::Sh;
    ZCtx c;
    if (!z_context<KP>(P, true, c)) return;
    float2 be[kCV], om[kCV];
    bool live[kCV], first[kCV];
#pragma unroll
    for (int v = 0; v < kCV; ++v) {
        const size_t s = (size_t)c.g * KP + c.j0 + v;
        live[v] = !P.conv[s];
        be[v] = make_float2((float)P.beta[s], (float)P.betaI[s]);
        om[v] = make_float2((float)P.omega[s], (float)P.omegaI[s]);
        first[v] = be[v].x == 0.f && be[v].y == 0.f;
    }
    DotAcc acc[2][kCV];
    for (int st = 0; st < Sh::STEPS; ++st) {
        const int row = c.rowBase + st * Sh::SUB;
        const size_t o = zoff(c, KP, row);
        float2 rv[kCV], yv[kCV], nv[kCV];
        ldz(P.r + o, rv);
        ldz(P.p + o, yv);
        ldz(P.q + o, nv);
        const float2 di = zdiag_inv(c.SRz, P.diagSlot, P.npad, row, c.alpha);
#pragma unroll
        for (int v = 0; v < kCV; ++v) {
            const float2 z = cmul(di, rv[v]);
            float2 upd = z;
            if (!first[v]) {
                const float2 w = cmul(om[v], cmul(di, nv[v]));
                upd = cfma(be[v], make_float2(yv[v].x - w.x, yv[v].y - w.y), z);
            }
            yv[v] = live[v] ? upd : yv[v];
            if (c.dc && row < c.sg.end) {
                acc[0][v].add(yv[v].x, 1.f);
                acc[1][v].add(yv[v].y, 1.f);
            }
        }
        stz(P.p + o, yv);
    }
    if (c.dc) zsum_finish<KP>(P, c, acc);
}

// nu = A y; alpha = rho / (nu, rHat)
template <int KP>
__global__ void __launch_bounds__(kThreads) k_zbi_spmv_nu(CgProblem P) {
    using Sh = typename ZShape<KP>::Sh;
    ZCtx c;
    if (!z_context<KP>(P, true, c)) return;
    DotAcc acc[2][kCV];
    for (int st = 0; st < Sh::STEPS; ++st) {
        const int row = c.rowBase + st * Sh::SUB;
        float2 y[kCV], h[kCV];
        zspmv_row<KP>(P, c, P.p, row, y);
        const size_t o = zoff(c, KP, row);
        stz(P.q + o, y);
        ldz(P.rhat + o, h);
#pragma unroll
        for (int v = 0; v < kCV; ++v) zdot_add(acc[0][v], acc[1][v], y[v], h[v]);
    }
    double* const parts[2] = {P.partA, P.partB};
    if (block_partials<KP, kCV, 2>(acc, parts, c.g, P.counter, c.nb)) {
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            const double2 den = make_double2(sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb),
                                             sum_partials(P.partB, c.g, KP, threadIdx.x, c.nb));
            const double2 a = P.conv[s] ? make_double2(0.0, 0.0) : ddiv(make_double2(P.rz[s], P.rzI[s]), den);
            P.pq[s] = a.x;
            P.pqI[s] = a.y;
        }
        if (threadIdx.x == 0) P.counter[c.g] = 0;
    }
}

// z = D^-1 (r - alpha nu)
template <int KP>
__global__ void __launch_bounds__(kThreads) k_zbi_s(CgProblem P) {
    using Sh = typename ZShape<KP>::Sh;
    ZCtx c;
    if (!z_context<KP>(P, true, c)) return;
    float2 a[kCV];
#pragma unroll
    for (int v = 0; v < kCV; ++v) {
        const size_t s = (size_t)c.g * KP + c.j0 + v;
        a[v] = make_float2((float)P.pq[s], (float)P.pqI[s]);
    }
    DotAcc acc[2][kCV];
    for (int st = 0; st < Sh::STEPS; ++st) {
        const int row = c.rowBase + st * Sh::SUB;
        const size_t o = zoff(c, KP, row);
        float2 rv[kCV], nv[kCV], zv[kCV];
        ldz(P.r + o, rv);
        ldz(P.q + o, nv);
        const float2 di = zdiag_inv(c.SRz, P.diagSlot, P.npad, row, c.alpha);
#pragma unroll
        for (int v = 0; v < kCV; ++v) {
            const float2 an = cmul(a[v], nv[v]);
            zv[v] = cmul(di, make_float2(rv[v].x - an.x, rv[v].y - an.y));
            if (c.dc && row < c.sg.end) {
                acc[0][v].add(zv[v].x, 1.f);
                acc[1][v].add(zv[v].y, 1.f);
            }
        }
        stz(P.zv + o, zv);
    }
    if (c.dc) zsum_finish<KP>(P, c, acc);
}

// t = A z; omega = (z, D^-1 t) / (D^-1 t, D^-1 t)
template <int KP>
__global__ void __launch_bounds__(kThreads) k_zbi_spmv_t(CgProblem P) {
    using Sh = typename ZShape<KP>::Sh;
    ZCtx c;
    if (!z_context<KP>(P, true, c)) return;
    DotAcc acc[3][kCV];
    for (int st = 0; st < Sh::STEPS; ++st) {
        const int row = c.rowBase + st * Sh::SUB;
        float2 t[kCV], zv[kCV];
        zspmv_row<KP>(P, c, P.zv, row, t);
        const size_t o = zoff(c, KP, row);
        stz(P.tv + o, t);
        ldz(P.zv + o, zv);
        const float2 di = zdiag_inv(c.SRz, P.diagSlot, P.npad, row, c.alpha);
#pragma unroll
        for (int v = 0; v < kCV; ++v) {
            const float2 tk = cmul(di, t[v]);
            zdot_add(acc[0][v], acc[1][v], zv[v], tk);
            acc[2][v].add(tk.x, tk.x);
            acc[2][v].add(tk.y, tk.y);
        }
    }
    double* const parts[3] = {P.partA, P.partB, P.partC};
    if (block_partials<KP, kCV, 3>(acc, parts, c.g, P.counter, c.nb)) {
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            const double zr = sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb);
            const double zi = sum_partials(P.partB, c.g, KP, threadIdx.x, c.nb);
            const double tt = sum_partials(P.partC, c.g, KP, threadIdx.x, c.nb);
            const bool ok = !P.conv[s] && tt > 0.0;
            P.omega[s] = ok ? zr / tt : 0.0;
            P.omegaI[s] = ok ? zi / tt : 0.0;
        }
        if (threadIdx.x == 0) P.counter[c.g] = 0;
    }
}

// x += alpha y + omega z, r = r - alpha nu - omega t; rho' = (r, rHat),
// |r|^2, beta = (rho' / rho)(alpha / omega), masks
template <int KP>
__global__ void __launch_bounds__(kThreads) k_zbi_update(CgProblem P) {
    using Sh = typename ZShape<KP>::Sh;
    ZCtx c;
    if (!z_context<KP>(P, true, c)) return;
    float2 a[kCV], om[kCV];
#pragma unroll
    for (int v = 0; v < kCV; ++v) {
        const size_t s = (size_t)c.g * KP + c.j0 + v;
        a[v] = make_float2((float)P.pq[s], (float)P.pqI[s]);
        om[v] = make_float2((float)P.omega[s], (float)P.omegaI[s]);
    }
    DotAcc acc[3][kCV];
    for (int st = 0; st < Sh::STEPS; ++st) {
        const int row = c.rowBase + st * Sh::SUB;
        const size_t o = zoff(c, KP, row);
        float2 xv[kCV], yv[kCV], zv[kCV], rv[kCV], nv[kCV], tv[kCV], hv[kCV];
        ldz(P.x + o, xv);
        ldz(P.p + o, yv);
        ldz(P.zv + o, zv);
        ldz(P.r + o, rv);
        ldz(P.q + o, nv);
        ldz(P.tv + o, tv);
        ldz(P.rhat + o, hv);
#pragma unroll
        for (int v = 0; v < kCV; ++v) {
            xv[v] = cfma(om[v], zv[v], cfma(a[v], yv[v], xv[v]));
            const float2 d = cfma(om[v], tv[v], cmul(a[v], nv[v]));
            rv[v] = make_float2(rv[v].x - d.x, rv[v].y - d.y);
            zdot_add(acc[0][v], acc[1][v], rv[v], hv[v]);
            acc[2][v].add(rv[v].x, rv[v].x);
            acc[2][v].add(rv[v].y, rv[v].y);
        }
        stz(P.x + o, xv);
        stz(P.r + o, rv);
    }
    double* const parts[3] = {P.partA, P.partB, P.partC};
    if (block_partials<KP, kCV, 3>(acc, parts, c.g, P.counter, c.nb)) {
        int notConv = 0;
        if (threadIdx.x < KP) {
            const size_t s = (size_t)c.g * KP + threadIdx.x;
            if (!P.conv[s]) {
                const double2 rhoN = make_double2(sum_partials(P.partA, c.g, KP, threadIdx.x, c.nb),
                                                  sum_partials(P.partB, c.g, KP, threadIdx.x, c.nb));
                const double rr = sum_partials(P.partC, c.g, KP, threadIdx.x, c.nb);
                const double2 rho = make_double2(P.rz[s], P.rzI[s]);
                const double2 al = make_double2(P.pq[s], P.pqI[s]), w = make_double2(P.omega[s], P.omegaI[s]);
                const double2 be = dmul(ddiv(rhoN, rho), ddiv(al, w));
                P.beta[s] = be.x;
                P.betaI[s] = be.y;
                P.rz[s] = rhoN.x;
                P.rzI[s] = rhoN.y;
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

// x += sign * shift[j] (real) on the real rows of every Neumann group
__global__ void k_zdc_shift(CgProblem P, const double* shift, float sign) {
    const int g = blockIdx.y;
    const int slice = g / P.M, mesh = g - slice * P.M;
    if (!P.dcFree[slice % P.Ca]) return;
    const Seg sg = segment(P, mesh);
    const size_t vb = ((size_t)slice * P.npad + (size_t)sg.tile0 * kRowTile) * P.KP;
    const size_t count = (size_t)(sg.end - sg.tile0 * kRowTile) * P.KP;
    shift += (size_t)mesh * P.KP;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        P.x[2 * (vb + i)] += sign * (float)shift[i % P.KP];
}

// Gm[g][u][v] = sum_n B0[n][u] X[g][n][v] (complex X, FP64 sums)
__global__ void k_zgram_meas(int KP, int npad, const int32_t* __restrict__ nzPtr, const int32_t* __restrict__ nzNode,
                             const double* __restrict__ nzVal, const float* __restrict__ X, double* __restrict__ Gm) {
    const int g = blockIdx.x;
    const float* Xg = X + 2 * (size_t)g * npad * KP;
    for (int pair = threadIdx.x; pair < KP * KP; pair += blockDim.x) {
        const int u = pair / KP, v = pair % KP;
        double re = 0.0, im = 0.0;
        for (int c = nzPtr[u]; c < nzPtr[u + 1]; ++c) {
            const float2 x = *reinterpret_cast<const float2*>(Xg + 2 * ((size_t)nzNode[c] * KP + v));
            re += nzVal[c] * (double)x.x;
            im += nzVal[c] * (double)x.y;
        }
        Gm[2 * ((size_t)g * KP * KP + pair)] = re;
        Gm[2 * ((size_t)g * KP * KP + pair) + 1] = im;
    }
}

__global__ void k_zvoltages(int F, int Ca, int KP, int Mm, int Md, const double* __restrict__ Gm,
                            const float* __restrict__ beta, const int32_t* __restrict__ measU,
                            const float* __restrict__ measScale, const int32_t* __restrict__ driveU,
                            const float* __restrict__ driveScale, float* __restrict__ V) {
    const int total = F * Mm * Md;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int f = i / (Mm * Md), r = i % (Mm * Md);
        const int m = r % Mm, d = r / Mm;
        const int um = measU[m], ud = driveU[d];
        double re = 0.0, im = 0.0;
        for (int ci = 0; ci < Ca; ++ci) {
            const size_t o = 2 * (((size_t)(f * Ca + ci) * KP + um) * KP + ud);
            re += (double)beta[ci] * Gm[o];
            im += (double)beta[ci] * Gm[o + 1];
        }
        const double sc = (double)measScale[m] * (double)driveScale[d];
        V[2 * i] = (float)(re * sc);
        V[2 * i + 1] = (float)(im * sc);
    }
}

// Complex Jacobian, the formula of the real k_jacobian (fem_kernels.cu) with
// complex fields Y_c and complex p'(gamma):
//   J[d*MP + m][e] += -h p'(gamma_e) sd sm sum_ij Y_c[n_i][ud] Ke[i+3j] Y_c[n_j][um]
// for harmonic ci (beta_c^2 folded into the fields as in the real kernel).
// A block owns 32 elements (one per lane) and stages the complex fields of
// their 3 nodes; warp w handles drive rows w, w + 8, ...; the harmonics
// accumulate into J [F][rowsJ][Epad] (complex) in global memory.
template <int KP, int MP>
__global__ void __launch_bounds__(256) k_zjacobian(JacPlan jp, int npad, const float* __restrict__ X,
                                                   const float2* __restrict__ gamma, float2* __restrict__ J,
                                                   int ci) {
    extern __shared__ float2 zjsm[];  // Ys [3][KP][33], then Ts [3][KP][33]
    float2(*Ys)[KP][33] = reinterpret_cast<float2(*)[KP][33]>(zjsm);
    float2(*Ts)[KP][33] = reinterpret_cast<float2(*)[KP][33]>(zjsm + 3 * KP * 33);
    __shared__ float Ke[32][9];
    const int f = blockIdx.y;
    const int e0 = blockIdx.x * 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int e = e0 + lane;
    const float mc = jp.massCoef[ci];
    for (int i = threadIdx.x; i < 32 * 9; i += blockDim.x) {
        const int el = i / 9, k = i % 9;
        const bool in = e0 + el < jp.E;
        Ke[el][k] = in ? jp.Kf[(size_t)(e0 + el) * 9 + k] + (jp.exact ? mc * jp.Mf[(size_t)(e0 + el) * 9 + k] : 0.f)
                       : 0.f;
    }
    const float2* Xg = reinterpret_cast<const float2*>(X) + ((size_t)f * jp.Ca + ci) * npad * KP;
    for (int i = threadIdx.x; i < 32 * 3 * KP; i += blockDim.x) {
        const int u = i % KP, l = (i / KP) % 3, el = i / (3 * KP);
        float2 v = make_float2(0.f, 0.f);
        if (e0 + el < jp.E) v = Xg[(size_t)jp.elements[(size_t)(e0 + el) * 3 + l] * KP + u];
        Ys[l][u][el] = v;
    }
    __syncthreads();
    const float b2 = jp.beta2[ci];
    for (int i = threadIdx.x; i < 32 * 3 * KP; i += blockDim.x) {
        const int el = i % 32, u = (i / 32) % KP, jj = i / (32 * KP);
        float2 t = make_float2(0.f, 0.f);
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) {
            const float k = b2 * Ke[el][ii * 3 + jj];
            t.x = fmaf(k, Ys[ii][u][el].x, t.x);
            t.y = fmaf(k, Ys[ii][u][el].y, t.y);
        }
        Ts[jj][u][el] = t;
    }
    __syncthreads();
    const bool valid = e < jp.E;
    float2 deriv = make_float2(0.f, 0.f);
    if (valid) {
        const float2 g = gamma[(size_t)f * jp.E + e];
        if (jp.logarithmic) {
            const float a = 0.2302585093f * g.x, b = 0.2302585093f * g.y;
            float sn, cs;
            sincosf(b, &sn, &cs);
            const float mag = -jp.height * 0.2302585093f * jp.ref * expf(a);
            deriv = make_float2(mag * cs, mag * sn);
        } else {
            deriv = make_float2(-jp.height * jp.ref, 0.f);
        }
    }
    const int drives = jp.rowsJ / MP;
    const size_t base = (size_t)f * jp.rowsJ * jp.Epad;
    for (int d = warp; d < drives; d += blockDim.x / 32) {
        const int ud = jp.rowD[d * MP];
        float2 acc[MP];
#pragma unroll
        for (int m = 0; m < MP; ++m) acc[m] = make_float2(0.f, 0.f);
        if (ud >= 0) {
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) {
                const float2 td = Ts[jj][ud][lane];
#pragma unroll
                for (int m = 0; m < MP; ++m) {
                    const int um = jp.rowM[m];
                    const float2 ym = um >= 0 ? Ys[jj][um][lane] : make_float2(0.f, 0.f);
                    acc[m] = cfma(td, ym, acc[m]);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < MP; ++m) {
            const int row = d * MP + m;
            const size_t o = base + (size_t)row * jp.Epad + e;
            const float2 v = valid ? cmul(deriv, make_float2(jp.rowScale[row] * acc[m].x, jp.rowScale[row] * acc[m].y))
                                   : make_float2(0.f, 0.f);
            if (ci == 0) {
                J[o] = v;
            } else {
                const float2 old = J[o];
                J[o] = make_float2(old.x + v.x, old.y + v.y);
            }
        }
    }
}

// [F][rowsJ][Epad] -> the reference layout [F][E][rowsJ] (column-major rowsJ x E)
__global__ void k_ztranspose(int rowsJ, int Epad, int E, const float2* __restrict__ J, float2* __restrict__ Jref) {
    __shared__ float2 tile[32][33];
    const int f = blockIdx.z, e0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const float2* Jf = J + (size_t)f * rowsJ * Epad;
    float2* Rf = Jref + (size_t)f * E * rowsJ;
    for (int k = ty; k < 32; k += 8) {
        const int r = r0 + k, e = e0 + tx;
        tile[k][tx] = (r < rowsJ && e < E) ? Jf[(size_t)r * Epad + e] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int e = e0 + k, r = r0 + tx;
        if (e < E && r < rowsJ) Rf[(size_t)e * rowsJ + r] = tile[tx][k];
    }
}

template <int KP>
int zinit_kp(const CgProblem& P, cudaStream_t s) {
    k_zbi_init<KP><<<dim3(P.nblk, P.G), kThreads, 0, s>>>(P);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

template <int KP>
int ziter_kp(const CgProblem& P, cudaStream_t s) {
    const dim3 grid(P.nblk, P.G);
    k_zbi_direction<KP><<<grid, kThreads, 0, s>>>(P);
    k_zbi_spmv_nu<KP><<<grid, kThreads, 0, s>>>(P);
    k_zbi_s<KP><<<grid, kThreads, 0, s>>>(P);
    k_zbi_spmv_t<KP><<<grid, kThreads, 0, s>>>(P);
    k_zbi_update<KP><<<grid, kThreads, 0, s>>>(P);
    MPF_CUDA(cudaGetLastError());
    return MPF_OK;
}

template <int KP, int MP>
int zjac_kp(int F, const JacPlan& jp, int npad, const float* X, const float* gamma2, float* Jz, cudaStream_t s) {
    const dim3 grid(jp.Epad / 32, F);
    const size_t smem = sizeof(float2) * 2 * 3 * KP * 33;
    if (smem > 48 * 1024)
        MPF_CUDA(cudaFuncSetAttribute(k_zjacobian<KP, MP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    for (int ci = 0; ci < jp.Ca; ++ci)
        k_zjacobian<KP, MP><<<grid, 256, smem, s>>>(jp, npad, X, reinterpret_cast<const float2*>(gamma2),
                                                    reinterpret_cast<float2*>(Jz), ci);
    MPF_LAUNCHED(jp.Ca);
    return MPF_OK;
}

}  // namespace

int fem_launch_zjacobian(int F, const JacPlan& jp, int MP, int npad, const float* Xz, const float* gamma2, float* Jz,
                         cudaStream_t s) {
#define MPF_ZJAC(KPv, MPv) \
    if (jp.KP == KPv && MP == MPv) return zjac_kp<KPv, MPv>(F, jp, npad, Xz, gamma2, Jz, s);
    MPF_ZJAC(16, 16)
    MPF_ZJAC(32, 16)
    MPF_ZJAC(32, 32)
    MPF_ZJAC(64, 32)
#undef MPF_ZJAC
    return fail(MPF_ENOTSUP, "complex Jacobian: %d unique excitations with %d measurement rows", jp.KP, MP);
}

int fem_launch_ztranspose_jacobian(int F, int rowsJ, int Epad, int E, const float* Jz, float* Jref, cudaStream_t s) {
    dim3 grid((E + 31) / 32, (rowsJ + 31) / 32, F);
    k_ztranspose<<<grid, dim3(32, 8), 0, s>>>(rowsJ, Epad, E, reinterpret_cast<const float2*>(Jz),
                                              reinterpret_cast<float2*>(Jref));
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int zbicgstab_launch_init(const CgProblem& P, cudaStream_t s) {
    switch (P.KP) {
        case 16: return zinit_kp<16>(P, s);
        case 32: return zinit_kp<32>(P, s);
        case 64: return zinit_kp<64>(P, s);
        default: return fail(MPF_ENOTSUP, "complex admittivity: %d unique excitations (at most 64)", P.KP);
    }
}

int zbicgstab_launch_iteration(const CgProblem& P, cudaStream_t s) {
    switch (P.KP) {
        case 16: return ziter_kp<16>(P, s);
        case 32: return ziter_kp<32>(P, s);
        case 64: return ziter_kp<64>(P, s);
        default: return fail(MPF_ENOTSUP, "complex admittivity: %d unique excitations (at most 64)", P.KP);
    }
}

int fem_launch_zassemble(int F, int W, int npad, int E, const int32_t* cptr, const int32_t* contrib, const float* Kf,
                         const float* Mf, const float* gamma2, float ref, int logarithmic, float4* SRz, cudaStream_t s) {
    const size_t slots = (size_t)W * npad;
    const int blocks = (int)std::min<size_t>((slots + 255) / 256, 4096);
    k_zassemble<<<dim3(blocks, F), 256, 0, s>>>(W, npad, E, cptr, contrib, Kf, Mf,
                                                reinterpret_cast<const float2*>(gamma2), ref, logarithmic, SRz);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int cg_launch_zdc_shift(const CgProblem& P, const double* shift, float sign, cudaStream_t s) {
    k_zdc_shift<<<dim3(64, P.G), 256, 0, s>>>(P, shift, sign);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

// Complex potentials in the reference layout (EIT::fields): as
// k_fields_export, with interleaved (re, im) pairs.
__global__ void k_zfields_export(int F, int Ca, int C, const int32_t* __restrict__ compOf, int npad, int KP,
                                 int dataRows, int cols, const int32_t* __restrict__ colU,
                                 const float* __restrict__ colScale, const float* __restrict__ betaC,
                                 const float* __restrict__ Xz, const int32_t* __restrict__ rowOf,
                                 float* __restrict__ out, int n) {
    const size_t per = (size_t)dataRows * cols;
    const size_t total = (size_t)F * C * per;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int f = (int)(i / ((size_t)C * per));
        const int c = (int)((i / per) % C);
        const size_t r = i % per;
        const int node = (int)(r % dataRows), col = (int)(r / dataRows);
        const int ci = compOf[c];
        float2 v = make_float2(0.f, 0.f);
        if (ci >= 0 && node < n) {
            const float sc = betaC[c] * colScale[col];
            const float2 x = *reinterpret_cast<const float2*>(
                Xz + 2 * ((((size_t)f * Ca + ci) * npad + rowOf[node]) * KP + colU[col]));
            v = make_float2(sc * x.x, sc * x.y);
        }
        *reinterpret_cast<float2*>(out + 2 * i) = v;
    }
}

int fem_launch_zfields_export(int F, int Ca, int C, const int32_t* compOf, int npad, int KP, int dataRows, int cols,
                              int n, const int32_t* colU, const float* colScale, const float* betaC, const float* Xz,
                              const int32_t* rowOf, float* out, cudaStream_t s) {
    k_zfields_export<<<2048, 256, 0, s>>>(F, Ca, C, compOf, npad, KP, dataRows, cols, colU, colScale, betaC, Xz,
                                          rowOf, out, n);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_zgram_meas(int G, int KP, int npad, const int32_t* nzPtr, const int32_t* nzNode, const double* nzVal,
                          const float* Xz, double* Gmz, cudaStream_t s) {
    k_zgram_meas<<<G, 256, 0, s>>>(KP, npad, nzPtr, nzNode, nzVal, Xz, Gmz);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_zvoltages(int F, int Ca, int KP, int Mm, int Md, const double* Gmz, const float* beta,
                         const int32_t* measU, const float* measScale, const int32_t* driveU, const float* driveScale,
                         float* Vz, cudaStream_t s) {
    const int total = F * Mm * Md;
    k_zvoltages<<<(total + 255) / 256, 256, 0, s>>>(F, Ca, KP, Mm, Md, Gmz, beta, measU, measScale, driveU, driveScale,
                                                    Vz);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

}  // namespace mpf
