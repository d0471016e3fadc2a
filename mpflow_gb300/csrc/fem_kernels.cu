// FEM kernels of the EIT hot path: assembly, electrode voltages, Jacobian,
// layout exports and the Gauss-Newton residual / parameter update.
#include <cuda_bf16.h>

#include <algorithm>

#include "model.h"

namespace mpf {
namespace {

// src/fem/equation_kernel.cu:35-53: linear or dB-like logarithmic parameter.
__device__ __forceinline__ float mat_param(float ref, float v, int logarithmic) {
    return logarithmic ? ref * expf(2.302585093f * v / 10.f) : ref * v;
}
__device__ __forceinline__ double mat_param64(double ref, double v, int logarithmic) {
    return logarithmic ? ref * exp(2.302585092994046 * v / 10.0) : ref * v;
}
__device__ __forceinline__ float mat_param_deriv(float ref, float v, int logarithmic) {
    return logarithmic ? (2.302585093f / 10.f) * ref * expf(2.302585093f * v / 10.f) : ref;
}

// Assembly, restating updateMatrixKernel (src/fem/equation_kernel.cu:60-82):
// every slot sums its element contributions K_e[ij] * p(gamma_e) in element
// order, which is the reference's level order.  One thread per slot; the
// output is slot-major so the SpMM reads it coalesced.
__global__ void k_assemble(int W, int npad, int E, const int32_t* __restrict__ cptr,
                           const int32_t* __restrict__ contrib, const float* __restrict__ Kf,
                           const float* __restrict__ Mf, const double* __restrict__ Kd,
                           const double* __restrict__ Md, const float* __restrict__ gamma, float ref,
                           int logarithmic, float2* __restrict__ SR, size_t ld, size_t frameStride,
                           double* __restrict__ S64, double* __restrict__ R64) {
    const int f = blockIdx.y;
    const size_t slots = (size_t)W * npad;
    const float* gf = gamma + (size_t)f * E;
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < slots; s += (size_t)gridDim.x * blockDim.x) {
        const int c0 = __ldg(&cptr[s]), c1 = __ldg(&cptr[s + 1]);
        float vs = 0.f, vr = 0.f;
        double ds = 0.0, dr = 0.0;
        for (int c = c0; c < c1; ++c) {
            const int code = __ldg(&contrib[c]);
            // elements past E are contact elements of the complete electrode
            // model: parameter-free (weight 1)
            const int el = code / 9;
            const float g = el < E ? __ldg(&gf[el]) : 0.f;
            const float pg = el < E ? mat_param(ref, g, logarithmic) : 1.f;
            vs = fmaf(__ldg(&Kf[code]), pg, vs);
            vr = fmaf(__ldg(&Mf[code]), pg, vr);
            if (S64) {
                const double pg64 = el < E ? mat_param64((double)ref, (double)g, logarithmic) : 1.0;
                ds = fma(Kd[code], pg64, ds);
                dr = fma(Md[code], pg64, dr);
            }
        }
        SR[(size_t)f * frameStride + (s / npad) * ld + s % npad] = make_float2(vs, vr);
        if (S64) {
            S64[(size_t)f * slots + s] = ds;
            R64[(size_t)f * slots + s] = dr;
        }
    }
}

// slot-major [W][npad] -> reference ELL [dataRows][32] (same slot order)
// (rowOf maps a reference node number to the internal row)
__global__ void k_export_ell(int W, int npad, int n, int dataRows, const float2* __restrict__ src, int component,
                             const int32_t* __restrict__ rowOf, float* __restrict__ dst) {
    const int f = blockIdx.y;
    const size_t total = (size_t)dataRows * kEllWidth;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int row = (int)(i / kEllWidth), slot = (int)(i % kEllWidth);
        float v = 0.f;
        if (row < n && slot < W) {
            const float2 e = src[(size_t)f * W * npad + (size_t)slot * npad + rowOf[row]];
            v = component == 0 ? e.x : e.y;
        }
        dst[(size_t)f * total + i] = v;
    }
}

// Gm[g][u][v] = sum_n B0[n][u] * X[g][n][v] over the nonzeros of B0 (the
// excitation vectors only touch electrode nodes).
__global__ void k_gram_meas(int KP, int npad, int nnz, const int32_t* __restrict__ nzPtr,
                            const int32_t* __restrict__ nzNode, const double* __restrict__ nzVal,
                            const float* __restrict__ X, double* __restrict__ Gm) {
    const int g = blockIdx.x;
    const float* Xg = X + (size_t)g * npad * KP;
    for (int pair = threadIdx.x; pair < KP * KP; pair += blockDim.x) {
        const int u = pair / KP, v = pair % KP;
        double s = 0.0;
        for (int c = nzPtr[u]; c < nzPtr[u + 1]; ++c) s += nzVal[c] * (double)Xg[(size_t)nzNode[c] * KP + v];
        Gm[(size_t)g * KP * KP + pair] = s;
    }
    (void)nnz;
}

// V[f](m, d) = sum_c beta_c * sd * sm * Gm[f,c](um(m), ud(d)): the
// applyMeasurementPattern GEMM of src/models/eit.cpp:220-245 summed over the
// harmonics, on the unique excitation columns.
__global__ void k_voltages(int F, int Ca, int KP, int Mm, int Md, const double* __restrict__ Gm,
                           const float* __restrict__ beta, const int32_t* __restrict__ measU,
                           const float* __restrict__ measScale, const int32_t* __restrict__ driveU,
                           const float* __restrict__ driveScale, float* __restrict__ V) {
    const int total = F * Mm * Md;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int f = i / (Mm * Md), r = i % (Mm * Md);
        const int m = r % Mm, d = r / Mm;
        const int um = measU[m], ud = driveU[d];
        double s = 0.0;
        for (int ci = 0; ci < Ca; ++ci)
            s += (double)beta[ci] * Gm[((size_t)(f * Ca + ci) * KP + um) * KP + ud];
        V[i] = (float)(s * (double)measScale[m] * (double)driveScale[d]);
    }
}

// Jacobian, restating calcJacobianKernel (src/fem/equation_kernel.cu:197-245)
// for all harmonics at once:
//   J[d*MP + m][e] = -h p'(gamma_e) sd sm sum_c beta_c^2
//                    sum_ij Y_c[n_i][ud] K_e[i+3j] Y_c[n_j][um]
// i.e. per element a sum of 3 Ca outer products of a drive vector and a
// measurement vector.  A block owns 32 consecutive elements (lane = element)
// and 8 * DPT drive rows (grid z covers the rest); warp w owns drive rows
// [w*DPT, (w+1)*DPT) of the block and all MP measurement rows, DPT x MP
// accumulators per thread.  The field rows of the 96 element nodes (KP
// floats each) are gathered per harmonic with cp.async into a double buffer,
// one harmonic ahead of the arithmetic; they are then expanded in shared
// memory into the block's drive rows (multiplied by the element matrix and
// the harmonic weight) and the measurement rows, so the inner loop is DPT +
// MP conflict-free shared-memory loads for DPT * MP FMAs with no index
// lookups.  Output rows are 32 consecutive elements: coalesced stores.
__device__ __forceinline__ void jac_cp16(float* dst, const float* src, bool valid) {
    // 16 bytes, zero-filled when !valid (src-size 0)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

template <int KP, int MP, int DPT, bool ID>
__global__ void __launch_bounds__(256, 1) k_jacobian(JacPlan jp, int npad, const float* __restrict__ X,
                                                     const float* __restrict__ gamma, float* __restrict__ J,
                                                     __nv_bfloat16* __restrict__ Jhi,
                                                     __nv_bfloat16* __restrict__ Jlo) {
    constexpr int DB = 8 * DPT;      // drive rows of a block
    constexpr int RS = KP + 4;       // row stride of the gathered field rows (16-byte multiple)
    constexpr int CH = KP / 4;       // 16-byte chunks per field row
    constexpr int MS = MP + 4;       // element row stride of the measurement rows
    constexpr int DS = DB + 4;       // element row stride of the drive rows
    static_assert(MP % 4 == 0 && DPT % 2 == 0, "vector loads of the staged rows");
    extern __shared__ __align__(16) float jsm[];
    float* Yr = jsm;                                  // [2][96][RS] gathered field rows
    float* Ym = jsm + 2 * 96 * RS;                    // [3][32][MS]: Ym[j][el][m] = Y[n_j][um(m)]
    float* Td = Ym + 3 * 32 * MS;                     // [3][32][DS]: Td[j][el][d]
    float(*Ks)[9] = reinterpret_cast<float(*)[9]>(Td + 3 * 32 * DS);
    float(*Ms)[9] = Ks + 32;
    float(*Ke)[9] = Ks + 64;
    __shared__ int um[MP], ud[DB], nodeOf[96];
    const int f = blockIdx.y;
    if (jp.frameMask && !jp.frameMask[f]) return;
    const int e0 = blockIdx.x * 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int e = e0 + lane;
    const int drives = jp.rowsJ / MP;
    const int d0 = blockIdx.z * DB;
    for (int i = threadIdx.x; i < 32 * 9; i += 256) {
        const int el = i / 9, k = i % 9;
        const bool in = e0 + el < jp.E;
        Ks[el][k] = in ? jp.Kf[(size_t)(e0 + el) * 9 + k] : 0.f;
        Ms[el][k] = (in && jp.exact) ? jp.Mf[(size_t)(e0 + el) * 9 + k] : 0.f;
    }
    for (int i = threadIdx.x; i < MP; i += 256) um[i] = jp.rowM[i];
    for (int i = threadIdx.x; i < DB; i += 256) ud[i] = d0 + i < drives ? jp.rowD[(size_t)(d0 + i) * MP] : -1;
    for (int i = threadIdx.x; i < 96; i += 256) nodeOf[i] = e0 + i / 3 < jp.E ? jp.elements[(size_t)e0 * 3 + i] : -1;
    __syncthreads();
    // gather the field rows of harmonic ci into buffer b (row r = el * 3 + l)
    auto gather = [&](int ci, int b) {
        const float* Xg = X + ((size_t)f * jp.Ca + ci) * npad * KP;
        for (int i = threadIdx.x; i < 96 * CH; i += 256) {
            const int r = i / CH, c = i % CH;
            const int nd = nodeOf[r];
            jac_cp16(Yr + ((size_t)b * 96 + r) * RS + c * 4, Xg + (size_t)(nd < 0 ? 0 : nd) * KP + c * 4, nd >= 0);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    // accumulators as pairs of measurement rows: packed FP32x2 FMAs
    float2 acc[DPT][MP / 2];
#pragma unroll
    for (int a = 0; a < DPT; ++a)
#pragma unroll
        for (int m = 0; m < MP / 2; ++m) acc[a][m] = make_float2(0.f, 0.f);
    gather(0, 0);
    if constexpr (ID) {
        // identity maps: measurement row m is field column m and drive row d
        // is column d, so each thread reads its element's rows directly and
        // forms its own drive values from the element matrix in registers
        for (int ci = 0; ci < jp.Ca; ++ci) {
            if (ci + 1 < jp.Ca) {
                gather(ci + 1, (ci + 1) & 1);
                asm volatile("cp.async.wait_group 1;" ::: "memory");
            } else {
                asm volatile("cp.async.wait_group 0;" ::: "memory");
            }
            __syncthreads();  // harmonic ci's rows are in
            const float* Yb = Yr + (size_t)(ci & 1) * 96 * RS;
            const float mc = jp.massCoef[ci], b2 = jp.beta2[ci];
            float kv[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) kv[k] = b2 * (Ks[lane][k] + mc * Ms[lane][k]);
            const int dc = d0 + warp * DPT;  // first drive column of this warp
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) {
                float4 ym[MP / 4];
                const float4* yrow = reinterpret_cast<const float4*>(Yb + (lane * 3 + jj) * RS);
#pragma unroll
                for (int k = 0; k < MP / 4; ++k) ym[k] = yrow[k];
                float td[DPT];
#pragma unroll
                for (int a = 0; a < DPT; ++a) td[a] = 0.f;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const float* drow = Yb + (lane * 3 + q) * RS + dc;
                    float yd[DPT];
                    if constexpr (DPT % 4 == 0) {
#pragma unroll
                        for (int k = 0; k < DPT / 4; ++k) {
                            const float4 t = reinterpret_cast<const float4*>(drow)[k];
                            yd[4 * k] = t.x;
                            yd[4 * k + 1] = t.y;
                            yd[4 * k + 2] = t.z;
                            yd[4 * k + 3] = t.w;
                        }
                    } else {
#pragma unroll
                        for (int k = 0; k < DPT / 2; ++k) {
                            const float2 t = reinterpret_cast<const float2*>(drow)[k];
                            yd[2 * k] = t.x;
                            yd[2 * k + 1] = t.y;
                        }
                    }
#pragma unroll
                    for (int a = 0; a < DPT; ++a) td[a] = fmaf(yd[a], kv[q * 3 + jj], td[a]);
                }
#pragma unroll
                for (int a = 0; a < DPT; ++a) {
                    const float2 t2 = make_float2(td[a], td[a]);
#pragma unroll
                    for (int k = 0; k < MP / 4; ++k) {
                        acc[a][2 * k] = __ffma2_rn(t2, make_float2(ym[k].x, ym[k].y), acc[a][2 * k]);
                        acc[a][2 * k + 1] = __ffma2_rn(t2, make_float2(ym[k].z, ym[k].w), acc[a][2 * k + 1]);
                    }
                }
            }
            __syncthreads();  // every thread is done with buffer ci & 1 before it is refilled
        }
    } else {
    for (int ci = 0; ci < jp.Ca; ++ci) {
        // the buffer of harmonic ci + 1 was last read by the expansion of
        // ci - 1, which every thread finished before the barrier ahead of its
        // arithmetic
        if (ci + 1 < jp.Ca) {
            gather(ci + 1, (ci + 1) & 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        // element matrix of this harmonic: K (reference mode) or K + alpha_c M
        // (exact derivative of the 2.5D system matrix); Ke was last read by
        // the expansion of ci - 1, finished before the previous barrier
        const float mc = jp.massCoef[ci], b2 = jp.beta2[ci];
        for (int i = threadIdx.x; i < 32 * 9; i += 256) {
            const int el = i / 9, k = i % 9;
            Ke[el][k] = Ks[el][k] + mc * Ms[el][k];
        }
        __syncthreads();  // harmonic ci's rows and Ke are in; Ym / Td are free
        const float* Yb = Yr + (size_t)(ci & 1) * 96 * RS;
        // measurement rows (lanes along m: contiguous reads and writes)
        for (int i = threadIdx.x; i < 3 * MP * 32; i += 256) {
            const int m = i % MP, el = (i / MP) % 32, jj = i / (MP * 32);
            Ym[(jj * 32 + el) * MS + m] = um[m] >= 0 ? Yb[(el * 3 + jj) * RS + um[m]] : 0.f;
        }
        // drive rows: b2 sum_i Y[n_i][ud(d)] Ke[i + 3j] (lanes along d)
        for (int i = threadIdx.x; i < 3 * DB * 32; i += 256) {
            const int dl = i % DB, el = (i / DB) % 32, jj = i / (DB * 32);
            const int u = ud[dl];
            float v = 0.f;
            if (u >= 0)
                v = Yb[(el * 3 + 0) * RS + u] * Ke[el][jj] + Yb[(el * 3 + 1) * RS + u] * Ke[el][3 + jj] +
                    Yb[(el * 3 + 2) * RS + u] * Ke[el][6 + jj];
            Td[(jj * 32 + el) * DS + dl] = b2 * v;
        }
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
            float4 ym[MP / 4];
            const float4* yrow = reinterpret_cast<const float4*>(Ym + (jj * 32 + lane) * MS);
#pragma unroll
            for (int k = 0; k < MP / 4; ++k) ym[k] = yrow[k];
            float td[DPT];
            const float4* trow = reinterpret_cast<const float4*>(Td + (jj * 32 + lane) * DS + warp * DPT);
#pragma unroll
            for (int k = 0; k < DPT / 4; ++k) {
                const float4 t = trow[k];
                td[4 * k] = t.x;
                td[4 * k + 1] = t.y;
                td[4 * k + 2] = t.z;
                td[4 * k + 3] = t.w;
            }
            if constexpr (DPT % 4 != 0) {
                const float2 t = reinterpret_cast<const float2*>(Td + (jj * 32 + lane) * DS + warp * DPT)[DPT / 2 - 1];
                td[DPT - 2] = t.x;
                td[DPT - 1] = t.y;
            }
#pragma unroll
            for (int a = 0; a < DPT; ++a) {
                const float2 t2 = make_float2(td[a], td[a]);
#pragma unroll
                for (int k = 0; k < MP / 4; ++k) {
                    acc[a][2 * k] = __ffma2_rn(t2, make_float2(ym[k].x, ym[k].y), acc[a][2 * k]);
                    acc[a][2 * k + 1] = __ffma2_rn(t2, make_float2(ym[k].z, ym[k].w), acc[a][2 * k + 1]);
                }
            }
        }
    }
    }
    const bool valid = e < jp.E;
    const float deriv = valid ? -jp.height * mat_param_deriv(jp.ref, gamma[(size_t)f * jp.E + e], jp.logarithmic) : 0.f;
    const size_t base = (size_t)f * jp.rowsJ * jp.Epad;
#pragma unroll
    for (int a = 0; a < DPT; ++a) {
        const int d = d0 + warp * DPT + a;
        if (d >= drives) continue;
#pragma unroll
        for (int m = 0; m < MP; ++m) {
            const int row = d * MP + m;
            const float am = (m & 1) ? acc[a][m / 2].y : acc[a][m / 2].x;
            const float sc = (ID && jp.uniformScale > 0.f) ? jp.uniformScale : __ldg(&jp.rowScale[row]);
            const float v = valid ? deriv * sc * am : 0.f;
            const size_t o = base + (size_t)row * jp.Epad + e;
            if (jp.writeF32) J[o] = v;
            if (Jhi) {
                const __nv_bfloat16 h = __float2bfloat16_rn(v);
                Jhi[o] = h;
                Jlo[o] = __float2bfloat16_rn(v - __bfloat162float(h));
            }
        }
    }
}

// J [rowsJ][Epad] -> reference layout [E][rowsJ] (column-major rowsJ x E)
__global__ void k_transpose(int rowsJ, int Epad, int E, const float* __restrict__ J, float* __restrict__ Jref) {
    __shared__ float tile[32][33];
    const int f = blockIdx.z;
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    const float* src = J + (size_t)f * rowsJ * Epad;
    float* dst = Jref + (size_t)f * rowsJ * E;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        tile[i][threadIdx.x] = (r < rowsJ && c < E) ? src[(size_t)r * Epad + c] : 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (c < E && r < rowsJ) dst[(size_t)c * rowsJ + r] = tile[threadIdx.x][i];
    }
}

// Fields in the reference layout: out[f][c] is dataRows x (Md + Mm)
// column-major; column col of harmonic c is beta_c * scale_col * Y[u(col)].
__global__ void k_fields_export(int F, int Ca, int C, const int32_t* __restrict__ compOf, int npad, int KP,
                                int dataRows, int cols, const int32_t* __restrict__ colU,
                                const float* __restrict__ colScale, const float* __restrict__ betaC,
                                const float* __restrict__ X, const int32_t* __restrict__ rowOf,
                                float* __restrict__ out, int n) {
    const size_t per = (size_t)dataRows * cols;
    const size_t total = (size_t)F * C * per;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int f = (int)(i / ((size_t)C * per));
        const int c = (int)((i / per) % C);
        const size_t r = i % per;
        const int node = (int)(r % dataRows), col = (int)(r / dataRows);
        const int ci = compOf[c];
        float v = 0.f;
        if (ci >= 0 && node < n)
            v = betaC[c] * colScale[col] * X[(((size_t)f * Ca + ci) * npad + rowOf[node]) * KP + colU[col]];
        out[i] = v;
    }
}

// y = vec(v_meas - V) in the Jacobian's row order (d * MP + m), res = |y|/|v_meas|
__global__ void k_residual(int rowsJ, int Mm, int Md, int MP, const float* __restrict__ vMeas,
                           const float* __restrict__ V, double* __restrict__ y, double* __restrict__ res) {
    const int f = blockIdx.x;
    __shared__ double sy[256], sm[256];
    double ay = 0.0, am = 0.0;
    for (int row = threadIdx.x; row < rowsJ; row += blockDim.x) {
        const int m = row % MP, d = row / MP;
        double v = 0.0;
        if (m < Mm && d < Md) {
            const double meas = vMeas[(size_t)f * Mm * Md + m + (size_t)d * Mm];
            v = meas - (double)V[(size_t)f * Mm * Md + m + (size_t)d * Mm];
            am += meas * meas;
        }
        y[(size_t)f * rowsJ + row] = v;
        ay += v * v;
    }
    sy[threadIdx.x] = ay;
    sm[threadIdx.x] = am;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sy[threadIdx.x] += sy[threadIdx.x + s];
            sm[threadIdx.x] += sm[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) res[f] = sm[0] > 0.0 ? sqrt(sy[0] / sm[0]) : sqrt(sy[0]);
}

// gamma[e] += sum_r J[r][e] w[r]  (J^T w of the dual Gauss-Newton step,
// src/solver/inverse.cpp:198-204 then src/solver/solver.cpp:222)
__global__ void k_update_gamma(int rowsJ, int Epad, int E, const __nv_bfloat16* __restrict__ Jhi,
                               const __nv_bfloat16* __restrict__ Jlo, const double* __restrict__ w,
                               const int* __restrict__ frameActive, float* __restrict__ gamma) {
    extern __shared__ float ws[];
    const int f = blockIdx.y;
    if (frameActive && !frameActive[f]) return;
    for (int r = threadIdx.x; r < rowsJ; r += blockDim.x) ws[r] = (float)w[(size_t)f * rowsJ + r];
    __syncthreads();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const __nv_bfloat16* Hf = Jhi + (size_t)f * rowsJ * Epad;
    const __nv_bfloat16* Lf = Jlo + (size_t)f * rowsJ * Epad;
    float s = 0.f, c = 0.f;
    for (int r = 0; r < rowsJ; ++r) {
        // compensated float sum of J[r][e] * w[r]
        const float a = __bfloat162float(Hf[(size_t)r * Epad + e]) + __bfloat162float(Lf[(size_t)r * Epad + e]);
        const float b = ws[r];
        const float p = __fmul_rn(a, b), pe = __fmaf_rn(a, b, -p);
        const float t = __fadd_rn(s, p), z = __fsub_rn(t, s);
        const float te = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
        s = t;
        c = __fadd_rn(c, __fadd_rn(te, pe));
    }
    gamma[(size_t)f * E + e] += (float)((double)s + (double)c);
}

// gamma[f][:] = value for the frames with frameMask[f] != 0 (all if null)
__global__ void k_fill_frames(int E, const int* __restrict__ frameMask, float value, float* __restrict__ gamma) {
    const int f = blockIdx.y;
    if (frameMask && !frameMask[f]) return;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x)
        gamma[(size_t)f * E + e] = value;
}

// Learned-start input x[f][i] = (v[f][i] - V0[i]) * invRms and, optionally,
// the relative data residual of the homogeneous start |v - V0| / |v| per
// frame (one block per frame, fixed-order reduction).
__global__ void __launch_bounds__(256) k_learned_input(int L, const float* __restrict__ vMeas,
                                                       const float* __restrict__ V0, float invRms,
                                                       float* __restrict__ x, double* __restrict__ res0) {
    __shared__ double red[2][256];
    const int f = blockIdx.x;
    double dd = 0.0, vv = 0.0;
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        const float v = vMeas[(size_t)f * L + i], d = v - V0[i];
        x[(size_t)f * L + i] = d * invRms;
        dd += (double)d * d;
        vv += (double)v * v;
    }
    red[0][threadIdx.x] = dd;
    red[1][threadIdx.x] = vv;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            red[0][threadIdx.x] += red[0][threadIdx.x + st];
            red[1][threadIdx.x] += red[1][threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && res0) res0[f] = red[1][0] > 0.0 ? sqrt(red[0][0] / red[1][0]) : 0.0;
}

// bad[f] = 1 when an active frame's parameters left the range the forward
// model can take: a non-finite value, |gamma| > 100 (dB, log-conductivity)
// or gamma <= 0 (linear conductivity).  One block per frame.
__global__ void k_gamma_check(int E, const float* __restrict__ gamma, const int* __restrict__ frameActive,
                              int logarithmic, int* __restrict__ bad) {
    const int f = blockIdx.x;
    __shared__ int flag;
    if (threadIdx.x == 0) flag = 0;
    __syncthreads();
    if (!frameActive || frameActive[f]) {
        int b = 0;
        for (int e = threadIdx.x; e < E; e += blockDim.x) {
            const float g = gamma[(size_t)f * E + e];
            b |= !isfinite(g) || (logarithmic ? fabsf(g) > 100.f : g <= 0.f);
        }
        if (b) flag = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) bad[f] = flag;
}

// Unit right-hand sides of the learned start's linear prior: column i of B
// (rowsJ x Mm*Md) is e_{row(i)}, row(i) = m + d * MP the Jacobian row of
// measurement i = m + d * Mm.
__global__ void k_prior_rhs(int rowsJ, int Mm, int MP, int L, double* __restrict__ B) {
    const int i = blockIdx.y;
    const int row = i % Mm + (i / Mm) * MP;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rowsJ; r += gridDim.x * blockDim.x)
        B[(size_t)i * rowsJ + r] = r == row ? 1.0 : 0.0;
}

__global__ void k_prior_convert(size_t count, const double* __restrict__ B, double scale, float* __restrict__ Q) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x)
        Q[k] = (float)(B[k] * scale);
}

}  // namespace

int fem_launch_assemble(int F, int W, int npad, int E, const int32_t* cptr, const int32_t* contrib,
                        const float* Kf, const float* Mf, const double* Kd, const double* Md,
                        const float* gamma, float ref, int logarithmic, float2* SR, double* S64, double* R64,
                        cudaStream_t s, size_t ld, size_t frameStride) {
    const size_t slots = (size_t)W * npad;
    if (ld == 0) ld = npad;
    if (frameStride == 0) frameStride = slots;
    int blocks = (int)std::min<size_t>((slots + 255) / 256, 4096);
    k_assemble<<<dim3(blocks, F), 256, 0, s>>>(W, npad, E, cptr, contrib, Kf, Mf, Kd, Md, gamma, ref,
                                               logarithmic, SR, ld, frameStride, S64, R64);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_export_ell(int F, int W, int npad, int n, int dataRows, const float2* SR, int component,
                          const int32_t* rowOf, float* refLayout, cudaStream_t s) {
    int blocks = (int)std::min<size_t>(((size_t)dataRows * kEllWidth + 255) / 256, 4096);
    k_export_ell<<<dim3(blocks, F), 256, 0, s>>>(W, npad, n, dataRows, SR, component, rowOf, refLayout);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_gram_meas(int G, int KP, int npad, const MeasPlan& mp, const float* X, double* Gm,
                         cudaStream_t s) {
    k_gram_meas<<<G, 256, 0, s>>>(KP, npad, mp.nnz, mp.nzPtr, mp.nzNode, mp.nzVal, X, Gm);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_voltages(int F, int Ca, int KP, int Mm, int Md, const double* Gm, const float* beta,
                        const int32_t* measU, const float* measScale, const int32_t* driveU,
                        const float* driveScale, float* V, cudaStream_t s) {
    int total = F * Mm * Md;
    k_voltages<<<(total + 255) / 256, 256, 0, s>>>(F, Ca, KP, Mm, Md, Gm, beta, measU, measScale, driveU,
                                                   driveScale, V);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

template <int KP, int MP, int DPT, bool ID>
static int launch_jac_v(int F, const JacPlan& jp, int npad, const float* X, const float* gamma, float* J,
                        __nv_bfloat16* Jhi, __nv_bfloat16* Jlo, cudaStream_t s) {
    const int drives = jp.rowsJ / MP;
    dim3 grid(jp.Epad / 32, F, (drives + 8 * DPT - 1) / (8 * DPT));
    const size_t smem = sizeof(float) * (2 * 96 * (KP + 4) + 3 * 32 * (MP + 4) + 3 * 32 * (8 * DPT + 4) + 3 * 32 * 9);
    if (smem > 48 * 1024)
        MPF_CUDA(cudaFuncSetAttribute(k_jacobian<KP, MP, DPT, ID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    k_jacobian<KP, MP, DPT, ID><<<grid, 256, smem, s>>>(jp, npad, X, gamma, J, Jhi, Jlo);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

// the direct path needs every drive and measurement row of the block to be a
// field column: rows up to MP and to the block's drive range within KP
template <int KP, int MP, int DPT>
static int launch_jac(int F, const JacPlan& jp, int npad, const float* X, const float* gamma, float* J,
                      __nv_bfloat16* Jhi, __nv_bfloat16* Jlo, cudaStream_t s) {
    const int drives = jp.rowsJ / MP;
    const int driveCols = (drives + 8 * DPT - 1) / (8 * DPT) * (8 * DPT);
    if (jp.identity && MP <= KP && driveCols <= KP)
        return launch_jac_v<KP, MP, DPT, true>(F, jp, npad, X, gamma, J, Jhi, Jlo, s);
    return launch_jac_v<KP, MP, DPT, false>(F, jp, npad, X, gamma, J, Jhi, Jlo, s);
}

int fem_launch_jacobian(int F, const JacPlan& jp, int MP, int npad, const float* X, const float* gamma,
                               float* J, __nv_bfloat16* Jhi, __nv_bfloat16* Jlo, cudaStream_t s) {
    const int drives = jp.rowsJ / MP;
    // thread tile DPT x MP: DPT 4 up to 32 measurement rows, 2 for 64; fewer
    // drive rows than a block covers only leave warps idle
#define MPF_JAC(KPv, MPv, DPTv) \
    if (jp.KP == KPv && MP == MPv) return launch_jac<KPv, MPv, DPTv>(F, jp, npad, X, gamma, J, Jhi, Jlo, s);
    MPF_JAC(16, 16, 2)
    MPF_JAC(32, 16, 2)
    MPF_JAC(32, 32, 4)
    MPF_JAC(64, 32, 4)
    MPF_JAC(64, 64, 2)
    MPF_JAC(128, 64, 2)
#undef MPF_JAC
    return fail(MPF_ENOTSUP, "jacobian: unsupported shape KP=%d MP=%d drives=%d", jp.KP, MP, drives);
}

int fem_launch_transpose_jacobian(int F, int rowsJ, int Epad, int E, const float* J, float* Jref,
                                  cudaStream_t s) {
    dim3 grid((E + 31) / 32, (rowsJ + 31) / 32, F);
    k_transpose<<<grid, dim3(32, 8), 0, s>>>(rowsJ, Epad, E, J, Jref);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_fields_export(int F, int Ca, int C, const int32_t* compOf, int npad, int KP, int dataRows,
                               int cols, int n, const int32_t* colU, const float* colScale,
                               const float* betaC, const float* X, const int32_t* rowOf, float* out,
                               cudaStream_t s) {
    k_fields_export<<<2048, 256, 0, s>>>(F, Ca, C, compOf, npad, KP, dataRows, cols, colU, colScale, betaC, X,
                                         rowOf, out, n);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_residual(int F, int rowsJ, int Mm, int Md, const float* vMeas, const float* V, double* y,
                        double* res, cudaStream_t s) {
    const int MP = rowsJ / (int)data_rows((uint32_t)Md);
    k_residual<<<F, 256, 0, s>>>(rowsJ, Mm, Md, MP, vMeas, V, y, res);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_update_gamma(int F, int rowsJ, int Epad, int E, const __nv_bfloat16* Jhi, const __nv_bfloat16* Jlo,
                            const double* w, const int* frameActive, float* gamma, cudaStream_t s) {
    dim3 grid((E + 255) / 256, F);
    k_update_gamma<<<grid, 256, rowsJ * sizeof(float), s>>>(rowsJ, Epad, E, Jhi, Jlo, w, frameActive, gamma);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_fill_frames(int F, int E, const int* frameMask, float value, float* gamma, cudaStream_t s) {
    k_fill_frames<<<dim3((E + 255) / 256, F), 256, 0, s>>>(E, frameMask, value, gamma);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_gamma_check(int F, int E, const float* gamma, const int* frameActive, bool logarithmic, int* bad,
                           cudaStream_t s) {
    k_gamma_check<<<F, 256, 0, s>>>(E, gamma, frameActive, logarithmic ? 1 : 0, bad);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_prior_rhs(int rowsJ, int Mm, int Md, double* B, cudaStream_t s) {
    const int MP = rowsJ / (int)data_rows((uint32_t)Md);
    MPF_CHECK(MP >= Mm && Mm * Md <= 65535, MPF_EINVAL, "learned prior: %d x %d measurements", Mm, Md);
    k_prior_rhs<<<dim3((rowsJ + 255) / 256, Mm * Md), 256, 0, s>>>(rowsJ, Mm, MP, Mm * Md, B);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_prior_convert(int rowsJ, int L, const double* B, double scale, float* Q, cudaStream_t s) {
    const size_t count = (size_t)rowsJ * L;
    k_prior_convert<<<(int)std::min<size_t>((count + 255) / 256, 4096), 256, 0, s>>>(count, B, scale, Q);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

int fem_launch_learned_input(int F, int L, const float* vMeas, const float* V0, float invRms, float* x,
                             double* res0, cudaStream_t s) {
    k_learned_input<<<F, 256, 0, s>>>(L, vMeas, V0, invRms, x, res0);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

}  // namespace mpf
