// Voltage (Fixed) sources, EIT::applyMixedBoundaryCondition and the current
// read-out of EIT::solve (src/models/eit.cpp:85-91,160-205,251-270,
// src/models/eit_kernel.cu:34-54).  The reference binarises the excitation
// matrix, overwrites the rows of every port node with identity rows (the
// port voltage is prescribed there) and runs CG on the resulting
// non-symmetric matrix; afterwards it measures the currents height * A x
// with the unmodified matrix.  Here the same Dirichlet problem is solved in
// its symmetric form, which CG is defined for: port-node rows and columns
// are cleared (diagonal 1) and the known port voltages move to the
// right-hand side of the interior rows,
//   b_i = -sum_{j in ports} A_ij g_j,   b_j = g_j.
// The solution is the same; only the iteration differs.
#include <algorithm>

#include "eit_state.h"

namespace mpf {
namespace {

// per group: b = 0 except port rows (g) and interior rows next to ports (lift)
__global__ void k_fixed_rhs(int nPort, const int32_t* __restrict__ portRow, int nLift,
                            const int32_t* __restrict__ liftPtr, const int32_t* __restrict__ liftRow,
                            const int32_t* __restrict__ liftSlot, const int32_t* __restrict__ liftCol, int W, int npad,
                            int KP, int Ca, const float2* __restrict__ SR, const float* __restrict__ alpha,
                            const float* __restrict__ B0, float* __restrict__ b) {
    const int g = blockIdx.y, f = g / Ca;
    const float a = alpha[g % Ca];
    const float2* sr = SR + (size_t)f * W * npad;
    float* bg = b + (size_t)g * npad * KP;
    const int total = (nPort + nLift) * KP;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int i = t / KP, u = t % KP;
        if (i < nPort) {
            const int r = portRow[i];
            bg[(size_t)r * KP + u] = B0[(size_t)r * KP + u];
        } else {
            const int l = i - nPort;
            float s = 0.f;
            for (int k = liftPtr[l]; k < liftPtr[l + 1]; ++k) {
                const float2 e = sr[liftSlot[k]];
                s = fmaf(e.x + a * e.y, B0[(size_t)liftCol[k] * KP + u], s);
            }
            bg[(size_t)liftRow[l] * KP + u] = -s;
        }
    }
}

__global__ void k_fixed_save(int nSlots, const int32_t* __restrict__ slots, int W, int npad,
                             const float2* __restrict__ SR, float2* __restrict__ saved) {
    const int f = blockIdx.y;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nSlots; t += gridDim.x * blockDim.x)
        saved[(size_t)f * nSlots + t] = SR[(size_t)f * W * npad + slots[t]];
}

__global__ void k_fixed_mask(int nZero, const int32_t* __restrict__ zero, int nDiag, const int32_t* __restrict__ diag,
                             int W, int npad, float2* __restrict__ SR) {
    float2* sr = SR + (size_t)blockIdx.y * W * npad;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nZero + nDiag; t += gridDim.x * blockDim.x) {
        if (t < nZero)
            sr[zero[t]] = make_float2(0.f, 0.f);
        else
            sr[diag[t - nZero]] = make_float2(1.f, 0.f);
    }
}

// port currents I[r] = sum over the (unmodified) slots of port row r of
// (S + alpha R) x[col], for every group and right-hand side
__global__ void k_fixed_currents(int nPort, const int32_t* __restrict__ curPtr, const int32_t* __restrict__ curRow,
                                 const int32_t* __restrict__ curCol, int nSlots, const float2* __restrict__ saved,
                                 int npad, int KP, int Ca, const float* __restrict__ alpha, const float* __restrict__ X,
                                 float* __restrict__ cur) {
    const int g = blockIdx.y, f = g / Ca;
    const float a = alpha[g % Ca];
    const float2* sv = saved + (size_t)f * nSlots;
    const float* xg = X + (size_t)g * npad * KP;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nPort * KP; t += gridDim.x * blockDim.x) {
        const int i = t / KP, u = t % KP;
        float s = 0.f;
        for (int k = curPtr[i]; k < curPtr[i + 1]; ++k) s = fmaf(sv[k].x + a * sv[k].y, xg[(size_t)curCol[k] * KP + u], s);
        cur[(size_t)g * npad * KP + (size_t)curRow[i] * KP + u] = s;
    }
}

}  // namespace

// Host plan: port nodes (rows with a nonzero binarised excitation), the slots
// to clear, the lift lists of interior rows and the read-out lists of port rows.
int fixed_plan(mpf_eit* m, const std::vector<double>& excBin) {
    const int n = m->n, P = m->npad, W = m->W;
    std::vector<char> port(n, 0);
    for (int p = 0; p < m->L; ++p)
        for (int r = 0; r < n; ++r)
            if (excBin[r + (size_t)p * n] != 0.0) port[r] = 1;
    std::vector<int32_t> zero, diag, liftPtr{0}, liftRow, liftSlot, liftCol, curPtr{0}, curRow, curSlot, curCol;
    for (int r = 0; r < n; ++r) {
        bool lifted = false;
        for (int k = 0; k < W; ++k) {
            const int32_t slot = k * P + r, c = m->fs.cols[(size_t)slot];
            if (c == r && k != m->fs.diagSlot[r]) continue;  // padding slot
            if (port[r]) {
                curSlot.push_back(slot);
                curCol.push_back(c);
                if (k == m->fs.diagSlot[r])
                    diag.push_back(slot);
                else
                    zero.push_back(slot);
            } else if (port[c]) {
                liftSlot.push_back(slot);
                liftCol.push_back(c);
                zero.push_back(slot);
                lifted = true;
            }
        }
        if (port[r]) {
            curRow.push_back(r);
            curPtr.push_back((int32_t)curSlot.size());
        } else if (lifted) {
            liftRow.push_back(r);
            liftPtr.push_back((int32_t)liftSlot.size());
        }
    }
    MPF_CHECK(!curRow.empty(), MPF_EINVAL, "mpf_eit_create: voltage sources need at least one port node");
    m->fxNZero = (int)zero.size();
    m->fxNLift = (int)liftRow.size();
    // keep every upload non-empty
    if (zero.empty()) zero.push_back(0);
    if (liftRow.empty()) liftRow.push_back(0);
    if (liftSlot.empty()) {
        liftSlot.push_back(0);
        liftCol.push_back(0);
    }
    MPF_TRY(m->fxZero.upload(zero));
    MPF_TRY(m->fxDiag.upload(diag));
    MPF_TRY(m->fxLiftPtr.upload(liftPtr));
    MPF_TRY(m->fxLiftRow.upload(liftRow));
    MPF_TRY(m->fxLiftSlot.upload(liftSlot));
    MPF_TRY(m->fxLiftCol.upload(liftCol));
    MPF_TRY(m->fxCurPtr.upload(curPtr));
    MPF_TRY(m->fxCurRow.upload(curRow));
    MPF_TRY(m->fxCurSlot.upload(curSlot));
    MPF_TRY(m->fxCurCol.upload(curCol));
    return MPF_OK;
}

// After assembly: keep the port rows' values, build the per-group
// right-hand sides, then clear the Dirichlet rows and columns.
int fixed_prepare(mpf_eit* m, int F, cudaStream_t s) {
    const int G = F * m->Ca, P = m->npad, KP = m->KP;
    const int nCur = (int)m->fxCurSlot.count, nPort = (int)m->fxCurRow.count, nLift = m->fxNLift;
    if (F > m->capFX) {
        MPF_TRY(m->bFix.alloc((size_t)G * P * KP));
        MPF_TRY(m->curX.alloc((size_t)G * P * KP));
        MPF_TRY(m->dVals.alloc((size_t)F * nCur));
        m->capFX = F;
    }
    k_fixed_save<<<dim3((nCur + 255) / 256, F), 256, 0, s>>>(nCur, m->fxCurSlot.ptr, m->W, P, m->SR.ptr, m->dVals.ptr);
    MPF_CUDA(cudaMemsetAsync(m->bFix.ptr, 0, sizeof(float) * (size_t)G * P * KP, s));
    const int work = (nPort + nLift) * KP;
    k_fixed_rhs<<<dim3(std::min((work + 255) / 256, 1024), G), 256, 0, s>>>(
        nPort, m->fxCurRow.ptr, nLift, m->fxLiftPtr.ptr, m->fxLiftRow.ptr, m->fxLiftSlot.ptr, m->fxLiftCol.ptr, m->W, P,
        KP, m->Ca, m->SR.ptr, m->alpha.ptr, m->Bc.ptr, m->bFix.ptr);
    const int nz = m->fxNZero, nd = (int)m->fxDiag.count;
    k_fixed_mask<<<dim3((nz + nd + 255) / 256, F), 256, 0, s>>>(nz, m->fxZero.ptr, nd, m->fxDiag.ptr, m->W, P,
                                                                  m->SR.ptr);
    MPF_LAUNCHED(3);
    return MPF_OK;
}

// Port currents of the solved fields (without the height, which the voltage
// weights carry) into curX.
int fixed_currents(mpf_eit* m, int F, cudaStream_t s) {
    const int G = F * m->Ca, P = m->npad, KP = m->KP, nPort = (int)m->fxCurRow.count;
    MPF_CUDA(cudaMemsetAsync(m->curX.ptr, 0, sizeof(float) * (size_t)G * P * KP, s));
    k_fixed_currents<<<dim3(std::min((nPort * KP + 255) / 256, 1024), G), 256, 0, s>>>(
        nPort, m->fxCurPtr.ptr, m->fxCurRow.ptr, m->fxCurCol.ptr, (int)m->fxCurSlot.count, m->dVals.ptr, P, KP, m->Ca,
        m->alpha.ptr, m->X.ptr, m->curX.ptr);
    MPF_LAUNCHED(1);
    return MPF_OK;
}

}  // namespace mpf
