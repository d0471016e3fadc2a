// State of one device-resident EIT model (the object behind mpf_eit_t),
// shared by the translation units that orchestrate it (model.cu, inverse.cu).
#pragma once

#include <array>
#include <map>
#include <string>
#include <vector>

#include "model.h"

struct mpf_eit {
    // sizes (n: rows of the system -- the mesh nodes, plus one electrode
    // voltage per port in the complete electrode model; nNodes: mesh nodes)
    int nNodes = 0;
    int cem = 0;
    double contactZ = 0.0;
    int n = 0, E = 0, dataRows = 0, npad = 0, nblk = 0, W = 0, levels = 0;
    int L = 0, Md = 0, Mm = 0, MdPad = 0, MmPad = 0, rowsJ = 0, Epad = 0;
    int K = 0, KP = 0, C = 0, Ca = 0;
    int sourceType = 0, logarithmic = 0, device = 0;
    float ref = 1.f;
    double height = 1.0, portHeight = 1.0;
    // host copies
    mpf::FemStructure fs;
    std::vector<int> compOf;          // component -> active index or -1
    std::vector<float> alphaH, betaH; // per active component
    std::vector<double> betaAll;      // per component
    // device: static structure
    mpf::DevBuf<int32_t> cols, diagSlot, cptr, contrib, elements;
    mpf::DevBuf<int32_t> haloRows, haloCnt;  // halo plan of the tile-staged SpMM (mpf::HaloPlan)
    mpf::DevBuf<uint16_t> haloLcol;
    int Hpad = 0;
    mpf::DevBuf<int32_t> rowOf;       // internal row of each node (Morton order, see eit_create)
    mpf::DevBuf<float> Kf, Mf;
    mpf::DevBuf<double> Kd, Md64;
    mpf::DevBuf<float> Bc;            // [Ca][npad][KP] right-hand sides per active harmonic
    mpf::DevBuf<double> Bc64;
    mpf::DevBuf<float> alpha, beta, beta2, betaC, massCoef;
    int exactJacobian = 0;
    int jacIdentity = 0;              // drive / measurement rows are the unique columns in order (JacPlan)
    float jacUniformScale = 0.f;      // the common row scale of the Jacobian, or 0
    mpf::DevBuf<int32_t> dcFree, compOfD;
    mpf::DevBuf<int32_t> nzPtr, nzNode;
    mpf::DevBuf<double> nzVal;
    mpf::DevBuf<int32_t> driveU, measU, rowD, rowM, colU;
    mpf::DevBuf<float> driveScale, measScale, rowScale, colScale;
    int anyDcFree = 0;
    float dcScale = 1.f;              // c' of the Neumann rank-one term
    mpf::DevBuf<double> dcShift;      // [KP] constant difference to the reference's solution
    // workspace, grown on demand
    int capF = 0, capF64 = 0, capFJ = 0;
    mpf::DevBuf<float2> SR;           // slot values {S, R} per frame
    mpf::DevBuf<float> X, Rv, Pv, Qv;
    mpf::DevBuf<double> S64, R64, X64;
    mpf::DevBuf<double> partA, partB, partC, rz, pq, bz, betaW, rr, bb, Gm, sumP, sumX;
    mpf::DevBuf<int> conv, active, iters, pend;
    mpf::DevBuf<unsigned> counter;
    mpf::DevBuf<double> alphaX;
    // BiCGSTAB vectors and scalars (grown on first use)
    int capFB = 0;
    mpf::DevBuf<float> Rhat, Zv, Tv;
    mpf::DevBuf<double> omegaW, rr2W;
    // complex admittivity (complex_kernels.cu): complex slot values, seven
    // complex vectors, imaginary parts of the scalars, complex Gram
    int capFZ = 0;
    mpf::DevBuf<float4> SRz;
    mpf::DevBuf<float> Xz, Rz, Yz, Nz, Hz, Zz, Tz, Vz;
    mpf::DevBuf<double> zRhoI, zAlphaI, zBetaI, zOmega, zOmegaI, zSumI, zRr, Gmz;
    mpf::DevBuf<float> Jz;  // complex Jacobian [F][rowsJ][Epad] (re, im), on request
    mpf::DevBuf<float> V, J, gramWork;
    mpf::DevBuf<__nv_bfloat16> Jhi, Jlo;
    mpf::DevBuf<double> A64, y, res;
    mpf::DevBuf<int> info, frameMask, redoMask, fbMask, solveMask, upMask, skipMask, groupMask;
    // FP32 factor of the Gauss-Newton system with FP64 refinement (gn_update)
    mpf::DevBuf<double> cholL, cholX, cholR, cholY, cholRR, cholYY, cholW;
    mpf::DevBuf<float> cholL32, cholD, cholInv, cholInvT;  // the FP32 factor, its inverse and transpose
    mpf::DevBuf<int> info32, cholMask;
    long long nnz = 0;                // used ELL slots (matrix nonzeros)
    std::vector<int> activeHost, itersHost;
    int* pinnedActive = nullptr;
    bool fieldsValid = false;
    int lastFrames = 0;
    bool zFieldsValid = false;  // complex fields of the last complex solve
    int zLastFrames = 0;
    // captured CG iteration chunks keyed by the problem bytes
    std::map<std::string, cudaGraphExec_t> graphs;
    // CG kernel variants {spmm, update, direction}: autotuned per frame count,
    // or fixed by the caller (-1 = autotune)
    std::map<int, std::array<int, 3>> cgVariants;
    std::array<int, 3> forcedVariants{-1, -1, -1};
    // two-level preconditioner: aggregate plan (static) and per-frame-count workspace
    int nc = 0, ncPad = 0, coarseOK = 0, capFC = 0;
    mpf::DevBuf<int32_t> cPairI, cPairJ, cPairPtr, cSlots;
    mpf::DevBuf<float> cAggSize;
    int cNnz = 0;
    mpf::DevBuf<double> Ac64, Lc64, rzFine, bzFine;
    mpf::DevBuf<float> Lc, LinvD, Binv, rcV, rcB, ycV;
    mpf::DevBuf<int> infoC;
    // voltage (Fixed) sources: Dirichlet rows on port nodes (fixed_kernels.cu)
    int fixed = 0;
    mpf::DevBuf<int32_t> fxZero, fxDiag;                               // slots to clear / Dirichlet diagonals
    mpf::DevBuf<int32_t> fxLiftPtr, fxLiftRow, fxLiftSlot, fxLiftCol;  // interior rows with port-node columns
    mpf::DevBuf<int32_t> fxCurPtr, fxCurRow, fxCurSlot, fxCurCol;      // port-node rows (all their slots)
    int fxNZero = 0, fxNLift = 0, capFX = 0;
    mpf::DevBuf<float> bFix, curX;                                     // per-group right-hand sides, port currents
    mpf::DevBuf<float2> dVals;                                         // unmasked slot values of port-node rows
    // host copy of the mesh (reference numbering) for the Laplacian regulariser
    std::vector<double> hostNodes;
    std::vector<int32_t> hostElements;
    // regularised inverse (mpf_inverse_solve) workspace
    mpf::DevBuf<float> invJ, invWork;
    mpf::DevBuf<__nv_bfloat16> invHi, invLo;
    mpf::DevBuf<double> invA, invY, invB, invYs, invR, invU;
    mpf::DevBuf<int> invInfo;
    mpf::DevBuf<int32_t> lapRow, lapCol;
    mpf::DevBuf<double> lapVal;
    // learned warm start: homogeneous voltages and the network input
    bool v0Ready = false;
    float v0InvRms = 1.f;
    mpf::DevBuf<float> V0, X0, learnX;
    mpf::DevBuf<double> res0;
    // Gauss-Newton loop: parameters before the update, frames it sent out of range
    mpf::DevBuf<float> gammaPrev;
    mpf::DevBuf<int> badFrame;
    // linear prior of the learned start (mpf_eit_learned_prior): W = J0^T
    // (J0 J0^T + mu I)^-1 / invRms, column-major E x L with ld Epad
    bool priorReady = false;
    double priorLambda = 0.0;
    mpf::DevBuf<float> priorW;
    // the prior as split-BF16 operands of the tensor-core product: W (E x L)
    // as [priorN][3 priorLp] (hi, hi, lo) and the inputs of a call as
    // [frames padded to 128][3 priorLp] (hi, lo, hi)
    mpf::DevBuf<__nv_bfloat16> priorB, priorA;
    int priorN = 0, priorLp = 0;

    // device-time breakdown by phase (mpf_eit_phase_times): while enabled,
    // phase_mark records an event on the stream at every change of phase;
    // phase_flush adds the time between consecutive marks to their phase
    bool phaseOn = false;
    std::vector<cudaEvent_t> phaseEvents;
    std::vector<int> phaseIds;
    int phaseUsed = 0;
    double phaseMs[MPF_PHASES] = {};
    long long phaseCalls = 0;

    ~mpf_eit() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        if (pinnedActive) cudaFreeHost(pinnedActive);
        for (auto e : phaseEvents) cudaEventDestroy(e);
    }
};

namespace mpf {
// phase timer (model.cu): the phase the stream's work enters after this point
int phase_mark(mpf_eit* m, int phase, cudaStream_t s);
// attribute the marked intervals to their phases (synchronises)
int phase_flush(mpf_eit* m, cudaStream_t s);
// fixed_kernels.cu: voltage (Fixed) sources
int fixed_plan(mpf_eit* m, const std::vector<double>& excBin);
int fixed_prepare(mpf_eit* m, int F, cudaStream_t s);
int fixed_currents(mpf_eit* m, int F, cudaStream_t s);
}  // namespace mpf
