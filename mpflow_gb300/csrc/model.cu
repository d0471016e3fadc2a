// EIT model: host-side setup of the device-resident structure and the
// orchestration of the forward solve (EIT::solve, src/models/eit.cpp:139-213),
// of the regularised Gauss-Newton step and loop (Solver::solveAbsolute,
// src/solver/solver.cpp:196-225 with Inverse, src/solver/inverse.cpp:60-238;
// per-frame masks, undo and freeze of diverging frames), and of the learned
// warm start (the linear one-step GN prior and the network's correction).
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>

#include "model.h"

#include "eit_state.h"

namespace mpf {
namespace {

int check_device(mpf_eit* m) {
    MPF_CUDA(cudaSetDevice(m->device));
    return MPF_OK;
}

// first nonzero entry of a pattern column, 0 for an all-zero column
double lead(const double* col, int L) {
    for (int i = 0; i < L; ++i)
        if (col[i] != 0.0) return col[i];
    return 0.0;
}

}  // namespace

int phase_mark(mpf_eit* m, int phase, cudaStream_t s) {
    if (!m->phaseOn) return MPF_OK;
    if (m->phaseUsed == (int)m->phaseEvents.size()) {
        cudaEvent_t e;
        MPF_CUDA(cudaEventCreate(&e));
        m->phaseEvents.push_back(e);
        m->phaseIds.push_back(0);
    }
    MPF_CUDA(cudaEventRecord(m->phaseEvents[m->phaseUsed], s));
    m->phaseIds[m->phaseUsed++] = phase;
    return MPF_OK;
}

int phase_flush(mpf_eit* m, cudaStream_t s) {
    if (!m->phaseOn || m->phaseUsed == 0) return MPF_OK;
    MPF_TRY(phase_mark(m, MPF_PHASE_HOST, s));
    MPF_CUDA(cudaEventSynchronize(m->phaseEvents[m->phaseUsed - 1]));
    for (int i = 0; i + 1 < m->phaseUsed; ++i) {
        float t = 0.f;
        MPF_CUDA(cudaEventElapsedTime(&t, m->phaseEvents[i], m->phaseEvents[i + 1]));
        m->phaseMs[m->phaseIds[i]] += t;
    }
    m->phaseUsed = 0;
    ++m->phaseCalls;
    return MPF_OK;
}

int phase_times(mpf_eit* m, int enable, double* ms, int cap, int64_t* calls) {
    if (ms)
        for (int i = 0; i < cap && i < MPF_PHASES; ++i) ms[i] = m->phaseMs[i];
    if (calls) *calls = m->phaseCalls;
    if (enable >= 0) {
        m->phaseOn = enable != 0;
        m->phaseUsed = 0;
        m->phaseCalls = 0;
        for (double& v : m->phaseMs) v = 0.0;
    }
    return MPF_OK;
}

int eit_create(const mpf_eit_desc* d, mpf_eit** out) {
    MPF_CHECK(d && out, MPF_EINVAL, "mpf_eit_create: null argument");
    MPF_CHECK(d->n_nodes > 0 && d->n_elements > 0 && d->nodes && d->elements && d->edges && d->port_edges,
              MPF_EINVAL, "mpf_eit_create: mesh == nullptr");
    MPF_CHECK(d->ports > 0 && d->drive_count > 1 && d->meas_count > 1, MPF_EINVAL,
              "mpf_eit_create: need ports > 0 and at least two drive and measurement patterns");
    MPF_CHECK(d->drive_pattern && d->meas_pattern && d->source_values, MPF_EINVAL,
              "mpf_eit_create: pattern == nullptr");
    MPF_CHECK(d->components >= 1, MPF_EINVAL, "mpflow::models::EIT::EIT: components < 1");
    MPF_CHECK(d->height > 0.0, MPF_EINVAL, "mpFlow::models::EIT::EIT: height <= 0.0");
    MPF_CHECK(d->port_height > 0.0, MPF_EINVAL, "mpFlow::models::EIT::EIT: portHeight <= 0.0");
    MPF_CHECK(d->source_type == MPF_SOURCE_OPEN || d->source_type == MPF_SOURCE_FIXED, MPF_EINVAL,
              "mpf_eit_create: unknown source type %d", d->source_type);
    MPF_CHECK(!(d->source_type == MPF_SOURCE_FIXED && d->jacobian_mode == 1), MPF_ENOTSUP,
              "mpf_eit_create: the exact 2.5D Jacobian is implemented for current (open) sources only");
    MPF_CHECK(d->contact_impedance >= 0.0 && std::isfinite(d->contact_impedance), MPF_EINVAL,
              "mpf_eit_create: contact_impedance must be >= 0 (0: gap model)");
    MPF_CHECK(!(d->contact_impedance > 0.0 && d->source_type == MPF_SOURCE_FIXED), MPF_ENOTSUP,
              "mpf_eit_create: the complete electrode model is implemented for current (open) sources only");
    auto m = std::make_unique<mpf_eit>();
    m->device = d->device;
    MPF_TRY(check_device(m.get()));
    m->nNodes = d->n_nodes;
    m->cem = d->contact_impedance > 0.0 ? 1 : 0;
    m->contactZ = d->contact_impedance;
    m->E = d->n_elements;
    m->L = d->ports;
    // complete electrode model: the electrode voltages are rows nNodes .. nNodes + L - 1
    m->n = m->nNodes + (m->cem ? m->L : 0);
    m->Md = d->drive_count;
    m->Mm = d->meas_count;
    m->MdPad = (int)data_rows((uint32_t)m->Md);
    m->MmPad = (int)data_rows((uint32_t)m->Mm);
    m->rowsJ = m->MdPad * m->MmPad;
    m->Epad = round_up(m->E, kElemTile);
    m->sourceType = d->source_type;
    m->ref = (float)d->reference_value;
    m->logarithmic = d->logarithmic ? 1 : 0;
    m->C = d->components;
    m->height = d->height;
    m->portHeight = d->port_height;

    m->hostNodes.assign(d->nodes, d->nodes + (size_t)2 * m->nNodes);
    m->hostElements.assign(d->elements, d->elements + (size_t)3 * m->E);

    // ---- internal node order: Morton (Z-order) of the coordinates, so that
    // consecutive rows are spatially compact patches (SpMM gathers stay in
    // L1, and the two-level preconditioner's aggregates of consecutive rows
    // are compact).  Elements keep their order; every node-indexed export
    // maps back through rowOf.
    const int N = m->nNodes;
    std::vector<int32_t> perm(N), rowOf(N);
    morton_order(N, d->nodes, perm.data());
    for (int i = 0; i < N; ++i) rowOf[perm[i]] = i;
    std::vector<int32_t> elems((size_t)3 * m->E);
    for (size_t k = 0; k < elems.size(); ++k) elems[k] = rowOf[d->elements[k]];
    std::vector<int32_t> edgesP((size_t)2 * d->n_edges);
    for (size_t k = 0; k < edgesP.size(); ++k) edgesP[k] = rowOf[d->edges[k]];
    std::vector<double> nodesP((size_t)2 * N);
    for (int i = 0; i < N; ++i) {
        nodesP[2 * i] = d->nodes[2 * (size_t)perm[i]];
        nodesP[2 * i + 1] = d->nodes[2 * (size_t)perm[i] + 1];
    }

    // ---- complete electrode model: every boundary edge (a, b) of port l is a
    // contact element on (a, b, U_l) with the element matrix of
    //   (1/z) int_edge (u - U_l)(v - V_l) ds,
    // 1/z [[h/3, h/6, -h/2], [h/6, h/3, -h/2], [-h/2, -h/2, h]] for an edge of
    // length h (P1 on the edge); it enters the structure and the assembly like
    // a triangle whose parameter is 1, so S carries it in every harmonic
    std::vector<int32_t> elemsAll = elems;
    std::vector<double> Kc, Mc;
    if (m->cem) {
        const double iz = 1.0 / m->contactZ;
        for (int l = 0; l < m->L; ++l) {
            int edgesOnPort = 0;
            for (int k = 0; k < d->port_edges_cap; ++k) {
                const int32_t eg = d->port_edges[(size_t)l * d->port_edges_cap + k];
                if (eg < 0) continue;
                MPF_CHECK(eg < d->n_edges, MPF_EINVAL, "mpf_eit_create: port %d names edge %d of %d", l, eg,
                          d->n_edges);
                const int32_t a = d->edges[2 * (size_t)eg], b = d->edges[2 * (size_t)eg + 1];
                const double h = std::hypot(d->nodes[2 * (size_t)a] - d->nodes[2 * (size_t)b],
                                            d->nodes[2 * (size_t)a + 1] - d->nodes[2 * (size_t)b + 1]);
                elemsAll.push_back(rowOf[a]);
                elemsAll.push_back(rowOf[b]);
                elemsAll.push_back(N + l);
                const double ke[9] = {h / 3, h / 6, -h / 2, h / 6, h / 3, -h / 2, -h / 2, -h / 2, h};
                for (double v : ke) {
                    Kc.push_back(iz * v);
                    Mc.push_back(0.0);
                }
                ++edgesOnPort;
            }
            MPF_CHECK(edgesOnPort > 0, MPF_EINVAL, "mpf_eit_create: port %d has no boundary edge", l);
        }
    }
    const int Eall = (int)(elemsAll.size() / 3);

    // ---- FEM structure and elemental integrals
    MPF_TRY(build_structure(m->n, Eall, elemsAll.data(), m->fs));
    m->dataRows = (int)data_rows((uint32_t)m->nNodes);  // node-indexed exports (mesh nodes only)
    m->npad = m->fs.npad;
    m->nblk = m->npad / kRowTile;
    m->W = m->fs.density;
    m->levels = m->fs.levels;
    for (uint32_t c : m->fs.refColIds) m->nnz += c != kInvalid;
    std::vector<double> K((size_t)m->E * 9), M((size_t)m->E * 9);
    p1_elemental(m->E, d->nodes, d->elements, K.data(), M.data());
    K.insert(K.end(), Kc.begin(), Kc.end());  // contact elements follow the triangles
    M.insert(M.end(), Mc.begin(), Mc.end());
    std::vector<float> Kf(K.begin(), K.end()), Mf(M.begin(), M.end());

    // ---- excitation matrix and unique right-hand sides
    std::vector<double> exc((size_t)m->n * m->L, 0.0);
    if (m->cem) {
        // the port current enters the electrode's voltage unknown
        for (int l = 0; l < m->L; ++l) exc[(size_t)(N + l) + (size_t)l * m->n] = 1.0;
    } else {
        excitation_matrix(m->n, nodesP.data(), edgesP.data(), m->L, d->port_edges, d->port_edges_cap, exc.data(),
                          m->n);
    }
    m->fixed = d->source_type == MPF_SOURCE_FIXED ? 1 : 0;
    // voltage sources: binarised excitation (src/models/eit_kernel.cu:40-41)
    if (m->fixed)
        for (auto& v : exc) v = std::fabs(v) >= 1e-9 ? 1.0 : 0.0;
    const int L = m->L, Md = m->Md, Mm = m->Mm;
    std::vector<std::vector<double>> canon;  // canonical pattern columns
    auto unique_of = [&](const std::vector<double>& col, int& u, float& scale) {
        double c = lead(col.data(), L);
        if (c == 0.0) {
            u = -1;
            scale = 0.f;
            return;
        }
        std::vector<double> nc(L);
        for (int i = 0; i < L; ++i) nc[i] = col[i] / c;
        for (size_t k = 0; k < canon.size(); ++k)
            if (canon[k] == nc) {
                u = (int)k;
                scale = (float)c;
                return;
            }
        canon.push_back(nc);
        u = (int)canon.size() - 1;
        scale = (float)c;
    };
    std::vector<int32_t> dU(Md), mU(Mm);
    std::vector<float> dS(Md), mS(Mm);
    for (int j = 0; j < Md; ++j) {
        std::vector<double> col(L);
        for (int i = 0; i < L; ++i) col[i] = d->source_values[j] * d->drive_pattern[i + (size_t)j * L];
        unique_of(col, dU[j], dS[j]);
    }
    for (int j = 0; j < Mm; ++j) {
        std::vector<double> col(L);
        for (int i = 0; i < L; ++i) col[i] = d->meas_pattern[i + (size_t)j * L];
        unique_of(col, mU[j], mS[j]);
    }
    if (canon.empty()) canon.push_back(std::vector<double>(L, 0.0));
    for (auto& u : dU) u = u < 0 ? 0 : u;
    for (auto& u : mU) u = u < 0 ? 0 : u;
    m->jacIdentity = 1;
    for (int j = 0; j < Md; ++j) m->jacIdentity &= dU[j] == j;
    for (int j = 0; j < Mm; ++j) m->jacIdentity &= mU[j] == j;
    // one scale for every (drive, measurement) row (adjacent patterns)
    m->jacUniformScale = dS[0] * mS[0];
    for (int d = 0; d < Md; ++d)
        for (int j = 0; j < Mm; ++j)
            if (dS[d] * mS[j] != m->jacUniformScale) m->jacUniformScale = 0.f;
    if (!(m->jacUniformScale > 0.f)) m->jacUniformScale = 0.f;
    m->K = (int)canon.size();
    m->KP = m->K <= 16 ? 16 : m->K <= 32 ? 32 : m->K <= 64 ? 64 : m->K <= 128 ? 128 : 0;
    MPF_CHECK(m->KP > 0, MPF_ENOTSUP, "mpf_eit_create: %d distinct excitation patterns (max 128)", m->K);
    const int KP = m->KP, P = m->npad;
    std::vector<double> B0((size_t)P * KP, 0.0);
    for (int u = 0; u < m->K; ++u)
        for (int nd = 0; nd < m->n; ++nd) {
            double s = 0.0;
            for (int i = 0; i < L; ++i) s += exc[nd + (size_t)i * m->n] * canon[u][i];
            B0[(size_t)nd * KP + u] = s;
        }
    // measurement plan: nonzeros of B0 by column
    std::vector<int32_t> nzPtr(KP + 1, 0), nzNode;
    std::vector<double> nzVal;
    for (int u = 0; u < KP; ++u) {
        for (int nd = 0; nd < m->n; ++nd) {
            double v = B0[(size_t)nd * KP + u];
            if (v != 0.0) {
                nzNode.push_back(nd);
                nzVal.push_back(v);
            }
        }
        nzPtr[u + 1] = (int32_t)nzNode.size();
    }
    if (nzNode.empty()) {
        nzNode.push_back(0);
        nzVal.push_back(0.0);
    }

    // ---- 2.5D components (src/models/eit.cpp:154-157)
    m->compOf.assign(m->C, -1);
    m->betaAll.assign(m->C, 0.0);
    std::vector<int32_t> dcf;
    double beta0 = 1.0 / m->height;
    for (int c = 0; c < m->C; ++c) {
        double alpha = std::pow(2.0 * c * M_PI / m->height, 2);
        double beta = c == 0 ? 1.0 / m->height
                             : 2.0 * std::sin(c * M_PI * m->portHeight / m->height) / (c * M_PI * m->portHeight);
        if (m->fixed) {
            // voltage sources: no beta weighting, the measured currents carry
            // the height (src/models/eit.cpp:170-197); the Dirichlet rows make
            // every harmonic nonsingular
            m->betaAll[c] = 1.0;
            m->compOf[c] = (int)m->alphaH.size();
            m->alphaH.push_back((float)alpha);
            m->betaH.push_back((float)m->height);
            dcf.push_back(0);
            continue;
        }
        m->betaAll[c] = beta;
        // a harmonic whose excitation vanishes to rounding contributes nothing
        if (std::fabs(beta) <= 1e-12 * std::fabs(beta0)) continue;
        m->compOf[c] = (int)m->alphaH.size();
        m->alphaH.push_back((float)alpha);
        m->betaH.push_back((float)beta);
        dcf.push_back(c == 0 ? 1 : 0);
    }
    m->Ca = (int)m->alphaH.size();
    m->anyDcFree = dcf.size() && dcf[0] ? 1 : 0;
    // right-hand sides per active harmonic (all equal to the unique excitations)
    std::vector<double> Bc((size_t)m->Ca * P * KP, 0.0);
    for (int ci = 0; ci < m->Ca; ++ci)
        std::memcpy(Bc.data() + (size_t)ci * P * KP, B0.data(), sizeof(double) * (size_t)P * KP);
    std::vector<float> Bcf(Bc.begin(), Bc.end());
    // rank-one scale c' = mean diagonal of S(ref) / n and the constant that
    // turns the (A + c' 1 1^T) solution into the reference's (A + 1 1^T) one
    {
        double diagSum = 0.0;
        for (int e = 0; e < m->E; ++e)
            for (int i = 0; i < 3; ++i) diagSum += K[(size_t)e * 9 + i * 3 + i] * d->reference_value;
        const double n = (double)m->n;
        const double c = diagSum / n / n;
        m->dcScale = (float)c;
        std::vector<double> shift(KP, 0.0);
        for (int u = 0; u < KP; ++u) {
            double s = 0.0;
            for (int nd = 0; nd < m->n; ++nd) s += B0[(size_t)nd * KP + u];
            shift[u] = s / (n * n) * (1.0 - 1.0 / c);
        }
        MPF_TRY(m->dcShift.upload(shift));
    }

    // ---- Jacobian row tables and field export tables
    std::vector<int32_t> rowD(m->rowsJ, -1), rowM(m->rowsJ, -1);
    std::vector<float> rowS(m->rowsJ, 0.f);
    for (int dd = 0; dd < m->MdPad; ++dd)
        for (int mm = 0; mm < m->MmPad; ++mm) {
            int row = dd * m->MmPad + mm;
            if (dd < Md && mm < Mm) {
                rowD[row] = dU[dd];
                rowM[row] = mU[mm];
                rowS[row] = dS[dd] * mS[mm];
            } else {
                rowD[row] = dd < Md ? dU[dd] : -1;
                rowM[row] = mm < Mm ? mU[mm] : -1;
                rowS[row] = 0.f;
            }
        }
    std::vector<int32_t> colU(Md + Mm);
    std::vector<float> colS(Md + Mm);
    for (int j = 0; j < Md; ++j) { colU[j] = dU[j]; colS[j] = dS[j]; }
    for (int j = 0; j < Mm; ++j) { colU[Md + j] = mU[j]; colS[Md + j] = mS[j]; }
    std::vector<float> beta2(m->Ca), betaC(m->C);
    std::vector<float> massCoef(m->Ca, 0.f);
    m->exactJacobian = d->jacobian_mode == 1 ? 1 : 0;
    for (int ci = 0; ci < m->Ca; ++ci) {
        // reference: -h sum_c beta_c^2 (Y K Y); exact: -sum_c beta_c (Y (K + alpha_c M) Y);
        // voltage sources: +h sum_c (Y K Y) (the sign is applied in eit_jacobian)
        beta2[ci] = m->fixed ? 1.f
                    : m->exactJacobian ? (float)(m->betaH[ci] / m->height) : m->betaH[ci] * m->betaH[ci];
        massCoef[ci] = m->exactJacobian ? m->alphaH[ci] : 0.f;
    }
    for (int c = 0; c < m->C; ++c) betaC[c] = m->compOf[c] >= 0 ? (float)m->betaAll[c] : 0.f;

    // ---- upload
    MPF_TRY(m->cols.upload(m->fs.cols));
    MPF_TRY(m->diagSlot.upload(m->fs.diagSlot));
    {
        HaloPlan hp;
        halo_plan(m->fs.cols, m->W, m->npad, hp);
        m->Hpad = hp.Hpad;
        MPF_TRY(m->haloRows.upload(hp.halo));
        MPF_TRY(m->haloCnt.upload(hp.hcnt));
        MPF_TRY(m->haloLcol.upload(hp.lcol));
    }
    MPF_TRY(m->cptr.upload(m->fs.contribPtr));
    MPF_TRY(m->contrib.upload(m->fs.contrib));
    MPF_TRY(m->elements.upload(elems));
    MPF_TRY(m->rowOf.upload(rowOf));
    MPF_TRY(m->Kf.upload(Kf));
    MPF_TRY(m->Mf.upload(Mf));
    MPF_TRY(m->Kd.upload(K));
    MPF_TRY(m->Md64.upload(M));
    MPF_TRY(m->Bc.upload(Bcf));
    MPF_TRY(m->Bc64.upload(Bc));
    MPF_TRY(m->alpha.upload(m->alphaH));
    MPF_TRY(m->beta.upload(m->betaH));
    MPF_TRY(m->beta2.upload(beta2));
    MPF_TRY(m->massCoef.upload(massCoef));
    MPF_TRY(m->betaC.upload(betaC));
    MPF_TRY(m->dcFree.upload(dcf));
    MPF_TRY(m->compOfD.upload(m->compOf));
    MPF_TRY(m->nzPtr.upload(nzPtr));
    MPF_TRY(m->nzNode.upload(nzNode));
    MPF_TRY(m->nzVal.upload(nzVal));
    MPF_TRY(m->driveU.upload(dU));
    MPF_TRY(m->measU.upload(mU));
    MPF_TRY(m->driveScale.upload(dS));
    MPF_TRY(m->measScale.upload(mS));
    MPF_TRY(m->rowD.upload(rowD));
    MPF_TRY(m->rowM.upload(rowM));
    MPF_TRY(m->rowScale.upload(rowS));
    MPF_TRY(m->colU.upload(colU));
    MPF_TRY(m->colScale.upload(colS));
    if (m->fixed) MPF_TRY(fixed_plan(m.get(), exc));

    // ---- two-level preconditioner plan: aggregates of kAgg consecutive rows
    // and, per nonzero aggregate pair (I, J), the matrix slots that sum into
    // the coarse entry (padding slots excluded)
    m->nc = (m->n + kAgg - 1) / kAgg;
    m->ncPad = round_up(m->nc, 64);
    m->coarseOK = coarse_supported(m->KP, m->ncPad) ? 1 : 0;
    if (m->coarseOK) {
        std::vector<std::vector<std::pair<int32_t, int32_t>>> byI(m->nc);
        for (int r = 0; r < m->n; ++r)
            for (int k = 0; k < m->W; ++k) {
                const int32_t c = m->fs.cols[(size_t)k * P + r];
                if (c == r && k != m->fs.diagSlot[r]) continue;
                byI[r / kAgg].push_back({c / kAgg, (int32_t)((size_t)k * P + r)});
            }
        std::vector<int32_t> pI, pJ, pPtr{0}, slots;
        for (int I = 0; I < m->nc; ++I) {
            auto& v = byI[I];
            std::sort(v.begin(), v.end());
            for (size_t t = 0; t < v.size(); ++t) {
                if (t == 0 || v[t].first != v[t - 1].first) {
                    if (t > 0) pPtr.push_back((int32_t)slots.size());
                    pI.push_back(I);
                    pJ.push_back(v[t].first);
                }
                slots.push_back(v[t].second);
            }
            if (!v.empty()) pPtr.push_back((int32_t)slots.size());
        }
        std::vector<float> aggSize(m->nc);
        for (int I = 0; I < m->nc; ++I) aggSize[I] = (float)std::min(kAgg, m->n - I * kAgg);
        m->cNnz = (int)pI.size();
        MPF_TRY(m->cPairI.upload(pI));
        MPF_TRY(m->cPairJ.upload(pJ));
        MPF_TRY(m->cPairPtr.upload(pPtr));
        MPF_TRY(m->cSlots.upload(slots));
        MPF_TRY(m->cAggSize.upload(aggSize));
    }
    MPF_CUDA(cudaMallocHost(&m->pinnedActive, sizeof(int) * (4096 + 1)));
    *out = m.release();
    return MPF_OK;
}

static int ensure_workspace(mpf_eit* m, int F, bool refine, bool jacobian) {
    const size_t G = (size_t)F * m->Ca;
    const size_t vec = G * m->npad * m->KP;
    if (F > m->capF) {
        const size_t slots = (size_t)F * m->W * m->npad;
        MPF_TRY(m->SR.alloc(slots));
        // fields survive growth only if the old contents are copied; simpler to invalidate
        m->X.release();
        MPF_TRY(m->X.alloc(vec));
        MPF_CUDA(cudaMemset(m->X.ptr, 0, vec * sizeof(float)));
        MPF_TRY(m->Rv.alloc(vec));
        MPF_TRY(m->Pv.alloc(vec));
        MPF_TRY(m->Qv.alloc(vec));
        const size_t parts = G * m->nblk * m->KP, sc = G * m->KP;
        MPF_TRY(m->partA.alloc(parts));
        MPF_TRY(m->partB.alloc(parts));
        MPF_TRY(m->partC.alloc(parts));
        MPF_TRY(m->rz.alloc(sc));
        MPF_TRY(m->pq.alloc(sc));
        MPF_TRY(m->bz.alloc(sc));
        MPF_TRY(m->betaW.alloc(sc));
        MPF_TRY(m->rr.alloc(sc));
        MPF_TRY(m->bb.alloc(sc));
        MPF_TRY(m->sumP.alloc(sc));
        MPF_TRY(m->sumX.alloc(sc));
        MPF_TRY(m->conv.alloc(sc));
        MPF_TRY(m->alphaX.alloc(sc));
        MPF_TRY(m->pend.alloc(G));
        MPF_CUDA(cudaMemset(m->pend.ptr, 0, G * sizeof(int)));
        MPF_TRY(m->active.alloc(G));
        MPF_TRY(m->iters.alloc(G));
        MPF_TRY(m->counter.alloc(G));
        MPF_CUDA(cudaMemset(m->counter.ptr, 0, G * sizeof(unsigned)));
        MPF_TRY(m->Gm.alloc(G * m->KP * m->KP));
        MPF_TRY(m->V.alloc((size_t)F * m->Mm * m->Md));
        m->activeHost.resize(G);
        m->itersHost.resize(G);
        MPF_CHECK(G <= 4096, MPF_EINVAL, "too many (frame, harmonic) groups in one call: %zu (max 4096)", G);
        m->capF = F;
        m->fieldsValid = false;
        cg_graphs_clear(m->graphs);
    }
    if (refine && F > m->capF64) {
        const size_t slots = (size_t)F * m->W * m->npad;
        MPF_TRY(m->S64.alloc(slots));
        MPF_TRY(m->R64.alloc(slots));
        MPF_TRY(m->X64.alloc(vec));
        m->capF64 = F;
    }
    if (jacobian && F > m->capFJ) {
        const size_t jsz = (size_t)F * m->rowsJ * m->Epad;
        MPF_TRY(m->Jhi.alloc(jsz));
        MPF_TRY(m->Jlo.alloc(jsz));
        MPF_TRY(m->gramWork.alloc(dense_gram_work_floats(F, m->rowsJ, m->Epad)));
        MPF_TRY(m->A64.alloc((size_t)F * m->rowsJ * m->rowsJ));
        MPF_TRY(m->y.alloc((size_t)F * m->rowsJ));
        MPF_TRY(m->res.alloc((size_t)F));
        MPF_TRY(m->info.alloc((size_t)F));
        m->capFJ = F;
    }
    return MPF_OK;
}

// Workspace of the two-level preconditioner for F frames (coarse vectors
// start at zero: their padding aggregates are never written).
static int ensure_coarse(mpf_eit* m, int F) {
    if (F <= m->capFC) return MPF_OK;
    const size_t G = (size_t)F * m->Ca, nc2 = (size_t)m->ncPad * m->ncPad, cv = G * m->ncPad * m->KP;
    MPF_TRY(m->Ac64.alloc(G * nc2));
    MPF_TRY(m->Lc64.alloc(G * nc2));
    MPF_TRY(m->Lc.alloc(G * nc2));
    MPF_TRY(m->LinvD.alloc(G * (m->ncPad / 32) * 1024));
    MPF_TRY(m->Binv.alloc(G * nc2));
    MPF_TRY(m->rcV.alloc(cv));
    MPF_TRY(m->rcB.alloc(cv));
    MPF_TRY(m->ycV.alloc(cv));
    MPF_CUDA(cudaMemset(m->rcV.ptr, 0, cv * sizeof(float)));
    MPF_CUDA(cudaMemset(m->rcB.ptr, 0, cv * sizeof(float)));
    MPF_CUDA(cudaMemset(m->ycV.ptr, 0, cv * sizeof(float)));
    MPF_TRY(m->rzFine.alloc(G * m->KP));
    MPF_TRY(m->bzFine.alloc(G * m->KP));
    MPF_TRY(m->infoC.alloc(2 * G));
    m->capFC = F;
    return MPF_OK;
}

// BiCGSTAB's three extra vectors and two scalar arrays for F frames.
static int ensure_bicgstab(mpf_eit* m, int F) {
    if (F <= m->capFB) return MPF_OK;
    const size_t G = (size_t)F * m->Ca, vec = G * m->npad * m->KP;
    MPF_TRY(m->Rhat.alloc(vec));
    MPF_TRY(m->Zv.alloc(vec));
    MPF_TRY(m->Tv.alloc(vec));
    MPF_TRY(m->omegaW.alloc(G * m->KP));
    MPF_TRY(m->rr2W.alloc(G * m->KP));
    m->capFB = F;
    return MPF_OK;
}

// Complex-admittivity workspace for F frames.
static int ensure_complex(mpf_eit* m, int F) {
    if (F <= m->capFZ) return MPF_OK;
    const size_t G = (size_t)F * m->Ca, vec2 = 2 * G * m->npad * m->KP, sc = G * m->KP;
    MPF_TRY(m->SRz.alloc((size_t)F * m->W * m->npad));
    for (auto* b : {&m->Xz, &m->Rz, &m->Yz, &m->Nz, &m->Hz, &m->Zz, &m->Tz}) MPF_TRY(b->alloc(vec2));
    for (auto* b : {&m->zRhoI, &m->zAlphaI, &m->zBetaI, &m->zOmega, &m->zOmegaI, &m->zSumI, &m->zRr})
        MPF_TRY(b->alloc(sc));
    MPF_TRY(m->Gmz.alloc(2 * G * m->KP * m->KP));
    MPF_TRY(m->Vz.alloc(2 * (size_t)F * m->Mm * m->Md));
    m->capFZ = F;
    return MPF_OK;
}

static CgProblem make_problem(mpf_eit* m, int F, double tol, bool coarse = false, int solver = 0) {
    CgProblem P{};
    P.n = m->n;
    P.npad = m->npad;
    P.W = m->W;
    P.KP = m->KP;
    P.G = F * m->Ca;
    P.Ca = m->Ca;
    P.nblk = m->nblk;
    P.M = 1;
    P.seg = nullptr;
    P.cols = m->cols.ptr;
    P.diagSlot = m->diagSlot.ptr;
    P.halo = m->haloRows.ptr;
    P.hcnt = m->haloCnt.ptr;
    P.lcol = m->haloLcol.ptr;
    P.Hpad = m->Hpad;
    P.abortFlag = abort_flag_device();
    P.SR = m->SR.ptr;
    P.alpha = m->alpha.ptr;
    P.x = m->X.ptr;
    P.r = m->Rv.ptr;
    P.p = m->Pv.ptr;
    P.q = m->Qv.ptr;
    P.b = m->fixed ? m->bFix.ptr : m->Bc.ptr;  // voltage sources: per-group Dirichlet right-hand sides
    P.bPerGroup = m->fixed ? 1 : 0;
    P.dcFree = m->dcFree.ptr;
    P.partA = m->partA.ptr;
    P.partB = m->partB.ptr;
    P.partC = m->partC.ptr;
    P.sumP = m->sumP.ptr;
    P.sumX0 = nullptr;
    P.dcScale = m->dcScale;
    P.rz = m->rz.ptr;
    P.pq = m->pq.ptr;
    P.bz = m->bz.ptr;
    P.beta = m->betaW.ptr;
    P.conv = m->conv.ptr;
    P.active = m->active.ptr;
    P.iters = m->iters.ptr;
    P.counter = m->counter.ptr;
    P.alphaX = m->alphaX.ptr;
    P.pend = m->pend.ptr;
    P.tol2 = tol * tol;
    if (coarse) {
        P.coarse = 1;
        P.nc = m->nc;
        P.ncPad = m->ncPad;
        P.rc = m->rcV.ptr;
        P.rcB = m->rcB.ptr;
        P.yc = m->ycV.ptr;
        P.Binv = m->Binv.ptr;
        P.rzFine = m->rzFine.ptr;
        P.bzFine = m->bzFine.ptr;
    }
    if (solver == 1) {
        P.solver = 1;
        P.rhat = m->Rhat.ptr;
        P.zv = m->Zv.ptr;
        P.tv = m->Tv.ptr;
        P.omega = m->omegaW.ptr;
        P.rr2 = m->rr2W.ptr;
    }
    auto it = m->cgVariants.find(F);
    for (int k = 0; k < 3; ++k) {
        int code = it != m->cgVariants.end() ? it->second[k] : cg_default_variant(m->KP);
        if (m->forcedVariants[k] >= 0) code = m->forcedVariants[k];
        cg_set_shape(P, k, code);
    }
    return P;
}

// Autotuner (cg_driver.cpp) on the model's own assembled systems (F frames);
// it overwrites the iteration vectors, so it runs only before a cold solve.
static int tune_cg(mpf_eit* m, int F, cudaStream_t s) {
    if (m->cgVariants.count(F)) return MPF_OK;
    if (m->forcedVariants[0] >= 0 && m->forcedVariants[1] >= 0 && m->forcedVariants[2] >= 0) return MPF_OK;
    std::array<int, 3> best{};
    MPF_TRY(cg_autotune(make_problem(m, F, 0.0), best, s));
    m->cgVariants[F] = best;
    m->fieldsValid = false;
    return MPF_OK;
}

// Runs CG iterations until every group converged or max_iter; returns the
// iteration count of the slowest group and the number of unconverged groups.
static int run_cg(mpf_eit* m, const CgProblem& P, int maxIter, int checkEvery, cudaStream_t s, int* itersOut,
                  int* notConverged) {
    return cg_run(m->graphs, m->pinnedActive, &P, 1, maxIter, checkEvery, s, m->itersHost, itersOut, notConverged);
}

static void fill_defaults(const mpf_solve_opts* in, mpf_solve_opts& o, int n) {
    o.tol = 1e-6;
    o.max_iter = 0;
    o.refine_tol = 0.0;
    o.max_refine = 6;
    o.warm_start = 0;
    o.check_every = 16;
    o.preconditioner = 0;
    o.solver = 0;
    o.gn_factor = 0;
    o.accept_tol = 0.0;
    o.accept_margin = 0.1;
    if (in) o = *in;
    if (o.preconditioner != 1) o.preconditioner = 0;
    if (o.solver != 1) o.solver = 0;
    if (o.solver == 1) o.preconditioner = 0;  // BiCGSTAB: Jacobi only
    if (o.gn_factor != 1) o.gn_factor = 0;  // 0: FP64 factor, 1: FP32 factor + FP64 refinement
    if (o.tol <= 0.0) o.tol = 1e-6;
    if (o.max_iter <= 0) o.max_iter = 10 * n;
    if (o.max_refine <= 0) o.max_refine = 6;
    if (o.check_every <= 0) o.check_every = 16;
    if (!(o.accept_tol > o.tol)) o.accept_tol = 0.0;  // only a looser acceptance solve is a saving
    if (!(o.accept_margin > 0.0) || o.accept_margin >= 1.0) o.accept_margin = 0.1;
}

int eit_assemble(mpf_eit* m, int F, const float* gamma, bool fp64, cudaStream_t s) {
    return fem_launch_assemble(F, m->W, m->npad, m->E, m->cptr.ptr, m->contrib.ptr, m->Kf.ptr, m->Mf.ptr,
                               m->Kd.ptr, m->Md64.ptr, gamma, m->ref, m->logarithmic, m->SR.ptr,
                               fp64 ? m->S64.ptr : nullptr, fp64 ? m->R64.ptr : nullptr, s);
}

int eit_assemble_export(mpf_eit* m, int F, const float* gamma, float* sOut, float* rOut, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(!m->cem, MPF_ENOTSUP, "mpf_eit_assemble: the reference ELL layout has no electrode rows "
              "(complete electrode model)");
    
    MPF_CHECK(F >= 1 && gamma, MPF_EINVAL, "mpf_eit_assemble: bad arguments");
    MPF_TRY(ensure_workspace(m, F, false, false));
    MPF_TRY(eit_assemble(m, F, gamma, false, s));
    if (sOut)
        MPF_TRY(fem_launch_export_ell(F, m->W, m->npad, m->n, m->dataRows, m->SR.ptr, 0, m->rowOf.ptr, sOut, s));
    if (rOut)
        MPF_TRY(fem_launch_export_ell(F, m->W, m->npad, m->n, m->dataRows, m->SR.ptr, 1, m->rowOf.ptr, rOut, s));
    return MPF_OK;
}

// Jacobian of the last forward solve's fields into the workspace: the BF16
// hi/lo split always, FP32 J only when `f32` (the C-ABI forward output);
// frames with frameMask[f] == 0 are skipped.
static int eit_jacobian(mpf_eit* m, int F, const float* gamma, const int* frameMask, bool f32, cudaStream_t s) {
    MPF_TRY(ensure_workspace(m, F, false, true));
    if (f32) MPF_TRY(m->J.alloc((size_t)m->capFJ * m->rowsJ * m->Epad));
    JacPlan jp{m->rowsJ, m->Epad, m->E, m->KP, m->Ca, m->rowD.ptr, m->rowM.ptr, m->rowScale.ptr,
               m->beta2.ptr, m->massCoef.ptr, m->elements.ptr, m->Kf.ptr, m->Mf.ptr, m->exactJacobian,
               m->ref, m->fixed ? -(float)m->height : (float)m->height, m->logarithmic, frameMask, f32 ? 1 : 0,
               m->jacIdentity, m->jacUniformScale};
    return fem_launch_jacobian(F, jp, m->MmPad, m->npad, m->X.ptr, gamma, f32 ? m->J.ptr : nullptr, m->Jhi.ptr,
                               m->Jlo.ptr, s);
}

static int ensure_v0(mpf_eit* m, cudaStream_t s);

// Forward solve into the workspace (fields X, voltages V, optional J).
// skipFrames (device, [F], optional): frames whose fields are kept as they
// are (not iterated).  reuseSystems: the systems of gamma are already
// assembled (and the coarse space set up) by the previous call with the same
// frames, as in the continuation of a looser solve.
int eit_forward_ws(mpf_eit* m, int F, const float* gamma, bool wantJ, const mpf_solve_opts* optsIn,
                   mpf_solve_stats* stats, cudaStream_t s, const int* skipFrames = nullptr,
                   bool reuseSystems = false) {
    auto t0 = std::chrono::steady_clock::now();
    mpf_solve_opts o;
    fill_defaults(optsIn, o, m->n);
    const bool refine = o.refine_tol > 0.0;
    MPF_TRY(ensure_workspace(m, F, refine, wantJ));
    MPF_TRY(phase_mark(m, MPF_PHASE_CG, s));
    if (o.warm_start == 2) {
        // every frame starts from the homogeneous fields
        MPF_TRY(ensure_v0(m, s));
        MPF_TRY(ensure_workspace(m, F, refine, wantJ));
        const size_t per = (size_t)m->Ca * m->npad * m->KP;
        for (int f = 0; f < F; ++f)
            MPF_CUDA(cudaMemcpyAsync(m->X.ptr + f * per, m->X0.ptr, per * sizeof(float), cudaMemcpyDeviceToDevice, s));
        m->fieldsValid = true;
        m->lastFrames = F;
    }
    const bool warm = o.warm_start && m->fieldsValid && m->lastFrames == F;
    MPF_CHECK(!(m->fixed && refine), MPF_ENOTSUP,
              "forward solve: FP64 refinement is implemented for current (open) sources only");
    reuseSystems = reuseSystems && warm && !refine && !m->fixed;
    MPF_TRY(phase_mark(m, MPF_PHASE_ASSEMBLY, s));
    if (!reuseSystems) MPF_TRY(eit_assemble(m, F, gamma, refine, s));
    if (m->fixed) MPF_TRY(fixed_prepare(m, F, s));
    MPF_TRY(phase_mark(m, MPF_PHASE_CG_SETUP, s));
    const bool bicg = o.solver == 1;
    if (bicg) MPF_TRY(ensure_bicgstab(m, F));
    if (!warm && !bicg) MPF_TRY(tune_cg(m, F, s));
    const bool coarse = o.preconditioner == 1 && m->coarseOK;
    if (coarse) MPF_TRY(ensure_coarse(m, F));
    CgProblem P = make_problem(m, F, o.tol, coarse, o.solver);
    if (coarse && !reuseSystems) {
        CoarsePlan cp{m->nc, m->ncPad, m->cNnz, m->cPairI.ptr, m->cPairJ.ptr, m->cPairPtr.ptr, m->cSlots.ptr,
                      m->cAggSize.ptr};
        // frames left out of the solve keep the coarse space of their
        // previous (warm) solve
        const int* groupMask = nullptr;
        if (skipFrames && warm && !refine) {
            MPF_TRY(m->groupMask.alloc((size_t)P.G));
            MPF_TRY(cg_launch_group_mask(P, skipFrames, m->groupMask.ptr, s));
            groupMask = m->groupMask.ptr;
        }
        MPF_TRY(coarse_launch_setup(P, cp, m->Ac64.ptr, m->infoC.ptr, s, m->Lc.ptr, m->LinvD.ptr, m->Binv.ptr,
                                    m->Lc64.ptr, groupMask));
    }
    MPF_TRY(phase_mark(m, MPF_PHASE_CG, s));
    int totalIters = 0, notConv = 0, refinements = 0;
    double maxRel = 0.0;
    // fields are kept in the reference's convention; the iteration works on
    // the c'-scaled Neumann system (see cg_kernels.cu)
    if (warm && m->anyDcFree) MPF_TRY(cg_launch_dc_shift(P, m->dcShift.ptr, -1.f, s));
    if (!refine) {
        if (warm && m->anyDcFree) {
            MPF_TRY(cg_launch_colsum(P, m->X.ptr, nullptr, m->sumX.ptr, s));
            P.sumX0 = m->sumX.ptr;
        }
        MPF_TRY(cg_launch_init(P, !warm, s));
        if (skipFrames && warm) MPF_TRY(cg_launch_skip(P, skipFrames, s));
        MPF_TRY(run_cg(m, P, o.max_iter, o.check_every, s, &totalIters, &notConv));
    } else {
        const size_t vec = (size_t)P.G * m->npad * m->KP;
        if (warm) {
            // X64 = X (float fields of the previous call)
            MPF_CUDA(cudaMemsetAsync(m->X64.ptr, 0, vec * sizeof(double), s));
            MPF_TRY(cg_launch_accumulate64(P, m->X64.ptr, s));
        } else {
            MPF_CUDA(cudaMemsetAsync(m->X64.ptr, 0, vec * sizeof(double), s));
        }
        std::vector<double> rrH((size_t)P.G * m->KP), bbH((size_t)P.G * m->KP);
        CgProblem Pin = P;
        Pin.b = m->Rv.ptr;  // inner right-hand side: the float image of the FP64 residual
        Pin.bPerGroup = 1;
        double prevRel = 1e300;
        for (int outer = 0; outer <= o.max_refine; ++outer) {
            if (m->anyDcFree) MPF_TRY(cg_launch_colsum(P, nullptr, m->X64.ptr, m->sumX.ptr, s));
            MPF_TRY(cg_launch_residual64(P, m->S64.ptr, m->R64.ptr, m->X64.ptr, m->Bc64.ptr, m->sumX.ptr,
                                         m->partA.ptr, m->partB.ptr, m->rr.ptr, m->bb.ptr, s));
            MPF_CUDA(cudaMemcpyAsync(rrH.data(), m->rr.ptr, sizeof(double) * rrH.size(), cudaMemcpyDeviceToHost, s));
            MPF_CUDA(cudaMemcpyAsync(bbH.data(), m->bb.ptr, sizeof(double) * bbH.size(), cudaMemcpyDeviceToHost, s));
            MPF_CUDA(cudaStreamSynchronize(s));
            maxRel = 0.0;
            for (size_t i = 0; i < rrH.size(); ++i)
                if (bbH[i] > 0.0) maxRel = std::max(maxRel, std::sqrt(rrH[i] / bbH[i]));
            // stop when converged, out of steps, or no longer gaining (FP32 inner limit)
            if (maxRel <= o.refine_tol || outer == o.max_refine || maxRel > 0.5 * prevRel) break;
            prevRel = maxRel;
            int it = 0, nc = 0;
            MPF_TRY(cg_launch_init(Pin, true, s));
            MPF_TRY(run_cg(m, Pin, o.max_iter, o.check_every, s, &it, &nc));
            totalIters += it;
            notConv = std::max(notConv, nc);
            ++refinements;
            MPF_TRY(cg_launch_accumulate64(P, m->X64.ptr, s));
        }
        MPF_TRY(cg_launch_to_float(P, m->X64.ptr, s));
        if (maxRel > o.refine_tol) notConv = std::max(notConv, 1);
    }
    if (m->anyDcFree) MPF_TRY(cg_launch_dc_shift(P, m->dcShift.ptr, 1.f, s));
    if (coarse) {
        std::vector<int> info(P.G);
        MPF_CUDA(cudaMemcpyAsync(info.data(), m->infoC.ptr, sizeof(int) * P.G, cudaMemcpyDeviceToHost, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        for (int g = 0; g < P.G; ++g)
            MPF_CHECK(info[g] == 0, MPF_EBREAKDOWN, "two-level preconditioner: coarse Cholesky failed at pivot %d "
                      "(group %d)", info[g], g);
    }
    m->fieldsValid = true;
    m->lastFrames = F;
    MPF_TRY(phase_mark(m, MPF_PHASE_VOLTAGES, s));
    MeasPlan mp{(int)m->nzNode.count, m->nzNode.ptr, nullptr, m->nzVal.ptr, m->nzPtr.ptr};
    if (m->fixed) MPF_TRY(fixed_currents(m, F, s));
    MPF_TRY(fem_launch_gram_meas(P.G, m->KP, m->npad, mp, m->fixed ? m->curX.ptr : m->X.ptr, m->Gm.ptr, s));
    MPF_TRY(fem_launch_voltages(F, m->Ca, m->KP, m->Mm, m->Md, m->Gm.ptr, m->beta.ptr, m->measU.ptr,
                                m->measScale.ptr, m->driveU.ptr, m->driveScale.ptr, m->V.ptr, s));
    if (wantJ) {
        MPF_TRY(phase_mark(m, MPF_PHASE_JACOBIAN, s));
        MPF_TRY(eit_jacobian(m, F, gamma, nullptr, true, s));
    }
    MPF_TRY(phase_mark(m, MPF_PHASE_HOST, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    MPF_CUDA(cudaGetLastError());
    if (stats) {
        stats->iterations = totalIters;
        stats->refinements = refinements;
        stats->not_converged = notConv;
        stats->max_rel_residual = maxRel;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return notConv ? fail(MPF_ENOCONV, "forward solve: %d systems did not converge", notConv) : MPF_OK;
}

// Forward solve for complex material values (complex_kernels.cu): gamma
// [F][E] complex, V [F][Mm][Md] complex (column-major per frame), both with
// interleaved real and imaginary parts.
int eit_forward_complex(mpf_eit* m, int F, const float* gamma, float* Vout, float* Jref, const mpf_solve_opts* optsIn,
                        mpf_solve_stats* stats, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma && Vout, MPF_EINVAL, "mpf_eit_forward_complex: bad arguments");
    MPF_CHECK(!m->cem, MPF_ENOTSUP, "mpf_eit_forward_complex: the complete electrode model is implemented for "
              "real parameters only");
    MPF_CHECK(!m->fixed, MPF_ENOTSUP, "mpf_eit_forward_complex: voltage (fixed) sources are not implemented");
    MPF_CHECK(m->KP <= 64, MPF_ENOTSUP, "mpf_eit_forward_complex: at most 64 unique excitations");
    auto t0 = std::chrono::steady_clock::now();
    mpf_solve_opts o;
    fill_defaults(optsIn, o, m->n);
    MPF_CHECK(o.refine_tol <= 0.0 && o.warm_start == 0, MPF_ENOTSUP,
              "mpf_eit_forward_complex: cold FP32 solves only (no refinement, no warm start)");
    MPF_TRY(ensure_workspace(m, F, false, false));
    MPF_TRY(ensure_complex(m, F));
    MPF_TRY(fem_launch_zassemble(F, m->W, m->npad, m->E, m->cptr.ptr, m->contrib.ptr, m->Kf.ptr, m->Mf.ptr, gamma,
                                 m->ref, m->logarithmic, m->SRz.ptr, s));
    CgProblem P = make_problem(m, F, o.tol);
    P.solver = 2;
    P.SR = nullptr;
    P.SRz = m->SRz.ptr;
    P.x = m->Xz.ptr;
    P.r = m->Rz.ptr;
    P.p = m->Yz.ptr;
    P.q = m->Nz.ptr;
    P.rhat = m->Hz.ptr;
    P.zv = m->Zz.ptr;
    P.tv = m->Tz.ptr;
    P.omega = m->zOmega.ptr;
    P.rr2 = m->zRr.ptr;
    P.rzI = m->zRhoI.ptr;
    P.pqI = m->zAlphaI.ptr;
    P.betaI = m->zBetaI.ptr;
    P.omegaI = m->zOmegaI.ptr;
    P.sumPI = m->zSumI.ptr;
    int iters = 0, notConv = 0;
    MPF_TRY(cg_launch_init(P, true, s));
    MPF_TRY(run_cg(m, P, o.max_iter, o.check_every, s, &iters, &notConv));
    if (m->anyDcFree) MPF_TRY(cg_launch_zdc_shift(P, m->dcShift.ptr, 1.f, s));
    m->zFieldsValid = true;
    m->zLastFrames = F;
    MPF_TRY(fem_launch_zgram_meas(P.G, m->KP, m->npad, m->nzPtr.ptr, m->nzNode.ptr, m->nzVal.ptr, m->Xz.ptr,
                                  m->Gmz.ptr, s));
    MPF_TRY(fem_launch_zvoltages(F, m->Ca, m->KP, m->Mm, m->Md, m->Gmz.ptr, m->beta.ptr, m->measU.ptr,
                                 m->measScale.ptr, m->driveU.ptr, m->driveScale.ptr, Vout, s));
    if (Jref) {
        MPF_TRY(m->Jz.alloc(2 * (size_t)F * m->rowsJ * m->Epad));
        JacPlan jp{m->rowsJ, m->Epad, m->E, m->KP, m->Ca, m->rowD.ptr, m->rowM.ptr, m->rowScale.ptr,
                   m->beta2.ptr, m->massCoef.ptr, m->elements.ptr, m->Kf.ptr, m->Mf.ptr, m->exactJacobian,
                   m->ref, (float)m->height, m->logarithmic, nullptr, 1};
        MPF_TRY(fem_launch_zjacobian(F, jp, m->MmPad, m->npad, m->Xz.ptr, gamma, m->Jz.ptr, s));
        MPF_TRY(fem_launch_ztranspose_jacobian(F, m->rowsJ, m->Epad, m->E, m->Jz.ptr, Jref, s));
    }
    MPF_CUDA(cudaStreamSynchronize(s));
    MPF_CUDA(cudaGetLastError());
    if (stats) {
        stats->iterations = iters;
        stats->refinements = 0;
        stats->not_converged = notConv;
        stats->max_rel_residual = 0.0;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return notConv ? fail(MPF_ENOCONV, "complex forward solve: %d systems did not converge", notConv) : MPF_OK;
}

int eit_forward(mpf_eit* m, int F, const float* gamma, float* V, float* Jref, const mpf_solve_opts* o,
                mpf_solve_stats* stats, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma, MPF_EINVAL, "mpFlow::models::EIT::solve: materialDistribution == nullptr");
    int st = eit_forward_ws(m, F, gamma, Jref != nullptr, o, stats, s);
    if (st != MPF_OK && st != MPF_ENOCONV) return st;
    if (V) MPF_CUDA(cudaMemcpyAsync(V, m->V.ptr, sizeof(float) * (size_t)F * m->Mm * m->Md, cudaMemcpyDeviceToDevice, s));
    if (Jref) MPF_TRY(fem_launch_transpose_jacobian(F, m->rowsJ, m->Epad, m->E, m->J.ptr, Jref, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    MPF_TRY(phase_flush(m, s));
    return st;
}

int eit_fields(mpf_eit* m, int F, float* out, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(m->fieldsValid && F >= 1 && F <= m->lastFrames && out, MPF_EINVAL,
              "mpf_eit_fields: no forward solve with that many frames");
    MPF_TRY(fem_launch_fields_export(F, m->Ca, m->C, m->compOfD.ptr, m->npad, m->KP, m->dataRows, m->Md + m->Mm,
                                     m->nNodes, m->colU.ptr, m->colScale.ptr, m->betaC.ptr, m->X.ptr, m->rowOf.ptr, out,
                                     s));
    return MPF_OK;
}

int eit_fields_complex(mpf_eit* m, int F, float* out, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(m->zFieldsValid && F >= 1 && F <= m->zLastFrames && out, MPF_EINVAL,
              "mpf_eit_fields_complex: no complex forward solve with that many frames");
    MPF_TRY(fem_launch_zfields_export(F, m->Ca, m->C, m->compOfD.ptr, m->npad, m->KP, m->dataRows, m->Md + m->Mm,
                                      m->nNodes, m->colU.ptr, m->colScale.ptr, m->betaC.ptr, m->Xz.ptr,
                                      m->rowOf.ptr, out, s));
    return MPF_OK;
}

// FP32 factor of A64 and FP64 iterative refinement of w = A64^-1 y for the
// frames in `act` (host, 1 = solve): on return y holds the solution of every
// frame that converged; fb[f] = 1 marks the frames that need the FP64 factor
// instead (FP32 breakdown, stalled or unconverged refinement).  A64's lower
// triangle is left intact (its upper triangle becomes the mirror image).
static int gn_solve_fp32(mpf_eit* m, int F, const std::vector<int>& act, std::vector<int>& fb, cudaStream_t s) {
    const int n = m->rowsJ, nbk = n / 32;  // residual partial sums per 32 rows
    MPF_TRY(m->cholL.alloc((size_t)F * n * n));
    MPF_TRY(m->cholX.alloc((size_t)F * n));
    MPF_TRY(m->cholR.alloc((size_t)F * n));
    MPF_TRY(m->cholY.alloc((size_t)F * n));
    MPF_TRY(m->cholRR.alloc((size_t)F * nbk));
    MPF_TRY(m->cholYY.alloc((size_t)F * nbk));
    MPF_TRY(m->cholW.alloc((size_t)F * n));
    MPF_TRY(m->cholD.alloc((size_t)F * n * 32));
    MPF_TRY(m->cholL32.alloc((size_t)F * n * n));
    MPF_TRY(m->cholInv.alloc((size_t)F * n * n));
    MPF_TRY(m->cholInvT.alloc((size_t)F * n * n));
    MPF_TRY(m->info32.alloc((size_t)F));
    MPF_TRY(m->cholMask.alloc((size_t)F));
    MPF_CUDA(cudaMemcpyAsync(m->cholMask.ptr, act.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
    // the residual below reads all of A64: make it the symmetric matrix whose
    // lower triangle the factors use
    MPF_TRY(dense_mirror_lower(F, n, m->A64.ptr, s, m->cholMask.ptr));
    MPF_TRY(dense_potrf32(F, n, m->A64.ptr, m->cholL.ptr, m->info32.ptr, s, m->cholMask.ptr));
    MPF_CUDA(cudaMemcpyAsync(m->cholY.ptr, m->y.ptr, sizeof(double) * F * n, cudaMemcpyDeviceToDevice, s));
    MPF_CUDA(cudaMemcpyAsync(m->cholR.ptr, m->y.ptr, sizeof(double) * F * n, cudaMemcpyDeviceToDevice, s));
    MPF_CUDA(cudaMemsetAsync(m->cholX.ptr, 0, sizeof(double) * F * n, s));
    std::vector<int> info(F), live(act);
    MPF_CUDA(cudaMemcpyAsync(info.data(), m->info32.ptr, sizeof(int) * F, cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    fb.assign(F, 0);
    bool any = false;
    for (int f = 0; f < F; ++f) {
        if (live[f] && info[f] != 0) {
            fb[f] = 1;
            live[f] = 0;
        }
        any |= live[f] != 0;
    }
    if (!any) return MPF_OK;
    MPF_CUDA(cudaMemcpyAsync(m->cholMask.ptr, live.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
    // L^-1 and L^-T in FP32 once, so that every refinement step is two
    // row-parallel matrix-vector products instead of two triangular solves
    // (a chain of n / 32 dependent block steps each)
    MPF_TRY(dense_trtri32(F, n, m->cholL.ptr, m->cholL32.ptr, m->cholD.ptr, m->cholInv.ptr, m->cholInvT.ptr, s,
                          m->cholMask.ptr));
    // refinement: x += L^-T L^-1 r, r = y - A x, until |r| <= 1e-10 |y| (the
    // split-BF16 Gram itself is accurate to ~1e-5) or the residual stops
    // shrinking; the first check comes after two steps (each step gains
    // about cond(A) * 6e-8, 1e-2 at the bench's conditioning)
    constexpr int kMaxRefine = 8;
    constexpr double kTol = 1e-10, kFloor = 1e-10;
    std::vector<double> rr((size_t)F * nbk), yy((size_t)F * nbk), prev(F, 1e300);
    std::vector<int> done(F, 0);
    for (int it = 0; it < kMaxRefine; ++it) {
        MPF_TRY(dense_tri_rows(F, n, m->cholInv.ptr, m->cholR.ptr, m->cholW.ptr, false, s, m->cholMask.ptr));
        MPF_TRY(dense_tri_rows(F, n, m->cholInvT.ptr, m->cholW.ptr, m->cholR.ptr, true, s, m->cholMask.ptr));
        MPF_TRY(dense_add_masked(F, n, m->cholX.ptr, m->cholR.ptr, s, m->cholMask.ptr));
        MPF_TRY(dense_sym_residual(F, n, m->A64.ptr, m->cholX.ptr, m->cholY.ptr, m->cholR.ptr, m->cholRR.ptr,
                                   m->cholYY.ptr, s, m->cholMask.ptr));
        if (it == 0) continue;
        MPF_CUDA(cudaMemcpyAsync(rr.data(), m->cholRR.ptr, sizeof(double) * rr.size(), cudaMemcpyDeviceToHost, s));
        MPF_CUDA(cudaMemcpyAsync(yy.data(), m->cholYY.ptr, sizeof(double) * yy.size(), cudaMemcpyDeviceToHost, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        bool pending = false;
        for (int f = 0; f < F; ++f) {
            if (!live[f] || done[f]) continue;
            double r2 = 0.0, y2 = 0.0;
            for (int k = 0; k < nbk; ++k) {
                r2 += rr[(size_t)f * nbk + k];
                y2 += yy[(size_t)f * nbk + k];
            }
            const double rel = y2 > 0.0 ? std::sqrt(r2 / y2) : 0.0;
            if (!(rel <= kTol)) {
                if (!(rel < 0.5 * prev[f])) {
                    // no longer gaining: at the FP64 floor (done), or stalled or
                    // non-finite above it (the FP64 factor takes over)
                    if (!(rel <= kFloor)) fb[f] = 1;
                    done[f] = 1;
                } else {
                    pending = true;
                }
            } else {
                done[f] = 1;
            }
            prev[f] = rel;
        }
        if (!pending) break;
    }
    for (int f = 0; f < F; ++f) {
        if (live[f] && !done[f]) fb[f] = 1;  // refinement ran out of steps
        if (fb[f]) live[f] = 0;
    }
    // y = x for the frames solved here
    for (int f = 0; f < F; ++f)
        if (live[f])
            MPF_CUDA(cudaMemcpyAsync(m->y.ptr + (size_t)f * n, m->cholX.ptr + (size_t)f * n, sizeof(double) * n,
                                     cudaMemcpyDeviceToDevice, s));
    return MPF_OK;
}

// J J^T + mu I (split-BF16 tensor cores) -> factor -> w -> gamma += J^T w
// for the frames in frameActive (all if null; hostActive: the same on the
// host, or null); y holds the residual on entry.  gnFactor 0: the FP64
// factor for every frame; 1: FP32 factor with FP64 refinement, the FP64
// factor for the frames where that fails.  With `broken`, a frame whose
// factorisation fails also with the FP64 Gram is left unchanged and flagged
// there; without it the failure is left in m->info for gn_check.  counts
// (optional): frames solved {FP32 + refinement, FP64}.  Every device mask
// has its own buffer and is copied in stream order.
static int gn_update(mpf_eit* m, int F, float* gamma, double lambda, const int* frameActive, cudaStream_t s,
                     const int* hostActive = nullptr, std::vector<int>* broken = nullptr, int gnFactor = 0,
                     int* counts = nullptr) {
    const double mu = (double)m->ref * lambda * (double)m->ref * lambda;
    MPF_TRY(phase_mark(m, MPF_PHASE_GRAM, s));
    MPF_TRY(dense_gram_f64_shift(F, m->rowsJ, m->Epad, m->Jhi.ptr, m->Jlo.ptr, m->Epad, mu, m->A64.ptr,
                                 m->gramWork.ptr, m->gramWork.count, s, frameActive));
    MPF_TRY(phase_mark(m, MPF_PHASE_CHOLESKY, s));
    std::vector<int> act(F);
    for (int f = 0; f < F; ++f) act[f] = hostActive ? (hostActive[f] != 0) : 1;
    // frames for the FP64 factor: all (gnFactor 0, or n outside the FP32
    // kernel's range) or the FP32 path's fallbacks
    std::vector<int> fb = act;
    const bool fp32 = gnFactor == 1 && m->rowsJ % 128 == 0 && m->rowsJ <= 1280;
    if (fp32) MPF_TRY(gn_solve_fp32(m, F, act, fb, s));
    int nfb = 0;
    for (int f = 0; f < F; ++f) nfb += fb[f];
    if (counts) {
        for (int f = 0; f < F; ++f) counts[0] += act[f] && !fb[f];
        counts[1] += nfb;
    }
    MPF_CUDA(cudaMemsetAsync(m->info.ptr, 0, sizeof(int) * F, s));
    if (nfb) {
        const int* fbMask = frameActive;
        if (fp32) {
            MPF_TRY(m->fbMask.alloc((size_t)F));
            MPF_CUDA(cudaMemcpyAsync(m->fbMask.ptr, fb.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
            fbMask = m->fbMask.ptr;
        }
        MPF_TRY(dense_cholesky_f64(F, m->rowsJ, m->A64.ptr, m->info.ptr, s, fbMask));
        // frames whose split-BF16 J J^T + mu I is not positive definite (mu below
        // the Gram's ~1e-5 relative error): FP32 J and the FP64 Gram, factor again
        std::vector<int> info(F), redo(F, 0);
        MPF_CUDA(cudaMemcpyAsync(info.data(), m->info.ptr, sizeof(int) * F, cudaMemcpyDeviceToHost, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        bool any = false;
        for (int f = 0; f < F; ++f) any |= (redo[f] = fb[f] && info[f] != 0) != 0;
        if (any) {
            MPF_TRY(m->redoMask.alloc((size_t)F));
            MPF_CUDA(cudaMemcpyAsync(m->redoMask.ptr, redo.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
            MPF_TRY(phase_mark(m, MPF_PHASE_JACOBIAN, s));
            MPF_TRY(eit_jacobian(m, F, gamma, m->redoMask.ptr, true, s));
            MPF_TRY(phase_mark(m, MPF_PHASE_GRAM, s));
            MPF_TRY(dense_gram_f64_exact(F, m->rowsJ, m->Epad, m->J.ptr, m->Epad, mu, m->A64.ptr, m->redoMask.ptr, s));
            MPF_TRY(phase_mark(m, MPF_PHASE_CHOLESKY, s));
            MPF_TRY(dense_cholesky_f64(F, m->rowsJ, m->A64.ptr, m->info.ptr, s, m->redoMask.ptr));
            if (broken) {
                MPF_CUDA(cudaMemcpyAsync(info.data(), m->info.ptr, sizeof(int) * F, cudaMemcpyDeviceToHost, s));
                MPF_CUDA(cudaStreamSynchronize(s));
                broken->assign(F, 0);
                for (int f = 0; f < F; ++f) (*broken)[f] = redo[f] && info[f] != 0;
            }
        }
        // triangular solves of the frames factored in FP64 (except broken ones)
        std::vector<int> solve64(F);
        for (int f = 0; f < F; ++f) solve64[f] = fb[f] && !(broken && !broken->empty() && (*broken)[f]);
        MPF_TRY(m->solveMask.alloc((size_t)F));
        MPF_CUDA(cudaMemcpyAsync(m->solveMask.ptr, solve64.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
        MPF_TRY(dense_cholesky_solve_f64(F, m->rowsJ, m->A64.ptr, m->y.ptr, 1, s, m->solveMask.ptr));
    }
    // the update, on the active frames that were not left broken
    const int* upMask = frameActive;
    if (broken && !broken->empty()) {
        std::vector<int> ok(F);
        for (int f = 0; f < F; ++f) ok[f] = act[f] && !(*broken)[f];
        MPF_TRY(m->upMask.alloc((size_t)F));
        MPF_CUDA(cudaMemcpyAsync(m->upMask.ptr, ok.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
        upMask = m->upMask.ptr;
    }
    MPF_TRY(phase_mark(m, MPF_PHASE_UPDATE, s));
    MPF_TRY(fem_launch_update_gamma(F, m->rowsJ, m->Epad, m->E, m->Jhi.ptr, m->Jlo.ptr, m->y.ptr, upMask, gamma, s));
    return MPF_OK;
}

static int gn_check(mpf_eit* m, int F, cudaStream_t s, const int* hostMask = nullptr) {
    std::vector<int> info(F);
    MPF_CUDA(cudaMemcpyAsync(info.data(), m->info.ptr, sizeof(int) * F, cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    bool aborted = false;
    MPF_TRY(dense_gram_check_abort(&aborted));
    MPF_CHECK(!aborted, MPF_ETIMEOUT, "gram kernel: a pipeline wait timed out");
    for (int f = 0; f < F; ++f)
        MPF_CHECK(info[f] == 0 || (hostMask && !hostMask[f]), MPF_EBREAKDOWN,
                  "Cholesky of (J J^T + mu I) failed at pivot %d (frame %d)", info[f], f);
    return MPF_OK;
}

int gn_step(mpf_eit* m, int F, float* gamma, const float* vMeas, double lambda, const mpf_solve_opts* o,
            double* residual, mpf_solve_stats* stats, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma && vMeas, MPF_EINVAL, "mpFlow::solver::Solver::solveAbsolute: bad arguments");
    int st = eit_forward_ws(m, F, gamma, false, o, stats, s);
    if (st != MPF_OK && st != MPF_ENOCONV) return st;
    MPF_TRY(ensure_workspace(m, F, false, true));
    MPF_TRY(phase_mark(m, MPF_PHASE_VOLTAGES, s));
    MPF_TRY(fem_launch_residual(F, m->rowsJ, m->Mm, m->Md, vMeas, m->V.ptr, m->y.ptr, m->res.ptr, s));
    MPF_TRY(phase_mark(m, MPF_PHASE_JACOBIAN, s));
    MPF_TRY(eit_jacobian(m, F, gamma, nullptr, false, s));
    mpf_solve_opts od;
    fill_defaults(o, od, m->n);
    MPF_TRY(gn_update(m, F, gamma, lambda, nullptr, s, nullptr, nullptr, od.gn_factor));
    MPF_TRY(phase_mark(m, MPF_PHASE_HOST, s));
    if (residual) MPF_CUDA(cudaMemcpyAsync(residual, m->res.ptr, sizeof(double) * F, cudaMemcpyDeviceToHost, s));
    MPF_TRY(gn_check(m, F, s));
    MPF_TRY(phase_flush(m, s));
    return st;
}

// Gauss-Newton iterations until every frame's relative data residual is at
// most `target` (frames that reach it are frozen) or maxIters updates.  With
// `fallback` (host, one threshold per frame), a frame whose residual at the
// start is not below its threshold restarts from gamma0 (accepted[f] = 0)
// before the first update.
static int gn_loop(mpf_eit* m, int F, float* gamma, const float* vMeas, double lambda, double target, int maxIters,
                   const mpf_solve_opts* oIn, const double* fallback, float gamma0, int32_t* accepted,
                   int32_t* itersOut, double* resOut, mpf_gn_stats* stats, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma && vMeas && maxIters >= 0, MPF_EINVAL, "mpf_gn_solve: bad arguments");
    auto t0 = std::chrono::steady_clock::now();
    mpf_solve_opts o;
    fill_defaults(oIn, o, m->n);
    MPF_TRY(m->frameMask.alloc((size_t)F));
    std::vector<int> mask(F, 1), iters(F, 0);
    std::vector<double> res(F, 0.0);
    int cgTotal = 0, gnIters = 0;
    int solves[2] = {0, 0};  // frame updates solved {FP32 factor + refinement, FP64 factor}
    int warm = o.warm_start, checkStart = fallback != nullptr;
    if (accepted)
        for (int f = 0; f < F; ++f) accepted[f] = 1;
    // the acceptance solve at the start's prediction may run at a looser
    // tolerance (o.accept_tol): frames that pass with the margin are decided
    // on it, the others continue from their fields to o.tol
    bool loosePass = checkStart && o.accept_tol > 0.0, reuse = false;
    if (stats) stats->accepted_loose = 0;
    // frames whose fields are final (decided, or finished) are not iterated again
    std::vector<int> skip(F, 0);
    MPF_TRY(m->skipMask.alloc((size_t)F));
    for (int it = 0;;) {
        mpf_solve_stats fs{};
        mpf_solve_opts oi = o;
        oi.warm_start = warm;
        if (loosePass) oi.tol = o.accept_tol;
        const bool anySkip = std::find(skip.begin(), skip.end(), 1) != skip.end();
        if (anySkip) MPF_CUDA(cudaMemcpyAsync(m->skipMask.ptr, skip.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
        int st = eit_forward_ws(m, F, gamma, false, &oi, &fs, s, anySkip ? m->skipMask.ptr : nullptr, reuse);
        if (st != MPF_OK && st != MPF_ENOCONV) return st;
        MPF_TRY(ensure_workspace(m, F, false, true));
        warm = 1;
        reuse = false;
        cgTotal += fs.iterations;
        MPF_TRY(phase_mark(m, MPF_PHASE_VOLTAGES, s));
        MPF_TRY(fem_launch_residual(F, m->rowsJ, m->Mm, m->Md, vMeas, m->V.ptr, m->y.ptr, m->res.ptr, s));
        MPF_CUDA(cudaMemcpyAsync(res.data(), m->res.ptr, sizeof(double) * F, cudaMemcpyDeviceToHost, s));
        MPF_TRY(phase_mark(m, MPF_PHASE_HOST, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        if (loosePass) {
            loosePass = false;
            int undecided = 0;
            for (int f = 0; f < F; ++f) {
                skip[f] = res[f] <= target * (1.0 - o.accept_margin);
                undecided += !skip[f];
            }
            if (stats) stats->accepted_loose = F - undecided;
            if (undecided) {
                reuse = true;  // same systems: continue from the fields to o.tol
                continue;
            }
        }
        if (checkStart) {
            checkStart = false;
            std::vector<int> reject(F, 0);
            int nrej = 0;
            for (int f = 0; f < F; ++f) {
                reject[f] = res[f] > target && !(res[f] < fallback[f]);
                if (accepted) accepted[f] = !reject[f];
                nrej += reject[f];
            }
            if (nrej) {
                MPF_TRY(phase_mark(m, MPF_PHASE_PRIOR, s));
                MPF_CUDA(cudaMemcpyAsync(m->frameMask.ptr, reject.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
                MPF_TRY(fem_launch_fill_frames(F, m->E, m->frameMask.ptr, gamma0, gamma, s));
                // a restarted frame begins from the homogeneous fields, which
                // already solve its system: the re-solve below converges at
                // once for every frame
                if (m->v0Ready) {
                    const size_t per = (size_t)m->Ca * m->npad * m->KP;
                    for (int f = 0; f < F; ++f)
                        if (reject[f])
                            MPF_CUDA(cudaMemcpyAsync(m->X.ptr + f * per, m->X0.ptr, per * sizeof(float),
                                                     cudaMemcpyDeviceToDevice, s));
                }
                continue;
            }
        }
        int live = 0;
        for (int f = 0; f < F; ++f) {
            if (mask[f] && res[f] <= target) mask[f] = 0;
            live += mask[f];
        }
        if (live == 0 || it == maxIters) break;
        for (int f = 0; f < F; ++f) skip[f] = !mask[f];
        for (int f = 0; f < F; ++f) iters[f] += mask[f];
        MPF_TRY(phase_mark(m, MPF_PHASE_JACOBIAN, s));
        MPF_CUDA(cudaMemcpyAsync(m->frameMask.ptr, mask.data(), sizeof(int) * F, cudaMemcpyHostToDevice, s));
        MPF_TRY(eit_jacobian(m, F, gamma, m->frameMask.ptr, false, s));
        // a frame whose J J^T + mu I cannot be factored (also with the FP64
        // Gram) keeps its gamma and leaves the iteration unconverged
        std::vector<int> broken;
        MPF_TRY(m->gammaPrev.alloc((size_t)F * m->E));
        MPF_TRY(m->badFrame.alloc((size_t)F));
        MPF_CUDA(cudaMemcpyAsync(m->gammaPrev.ptr, gamma, sizeof(float) * F * m->E, cudaMemcpyDeviceToDevice, s));
        MPF_TRY(gn_update(m, F, gamma, lambda, m->frameMask.ptr, s, mask.data(), &broken, o.gn_factor, solves));
        for (int f = 0; f < F && !broken.empty(); ++f)
            if (broken[f]) mask[f] = 0;
        // an update that sends a frame's parameters out of the forward
        // model's range (a diverging step) is undone and the frame frozen
        // unconverged, so that it cannot break the batch's next solve
        std::vector<int> bad(F);
        MPF_TRY(fem_launch_gamma_check(F, m->E, gamma, m->frameMask.ptr, m->logarithmic, m->badFrame.ptr, s));
        MPF_CUDA(cudaMemcpyAsync(bad.data(), m->badFrame.ptr, sizeof(int) * F, cudaMemcpyDeviceToHost, s));
        MPF_TRY(phase_mark(m, MPF_PHASE_HOST, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        for (int f = 0; f < F; ++f)
            if (bad[f]) {
                mask[f] = 0;
                MPF_CUDA(cudaMemcpyAsync(gamma + (size_t)f * m->E, m->gammaPrev.ptr + (size_t)f * m->E,
                                         sizeof(float) * m->E, cudaMemcpyDeviceToDevice, s));
            }
        MPF_TRY(gn_check(m, F, s, mask.data()));
        ++gnIters;
        ++it;
    }
    MPF_TRY(phase_flush(m, s));
    int converged = 0;
    for (int f = 0; f < F; ++f) converged += res[f] <= target;
    if (itersOut) std::copy(iters.begin(), iters.end(), itersOut);
    if (resOut) std::copy(res.begin(), res.end(), resOut);
    if (stats) {
        stats->gn_iterations = gnIters;
        stats->cg_iterations = cgTotal;
        stats->frames_converged = converged;
        stats->solves_fp32 = solves[0];
        stats->solves_fp64 = solves[1];
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return MPF_OK;
}

int gn_solve(mpf_eit* m, int F, float* gamma, const float* vMeas, double lambda, double target, int maxIters,
             const mpf_solve_opts* oIn, int32_t* itersOut, double* resOut, mpf_gn_stats* stats, cudaStream_t s) {
    return gn_loop(m, F, gamma, vMeas, lambda, target, maxIters, oIn, nullptr, 0.f, nullptr, itersOut, resOut, stats,
                   s);
}

// ---------------------------------------------------------------------------
// Learned warm start.  The network sees the measured voltages relative to
// those of the homogeneous distribution, scaled by their RMS, and predicts
// the parameter vector gamma directly.

static float homogeneous_gamma(const mpf_eit* m) { return m->logarithmic ? 0.f : 1.f; }

// V0 = voltages of the homogeneous distribution (solved once, FP64-refined).
static int ensure_v0(mpf_eit* m, cudaStream_t s) {
    if (m->v0Ready) return MPF_OK;
    const int L = m->Mm * m->Md;
    DevBuf<float> g0;
    MPF_TRY(g0.alloc((size_t)m->E));
    MPF_TRY(fem_launch_fill_frames(1, m->E, nullptr, homogeneous_gamma(m), g0.ptr, s));
    mpf_solve_opts o{};
    o.tol = 1e-6;
    o.refine_tol = 1e-9;
    MPF_TRY(eit_forward_ws(m, 1, g0.ptr, false, &o, nullptr, s));
    const size_t per = (size_t)m->Ca * m->npad * m->KP;
    MPF_TRY(m->X0.alloc(per));
    MPF_CUDA(cudaMemcpyAsync(m->X0.ptr, m->X.ptr, per * sizeof(float), cudaMemcpyDeviceToDevice, s));
    MPF_TRY(m->V0.alloc((size_t)L));
    MPF_CUDA(cudaMemcpyAsync(m->V0.ptr, m->V.ptr, sizeof(float) * L, cudaMemcpyDeviceToDevice, s));
    std::vector<float> h(L);
    MPF_CUDA(cudaMemcpyAsync(h.data(), m->V.ptr, sizeof(float) * L, cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    double ss = 0.0;
    for (float v : h) ss += (double)v * v;
    MPF_CHECK(ss > 0.0, MPF_EINVAL, "learned input: the homogeneous voltages are all zero");
    m->v0InvRms = (float)(1.0 / std::sqrt(ss / L));
    m->v0Ready = true;
    return MPF_OK;
}

int learned_input(mpf_eit* m, int F, const float* vMeas, float* x, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && vMeas && x, MPF_EINVAL, "mpf_eit_learned_input: bad arguments");
    MPF_TRY(ensure_v0(m, s));
    return fem_launch_learned_input(F, m->Mm * m->Md, vMeas, m->V0.ptr, m->v0InvRms, x, nullptr, s);
}

// Linear prior of the learned start: the first Gauss-Newton update from the
// homogeneous distribution gamma_h as a fixed linear map of the network input
// x = (v - V0) invRms,
//   prior(x) = gamma_h + J0^T (J0 J0^T + mu I)^-1 x / invRms,  mu = (ref lambda)^2,
// J0 the FP32 Jacobian at gamma_h, the Gram J0 J0^T in FP64 and its inverse
// from the FP64 Cholesky factor.  Stored as W = J0^T (J0 J0^T + mu I)^-1 /
// invRms restricted to the measurement rows (E x L, column-major).
int learned_prior(mpf_eit* m, double lambda, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(lambda >= 0.0 && std::isfinite(lambda), MPF_EINVAL, "mpf_eit_learned_prior: lambda must be >= 0");
    m->priorReady = false;
    if (lambda == 0.0) {
        m->priorW.release();
        m->priorB.release();
        m->priorA.release();
        return MPF_OK;
    }
    MPF_TRY(ensure_v0(m, s));
    const int L = m->Mm * m->Md, R = m->rowsJ;
    DevBuf<float> g0, Q;
    DevBuf<double> A0, B;
    DevBuf<int> info;
    MPF_TRY(g0.alloc((size_t)m->E));
    MPF_TRY(fem_launch_fill_frames(1, m->E, nullptr, homogeneous_gamma(m), g0.ptr, s));
    mpf_solve_opts o{};
    o.tol = 1e-6;
    o.refine_tol = 1e-9;
    MPF_TRY(eit_forward_ws(m, 1, g0.ptr, false, &o, nullptr, s));
    MPF_TRY(eit_jacobian(m, 1, g0.ptr, nullptr, true, s));
    const double mu = (double)m->ref * lambda * (double)m->ref * lambda;
    MPF_TRY(A0.alloc((size_t)R * R));
    MPF_TRY(info.alloc(1));
    MPF_TRY(dense_gram_f64_exact(1, R, m->Epad, m->J.ptr, m->Epad, mu, A0.ptr, nullptr, s));
    MPF_TRY(dense_cholesky_f64(1, R, A0.ptr, info.ptr, s));
    int hinfo = 0;
    MPF_CUDA(cudaMemcpyAsync(&hinfo, info.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    MPF_CHECK(hinfo == 0, MPF_EBREAKDOWN, "learned prior: Cholesky of J0 J0^T + mu I failed at pivot %d", hinfo);
    MPF_TRY(B.alloc((size_t)R * L));
    MPF_TRY(Q.alloc((size_t)R * L));
    MPF_TRY(fem_launch_prior_rhs(R, m->Mm, m->Md, B.ptr, s));
    MPF_TRY(dense_cholesky_solve_f64(1, R, A0.ptr, B.ptr, L, s));
    MPF_TRY(fem_launch_prior_convert(R, L, B.ptr, 1.0 / (double)m->v0InvRms, Q.ptr, s));
    MPF_TRY(m->priorW.alloc((size_t)m->Epad * L));
    MPF_TRY(matrix_multiply_scaled(0, 0, m->E, L, R, 1.f, m->J.ptr, m->Epad, Q.ptr, R, 0.f, m->priorW.ptr, m->Epad,
                                   s));
    // W (column-major E x L) as the B operand of the split-BF16 product
    m->priorN = round_up(m->E, 128);
    m->priorLp = round_up(L, 64);
    MPF_TRY(m->priorB.alloc((size_t)m->priorN * 3 * m->priorLp));
    MPF_TRY(split3_bf16(m->E, m->priorN, L, m->priorLp, m->priorW.ptr, 1, (size_t)m->Epad, 1, m->priorB.ptr, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    m->priorW.release();
    m->priorLambda = lambda;
    m->priorReady = true;
    return MPF_OK;
}

// out (frames x ldo) = prior(x) (mode 0), += prior(x) (mode 1) or -= prior(x) (mode -1)
int learned_prior_apply(mpf_eit* m, int F, const float* x, float* out, int ldo, int mode, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(m->priorReady, MPF_EINVAL, "mpf_eit_learned_prior_apply: no prior (call mpf_eit_learned_prior first)");
    MPF_CHECK(F >= 1 && x && out && ldo >= m->E && mode >= -1 && mode <= 1, MPF_EINVAL,
              "mpf_eit_learned_prior_apply: bad arguments");
    // out = alpha (W x + gamma_h) + beta out as one split-BF16 product on the
    // tensor cores (hi.hi + lo.hi + hi.lo, FP32 accumulation: about FP32
    // accuracy) with the update in its epilogue
    const int L = m->Mm * m->Md, Fp = round_up(F, 128), Lp = m->priorLp;
    const float alpha = mode < 0 ? -1.f : 1.f, beta = mode == 0 ? 0.f : 1.f;
    MPF_TRY(m->priorA.alloc((size_t)Fp * 3 * Lp));
    MPF_TRY(split3_bf16(F, Fp, L, Lp, x, (size_t)L, 1, 0, m->priorA.ptr, s));
    int* flag = abort_flag_device();
    MPF_CHECK(flag != nullptr, MPF_ENOMEM, "learned prior: abort flag allocation failed");
    MPF_TRY(tc_gemm_axpby(m->priorA.ptr, Fp, 3 * Lp, m->priorB.ptr, m->priorN, 3 * Lp, 3 * Lp, out, ldo, F, m->E,
                          alpha, beta, alpha * homogeneous_gamma(m), flag, s));
    int aborted = 0;
    MPF_CUDA(cudaMemcpyAsync(&aborted, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPF_CUDA(cudaStreamSynchronize(s));
    if (aborted) MPF_CUDA(cudaMemset(flag, 0, sizeof(int)));
    MPF_CHECK(!aborted, MPF_ETIMEOUT, "mpf_eit_learned_prior_apply: a tensor-core pipeline wait timed out");
    return MPF_OK;
}

int gn_solve_learned(mpf_eit* m, mpf_mlp* net, int F, float* gamma, const float* vMeas, double lambda,
                     double target, int maxIters, const mpf_solve_opts* o, int32_t* itersOut, double* resOut,
                     int32_t* accepted, mpf_gn_stats* stats, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma && vMeas && maxIters >= 0, MPF_EINVAL, "mpf_gn_solve_learned: bad arguments");
    const int L = m->Mm * m->Md;
    int in = 0, out = 0;
    mlp_dims(net, &in, &out);
    MPF_CHECK(in == L && out >= m->E, MPF_EINVAL,
              "mpf_gn_solve_learned: the network maps %d -> %d values, the model needs %d -> %d", in, out, L, m->E);
    auto t0 = std::chrono::steady_clock::now();
    MPF_TRY(ensure_v0(m, s));
    MPF_TRY(m->learnX.alloc((size_t)F * L));
    MPF_TRY(m->res0.alloc((size_t)F));
    MPF_TRY(phase_mark(m, MPF_PHASE_PRIOR, s));
    MPF_TRY(fem_launch_learned_input(F, L, vMeas, m->V0.ptr, m->v0InvRms, m->learnX.ptr, m->res0.ptr, s));
    std::vector<double> res0(F);
    MPF_CUDA(cudaMemcpyAsync(res0.data(), m->res0.ptr, sizeof(double) * F, cudaMemcpyDeviceToHost, s));
    MPF_TRY(phase_mark(m, MPF_PHASE_NETWORK, s));
    MPF_TRY(mlp_forward(net, F, m->learnX.ptr, gamma, m->E, s));  // synchronises
    MPF_TRY(phase_mark(m, MPF_PHASE_PRIOR, s));
    if (m->priorReady) MPF_TRY(learned_prior_apply(m, F, m->learnX.ptr, gamma, m->E, 1, s));
    // a prediction outside the forward model's range (non-finite, |gamma| >
    // 100 dB logarithmic, gamma <= 0 linear) is replaced by the homogeneous
    // start, which the acceptance check below then rejects
    MPF_TRY(m->badFrame.alloc((size_t)F));
    MPF_TRY(fem_launch_gamma_check(F, m->E, gamma, nullptr, m->logarithmic, m->badFrame.ptr, s));
    MPF_TRY(fem_launch_fill_frames(F, m->E, m->badFrame.ptr, homogeneous_gamma(m), gamma, s));
    MPF_TRY(gn_loop(m, F, gamma, vMeas, lambda, target, maxIters, o, res0.data(), homogeneous_gamma(m), accepted,
                    itersOut, resOut, stats, s));
    if (stats) stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return MPF_OK;
}

// Times the three CG kernels of one iteration with CUDA events on `s`
// (tolerance 0, so no group retires during the measurement).
int profile_cg(mpf_eit* m, int F, const float* gamma, int reps, double* ms, double* bytes, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma && reps >= 1 && ms && bytes, MPF_EINVAL, "mpf_eit_profile_cg: bad arguments");
    MPF_TRY(ensure_workspace(m, F, false, false));
    MPF_TRY(eit_assemble(m, F, gamma, false, s));
    MPF_TRY(tune_cg(m, F, s));
    m->fieldsValid = false;  // the iteration vectors are overwritten below
    CgProblem P = make_problem(m, F, 0.0);
    MPF_TRY(cg_launch_init(P, true, s));
    cudaEvent_t ev[4];
    for (auto& e : ev) MPF_CUDA(cudaEventCreate(&e));
    double acc[3] = {0, 0, 0};
    for (int r = 0; r < reps; ++r) {
        MPF_CUDA(cudaEventRecord(ev[0], s));
        MPF_TRY(cg_launch_kernel(P, 0, s));
        MPF_CUDA(cudaEventRecord(ev[1], s));
        MPF_TRY(cg_launch_kernel(P, 1, s));
        MPF_CUDA(cudaEventRecord(ev[2], s));
        MPF_TRY(cg_launch_kernel(P, 2, s));
        MPF_CUDA(cudaEventRecord(ev[3], s));
        MPF_CUDA(cudaEventSynchronize(ev[3]));
        for (int k = 0; k < 3; ++k) {
            float t = 0.f;
            MPF_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            acc[k] += t;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    const double G = (double)F * m->Ca, n = m->n, K = m->K;
    for (int k = 0; k < 3; ++k) ms[k] = acc[k] / reps;
    bytes[0] = G * ((double)m->nnz * 12.0 + 2.0 * K * n * 4.0);   // S, R, column + p gather + q
    bytes[1] = G * (3.0 * K * n * 4.0 + 2.0 * n * 4.0);            // r rw, q read; diagonal
    bytes[2] = G * (5.0 * K * n * 4.0 + 2.0 * n * 4.0);            // r, p, x read; p, x write; diagonal
    return MPF_OK;
}

// Launch and graph overhead of the CG loop.  ms[0]: per-iteration time of
// the loop exactly as a solve runs it (graphs of 16 iterations, the active
// flags and abort flag read back and the stream synchronised after each
// graph), CUDA events around the whole loop; ms[1]: per-iteration sum of the
// same kernels launched one at a time between CUDA events (the kernels'
// own time); ms[2]: host wall clock of the loop per iteration.  Tolerance 0,
// so no group retires and every iteration does the same work.
int profile_cg_loop(mpf_eit* m, int F, const float* gamma, int graphs, double* ms, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma && graphs >= 1 && graphs <= 4096 && ms, MPF_EINVAL,
              "mpf_eit_profile_cg_loop: bad arguments");
    constexpr int kEvery = 16;
    MPF_TRY(ensure_workspace(m, F, false, false));
    MPF_TRY(eit_assemble(m, F, gamma, false, s));
    MPF_TRY(tune_cg(m, F, s));
    m->fieldsValid = false;  // the iteration vectors are overwritten below
    CgProblem P = make_problem(m, F, 0.0);
    MPF_TRY(cg_launch_init(P, true, s));
    cudaEvent_t ev[2];
    for (auto& e : ev) MPF_CUDA(cudaEventCreate(&e));
    auto timed = [&](auto&& launch, double* acc) -> int {
        MPF_CUDA(cudaEventRecord(ev[0], s));
        MPF_TRY(launch());
        MPF_CUDA(cudaEventRecord(ev[1], s));
        MPF_CUDA(cudaEventSynchronize(ev[1]));
        float t = 0.f;
        MPF_CUDA(cudaEventElapsedTime(&t, ev[0], ev[1]));
        *acc += t;
        return MPF_OK;
    };
    double kernels = 0.0;
    int st = MPF_OK;
    for (int it = 0; it < kEvery && st == MPF_OK; ++it) {
        st = timed([&] { return cg_launch_kernel(P, 0, s); }, &kernels);
        if (st == MPF_OK) st = timed([&] { return cg_launch_kernel(P, 1, s); }, &kernels);
        if (st == MPF_OK && P.coarse) st = timed([&] { return cg_launch_coarse(P, false, s); }, &kernels);
        if (st == MPF_OK) st = timed([&] { return cg_launch_kernel(P, 2, s); }, &kernels);
    }
    double loop = 0.0, wall = 0.0;
    if (st == MPF_OK) st = cg_launch_init(P, true, s);
    if (st == MPF_OK) {
        // one untimed graph so that capture and instantiation stay outside
        int it = 0, nc = 0;
        st = run_cg(m, P, kEvery, kEvery, s, &it, &nc);
    }
    if (st == MPF_OK) {
        int it = 0, nc = 0;
        const auto t0 = std::chrono::steady_clock::now();
        MPF_CUDA(cudaEventRecord(ev[0], s));
        st = run_cg(m, P, graphs * kEvery, kEvery, s, &it, &nc);
        MPF_CUDA(cudaEventRecord(ev[1], s));
        MPF_CUDA(cudaEventSynchronize(ev[1]));
        wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        float t = 0.f;
        MPF_CUDA(cudaEventElapsedTime(&t, ev[0], ev[1]));
        loop = t;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    MPF_TRY(st);
    ms[0] = loop / ((double)graphs * kEvery);
    ms[1] = kernels / kEvery;
    ms[2] = wall / ((double)graphs * kEvery);
    return MPF_OK;
}

// Times the assembly and Jacobian kernels with CUDA events on `s`, on the
// fields of a forward solve of gamma.  Algorithmic bytes per launch:
//   assembly: E (12 connectivity + 36 K + 36 M) read once, and per frame
//             4 E (gamma) + 8 nnz (S, R slot values written);
//   Jacobian: per frame Ca K n 4 (fields of the active harmonics) + 52 E
//             (connectivity, elemental matrices, gamma) + 4 rowsJ E (the
//             split-BF16 J written).
int profile_fem(mpf_eit* m, int F, const float* gamma, int reps, double* ms, double* bytes, cudaStream_t s) {
    MPF_TRY(check_device(m));
    MPF_CHECK(F >= 1 && gamma && reps >= 1 && ms && bytes, MPF_EINVAL, "mpf_eit_profile_fem: bad arguments");
    mpf_solve_opts o{};
    o.tol = 1e-5;
    const int st = eit_forward_ws(m, F, gamma, false, &o, nullptr, s);
    if (st != MPF_OK && st != MPF_ENOCONV) return st;
    MPF_TRY(ensure_workspace(m, F, false, true));
    cudaEvent_t ev[3];
    for (auto& e : ev) MPF_CUDA(cudaEventCreate(&e));
    double acc[2] = {0.0, 0.0};
    for (int r = 0; r < reps; ++r) {
        MPF_CUDA(cudaEventRecord(ev[0], s));
        MPF_TRY(eit_assemble(m, F, gamma, false, s));
        MPF_CUDA(cudaEventRecord(ev[1], s));
        MPF_TRY(eit_jacobian(m, F, gamma, nullptr, false, s));
        MPF_CUDA(cudaEventRecord(ev[2], s));
        MPF_CUDA(cudaEventSynchronize(ev[2]));
        for (int k = 0; k < 2; ++k) {
            float t = 0.f;
            MPF_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            acc[k] += t;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    const double E = m->E, n = m->n, K = m->K, Ca = m->Ca, rows = m->rowsJ;
    ms[0] = acc[0] / reps;
    ms[1] = acc[1] / reps;
    bytes[0] = E * 84.0 + F * (E * 4.0 + 8.0 * (double)m->nnz);
    bytes[1] = F * (Ca * K * n * 4.0 + 52.0 * E + 4.0 * rows * E);
    return MPF_OK;
}

// Fixes the CG kernel variants (-1 = autotune); returns the variants a solve
// with F frames uses (the autotuned ones once a cold solve has run).
int cg_variants(mpf_eit* m, const int32_t* set, int F, int32_t* get) {
    if (set) {
        for (int k = 0; k < 3; ++k)
            MPF_CHECK(set[k] < 0 || cg_shape_fits(m->KP, m->W, m->Hpad, true, k, set[k]),
                      MPF_EINVAL, "CG launch shape %d is not available for kernel %d with %d right-hand sides",
                      set[k], k, m->KP);
        for (int k = 0; k < 3; ++k) m->forcedVariants[k] = set[k] < 0 ? -1 : set[k];
        cg_graphs_clear(m->graphs);
    }
    if (get) {
        CgProblem P = make_problem(m, F < 1 ? 1 : F, 0.0);
        for (int k = 0; k < 3; ++k) get[k] = cg_shape_code(P, k);
    }
    return MPF_OK;
}

int group_iterations(mpf_eit* m, int32_t* out, int cap, int32_t* count) {
    MPF_CHECK(out && count, MPF_EINVAL, "mpf_eit_group_iterations: null argument");
    const int n = (int)m->itersHost.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = m->itersHost[i];
    *count = n;
    return MPF_OK;
}

void eit_destroy(mpf_eit* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    delete m;
}

void eit_info(const mpf_eit* m, mpf_eit_info* i) {
    i->n_nodes = m->nNodes;
    i->n_elements = m->E;
    i->data_rows = m->dataRows;
    i->ports = m->L;
    i->drive_count = m->Md;
    i->meas_count = m->Mm;
    i->drive_cols_pad = m->MdPad;
    i->meas_cols_pad = m->MmPad;
    i->jacobian_rows = m->rowsJ;
    i->elements_pad = m->Epad;
    i->density = m->W;
    i->levels = m->levels;
    i->unique_columns = m->K;
    i->components = m->C;
    i->active_components = m->Ca;
}

}  // namespace mpf
