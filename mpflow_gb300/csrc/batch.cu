// Batches of uneven meshes: the forward solves of many EIT models (meshes of
// different size, 16 or 32 electrodes, one harmonic set) run as independent
// systems in the same CG launches.
//
// The reference solves one model at a time (EIT::solve,
// src/models/eit.cpp:139-213).  Here the meshes of a batch are grouped by
// right-hand-side width KP (the kernels are compiled per KP); within a width
// class their rows are stacked: mesh j owns 128-row tiles [tile0_j,
// tile0_j + tiles_j) of one column array, one slot-value array per frame and
// one vector slice per (frame, harmonic).  The stacked matrix is block
// diagonal (columns are global rows), so the kernels of cg_kernels.cu run
// unchanged over it; a segment table gives each (frame, harmonic, mesh) group
// its own rows, CG scalars, convergence mask and block reductions.  All width
// classes are recorded in one CUDA graph per check interval.
//
// The two-level preconditioner (preconditioner = 1) works per mesh as well:
// every group gets the coarse space of its own mesh (aggregates of 64
// Morton-ordered rows), padded to the largest coarse size of its width class
// with identity blocks, so the coarse setup and product run as one batch.
//
// The models stay usable on their own: the batch reads their static device
// arrays (assembly lists, right-hand sides, measurement tables) and keeps its
// own workspace, so every model must outlive the batch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>

#include "eit_state.h"

namespace mpf {

struct BatchClass {
    int KP = 0, W = 0, npad = 0, nblkMax = 0;
    std::vector<int> members;   // batch mesh index of each stacked mesh
    std::vector<int> tile0;     // its first 128-row tile
    DevBuf<int32_t> cols, diagSlot;
    DevBuf<int32_t> haloRows, haloCnt;  // halo plan of the tile-staged SpMM (HaloPlan)
    DevBuf<uint16_t> haloLcol;
    int Hpad = 0;
    DevBuf<int4> seg;
    DevBuf<float> Bc;           // [Ca][npad][KP]
    DevBuf<double> dcShift;     // [members][KP]
    // workspace for capF frames
    DevBuf<float2> SR;          // [F][W][npad]
    DevBuf<float> X, Rv, Pv, Qv;
    DevBuf<double> partA, partB, partC, rz, pq, bz, betaW, sumP, Gm;
    DevBuf<int> conv, active, iters, pend;
    DevBuf<unsigned> counter;
    DevBuf<double> alphaX;
    // BiCGSTAB vectors and scalars (grown on first use)
    int capFB = 0;
    DevBuf<float> Rhat, Zv, Tv;
    DevBuf<double> omegaW, rr2W;
    // two-level preconditioner: stacked coarse plan (static) and workspace
    int coarseOK = 0, ncPad = 0, cNnz = 0, capFC = 0;
    DevBuf<int32_t> cPairI, cPairJ, cPairPtr, cSlots, cMeshPairPtr, cMeshNc;
    DevBuf<float> cAggSize;
    DevBuf<double> Ac64, Lc64, rzFine, bzFine;
    DevBuf<float> Lc, LinvD, Binv, rcV, rcB, ycV;
    DevBuf<int> infoC;
};

}  // namespace mpf

struct mpf_batch {
    int device = 0, M = 0, Ca = 0, anyDcFree = 0, capF = 0, maxN = 0;
    std::vector<mpf_eit*> models;
    std::vector<std::unique_ptr<mpf::BatchClass>> classes;
    mpf::DevBuf<float> alpha;
    mpf::DevBuf<int32_t> dcFree;
    int* pinned = nullptr;
    size_t pinnedCount = 0;
    mpf::CgGraphCache graphs;
    std::map<int, std::vector<std::array<int, 3>>> variants;  // per frame count, per class
    std::array<int, 3> forced{-1, -1, -1};
    std::vector<int> iters;     // [mesh][frame][harmonic] of the last solve
    int lastFrames = 0;
    double lastCgMs = 0.0, lastCgBytes = 0.0;

    ~mpf_batch() {
        mpf::cg_graphs_clear(graphs);
        if (pinned) cudaFreeHost(pinned);
    }
};

namespace mpf {

// Stacked coarse plan of a width class: every member's (I, J) pairs with
// its slot indices moved to the stacked layout, per-mesh pair ranges,
// aggregate counts and sizes.  Built from the same rule as the model's own
// plan (model.cu): aggregates of kAgg consecutive rows, padding slots out.
static int class_coarse_plan(mpf_eit* const* models, BatchClass& cl) {
    const int Mc = (int)cl.members.size();
    cl.ncPad = 0;
    for (int j = 0; j < Mc; ++j) cl.ncPad = std::max(cl.ncPad, models[cl.members[j]]->ncPad);
    cl.coarseOK = coarse_supported(cl.KP, cl.ncPad) ? 1 : 0;
    if (!cl.coarseOK) return MPF_OK;
    std::vector<int32_t> pI, pJ, pPtr{0}, slots, meshPtr{0}, meshNc(Mc);
    std::vector<float> aggSize((size_t)Mc * cl.ncPad, 0.f);
    for (int j = 0; j < Mc; ++j) {
        const mpf_eit* m = models[cl.members[j]];
        const int row0 = cl.tile0[j] * kRowTile, n = m->n, P = m->npad;
        meshNc[j] = m->nc;
        for (int I = 0; I < m->nc; ++I) aggSize[(size_t)j * cl.ncPad + I] = (float)std::min(kAgg, n - I * kAgg);
        std::vector<std::vector<std::pair<int32_t, int32_t>>> byI(m->nc);
        for (int r = 0; r < n; ++r)
            for (int k = 0; k < m->W; ++k) {
                const int32_t c = m->fs.cols[(size_t)k * P + r];
                if (c == r && k != m->fs.diagSlot[r]) continue;
                byI[r / kAgg].push_back({c / kAgg, (int32_t)((size_t)k * cl.npad + row0 + r)});
            }
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
        meshPtr.push_back((int32_t)pI.size());
    }
    cl.cNnz = (int)pI.size();
    MPF_TRY(cl.cPairI.upload(pI));
    MPF_TRY(cl.cPairJ.upload(pJ));
    MPF_TRY(cl.cPairPtr.upload(pPtr));
    MPF_TRY(cl.cSlots.upload(slots));
    MPF_TRY(cl.cMeshPairPtr.upload(meshPtr));
    MPF_TRY(cl.cMeshNc.upload(meshNc));
    MPF_TRY(cl.cAggSize.upload(aggSize));
    return MPF_OK;
}

static int class_coarse_workspace(mpf_batch* b, BatchClass& cl, int F) {
    if (F <= cl.capFC) return MPF_OK;
    const size_t G = (size_t)F * b->Ca * cl.members.size(), nc2 = (size_t)cl.ncPad * cl.ncPad;
    const size_t cv = G * cl.ncPad * cl.KP;
    MPF_TRY(cl.Ac64.alloc(G * nc2));
    MPF_TRY(cl.Lc64.alloc(G * nc2));
    MPF_TRY(cl.Lc.alloc(G * nc2));
    MPF_TRY(cl.LinvD.alloc(G * (cl.ncPad / 32) * 1024));
    MPF_TRY(cl.Binv.alloc(G * nc2));
    MPF_TRY(cl.rcV.alloc(cv));
    MPF_TRY(cl.rcB.alloc(cv));
    MPF_TRY(cl.ycV.alloc(cv));
    MPF_CUDA(cudaMemset(cl.rcV.ptr, 0, cv * sizeof(float)));
    MPF_CUDA(cudaMemset(cl.rcB.ptr, 0, cv * sizeof(float)));
    MPF_CUDA(cudaMemset(cl.ycV.ptr, 0, cv * sizeof(float)));
    MPF_TRY(cl.rzFine.alloc(G * cl.KP));
    MPF_TRY(cl.bzFine.alloc(G * cl.KP));
    MPF_TRY(cl.infoC.alloc(2 * G));
    cl.capFC = F;
    return MPF_OK;
}

int batch_create(mpf_eit* const* models, int count, mpf_batch** out) {
    MPF_CHECK(models && out && count >= 1, MPF_EINVAL, "mpf_batch_create: bad arguments");
    auto b = std::make_unique<mpf_batch>();
    b->M = count;
    const mpf_eit* m0 = models[0];
    MPF_CHECK(m0, MPF_EINVAL, "mpf_batch_create: model 0 == nullptr");
    b->device = m0->device;
    b->Ca = m0->Ca;
    b->anyDcFree = m0->anyDcFree;
    for (int i = 0; i < count; ++i) {
        const mpf_eit* m = models[i];
        MPF_CHECK(m, MPF_EINVAL, "mpf_batch_create: model %d == nullptr", i);
        MPF_CHECK(m->device == b->device, MPF_EINVAL, "mpf_batch_create: model %d is on another device", i);
        MPF_CHECK(!m->fixed, MPF_ENOTSUP, "mpf_batch_create: model %d has voltage (fixed) sources", i);
        MPF_CHECK(!m->cem, MPF_ENOTSUP, "mpf_batch_create: model %d uses the complete electrode model", i);
        MPF_CHECK(m->Ca == b->Ca && m->anyDcFree == b->anyDcFree, MPF_EINVAL,
                  "mpf_batch_create: model %d has another harmonic set (components, height)", i);
        for (int c = 0; c < b->Ca; ++c)
            MPF_CHECK(std::fabs(m->alphaH[c] - m0->alphaH[c]) <= 1e-6f * std::max(1.f, std::fabs(m0->alphaH[c])),
                      MPF_EINVAL, "mpf_batch_create: model %d has another harmonic set (components, height)", i);
        b->models.push_back(models[i]);
        b->maxN = std::max(b->maxN, m->n);
    }
    MPF_CUDA(cudaSetDevice(b->device));
    MPF_TRY(b->alpha.upload(m0->alphaH));
    std::vector<int32_t> dcf(b->Ca, 0);
    if (b->anyDcFree) dcf[0] = 1;
    MPF_TRY(b->dcFree.upload(dcf));
    // width classes, members in batch order
    for (int KP : {16, 32, 64, 128}) {
        auto cl = std::make_unique<BatchClass>();
        cl->KP = KP;
        int tiles = 0;
        for (int i = 0; i < count; ++i) {
            if (models[i]->KP != KP) continue;
            cl->members.push_back(i);
            cl->tile0.push_back(tiles);
            tiles += models[i]->nblk;
            cl->W = std::max(cl->W, models[i]->W);
            cl->nblkMax = std::max(cl->nblkMax, models[i]->nblk);
        }
        if (cl->members.empty()) continue;
        cl->npad = tiles * kRowTile;
        const int Mc = (int)cl->members.size();
        std::vector<int32_t> cols((size_t)cl->W * cl->npad), diag(cl->npad);
        std::vector<int4> seg(Mc);
        MPF_TRY(cl->Bc.alloc((size_t)b->Ca * cl->npad * KP));
        MPF_TRY(cl->dcShift.alloc((size_t)Mc * KP));
        for (int j = 0; j < Mc; ++j) {
            const mpf_eit* m = models[cl->members[j]];
            const int row0 = cl->tile0[j] * kRowTile;
            std::vector<int32_t> mc((size_t)m->W * m->npad), md(m->npad);
            MPF_CUDA(cudaMemcpy(mc.data(), m->cols.ptr, sizeof(int32_t) * mc.size(), cudaMemcpyDeviceToHost));
            MPF_CUDA(cudaMemcpy(md.data(), m->diagSlot.ptr, sizeof(int32_t) * md.size(), cudaMemcpyDeviceToHost));
            for (int k = 0; k < cl->W; ++k)
                for (int r = 0; r < m->npad; ++r)
                    cols[(size_t)k * cl->npad + row0 + r] = row0 + (k < m->W ? mc[(size_t)k * m->npad + r] : r);
            for (int r = 0; r < m->npad; ++r) diag[row0 + r] = md[r];
            int dcBits;
            std::memcpy(&dcBits, &m->dcScale, sizeof(int));
            seg[j] = make_int4(cl->tile0[j], m->nblk, row0 + m->n, dcBits);
            for (int c = 0; c < b->Ca; ++c)
                MPF_CUDA(cudaMemcpy(cl->Bc.ptr + ((size_t)c * cl->npad + row0) * KP, m->Bc.ptr + (size_t)c * m->npad * KP,
                                    sizeof(float) * (size_t)m->npad * KP, cudaMemcpyDeviceToDevice));
            if (m->anyDcFree)
                MPF_CUDA(cudaMemcpy(cl->dcShift.ptr + (size_t)j * KP, m->dcShift.ptr, sizeof(double) * KP,
                                    cudaMemcpyDeviceToDevice));
        }
        MPF_TRY(cl->cols.upload(cols));
        MPF_TRY(cl->diagSlot.upload(diag));
        {
            HaloPlan hp;
            halo_plan(cols, cl->W, cl->npad, hp);
            cl->Hpad = hp.Hpad;
            MPF_TRY(cl->haloRows.upload(hp.halo));
            MPF_TRY(cl->haloCnt.upload(hp.hcnt));
            MPF_TRY(cl->haloLcol.upload(hp.lcol));
        }
        MPF_TRY(cl->seg.upload(seg));
        MPF_TRY(class_coarse_plan(models, *cl));
        b->classes.push_back(std::move(cl));
    }
    *out = b.release();
    return MPF_OK;
}

static int batch_workspace(mpf_batch* b, int F) {
    if (F <= b->capF) return MPF_OK;
    size_t Gtot = 0;
    for (auto& cp : b->classes) {
        BatchClass& cl = *cp;
        const size_t S = (size_t)F * b->Ca, Mc = cl.members.size(), G = S * Mc;
        MPF_CHECK(G <= 65535, MPF_EINVAL, "batch: %zu (frame, harmonic, mesh) groups of width %d in one launch "
                  "(max 65535)", G, cl.KP);
        const size_t vec = S * cl.npad * cl.KP;
        MPF_TRY(cl.SR.alloc((size_t)F * cl.W * cl.npad));
        // slots past a mesh's own density are never assembled: they stay zero
        MPF_CUDA(cudaMemset(cl.SR.ptr, 0, sizeof(float2) * (size_t)F * cl.W * cl.npad));
        MPF_TRY(cl.X.alloc(vec));
        MPF_TRY(cl.Rv.alloc(vec));
        MPF_TRY(cl.Pv.alloc(vec));
        MPF_TRY(cl.Qv.alloc(vec));
        const size_t parts = G * cl.nblkMax * cl.KP, sc = G * cl.KP;
        MPF_TRY(cl.partA.alloc(parts));
        MPF_TRY(cl.partB.alloc(parts));
        MPF_TRY(cl.partC.alloc(parts));
        MPF_TRY(cl.rz.alloc(sc));
        MPF_TRY(cl.pq.alloc(sc));
        MPF_TRY(cl.bz.alloc(sc));
        MPF_TRY(cl.betaW.alloc(sc));
        MPF_TRY(cl.sumP.alloc(sc));
        MPF_TRY(cl.conv.alloc(sc));
        MPF_TRY(cl.alphaX.alloc(sc));
        MPF_TRY(cl.pend.alloc(G));
        MPF_CUDA(cudaMemset(cl.pend.ptr, 0, G * sizeof(int)));
        MPF_TRY(cl.active.alloc(G));
        MPF_TRY(cl.iters.alloc(G));
        MPF_TRY(cl.counter.alloc(G));
        MPF_CUDA(cudaMemset(cl.counter.ptr, 0, G * sizeof(unsigned)));
        MPF_TRY(cl.Gm.alloc(G * cl.KP * cl.KP));
        Gtot += G;
    }
    if (b->pinned) cudaFreeHost(b->pinned);
    b->pinned = nullptr;
    MPF_CUDA(cudaMallocHost(&b->pinned, sizeof(int) * (Gtot + 1)));
    b->pinnedCount = Gtot;
    cg_graphs_clear(b->graphs);
    b->capF = F;
    return MPF_OK;
}

static int class_bicgstab(mpf_batch* b, BatchClass& cl, int F) {
    if (F <= cl.capFB) return MPF_OK;
    const size_t G = (size_t)F * b->Ca * cl.members.size(), vec = (size_t)F * b->Ca * cl.npad * cl.KP;
    MPF_TRY(cl.Rhat.alloc(vec));
    MPF_TRY(cl.Zv.alloc(vec));
    MPF_TRY(cl.Tv.alloc(vec));
    MPF_TRY(cl.omegaW.alloc(G * cl.KP));
    MPF_TRY(cl.rr2W.alloc(G * cl.KP));
    cl.capFB = F;
    return MPF_OK;
}

static CgProblem class_problem(mpf_batch* b, BatchClass& cl, int F, double tol, const std::array<int, 3>* shapes,
                               int solver = 0, bool coarse = false) {
    CgProblem P{};
    P.npad = cl.npad;
    P.n = cl.npad;
    P.W = cl.W;
    P.KP = cl.KP;
    P.Ca = b->Ca;
    P.M = (int)cl.members.size();
    P.G = F * b->Ca * P.M;
    P.nblk = cl.nblkMax;
    P.seg = cl.seg.ptr;
    P.cols = cl.cols.ptr;
    P.diagSlot = cl.diagSlot.ptr;
    P.halo = cl.haloRows.ptr;
    P.hcnt = cl.haloCnt.ptr;
    P.lcol = cl.haloLcol.ptr;
    P.Hpad = cl.Hpad;
    P.abortFlag = abort_flag_device();
    P.SR = cl.SR.ptr;
    P.alpha = b->alpha.ptr;
    P.x = cl.X.ptr;
    P.r = cl.Rv.ptr;
    P.p = cl.Pv.ptr;
    P.q = cl.Qv.ptr;
    P.b = cl.Bc.ptr;
    P.bPerGroup = 0;
    P.dcFree = b->dcFree.ptr;
    P.partA = cl.partA.ptr;
    P.partB = cl.partB.ptr;
    P.partC = cl.partC.ptr;
    P.sumP = cl.sumP.ptr;
    P.rz = cl.rz.ptr;
    P.pq = cl.pq.ptr;
    P.bz = cl.bz.ptr;
    P.beta = cl.betaW.ptr;
    P.conv = cl.conv.ptr;
    P.active = cl.active.ptr;
    P.iters = cl.iters.ptr;
    P.counter = cl.counter.ptr;
    P.alphaX = cl.alphaX.ptr;
    P.pend = cl.pend.ptr;
    P.tol2 = tol * tol;
    if (coarse) {
        P.coarse = 1;
        P.ncPad = cl.ncPad;
        P.rc = cl.rcV.ptr;
        P.rcB = cl.rcB.ptr;
        P.yc = cl.ycV.ptr;
        P.Binv = cl.Binv.ptr;
        P.rzFine = cl.rzFine.ptr;
        P.bzFine = cl.bzFine.ptr;
    }
    if (solver == 1) {
        P.solver = 1;
        P.rhat = cl.Rhat.ptr;
        P.zv = cl.Zv.ptr;
        P.tv = cl.Tv.ptr;
        P.omega = cl.omegaW.ptr;
        P.rr2 = cl.rr2W.ptr;
    }
    for (int k = 0; k < 3; ++k) {
        int code = shapes ? (*shapes)[k] : cg_default_variant(cl.KP);
        if (b->forced[k] >= 0) code = b->forced[k];
        cg_set_shape(P, k, code);
    }
    return P;
}

int batch_forward(mpf_batch* b, int F, const float* const* gamma, float* const* V, const mpf_solve_opts* in,
                  mpf_solve_stats* stats, cudaStream_t s) {
    auto t0 = std::chrono::steady_clock::now();
    MPF_CHECK(F >= 1 && gamma && V, MPF_EINVAL, "mpf_batch_forward: bad arguments");
    for (int i = 0; i < b->M; ++i)
        MPF_CHECK(gamma[i] && V[i], MPF_EINVAL, "mpf_batch_forward: gamma[%d] or voltages[%d] == nullptr", i, i);
    mpf_solve_opts o{};
    o.tol = 1e-6;
    o.max_refine = 6;
    o.check_every = 16;
    if (in) o = *in;
    MPF_CHECK(o.refine_tol <= 0.0 && o.warm_start == 0, MPF_ENOTSUP,
              "mpf_batch_forward: batches solve cold without FP64 refinement");
    const int solver = o.solver == 1 ? 1 : 0;
    const bool coarse = o.preconditioner == 1 && solver == 0;
    if (o.tol <= 0.0) o.tol = 1e-6;
    if (o.max_iter <= 0) o.max_iter = 10 * b->maxN;
    if (o.check_every <= 0) o.check_every = 16;
    MPF_CUDA(cudaSetDevice(b->device));
    MPF_TRY(batch_workspace(b, F));
    // assembly of every mesh into its rows of the stacked slot arrays
    for (auto& cp : b->classes) {
        BatchClass& cl = *cp;
        for (size_t j = 0; j < cl.members.size(); ++j) {
            const int i = cl.members[j];
            const mpf_eit* m = b->models[i];
            MPF_TRY(fem_launch_assemble(F, m->W, m->npad, m->E, m->cptr.ptr, m->contrib.ptr, m->Kf.ptr, m->Mf.ptr,
                                        nullptr, nullptr, gamma[i], m->ref, m->logarithmic,
                                        cl.SR.ptr + (size_t)cl.tile0[j] * kRowTile, nullptr, nullptr, s,
                                        (size_t)cl.npad, (size_t)cl.W * cl.npad));
        }
    }
    const int nC = (int)b->classes.size();
    if (solver == 1)
        for (auto& cp : b->classes) MPF_TRY(class_bicgstab(b, *cp, F));
    if (!b->variants.count(F) && solver == 0) {
        std::vector<std::array<int, 3>> best(nC);
        for (int c = 0; c < nC; ++c) {
            if (b->forced[0] >= 0 && b->forced[1] >= 0 && b->forced[2] >= 0) {
                best[c] = b->forced;
                continue;
            }
            MPF_TRY(cg_autotune(class_problem(b, *b->classes[c], F, 0.0, nullptr), best[c], s));
        }
        b->variants[F] = best;
    }
    std::vector<CgProblem> Ps;
    for (int c = 0; c < nC; ++c) {
        BatchClass& cl = *b->classes[c];
        auto it = b->variants.find(F);
        const bool cc = coarse && cl.coarseOK;
        Ps.push_back(class_problem(b, cl, F, o.tol, it != b->variants.end() ? &it->second[c] : nullptr, solver, cc));
        if (cc) {
            MPF_TRY(class_coarse_workspace(b, cl, F));
            Ps.back() = class_problem(b, cl, F, o.tol, it != b->variants.end() ? &it->second[c] : nullptr, solver, cc);
            CoarsePlan cp{0, cl.ncPad, cl.cNnz, cl.cPairI.ptr, cl.cPairJ.ptr, cl.cPairPtr.ptr, cl.cSlots.ptr,
                          cl.cAggSize.ptr, cl.cMeshPairPtr.ptr, cl.cMeshNc.ptr};
            MPF_TRY(coarse_launch_setup(Ps.back(), cp, cl.Ac64.ptr, cl.infoC.ptr, s, cl.Lc.ptr, cl.LinvD.ptr,
                                        cl.Binv.ptr, cl.Lc64.ptr));
        }
    }
    cudaEvent_t e0, e1;
    MPF_CUDA(cudaEventCreate(&e0));
    MPF_CUDA(cudaEventCreate(&e1));
    int st = MPF_OK, maxIt = 0, notConv = 0;
    std::vector<int> iters;
    cudaEventRecord(e0, s);
    for (int c = 0; c < nC && st == MPF_OK; ++c) st = cg_launch_init(Ps[c], true, s);
    if (st == MPF_OK) st = cg_run(b->graphs, b->pinned, Ps.data(), nC, o.max_iter, o.check_every, s, iters, &maxIt,
                                  &notConv);
    cudaEventRecord(e1, s);
    float cgMs = 0.f;
    if (st == MPF_OK) {
        cudaError_t e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&cgMs, e0, e1);
        if (e != cudaSuccess) st = fail(MPF_ECUDA, "batch CG timing: %s", cudaGetErrorString(e));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != MPF_OK) return st;
    for (int c = 0; c < nC; ++c) {
        if (!Ps[c].coarse) continue;
        std::vector<int> info(Ps[c].G);
        MPF_CUDA(cudaMemcpy(info.data(), b->classes[c]->infoC.ptr, sizeof(int) * info.size(), cudaMemcpyDeviceToHost));
        for (int g = 0; g < Ps[c].G; ++g)
            MPF_CHECK(info[g] == 0, MPF_EBREAKDOWN, "two-level preconditioner: coarse Cholesky failed at pivot %d "
                      "(group %d of width class %d)", info[g], g, Ps[c].KP);
    }
    // per-group iterations in [mesh][frame][harmonic] order and the
    // algorithmic bytes the iterations moved (CG, per iteration and group:
    // the SpMM's nnz*12 + 2*K*n*4, the update's 3*K*n*4 + 2*n*4 and the
    // direction's 5*K*n*4 + 2*n*4, K = unique excitation columns)
    b->iters.assign((size_t)b->M * F * b->Ca, 0);
    double bytes = 0.0;
    size_t off = 0;
    for (int c = 0; c < nC; ++c) {
        BatchClass& cl = *b->classes[c];
        const int Mc = (int)cl.members.size();
        for (int sl = 0; sl < F * b->Ca; ++sl)
            for (int j = 0; j < Mc; ++j) {
                const mpf_eit* m = b->models[cl.members[j]];
                const int it = iters[off + (size_t)sl * Mc + j];
                b->iters[(size_t)cl.members[j] * F * b->Ca + sl] = it;
                const double n = m->n, K = m->K;
                // BiCGSTAB: two SpMVs, 21 vector passes, three diagonal reads;
                // two-level CG: plus the coarse inverse and coarse vectors
                const double coarseBytes =
                    Ps[c].coarse ? (double)cl.ncPad * cl.ncPad * 4.0 + 3.0 * cl.ncPad * K * 4.0 : 0.0;
                bytes += solver == 1 ? it * (2.0 * m->nnz * 12.0 + 21.0 * K * n * 4.0 + 6.0 * n * 4.0)
                                     : it * ((double)m->nnz * 12.0 + 10.0 * K * n * 4.0 + 4.0 * n * 4.0 + coarseBytes);
            }
        off += (size_t)F * b->Ca * Mc;
    }
    b->lastFrames = F;
    b->lastCgMs = cgMs;
    b->lastCgBytes = bytes;
    // the reference's (A + 1 1^T) solution on the Neumann harmonic, then voltages
    for (int c = 0; c < nC; ++c) {
        BatchClass& cl = *b->classes[c];
        if (b->anyDcFree) MPF_TRY(cg_launch_dc_shift(Ps[c], cl.dcShift.ptr, 1.f, s));
        const int S = F * b->Ca;
        for (size_t j = 0; j < cl.members.size(); ++j) {
            const int i = cl.members[j];
            const mpf_eit* m = b->models[i];
            double* Gm = cl.Gm.ptr + j * (size_t)S * cl.KP * cl.KP;
            MeasPlan mp{(int)m->nzNode.count, m->nzNode.ptr, nullptr, m->nzVal.ptr, m->nzPtr.ptr};
            MPF_TRY(fem_launch_gram_meas(S, cl.KP, cl.npad, mp, cl.X.ptr + (size_t)cl.tile0[j] * kRowTile * cl.KP, Gm,
                                         s));
            MPF_TRY(fem_launch_voltages(F, b->Ca, cl.KP, m->Mm, m->Md, Gm, m->beta.ptr, m->measU.ptr,
                                        m->measScale.ptr, m->driveU.ptr, m->driveScale.ptr, V[i], s));
        }
    }
    MPF_CUDA(cudaStreamSynchronize(s));
    MPF_CUDA(cudaGetLastError());
    if (stats) {
        stats->iterations = maxIt;
        stats->refinements = 0;
        stats->not_converged = notConv;
        stats->max_rel_residual = 0.0;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return notConv ? fail(MPF_ENOCONV, "batch forward solve: %d groups did not converge", notConv) : MPF_OK;
}

int batch_iterations(mpf_batch* b, int32_t* out, int cap, int32_t* count) {
    const int n = (int)b->iters.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = b->iters[i];
    if (count) *count = n;
    return MPF_OK;
}

int batch_cg_stats(mpf_batch* b, double* ms, double* bytes) {
    if (ms) *ms = b->lastCgMs;
    if (bytes) *bytes = b->lastCgBytes;
    return MPF_OK;
}

int batch_cg_variants(mpf_batch* b, const int32_t* set, int F, int32_t* get, int cap, int32_t* classes) {
    if (set) {
        for (int k = 0; k < 3; ++k) {
            for (auto& cp : b->classes)
                MPF_CHECK(set[k] < 0 || cg_shape_fits(cp->KP, cp->W, cp->Hpad, true, k, set[k]), MPF_EINVAL,
                          "mpf_batch_cg_variants: shape %d not available for %d right-hand sides", set[k], cp->KP);
            b->forced[k] = set[k];
        }
        b->variants.clear();
        cg_graphs_clear(b->graphs);
    }
    const int nC = (int)b->classes.size();
    if (classes) *classes = nC;
    if (get) {
        auto it = b->variants.find(F);
        for (int c = 0; c < nC && 3 * c + 2 < cap; ++c)
            for (int k = 0; k < 3; ++k) {
                int code = it != b->variants.end() ? it->second[c][k] : cg_default_variant(b->classes[c]->KP);
                if (b->forced[k] >= 0) code = b->forced[k];
                get[3 * c + k] = code;
            }
    }
    return MPF_OK;
}

void batch_destroy(mpf_batch* b) {
    if (b) cudaSetDevice(b->device);
    delete b;
}

}  // namespace mpf
