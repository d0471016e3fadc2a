// Host drivers of the batched CG: launch-shape autotuning and the iteration
// loop (CUDA-graph replays with a host convergence check per replay).  Used
// by single models (model.cu) and by batches of uneven meshes (batch.cu).
//
// The loop restates the outer loop of ConjugateGradient::solve
// (src/numeric/conjugate_gradient.cpp:61-161) for many systems: instead of a
// D2H copy of column 0's residual after every iteration, the device keeps a
// per-group active flag (every right-hand side of the group converged) and
// the host reads the flags once per `checkEvery` iterations.
#include <algorithm>

#include "model.h"

namespace mpf {

void halo_plan(const std::vector<int32_t>& cols, int W, int npad, HaloPlan& out) {
    const int tiles = npad / kRowTile;
    std::vector<std::vector<int32_t>> lists(tiles);
    int hmax = 0;
    for (int t = 0; t < tiles; ++t) {
        const int r0 = t * kRowTile;
        auto& h = lists[t];
        for (int k = 0; k < W; ++k)
            for (int r = r0; r < r0 + kRowTile; ++r) {
                const int32_t c = cols[(size_t)k * npad + r];
                if (c < r0 || c >= r0 + kRowTile) h.push_back(c);
            }
        std::sort(h.begin(), h.end());
        h.erase(std::unique(h.begin(), h.end()), h.end());
        hmax = std::max(hmax, (int)h.size());
    }
    out.Hpad = std::max(8, round_up(hmax, 8));
    out.halo.assign((size_t)tiles * out.Hpad, -1);  // -1: no halo row in this place
    out.hcnt.assign(tiles, 0);
    out.lcol.assign((size_t)tiles * W * kRowTile, 0);
    for (int t = 0; t < tiles; ++t) {
        const int r0 = t * kRowTile;
        const auto& h = lists[t];
        out.hcnt[t] = (int32_t)h.size();
        std::copy(h.begin(), h.end(), out.halo.begin() + (size_t)t * out.Hpad);
        for (int k = 0; k < W; ++k)
            for (int r = 0; r < kRowTile; ++r) {
                const int32_t c = cols[(size_t)k * npad + r0 + r];
                const int local = (c >= r0 && c < r0 + kRowTile)
                                      ? c - r0
                                      : kRowTile + (int)(std::lower_bound(h.begin(), h.end(), c) - h.begin());
                out.lcol[((size_t)t * W + k) * kRowTile + r] = (uint16_t)local;
            }
    }
}

void cg_graphs_clear(CgGraphCache& cache) {
    for (auto& kv : cache) cudaGraphExecDestroy(kv.second);
    cache.clear();
}

void cg_set_shape(CgProblem& P, int which, int code) {
    const int group = kCgVariants * kCgTileChoices;
    P.variant[which] = code % kCgVariants + kCgVariants * (code / group);
    // the tile-staged SpMM walks longer tile ranges: 4, 8, 16 or 32 tiles
    const int shift = (which == 0 && cg_spmm_form(code) >= 2) ? 2 : 0;
    P.tiles[which] = 1 << ((code % group) / kCgVariants + shift);
}

int cg_autotune(const CgProblem& P0, std::array<int, 3>& best, cudaStream_t s) {
    CgProblem P = P0;
    P.tol2 = 0.0;  // no group retires while timing
    cudaEvent_t e0, e1;
    MPF_CUDA(cudaEventCreate(&e0));
    MPF_CUDA(cudaEventCreate(&e1));
    int st = MPF_OK;
    for (int which = 0; which < 3 && st == MPF_OK; ++which) {
        float bestMs = 1e30f;
        best[which] = cg_default_variant(P.KP);
        for (int v = 0; v < cg_shape_count(which) && st == MPF_OK; ++v) {
            if (!cg_shape_fits(P.KP, P.W, P.Hpad, P.halo != nullptr, which, v)) continue;
            CgProblem Q = P;
            cg_set_shape(Q, which, v);
            // fresh state with valid p.q, then one untimed launch
            st = cg_launch_init(Q, true, s);
            if (st == MPF_OK) st = cg_launch_kernel(Q, 0, s);
            if (st == MPF_OK) st = cg_launch_kernel(Q, which, s);
            float msMin = 1e30f;
            for (int rep = 0; rep < 2 && st == MPF_OK; ++rep) {
                cudaEventRecord(e0, s);
                for (int i = 0; i < 4 && st == MPF_OK; ++i) st = cg_launch_kernel(Q, which, s);
                cudaEventRecord(e1, s);
                cudaError_t e = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess && st == MPF_OK) st = fail(MPF_ECUDA, "autotune timing: %s", cudaGetErrorString(e));
                msMin = std::min(msMin, ms);
            }
            if (st == MPF_OK && msMin < bestMs) {
                bestMs = msMin;
                best[which] = v;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

int cg_run(CgGraphCache& cache, int* pinned, const CgProblem* Ps, int nP, int maxIter, int checkEvery,
           cudaStream_t s, std::vector<int>& iters, int* maxIters, int* notConverged) {
    std::string key(reinterpret_cast<const char*>(Ps), sizeof(CgProblem) * (size_t)nP);
    key += std::to_string(checkEvery);
    int Gtot = 0;
    long long perIteration = 0;
    for (int i = 0; i < nP; ++i) {
        Gtot += Ps[i].G;
        perIteration += cg_iteration_launches(Ps[i]);
    }
    cudaGraphExec_t exec = nullptr;
    auto it = cache.find(key);
    if (it != cache.end()) {
        exec = it->second;
    } else {
        for (int i = 0; i < nP; ++i) MPF_TRY(cg_prepare_launch(Ps[i]));
        cudaStream_t cap;
        MPF_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t graph;
        MPF_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        int st = MPF_OK;
        for (int k = 0; k < checkEvery && st == MPF_OK; ++k)
            for (int i = 0; i < nP && st == MPF_OK; ++i) st = cg_launch_iteration(Ps[i], cap);
        cudaError_t e = cudaStreamEndCapture(cap, &graph);
        cudaStreamDestroy(cap);
        if (st != MPF_OK) return st;
        MPF_CHECK(e == cudaSuccess, MPF_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        MPF_CHECK(e == cudaSuccess, MPF_ECUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
        cache[key] = exec;
    }
    // the bulk-copy SpMM raises the device's abort flag when a wait gives up:
    // it is read with the active flags (pinned[Gtot]) and ends the solve
    int* abortFlag = nullptr;
    for (int i = 0; i < nP; ++i)
        if (Ps[i].abortFlag) abortFlag = Ps[i].abortFlag;
    auto fetch = [&](bool activeFlags) -> int {
        int off = 0;
        for (int i = 0; i < nP; ++i) {
            MPF_CUDA(cudaMemcpyAsync(pinned + off, activeFlags ? Ps[i].active : Ps[i].iters, sizeof(int) * Ps[i].G,
                                     cudaMemcpyDeviceToHost, s));
            off += Ps[i].G;
        }
        pinned[Gtot] = 0;
        if (abortFlag) MPF_CUDA(cudaMemcpyAsync(pinned + Gtot, abortFlag, sizeof(int), cudaMemcpyDeviceToHost, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        if (pinned[Gtot]) {
            // the result is undefined: clear the flag and the reduction counters
            MPF_CUDA(cudaMemset(abortFlag, 0, sizeof(int)));
            for (int i = 0; i < nP; ++i) MPF_CUDA(cudaMemset(Ps[i].counter, 0, sizeof(unsigned) * Ps[i].G));
            return fail(MPF_ETIMEOUT, "CG: a bulk-copy wait of the tile-staged SpMM timed out");
        }
        return MPF_OK;
    };
    int done = 0;
    bool anyActive = true;
    while (done < maxIter) {
        MPF_CUDA(cudaGraphLaunch(exec, s));
        add_launches(perIteration * checkEvery);
        done += checkEvery;
        MPF_TRY(fetch(true));
        anyActive = false;
        for (int g = 0; g < Gtot; ++g) anyActive |= pinned[g] != 0;
        if (!anyActive) break;
    }
    int nc = 0;
    if (anyActive) {
        for (int g = 0; g < Gtot; ++g) nc += pinned[g] != 0;
    }
    // the x update of groups that retired in their last k_update
    for (int i = 0; i < nP; ++i) MPF_TRY(cg_launch_finalize(Ps[i], s));
    MPF_TRY(fetch(false));
    iters.assign(pinned, pinned + Gtot);
    *maxIters = Gtot ? *std::max_element(iters.begin(), iters.end()) : 0;
    *notConverged = nc;
    return MPF_OK;
}

}  // namespace mpf
