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

void cg_graphs_clear(CgGraphCache& cache) {
    for (auto& kv : cache) cudaGraphExecDestroy(kv.second);
    cache.clear();
}

void cg_set_shape(CgProblem& P, int which, int code) {
    const int group = kCgVariants * kCgTileChoices;
    P.variant[which] = code % kCgVariants + kCgVariants * (code / group);
    P.tiles[which] = 1 << ((code % group) / kCgVariants);
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
            if (!cg_shape_valid(P.KP, which, v)) continue;
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
    auto fetch = [&](bool activeFlags) -> int {
        int off = 0;
        for (int i = 0; i < nP; ++i) {
            MPF_CUDA(cudaMemcpyAsync(pinned + off, activeFlags ? Ps[i].active : Ps[i].iters, sizeof(int) * Ps[i].G,
                                     cudaMemcpyDeviceToHost, s));
            off += Ps[i].G;
        }
        MPF_CUDA(cudaStreamSynchronize(s));
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
