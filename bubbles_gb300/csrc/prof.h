// prof.h -- optional per-launch CUDA-event timing of the solver's kernels.
//
// The reference wraps every GPULaunch in ProfilerPrepare / ProfilerFinish with CUDA
// events (src/cuda/cutil.h:237-244, src/core/profiler.cpp:90-248).  Here the events are
// recorded on the launching stream only while profiling is enabled, without any
// per-launch synchronisation; durations are resolved when the report is drained.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace bbg {

enum KernelId {
    KID_HASH_COUNT = 0, KID_SCAN, KID_PLACE, KID_RANK_GATHER, KID_DENSITY, KID_NON_PRESSURE,
    KID_PREDICT_FIRST, KID_PRED_DENSITY, KID_PRESSURE_FORCE, KID_SPH_FORCES, KID_INTEGRATE,
    KID_PSEUDO_VISCOSITY, KID_LAYOUT, KID_MAX_FORCE, KID_MLP, KID_MLP_TRAIN, KID_COUNT
};

inline const char *kernel_name(int id) {
    static const char *names[KID_COUNT] = {
        "k_hash_count", "k_scan", "k_place", "k_rank_gather", "k_density", "k_non_pressure",
        "k_predict_first", "k_pred_density", "k_pressure_force", "k_sph_forces", "k_integrate",
        "k_pseudo_viscosity", "k_layout", "k_max_force", "k_mlp_warm_start", "k_mlp_train"};
    return (id >= 0 && id < KID_COUNT) ? names[id] : "?";
}

struct Prof {
    struct Rec {
        int id, iter;
        long long substep;
        cudaEvent_t a, b;
        bool skipped;
    };
    bool on = false;
    long long substep = 0;
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    size_t launches = 0;
    cudaEvent_t pending_a = nullptr;
    int pending_id = -1, pending_iter = -1;

    cudaEvent_t take() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void begin(int id, cudaStream_t s, int iter = -1) {
        if (!on) return;
        pending_a = take();
        pending_id = id;
        pending_iter = iter;
        cudaEventRecord(pending_a, s);
    }
    void end(cudaStream_t s) {
        if (!on || !pending_a) return;
        cudaEvent_t b = take();
        cudaEventRecord(b, s);
        recs.push_back(Rec{pending_id, pending_iter, substep, pending_a, b, false});
        pending_a = nullptr;
        launches++;
    }
    // Corrector launches of iterations at or after `iters` in the current substep returned
    // without work; keep them out of the per-kernel averages.
    void mark_iterations(int iters) {
        for (auto &r : recs)
            if (r.substep == substep && r.iter >= iters) r.skipped = true;
    }
    void release() {
        for (auto &r : recs) {
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        recs.clear();
        launches = 0;
    }
    ~Prof() {
        for (auto &r : recs) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace bbg
