// batch.cuh -- the engine under gs_batch and gs_server: a set of member systems, their
// plan on the device, and the streams that batched steps run on.
#pragma once
#include <vector>

#include "internal.cuh"

namespace gsim {

// A new plan reaches the device stream-ordered: it is written to pinned staging and
// copied on the root stream into whichever of two device blocks the steps already in
// flight are not reading.  Changing the members therefore never waits for the GPU.
struct BatchEngine {
    int device = 0;
    cudaStream_t root = nullptr;  // Barnes-Hut stages; the step's order point
    cudaStream_t side = nullptr;  // the direct-sum launch, beside the Barnes-Hut stages
    cudaEvent_t fork = nullptr, join = nullptr;
    StepFork moments;            // the quadrupole moment prefix, beside the node layout
    std::vector<gs_sim*> order;  // plan order: Barnes-Hut largest first, then direct sum
    std::vector<int> parity0;    // each member's compute-input set when the plan was built
    uint64_t step = 0;           // steps enqueued since then
    BatchPlan plan;
    int cur = 1;
    void* d_block[2] = {nullptr, nullptr};
    size_t d_bytes[2] = {0, 0};
    void* h_stage[2] = {nullptr, nullptr};
    size_t h_bytes[2] = {0, 0};
    cudaEvent_t staged[2] = {nullptr, nullptr};  // the copy out of staging k is done
    uint2* d_heavy = nullptr;                    // costly groups of a step, all members
    size_t heavy_cap = 0;                        // entries d_heavy holds
    gs_shape shape{};                            // launch shapes of the batched kernels

    cudaError_t init(int dev);
    void destroy();
    // Plans `members` (any order; may be empty) with their current parities.
    gs_status set_members(const std::vector<gs_sim*>& members);
    // Enqueues one batched step for step parity `par` (no host bookkeeping); `estimate`
    // adds the |a| estimate pass for members without a previous |a|.
    cudaError_t enqueue(uint32_t par, bool estimate);
    // A member has no previous |a| for the relative criterion (it joined or was reset).
    bool needs_estimate() const;
    // Host bookkeeping of one enqueued step: member parities flip, |a| becomes known.
    void advance();
    // True while every member is at the parity the plan expects.
    bool in_step() const;
    uint32_t launches_per_step() const;
};

// Members that can share one plan (same device; Barnes-Hut members share box mode, math
// mode and the accurate-mode / counting flags; direct-sum members share math mode).
gs_status check_batch_members(gs_sim* const* sims, size_t count, const char* who);

}  // namespace gsim
