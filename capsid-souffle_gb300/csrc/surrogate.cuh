// Hooks of the learned far-field part (surrogate.cu) into the launch sequences of souffle_gpu.cu.
// All of them only enqueue work on the system's stream, so they can be captured in CUDA graphs.
#pragma once
#include "kernels.cuh"

struct souffle_gpu_system;

namespace souffle {

struct SurrogateCtx;
void surrogate_free(SurrogateCtx* s);

// attached, trained and switched on
bool surrogate_enabled(const souffle_gpu_system* h);
// between the candidate search and the bead-pair build of a rebuild: marks far candidate subunit
// pairs and lets k_pairs skip them
void surrogate_classify(souffle_gpu_system* h, PairArgs& pa);
// after the bead-pair build: the far-pair list in candidate order
void surrogate_compact(souffle_gpu_system* h);
// before k_forces: frames, descriptors, network, per-bead far-field forces for k_forces to add
void surrogate_forces(souffle_gpu_system* h, ForceArgs& fa);
// exact re-evaluation of a sampled fraction of the far pairs, after surrogate_forces of the same
// positions; classes whose error exceeds the tolerance revert to exact at the next rebuild
bool surrogate_judge_due(const souffle_gpu_system* h, long long step);
void surrogate_judge(souffle_gpu_system* h);

}  // namespace souffle
