// Gate-list execution: the planner that groups consecutive gates into shared-memory passes, and
// the QFT sequence.
#pragma once

#include "engine.cuh"

namespace qcs {

// one gate through the per-gate kernels (api.cu)
cudaError_t apply_one(qcs_handle h, const qcs_gate& g);

// ApplyGates: results identical to applying the gates one by one
int batch_apply(qcs_handle h, const qcs_gate* gates, size_t count);
// QuantumFourierTransform::QFT / IQFT over [start, end]
int qft_apply(qcs_handle h, uint32_t start, uint32_t end, bool inverse, bool do_swap);
void batch_release(qcs_handle h);

}  // namespace qcs
