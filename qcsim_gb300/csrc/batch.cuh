// Gate-list execution: the planner that groups consecutive gates into shared-memory passes, and
// the QFT sequence.
#pragma once

#include <vector>

#include "engine.cuh"
#include "fusion.cuh"

namespace qcs {

// one gate through the per-gate kernels (api.cu)
cudaError_t apply_one(qcs_handle h, const qcs_gate& g);

// ApplyGates: results identical to applying the gates one by one
int batch_apply(qcs_handle h, const qcs_gate* gates, size_t count);
// QuantumFourierTransform::QFT / IQFT over [start, end]
int qft_apply(qcs_handle h, uint32_t start, uint32_t end, bool inverse, bool do_swap);
// SchrodingerSimulation::Execute's Suzuki-Trotter steps (Schrodinger.h:32-45) with its potential and
// kinetic diagonals already on the device (2^n entries each, the register's precision)
int schrodinger_apply(qcs_handle h, const void* d_potential, const void* d_kinetic, uint64_t steps);
void batch_release(qcs_handle h);

// dense blocks applied in shared-memory passes
int apply_blocks(qcs_handle h, std::vector<FusedBlock> blocks);
// the candidate partition with the lowest predicted time (costmodel.cu)
int choose_partition(qcs_handle h, const std::vector<CompiledGate>& gates, int kmax, int L0, std::vector<FusedBlock>& best,
                     double* predicted_ms);
void release_cost_model(qcs_handle h);

}  // namespace qcs
