// Gate fusion for the FP32 path: consecutive gates are grouped into blocks of at most `max_qubits`
// qubits, and each block becomes one dense 2^m x 2^m complex matrix (the product of its gates'
// effective operators, computed in FP64 on the host).
#pragma once

#include <complex>
#include <vector>

#include "compile.cuh"

namespace qcs {

struct FusedBlock {
	std::vector<uint32_t> qubits;             // ascending; matrix bit j <-> qubits[j]
	std::vector<std::complex<double>> M;      // 2^m x 2^m, row-major
	uint32_t ngates = 0;                      // original gates folded in
};

// cost callback for the partition search: predicted device time of one block application
// (qubits ascending), in arbitrary units; nullptr = plain greedy
using BlockCost = double (*)(const std::vector<uint32_t>& qubits, uint32_t ngates, int nqubits_register, void* ctx);

struct FusionPolicy {
	int max_qubits = 5;
	BlockCost cost = nullptr;   // when set, merges are accepted only if the predicted cost does not grow
	void* ctx = nullptr;
	int nqubits = 0;
};

// greedy fusion that reorders only gates on disjoint qubits (which commute)
std::vector<FusedBlock> fuse(const std::vector<CompiledGate>& gates, const FusionPolicy& policy);

// packs blocks into shared-memory passes of at most kmax tile qubits (qubits below L0 always in the
// tile): each pass takes, in order, every block that fits and shares no qubit with an earlier block
// still waiting (blocks on disjoint qubits commute), looking at most `window` blocks ahead.  With
// tc_budget > 0 (tensor-core passes), every block also draws 32 x 4^max(m, 4) bytes of resident
// matrices from that budget.  Blocks without qubits (global factors) take no pass.  Returns the block indices of each
// pass, each in the original order.
std::vector<std::vector<size_t>> pack_blocks(const std::vector<FusedBlock>& blocks, int kmax, int L0, uint32_t tc_budget,
                                             size_t window = 64);

// apply one compiled gate (its effective operator, including its factored scale) to a vector over
// the block's qubits, in block-local indexing
void apply_compiled_local(const CompiledGate& c, const std::vector<uint32_t>& qubits, std::complex<double>* v);

}  // namespace qcs
