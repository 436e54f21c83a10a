// Gate compilation: QubitRegister::ApplyGate's trait dispatch (QubitRegister.h:434-486 and
// QubitRegisterCalculator.h:39-227) turned into a kernel operation that the per-gate kernels and the
// shared-memory pass kernels both execute.
#pragma once

#include <complex>
#include <vector>

#include "engine.cuh"

namespace qcs {

enum class GKind : int {
	Identity = 0,  // nothing to do (e.g. a diagonal gate whose read entries are both 1)
	Ctrl1q,        // 2x2 block on `target`, under `controls`
	Swap,          // exchange base|bitA with base|bitB, under `controls`
	Dense,         // 4x4 or 8x8 block on dense_q, under `controls`
	Block,         // fused block: dense 2^m x 2^m matrix on block_q (ascending), no controls
	PhaseRow,      // the QFT's run of controlled phases on one target (see below); shared-memory passes only
	TableDiag      // diagonal operator from a device table: amplitude i *= table[i] (table in the register's precision)
};

struct CompiledGate {
	GKind kind = GKind::Identity;
	Op1 op = Op1::Generic;
	SwapKind sk = SwapKind::Plain;
	Mat2<double> m{};
	uint32_t target = 0;        // Ctrl1q: the 2x2 block's qubit
	bool phase_on_a0 = false;   // Phase*: the factor sits on the target-bit-0 half
	uint32_t ncontrols = 0;
	uint32_t controls[2] = {0, 0};
	uint32_t qa = 0, qb = 0;    // Swap: exchange |..qa=1..qb=0..> with |..qa=0..qb=1..>
	int dense_k = 0;
	uint32_t dense_q[3] = {0, 0, 0};  // qubit of matrix bit 0, 1, 2
	double dense_m[128] = {};
	std::complex<double> scale{1.0, 0.0};  // global factor taken out of the matrix
	std::vector<uint32_t> block_q;          // Block: qubits, ascending (matrix bit j <-> block_q[j])
	std::vector<std::complex<double>> block_m;  // Block: row-major 2^m x 2^m
	uint32_t block_gates = 0;               // Block: original gates folded in
	// PhaseRow: amplitudes with bit `target` set get exp(+-2 pi i y / 2^(row_bits + 1)), y = the integer
	// in bits row_lo .. row_lo + row_bits - 1: the product of ControlledPhaseShift(pi / 2^(target - c))
	// over controls c = target - 1 .. row_lo, the phases one QFT step applies to one target
	uint32_t row_lo = 0, row_bits = 0;
	bool row_inverse = false;
	const void* table = nullptr;  // TableDiag: 2^n entries on the device

	// qubits whose bit a tile must hold locally to apply this gate (targets of non-diagonal blocks)
	uint64_t local_mask() const;
	// every qubit the gate depends on
	uint64_t touch_mask() const;
};

// kernel family name (profiling) and the fraction of amplitudes the gate reads and writes
const char* kernel_name(const CompiledGate& c);
double touched_fraction(const CompiledGate& c);

// `factor` allows taking a global scalar out of uncontrolled one-qubit gates
CompiledGate compile_gate(const qcs_gate& g, bool factor);

// run one compiled gate with the per-gate kernels
template <typename T> cudaError_t launch_compiled(cplx_t<T>* s, uint64_t N, const CompiledGate& cg, int sms, cudaStream_t st);

template <typename T>
cudaError_t launch_scale_complex(cplx_t<T>* s, uint64_t N, double re, double im, int sms, cudaStream_t st);

// amplitude i *= d[i] over the whole register (operator.cu)
template <typename T>
cudaError_t launch_table_diag(cplx_t<T>* s, uint64_t N, const cplx_t<T>* d, int sms, cudaStream_t st);

}  // namespace qcs
