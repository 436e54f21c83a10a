// Gate-list execution (ApplyGates, QubitRegister.h:493-497) and the QFT gate sequence
// (QuantumFourierTransform.h:35-87, QubitsSwapper.h:23-34).
#include <cmath>
#include <cstring>
#include <vector>

#include "batch.cuh"

namespace qcs {
namespace {

qcs_gate make_h(uint32_t q) {
	qcs_gate g;
	std::memset(&g, 0, sizeof(g));
	const double r2 = 1. / std::sqrt(2.);
	g.k = 1;
	g.q0 = q;
	g.m[0] = r2; g.m[2] = r2; g.m[4] = r2; g.m[6] = -r2;
	return g;
}

// ControlledPhaseShiftGate(phase) (QuantumGate.h:251-271) on (target, control)
qcs_gate make_cp(uint32_t target, uint32_t control, double phase) {
	qcs_gate g;
	std::memset(&g, 0, sizeof(g));
	g.k = 2;
	g.q0 = target;
	g.q1 = control;
	g.traits = QCS_TRAIT_CONTROLLED | QCS_TRAIT_DIAGONAL;
	for (int i = 0; i < 3; ++i) g.m[2 * (i * 4 + i)] = 1;
	g.m[2 * 15] = std::cos(phase);
	g.m[2 * 15 + 1] = std::sin(phase);
	return g;
}

qcs_gate make_swap(uint32_t a, uint32_t b) {
	qcs_gate g;
	std::memset(&g, 0, sizeof(g));
	g.k = 2;
	g.q0 = a;
	g.q1 = b;
	g.traits = QCS_TRAIT_SWAP;
	g.m[0] = 1; g.m[2 * (1 * 4 + 2)] = 1; g.m[2 * (2 * 4 + 1)] = 1; g.m[2 * 15] = 1;
	return g;
}

}  // namespace

int batch_apply(qcs_handle h, const qcs_gate* gates, size_t count) {
	for (size_t i = 0; i < count; ++i) {
		cudaError_t e = apply_one(h, gates[i]);
		if (e != cudaSuccess) {
			h->err = std::string("apply gates: ") + cudaGetErrorString(e);
			return QCS_CUDA_ERROR;
		}
	}
	return QCS_OK;
}

std::vector<qcs_gate> qft_gates(uint32_t start, uint32_t end, bool inverse, bool do_swap) {
	std::vector<qcs_gate> gs;
	const int sq = static_cast<int>(start), eq = static_cast<int>(end);
	auto swaps = [&]() {
		uint32_t a = start, b = end;
		while (a < b) gs.push_back(make_swap(a++, b--));
	};
	if (!inverse) {
		gs.push_back(make_h(eq));
		for (int cur = eq; cur > sq; --cur) {
			double phase = M_PI_2;
			for (int c = cur - 1; c >= sq; --c) {
				gs.push_back(make_cp(cur, c, phase));
				phase *= 0.5;
			}
			gs.push_back(make_h(cur - 1));
		}
		if (do_swap) swaps();
	} else {
		if (do_swap) swaps();
		for (int cur = sq + 1; cur <= eq; ++cur) {
			gs.push_back(make_h(cur - 1));
			double phase = -M_PI_2;
			for (int c = cur - 1; c >= sq; --c) {
				gs.push_back(make_cp(cur, c, phase));
				phase *= 0.5;
			}
		}
		gs.push_back(make_h(eq));
	}
	return gs;
}

int qft_apply(qcs_handle h, uint32_t start, uint32_t end, bool inverse, bool do_swap) {
	const std::vector<qcs_gate> gs = qft_gates(start, end, inverse, do_swap);
	return batch_apply(h, gs.data(), gs.size());
}

void batch_release(qcs_handle) {}

}  // namespace qcs
