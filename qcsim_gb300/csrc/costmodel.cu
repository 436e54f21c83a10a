// The learned partition choice of the FP32 path and the dense k-qubit operator entry point.
//
// A fused block's features (its width, gate count, qubit positions, register size) feed the MLP of
// mlp.cu, which predicts the log of the block's marginal device time inside a shared-memory pass (a
// tensor-core pass for blocks of 4 and 5 qubits, a CUDA-core pass for smaller ones).  A candidate
// partition (the greedy fuser run with a given largest block) is scored as
//   sum over blocks of exp(prediction) + passes x (time of one streaming pass over the register),
// a candidate on the tensor cores scoring its smaller blocks as the 4-qubit blocks they are widened to,
// and the cheapest candidate is applied.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "compile.cuh"
#include "fusion.cuh"
#include "tile.cuh"

namespace qcs {

constexpr int kFeatures = 13;

// the feature vector of a block (qubits ascending); shared by training and inference
void block_features(int n, const uint32_t* q, uint32_t m, uint32_t ngates, float* f) {
	std::memset(f, 0, sizeof(float) * kFeatures);
	uint32_t low = 0, top = 0;
	for (uint32_t j = 0; j < m; ++j) {
		if (q[j] < 5) ++low;
		if (static_cast<int>(q[j]) >= n - 3) ++top;
	}
	f[0] = static_cast<float>(m) / 5.f;
	f[1] = static_cast<float>(std::min<uint32_t>(ngates, 64)) / 32.f;
	f[2] = static_cast<float>(n) / 32.f;
	f[3] = m ? static_cast<float>(q[0]) / 32.f : 0.f;
	f[4] = m ? static_cast<float>(q[m - 1]) / 32.f : 0.f;
	f[5] = static_cast<float>(low) / 5.f;
	f[6] = static_cast<float>(top) / 5.f;
	f[7] = m ? static_cast<float>(q[m - 1] - q[0]) / 32.f : 0.f;
	if (m >= 1 && m <= 5) f[7 + m] = 1.f;  // one-hot width 1..5 at 8..12
}

struct CostModel {
	qcs_mlp_handle mlp = nullptr;
	std::vector<double> pass_ms;  // index: register qubits (entries 64 + n, when given: a tensor-core pass, not used)
};

// passes the planner forms for these blocks (the packing of apply_blocks)
static int count_passes(const std::vector<FusedBlock>& blocks, int kmax, int L0, bool tc) {
	return static_cast<int>(pack_blocks(blocks, kmax, L0, tc ? kTcMatBudget : 0u).size());
}

int choose_partition(qcs_handle h, const std::vector<CompiledGate>& gates, int kmax, int L0, std::vector<FusedBlock>& best,
                     double* predicted_ms) {
	auto* cm = static_cast<CostModel*>(h->cost_ctx);
	const int n = static_cast<int>(h->n);
	const int top = std::min(h->fusion_limit(), h->prec == QCS_FP64 ? 4 : 5);
	double best_cost = 1e300;
	for (int mq = 1; mq <= top; ++mq) {
		FusionPolicy pol;
		pol.max_qubits = mq;
		pol.nqubits = n;
		std::vector<FusedBlock> cand = fuse(gates, pol);
		bool big = false;
		for (const FusedBlock& b : cand) big = big || b.qubits.size() >= 4;
		const bool tc = h->prec == QCS_FP32 && h->tensor_cores && big && n >= kTcTileQubits;
		std::vector<float> x(cand.size() * kFeatures);
		for (size_t i = 0; i < cand.size(); ++i) {
			// in tensor-core passes a smaller block runs widened to 4 qubits (the lowest ones it lacks)
			std::vector<uint32_t> q = cand[i].qubits;
			if (tc && !q.empty())
				for (uint32_t b = 0; q.size() < 4 && b < static_cast<uint32_t>(n); ++b)
					if (std::find(q.begin(), q.end(), b) == q.end()) q.push_back(b);
			std::sort(q.begin(), q.end());
			block_features(n, q.data(), static_cast<uint32_t>(q.size()), cand[i].ngates, &x[i * kFeatures]);
		}
		std::vector<float> y(cand.size());
		if (!cand.empty()) {
			const int st = qcs_mlp_predict(cm->mlp, x.data(), static_cast<int>(cand.size()), y.data());
			if (st != QCS_OK) return st;
		}
		double cost = 0;
		for (float v : y) cost += std::exp(static_cast<double>(v));
		// every block's predicted cost is its whole cost beyond one streaming pass over the register, so the
		// pass term is the CUDA-core pass time for both kinds of candidate
		const double pms = static_cast<size_t>(n) < cm->pass_ms.size() ? cm->pass_ms[static_cast<size_t>(n)] : 0.0;
		cost += pms * count_passes(cand, tc ? std::min(kmax, kTcTileQubits) : kmax, L0, tc);
		if (cost < best_cost) {
			best_cost = cost;
			best = std::move(cand);
		}
	}
	if (predicted_ms) *predicted_ms = best_cost;
	return QCS_OK;
}

void release_cost_model(qcs_handle h) {
	delete static_cast<CostModel*>(h->cost_ctx);
	h->cost_ctx = nullptr;
}

}  // namespace qcs

extern "C" {

int qcs_block_features(uint32_t nqubits, const uint32_t* qubits, uint32_t k, uint32_t ngates, float* out) {
	if (!qubits || !out || k > 5) return QCS_INVALID_ARGUMENT;
	qcs::block_features(static_cast<int>(nqubits), qubits, k, ngates, out);
	return QCS_OK;
}

int qcs_fusion_plan(uint32_t nqubits, const qcs_gate* gates, size_t count, int max_qubits, uint64_t* block_masks,
                    uint32_t* block_gates, size_t capacity, size_t* nblocks_out) {
	if ((!gates && count) || !nblocks_out || max_qubits < 1 || max_qubits > 5) return QCS_INVALID_ARGUMENT;
	std::vector<qcs::CompiledGate> cg;
	cg.reserve(count);
	for (size_t i = 0; i < count; ++i) {
		const qcs_gate& g = gates[i];
		if (g.k < 1 || g.k > 3 || g.q0 >= nqubits || (g.k > 1 && g.q1 >= nqubits) || (g.k > 2 && g.q2 >= nqubits))
			return QCS_INVALID_ARGUMENT;
		cg.push_back(qcs::compile_gate(g, false));
	}
	qcs::FusionPolicy pol;
	pol.max_qubits = max_qubits;
	pol.nqubits = static_cast<int>(nqubits);
	const std::vector<qcs::FusedBlock> blocks = qcs::fuse(cg, pol);
	size_t k = 0;
	for (const qcs::FusedBlock& b : blocks) {
		if (b.qubits.empty()) continue;
		if (k < capacity) {
			uint64_t m = 0;
			for (uint32_t q : b.qubits) m |= 1ULL << q;
			if (block_masks) block_masks[k] = m;
			if (block_gates) block_gates[k] = b.ngates;
		}
		++k;
	}
	*nblocks_out = k;
	return QCS_OK;
}

int qcs_fusion_passes(uint32_t nqubits, const qcs_gate* gates, size_t count, int max_qubits, int tile_qubits, int tensor_cores,
                      uint32_t* pass_of_block, size_t capacity, size_t* nblocks_out, size_t* npasses_out) {
	if ((!gates && count) || !nblocks_out || !npasses_out || max_qubits < 1 || max_qubits > 5 || tile_qubits < 5 || tile_qubits > 13)
		return QCS_INVALID_ARGUMENT;
	std::vector<qcs::CompiledGate> cg;
	cg.reserve(count);
	for (size_t i = 0; i < count; ++i) {
		const qcs_gate& g = gates[i];
		if (g.k < 1 || g.k > 3 || g.q0 >= nqubits || (g.k > 1 && g.q1 >= nqubits) || (g.k > 2 && g.q2 >= nqubits))
			return QCS_INVALID_ARGUMENT;
		cg.push_back(qcs::compile_gate(g, false));
	}
	qcs::FusionPolicy pol;
	pol.max_qubits = max_qubits;
	pol.nqubits = static_cast<int>(nqubits);
	std::vector<qcs::FusedBlock> blocks = qcs::fuse(cg, pol);
	// the numbering of qcs_fusion_plan: blocks with qubits only
	std::vector<qcs::FusedBlock> real;
	for (qcs::FusedBlock& b : blocks)
		if (!b.qubits.empty()) real.push_back(std::move(b));
	const int kmax = std::min(tile_qubits, static_cast<int>(nqubits));
	const int L0 = qcs::low_run_qubits(static_cast<int>(nqubits), kmax);
	const auto passes = qcs::pack_blocks(real, kmax, L0, tensor_cores ? qcs::kTcMatBudget : 0u);
	if (pass_of_block)
		for (size_t p = 0; p < passes.size(); ++p)
			for (size_t i : passes[p])
				if (i < capacity) pass_of_block[i] = static_cast<uint32_t>(p);
	*nblocks_out = real.size();
	*npasses_out = passes.size();
	return QCS_OK;
}

int qcs_set_cost_model(qcs_handle h, qcs_mlp_handle mlp, const double* pass_ms, size_t len) {
	if (!h) return QCS_INVALID_ARGUMENT;
	auto* cm = static_cast<qcs::CostModel*>(h->cost_ctx);
	if (!mlp) {
		delete cm;
		h->cost_ctx = nullptr;
		return QCS_OK;
	}
	if (!cm) cm = new qcs::CostModel;
	cm->mlp = mlp;
	cm->pass_ms.assign(pass_ms, pass_ms + len);
	h->cost_ctx = cm;
	return QCS_OK;
}

// dense 2^k x 2^k operator on the given qubits (ascending matrix bits: qubits[j] is matrix bit j),
// applied as one fused block in a shared-memory pass
int qcs_apply_matrix(qcs_handle h, const uint32_t* qubits, uint32_t k, const double* m) {
	if (!h || !qubits || !m || k < 1) return QCS_INVALID_ARGUMENT;
	if (k > (h->prec == QCS_FP64 ? 4u : 5u)) {
		h->err = "dense operators act on at most 4 (FP64) or 5 (FP32) qubits";
		return QCS_UNSUPPORTED;
	}
	for (uint32_t i = 0; i < k; ++i) {
		if (qubits[i] >= h->n) {
			h->err = "Qubit number is too high";
			return QCS_INVALID_ARGUMENT;
		}
		for (uint32_t j = 0; j < i; ++j)
			if (qubits[i] == qubits[j]) {
				h->err = "Qubits must be different";
				return QCS_INVALID_ARGUMENT;
			}
	}
	// reorder the matrix bits so the qubits ascend
	std::vector<uint32_t> perm(k);
	for (uint32_t i = 0; i < k; ++i) perm[i] = i;
	std::sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return qubits[a] < qubits[b]; });
	const uint32_t D = 1u << k;
	auto remap = [&](uint32_t r) {  // index in ascending order -> index in the caller's bit order
		uint32_t o = 0;
		for (uint32_t j = 0; j < k; ++j)
			if ((r >> j) & 1u) o |= 1u << perm[j];
		return o;
	};
	qcs::FusedBlock b;
	for (uint32_t j = 0; j < k; ++j) b.qubits.push_back(qubits[perm[j]]);
	b.M.resize(static_cast<size_t>(D) * D);
	for (uint32_t r = 0; r < D; ++r)
		for (uint32_t c = 0; c < D; ++c) {
			const size_t src = (static_cast<size_t>(remap(r)) * D + remap(c)) * 2;
			b.M[static_cast<size_t>(r) * D + c] = std::complex<double>(m[src], m[src + 1]);
		}
	b.ngates = 1;
	return qcs::apply_blocks(h, std::vector<qcs::FusedBlock>{b});
}

}  // extern "C"
