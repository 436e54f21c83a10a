// Gate fusion for the FP32 path (see fusion.cuh).
#include <algorithm>
#include <cstring>

#include "fusion.cuh"

namespace qcs {
namespace {

using cd = std::complex<double>;

cd c2(const double2& v) { return cd(v.x, v.y); }

cd unit_of(double code) {
	switch (static_cast<int>(code) & 3) {
	case 0: return cd(1, 0);
	case 1: return cd(0, 1);
	case 2: return cd(-1, 0);
	default: return cd(0, -1);
	}
}

int local_bit(const std::vector<uint32_t>& qubits, uint32_t q) {
	for (size_t i = 0; i < qubits.size(); ++i)
		if (qubits[i] == q) return static_cast<int>(i);
	return -1;
}

int popc(uint64_t x) { return __builtin_popcountll(x); }

}  // namespace

void apply_compiled_local(const CompiledGate& c, const std::vector<uint32_t>& qubits, cd* v) {
	const uint32_t D = 1u << qubits.size();
	uint32_t cmask = 0;
	for (uint32_t i = 0; i < c.ncontrols; ++i) cmask |= 1u << local_bit(qubits, c.controls[i]);
	if (c.kind == GKind::Ctrl1q) {
		const uint32_t tb = 1u << local_bit(qubits, c.target);
		const Mat2<double>& m = c.m;
		for (uint32_t i = 0; i < D; ++i) {
			if ((i & tb) || (i & cmask) != cmask) continue;
			cd& a0 = v[i];
			cd& a1 = v[i | tb];
			const cd x0 = a0, x1 = a1;
			switch (c.op) {
			case Op1::Diag: a0 = x0 * c2(m.m00); a1 = x1 * c2(m.m11); break;
			case Op1::Phase: case Op1::PhaseNeg: case Op1::PhaseI:
				if (c.phase_on_a0) a0 = x0 * c2(m.m11);
				else a1 = x1 * c2(m.m11);
				break;
			case Op1::Antidiag: a0 = c2(m.m01) * x1; a1 = c2(m.m10) * x0; break;
			case Op1::AntidiagUnit: a0 = unit_of(m.m01.x) * x1; a1 = unit_of(m.m10.x) * x0; break;
			case Op1::Swap: a0 = x1; a1 = x0; break;
			case Op1::UnitRe01: a0 = m.m00.x * x0 + m.m00.y * x1; a1 = m.m01.x * x1 + m.m01.y * x0; break;
			case Op1::UnitRe10: a0 = m.m00.x * x1 + m.m00.y * x0; a1 = m.m01.x * x0 + m.m01.y * x1; break;
			case Op1::UnitIm01: a0 = m.m00.x * x0 + cd(0, m.m00.y) * x1; a1 = m.m01.x * x1 + cd(0, m.m01.y) * x0; break;
			case Op1::UnitIm10: a0 = m.m00.x * x1 + cd(0, m.m00.y) * x0; a1 = m.m01.x * x0 + cd(0, m.m01.y) * x1; break;
			default: a0 = c2(m.m00) * x0 + c2(m.m01) * x1; a1 = c2(m.m10) * x0 + c2(m.m11) * x1; break;
			}
		}
	} else if (c.kind == GKind::Swap) {
		const uint32_t ba = 1u << local_bit(qubits, c.qa), bb = 1u << local_bit(qubits, c.qb);
		const cd f = c.sk == SwapKind::Plain ? cd(1, 0) : (c.sk == SwapKind::ISwap ? cd(0, 1) : cd(0, -1));
		for (uint32_t i = 0; i < D; ++i) {
			if ((i & (ba | bb)) != ba || (i & cmask) != cmask) continue;
			const uint32_t o = i ^ (ba | bb);
			const cd t = v[i];
			v[i] = f * v[o];
			v[o] = f * t;
		}
	} else if (c.kind == GKind::Dense) {
		const int k = c.dense_k;
		const uint32_t d = 1u << k;
		uint32_t bits[3] = {0, 0, 0}, all = 0;
		for (int j = 0; j < k; ++j) {
			bits[j] = 1u << local_bit(qubits, c.dense_q[j]);
			all |= bits[j];
		}
		for (uint32_t i = 0; i < D; ++i) {
			if ((i & all) || (i & cmask) != cmask) continue;
			cd in[8], outv[8];
			uint32_t idx[8];
			for (uint32_t r = 0; r < d; ++r) {
				uint32_t x = i;
				for (int j = 0; j < k; ++j)
					if ((r >> j) & 1u) x |= bits[j];
				idx[r] = x;
				in[r] = v[x];
			}
			for (uint32_t r = 0; r < d; ++r) {
				cd acc(0, 0);
				for (uint32_t cc = 0; cc < d; ++cc) acc += cd(c.dense_m[2 * (r * d + cc)], c.dense_m[2 * (r * d + cc) + 1]) * in[cc];
				outv[r] = acc;
			}
			for (uint32_t r = 0; r < d; ++r) v[idx[r]] = outv[r];
		}
	}
	if (c.scale != cd(1, 0))
		for (uint32_t i = 0; i < D; ++i) v[i] *= c.scale;
}

namespace {

struct Open {
	uint64_t mask = 0;
	std::vector<const CompiledGate*> gates;
};

FusedBlock build(const Open& o) {
	FusedBlock b;
	for (int q = 0; q < 64; ++q)
		if ((o.mask >> q) & 1ULL) b.qubits.push_back(static_cast<uint32_t>(q));
	const uint32_t D = 1u << b.qubits.size();
	b.M.assign(static_cast<size_t>(D) * D, cd(0, 0));
	std::vector<cd> col(D);
	for (uint32_t j = 0; j < D; ++j) {
		std::fill(col.begin(), col.end(), cd(0, 0));
		col[j] = 1;
		for (const CompiledGate* g : o.gates) apply_compiled_local(*g, b.qubits, col.data());
		for (uint32_t r = 0; r < D; ++r) b.M[static_cast<size_t>(r) * D + j] = col[r];
	}
	b.ngates = static_cast<uint32_t>(o.gates.size());
	return b;
}

double block_cost(const FusionPolicy& p, uint64_t mask, size_t ngates) {
	std::vector<uint32_t> q;
	for (int i = 0; i < 64; ++i)
		if ((mask >> i) & 1ULL) q.push_back(static_cast<uint32_t>(i));
	return p.cost(q, static_cast<uint32_t>(ngates), p.nqubits, p.ctx);
}

}  // namespace

std::vector<FusedBlock> fuse(const std::vector<CompiledGate>& gates, const FusionPolicy& policy) {
	std::vector<FusedBlock> out;
	std::vector<Open> open;
	const int maxq = std::max(1, std::min(policy.max_qubits, 5));
	auto close_at = [&](size_t i) {
		out.push_back(build(open[i]));
		open.erase(open.begin() + static_cast<long>(i));
	};
	for (const CompiledGate& g : gates) {
		const uint64_t q = g.touch_mask();
		if (q == 0) {  // an identity that only carries a global factor: fold into any block
			if (open.empty()) open.emplace_back();
			open.back().gates.push_back(&g);
			continue;
		}
		std::vector<size_t> inter;
		uint64_t uni = q;
		for (size_t i = 0; i < open.size(); ++i)
			if (open[i].mask & q) {
				inter.push_back(i);
				uni |= open[i].mask;
			}
		if (!inter.empty() && popc(uni) <= maxq) {
			bool take = true;
			if (policy.cost && inter.size() > 1) {
				// merging blocks that a gate spans: accept when the merged block is predicted cheaper
				double sep = 0;
				size_t ng = 1;
				for (size_t i : inter) {
					sep += block_cost(policy, open[i].mask, open[i].gates.size());
					ng += open[i].gates.size();
				}
				take = block_cost(policy, uni, ng) <= sep + block_cost(policy, q, 1);
			}
			if (take) {
				Open merged;
				merged.mask = uni;
				for (size_t i : inter)
					for (const CompiledGate* x : open[i].gates) merged.gates.push_back(x);
				merged.gates.push_back(&g);
				for (size_t k = inter.size(); k-- > 0;) open.erase(open.begin() + static_cast<long>(inter[k]));
				open.push_back(std::move(merged));
				continue;
			}
		}
		// the gate cannot join: close the blocks it touches, in creation order
		std::sort(inter.begin(), inter.end());
		for (size_t k = 0; k < inter.size(); ++k) close_at(inter[k] - k);
		// join an open block with room (the fullest), else start one
		int best = -1;
		for (size_t i = 0; i < open.size(); ++i) {
			if (popc(open[i].mask | q) > maxq) continue;
			if (policy.cost) {
				const double joined = block_cost(policy, open[i].mask | q, open[i].gates.size() + 1);
				const double apart = block_cost(policy, open[i].mask, open[i].gates.size()) + block_cost(policy, q, 1);
				if (joined > apart) continue;
			}
			if (best < 0 || popc(open[i].mask) > popc(open[static_cast<size_t>(best)].mask)) best = static_cast<int>(i);
		}
		if (best >= 0) {
			open[static_cast<size_t>(best)].mask |= q;
			open[static_cast<size_t>(best)].gates.push_back(&g);
		} else {
			Open o;
			o.mask = q;
			o.gates.push_back(&g);
			open.push_back(std::move(o));
		}
	}
	while (!open.empty()) close_at(0);
	return out;
}

std::vector<std::vector<size_t>> pack_blocks(const std::vector<FusedBlock>& blocks, int kmax, int L0, uint32_t tc_budget,
                                             size_t window) {
	std::vector<std::vector<size_t>> passes;
	std::vector<char> placed(blocks.size(), 0);
	std::vector<uint64_t> mask(blocks.size(), 0);
	std::vector<uint32_t> tcb(blocks.size(), 0);
	size_t first = 0;  // first block not yet placed
	for (size_t i = 0; i < blocks.size(); ++i) {
		for (uint32_t q : blocks[i].qubits) mask[i] |= 1ULL << q;
		if (blocks[i].qubits.empty()) placed[i] = 1;
		// tensor-core passes widen smaller blocks to 4 qubits
		if (tc_budget && !blocks[i].qubits.empty()) tcb[i] = 32u << (2 * std::max<size_t>(4, blocks[i].qubits.size()));
	}
	const uint64_t low = (L0 >= 64) ? ~0ULL : ((1ULL << L0) - 1);
	while (true) {
		while (first < blocks.size() && placed[first]) ++first;
		if (first == blocks.size()) break;
		std::vector<size_t> pass;
		uint64_t tmask = low, waiting = 0;
		uint32_t bytes = 0;
		size_t scanned = 0;
		for (size_t i = first; i < blocks.size() && scanned < window; ++i) {
			if (placed[i]) continue;
			++scanned;
			const bool fits = __builtin_popcountll(tmask | mask[i]) <= kmax && (!tc_budget || bytes + tcb[i] <= tc_budget);
			if ((mask[i] & waiting) == 0 && (fits || pass.empty())) {
				placed[i] = 1;
				pass.push_back(i);
				tmask |= mask[i];
				bytes += tcb[i];
			} else {
				waiting |= mask[i];
			}
		}
		passes.push_back(std::move(pass));
	}
	return passes;
}

}  // namespace qcs
