// Gate-list execution (ApplyGates, QubitRegister.h:493-497) and the QFT gate sequence
// (QuantumFourierTransform.h:35-87, QubitsSwapper.h:23-34).
//
// The planner walks the gate list in order and packs consecutive gates into shared-memory passes:
// a gate joins the open pass when the qubits it must hold locally (targets of non-diagonal blocks;
// controls and diagonal targets never need to be local) fit in the pass's tile.  Every gate keeps its
// own arithmetic and order, so results equal those of the per-gate kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "batch.cuh"
#include "compile.cuh"
#include "fusion.cuh"
#include "tcgen05.cuh"
#include "tile.cuh"

namespace qcs {
namespace {

int fail_cuda(qcs_handle h, cudaError_t e, const char* where) {
	h->err = std::string(where) + ": " + cudaGetErrorString(e);
	return QCS_CUDA_ERROR;
}

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

struct PlannedPass {
	uint64_t tmask = 0;
	std::vector<CompiledGate> gates;
	std::complex<double> fold_after{1.0, 0.0};  // scale folded into the amplitudes after this pass
};

int popcount64(uint64_t x) { return __builtin_popcountll(x); }

// device buffers of the planner, per register
struct BatchBuffers {
	void* d_ops = nullptr;
	size_t ops_cap = 0;
	void* d_mats = nullptr;
	size_t mats_cap = 0;
	int* d_err = nullptr;     // status word of the tensor-core passes
	void* d_roots = nullptr;  // all 2^roots_M-th roots of unity for the phase rows (0: none built)
	uint32_t roots_M = 0;
};

// phase rows of at most kRootsM - 1 bits read their root from one table of 2^kRootsM entries (4 FP64
// operations per amplitude fewer than combining two factors); 2^24 complex doubles = 256 MiB
constexpr uint32_t kRootsM = 24;

// QFT rows narrower than this stay individual controlled phases (a row costs one or two complex products
// on half the amplitudes; a controlled phase one product on a quarter)
constexpr uint32_t kMinRowBits = 5;

cudaError_t ensure(void** p, size_t* cap, size_t bytes) {
	if (*cap >= bytes) return cudaSuccess;
	if (*p) cudaFree(*p);
	*p = nullptr;
	*cap = 0;
	cudaError_t e = cudaMalloc(p, bytes);
	if (e == cudaSuccess) *cap = bytes;
	return e;
}

template <typename T> cplx_t<T> mk_host(double re, double im) {
	cplx_t<T> c;
	c.x = static_cast<T>(re);
	c.y = static_cast<T>(im);
	return c;
}

template <typename T> void push_mat2(std::vector<cplx_t<T>>& mats, const Mat2<double>& m) {
	const double2 v[4] = {m.m00, m.m01, m.m10, m.m11};
	for (const double2& x : v) {
		cplx_t<T> c;
		c.x = static_cast<T>(x.x);
		c.y = static_cast<T>(x.y);
		mats.push_back(c);
	}
}

// round to TF32 (10 mantissa bits), to nearest with ties away from zero, as cvt.rna.tf32.f32
float tf32_rna_host(float x) {
	uint32_t u;
	std::memcpy(&u, &x, 4);
	u = (u + 0x1000u) & 0xFFFFE000u;
	float r;
	std::memcpy(&r, &u, 4);
	return r;
}

// a fused block's real-expanded matrix B (2D x 2D, B[2j + p][2i + q]; see the tensor-core pass kernel)
// as the MMA's B operand: rows = outputs 2i + q, K = inputs 2j + p, K-major; TF32 hi split then lo
void push_block_tc(std::vector<float2>& mats, const std::vector<std::complex<double>>& M, uint32_t D) {
	const uint32_t kdim = 2 * D, split = 4 * D * D;  // floats per split (16 D^2 bytes)
	if (mats.size() & 1) mats.push_back(make_float2(0.f, 0.f));  // 16-byte alignment of the block
	std::vector<float> f(2 * split, 0.f);
	for (uint32_t i = 0; i < D; ++i)
		for (uint32_t j = 0; j < D; ++j) {
			const double re = M[static_cast<size_t>(i) * D + j].real(), im = M[static_cast<size_t>(i) * D + j].imag();
			const double e[2][2] = {{re, im}, {-im, re}};  // [p][q]: input part p -> output part q
			for (uint32_t pi = 0; pi < 2; ++pi)
				for (uint32_t qo = 0; qo < 2; ++qo) {
					const double x = e[pi][qo];
					const float hi = tf32_rna_host(static_cast<float>(x));
					const float lo = tf32_rna_host(static_cast<float>(x - static_cast<double>(hi)));
					const uint32_t off = tc::kmajor_offset(2 * i + qo, 2 * j + pi, kdim) / 4;
					f[off] = hi;
					f[split + off] = lo;
				}
		}
	for (size_t k = 0; k < f.size(); k += 2) mats.push_back(make_float2(f[k], f[k + 1]));
}

// a fused block on fewer than 4 tile positions, widened to 4 by the lowest tile positions it does not
// use (identity on them), for the tensor-core pass; pos becomes the ascending positions of the result,
// and the returned matrix has bit t <-> pos[t]
std::vector<std::complex<double>> pad_block(std::vector<int>& pos, const std::vector<std::complex<double>>& M, int k) {
	std::vector<int> all = pos;
	for (int b = 0; b < k && all.size() < 4; ++b)
		if (std::find(all.begin(), all.end(), b) == all.end()) all.push_back(b);
	std::sort(all.begin(), all.end());
	const uint32_t d = 1u << pos.size();
	std::vector<uint32_t> inner(all.size(), 0);  // bit t of the new index: bit of the old matrix, or 0 (extra)
	uint32_t extra = 0;
	for (size_t t = 0; t < all.size(); ++t) {
		const auto it = std::find(pos.begin(), pos.end(), all[t]);
		if (it != pos.end()) inner[t] = 1u << static_cast<uint32_t>(it - pos.begin());
		else extra |= 1u << t;
	}
	auto old_index = [&](uint32_t i) {
		uint32_t o = 0;
		for (size_t t = 0; t < all.size(); ++t)
			if ((i >> t) & 1u) o |= inner[t];
		return o;
	};
	const uint32_t D = 1u << all.size();
	std::vector<std::complex<double>> out(static_cast<size_t>(D) * D, 0.0);
	for (uint32_t i = 0; i < D; ++i)
		for (uint32_t j = 0; j < D; ++j)
			if ((i & extra) == (j & extra)) out[static_cast<size_t>(i) * D + j] = M[static_cast<size_t>(old_index(i)) * d + old_index(j)];
	pos = all;
	return out;
}

// the tile bits outside a tensor-core block, in the order that makes up the row (tensor-memory lane)
// index: first four whose swizzled offsets differ in independent low-four-bit vectors (conflict-free
// gathers, tc_swizzle), then the rest ascending; packed 4 bits each, row bit r in bits 4r..4r+3
uint64_t tc_row_order(uint32_t insmask) {
	std::vector<int> first, rest;
	uint32_t basis[4] = {0, 0, 0, 0};  // reduced vectors by leading bit
	for (int b = 0; b < kTcTileQubits; ++b) {
		if ((insmask >> b) & 1u) continue;
		uint32_t v = tc_bit_offset(b) & 15u;
		for (int l = 3; l >= 0; --l)
			if (((v >> l) & 1u) && basis[l]) v ^= basis[l];
		if (first.size() < 4 && v) {
			int l = 3;
			while (!((v >> l) & 1u)) --l;
			basis[l] = v;
			first.push_back(b);
		} else {
			rest.push_back(b);
		}
	}
	first.insert(first.end(), rest.begin(), rest.end());
	uint64_t packed = 0;
	for (size_t r = 0; r < first.size(); ++r) packed |= static_cast<uint64_t>(first[r]) << (4 * r);
	return packed;
}

// host check of one tile operation: inserted positions strictly ascending and below k, the bits it
// reads or forces inside the inserted set, its matrix entries inside the table
bool op_in_bounds(const TileOp& op, int k, size_t mats) {
	if (op.nins > 8 || static_cast<int>(op.nins) > k) return false;
	uint32_t insmask = 0;
	int prev = -1;
	for (int j = 0; j < op.nins; ++j) {
		const int b = static_cast<int>((op.ins >> (8 * j)) & 0xffu);
		if (b <= prev || b >= k) return false;
		prev = b;
		insmask |= 1u << b;
	}
	if ((op.lset & ~insmask) != 0) return false;
	if (static_cast<TKind>(op.kind) == TKind::DenseTC) {
		const uint32_t D = 1u << op.nins;
		if (k != kTcTileQubits || op.nins < 4 || op.nins > 5 || op.lset != 0 || op.lbit0 != 0 || op.lbit2 != 0 || (op.mat & 1u) ||
		    (op.lbit1 & 15u) || op.lbit1 + 32 * D * D > kTcMatBudget || op.gmask != 0)
			return false;
		// the row order: every tile bit outside the block exactly once
		uint32_t rows = 0;
		for (int r = 0; r < kTcTileQubits - op.nins; ++r) rows |= 1u << ((op.gtbit >> (4 * r)) & 15u);
		if (rows != (((1u << kTcTileQubits) - 1) & ~insmask) || (op.gtbit >> (4 * (kTcTileQubits - op.nins))) != 0) return false;
		return op.mat + size_t(4) * D * D <= mats;
	}
	if (static_cast<TKind>(op.kind) == TKind::TileFactor)  // one scalar per tile: entries mat and mat + 1
		return op.nins == 0 && op.lset == 0 && op.gtbit != 0 && (op.gtbit & (op.gtbit - 1)) == 0 && op.mat + 2 <= mats;
	if (static_cast<TKind>(op.kind) == TKind::TableDiag)  // every amplitude of the tile, from the table at gtbit
		return op.nins == 0 && op.lset == 0 && op.gmask == 0 && op.gtbit != 0 && (op.gtbit & 15u) == 0;
	if (static_cast<TKind>(op.kind) == TKind::PhaseRow) {
		// lbit1 / lbit2 hold the row's first bit and width; the table covers every z = y << shift
		const uint32_t shift = op.pad[0], S = op.pad[1], M = op.pad[3];
		if (op.nins > 1 || op.lbit0 != 0 || M < 1 || M > 40 || S > M || op.lbit1 + op.lbit2 > 64 || op.lbit2 + shift > M)
			return false;
		if (op.pad[4]) return M <= kRootsM && op.gtbit != 0 && (op.gtbit & 15u) == 0;  // the full table: 2^M entries
		return op.mat + (size_t(1) << (M - S)) + (size_t(1) << S) <= mats;
	}
	const bool flag0 = static_cast<TKind>(op.kind) == TKind::GlobalDiag;  // lbit0 is a side flag there
	for (uint32_t bit : {flag0 ? 0u : op.lbit0, op.lbit1, op.lbit2})
		if ((bit & ~insmask) != 0 || (bit & (bit - 1)) != 0) return false;
	size_t need = 0;
	switch (static_cast<TKind>(op.kind)) {
	case TKind::Ctrl1q: case TKind::GlobalDiag: need = 4; break;
	case TKind::Swap: need = 0; break;
	case TKind::Dense2: need = 16; break;
	case TKind::Dense3: need = 64; break;
	case TKind::DenseN: need = size_t(1) << (2 * op.nins); break;
	default: return false;
	}
	return op.mat + need <= mats;
}

// floating-point instructions (FMA, multiply or add: one each) that one work item of a pass operation
// issues, read off the forms in gate_math.cuh and tile_kernels.cu; tensor-core blocks count 0 here
// (their products run on the tensor pipe)
double fp_ops_per_item(const TileOp& op) {
	const TKind kind = static_cast<TKind>(op.kind);
	if (kind == TKind::Ctrl1q || kind == TKind::GlobalDiag) {
		switch (static_cast<Op1>(op.op)) {
		case Op1::Diag: return kind == TKind::GlobalDiag ? 4 : 8;  // one or two complex products
		case Op1::Phase: return 4;
		case Op1::PhaseI: return 2;
		case Op1::Antidiag: case Op1::Real: case Op1::RxLike: return 8;
		case Op1::Generic: return 16;
		case Op1::UnitRe01: case Op1::UnitRe10: case Op1::UnitIm01: case Op1::UnitIm10: return 4;
		default: return 0;  // sign flips, unit factors and moves
		}
	}
	switch (kind) {
	case TKind::PhaseRow: return op.pad[4] ? 4 : 8;  // the root from the full table or from two factors, then the product
	case TKind::TableDiag: return 4;  // one complex product
	case TKind::Dense2: return 4 * 16;
	case TKind::Dense3: return 4 * 64;
	case TKind::DenseN: return 4.0 * static_cast<double>(1u << (2 * op.nins));
	default: return 0;
	}
}

// a pass's floating-point instructions: per operation, work items per tile x tiles it runs in
// (non-tile controls halve the tiles each; a non-tile phase target runs in half of them)
double pass_fp_ops(const TilePass& tp, const std::vector<TileOp>& ops, int n) {
	double total = 0;
	if (tp.nfactor) {
		// the TileFactor product multiplies the tiles where it is not one (one complex product per amplitude);
		// the fraction of such tiles is estimated as if the operations' bits were independent
		double one = 1.0;
		for (uint32_t i = tp.op_begin; i < tp.op_begin + tp.nfactor; ++i) {
			const TileOp& op = ops[i];
			const double applies = std::ldexp(1.0, -popcount64(op.gmask));
			const bool both = op.pad[0] != 0;  // a diagonal with two non-unit entries
			one *= 1.0 - applies * (both ? 1.0 : 0.5);
		}
		total += 4.0 * std::ldexp(1.0, n) * (1.0 - one);
	}
	for (uint32_t i = tp.op_begin; i < tp.op_begin + tp.op_count; ++i) {
		const TileOp& op = ops[i];
		double tiles = std::ldexp(1.0, n - tp.k - popcount64(op.gmask));
		if (static_cast<TKind>(op.kind) == TKind::GlobalDiag && static_cast<Op1>(op.op) != Op1::Diag) tiles *= 0.5;
		total += tiles * static_cast<double>((1u << tp.k) >> op.nins) * fp_ops_per_item(op);
	}
	return total;
}

// the tiles, operations and matrix table of planned passes, before any device buffer is touched
template <typename T>
struct PassOps {
	std::vector<TilePass> tps;
	std::vector<TileOp> ops;
	std::vector<cplx_t<T>> mats;
	uint32_t rowM = 0;  // QFT phase rows: bits of the widest row's table of roots, 0 without rows
};

// builds the passes' operations for a register of n qubits (host only); tensor-core passes only where
// tensor_passes and tensor_cores are both set; false, with err set, on an internal error
template <typename T>
bool build_pass_ops(int n, bool tensor_cores, const std::vector<PlannedPass>& passes, int kmax, int L0, bool tensor_passes,
                    PassOps<T>& po, std::string& err) {
	std::vector<TilePass>& tps = po.tps;
	std::vector<TileOp>& ops = po.ops;
	std::vector<cplx_t<T>>& mats = po.mats;
	// QFT phase rows share one pair of tables of 2^M-th roots of unity: hi[u] = w^(u 2^S), lo[v] = w^v
	uint32_t& rowM = po.rowM;
	uint32_t rowS = 0, row_tab = 0;
	for (const PlannedPass& pp : passes)
		for (const CompiledGate& c : pp.gates)
			if (c.kind == GKind::PhaseRow) rowM = std::max(rowM, c.row_bits + 1);
	if (rowM > 0) {
		rowS = (rowM + 1) / 2;
		row_tab = static_cast<uint32_t>(mats.size());
		const double two_pi = 2.0 * M_PI;
		for (uint64_t u = 0; u < (1ULL << (rowM - rowS)); ++u) {
			const double a = two_pi * std::ldexp(static_cast<double>(u), static_cast<int>(rowS) - static_cast<int>(rowM));
			mats.push_back(mk_host<T>(std::cos(a), std::sin(a)));
		}
		for (uint64_t v = 0; v < (1ULL << rowS); ++v) {
			const double a = two_pi * std::ldexp(static_cast<double>(v), -static_cast<int>(rowM));
			mats.push_back(mk_host<T>(std::cos(a), std::sin(a)));
		}
	}
	for (const PlannedPass& pp : passes) {
		// tile qubits: the required ones, completed from the bottom up to kmax
		uint64_t T_ = pp.tmask | ((1ULL << L0) - 1);
		for (int q = 0; q < n && popcount64(T_) < kmax; ++q) T_ |= 1ULL << q;
		TilePass tp;
		std::memset(&tp, 0, sizeof(tp));
		tp.k = popcount64(T_);
		int L = 0;
		while (L < n && ((T_ >> L) & 1ULL)) ++L;
		tp.L = L;
		int lpos[64];
		int nh = 0;
		for (int q = 0; q < n; ++q) {
			if (!((T_ >> q) & 1ULL)) continue;
			if (q < L) lpos[q] = q;
			else {
				lpos[q] = L + nh;
				tp.high[nh++] = static_cast<uint8_t>(q);
			}
		}
		int nf = 0;
		for (int q = 0; q < n; ++q)
			if (!((T_ >> q) & 1ULL)) tp.fixed[nf++] = static_cast<uint8_t>(q);
		tp.nfixed = nf;
		tp.op_begin = static_cast<uint32_t>(ops.size());
		uint32_t tc_slot = 0;  // bytes of resident block matrices used in this pass
		// a tensor-core pass: FP32, a fused gate list with a block of 4 or 5 qubits (apply_blocks), a 12-qubit
		// tile, and nothing but fused blocks (smaller ones are widened to 4 qubits); every operation of it
		// runs on the tensor cores
		bool tc_pass = tensor_passes && sizeof(T) == 4 && tensor_cores && tp.k == kTcTileQubits && L >= kMinLowRun && tp.k - L <= kMaxHigh &&
		               !pp.gates.empty();
		for (const CompiledGate& c : pp.gates) tc_pass = tc_pass && c.kind == GKind::Block && !c.block_q.empty();
		for (const CompiledGate& c : pp.gates) {
			TileOp op;
			std::memset(&op, 0, sizeof(op));
			std::vector<int> ins;
			for (uint32_t i = 0; i < c.ncontrols; ++i) {
				const uint32_t q = c.controls[i];
				if ((T_ >> q) & 1ULL) {
					op.lset |= 1u << lpos[q];
					ins.push_back(lpos[q]);
				} else {
					op.gmask |= 1ULL << q;
				}
			}
			op.mat = static_cast<uint32_t>(mats.size());
			if (c.kind == GKind::Ctrl1q) {
				op.op = static_cast<uint8_t>(c.op);
				push_mat2<T>(mats, c.m);
				if ((T_ >> c.target) & 1ULL) {
					op.kind = static_cast<uint8_t>(TKind::Ctrl1q);
					ins.push_back(lpos[c.target]);
					op.lbit0 = c.phase_on_a0 ? 0u : (1u << lpos[c.target]);
				} else {
					op.kind = static_cast<uint8_t>(TKind::GlobalDiag);
					op.gtbit = 1ULL << c.target;
					op.lbit0 = c.phase_on_a0 ? 0u : 1u;
				}
			} else if (c.kind == GKind::Swap) {
				op.kind = static_cast<uint8_t>(TKind::Swap);
				op.op = static_cast<uint8_t>(c.sk);
				ins.push_back(lpos[c.qa]);
				ins.push_back(lpos[c.qb]);
				op.lbit0 = 1u << lpos[c.qa];
				op.lbit1 = 1u << lpos[c.qb];
			} else if (c.kind == GKind::Dense) {
				op.kind = static_cast<uint8_t>(c.dense_k == 2 ? TKind::Dense2 : TKind::Dense3);
				const uint32_t lb[3] = {c.dense_k > 0 ? 1u << lpos[c.dense_q[0]] : 0u, c.dense_k > 1 ? 1u << lpos[c.dense_q[1]] : 0u,
				                        c.dense_k > 2 ? 1u << lpos[c.dense_q[2]] : 0u};
				op.lbit0 = lb[0];
				op.lbit1 = lb[1];
				op.lbit2 = lb[2];
				for (int j = 0; j < c.dense_k; ++j) ins.push_back(lpos[c.dense_q[j]]);
				const int D = 1 << c.dense_k;
				for (int i = 0; i < D * D; ++i) {
					cplx_t<T> v;
					v.x = static_cast<T>(c.dense_m[2 * i]);
					v.y = static_cast<T>(c.dense_m[2 * i + 1]);
					mats.push_back(v);
				}
			} else if (c.kind == GKind::PhaseRow) {
				op.kind = static_cast<uint8_t>(TKind::PhaseRow);
				if ((T_ >> c.target) & 1ULL) {
					op.lset |= 1u << lpos[c.target];
					ins.push_back(lpos[c.target]);
				} else {
					op.gmask |= 1ULL << c.target;
				}
				op.lbit1 = c.row_lo;
				op.lbit2 = c.row_bits;
				op.pad[0] = static_cast<uint8_t>(rowM - 1 - c.row_bits);
				op.pad[1] = static_cast<uint8_t>(rowS);
				op.pad[2] = c.row_inverse ? 1 : 0;
				op.pad[3] = static_cast<uint8_t>(rowM);
				op.mat = row_tab;
			} else if (c.kind == GKind::Block && tc_pass) {
				if constexpr (sizeof(T) == 4) {
					std::vector<int> pos;
					for (uint32_t q : c.block_q) pos.push_back(lpos[q]);
					std::vector<std::complex<double>> M = c.block_m;
					if (pos.size() < 4) M = pad_block(pos, M, tp.k);
					const uint32_t K = static_cast<uint32_t>(pos.size());
					if (tc_slot + 32u * (1u << (2 * K)) > kTcMatBudget) {
						err = "apply gates: internal error (tensor-core pass over its matrix budget)";
						return false;
					}
					op.kind = static_cast<uint8_t>(TKind::DenseTC);
					uint32_t insmask = 0;
					for (int b : pos) {
						ins.push_back(b);
						insmask |= 1u << b;
					}
					op.gtbit = tc_row_order(insmask);
					if (mats.size() & 1) mats.push_back(mk_host<T>(0.0, 0.0));
					op.mat = static_cast<uint32_t>(mats.size());
					push_block_tc(mats, M, 1u << K);
					op.lbit1 = tc_slot;
					tc_slot += 32u * (1u << (2 * K));
					tp.dense = 2;
				}
			} else if (c.kind == GKind::TableDiag) {
				op.kind = static_cast<uint8_t>(TKind::TableDiag);
				op.gtbit = reinterpret_cast<uint64_t>(c.table);
			} else if (c.kind == GKind::Block) {
				op.kind = static_cast<uint8_t>(TKind::DenseN);
				for (uint32_t q : c.block_q) ins.push_back(lpos[q]);
				for (const std::complex<double>& x : c.block_m) {
					cplx_t<T> v;
					v.x = static_cast<T>(x.real());
					v.y = static_cast<T>(x.imag());
					mats.push_back(v);
				}
			} else {
				continue;
			}
			if ((op.kind == static_cast<uint8_t>(TKind::Dense2) || op.kind == static_cast<uint8_t>(TKind::Dense3) ||
			     op.kind == static_cast<uint8_t>(TKind::DenseN)) && tp.dense == 0)
				tp.dense = 1;
			std::sort(ins.begin(), ins.end());
			op.nins = static_cast<uint8_t>(ins.size());
			for (size_t i = 0; i < ins.size(); ++i) op.ins |= static_cast<uint64_t>(ins[i]) << (8 * i);
			ops.push_back(op);
		}
		// diagonal gates whose target and controls all lie outside the tile each scale a whole tile by one
		// factor, so they commute with every other operation of the pass: with two or more of Diag or Phase
		// form, they become TileFactor operations at the front of the pass, whose product the kernel applies
		// as it stores the tile; the pass's sign and +-i phases of that kind join them (exact products)
		if (!tc_pass) {
			std::vector<TileOp> front, rest;
			size_t products = 0;
			for (size_t i = tp.op_begin; i < ops.size(); ++i) {
				const TileOp& op = ops[i];
				const Op1 form = static_cast<Op1>(op.op);
				const bool merge = static_cast<TKind>(op.kind) == TKind::GlobalDiag && op.lset == 0 && op.nins == 0 &&
				                   (form == Op1::Diag || form == Op1::Phase || form == Op1::PhaseNeg || form == Op1::PhaseI);
				(merge ? front : rest).push_back(op);
				if (merge && (form == Op1::Diag || form == Op1::Phase)) ++products;
			}
			if (products >= 2) {
				for (TileOp& op : front) {
					const bool diag = static_cast<Op1>(op.op) == Op1::Diag;
					const bool flag = op.lbit0 != 0;  // a phase acts where the target bit equals it
					const cplx_t<T> one = mk_host<T>(1.0, 0.0), m00 = mats[op.mat], m11 = mats[op.mat + 3];
					mats[op.mat] = diag ? m00 : (flag ? one : m11);
					mats[op.mat + 1] = diag ? m11 : (flag ? m11 : one);
					op.kind = static_cast<uint8_t>(TKind::TileFactor);
					op.op = 0;
					op.lbit0 = 0;
					op.pad[0] = diag ? 1 : 0;
				}
				ops.resize(tp.op_begin);
				ops.insert(ops.end(), front.begin(), front.end());
				ops.insert(ops.end(), rest.begin(), rest.end());
				tp.nfactor = static_cast<uint32_t>(front.size());
			}
		}
		tp.op_count = static_cast<uint32_t>(ops.size()) - tp.op_begin;
		tps.push_back(tp);
	}
	return true;
}

template <typename T>
int run_planned(qcs_handle h, const std::vector<PlannedPass>& passes, int kmax, int L0, bool tensor_passes = false) {
	const int n = static_cast<int>(h->n);
	PassOps<T> po;
	if (!build_pass_ops<T>(n, h->tensor_cores, passes, kmax, L0, tensor_passes, po, h->err)) return QCS_CUDA_ERROR;
	std::vector<TilePass>& tps = po.tps;
	std::vector<TileOp>& ops = po.ops;
	std::vector<cplx_t<T>>& mats = po.mats;
	const uint32_t rowM = po.rowM;
	BatchBuffers* bb = static_cast<BatchBuffers*>(h->batch);
	if (!bb) {
		bb = new BatchBuffers;
		h->batch = bb;
	}
	// rows narrow enough for the full table of 2^M0 roots read it (z = y << (M0 - 1 - bits)); it is built
	// on the device from the two-level tables once per register and size
	const uint32_t M0 = std::min(rowM, kRootsM);
	bool build_roots = false;
	if (rowM > 0 && M0 >= kMinRowBits + 1) {
		if (bb->roots_M != M0) {
			if (bb->d_roots) cudaFree(bb->d_roots);
			bb->d_roots = nullptr;
			bb->roots_M = 0;
			if (cudaMalloc(&bb->d_roots, (size_t(1) << M0) * sizeof(cplx_t<T>)) == cudaSuccess) {
				bb->roots_M = M0;
				build_roots = true;
			} else {
				cudaGetLastError();  // no room: the rows keep the two-level form
			}
		}
		if (bb->roots_M == M0)
			for (TileOp& op : ops)
				if (static_cast<TKind>(op.kind) == TKind::PhaseRow && op.lbit2 + 1 <= M0) {
					op.pad[0] = static_cast<uint8_t>(M0 - 1 - op.lbit2);
					op.pad[3] = static_cast<uint8_t>(M0);
					op.pad[4] = 1;
					op.gtbit = reinterpret_cast<uint64_t>(bb->d_roots);
				}
	}
	// every index a kernel will form stays inside its tile and every matrix read inside the table
	for (const TilePass& tp : tps) {
		if (tp.k < 1 || tp.k > tile_qubits<T>() || tp.L > tp.k || tp.k - tp.L > kMaxHigh || tp.nfixed + tp.k != n ||
		    tp.nfactor > tp.op_count) {
			h->err = "apply gates: internal error (tile geometry)";
			return QCS_CUDA_ERROR;
		}
		for (uint32_t i = tp.op_begin; i < tp.op_begin + tp.op_count; ++i)
			if ((static_cast<TKind>(ops[i].kind) == TKind::TileFactor) != (i < tp.op_begin + tp.nfactor)) {
				h->err = "apply gates: internal error (tile factor order)";
				return QCS_CUDA_ERROR;
			}
		for (uint32_t i = tp.op_begin; i < tp.op_begin + tp.op_count; ++i)
			if (!op_in_bounds(ops[i], tp.k, mats.size()) || (tp.dense == 2) != (static_cast<TKind>(ops[i].kind) == TKind::DenseTC) ||
			    (static_cast<TKind>(ops[i].kind) == TKind::PhaseRow && ops[i].pad[4] &&
			     (ops[i].pad[3] != bb->roots_M || ops[i].gtbit != reinterpret_cast<uint64_t>(bb->d_roots)))) {
				h->err = "apply gates: internal error (tile operation out of range)";
				return QCS_CUDA_ERROR;
			}
	}
	cudaError_t e = ensure(&bb->d_ops, &bb->ops_cap, std::max<size_t>(1, ops.size()) * sizeof(TileOp));
	if (e == cudaSuccess) e = ensure(&bb->d_mats, &bb->mats_cap, std::max<size_t>(1, mats.size()) * sizeof(cplx_t<T>));
	if (e == cudaSuccess && !ops.empty())
		e = cudaMemcpyAsync(bb->d_ops, ops.data(), ops.size() * sizeof(TileOp), cudaMemcpyHostToDevice, h->stream);
	if (e == cudaSuccess && !mats.empty())
		e = cudaMemcpyAsync(bb->d_mats, mats.data(), mats.size() * sizeof(cplx_t<T>), cudaMemcpyHostToDevice, h->stream);
	if (e == cudaSuccess && build_roots) {
		// the two-level tables of size M0: the first row table's entries were built for rowM, so the
		// full table gets its own pair, computed here on the host the same way
		std::vector<cplx_t<T>> pair;
		const uint32_t S0 = (M0 + 1) / 2;
		for (uint64_t u = 0; u < (1ULL << (M0 - S0)); ++u) {
			const double a = 2.0 * M_PI * std::ldexp(static_cast<double>(u), static_cast<int>(S0) - static_cast<int>(M0));
			pair.push_back(mk_host<T>(std::cos(a), std::sin(a)));
		}
		for (uint64_t v = 0; v < (1ULL << S0); ++v) {
			const double a = 2.0 * M_PI * std::ldexp(static_cast<double>(v), -static_cast<int>(M0));
			pair.push_back(mk_host<T>(std::cos(a), std::sin(a)));
		}
		void* d_pair = nullptr;
		e = cudaMallocAsync(&d_pair, pair.size() * sizeof(cplx_t<T>), h->stream);
		if (e == cudaSuccess) e = cudaMemcpyAsync(d_pair, pair.data(), pair.size() * sizeof(cplx_t<T>), cudaMemcpyHostToDevice, h->stream);
		if (e == cudaSuccess)
			e = launch_build_roots<T>(static_cast<cplx_t<T>*>(bb->d_roots), static_cast<const cplx_t<T>*>(d_pair), M0, S0, h->sms, h->stream);
		if (d_pair) {
			const cudaError_t ef = cudaFreeAsync(d_pair, h->stream);
			if (e == cudaSuccess) e = ef;
		}
		if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);  // the host pair must outlive its copy
		if (e != cudaSuccess) bb->roots_M = 0;
	}
	bool any_tc = false;
	for (const TilePass& tp : tps) any_tc = any_tc || tp.dense == 2;
	if (e == cudaSuccess && any_tc && !bb->d_err) e = cudaMalloc(&bb->d_err, sizeof(int));
	if (e == cudaSuccess && any_tc) e = cudaMemsetAsync(bb->d_err, 0, sizeof(int), h->stream);
	auto* s = static_cast<cplx_t<T>*>(h->d_state);
	for (size_t i = 0; i < tps.size() && e == cudaSuccess; ++i) {
		if (tps[i].op_count > 0) {
			prof_begin(h, tps[i].dense == 2 ? "tile_pass_tc" : "tile_pass", 2.0 * sizeof(cplx_t<T>) * static_cast<double>(h->N),
			           h->prof ? pass_fp_ops(tps[i], ops, static_cast<int>(h->n)) : 0.0);
			e = launch_tile_pass<T>(s, tps[i], static_cast<const TileOp*>(bb->d_ops), static_cast<const cplx_t<T>*>(bb->d_mats), h->sms,
			                        h->stream, bb->d_err);
			prof_end(h);
		}
		const std::complex<double> f = passes[i].fold_after;
		if (e == cudaSuccess && f != std::complex<double>(1.0, 0.0))
			e = launch_scale_complex<T>(s, h->N, f.real(), f.imag(), h->sms, h->stream);
	}
	// the host vectors must outlive the (pageable, stream-ordered) copies
	int tc_status = 0;
	if (e == cudaSuccess && any_tc) e = cudaMemcpyAsync(&tc_status, bb->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
	if (e != cudaSuccess) {
		h->err = std::string("apply gates: ") + cudaGetErrorString(e);
		return QCS_CUDA_ERROR;
	}
	if (tc_status != 0) {
		h->err = tc_status == 1 ? "apply gates: a tensor-core block did not complete within its wait limit"
		                        : "apply gates: a tile load did not complete within its wait limit";
		return QCS_CUDA_ERROR;
	}
	return QCS_OK;
}

}  // namespace

// dense blocks applied in shared-memory passes (the fused path and qcs_apply_matrix)
int apply_blocks(qcs_handle h, std::vector<FusedBlock> blocks) {
	const int n = static_cast<int>(h->n);
	bool big = false;  // blocks of 4 or 5 qubits go to the tensor cores (FP32), whose passes use smaller tiles
	for (const FusedBlock& b : blocks) big = big || b.qubits.size() >= 4;
	const bool tc = h->prec == QCS_FP32 && h->tensor_cores && big;
	const int kmax = std::min(tc ? kTcTileQubits : (h->prec == QCS_FP64 ? tile_qubits<double>() : tile_qubits<float>()), n);
	const int L0 = low_run_qubits(n, kmax);
	for (const FusedBlock& b : blocks)
		if (b.qubits.empty()) h->scale *= b.M[0];  // a global factor only
	std::vector<PlannedPass> passes;
	for (const std::vector<size_t>& ids : pack_blocks(blocks, kmax, L0, tc ? kTcMatBudget : 0u)) {
		PlannedPass pp;
		pp.tmask = (1ULL << L0) - 1;
		for (size_t i : ids) {
			CompiledGate c;
			c.kind = GKind::Block;
			c.block_q = blocks[i].qubits;
			c.block_m = std::move(blocks[i].M);
			c.block_gates = blocks[i].ngates;
			pp.tmask |= c.local_mask();
			pp.gates.push_back(std::move(c));
		}
		passes.push_back(std::move(pp));
	}
	if (passes.empty()) {
		passes.emplace_back();
		passes.back().tmask = (1ULL << L0) - 1;
	}
	h->last_blocks = blocks.size();
	return h->prec == QCS_FP64 ? run_planned<double>(h, passes, kmax, L0) : run_planned<float>(h, passes, kmax, L0, tc);
}

// the fused path: blocks of up to fusion_max qubits (or the partition the cost model picks)
int fused_apply(qcs_handle h, const qcs_gate* gates, size_t count) {
	const int n = static_cast<int>(h->n);
	std::vector<CompiledGate> cg;
	cg.reserve(count);
	for (size_t i = 0; i < count; ++i) cg.push_back(compile_gate(gates[i], false));
	std::vector<FusedBlock> blocks;
	if (h->fusion == 2 && h->cost_ctx) {
		// the non-tensor-core tile; candidates with tensor-core blocks use kTcTileQubits (costmodel.cu)
		const int kmax = std::min(h->prec == QCS_FP64 ? tile_qubits<double>() : tile_qubits<float>(), n);
		const int L0 = low_run_qubits(n, kmax);
		const int st = choose_partition(h, cg, kmax, L0, blocks, &h->last_predicted_ms);
		if (st != QCS_OK) return st;
	} else {
		FusionPolicy pol;
		pol.max_qubits = std::min(h->fusion_limit(), h->prec == QCS_FP64 ? 4 : 5);
		pol.nqubits = n;
		blocks = fuse(cg, pol);
	}
	return apply_blocks(h, std::move(blocks));
}

namespace {

// packs compiled gates into shared-memory passes (plan_and_run then runs them).  Each pass takes, in
// order, every gate whose local qubits fit its tile and which shares no qubit with an earlier gate still
// waiting (gates on disjoint qubits commute), looking at most kGateWindow gates ahead.  The global factors
// taken out of the gates multiply into `scale` (the register's) in placement order; when its magnitude
// leaves [1/limit, limit] (scale_limit_of: 1e100 in FP64, 1e15 in FP32) the pass closes and the scale is
// folded into the amplitudes after it.
constexpr size_t kGateWindow = 64;

std::vector<PlannedPass> place_gates(const std::vector<CompiledGate>& cg, int kmax, int L0, std::complex<double>& scale, double limit) {
	const uint64_t low = (1ULL << L0) - 1;
	std::vector<PlannedPass> passes;
	std::vector<char> placed(cg.size(), 0);
	size_t first = 0;
	while (true) {
		while (first < cg.size() && placed[first]) ++first;
		if (first == cg.size()) break;
		PlannedPass pp;
		pp.tmask = low;
		uint64_t waiting = 0;
		size_t scanned = 0;
		bool fold = false;
		for (size_t i = first; i < cg.size() && scanned < kGateWindow && !fold; ++i) {
			if (placed[i]) continue;
			++scanned;
			const CompiledGate& c = cg[i];
			const uint64_t touch = c.touch_mask(), need = c.local_mask();
			const bool fits = popcount64(pp.tmask | need) <= kmax;
			if ((touch & waiting) == 0 && (fits || pp.gates.empty())) {
				placed[i] = 1;
				scale *= c.scale;
				if (c.kind != GKind::Identity) {
					pp.tmask |= need;
					pp.gates.push_back(c);
				}
				const double mag = std::abs(scale);
				if (mag > limit || mag < 1.0 / limit) {
					pp.fold_after = scale;
					scale = std::complex<double>(1.0, 0.0);
					fold = true;
				}
			} else {
				waiting |= touch;
			}
		}
		passes.push_back(std::move(pp));
	}
	if (passes.empty()) {
		passes.emplace_back();
		passes.back().tmask = low;
	}
	return passes;
}

int plan_and_run(qcs_handle h, const std::vector<CompiledGate>& cg, int kmax) {
	const int L0 = low_run_qubits(static_cast<int>(h->n), kmax);
	const std::vector<PlannedPass> passes = place_gates(cg, kmax, L0, h->scale, h->scale_limit());
	return h->prec == QCS_FP64 ? run_planned<double>(h, passes, kmax, L0) : run_planned<float>(h, passes, kmax, L0);
}

// whether a gate list on this register runs one kernel per gate (small registers, short lists, or
// passes switched off)
bool per_gate_mode(qcs_handle h, size_t count, int kmax) {
	return static_cast<int>(h->n) < kmax + 2 || count < 2 || h->batch_mode == 0;
}

}  // namespace

int batch_apply(qcs_handle h, const qcs_gate* gates, size_t count) {
	const int fusion = h->fusion >= 0 ? h->fusion : (h->prec == QCS_FP32 ? 1 : 0);
	if (fusion > 0 && count > 0) return fused_apply(h, gates, count);
	const int kmax = h->prec == QCS_FP64 ? tile_qubits<double>() : tile_qubits<float>();
	if (per_gate_mode(h, count, kmax)) {
		for (size_t i = 0; i < count; ++i) {
			cudaError_t e = apply_one(h, gates[i]);
			if (e != cudaSuccess) {
				h->err = std::string("apply gates: ") + cudaGetErrorString(e);
				return QCS_CUDA_ERROR;
			}
		}
		return QCS_OK;
	}
	std::vector<CompiledGate> cg;
	cg.reserve(count);
	for (size_t i = 0; i < count; ++i) cg.push_back(compile_gate(gates[i], true));
	return plan_and_run(h, cg, kmax);
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

namespace {


// the QFT's gate sequence with each target's run of controlled phases as one PhaseRow: the phases
// commute (all diagonal) and sit between the same two Hadamards, so their product is applied at once
std::vector<CompiledGate> qft_compiled(uint32_t start, uint32_t end, bool inverse, bool do_swap) {
	std::vector<CompiledGate> cg;
	const int sq = static_cast<int>(start), eq = static_cast<int>(end);
	auto swaps = [&]() {
		uint32_t a = start, b = end;
		while (a < b) cg.push_back(compile_gate(make_swap(a++, b--), true));
	};
	auto row = [&](int cur) {
		const uint32_t bits = static_cast<uint32_t>(cur - sq);
		if (bits >= kMinRowBits) {
			CompiledGate c;
			c.kind = GKind::PhaseRow;
			c.target = static_cast<uint32_t>(cur);
			c.row_lo = start;
			c.row_bits = bits;
			c.row_inverse = inverse;
			cg.push_back(c);
			return;
		}
		double phase = inverse ? -M_PI_2 : M_PI_2;
		for (int c = cur - 1; c >= sq; --c) {
			cg.push_back(compile_gate(make_cp(cur, c, phase), true));
			phase *= 0.5;
		}
	};
	if (!inverse) {
		cg.push_back(compile_gate(make_h(eq), true));
		for (int cur = eq; cur > sq; --cur) {
			row(cur);
			cg.push_back(compile_gate(make_h(cur - 1), true));
		}
		if (do_swap) swaps();
	} else {
		if (do_swap) swaps();
		for (int cur = sq + 1; cur <= eq; ++cur) {
			cg.push_back(compile_gate(make_h(cur - 1), true));
			row(cur);
		}
		cg.push_back(compile_gate(make_h(eq), true));
	}
	return cg;
}

}  // namespace

// the QFT always runs through the pass planner with phase rows (also on fused FP32 registers: its
// controlled phases couple distant qubits, which dense blocks would spread over many passes)
int qft_apply(qcs_handle h, uint32_t start, uint32_t end, bool inverse, bool do_swap) {
	const std::vector<qcs_gate> gs = qft_gates(start, end, inverse, do_swap);
	const int kmax = h->prec == QCS_FP64 ? tile_qubits<double>() : tile_qubits<float>();
	if (per_gate_mode(h, gs.size(), kmax)) {
		for (const qcs_gate& g : gs) {
			cudaError_t e = apply_one(h, g);
			if (e != cudaSuccess) {
				h->err = std::string("qft: ") + cudaGetErrorString(e);
				return QCS_CUDA_ERROR;
			}
		}
		return QCS_OK;
	}
	return plan_and_run(h, qft_compiled(start, end, inverse, do_swap), kmax);
}

// Each step: potential diagonal, IQFT of the whole register (with the swaps), kinetic diagonal, QFT.
// The diagonals are TableDiag operations, so the planner puts them inside the passes of the
// neighbouring transforms (no sweep of their own); steps are planned a few at a time.
int schrodinger_apply(qcs_handle h, const void* d_potential, const void* d_kinetic, uint64_t steps) {
	const int kmax = h->prec == QCS_FP64 ? tile_qubits<double>() : tile_qubits<float>();
	const uint32_t end = h->n - 1;
	CompiledGate pot, kin;
	pot.kind = kin.kind = GKind::TableDiag;
	pot.table = d_potential;
	kin.table = d_kinetic;
	if (per_gate_mode(h, 2, kmax)) {
		for (uint64_t s = 0; s < steps; ++s) {
			cudaError_t e = h->prec == QCS_FP64 ? launch_compiled<double>(static_cast<double2*>(h->d_state), h->N, pot, h->sms, h->stream)
			                                    : launch_compiled<float>(static_cast<float2*>(h->d_state), h->N, pot, h->sms, h->stream);
			if (e != cudaSuccess) return fail_cuda(h, e, "schrodinger");
			if (int st = qft_apply(h, 0, end, true, true)) return st;
			e = h->prec == QCS_FP64 ? launch_compiled<double>(static_cast<double2*>(h->d_state), h->N, kin, h->sms, h->stream)
			                        : launch_compiled<float>(static_cast<float2*>(h->d_state), h->N, kin, h->sms, h->stream);
			if (e != cudaSuccess) return fail_cuda(h, e, "schrodinger");
			if (int st = qft_apply(h, 0, end, false, true)) return st;
		}
		return QCS_OK;
	}
	const std::vector<CompiledGate> inv = qft_compiled(0, end, true, true), fwd = qft_compiled(0, end, false, true);
	constexpr uint64_t kStepsPerPlan = 8;
	for (uint64_t s0 = 0; s0 < steps; s0 += kStepsPerPlan) {
		std::vector<CompiledGate> cg;
		for (uint64_t s = s0; s < std::min(steps, s0 + kStepsPerPlan); ++s) {
			cg.push_back(pot);
			cg.insert(cg.end(), inv.begin(), inv.end());
			cg.push_back(kin);
			cg.insert(cg.end(), fwd.begin(), fwd.end());
		}
		if (int st = plan_and_run(h, cg, kmax)) return st;
	}
	return QCS_OK;
}

void batch_release(qcs_handle h) {
	BatchBuffers* bb = static_cast<BatchBuffers*>(h->batch);
	if (!bb) return;
	if (bb->d_ops) cudaFree(bb->d_ops);
	if (bb->d_mats) cudaFree(bb->d_mats);
	if (bb->d_err) cudaFree(bb->d_err);
	if (bb->d_roots) cudaFree(bb->d_roots);
	delete bb;
	h->batch = nullptr;
}

}  // namespace qcs

extern "C" int qcs_plan_gate_passes(uint32_t nqubits, int precision, const qcs_gate* gates, size_t count, uint32_t* pass_ops,
                                    uint32_t* pass_factors, size_t capacity, size_t* npasses_out) {
	if ((!gates && count) || !npasses_out || (precision != QCS_FP64 && precision != QCS_FP32) || nqubits < 1 || nqubits > 36)
		return QCS_INVALID_ARGUMENT;
	std::vector<qcs::CompiledGate> cg;
	cg.reserve(count);
	for (size_t i = 0; i < count; ++i) {
		const qcs_gate& g = gates[i];
		if (g.k < 1 || g.k > 3 || g.q0 >= nqubits || (g.k > 1 && g.q1 >= nqubits) || (g.k > 2 && g.q2 >= nqubits))
			return QCS_INVALID_ARGUMENT;
		cg.push_back(qcs::compile_gate(g, true));
	}
	*npasses_out = 0;
	const int n = static_cast<int>(nqubits);
	const int kmax = precision == QCS_FP64 ? qcs::tile_qubits<double>() : qcs::tile_qubits<float>();
	if (n < kmax + 2 || count < 2) return QCS_OK;  // such lists run one kernel per gate
	const int L0 = qcs::low_run_qubits(n, kmax);
	std::complex<double> scale(1.0, 0.0);
	const std::vector<qcs::PlannedPass> passes = qcs::place_gates(cg, kmax, L0, scale, qcs::scale_limit_of(precision));
	std::string err;
	std::vector<qcs::TilePass> tps;
	if (precision == QCS_FP64) {
		qcs::PassOps<double> po;
		if (!qcs::build_pass_ops<double>(n, false, passes, kmax, L0, false, po, err)) return QCS_UNSUPPORTED;
		tps = std::move(po.tps);
	} else {
		qcs::PassOps<float> po;
		if (!qcs::build_pass_ops<float>(n, false, passes, kmax, L0, false, po, err)) return QCS_UNSUPPORTED;
		tps = std::move(po.tps);
	}
	for (size_t p = 0; p < tps.size() && p < capacity; ++p) {
		if (pass_ops) pass_ops[p] = tps[p].op_count;
		if (pass_factors) pass_factors[p] = tps[p].nfactor;
	}
	*npasses_out = tps.size();
	return QCS_OK;
}
