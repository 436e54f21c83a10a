// Gate compilation (trait dispatch -> kernel operation) and the per-gate launch of a compiled gate.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "compile.cuh"
#include "gate_math.cuh"

namespace qcs {
namespace {

using cd = std::complex<double>;

cd entry(const double* m, int dim, int r, int c) { return cd(m[2 * (r * dim + c)], m[2 * (r * dim + c) + 1]); }

double2 d2(const cd& v) { return make_double2(v.real(), v.imag()); }

// unit code of v: 0 for 1, 1 for i, 2 for -1, 3 for -i, -1 otherwise
int unit_code(const cd& v) {
	if (v == cd(1, 0)) return 0;
	if (v == cd(0, 1)) return 1;
	if (v == cd(-1, 0)) return 2;
	if (v == cd(0, -1)) return 3;
	return -1;
}

void set_phase(CompiledGate& c, const cd& f, bool on_a0) {
	c.kind = GKind::Ctrl1q;
	c.phase_on_a0 = on_a0;
	c.m.m00 = make_double2(1, 0);
	c.m.m11 = d2(f);
	if (f == cd(-1, 0)) c.op = Op1::PhaseNeg;
	else if (f == cd(0, 1) || f == cd(0, -1)) c.op = Op1::PhaseI;
	else c.op = Op1::Phase;
}

// diagonal block diag(d0, d1): ApplyOneQubitGate's diagonal branch (QubitRegisterCalculator.h:41-52),
// ApplyDiagonalControlGate (:357-371), ApplyDiagonalCCGate (:642-656)
void diag(CompiledGate& c, cd d0, cd d1, bool factor) {
	const cd one(1, 0);
	if (factor && d0 != one && d0 != cd(0, 0) && std::abs(std::abs(d0) - 1.0) < 1e-13) {
		// diag(d0, d1) = d0 * diag(1, d1/d0): the global factor goes to the register's scale
		c.scale = d0;
		d1 = d1 / d0;
		d0 = one;
	}
	if (d0 == one && d1 == one) {
		c.kind = GKind::Identity;
		return;
	}
	if (d0 == one) return set_phase(c, d1, false);
	if (d1 == one) return set_phase(c, d0, true);
	c.kind = GKind::Ctrl1q;
	c.op = Op1::Diag;
	c.m.m00 = d2(d0);
	c.m.m11 = d2(d1);
}

// antidiagonal block: ApplyOneQubitGate (:57-67), ApplyAntidiagonalControlGate (:373-393),
// ApplyAntidiagonalCCGate (:658-680); new a0 = v01 * a1, new a1 = v10 * a0
void antidiag(CompiledGate& c, const cd& v01, const cd& v10) {
	c.kind = GKind::Ctrl1q;
	const int u01 = unit_code(v01), u10 = unit_code(v10);
	if (u01 == 0 && u10 == 0) {
		c.op = Op1::Swap;
	} else if (u01 >= 0 && u10 >= 0) {
		c.op = Op1::AntidiagUnit;
		c.m.m01 = make_double2(u01, 0);
		c.m.m10 = make_double2(u10, 0);
	} else {
		c.op = Op1::Antidiag;
		c.m.m01 = d2(v01);
		c.m.m10 = d2(v10);
	}
}

// general block [[a, b], [c, d]]: ApplyOneQubitGate (:68-79), ApplyGenericControlGate (:395-417),
// ApplyGenericCCGate (:682-707)
void general(CompiledGate& c, const cd& a, const cd& b, const cd& cc, const cd& d, bool factor) {
	c.kind = GKind::Ctrl1q;
	const bool real = a.imag() == 0 && b.imag() == 0 && cc.imag() == 0 && d.imag() == 0;
	const bool rxl = a.imag() == 0 && d.imag() == 0 && b.real() == 0 && cc.real() == 0;
	if (factor && (real || rxl)) {
		const double A = a.real(), D = d.real();
		const double B = real ? b.real() : b.imag(), C = real ? cc.real() : cc.imag();
		if (A != 0 && std::abs(A) >= std::abs(B) && std::abs(D) == std::abs(A)) {
			// M = a * [[1, b/a], [c/a, d/a]]
			c.scale = cd(A, 0);
			c.op = real ? Op1::UnitRe01 : Op1::UnitIm01;
			c.m.m00 = make_double2(1.0, B / A);
			c.m.m01 = make_double2(D / A, C / A);
			return;
		}
		if (B != 0 && std::abs(B) > std::abs(A) && std::abs(C) == std::abs(B)) {
			// M = b * [[a/b, 1], [c/b, d/b]]
			if (real) {
				c.scale = cd(B, 0);
				c.op = Op1::UnitRe10;
				c.m.m00 = make_double2(1.0, A / B);
				c.m.m01 = make_double2(C / B, D / B);
			} else {
				c.scale = cd(0, B);
				c.op = Op1::UnitIm10;
				c.m.m00 = make_double2(1.0, -A / B);
				c.m.m01 = make_double2(C / B, -D / B);
			}
			return;
		}
	}
	c.op = real ? Op1::Real : (rxl ? Op1::RxLike : Op1::Generic);
	c.m.m00 = d2(a);
	c.m.m01 = d2(b);
	c.m.m10 = d2(cc);
	c.m.m11 = d2(d);
}

void add_ctrl(CompiledGate& c, uint32_t q) { c.controls[c.ncontrols++] = q; }

}  // namespace

const char* kernel_name(const CompiledGate& c) {
	static const char* ops[] = {"ctrl1q_diag", "ctrl1q_phase", "ctrl1q_phaseneg", "ctrl1q_phasei", "ctrl1q_antidiag",
	                            "ctrl1q_swap", "ctrl1q_real", "ctrl1q_rxlike", "ctrl1q_generic", "ctrl1q_antidiagunit",
	                            "ctrl1q_unitre01", "ctrl1q_unitre10", "ctrl1q_unitim01", "ctrl1q_unitim10"};
	switch (c.kind) {
	case GKind::Ctrl1q: return ops[static_cast<int>(c.op)];
	case GKind::Swap: return c.ncontrols ? "swap_controlled" : "swap";
	case GKind::Dense: return c.dense_k == 2 ? "dense2" : "dense3";
	case GKind::Block: return "block";
	case GKind::PhaseRow: return "phase_row";
	case GKind::TableDiag: return "table_diag";
	default: return "identity";
	}
}

double touched_fraction(const CompiledGate& c) {
	const double ctl = 1.0 / static_cast<double>(1u << c.ncontrols);
	switch (c.kind) {
	case GKind::Ctrl1q:
		if (c.op == Op1::Phase || c.op == Op1::PhaseNeg || c.op == Op1::PhaseI) return ctl * 0.5;
		return ctl;
	case GKind::Swap: return ctl * 0.5;
	case GKind::Dense: return ctl;
	case GKind::Block: return 1.0;
	case GKind::PhaseRow: return 0.5;
	case GKind::TableDiag: return 1.0;
	default: return 0.0;
	}
}

uint64_t CompiledGate::local_mask() const {
	switch (kind) {
	case GKind::Ctrl1q:
		if (op == Op1::Diag || op == Op1::Phase || op == Op1::PhaseNeg || op == Op1::PhaseI) return 0;
		return 1ULL << target;
	case GKind::Swap: return (1ULL << qa) | (1ULL << qb);
	case GKind::Dense: {
		uint64_t m = 0;
		for (int j = 0; j < dense_k; ++j) m |= 1ULL << dense_q[j];
		return m;
	}
	case GKind::Block: {
		uint64_t m = 0;
		for (uint32_t q : block_q) m |= 1ULL << q;
		return m;
	}
	default: return 0;
	}
}

uint64_t CompiledGate::touch_mask() const {
	if (kind == GKind::TableDiag) return ~0ULL;  // a general diagonal depends on every qubit
	uint64_t m = local_mask();
	if (kind == GKind::Ctrl1q) m |= 1ULL << target;
	if (kind == GKind::PhaseRow) m |= (1ULL << target) | (((1ULL << row_bits) - 1) << row_lo);
	for (uint32_t i = 0; i < ncontrols; ++i) m |= 1ULL << controls[i];
	return m;
}

CompiledGate compile_gate(const qcs_gate& g, bool factor) {
	CompiledGate c;
	const double* m = g.m;
	const uint32_t tr = g.traits;
	c.target = g.q0;
	if (g.k == 1) {
		if (tr & QCS_TRAIT_DIAGONAL) diag(c, entry(m, 2, 0, 0), entry(m, 2, 1, 1), factor);
		else if (tr & QCS_TRAIT_ANTIDIAGONAL) antidiag(c, entry(m, 2, 0, 1), entry(m, 2, 1, 0));
		else general(c, entry(m, 2, 0, 0), entry(m, 2, 0, 1), entry(m, 2, 1, 0), entry(m, 2, 1, 1), factor);
		return c;
	}
	if (g.k == 2) {
		if (tr & (QCS_TRAIT_SWAP | QCS_TRAIT_ISWAP | QCS_TRAIT_ISWAPDAG)) {
			// ApplySwapGate / ApplyISwapGate / ApplyISwapDagGate (QubitRegisterCalculator.h:230-355)
			c.kind = GKind::Swap;
			c.sk = (tr & QCS_TRAIT_SWAP) ? SwapKind::Plain : ((tr & QCS_TRAIT_ISWAP) ? SwapKind::ISwap : SwapKind::ISwapDag);
			c.qa = g.q1;
			c.qb = g.q0;
			return c;
		}
		if (tr & QCS_TRAIT_CONTROLLED) {
			add_ctrl(c, g.q1);
			if (tr & QCS_TRAIT_DIAGONAL) diag(c, entry(m, 4, 2, 2), entry(m, 4, 3, 3), false);
			else if (tr & QCS_TRAIT_ANTIDIAGONAL) antidiag(c, entry(m, 4, 2, 3), entry(m, 4, 3, 2));
			else general(c, entry(m, 4, 2, 2), entry(m, 4, 2, 3), entry(m, 4, 3, 2), entry(m, 4, 3, 3), false);
			return c;
		}
		c.kind = GKind::Dense;  // ApplyGenericTwoQubitsGate (:419-465)
		c.dense_k = 2;
		c.dense_q[0] = g.q0;
		c.dense_q[1] = g.q1;
		std::memcpy(c.dense_m, m, sizeof(double) * 32);
		return c;
	}
	if (tr & QCS_TRAIT_SWAP) {
		// Fredkin (:181-194): controllingQubit2 controls the exchange of qubit and controllingQubit1
		c.kind = GKind::Swap;
		c.qa = g.q1;
		c.qb = g.q0;
		add_ctrl(c, g.q2);
		return c;
	}
	if (tr & QCS_TRAIT_CONTROLLED) {
		if (tr & QCS_TRAIT_CONTROLQ1) {
			add_ctrl(c, g.q1);
			add_ctrl(c, g.q2);
			if (tr & QCS_TRAIT_DIAGONAL) diag(c, entry(m, 8, 6, 6), entry(m, 8, 7, 7), false);
			else if (tr & QCS_TRAIT_ANTIDIAGONAL) antidiag(c, entry(m, 8, 6, 7), entry(m, 8, 7, 6));
			else general(c, entry(m, 8, 6, 6), entry(m, 8, 6, 7), entry(m, 8, 7, 6), entry(m, 8, 7, 7), false);
			return c;
		}
		// one control on controllingQubit2: the 4x4 block of rows/columns 4..7 (:610-638)
		c.kind = GKind::Dense;
		c.dense_k = 2;
		c.dense_q[0] = g.q0;
		c.dense_q[1] = g.q1;
		add_ctrl(c, g.q2);
		for (int r = 0; r < 4; ++r)
			for (int cc = 0; cc < 4; ++cc) {
				c.dense_m[2 * (r * 4 + cc)] = m[2 * ((4 + r) * 8 + 4 + cc)];
				c.dense_m[2 * (r * 4 + cc) + 1] = m[2 * ((4 + r) * 8 + 4 + cc) + 1];
			}
		return c;
	}
	c.kind = GKind::Dense;  // ApplyThreeQubitsGenericGate (:710-762)
	c.dense_k = 3;
	c.dense_q[0] = g.q0;
	c.dense_q[1] = g.q1;
	c.dense_q[2] = g.q2;
	std::memcpy(c.dense_m, m, sizeof(double) * 128);
	return c;
}

template <typename T> static Mat2<T> cast_mat(const Mat2<double>& m) {
	Mat2<T> r;
	r.m00.x = static_cast<T>(m.m00.x); r.m00.y = static_cast<T>(m.m00.y);
	r.m01.x = static_cast<T>(m.m01.x); r.m01.y = static_cast<T>(m.m01.y);
	r.m10.x = static_cast<T>(m.m10.x); r.m10.y = static_cast<T>(m.m10.y);
	r.m11.x = static_cast<T>(m.m11.x); r.m11.y = static_cast<T>(m.m11.y);
	return r;
}

static BitPlan plan_for(std::vector<uint32_t> ins, uint64_t set) {
	std::sort(ins.begin(), ins.end());
	BitPlan p;
	p.nins = static_cast<int>(ins.size());
	for (int i = 0; i < p.nins; ++i) p.ins[i] = static_cast<int>(ins[i]);
	p.set_mask = set;
	return p;
}

template <typename T> cudaError_t launch_compiled(cplx_t<T>* s, uint64_t N, const CompiledGate& c, int sms, cudaStream_t st) {
	uint64_t set = 0;
	std::vector<uint32_t> ins;
	for (uint32_t i = 0; i < c.ncontrols; ++i) {
		set |= 1ULL << c.controls[i];
		ins.push_back(c.controls[i]);
	}
	switch (c.kind) {
	case GKind::Identity: return cudaSuccess;
	case GKind::Ctrl1q: {
		ins.push_back(c.target);
		const uint64_t tbit = c.phase_on_a0 ? 0 : (1ULL << c.target);
		return launch_ctrl1q<T>(s, N, c.op, cast_mat<T>(c.m), tbit, plan_for(ins, set), sms, st);
	}
	case GKind::Swap:
		ins.push_back(c.qa);
		ins.push_back(c.qb);
		return launch_swap<T>(s, N, c.sk, 1ULL << c.qa, 1ULL << c.qb, plan_for(ins, set), sms, st);
	case GKind::Dense: {
		DenseArgs a;
		a.k = c.dense_k;
		for (int j = 0; j < c.dense_k; ++j) {
			a.bit[j] = 1ULL << c.dense_q[j];
			ins.push_back(c.dense_q[j]);
		}
		std::memcpy(a.m, c.dense_m, sizeof(a.m));
		return launch_dense<T>(s, N, a, plan_for(ins, set), sms, st);
	}
	case GKind::TableDiag: return launch_table_diag<T>(s, N, static_cast<const cplx_t<T>*>(c.table), sms, st);
	case GKind::Block:
	case GKind::PhaseRow: break;  // shared-memory passes only
	}
	return cudaErrorInvalidValue;
}

namespace {
template <typename T> __global__ void k_scale_complex(cplx_t<T>* s, uint64_t N, double re, double im) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	const cplx_t<T> f = mk<T>(static_cast<T>(re), static_cast<T>(im));
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) s[i] = cmul<T>(s[i], f);
}
}  // namespace

template <typename T>
cudaError_t launch_scale_complex(cplx_t<T>* s, uint64_t N, double re, double im, int sms, cudaStream_t st) {
	k_scale_complex<T><<<grid_for(N, 256, sms), 256, 0, st>>>(s, N, re, im);
	note_launches(1);
	return cudaGetLastError();
}

template cudaError_t launch_compiled<double>(double2*, uint64_t, const CompiledGate&, int, cudaStream_t);
template cudaError_t launch_compiled<float>(float2*, uint64_t, const CompiledGate&, int, cudaStream_t);
template cudaError_t launch_scale_complex<double>(double2*, uint64_t, double, double, int, cudaStream_t);
template cudaError_t launch_scale_complex<float>(float2*, uint64_t, double, double, int, cudaStream_t);

}  // namespace qcs
