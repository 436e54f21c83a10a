// Per-amplitude arithmetic of the gate kernels, shared by the per-gate kernels and the
// shared-memory pass kernels so both produce identical results.
//
// GB300 executes FP64 instructions at about 1/64 of its FP32 rate, so the FP64 amplitude updates are written
// to use as few FP64 operations as the gate allows: permutations and sign/i flips use none, phases
// touch only the half of the amplitudes they change, and rotations whose global scalar was factored
// out on the host (the Unit* forms) cost one FMA per real component.
#pragma once

#include "engine.cuh"

namespace qcs {

template <typename T> __device__ __forceinline__ cplx_t<T> mk(T x, T y) {
	cplx_t<T> r;
	r.x = x;
	r.y = y;
	return r;
}

template <typename T> __device__ __forceinline__ cplx_t<T> cmul(const cplx_t<T>& a, const cplx_t<T>& b) {
	return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// v * u for u in {1, i, -1, -i} (code 0..3): component moves and sign flips only
template <typename T> __device__ __forceinline__ cplx_t<T> mul_unit(const cplx_t<T>& v, int code) {
	switch (code & 3) {
	case 0: return v;
	case 1: return mk<T>(-v.y, v.x);
	case 2: return mk<T>(-v.x, -v.y);
	default: return mk<T>(v.y, -v.x);
	}
}

// v or -v, chosen at compile time (the negation folds into the consuming FMA)
template <int NEG, typename T> __device__ __forceinline__ T sg(T v) { return NEG ? -v : v; }

// 2x2 block update of (a0, a1) = (amplitude with target bit 0, with target bit 1).
// Mat2 field use per op:
//   Diag/Phase*: m00, m11 diagonal entries        Antidiag: m01, m10
//   AntidiagUnit: m01.x, m10.x hold unit codes    Real/RxLike/Generic: the four entries
//   Unit*: m00 = (sigma0, x0), m01 = (sigma1, x1) -- see below
// SG: signs of the unit entries of the Unit* forms (bit 0: row 0 negative, bit 1: row 1 negative)
template <typename T, Op1 OP, int SG = 0>
__device__ __forceinline__ void op2(cplx_t<T>& a0, cplx_t<T>& a1, const Mat2<T>& m) {
	if constexpr (OP == Op1::Diag) {
		a0 = cmul<T>(a0, m.m00);
		a1 = cmul<T>(a1, m.m11);
	} else if constexpr (OP == Op1::Phase) {
		a1 = cmul<T>(a1, m.m11);
	} else if constexpr (OP == Op1::PhaseNeg) {
		a1 = mk<T>(-a1.x, -a1.y);
	} else if constexpr (OP == Op1::PhaseI) {
		// (x + iy) * (i*s) = -s*y + i*s*x
		const T sgn = m.m11.y;
		a1 = mk<T>(-sgn * a1.y, sgn * a1.x);
	} else if constexpr (OP == Op1::Antidiag) {
		const cplx_t<T> n0 = cmul<T>(m.m01, a1);
		a1 = cmul<T>(m.m10, a0);
		a0 = n0;
	} else if constexpr (OP == Op1::AntidiagUnit) {
		const cplx_t<T> n0 = mul_unit<T>(a1, static_cast<int>(m.m01.x));
		a1 = mul_unit<T>(a0, static_cast<int>(m.m10.x));
		a0 = n0;
	} else if constexpr (OP == Op1::Swap) {
		const cplx_t<T> t = a0;
		a0 = a1;
		a1 = t;
	} else if constexpr (OP == Op1::Real) {
		const cplx_t<T> n0 = mk<T>(m.m00.x * a0.x + m.m01.x * a1.x, m.m00.x * a0.y + m.m01.x * a1.y);
		a1 = mk<T>(m.m10.x * a0.x + m.m11.x * a1.x, m.m10.x * a0.y + m.m11.x * a1.y);
		a0 = n0;
	} else if constexpr (OP == Op1::RxLike) {
		const cplx_t<T> n0 = mk<T>(m.m00.x * a0.x - m.m01.y * a1.y, m.m00.x * a0.y + m.m01.y * a1.x);
		a1 = mk<T>(m.m11.x * a1.x - m.m10.y * a0.y, m.m11.x * a1.y + m.m10.y * a0.x);
		a0 = n0;
	} else if constexpr (OP == Op1::UnitRe01) {
		// out0 = s0*a0 + x0*a1, out1 = s1*a1 + x1*a0 (s = +-1, x real)
		const T x0 = m.m00.y, x1 = m.m01.y;
		const cplx_t<T> n0 = mk<T>(fma(x0, a1.x, sg<SG & 1>(a0.x)), fma(x0, a1.y, sg<SG & 1>(a0.y)));
		a1 = mk<T>(fma(x1, a0.x, sg<(SG >> 1) & 1>(a1.x)), fma(x1, a0.y, sg<(SG >> 1) & 1>(a1.y)));
		a0 = n0;
	} else if constexpr (OP == Op1::UnitRe10) {
		// out0 = s0*a1 + x0*a0, out1 = s1*a0 + x1*a1
		const T x0 = m.m00.y, x1 = m.m01.y;
		const cplx_t<T> n0 = mk<T>(fma(x0, a0.x, sg<SG & 1>(a1.x)), fma(x0, a0.y, sg<SG & 1>(a1.y)));
		a1 = mk<T>(fma(x1, a1.x, sg<(SG >> 1) & 1>(a0.x)), fma(x1, a1.y, sg<(SG >> 1) & 1>(a0.y)));
		a0 = n0;
	} else if constexpr (OP == Op1::UnitIm01) {
		// out0 = s0*a0 + i*x0*a1, out1 = s1*a1 + i*x1*a0
		const T x0 = m.m00.y, x1 = m.m01.y;
		const cplx_t<T> n0 = mk<T>(fma(-x0, a1.y, sg<SG & 1>(a0.x)), fma(x0, a1.x, sg<SG & 1>(a0.y)));
		a1 = mk<T>(fma(-x1, a0.y, sg<(SG >> 1) & 1>(a1.x)), fma(x1, a0.x, sg<(SG >> 1) & 1>(a1.y)));
		a0 = n0;
	} else if constexpr (OP == Op1::UnitIm10) {
		// out0 = s0*a1 + i*x0*a0, out1 = s1*a0 + i*x1*a1
		const T x0 = m.m00.y, x1 = m.m01.y;
		const cplx_t<T> n0 = mk<T>(fma(-x0, a0.y, sg<SG & 1>(a1.x)), fma(x0, a0.x, sg<SG & 1>(a1.y)));
		a1 = mk<T>(fma(-x1, a1.y, sg<(SG >> 1) & 1>(a0.x)), fma(x1, a1.x, sg<(SG >> 1) & 1>(a0.y)));
		a0 = n0;
	} else {
		const cplx_t<T> n0 = mk<T>(m.m00.x * a0.x - m.m00.y * a0.y + m.m01.x * a1.x - m.m01.y * a1.y,
		                           m.m00.x * a0.y + m.m00.y * a0.x + m.m01.x * a1.y + m.m01.y * a1.x);
		a1 = mk<T>(m.m10.x * a0.x - m.m10.y * a0.y + m.m11.x * a1.x - m.m11.y * a1.y,
		           m.m10.x * a0.y + m.m10.y * a0.x + m.m11.x * a1.y + m.m11.y * a1.x);
		a0 = n0;
	}
}

template <Op1 OP> __host__ __device__ constexpr bool touches_a0() {
	return !(OP == Op1::Phase || OP == Op1::PhaseNeg || OP == Op1::PhaseI);
}

// item number -> base index: zero bits inserted at the sorted positions, control bits set
template <int NINS> __device__ __forceinline__ uint64_t expand(uint64_t p, const BitPlan& pl) {
#pragma unroll
	for (int j = 0; j < NINS; ++j) {
		const int b = pl.ins[j];
		p = ((p >> b) << (b + 1)) | (p & ((1ULL << b) - 1));
	}
	return p | pl.set_mask;
}

}  // namespace qcs
