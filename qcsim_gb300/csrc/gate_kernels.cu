// Per-gate statevector kernels, in place.
//
// A gate touches groups of amplitudes that differ only in the gate's qubits.  A work item is one
// group: its base index is the item number with zero bits inserted at the gate's (sorted) bit
// positions, OR-ed with the control bits that must be one.  Consecutive threads get consecutive
// items, so for every bit position above the lowest inserted one the warp reads 32 consecutive
// 16-byte amplitudes (128-bit loads, full sectors).  Each thread keeps two items in flight.
//
// Semantics follow QCSim's QubitRegisterCalculator loops (cited per kernel); the reference's
// out-of-place copies of untouched amplitudes become "leave in place".
#include "gate_math.cuh"

namespace qcs {
namespace {

template <typename T, Op1 OP, int NINS, int SG>
__global__ void __launch_bounds__(256) k_ctrl1q(cplx_t<T>* __restrict__ s, uint64_t items, Mat2<T> m, uint64_t tbit, BitPlan pl) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	uint64_t p = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	for (; p + stride < items; p += 2 * stride) {
		const uint64_t b0 = expand<NINS>(p, pl), b1 = expand<NINS>(p + stride, pl);
		cplx_t<T> x0, x1, y0, y1;
		if constexpr (touches_a0<OP>()) { x0 = s[b0]; y0 = s[b1]; }
		x1 = s[b0 | tbit];
		y1 = s[b1 | tbit];
		op2<T, OP, SG>(x0, x1, m);
		op2<T, OP, SG>(y0, y1, m);
		if constexpr (touches_a0<OP>()) { s[b0] = x0; s[b1] = y0; }
		s[b0 | tbit] = x1;
		s[b1 | tbit] = y1;
	}
	if (p < items) {
		const uint64_t b0 = expand<NINS>(p, pl);
		cplx_t<T> x0, x1;
		if constexpr (touches_a0<OP>()) x0 = s[b0];
		x1 = s[b0 | tbit];
		op2<T, OP, SG>(x0, x1, m);
		if constexpr (touches_a0<OP>()) s[b0] = x0;
		s[b0 | tbit] = x1;
	}
}

// swap / iSwap / iSwap-dagger (QubitRegisterCalculator.h:230-355) and Fredkin (:181-194):
// exchange the amplitudes at base|bitA and base|bitB
template <typename T, SwapKind K, int NINS>
__global__ void __launch_bounds__(256) k_swap(cplx_t<T>* __restrict__ s, uint64_t items, uint64_t bitA, uint64_t bitB, BitPlan pl) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t p = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < items; p += stride) {
		const uint64_t b = expand<NINS>(p, pl);
		const cplx_t<T> a = s[b | bitA], c = s[b | bitB];
		if constexpr (K == SwapKind::Plain) {
			s[b | bitA] = c;
			s[b | bitB] = a;
		} else if constexpr (K == SwapKind::ISwap) {
			s[b | bitA] = mk<T>(-c.y, c.x);
			s[b | bitB] = mk<T>(-a.y, a.x);
		} else {
			s[b | bitA] = mk<T>(c.y, -c.x);
			s[b | bitB] = mk<T>(a.y, -a.x);
		}
	}
}

template <typename T> struct DenseArgsT {
	uint64_t bit[3];
	cplx_t<T> m[64];
};

// dense 4x4 (QubitRegisterCalculator.h:419-465), the single-control 4x4 block (:610-638) and the
// dense 8x8 (:710-762)
template <typename T, int K, int NINS>
__global__ void __launch_bounds__(256) k_dense(cplx_t<T>* __restrict__ s, uint64_t items, DenseArgsT<T> a, BitPlan pl) {
	constexpr int D = 1 << K;
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t p = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < items; p += stride) {
		const uint64_t b = expand<NINS>(p, pl);
		uint64_t idx[D];
		cplx_t<T> v[D];
#pragma unroll
		for (int r = 0; r < D; ++r) {
			uint64_t x = b;
			if (r & 1) x |= a.bit[0];
			if (K > 1 && (r & 2)) x |= a.bit[1];
			if (K > 2 && (r & 4)) x |= a.bit[2];
			idx[r] = x;
			v[r] = s[x];
		}
#pragma unroll
		for (int r = 0; r < D; ++r) {
			T re = 0, im = 0;
#pragma unroll
			for (int c = 0; c < D; ++c) {
				const cplx_t<T> mm = a.m[r * D + c];
				re += mm.x * v[c].x - mm.y * v[c].y;
				im += mm.x * v[c].y + mm.y * v[c].x;
			}
			s[idx[r]] = mk<T>(re, im);
		}
	}
}

template <typename T, Op1 OP, int SG>
cudaError_t ctrl1q_sg(cplx_t<T>* s, uint64_t N, const Mat2<T>& m, uint64_t tbit, const BitPlan& pl, int sms, cudaStream_t st) {
	const uint64_t items = N >> pl.nins;
	const int grid = grid_for((items + 1) / 2, 256, sms);
	switch (pl.nins) {
	case 1: k_ctrl1q<T, OP, 1, SG><<<grid, 256, 0, st>>>(s, items, m, tbit, pl); break;
	case 2: k_ctrl1q<T, OP, 2, SG><<<grid, 256, 0, st>>>(s, items, m, tbit, pl); break;
	case 3: k_ctrl1q<T, OP, 3, SG><<<grid, 256, 0, st>>>(s, items, m, tbit, pl); break;
	default: return cudaErrorInvalidValue;
	}
	note_launches(1);
	return cudaGetLastError();
}

// the Unit* forms carry the signs of their unit entries in m00.x / m01.x; they select the kernel
template <typename T, Op1 OP>
cudaError_t ctrl1q_nins(cplx_t<T>* s, uint64_t N, const Mat2<T>& m, uint64_t tbit, const BitPlan& pl, int sms, cudaStream_t st) {
	if constexpr (OP == Op1::UnitRe01 || OP == Op1::UnitRe10 || OP == Op1::UnitIm01 || OP == Op1::UnitIm10) {
		const int sgn = (m.m00.x < 0 ? 1 : 0) | (m.m01.x < 0 ? 2 : 0);
		switch (sgn) {
		case 0: return ctrl1q_sg<T, OP, 0>(s, N, m, tbit, pl, sms, st);
		case 1: return ctrl1q_sg<T, OP, 1>(s, N, m, tbit, pl, sms, st);
		case 2: return ctrl1q_sg<T, OP, 2>(s, N, m, tbit, pl, sms, st);
		default: return ctrl1q_sg<T, OP, 3>(s, N, m, tbit, pl, sms, st);
		}
	} else {
		return ctrl1q_sg<T, OP, 0>(s, N, m, tbit, pl, sms, st);
	}
}

template <typename T, SwapKind K>
cudaError_t swap_nins(cplx_t<T>* s, uint64_t N, uint64_t bitA, uint64_t bitB, const BitPlan& pl, int sms, cudaStream_t st) {
	const uint64_t items = N >> pl.nins;
	const int grid = grid_for(items, 256, sms);
	switch (pl.nins) {
	case 2: k_swap<T, K, 2><<<grid, 256, 0, st>>>(s, items, bitA, bitB, pl); break;
	case 3: k_swap<T, K, 3><<<grid, 256, 0, st>>>(s, items, bitA, bitB, pl); break;
	default: return cudaErrorInvalidValue;
	}
	note_launches(1);
	return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_ctrl1q(cplx_t<T>* s, uint64_t N, Op1 op, const Mat2<T>& m, uint64_t tbit, const BitPlan& pl, int sms,
                          cudaStream_t st) {
	if ((N >> pl.nins) == 0) return cudaSuccess;
	switch (op) {
	case Op1::Diag: return ctrl1q_nins<T, Op1::Diag>(s, N, m, tbit, pl, sms, st);
	case Op1::Phase: return ctrl1q_nins<T, Op1::Phase>(s, N, m, tbit, pl, sms, st);
	case Op1::PhaseNeg: return ctrl1q_nins<T, Op1::PhaseNeg>(s, N, m, tbit, pl, sms, st);
	case Op1::PhaseI: return ctrl1q_nins<T, Op1::PhaseI>(s, N, m, tbit, pl, sms, st);
	case Op1::Antidiag: return ctrl1q_nins<T, Op1::Antidiag>(s, N, m, tbit, pl, sms, st);
	case Op1::Swap: return ctrl1q_nins<T, Op1::Swap>(s, N, m, tbit, pl, sms, st);
	case Op1::Real: return ctrl1q_nins<T, Op1::Real>(s, N, m, tbit, pl, sms, st);
	case Op1::RxLike: return ctrl1q_nins<T, Op1::RxLike>(s, N, m, tbit, pl, sms, st);
	case Op1::Generic: return ctrl1q_nins<T, Op1::Generic>(s, N, m, tbit, pl, sms, st);
	case Op1::AntidiagUnit: return ctrl1q_nins<T, Op1::AntidiagUnit>(s, N, m, tbit, pl, sms, st);
	case Op1::UnitRe01: return ctrl1q_nins<T, Op1::UnitRe01>(s, N, m, tbit, pl, sms, st);
	case Op1::UnitRe10: return ctrl1q_nins<T, Op1::UnitRe10>(s, N, m, tbit, pl, sms, st);
	case Op1::UnitIm01: return ctrl1q_nins<T, Op1::UnitIm01>(s, N, m, tbit, pl, sms, st);
	case Op1::UnitIm10: return ctrl1q_nins<T, Op1::UnitIm10>(s, N, m, tbit, pl, sms, st);
	}
	return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_swap(cplx_t<T>* s, uint64_t N, SwapKind kind, uint64_t bitA, uint64_t bitB, const BitPlan& pl, int sms,
                        cudaStream_t st) {
	if ((N >> pl.nins) == 0) return cudaSuccess;
	switch (kind) {
	case SwapKind::Plain: return swap_nins<T, SwapKind::Plain>(s, N, bitA, bitB, pl, sms, st);
	case SwapKind::ISwap: return swap_nins<T, SwapKind::ISwap>(s, N, bitA, bitB, pl, sms, st);
	case SwapKind::ISwapDag: return swap_nins<T, SwapKind::ISwapDag>(s, N, bitA, bitB, pl, sms, st);
	}
	return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_dense(cplx_t<T>* s, uint64_t N, const DenseArgs& a, const BitPlan& pl, int sms, cudaStream_t st) {
	const uint64_t items = N >> pl.nins;
	if (items == 0) return cudaSuccess;
	DenseArgsT<T> t;
	const int D = 1 << a.k;
	for (int j = 0; j < 3; ++j) t.bit[j] = a.bit[j];
	for (int i = 0; i < 64; ++i) { t.m[i].x = 0; t.m[i].y = 0; }
	for (int i = 0; i < D * D; ++i) {
		t.m[i].x = static_cast<T>(a.m[2 * i]);
		t.m[i].y = static_cast<T>(a.m[2 * i + 1]);
	}
	const int grid = grid_for(items, 256, sms);
	if (a.k == 2 && pl.nins == 2) k_dense<T, 2, 2><<<grid, 256, 0, st>>>(s, items, t, pl);
	else if (a.k == 2 && pl.nins == 3) k_dense<T, 2, 3><<<grid, 256, 0, st>>>(s, items, t, pl);
	else if (a.k == 3 && pl.nins == 3) k_dense<T, 3, 3><<<grid, 256, 0, st>>>(s, items, t, pl);
	else return cudaErrorInvalidValue;
	note_launches(1);
	return cudaGetLastError();
}

template cudaError_t launch_ctrl1q<double>(double2*, uint64_t, Op1, const Mat2<double>&, uint64_t, const BitPlan&, int, cudaStream_t);
template cudaError_t launch_ctrl1q<float>(float2*, uint64_t, Op1, const Mat2<float>&, uint64_t, const BitPlan&, int, cudaStream_t);
template cudaError_t launch_swap<double>(double2*, uint64_t, SwapKind, uint64_t, uint64_t, const BitPlan&, int, cudaStream_t);
template cudaError_t launch_swap<float>(float2*, uint64_t, SwapKind, uint64_t, uint64_t, const BitPlan&, int, cudaStream_t);
template cudaError_t launch_dense<double>(double2*, uint64_t, const DenseArgs&, const BitPlan&, int, cudaStream_t);
template cudaError_t launch_dense<float>(float2*, uint64_t, const DenseArgs&, const BitPlan&, int, cudaStream_t);

}  // namespace qcs
