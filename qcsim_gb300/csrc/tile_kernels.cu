// Shared-memory pass kernel: each CTA loads a tile of 2^k amplitudes (contiguous runs of 2^L), applies
// every gate of the pass with the same per-amplitude arithmetic as the per-gate kernels (gate_math.cuh),
// and writes the tile back.  A persistent grid walks the 2^(n-k) tiles.
#include "gate_math.cuh"
#include "tile.cuh"

namespace qcs {
namespace {

constexpr int kTileThreads = 512;
constexpr int kMaxHigh = 8;  // at most 8 tile qubits above the contiguous low block

// the loop-invariant fields of a TileOp, held in registers
struct OpRegs {
	uint64_t ins;
	uint32_t nins, lset, lbit0, lbit1, lbit2, mat;
};

__device__ __forceinline__ uint32_t expand_local(uint32_t i, const OpRegs& op) {
	uint64_t packed = op.ins;
	for (uint32_t j = 0; j < op.nins; ++j) {
		const uint32_t b = static_cast<uint32_t>(packed & 0xffu);
		packed >>= 8;
		i = ((i >> b) << (b + 1)) | (i & ((1u << b) - 1));
	}
	return i | op.lset;
}

template <typename T> __device__ __forceinline__ Mat2<T> load_mat2(const cplx_t<T>* mats, uint32_t off) {
	Mat2<T> m;
	m.m00 = mats[off];
	m.m01 = mats[off + 1];
	m.m10 = mats[off + 2];
	m.m11 = mats[off + 3];
	return m;
}

template <typename T, Op1 OP, int SG = 0>
__device__ __forceinline__ void tile_ctrl1q(cplx_t<T>* sm, uint32_t items, const OpRegs op, const Mat2<T> m) {
	for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
		const uint32_t b = expand_local(i, op);
		cplx_t<T> a0, a1;
		if constexpr (touches_a0<OP>()) a0 = sm[b];
		a1 = sm[b | op.lbit0];
		op2<T, OP, SG>(a0, a1, m);
		if constexpr (touches_a0<OP>()) sm[b] = a0;
		sm[b | op.lbit0] = a1;
	}
}

template <typename T, Op1 OP>
__device__ __forceinline__ void tile_unit(cplx_t<T>* sm, uint32_t items, const OpRegs op, const Mat2<T> m) {
	const int sgn = (m.m00.x < 0 ? 1 : 0) | (m.m01.x < 0 ? 2 : 0);
	switch (sgn) {
	case 0: tile_ctrl1q<T, OP, 0>(sm, items, op, m); break;
	case 1: tile_ctrl1q<T, OP, 1>(sm, items, op, m); break;
	case 2: tile_ctrl1q<T, OP, 2>(sm, items, op, m); break;
	default: tile_ctrl1q<T, OP, 3>(sm, items, op, m); break;
	}
}

// diagonal whose target is not a tile qubit: one factor for the whole tile (restricted to local controls)
template <typename T, Op1 OP>
__device__ __forceinline__ void tile_globaldiag(cplx_t<T>* sm, uint32_t items, const OpRegs op, const Mat2<T> m, bool bit_set) {
	Mat2<T> mm = m;
	if constexpr (OP == Op1::Diag) {
		mm.m11 = bit_set ? m.m11 : m.m00;
	} else {
		if (bit_set != (op.lbit0 != 0)) return;
	}
	for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
		const uint32_t b = expand_local(i, op);
		cplx_t<T> a0, a1 = sm[b];
		if constexpr (OP == Op1::Diag) {
			a1 = cmul<T>(a1, mm.m11);
		} else {
			op2<T, OP>(a0, a1, mm);
		}
		sm[b] = a1;
	}
}

template <typename T, int K>
__device__ __forceinline__ void tile_dense(cplx_t<T>* sm, uint32_t items, const OpRegs op, const cplx_t<T>* __restrict__ mats) {
	constexpr int D = 1 << K;
	for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
		const uint32_t b = expand_local(i, op);
		// all inputs in registers first; each output row then goes straight to shared memory (no other
		// thread touches this group)
		cplx_t<T> v[D];
#pragma unroll
		for (int c = 0; c < D; ++c) {
			uint32_t x = b;
			if (c & 1) x |= op.lbit0;
			if (K > 1 && (c & 2)) x |= op.lbit1;
			if (K > 2 && (c & 4)) x |= op.lbit2;
			v[c] = sm[x];
		}
#pragma unroll 1
		for (int r = 0; r < D; ++r) {
			T re = 0, im = 0;
#pragma unroll
			for (int c = 0; c < D; ++c) {
				const cplx_t<T> mm = mats[op.mat + r * D + c];
				re += mm.x * v[c].x - mm.y * v[c].y;
				im += mm.x * v[c].y + mm.y * v[c].x;
			}
			uint32_t x = b;
			if (r & 1) x |= op.lbit0;
			if (K > 1 && (r & 2)) x |= op.lbit1;
			if (K > 2 && (r & 4)) x |= op.lbit2;
			sm[x] = mk<T>(re, im);
		}
	}
}

// fused block: 2^K x 2^K complex matrix, matrix bit j = the j-th (ascending) inserted local position
template <typename T, int K>
__device__ __forceinline__ void tile_denseN(cplx_t<T>* sm, uint32_t items, const OpRegs op, const cplx_t<T>* __restrict__ mats) {
	constexpr int D = 1 << K;
	uint32_t bits[K];
#pragma unroll
	for (int j = 0; j < K; ++j) bits[j] = 1u << static_cast<uint32_t>((op.ins >> (8 * j)) & 0xffu);
	for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
		const uint32_t b = expand_local(i, op);
		cplx_t<T> v[D];
#pragma unroll
		for (int c = 0; c < D; ++c) {
			uint32_t x = b;
#pragma unroll
			for (int j = 0; j < K; ++j)
				if ((c >> j) & 1) x |= bits[j];
			v[c] = sm[x];
		}
#pragma unroll 1
		for (int r = 0; r < D; ++r) {
			T re = 0, im = 0;
			const cplx_t<T>* row = mats + op.mat + r * D;
#pragma unroll
			for (int c = 0; c < D; ++c) {
				const cplx_t<T> mm = row[c];
				re = fma(mm.x, v[c].x, re);
				re = fma(-mm.y, v[c].y, re);
				im = fma(mm.x, v[c].y, im);
				im = fma(mm.y, v[c].x, im);
			}
			uint32_t x = b;
#pragma unroll
			for (int j = 0; j < K; ++j)
				if ((r >> j) & 1) x |= bits[j];
			sm[x] = mk<T>(re, im);
		}
	}
}

// QFT phase row: amplitudes with the target bit set (forced through lset when the target is a tile
// qubit, selected through gmask otherwise) are multiplied by exp(+-2 pi i y / 2^m), y read from the
// amplitude's global index; the root comes from two tables (high and low bits of z = y << shift)
template <typename T>
__device__ __forceinline__ void tile_phaserow(cplx_t<T>* sm, uint32_t items, const OpRegs op, const TileOp& top,
                                              const cplx_t<T>* __restrict__ mats, uint64_t base, const uint64_t* highoff, int L) {
	const uint32_t row_lo = op.lbit1, row_bits = op.lbit2;
	const uint32_t shift = top.pad[0], S = top.pad[1], M = top.pad[3];
	const bool inverse = top.pad[2] != 0;
	const uint64_t ymask = (1ULL << row_bits) - 1, smask = (1ULL << S) - 1;
	const cplx_t<T>* hi = mats + op.mat;
	const cplx_t<T>* lo = hi + (1ULL << (M - S));
	const uint32_t lowmask = (1u << L) - 1;
	for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
		const uint32_t b = expand_local(i, op);
		const uint64_t g = base | highoff[b >> L] | (b & lowmask);
		const uint64_t z = ((g >> row_lo) & ymask) << shift;
		cplx_t<T> w = cmul<T>(hi[z >> S], lo[z & smask]);
		if (inverse) w.y = -w.y;
		sm[b] = cmul<T>(sm[b], w);
	}
}

// DENSE: whether this instantiation carries the dense-block paths (they need many registers; passes
// without dense blocks run the lighter instantiation at higher occupancy)
template <typename T, bool DENSE>
__device__ __forceinline__ void tile_apply(cplx_t<T>* sm, int k, const TileOp& top, const cplx_t<T>* __restrict__ mats, uint64_t base,
                                           const uint64_t* highoff, int L) {
	const OpRegs op{top.ins, top.nins, top.lset, top.lbit0, top.lbit1, top.lbit2, top.mat};
	const uint32_t items = (1u << k) >> op.nins;
	const TKind kind = static_cast<TKind>(top.kind);
	if (kind == TKind::Ctrl1q) {
		const Mat2<T> m = load_mat2<T>(mats, op.mat);
		switch (static_cast<Op1>(top.op)) {
		case Op1::Diag: tile_ctrl1q<T, Op1::Diag>(sm, items, op, m); break;
		case Op1::Phase: tile_ctrl1q<T, Op1::Phase>(sm, items, op, m); break;
		case Op1::PhaseNeg: tile_ctrl1q<T, Op1::PhaseNeg>(sm, items, op, m); break;
		case Op1::PhaseI: tile_ctrl1q<T, Op1::PhaseI>(sm, items, op, m); break;
		case Op1::Antidiag: tile_ctrl1q<T, Op1::Antidiag>(sm, items, op, m); break;
		case Op1::AntidiagUnit: tile_ctrl1q<T, Op1::AntidiagUnit>(sm, items, op, m); break;
		case Op1::Swap: tile_ctrl1q<T, Op1::Swap>(sm, items, op, m); break;
		case Op1::Real: tile_ctrl1q<T, Op1::Real>(sm, items, op, m); break;
		case Op1::RxLike: tile_ctrl1q<T, Op1::RxLike>(sm, items, op, m); break;
		case Op1::Generic: tile_ctrl1q<T, Op1::Generic>(sm, items, op, m); break;
		case Op1::UnitRe01: tile_unit<T, Op1::UnitRe01>(sm, items, op, m); break;
		case Op1::UnitRe10: tile_unit<T, Op1::UnitRe10>(sm, items, op, m); break;
		case Op1::UnitIm01: tile_unit<T, Op1::UnitIm01>(sm, items, op, m); break;
		case Op1::UnitIm10: tile_unit<T, Op1::UnitIm10>(sm, items, op, m); break;
		}
	} else if (kind == TKind::GlobalDiag) {
		const Mat2<T> m = load_mat2<T>(mats, op.mat);
		const bool bit = (base & top.gtbit) != 0;
		switch (static_cast<Op1>(top.op)) {
		case Op1::Diag: tile_globaldiag<T, Op1::Diag>(sm, items, op, m, bit); break;
		case Op1::Phase: tile_globaldiag<T, Op1::Phase>(sm, items, op, m, bit); break;
		case Op1::PhaseNeg: tile_globaldiag<T, Op1::PhaseNeg>(sm, items, op, m, bit); break;
		case Op1::PhaseI: tile_globaldiag<T, Op1::PhaseI>(sm, items, op, m, bit); break;
		default: break;
		}
	} else if (kind == TKind::Swap) {
		const SwapKind sk = static_cast<SwapKind>(top.op);
		for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
			const uint32_t b = expand_local(i, op);
			const cplx_t<T> a = sm[b | op.lbit0], c = sm[b | op.lbit1];
			if (sk == SwapKind::Plain) {
				sm[b | op.lbit0] = c;
				sm[b | op.lbit1] = a;
			} else if (sk == SwapKind::ISwap) {
				sm[b | op.lbit0] = mk<T>(-c.y, c.x);
				sm[b | op.lbit1] = mk<T>(-a.y, a.x);
			} else {
				sm[b | op.lbit0] = mk<T>(c.y, -c.x);
				sm[b | op.lbit1] = mk<T>(a.y, -a.x);
			}
		}
	} else if (kind == TKind::PhaseRow) {
		tile_phaserow<T>(sm, items, op, top, mats, base, highoff, L);
	} else if constexpr (!DENSE) {
		return;
	} else if (kind == TKind::Dense2) {
		tile_dense<T, 2>(sm, items, op, mats);
	} else if (kind == TKind::Dense3) {
		tile_dense<T, 3>(sm, items, op, mats);
	} else if constexpr (sizeof(T) == 4) {
		// fused blocks (the FP32 path)
		switch (op.nins) {
		case 1: tile_denseN<T, 1>(sm, items, op, mats); break;
		case 2: tile_denseN<T, 2>(sm, items, op, mats); break;
		case 3: tile_denseN<T, 3>(sm, items, op, mats); break;
		case 4: tile_denseN<T, 4>(sm, items, op, mats); break;
		default: tile_denseN<T, 5>(sm, items, op, mats); break;
		}
	} else {
		switch (op.nins) {
		case 1: tile_denseN<T, 1>(sm, items, op, mats); break;
		case 2: tile_denseN<T, 2>(sm, items, op, mats); break;
		case 3: tile_denseN<T, 3>(sm, items, op, mats); break;
		default: tile_denseN<T, 4>(sm, items, op, mats); break;
		}
	}
}

template <typename T, bool DENSE>
__global__ void __launch_bounds__(kTileThreads) k_tile(cplx_t<T>* __restrict__ s, TilePass p, const TileOp* __restrict__ ops,
                                                      const cplx_t<T>* __restrict__ mats, uint64_t ntiles) {
	extern __shared__ __align__(16) unsigned char smraw[];
	__shared__ uint64_t highoff[1 << kMaxHigh];
	cplx_t<T>* sm = reinterpret_cast<cplx_t<T>*>(smraw);
	const uint32_t K = 1u << p.k;
	const uint32_t lowmask = (1u << p.L) - 1;
	const int nh = p.k - p.L;
	for (uint32_t h = threadIdx.x; h < (1u << nh); h += blockDim.x) {
		uint64_t off = 0;
		for (int b = 0; b < nh; ++b)
			if ((h >> b) & 1u) off |= 1ULL << p.high[b];
		highoff[h] = off;
	}
	__syncthreads();
	for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
		uint64_t base = 0;
		for (int j = 0; j < p.nfixed; ++j)
			if ((tile >> j) & 1ULL) base |= 1ULL << p.fixed[j];
		for (uint32_t j = threadIdx.x; j < K; j += blockDim.x) sm[j] = s[base | highoff[j >> p.L] | (j & lowmask)];
		__syncthreads();
		for (uint32_t oi = 0; oi < p.op_count; ++oi) {
			const TileOp op = ops[p.op_begin + oi];
			if ((base & op.gmask) != op.gmask) continue;
			tile_apply<T, DENSE>(sm, p.k, op, mats, base, highoff, p.L);
			__syncthreads();
		}
		for (uint32_t j = threadIdx.x; j < K; j += blockDim.x) s[base | highoff[j >> p.L] | (j & lowmask)] = sm[j];
		__syncthreads();
	}
}

}  // namespace

template <> int tile_qubits<double>() { return 12; }
template <> int tile_qubits<float>() { return 13; }

template <typename T>
cudaError_t launch_tile_pass(cplx_t<T>* s, const TilePass& p, const TileOp* d_ops, const cplx_t<T>* d_mats, int sms, cudaStream_t st) {
	static bool configured = false;
	const size_t smem = (size_t(1) << p.k) * sizeof(cplx_t<T>);
	if (!configured) {
		const int maxs = static_cast<int>((size_t(1) << tile_qubits<T>()) * sizeof(cplx_t<T>));
		cudaError_t e = cudaFuncSetAttribute(k_tile<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxs);
		if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tile<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxs);
		if (e != cudaSuccess) return e;
		configured = true;
	}
	if (p.k - p.L > kMaxHigh || p.k > tile_qubits<T>()) return cudaErrorInvalidValue;
	const uint64_t ntiles = 1ULL << p.nfixed;
	int per_sm = static_cast<int>((200 * 1024) / (smem + 4096));
	if (per_sm < 1) per_sm = 1;
	if (per_sm > 4) per_sm = 4;
	uint64_t grid = static_cast<uint64_t>(sms) * per_sm;
	if (grid > ntiles) grid = ntiles;
	if (p.dense) k_tile<T, true><<<static_cast<unsigned>(grid), kTileThreads, smem, st>>>(s, p, d_ops, d_mats, ntiles);
	else k_tile<T, false><<<static_cast<unsigned>(grid), kTileThreads, smem, st>>>(s, p, d_ops, d_mats, ntiles);
	note_launches(1);
	return cudaGetLastError();
}

template cudaError_t launch_tile_pass<double>(double2*, const TilePass&, const TileOp*, const double2*, int, cudaStream_t);
template cudaError_t launch_tile_pass<float>(float2*, const TilePass&, const TileOp*, const float2*, int, cudaStream_t);

}  // namespace qcs
