// Shared-memory pass kernel: each CTA loads a tile of 2^k amplitudes (contiguous runs of 2^L), applies
// every gate of the pass with the same per-amplitude arithmetic as the per-gate kernels (gate_math.cuh),
// and writes the tile back.  A persistent grid walks the 2^(n-k) tiles.
#include <algorithm>
#include <mutex>

#include "gate_math.cuh"
#include "tcgen05.cuh"
#include "tile.cuh"

namespace qcs {
namespace {

constexpr int kTileThreads = 512;
// tile loads in flight per thread (FP64 passes are FP64-pipe bound and keep their registers for occupancy)
template <typename T> constexpr int load_batch() { return sizeof(T) == 4 ? 8 : 1; }
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
		auto row_out = [&](int r) {
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
		};
		// small FP32 blocks: several rows in flight at once (their matrix loads overlap); larger
		// blocks one row at a time to bound the registers
		if constexpr (K <= 2 && sizeof(T) == 4) {
#pragma unroll
			for (int r = 0; r < D; ++r) row_out(r);
		} else if constexpr (K == 3 && sizeof(T) == 4) {
#pragma unroll 2
			for (int r = 0; r < D; ++r) row_out(r);
		} else {
#pragma unroll 1
			for (int r = 0; r < D; ++r) row_out(r);
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
	const cplx_t<T>* full = top.pad[4] ? reinterpret_cast<const cplx_t<T>*>(top.gtbit) : nullptr;
	const uint32_t lowmask = (1u << L) - 1;
	for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
		const uint32_t b = expand_local(i, op);
		const uint64_t g = base | highoff[b >> L] | (b & lowmask);
		const uint64_t z = ((g >> row_lo) & ymask) << shift;
		cplx_t<T> w = full ? full[z] : cmul<T>(hi[z >> S], lo[z & smask]);
		if (inverse) w.y = -w.y;
		sm[b] = cmul<T>(sm[b], w);
	}
}

// small fused FP32 blocks: each thread holds IPT items' inputs in registers, so that every matrix
// entry loaded serves IPT items (the matrix loads, not the FMAs, bound the one-item form)
template <typename T, int K, int IPT>
__device__ __forceinline__ void tile_denseN_multi(cplx_t<T>* sm, uint32_t items, const OpRegs op, const cplx_t<T>* __restrict__ mats) {
	constexpr int D = 1 << K;
	uint32_t bits[K];
#pragma unroll
	for (int j = 0; j < K; ++j) bits[j] = 1u << static_cast<uint32_t>((op.ins >> (8 * j)) & 0xffu);
	for (uint32_t i0 = threadIdx.x; i0 < items; i0 += blockDim.x * IPT) {
		uint32_t b[IPT];
		cplx_t<T> v[IPT][D];
#pragma unroll
		for (int it = 0; it < IPT; ++it) {
			const uint32_t i = i0 + it * blockDim.x;
			b[it] = expand_local(i < items ? i : i0, op);
#pragma unroll
			for (int c = 0; c < D; ++c) {
				uint32_t x = b[it];
#pragma unroll
				for (int j = 0; j < K; ++j)
					if ((c >> j) & 1) x |= bits[j];
				v[it][c] = sm[x];
			}
		}
#pragma unroll 1
		for (int r = 0; r < D; ++r) {
			const cplx_t<T>* row = mats + op.mat + r * D;
			T re[IPT], im[IPT];
#pragma unroll
			for (int it = 0; it < IPT; ++it) re[it] = im[it] = 0;
#pragma unroll
			for (int c = 0; c < D; ++c) {
				const cplx_t<T> mm = row[c];
#pragma unroll
				for (int it = 0; it < IPT; ++it) {
					re[it] = fma(mm.x, v[it][c].x, re[it]);
					re[it] = fma(-mm.y, v[it][c].y, re[it]);
					im[it] = fma(mm.x, v[it][c].y, im[it]);
					im[it] = fma(mm.y, v[it][c].x, im[it]);
				}
			}
			uint32_t rb = 0;
#pragma unroll
			for (int j = 0; j < K; ++j)
				if ((r >> j) & 1) rb |= bits[j];
#pragma unroll
			for (int it = 0; it < IPT; ++it)
				if (i0 + it * blockDim.x < items) sm[b[it] | rb] = mk<T>(re[it], im[it]);
		}
	}
}

// tile index -> the global bits of its non-tile qubits: three 256-entry tables over the index's bytes
// (a tile index has at most 24 bits: registers of at most 36 qubits, tiles of at least 12), built
// once per CTA so that a tile's base costs three shared-memory loads
constexpr int kFixChunks = 3;
__device__ __forceinline__ void build_fix_tables(uint64_t (*fixtab)[256], const TilePass& p) {
	for (uint32_t i = threadIdx.x; i < kFixChunks * 256; i += blockDim.x) {
		const uint32_t c = i >> 8, v = i & 255u;
		uint64_t off = 0;
		for (int b = 0; b < 8; ++b) {
			const int j = static_cast<int>(8 * c) + b;
			if (j < p.nfixed && ((v >> b) & 1u)) off |= 1ULL << p.fixed[j];
		}
		fixtab[c][v] = off;
	}
}
__device__ __forceinline__ uint64_t fixed_base(const uint64_t (*fixtab)[256], uint64_t tile) {
	return fixtab[0][tile & 255u] | fixtab[1][(tile >> 8) & 255u] | fixtab[2][(tile >> 16) & 255u];
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
		case 1: tile_denseN_multi<T, 1, 4>(sm, items, op, mats); break;
		case 2: tile_denseN_multi<T, 2, 4>(sm, items, op, mats); break;
		case 3: tile_denseN_multi<T, 3, 2>(sm, items, op, mats); break;
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

template <typename T>
__global__ void k_build_roots(cplx_t<T>* __restrict__ full, const cplx_t<T>* __restrict__ hilo, uint32_t M, uint32_t S) {
	const uint64_t n = 1ULL << M, smask = (1ULL << S) - 1;
	const cplx_t<T>* lo = hilo + (1ULL << (M - S));
	for (uint64_t z = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; z < n; z += static_cast<uint64_t>(gridDim.x) * blockDim.x)
		full[z] = cmul<T>(hilo[z >> S], lo[z & smask]);
}

template <typename T, bool DENSE, int THREADS>
__global__ void __launch_bounds__(THREADS) k_tile(cplx_t<T>* __restrict__ s, TilePass p, const TileOp* __restrict__ ops,
                                                 const cplx_t<T>* __restrict__ mats, uint64_t ntiles) {
	extern __shared__ __align__(1024) unsigned char smraw[];
	__shared__ uint64_t highoff[1 << kMaxHigh];
	__shared__ uint64_t fixtab[kFixChunks][256];
	cplx_t<T>* sm = reinterpret_cast<cplx_t<T>*>(smraw);
	const uint32_t K = 1u << p.k;
	build_fix_tables(fixtab, p);
	// the pass's operations: from shared memory (behind the tile) when the launcher left room for them
	const TileOp* opsrc = ops + p.op_begin;
	if (p.ops_in_smem) {
		TileOp* sops = reinterpret_cast<TileOp*>(smraw + static_cast<size_t>(K) * sizeof(cplx_t<T>));
		for (uint32_t i = threadIdx.x; i < p.op_count; i += blockDim.x) sops[i] = ops[p.op_begin + i];
		opsrc = sops;
	}
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
		const uint64_t base = fixed_base(fixtab, tile);
		// asynchronous 16-byte copies (one FP64 or two FP32 amplitudes, inside one run of 2^L >= 32),
		// all in flight at once without holding registers
		constexpr uint32_t kPer = 16 / sizeof(cplx_t<T>);
		for (uint32_t j = threadIdx.x * kPer; j < K; j += blockDim.x * kPer)
			tc::cp_async16(sm + j, s + (base | highoff[j >> p.L] | (j & lowmask)));
		tc::cp_async_wait_all();
		__syncthreads();
		for (uint32_t oi = 0; oi < p.op_count; ++oi) {
			const TileOp op = opsrc[oi];
			if ((base & op.gmask) != op.gmask) continue;
			if (static_cast<TKind>(op.kind) == TKind::TableDiag) {
				const cplx_t<T>* tab = reinterpret_cast<const cplx_t<T>*>(op.gtbit);
				for (uint32_t j = threadIdx.x; j < K; j += blockDim.x) sm[j] = cmul<T>(sm[j], tab[base | highoff[j >> p.L] | (j & lowmask)]);
			} else {
				tile_apply<T, DENSE>(sm, p.k, op, mats, base, highoff, p.L);
			}
			__syncthreads();
		}
		for (uint32_t j0 = threadIdx.x; j0 < K; j0 += blockDim.x * load_batch<T>()) {
			cplx_t<T> r[load_batch<T>()];
#pragma unroll
			for (int b = 0; b < load_batch<T>(); ++b) {
				const uint32_t j = j0 + b * blockDim.x;
				if (j < K) r[b] = sm[j];
			}
#pragma unroll
			for (int b = 0; b < load_batch<T>(); ++b) {
				const uint32_t j = j0 + b * blockDim.x;
				if (j < K) s[base | highoff[j >> p.L] | (j & lowmask)] = r[b];
			}
		}
		__syncthreads();
	}
}

// ---- tensor-core passes (FP32 registers, fused 4- and 5-qubit blocks) ----
//
// A block of K qubits (D = 2^K) acts on the tile's C = 2^12 / D "columns" (assignments of the other
// tile qubits).  As a real product: out (C x 2D) = in (C x 2D) * B (2D x 2D), in[c][2j + p] = part p of
// amplitude j of column c, B[2j][2i] = Re M[i][j], B[2j + 1][2i] = -Im M[i][j], B[2j][2i + 1] = Im M[i][j],
// B[2j + 1][2i + 1] = Re M[i][j].  Columns are the MMA's M dimension (tiles of 128 rows), 2D its N and
// K.  3xTF32: each operand is split into TF32 hi + lo parts and out = in_hi B_hi + in_hi B_lo + in_lo B_hi,
// accumulated in FP32 in tensor memory.
//
// Shared memory: the 32 KiB tile, the A operand (hi and lo splits) and the pass's block matrices (hi
// and lo, kTcMatBudget bytes), loaded once per CTA.
constexpr uint32_t kTcTileBytes = (1u << kTcTileQubits) * sizeof(float2);
constexpr uint32_t kTcLboA = 144;     // A operand: a row's core matrices fall in different bank groups
constexpr uint32_t kTcABytes = 36864;  // one split of A: 16 row groups x 16 core matrices x 144 bytes
constexpr uint32_t kTcSmem = kTcTileBytes + 2 * kTcABytes + kTcMatBudget;  // plus the pass's operations
constexpr uint32_t kTcSmemLimit = 216 * 1024;                                 // dynamic, with 9 KB static beside it
constexpr uint32_t kTcTmemCols = 128;  // per M tile: kdim accumulator columns + kdim hi*lo columns
constexpr uint32_t kTcWaitTries = 1u << 22;

__device__ __forceinline__ float tf32_rna(float x) {
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return __uint_as_float(r);
}

// the K block positions of a DenseTC op, ascending
template <int K> struct BlockBits {
	uint32_t pos[K];
	__device__ __forceinline__ explicit BlockBits(uint64_t ins) {
#pragma unroll
		for (int t = 0; t < K; ++t) pos[t] = static_cast<uint32_t>((ins >> (8 * t)) & 0xffu);
	}
	// tile index -> column (the index without the block bits)
	__device__ __forceinline__ uint32_t column(uint32_t x) const {
#pragma unroll
		for (int t = K - 1; t >= 0; --t) x = ((x >> (pos[t] + 1)) << pos[t]) | (x & ((1u << pos[t]) - 1));
		return x;
	}
	// tile index -> block index j
	__device__ __forceinline__ uint32_t index(uint32_t x) const {
		uint32_t j = 0;
#pragma unroll
		for (int t = 0; t < K; ++t) j |= ((x >> pos[t]) & 1u) << t;
		return j;
	}
	// (column, block index) -> tile index
	__device__ __forceinline__ uint32_t place(uint32_t c, uint32_t j) const {
#pragma unroll
		for (int t = 0; t < K; ++t) c = ((c >> pos[t]) << (pos[t] + 1)) | (c & ((1u << pos[t]) - 1)) | (((j >> t) & 1u) << pos[t]);
		return c;
	}
	__device__ __forceinline__ uint32_t low_count() const {
		uint32_t n = 0;
#pragma unroll
		for (int t = 0; t < K; ++t) n += pos[t] < 5 ? 1u : 0u;
		return n;
	}
};

// applies one DenseTC op of K qubits to the tile; false when the MMA completion wait ran out.
// Every index map of the op (tile index -> A-operand byte offset, tile index -> staging slot) is a sum
// of one weight per set tile bit, so a thread's eight elements (tile index = thread + 512 b) cost one
// 9-term sum for the thread's bits and three weights for b.
template <int K>
__device__ bool tile_block_tc(float2* sm, uint64_t ins, unsigned char* sA, const unsigned char* sBop, uint32_t tmem, uint64_t* mbar,
                              uint32_t& phase) {
	constexpr uint32_t D = 1u << K, kdim = 2 * D;
	constexpr uint32_t sbo_a = (kdim / 4) * kTcLboA, sbo_b = (kdim / 4) * 128;
	constexpr uint32_t cols = (1u << kTcTileQubits) >> K;  // 128 (K = 5) or 256 (K = 4)
	constexpr uint32_t mt_bytes = 16 * sbo_a;                // one 128-row M tile of one split
	constexpr uint32_t kTidBits = 9;                          // kTileThreads = 2^9
	static_assert(kTileThreads == (1 << kTidBits) && kTcTileQubits == kTidBits + 3, "tile index = thread + 512 b");
	const BlockBits<K> bb(ins);
	// per tile bit: byte offset in one A split (a block bit is bit t of j, the K index is 2j + part; a
	// column bit is bit r of the column: rows within a core matrix, row groups, then the M tile) and
	// slot in the staging area (slot = j (cols + 1) + column)
	uint32_t wa[kTcTileQubits], ws[kTcTileQubits];
	{
		uint32_t t = 0;
#pragma unroll
		for (uint32_t i = 0; i < kTcTileQubits; ++i) {
			if (t < K && bb.pos[t == K ? 0 : t] == i) {
				wa[i] = t == 0 ? 8u : (kTcLboA << (t - 1));
				ws[i] = (cols + 1) << t;
				++t;
			} else {
				const uint32_t r = i - t;
				wa[i] = r < 3 ? (16u << r) : (r < 7 ? (sbo_a << (r - 3)) : mt_bytes);
				ws[i] = 1u << r;
			}
		}
	}
	uint32_t a_tid = 0, s_tid = 0;
#pragma unroll
	for (uint32_t i = 0; i < kTidBits; ++i)
		if ((threadIdx.x >> i) & 1u) {
			a_tid += wa[i];
			s_tid += ws[i];
		}
	// gather in tile order (conflict-free reads) into the A operand, split into TF32 hi and lo
#pragma unroll
	for (uint32_t b = 0; b < 8; ++b) {
		const float2 v = sm[threadIdx.x + (b << kTidBits)];
		const uint32_t off = a_tid + ((b & 1u) ? wa[9] : 0u) + ((b & 2u) ? wa[10] : 0u) + ((b & 4u) ? wa[11] : 0u);
		const float hx = tf32_rna(v.x), hy = tf32_rna(v.y);
		*reinterpret_cast<float2*>(sA + off) = make_float2(hx, hy);
		*reinterpret_cast<float2*>(sA + kTcABytes + off) = make_float2(tf32_rna(v.x - hx), tf32_rna(v.y - hy));
	}
	tc::fence_proxy_async();
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	if (threadIdx.x == 0) {
		constexpr uint32_t idesc = tc::idesc_tf32(128, kdim), idesc2 = tc::idesc_tf32(128, 2 * kdim);
		const uint32_t a_hi = tc::smem_addr(sA), b_hi = tc::smem_addr(sBop);
		// descriptors of k-step 0; each k-step advances the start address (16-byte units, low bits)
		const uint64_t ah0 = tc::smem_desc(a_hi, kTcLboA, sbo_a), al0 = tc::smem_desc(a_hi + kTcABytes, kTcLboA, sbo_a);
		const uint64_t bh0 = tc::smem_desc(b_hi, 128, sbo_b);
#pragma unroll
		for (uint32_t mt = 0; mt < cols / 128; ++mt) {
#pragma unroll
			for (uint32_t ks = 0; ks < kdim / 8; ++ks) {
				const uint64_t da = (mt * mt_bytes + ks * 2 * kTcLboA) >> 4, db = (ks * 2 * 128) >> 4;
				// B_lo directly follows B_hi: one N = 2 kdim product gives hi*hi in the first kdim columns
				// and hi*lo in the next kdim; lo*hi accumulates onto the first
				tc::mma_tf32(tmem + mt * 2 * kdim, ah0 + da, bh0 + db, idesc2, ks > 0 ? 1u : 0u);
				tc::mma_tf32(tmem + mt * 2 * kdim, al0 + da, bh0 + db, idesc, 1u);
			}
		}
		tc::mma_commit(mbar);
	}
	const bool ok = tc::mbar_wait(mbar, phase, kTcWaitTries);
	phase ^= 1u;
	tc::fence_after_sync();
	// warp w reads tensor-memory lanes 32 (w % 4) + 0..31 (M-tile rows = columns), 16 accumulator
	// columns (8 complex outputs i0..i0 + 7) and the matching 16 hi*lo columns kdim further on
	const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
	const uint32_t quad = warp & 3u, cc = warp >> 2;
	const uint32_t mt = (16u * cc) / kdim, within = (16u * cc) % kdim, i0 = within / 2;  // i0: a multiple of 8
	float v[16], w[16];
	const uint32_t tcol = tmem + ((32u * quad) << 16) + mt * 2 * kdim + within;
	tc::tmem_ld16(tcol, v);
	tc::tmem_ld16(tcol + kdim, w);
#pragma unroll
	for (int q = 0; q < 16; ++q) v[q] += w[q];
	const uint32_t c = mt * 128u + 32u * quad + lane;
	// blocks on three or more of the five lowest tile bits: outputs go through a padded staging area
	// (the A operand is free now) and back to the tile in tile order; otherwise straight to the tile
	const bool staged = bb.low_count() >= 3;
	if (!staged) {
		const uint32_t x0 = bb.place(c, i0);
		const uint32_t p0 = 1u << bb.pos[0], p1 = 1u << bb.pos[1], p2 = 1u << bb.pos[2];
#pragma unroll
		for (uint32_t t = 0; t < 8; ++t)
			sm[x0 + ((t & 1u) ? p0 : 0u) + ((t & 2u) ? p1 : 0u) + ((t & 4u) ? p2 : 0u)] = make_float2(v[2 * t], v[2 * t + 1]);
	} else {
		float2* stage = reinterpret_cast<float2*>(sA);
#pragma unroll
		for (uint32_t t = 0; t < 8; ++t) stage[(i0 + t) * (cols + 1) + c] = make_float2(v[2 * t], v[2 * t + 1]);
	}
	tc::fence_before_sync();
	if (staged) {
		__syncthreads();
		const float2* stage = reinterpret_cast<const float2*>(sA);
#pragma unroll
		for (uint32_t b = 0; b < 8; ++b)
			sm[threadIdx.x + (b << kTidBits)] = stage[s_tid + ((b & 1u) ? ws[9] : 0u) + ((b & 2u) ? ws[10] : 0u) + ((b & 4u) ? ws[11] : 0u)];
	}
	return ok;
}

__global__ void __launch_bounds__(kTileThreads, 1) k_tile_tc(float2* __restrict__ s, TilePass p, const TileOp* __restrict__ ops,
                                                              const float2* __restrict__ mats, uint64_t ntiles, int* err) {
	extern __shared__ __align__(1024) unsigned char smraw[];
	__shared__ uint64_t highoff[1 << kMaxHigh];
	__shared__ uint64_t fixtab[kFixChunks][256];
	__shared__ __align__(8) uint64_t mbar_mma;
	__shared__ uint32_t tmem_slot;
	__shared__ int stop;
	float2* sm = reinterpret_cast<float2*>(smraw);
	unsigned char* sA = smraw + kTcTileBytes;
	unsigned char* sB = sA + 2 * kTcABytes;
	// the pass's operations, copied once (behind the block matrices)
	TileOp* sops = reinterpret_cast<TileOp*>(sB + kTcMatBudget);
	for (uint32_t i = threadIdx.x; i < p.op_count; i += blockDim.x) sops[i] = ops[p.op_begin + i];
	build_fix_tables(fixtab, p);
	const uint32_t warp = threadIdx.x >> 5;
	const uint32_t lowmask = (1u << p.L) - 1;
	const int nh = p.k - p.L;
	for (uint32_t h = threadIdx.x; h < (1u << nh); h += blockDim.x) {
		uint64_t off = 0;
		for (int b = 0; b < nh; ++b)
			if ((h >> b) & 1u) off |= 1ULL << p.high[b];
		highoff[h] = off;
	}
	if (warp == 0) tc::tmem_alloc<kTcTmemCols>(&tmem_slot);
	if (threadIdx.x == 0) {
		tc::mbar_init(&mbar_mma, 1);
		stop = 0;
	}
	// the pass's block matrices stay resident for every tile
	for (uint32_t oi = 0; oi < p.op_count; ++oi) {
		const TileOp& op = ops[p.op_begin + oi];
		if (static_cast<TKind>(op.kind) != TKind::DenseTC) continue;
		const uint32_t bytes = 32u << (2 * op.nins);
		const uint4* src = reinterpret_cast<const uint4*>(mats + op.mat);
		uint4* dst = reinterpret_cast<uint4*>(sB + op.lbit1);
		for (uint32_t i = threadIdx.x; i < bytes / 16; i += blockDim.x) dst[i] = src[i];
	}
	tc::fence_proxy_async();
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = tmem_slot;
	constexpr uint32_t kAmps = 1u << kTcTileQubits;
	constexpr int kBatch = kAmps / kTileThreads;  // 8 loads in flight per thread
	uint32_t mma_phase = 0;
	auto tile_base = [&](uint64_t tile) { return fixed_base(fixtab, tile); };
	// the next tile's amplitudes are loaded into registers while the current tile is processed
	float2 pre[kBatch];
	if (blockIdx.x < ntiles) {
		const uint64_t b0 = tile_base(blockIdx.x);
#pragma unroll
		for (int b = 0; b < kBatch; ++b) {
			const uint32_t j = threadIdx.x + b * kTileThreads;
			pre[b] = s[b0 | highoff[j >> p.L] | (j & lowmask)];
		}
	}
	for (uint64_t tile = blockIdx.x; tile < ntiles && !stop; tile += gridDim.x) {
		const uint64_t base = tile_base(tile);
#pragma unroll
		for (int b = 0; b < kBatch; ++b) sm[threadIdx.x + b * kTileThreads] = pre[b];
		const uint64_t next = tile + gridDim.x;
		if (next < ntiles) {
			const uint64_t nb = tile_base(next);
#pragma unroll
			for (int b = 0; b < kBatch; ++b) {
				const uint32_t j = threadIdx.x + b * kTileThreads;
				pre[b] = s[nb | highoff[j >> p.L] | (j & lowmask)];
			}
		}
		__syncthreads();
		for (uint32_t oi = 0; oi < p.op_count; ++oi) {
			const TileOp op = sops[oi];
			if ((base & op.gmask) != op.gmask) continue;
			if (static_cast<TKind>(op.kind) == TKind::DenseTC) {
				const bool ok = op.nins == 5 ? tile_block_tc<5>(sm, op.ins, sA, sB + op.lbit1, tmem, &mbar_mma, mma_phase)
				                             : tile_block_tc<4>(sm, op.ins, sA, sB + op.lbit1, tmem, &mbar_mma, mma_phase);
				if (!ok) {
					atomicExch(err, 1);
					stop = 1;
				}
			} else {
				tile_apply<float, true>(sm, p.k, op, mats, base, highoff, p.L);
			}
			__syncthreads();
			if (stop) break;
		}
		if (stop) break;
		{
			float2 r[kBatch];
#pragma unroll
			for (int b = 0; b < kBatch; ++b) r[b] = sm[threadIdx.x + b * kTileThreads];
#pragma unroll
			for (int b = 0; b < kBatch; ++b) {
				const uint32_t j = threadIdx.x + b * kTileThreads;
				s[base | highoff[j >> p.L] | (j & lowmask)] = r[b];
			}
		}
		__syncthreads();
	}
	if (stop) {
		// an MMA completion wait ran out (the error flag is set; the register's state is then undefined
		// and the host reports QCS_CUDA_ERROR): wait once more, again bounded, for the MMAs still in
		// flight, so that their tensor memory is not released under them
		tc::mbar_wait(&mbar_mma, mma_phase ^ 1u, kTcWaitTries);
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) tc::tmem_dealloc<kTcTmemCols>(tmem);
}

}  // namespace

template <> int tile_qubits<double>() { return 12; }
template <> int tile_qubits<float>() { return 13; }

namespace {
// kernel attributes and occupancies are per device: set up once per device (and per precision)
constexpr int kMaxDevices = 64;
std::mutex g_launch_mutex;

cudaError_t current_device(int* dev) {
	cudaError_t e = cudaGetDevice(dev);
	if (e == cudaSuccess && (*dev < 0 || *dev >= kMaxDevices)) e = cudaErrorInvalidDevice;
	return e;
}
}  // namespace

// largest dynamic shared memory of a pass CTA: the largest tile plus room for its operations
template <typename T> constexpr int maxs_of() {
	return static_cast<int>((size_t(1) << (sizeof(T) == 4 ? 13 : 12)) * sizeof(cplx_t<T>)) + 48 * 1024;
}

template <typename T>
cudaError_t launch_tile_pass(cplx_t<T>* s, const TilePass& p, const TileOp* d_ops, const cplx_t<T>* d_mats, int sms, cudaStream_t st,
                             int* d_err) {
	int dev = 0;
	if (cudaError_t e = current_device(&dev)) return e;
	if constexpr (sizeof(T) == 4) {
		if (p.dense == 2) {
			static bool tc_configured[kMaxDevices] = {};
			{
				std::lock_guard<std::mutex> lock(g_launch_mutex);
				if (!tc_configured[dev]) {
					cudaError_t e = cudaFuncSetAttribute(k_tile_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTcSmemLimit));
					if (e != cudaSuccess) return e;
					tc_configured[dev] = true;
				}
			}
			const size_t smem = kTcSmem + static_cast<size_t>(p.op_count) * sizeof(TileOp);
			if (p.k != kTcTileQubits || p.L < 5 || p.k - p.L > kMaxHigh || p.nfixed > 8 * kFixChunks || !d_err ||
			    smem > kTcSmemLimit)
				return cudaErrorInvalidValue;
			const uint64_t ntiles = 1ULL << p.nfixed;
			const uint64_t grid = std::min<uint64_t>(static_cast<uint64_t>(sms), ntiles);
			k_tile_tc<<<static_cast<unsigned>(grid), kTileThreads, smem, st>>>(s, p, d_ops, d_mats, ntiles, d_err);
			note_launches(1);
			return cudaGetLastError();
		}
	}
	// dense FP32 passes need many registers: 256 threads per CTA so that two CTAs share an SM (one
	// loading or storing its tile while the other computes)
	constexpr int kDenseThreads = sizeof(T) == 4 ? 256 : kTileThreads;
	auto* light = k_tile<T, false, kTileThreads>;
	auto* dense = k_tile<T, true, kDenseThreads>;
	static int per_sm_dev[kMaxDevices][2] = {};
	int* per_sm = per_sm_dev[dev];
	const size_t smem = (size_t(1) << p.k) * sizeof(cplx_t<T>);
	{
		std::lock_guard<std::mutex> lock(g_launch_mutex);
		if (!per_sm[0]) {
			const int maxs = static_cast<int>((size_t(1) << tile_qubits<T>()) * sizeof(cplx_t<T>));
			int occ[2] = {0, 0};
			cudaError_t e = cudaFuncSetAttribute(light, cudaFuncAttributeMaxDynamicSharedMemorySize, maxs_of<T>());
			if (e == cudaSuccess) e = cudaFuncSetAttribute(dense, cudaFuncAttributeMaxDynamicSharedMemorySize, maxs_of<T>());
			// resident CTAs per SM at the largest tile (registers and shared memory both counted)
			if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[0], light, kTileThreads, static_cast<size_t>(maxs));
			if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[1], dense, kDenseThreads, static_cast<size_t>(maxs));
			if (e != cudaSuccess) return e;
			per_sm[1] = std::max(occ[1], 1);
			per_sm[0] = std::max(occ[0], 1);
		}
	}
	if (p.k - p.L > kMaxHigh || p.k > tile_qubits<T>() || p.nfixed > 8 * kFixChunks) return cudaErrorInvalidValue;
	const uint64_t ntiles = 1ULL << p.nfixed;
	const int resident = per_sm[p.dense ? 1 : 0];
	const uint64_t grid = std::min<uint64_t>(static_cast<uint64_t>(sms) * resident, ntiles);
	// stage the operations in shared memory when that keeps the same number of CTAs per SM (228 KB per
	// SM, 1 KB reserved per CTA, 9 KB static per CTA)
	TilePass q = p;
	const size_t ops_bytes = static_cast<size_t>(p.op_count) * sizeof(TileOp);
	const size_t per_cta = (size_t(228) * 1024) / static_cast<size_t>(resident);
	q.ops_in_smem = smem + ops_bytes + 10 * 1024 <= per_cta && smem + ops_bytes <= static_cast<size_t>(maxs_of<T>()) ? 1 : 0;
	const size_t dyn = smem + (q.ops_in_smem ? ops_bytes : 0);
	if (p.dense) dense<<<static_cast<unsigned>(grid), kDenseThreads, dyn, st>>>(s, q, d_ops, d_mats, ntiles);
	else light<<<static_cast<unsigned>(grid), kTileThreads, dyn, st>>>(s, q, d_ops, d_mats, ntiles);
	note_launches(1);
	return cudaGetLastError();
}

template cudaError_t launch_tile_pass<double>(double2*, const TilePass&, const TileOp*, const double2*, int, cudaStream_t, int*);
template cudaError_t launch_tile_pass<float>(float2*, const TilePass&, const TileOp*, const float2*, int, cudaStream_t, int*);

template <typename T>
cudaError_t launch_build_roots(cplx_t<T>* full, const cplx_t<T>* hilo, uint32_t M, uint32_t S, int sms, cudaStream_t st) {
	k_build_roots<T><<<grid_for(1ULL << M, 256, sms), 256, 0, st>>>(full, hilo, M, S);
	note_launches(1);
	return cudaGetLastError();
}
template cudaError_t launch_build_roots<double>(double2*, const double2*, uint32_t, uint32_t, int, cudaStream_t);
template cudaError_t launch_build_roots<float>(float2*, const float2*, uint32_t, uint32_t, int, cudaStream_t);

}  // namespace qcs
