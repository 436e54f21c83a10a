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
	__shared__ cplx_t<T> tile_factor;
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
		// asynchronous 16-byte copies (one FP64 or two FP32 amplitudes, inside one run of 2^L >= 16),
		// all in flight at once without holding registers
		constexpr uint32_t kPer = 16 / sizeof(cplx_t<T>);
		for (uint32_t j = threadIdx.x * kPer; j < K; j += blockDim.x * kPer)
			tc::cp_async16(sm + j, s + (base | highoff[j >> p.L] | (j & lowmask)));
		if (threadIdx.x == 0) {
			// the product of the pass's TileFactor operations for this tile, while the copies are in flight
			cplx_t<T> f = mk<T>(T(1), T(0));
			for (uint32_t oi = 0; oi < p.nfactor; ++oi) {
				const TileOp& op = opsrc[oi];
				if ((base & op.gmask) == op.gmask) f = cmul<T>(f, mats[op.mat + ((base & op.gtbit) ? 1u : 0u)]);
			}
			tile_factor = f;
		}
		tc::cp_async_wait_all();
		__syncthreads();
		for (uint32_t oi = p.nfactor; oi < p.op_count; ++oi) {
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
		const cplx_t<T> f = tile_factor;
		const bool scaled = f.x != T(1) || f.y != T(0);
		for (uint32_t j0 = threadIdx.x; j0 < K; j0 += blockDim.x * load_batch<T>()) {
			cplx_t<T> r[load_batch<T>()];
#pragma unroll
			for (int b = 0; b < load_batch<T>(); ++b) {
				const uint32_t j = j0 + b * blockDim.x;
				if (j < K) r[b] = scaled ? cmul<T>(sm[j], f) : sm[j];
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

// ---- tensor-core passes (FP32 registers, fused blocks on 4 or 5 tile qubits) ----
//
// A block of K qubits (D = 2^K) acts on the tile's 2^12 / D "columns" (assignments of the other tile
// qubits).  As a real product: out (C x 2D) = in (C x 2D) * B (2D x 2D), in[c][2j + p] = part p of
// amplitude j of column c, B[2j][2i] = Re M[i][j], B[2j + 1][2i] = -Im M[i][j], B[2j][2i + 1] = Im M[i][j],
// B[2j + 1][2i + 1] = Re M[i][j].  Columns are the MMA's M dimension (tiles of 128 rows), 2D its N and K.
// 3xTF32: each operand is split into TF32 hi + lo parts and out = in_hi B_hi + in_hi B_lo + in_lo B_hi,
// accumulated in FP32 in tensor memory.
//
// The A operand goes to tensor memory, not shared memory: each thread gathers the amplitudes of one
// column (one tensor-memory lane) from the swizzled tile, splits them and writes them with tcgen05.st;
// the MMAs read A from tensor memory and B (the pass's block matrices, resident in shared memory).
// Tensor memory per CTA: accumulators in columns [0, 128), A (hi and lo) in [128, 256).  Which tile
// bits make up the row (lane) index is chosen on the host per block (op.gtbit: 4-bit tile positions,
// row bit r in bits 4r..4r+3), so that the lanes of a half-warp read 16 different bank pairs.
// Shared memory: the 32 KiB tile and kTcMatBudget bytes of block matrices: two CTAs per SM, one
// computing while the other's MMAs run.
constexpr int kTcThreads = 256;
constexpr uint32_t kTcTileBytes = (1u << kTcTileQubits) * sizeof(float2);
constexpr uint32_t kTcSmem = kTcTileBytes + kTcMatBudget;  // plus the pass's operations
constexpr uint32_t kTcSmemLimit = 100 * 1024;               // dynamic; two CTAs per SM with the static tables
constexpr uint32_t kTcTmemCols = 256;
constexpr uint32_t kTcAcol = 128;  // first tensor-memory column of the A operands
constexpr uint32_t kTcWaitTries = 1u << 22;
constexpr int kTcLoads = (1 << kTcTileQubits) / kTcThreads;  // 16 amplitudes per thread and tile
static_assert(kTcThreads == 256 && kTcTileQubits == 12, "tile index = thread + 256 i");

// swizzled offset of tile index x (XOR of the offsets of its set bits)
__host__ __device__ constexpr uint32_t tc_offset(uint32_t x) {
	uint32_t o = 0;
	for (int b = 0; b < kTcTileQubits; ++b)
		if ((x >> b) & 1u) o ^= tc_bit_offset(b);
	return o;
}

// per block of a pass, computed once per CTA: the swizzled offset of every row index inside an M tile, and
// w[0..4] = the offsets of the block bits, w[5] = that of the M-tile row bit (K = 4)
struct TcTab {
	uint16_t row[128];
	uint16_t w[8];
};

// one block of K = 4 or 5 qubits on the tile: gather and split into tensor memory, 3xTF32 MMAs, then the
// outputs back into the tile.  false when the MMA completion wait ran out.
//   K = 5: one M tile (128 columns of 32 amplitudes); warp w: lanes 32 (w % 4) + 0..31, amplitudes
//          j in [16 (w / 4), 16 (w / 4) + 16)
//   K = 4: two M tiles (256 columns of 16 amplitudes); warp w: M tile w / 4, lanes 32 (w % 4) + 0..31,
//          all 16 amplitudes
template <int K>
__device__ bool tc_block(float2* sm, const TcTab& tab, const unsigned char* sBop, uint32_t tmem, uint64_t* mbar, uint32_t& phase,
                         int* mma_ok) {
	constexpr uint32_t D = 1u << K, kdim = 2 * D;
	constexpr uint32_t sbo_b = (kdim / 4) * 128;
	const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
	const uint32_t quad = warp & 3u, h = warp >> 2;
	const uint32_t m = 32u * quad + lane;  // row in the M tile
	// swizzled offsets of the block bits and of this thread's row
	uint32_t bw[K];
#pragma unroll
	for (int t = 0; t < K; ++t) bw[t] = tab.w[t];
	uint32_t rb = tab.row[m];
	if (K == 4 && h) rb ^= tab.w[5];     // the M tile's row bit
	if (K == 5 && h) rb ^= bw[K - 1];    // j = 16 h + jj
	// tensor-memory columns of this thread's A values and accumulators
	const uint32_t lanes = (32u * quad) << 16;
	const uint32_t a_hi = K == 5 ? kTcAcol + 32u * h : kTcAcol + 64u * h;
	const uint32_t a_lo = K == 5 ? kTcAcol + 64u + 32u * h : kTcAcol + 64u * h + 32u;
	const uint32_t acc = K == 5 ? 32u * h : 64u * h;
	const uint32_t hilo = K == 5 ? 64u + 32u * h : 64u * h + 32u;
	float2 av[16];
#pragma unroll
	for (uint32_t u = 0; u < 16; ++u)
		av[u] = sm[rb ^ ((u & 1u) ? bw[0] : 0u) ^ ((u & 2u) ? bw[1] : 0u) ^ ((u & 4u) ? bw[2] : 0u) ^ ((u & 8u) ? bw[3] : 0u)];
#pragma unroll
	for (uint32_t c8 = 0; c8 < 2; ++c8) {
		float hi[16], lo[16];
#pragma unroll
		for (uint32_t u = 0; u < 8; ++u) {
			const float2 v = av[8 * c8 + u];
			const float hx = tc::tf32_rna(v.x), hy = tc::tf32_rna(v.y);
			hi[2 * u] = hx;
			hi[2 * u + 1] = hy;
			lo[2 * u] = v.x - hx;  // exact; the tensor core reads it as TF32
			lo[2 * u + 1] = v.y - hy;
		}
		tc::tmem_st16(tmem + lanes + a_hi + 16u * c8, hi);
		tc::tmem_st16(tmem + lanes + a_lo + 16u * c8, lo);
	}
	tc::tmem_wait_st();
	tc::fence_before_sync();
	__syncthreads();
	if (threadIdx.x == 0) {
		tc::fence_after_sync();
		const uint64_t bh0 = tc::smem_desc(tc::smem_addr(sBop), 128, sbo_b);
		constexpr uint32_t nmt = K == 5 ? 1u : 2u;
		constexpr uint32_t idesc2 = tc::idesc_tf32(128, 2 * kdim), idesc1 = tc::idesc_tf32(128, kdim);
#pragma unroll
		for (uint32_t mt = 0; mt < nmt; ++mt) {
			const uint32_t d = tmem + mt * 2u * kdim;
			const uint32_t ah = tmem + kTcAcol + mt * 2u * kdim, al = ah + kdim;
#pragma unroll
			for (uint32_t ks = 0; ks < kdim / 8; ++ks) {
				const uint64_t db = (ks * 2 * 128) >> 4;  // a k-step is two core matrices of B along K
				// B_lo directly follows B_hi: one N = 2 kdim product gives hi*hi in the first kdim columns
				// and hi*lo in the next kdim; lo*hi accumulates onto the first
				tc::mma_tf32_ta(d, ah + 8u * ks, bh0 + db, idesc2, ks > 0 ? 1u : 0u);
				tc::mma_tf32_ta(d, al + 8u * ks, bh0 + db, idesc1, 1u);
			}
		}
		tc::mma_commit(mbar);
		// the issuing thread alone waits for the MMAs (bounded); the others wait at the barrier below
		// instead of polling the mbarrier, which leaves the issue slots to the SM's other CTA
		*mma_ok = tc::mbar_wait(mbar, phase, kTcWaitTries) ? 1 : 0;
		tc::fence_before_sync();
	}
	__syncthreads();
	tc::fence_after_sync();
	const bool ok = *mma_ok != 0;
	phase ^= 1u;
#pragma unroll
	for (uint32_t c8 = 0; c8 < 2; ++c8) {
		float v[16], w[16];
		tc::tmem_ld16x2(tmem + lanes + acc + 16u * c8, tmem + lanes + hilo + 16u * c8, v, w);
		const uint32_t base = rb ^ (c8 ? bw[3] : 0u);
#pragma unroll
		for (uint32_t u = 0; u < 8; ++u) {
			const uint32_t off = base ^ ((u & 1u) ? bw[0] : 0u) ^ ((u & 2u) ? bw[1] : 0u) ^ ((u & 4u) ? bw[2] : 0u);
			sm[off] = make_float2(v[2 * u] + w[2 * u], v[2 * u + 1] + w[2 * u + 1]);
		}
	}
	tc::fence_before_sync();
	return ok;
}

__global__ void __launch_bounds__(kTcThreads, 2) k_tile_tc(float2* __restrict__ s, TilePass p, const TileOp* __restrict__ ops,
                                                           const float2* __restrict__ mats, uint64_t ntiles, int* err) {
	extern __shared__ __align__(1024) unsigned char smraw[];
	__shared__ uint64_t highoff[1 << kMaxHigh];
	__shared__ uint64_t fixtab[kFixChunks][256];
	__shared__ __align__(8) uint64_t mbar_mma;
	__shared__ uint32_t tmem_slot;
	__shared__ int stop;
	__shared__ int mma_ok;
	float2* sm = reinterpret_cast<float2*>(smraw);
	unsigned char* sB = smraw + kTcTileBytes;
	// the pass's operations, copied once (behind the block matrices), and their row tables
	TileOp* sops = reinterpret_cast<TileOp*>(sB + kTcMatBudget);
	TcTab* tabs = reinterpret_cast<TcTab*>(sops + p.op_count);
	for (uint32_t i = threadIdx.x; i < p.op_count; i += blockDim.x) {
		const TileOp op = ops[p.op_begin + i];
		sops[i] = op;
		for (int t = 0; t < 8; ++t)
			tabs[i].w[t] = static_cast<uint16_t>(t < op.nins ? tc_bit_offset(static_cast<int>((op.ins >> (8 * t)) & 0xffu))
			                                     : (t == 5 ? tc_bit_offset(static_cast<int>((op.gtbit >> 28) & 15u)) : 0u));
	}
	for (uint32_t e = threadIdx.x; e < p.op_count * 128u; e += blockDim.x) {
		const uint32_t i = e >> 7, m = e & 127u;
		const uint64_t order = ops[p.op_begin + i].gtbit;
		uint32_t o = 0;
		for (int r = 0; r < 7; ++r)
			if ((m >> r) & 1u) o ^= tc_bit_offset(static_cast<int>((order >> (4 * r)) & 15u));
		tabs[i].row[m] = static_cast<uint16_t>(o);
	}
	build_fix_tables(fixtab, p);
	const uint32_t warp = threadIdx.x >> 5;
	const uint32_t L = static_cast<uint32_t>(p.L), nops = p.op_count;
	const uint32_t lowmask = (1u << L) - 1;
	const int nh = p.k - p.L;
	for (uint32_t hh = threadIdx.x; hh < (1u << nh); hh += blockDim.x) {
		uint64_t off = 0;
		for (int b = 0; b < nh; ++b)
			if ((hh >> b) & 1u) off |= 1ULL << p.high[b];
		highoff[hh] = off;
	}
	if (warp == 0) tc::tmem_alloc<kTcTmemCols>(&tmem_slot);
	if (threadIdx.x == 0) {
		tc::mbar_init(&mbar_mma, 1);
		stop = 0;
	}
	// the pass's block matrices stay resident for every tile
	for (uint32_t oi = 0; oi < p.op_count; ++oi) {
		const TileOp& op = ops[p.op_begin + oi];
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
	uint32_t mma_phase = 0;
	// this thread's amplitudes of a tile: x = thread + 256 i; swizzled offsets tid_off ^ tc_offset(256 i)
	const uint32_t tid_off = tc_offset(threadIdx.x);
	float2 pre[kTcLoads];
	if (blockIdx.x < ntiles) {
		const uint64_t b0 = fixed_base(fixtab, blockIdx.x);
#pragma unroll
		for (int i = 0; i < kTcLoads; ++i) {
			const uint32_t x = threadIdx.x + kTcThreads * i;
			pre[i] = s[b0 | highoff[x >> L] | (x & lowmask)];
		}
	}
	for (uint64_t tile = blockIdx.x; tile < ntiles && !stop; tile += gridDim.x) {
		const uint64_t base = fixed_base(fixtab, tile);
#pragma unroll
		for (int i = 0; i < kTcLoads; ++i) sm[tid_off ^ tc_offset(kTcThreads * i)] = pre[i];
		const uint64_t next = tile + gridDim.x;
		if (next < ntiles) {
			const uint64_t nb = fixed_base(fixtab, next);
#pragma unroll
			for (int i = 0; i < kTcLoads; ++i) {
				const uint32_t x = threadIdx.x + kTcThreads * i;
				pre[i] = s[nb | highoff[x >> L] | (x & lowmask)];
			}
		}
		__syncthreads();
		for (uint32_t oi = 0; oi < nops; ++oi) {
			const TileOp& op = sops[oi];
			const bool ok = op.nins == 5 ? tc_block<5>(sm, tabs[oi], sB + op.lbit1, tmem, &mbar_mma, mma_phase, &mma_ok)
			                             : tc_block<4>(sm, tabs[oi], sB + op.lbit1, tmem, &mbar_mma, mma_phase, &mma_ok);
			if (!ok) {
				atomicExch(err, 1);
				stop = 1;
			}
			__syncthreads();
			if (stop) break;
		}
		if (stop) break;
		{
			float2 r[kTcLoads];
#pragma unroll
			for (int i = 0; i < kTcLoads; ++i) r[i] = sm[tid_off ^ tc_offset(kTcThreads * i)];
#pragma unroll
			for (int i = 0; i < kTcLoads; ++i) {
				const uint32_t x = threadIdx.x + kTcThreads * i;
				s[base | highoff[x >> L] | (x & lowmask)] = r[i];
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
			const size_t smem = kTcSmem + static_cast<size_t>(p.op_count) * (sizeof(TileOp) + sizeof(TcTab));
			if (p.k != kTcTileQubits || p.L < kMinLowRun || p.k - p.L > kMaxHigh || p.nfixed > 8 * kFixChunks || !d_err ||
			    smem > kTcSmemLimit)
				return cudaErrorInvalidValue;
			const uint64_t ntiles = 1ULL << p.nfixed;
			const uint64_t grid = std::min<uint64_t>(2ULL * static_cast<uint64_t>(sms), ntiles);
			k_tile_tc<<<static_cast<unsigned>(grid), kTcThreads, smem, st>>>(s, p, d_ops, d_mats, ntiles, d_err);
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
