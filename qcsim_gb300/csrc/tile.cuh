// Shared-memory passes: one kernel applies a run of consecutive gates to the state with each CTA
// holding a tile of 2^k amplitudes in shared memory (the k "tile qubits" vary inside a tile, the
// other qubits are fixed per tile).  Low qubits 0..L-1 are always tile qubits, so every tile is read
// and written as contiguous runs of 2^L amplitudes.
#pragma once

#include <algorithm>

#include "engine.cuh"

namespace qcs {

// DenseN: a fused block's 2^nins x 2^nins matrix whose bit j is the j-th inserted position
// PhaseRow: a QFT phase row (CompiledGate::PhaseRow): lbit1 = row_lo, lbit2 = row_bits, pad[0] = the
// shift taking y to the table's 2^M-th roots, pad[1] = S, pad[2] = inverse, pad[3] = M; the factor
// exp(2 pi i z / 2^M), z = y << shift, is table[mat + (z >> S)] * table[mat + 2^(M-S) + (z & (2^S - 1))];
// with pad[4] = 1 it is full[z] instead, from a table of all 2^M roots at address gtbit
// DenseTC: a fused 4- or 5-qubit block (FP32 registers) on the tensor cores; ins = its local positions,
// mat = offset (complex entries, even) of its real-expanded 2D x 2D matrix as two TF32 splits in the
// K-major operand layout (hi then lo, 16 D^2 bytes each), lbit1 = its byte offset in the kernel's
// resident matrix area, gtbit = the tile positions that make up the row (tensor-memory lane) index,
// 4 bits each, row bit r in bits 4r..4r+3
// TableDiag: every amplitude of the tile times its entry of a 2^n-entry diagonal on the device (the
// table's address in gtbit); no inserted positions
// TileFactor: a diagonal gate whose target (gtbit) and controls (gmask) all lie outside the tile, so that it
// multiplies each tile by one scalar: mat[0] where the tile's target bit is clear, mat[1] where it is set, in
// tiles whose fixed bits include gmask; pad[0] = 1 when both entries differ from one (instruction counts
// only).  A pass's TileFactor operations come first (TilePass::nfactor); the kernel multiplies their product
// into the tile as it stores it, in place of one sweep of the tile per gate.
enum class TKind : uint8_t { Ctrl1q = 0, Swap = 1, Dense2 = 2, Dense3 = 3, GlobalDiag = 4, DenseN = 5, PhaseRow = 6, DenseTC = 7,
                             TableDiag = 8, TileFactor = 9 };

// every pass's tile holds qubits 0..L0-1, so that a tile moves between HBM and shared memory in runs of
// 2^L0 contiguous amplitudes (at least 128 bytes, a whole cache line); at most kMaxHigh tile qubits lie
// above the run.  The fewer qubits the run pins, the more gates or blocks one pass takes.
constexpr int kMinLowRun = 4;
constexpr int kMaxHigh = 8;
inline int low_run_qubits(int n, int kmax) { return std::min(n, std::max(kMinLowRun, kmax - kMaxHigh)); }

// tensor-core passes: tiles of exactly kTcTileQubits qubits; resident block matrices per pass
constexpr int kTcTileQubits = 12;
constexpr uint32_t kTcMatBudget = 65536;  // two 5-qubit blocks, or eight 4-qubit blocks

// A tensor-core pass keeps its tile in shared memory under an XOR swizzle: amplitude x of the tile sits
// at x ^ S(x >> 4), S linear over GF(2) with the 4-bit vectors tc_swizzle(b) for tile bits b = 4..11.
// Bits 0..3 add the unit vectors, and the twelve vectors are distinct and nonzero and avoid
// {0011, 1100, 1111}, which meets every 3-dimensional subspace of GF(2)^4; so any seven of them span
// GF(2)^4.  For a block on 4 or 5 tile bits, four of the remaining bits therefore change the low four
// bits of the address independently: 16 lanes reading 8-byte amplitudes along them use 16 bank pairs.
__host__ __device__ constexpr uint32_t tc_swizzle(int b) {
	return b < 4 ? 0u : static_cast<uint32_t>((0xEDBA9765ULL >> (4 * (b - 4))) & 15u);
}
// swizzled offset (in amplitudes) of tile bit b: the address of amplitude x is the XOR over its set bits
__host__ __device__ constexpr uint32_t tc_bit_offset(int b) { return (1u << b) ^ tc_swizzle(b); }

// one gate inside a pass, in tile-local bit positions
struct TileOp {
	uint8_t kind;      // TKind
	uint8_t op;        // Op1 (Ctrl1q, GlobalDiag) or SwapKind (Swap)
	uint8_t nins;      // number of local bit positions a work item does not enumerate (at most 8)
	uint8_t pad[5];
	uint64_t ins;      // those positions, ascending, 8 bits each (lowest byte first)
	uint32_t lset;     // local control bits (forced to one in every work item)
	uint32_t lbit0;    // Ctrl1q: target bit (0 = the factor sits on the target-bit-0 half); Swap: bit A; Dense: matrix bit 0
	uint32_t lbit1;    // Swap: bit B; Dense: matrix bit 1
	uint32_t lbit2;    // Dense3: matrix bit 2
	uint32_t mat;      // offset of the op's entries in the pass matrix table (complex entries)
	uint64_t gmask;    // non-tile controls: the op applies only in tiles whose fixed bits include these
	uint64_t gtbit;    // GlobalDiag: the non-tile target bit selecting m00 (clear) or m11 (set); TableDiag: the table's address
};

// per-pass geometry
struct TilePass {
	int k;                 // tile qubits
	int L;                 // qubits 0..L-1 are tile qubits
	int nfixed;            // n - k
	uint8_t high[32];      // global positions of local bits L..k-1
	uint8_t fixed[40];     // global positions of the non-tile qubits, ascending
	uint32_t op_begin, op_count;
	uint32_t nfactor;      // the first nfactor operations are TileFactor ones
	int dense;             // 0: light operations only; 1: dense blocks on the CUDA cores; 2: tensor-core blocks
	int ops_in_smem;       // set by the launcher: the CTA copies the pass's operations into shared memory
};

// d_err: set non-zero by a tensor-core pass whose bounded waits ran out (1: MMA completion, 2: tile load)
template <typename T>
cudaError_t launch_tile_pass(cplx_t<T>* s, const TilePass& p, const TileOp* d_ops, const cplx_t<T>* d_mats, int sms,
                             cudaStream_t st, int* d_err);

// full[z] = hilo[z >> S] * hilo[2^(M-S) + (z & (2^S - 1))] for z < 2^M: every 2^M-th root of unity, from the
// two-level tables of the phase rows (the same products the two-level form computes per amplitude)
template <typename T>
cudaError_t launch_build_roots(cplx_t<T>* full, const cplx_t<T>* hilo, uint32_t M, uint32_t S, int sms, cudaStream_t st);

// largest tile (qubits) for the precision, given the shared memory per block
template <typename T> int tile_qubits();

}  // namespace qcs
