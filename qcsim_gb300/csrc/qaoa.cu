// Batched QAOA: many Ising instances of different sizes, all statevectors resident in HBM, every
// layer of every instance in one persistent kernel launch (replayed from a CUDA graph).
//
// The circuit is the reference's QAOAIsingSubalgorithm::Exec (IsingModel.h:557-567): H on every
// qubit, then per layer the Ising operator -- CNOT(i<-j) RZ(2 gamma J_ij)(i) CNOT(i<-j) per edge and
// RZ(gamma h_i) per field (IsingModel.h:491-531) -- and the mixer RX(2 beta) on every qubit
// (:533-554).  The Ising operator is diagonal: amplitude x gets exp(-i gamma (K(x) + sum_q h_q s_q / 2))
// with s = +1 for a 0 bit and K(x) = sum_ij J_ij s_i s_j.  With integer J, exp(-i gamma K) comes from a
// table over K; the field factor from two tables over the low and high qubit groups.  The mixer is
// the factored RX of the per-gate kernels (one FMA per real component), its scalar kept per instance.
// <H> = sum_x |psi_x|^2 E(x), E(x) = -(sum h_q s_q + sum J_ij s_i s_j) (IsingModel.h:106-119, 203-206),
// is reduced in FP64 in a fixed order.
//
// K(x) is never summed edge by edge per amplitude.  With the qubits split into the low group (the
// first g0 = min(n, 12) qubits, one tile) and the high group, K = K_low(x_low) + K_high(x_high) +
// sum_{i low} s_i c_i(x_high), c_i = sum of J_ij s_j over i's edges into the high group.  K_low is a
// per-instance table; per tile (x_high fixed) K_high and the c_i are computed once, and the cross
// term comes from two 64-entry tables over the low group's two 6-bit halves.
//
// Work split: instances sorted by size (largest first) are dealt round-robin to thread-block
// clusters; the CTAs of a cluster share an instance's tiles and meet at a cluster barrier between
// passes.  No CTA waits on another cluster, so the kernel needs no inter-CTA flags.
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include <cooperative_groups.h>

#include "engine.cuh"
#include "gate_math.cuh"
#include "tcgen05.cuh"

namespace cg = cooperative_groups;

namespace qcs {
namespace {

constexpr int kQThreads = 512;
constexpr int kGroupBits = 12;   // tile / table group size
constexpr int kMaxEdges = 64;
constexpr int kMaxK = 192;       // |K| bound for the table over K (integer couplings)
constexpr int kMaxLayers = 16;

struct QInst {
	uint64_t offset;       // first amplitude in the batch buffer
	uint64_t part_offset;  // first energy partial
	uint32_t n, nedges;
	uint32_t g0;           // low group bits = min(n, 12)
	uint32_t kmax;         // sum |J|
	uint32_t tab;          // complex-table offset: per layer [2*kmax+1] + [2^g0] + [2^(n-g0)]
	uint32_t eh;           // double-table offset: [2^g0] + [2^(n-g0)] field energies
	uint32_t kl;           // int16-table offset: [2^g0] K over the edges inside the low group
	uint16_t nlow, nhigh;  // edges [0, nlow) inside the low group, [nlow, nlow + nhigh) inside the high
	                       // group, the rest cross the groups with ei low and ej high
	uint8_t ei[kMaxEdges], ej[kMaxEdges];
	int8_t J[kMaxEdges];
	uint32_t tab_stride;   // complex entries per layer
	uint32_t pad;
};

struct QLayer {
	double x0, x1;  // factored RX coefficients
	int form;       // 0: UnitIm01, 1: UnitIm10
	int pad;
};

template <typename T> struct QParams {
	cplx_t<T>* amps;
	const QInst* inst;
	const uint32_t* order;        // instance indices, largest first
	uint32_t ninst;
	uint32_t p;
	const cplx_t<T>* tabs;
	const double* etab;
	const int16_t* kltab;
	const QLayer* layers;         // [inst][layer]
	double* parts;                // energy partials
	double* energies;             // out
	double* scale2;               // |scale|^2 per instance
	uint32_t stage_low, stage_high;  // mixer-pass tile: 2^stage_low contiguous amplitudes x stage_high qubits
};

// tile of the pass: qubits 0..L-1 and `nh` high qubits starting at `hq0`; the other qubits index tiles
struct TileGeo {
	uint32_t L, hq0, nh, n;
	__device__ uint64_t addr(uint64_t tile, uint32_t j) const {
		const uint64_t low = j & ((1u << L) - 1);
		const uint64_t high = static_cast<uint64_t>(j >> L) << hq0;
		// tile bits fill the positions outside [0, L) and [hq0, hq0 + nh)
		const uint32_t gap = hq0 - L;  // qubits L..hq0-1
		const uint64_t tmid = tile & ((1ULL << gap) - 1);
		const uint64_t thigh = tile >> gap;
		return low | (tmid << L) | high | (thigh << (hq0 + nh));
	}
	__device__ uint64_t ntiles() const { return 1ULL << (n - L - nh); }
	__device__ uint32_t size() const { return 1u << (L + nh); }
};

template <typename T>
__device__ __forceinline__ void rx_pair(cplx_t<T>& a0, cplx_t<T>& a1, const Mat2<T>& m, int form) {
	if (form == 0) op2<T, Op1::UnitIm01, 0>(a0, a1, m);
	else op2<T, Op1::UnitIm10, 0>(a0, a1, m);
}

template <typename T>
__device__ void rx_local(cplx_t<T>* sm, uint32_t k, uint32_t lo, uint32_t hi, const QLayer& L) {
	// RX on local bits lo..hi-1 of a 2^k tile; in a two-bit sweep each item holds the four amplitudes
	// of one (bit a, bit b) square and applies RX on a to both a-pairs, then on b
	Mat2<T> m;
	m.m00 = mk<T>(1, static_cast<T>(L.x0));
	m.m01 = mk<T>(1, static_cast<T>(L.x1));
	uint32_t b = lo;
	// FP32: two bits per sweep; FP64 keeps one (four double amplitudes per item cost the registers
	// that hold two CTAs per SM)
	for (; sizeof(T) == 4 && b + 1 < hi; b += 2) {
		const uint32_t ba = 1u << b, bb = 2u << b;
		const uint32_t items = (1u << k) >> 2;
		for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
			// insert zeros at bits b and b + 1
			const uint32_t i0 = ((i >> b) << (b + 2)) | (i & (ba - 1));
			cplx_t<T> a00 = sm[i0], a10 = sm[i0 | ba], a01 = sm[i0 | bb], a11 = sm[i0 | ba | bb];
			rx_pair<T>(a00, a10, m, L.form);
			rx_pair<T>(a01, a11, m, L.form);
			rx_pair<T>(a00, a01, m, L.form);
			rx_pair<T>(a10, a11, m, L.form);
			sm[i0] = a00;
			sm[i0 | ba] = a10;
			sm[i0 | bb] = a01;
			sm[i0 | ba | bb] = a11;
		}
		__syncthreads();
	}
	for (; b < hi; ++b) {
		const uint32_t bit = 1u << b;
		const uint32_t items = (1u << k) >> 1;
		for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
			const uint32_t i0 = ((i >> b) << (b + 1)) | (i & (bit - 1));
			cplx_t<T> a0 = sm[i0], a1 = sm[i0 | bit];
			rx_pair<T>(a0, a1, m, L.form);
			sm[i0] = a0;
			sm[i0 | bit] = a1;
		}
		__syncthreads();
	}
}

// tile loads and stores with several loads in flight per thread
template <typename T> constexpr int qaoa_batch() { return sizeof(T) == 4 ? 4 : 2; }

template <typename T>
__device__ __forceinline__ void tile_load(cplx_t<T>* sm, const cplx_t<T>* s, const TileGeo& G, uint64_t t, uint32_t K) {
	// asynchronous 16-byte copies (one FP64 or two FP32 amplitudes, inside one run of 2^L >= 2)
	constexpr uint32_t kPer = 16 / sizeof(cplx_t<T>);
	for (uint32_t j = threadIdx.x * kPer; j < K; j += kQThreads * kPer) tc::cp_async16(sm + j, s + G.addr(t, j));
	tc::cp_async_wait_all();
	__syncthreads();
}

template <typename T>
__device__ __forceinline__ void tile_store(const cplx_t<T>* sm, cplx_t<T>* s, const TileGeo& G, uint64_t t, uint32_t K) {
	constexpr int B = qaoa_batch<T>();
	for (uint32_t j0 = threadIdx.x; j0 < K; j0 += kQThreads * B) {
		cplx_t<T> r[B];
#pragma unroll
		for (int b = 0; b < B; ++b) {
			const uint32_t j = j0 + b * kQThreads;
			if (j < K) r[b] = sm[j];
		}
#pragma unroll
		for (int b = 0; b < B; ++b) {
			const uint32_t j = j0 + b * kQThreads;
			if (j < K) s[G.addr(t, j)] = r[b];
		}
	}
}

// per tile of the low-group geometry (x_high = t): K_high and the cross-term tables kc[0..63] (low
// bits 0-5) and kc[64..127] (low bits 6-11); ends with a barrier
__device__ __forceinline__ void cross_tables(const QInst& I, uint64_t t, int* kc, int* khigh, int* cvec) {
	const uint32_t g0 = I.g0;
	if (threadIdx.x < g0) {
		int c = 0;
		for (uint32_t e = I.nlow + I.nhigh; e < I.nedges; ++e)
			if (I.ei[e] == threadIdx.x) c += ((t >> (I.ej[e] - g0)) & 1ULL) ? -I.J[e] : I.J[e];
		cvec[threadIdx.x] = c;
	} else if (threadIdx.x == 32) {
		int k = 0;
		for (uint32_t e = I.nlow; e < I.nlow + I.nhigh; ++e) {
			const uint64_t par = ((t >> (I.ei[e] - g0)) ^ (t >> (I.ej[e] - g0))) & 1ULL;
			k += par ? -I.J[e] : I.J[e];
		}
		*khigh = k;
	}
	__syncthreads();
	if (threadIdx.x < 128) {
		const uint32_t half = threadIdx.x >> 6, u = threadIdx.x & 63u;
		int k = 0;
		for (uint32_t b = 0; b < 6; ++b) {
			const uint32_t q = 6 * half + b;
			if (q < g0) k += ((u >> b) & 1u) ? -cvec[q] : cvec[q];
		}
		kc[threadIdx.x] = k;
	}
	__syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kQThreads, 2) k_qaoa(QParams<T> P) {
	extern __shared__ __align__(16) unsigned char smraw[];
	cplx_t<T>* sm = reinterpret_cast<cplx_t<T>*>(smraw);
	__shared__ double red[kQThreads];
	__shared__ int kc[128];
	__shared__ int cvec[kGroupBits];
	__shared__ int khigh;
	cg::cluster_group cluster = cg::this_cluster();
	const uint32_t crank = cluster.block_rank();
	const uint32_t csize = cluster.num_blocks();
	const uint32_t nclusters = gridDim.x / csize;
	const uint32_t cid = blockIdx.x / csize;
	for (uint32_t w = cid; w < P.ninst; w += nclusters) {
		const QInst& I = P.inst[P.order[w]];
		cplx_t<T>* s = P.amps + I.offset;
		const uint32_t n = I.n;
		const uint32_t g0 = I.g0;
		const uint32_t sh = P.stage_high;
		const uint32_t nstages = (n > g0) ? ((n - g0 + sh - 1) / sh) : 0;  // high-qubit mixer passes
		const int16_t* KL = P.kltab + I.kl;
		TileGeo G0;  // the low-group geometry: tile = x_low, tile index = x_high
		G0.n = n; G0.L = g0; G0.hq0 = g0; G0.nh = 0;
		for (uint32_t l = 0; l < P.p; ++l) {
			const QLayer Lr = P.layers[static_cast<size_t>(P.order[w]) * P.p + l];
			const cplx_t<T>* tabJ = P.tabs + I.tab + static_cast<size_t>(l) * I.tab_stride;
			const cplx_t<T>* tab0 = tabJ + (2 * I.kmax + 1);
			const cplx_t<T>* tab1 = tab0 + (1u << g0);
			for (uint32_t stage = 0; stage <= nstages; ++stage) {
				TileGeo G = G0;
				if (stage > 0) {
					const uint32_t lo = g0 + sh * (stage - 1);
					G.L = P.stage_low; G.hq0 = lo; G.nh = min(sh, n - lo);
				}
				const uint64_t ntiles = G.ntiles();
				const uint32_t K = G.size();
				for (uint64_t t = crank; t < ntiles; t += csize) {
					tile_load<T>(sm, s, G, t, K);
					if (stage == 0) {
						// the Ising operator on every amplitude of the tile, then RX on the low qubits
						cross_tables(I, t, kc, &khigh, cvec);
						const int kbase = khigh + static_cast<int>(I.kmax);
						const cplx_t<T> fh = tab1[t];
						for (uint32_t j = threadIdx.x; j < K; j += blockDim.x) {
							const int kk = KL[j] + kbase + kc[j & 63u] + kc[64 + (j >> 6)];
							const cplx_t<T> f = cmul<T>(cmul<T>(tabJ[kk], tab0[j]), fh);
							sm[j] = cmul<T>(sm[j], f);
						}
						__syncthreads();
						rx_local<T>(sm, G.L, 0, G.L, Lr);
					} else {
						__syncthreads();
						rx_local<T>(sm, G.L + G.nh, G.L, G.L + G.nh, Lr);
					}
					tile_store<T>(sm, s, G, t, K);
					__syncthreads();
				}
				cluster.sync();
			}
		}
		// <H> = sum |a|^2 E(x): one read-only pass in the low-group geometry, partials per tile
		{
			const double* eh0 = P.etab + I.eh;
			const double* eh1 = eh0 + (1u << g0);
			const uint64_t ntiles = G0.ntiles();
			const uint32_t K = G0.size();
			for (uint64_t t = crank; t < ntiles; t += csize) {
				tile_load<T>(sm, s, G0, t, K);
				cross_tables(I, t, kc, &khigh, cvec);
				const double ebase = static_cast<double>(khigh) + eh1[t];
				double acc = 0;
				for (uint32_t j = threadIdx.x; j < K; j += blockDim.x) {
					const int kk = KL[j] + kc[j & 63u] + kc[64 + (j >> 6)];
					const double E = -(static_cast<double>(kk) + ebase + eh0[j]);
					const double ax = sm[j].x, ay = sm[j].y;
					acc += (ax * ax + ay * ay) * E;
				}
				red[threadIdx.x] = acc;
				__syncthreads();
				for (int wdt = blockDim.x / 2; wdt > 0; wdt >>= 1) {
					if (threadIdx.x < wdt) red[threadIdx.x] += red[threadIdx.x + wdt];
					__syncthreads();
				}
				if (threadIdx.x == 0) P.parts[I.part_offset + t] = red[0];
				__syncthreads();
			}
			cluster.sync();
		}
		// fixed-order final reduction by the cluster's first CTA
		if (crank == 0) {
			const uint64_t ntiles = G0.ntiles();
			double acc = 0;
			for (uint64_t t = threadIdx.x; t < ntiles; t += blockDim.x) acc += P.parts[I.part_offset + t];
			red[threadIdx.x] = acc;
			__syncthreads();
			for (int wdt = blockDim.x / 2; wdt > 0; wdt >>= 1) {
				if (threadIdx.x < wdt) red[threadIdx.x] += red[threadIdx.x + wdt];
				__syncthreads();
			}
			if (threadIdx.x == 0) P.energies[P.order[w]] = red[0] * P.scale2[P.order[w]];
			__syncthreads();
		}
		cluster.sync();
	}
}

}  // namespace
}  // namespace qcs

using cd = std::complex<double>;

struct qcs_qaoa_batch {
	int prec = QCS_FP64;
	uint32_t p = 0;
	size_t count = 0;
	std::vector<qcs::QInst> inst;
	std::vector<std::vector<double>> h;      // fields per instance
	std::vector<uint32_t> order;
	uint64_t total_amps = 0, total_parts = 0;
	size_t tab_entries = 0, etab_entries = 0;
	void* d_amps = nullptr;
	qcs::QInst* d_inst = nullptr;
	uint32_t* d_order = nullptr;
	void* d_tabs = nullptr;
	double* d_etab = nullptr;
	int16_t* d_kltab = nullptr;
	size_t kl_entries = 0;
	qcs::QLayer* d_layers = nullptr;
	double* d_parts = nullptr;
	double* d_energies = nullptr;
	double* d_scale2 = nullptr;
	double* h_energies = nullptr;  // pinned
	std::vector<cd> scale;         // complex scale per instance (amplitudes = scale * stored)
	cudaStream_t stream = nullptr;
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	int cluster = 0;               // CTAs per cluster (0: choose)
	int stage_low = 6, stage_high = 6;  // mixer-pass tile shape
	int sms = 148;
	std::string err;
};

namespace {

int qfail(qcs_qaoa_batch* b, int st, const std::string& m) {
	if (b) b->err = m;
	return st;
}

template <typename T> typename qcs::cplx_t<T> cc(const cd& v) {
	typename qcs::cplx_t<T> r;
	r.x = static_cast<T>(v.real());
	r.y = static_cast<T>(v.imag());
	return r;
}

template <typename T>
cudaError_t launch(qcs_qaoa_batch* b) {
	qcs::QParams<T> P;
	P.amps = static_cast<qcs::cplx_t<T>*>(b->d_amps);
	P.inst = b->d_inst;
	P.order = b->d_order;
	P.ninst = static_cast<uint32_t>(b->count);
	P.p = b->p;
	P.tabs = static_cast<const qcs::cplx_t<T>*>(b->d_tabs);
	P.etab = b->d_etab;
	P.kltab = b->d_kltab;
	P.layers = b->d_layers;
	P.parts = b->d_parts;
	P.energies = b->d_energies;
	P.scale2 = b->d_scale2;
	P.stage_low = static_cast<uint32_t>(b->stage_low);
	P.stage_high = static_cast<uint32_t>(b->stage_high);
	const size_t smem = (size_t(1) << qcs::kGroupBits) * sizeof(qcs::cplx_t<T>);
	cudaError_t e = cudaFuncSetAttribute(qcs::k_qaoa<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
	if (e == cudaSuccess) e = cudaFuncSetAttribute(qcs::k_qaoa<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
	if (e != cudaSuccess) return e;
	const int csize = b->cluster > 0 ? b->cluster : 8;
	int per_sm = static_cast<int>((200 * 1024) / (smem + 8192));
	per_sm = std::max(1, std::min(per_sm, 3));
	int grid = (b->sms * per_sm / csize) * csize;
	if (grid < csize) grid = csize;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(static_cast<unsigned>(grid));
	cfg.blockDim = dim3(qcs::kQThreads);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = b->stream;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = static_cast<unsigned>(csize);
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	e = cudaLaunchKernelEx(&cfg, qcs::k_qaoa<T>, P);
	qcs::note_launches(1);
	return e;
}

cudaError_t record(qcs_qaoa_batch* b) {
	// initial state H^n|0>: every amplitude (1/sqrt2)^n, as the reference's n Hadamards produce it
	cudaError_t e = cudaSuccess;
	for (size_t i = 0; i < b->count && e == cudaSuccess; ++i) {
		const qcs::QInst& I = b->inst[i];
		double v = 1.0;
		const double r2 = 1. / std::sqrt(2.);
		for (uint32_t q = 0; q < I.n; ++q) v *= r2;
		const uint64_t N = 1ULL << I.n;
		e = b->prec == QCS_FP64 ? qcs::launch_fill_const<double>(static_cast<double2*>(b->d_amps) + I.offset, N, v, 0, b->stream)
		                        : qcs::launch_fill_const<float>(static_cast<float2*>(b->d_amps) + I.offset, N, v, 0, b->stream);
	}
	if (e == cudaSuccess) e = b->prec == QCS_FP64 ? launch<double>(b) : launch<float>(b);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(b->h_energies, b->d_energies, b->count * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
	return e;
}

}  // namespace

extern "C" {

int qcs_qaoa_batch_create(const qcs_qaoa_instance* instances, size_t count, uint32_t p, int precision, qcs_qaoa_batch_handle* out) {
	if (!instances || !out || count == 0 || p == 0 || p > static_cast<uint32_t>(qcs::kMaxLayers)) return QCS_INVALID_ARGUMENT;
	if (precision != QCS_FP64 && precision != QCS_FP32) return QCS_INVALID_ARGUMENT;
	*out = nullptr;
	auto* b = new qcs_qaoa_batch;
	b->prec = precision;
	b->p = p;
	b->count = count;
	b->inst.resize(count);
	b->h.resize(count);
	b->scale.assign(count, cd(1, 0));
	for (size_t i = 0; i < count; ++i) {
		const qcs_qaoa_instance& in = instances[i];
		qcs::QInst& I = b->inst[i];
		std::memset(&I, 0, sizeof(I));
		if (in.n < 2 || in.n > 30 || in.nedges > static_cast<uint32_t>(qcs::kMaxEdges)) {
			delete b;
			return QCS_UNSUPPORTED;
		}
		I.n = in.n;
		I.nedges = in.nedges;
		I.g0 = std::min<uint32_t>(in.n, qcs::kGroupBits);
		int ksum = 0;
		// edges grouped: inside the low group, inside the high group, across (low end first)
		std::vector<std::array<int, 3>> lowe, highe, crosse;
		for (uint32_t e = 0; e < in.nedges; ++e) {
			const double J = in.J[e];
			if (J != std::floor(J) || std::abs(J) > 16 || in.edges[2 * e] >= in.n || in.edges[2 * e + 1] >= in.n ||
			    in.edges[2 * e] == in.edges[2 * e + 1]) {
				delete b;
				return QCS_UNSUPPORTED;  // the batch kernel takes small integer couplings
			}
			int a = static_cast<int>(in.edges[2 * e]), c = static_cast<int>(in.edges[2 * e + 1]);
			const bool al = a < static_cast<int>(I.g0), cl = c < static_cast<int>(I.g0);
			if (al && cl) lowe.push_back({a, c, static_cast<int>(J)});
			else if (!al && !cl) highe.push_back({a, c, static_cast<int>(J)});
			else crosse.push_back(al ? std::array<int, 3>{a, c, static_cast<int>(J)} : std::array<int, 3>{c, a, static_cast<int>(J)});
			ksum += static_cast<int>(std::abs(J));
		}
		uint32_t e = 0;
		for (const auto* group : {&lowe, &highe, &crosse})
			for (const auto& x : *group) {
				I.ei[e] = static_cast<uint8_t>(x[0]);
				I.ej[e] = static_cast<uint8_t>(x[1]);
				I.J[e] = static_cast<int8_t>(x[2]);
				++e;
			}
		I.nlow = static_cast<uint16_t>(lowe.size());
		I.nhigh = static_cast<uint16_t>(highe.size());
		I.kl = static_cast<uint32_t>(b->kl_entries);
		b->kl_entries += 1u << I.g0;
		if (ksum > qcs::kMaxK) {
			delete b;
			return QCS_UNSUPPORTED;
		}
		I.kmax = static_cast<uint32_t>(ksum);
		b->h[i].assign(in.h, in.h + in.n);
		I.offset = b->total_amps;
		b->total_amps += 1ULL << in.n;
		I.tab_stride = (2 * I.kmax + 1) + (1u << I.g0) + (1u << (in.n - I.g0));
		I.tab = static_cast<uint32_t>(b->tab_entries);
		b->tab_entries += static_cast<size_t>(I.tab_stride) * p;
		I.eh = static_cast<uint32_t>(b->etab_entries);
		b->etab_entries += (1u << I.g0) + (1u << (in.n - I.g0));
		I.part_offset = b->total_parts;
		b->total_parts += 1ULL << (I.n - I.g0);  // one energy partial per low-group tile
	}
	b->order.resize(count);
	std::iota(b->order.begin(), b->order.end(), 0u);
	std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t a, uint32_t c) { return b->inst[a].n > b->inst[c].n; });
	int dev = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
	const size_t ab = b->prec == QCS_FP64 ? 16 : 8;
	cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaMalloc(&b->d_amps, b->total_amps * ab);
	if (e == cudaSuccess) e = cudaMalloc(&b->d_inst, count * sizeof(qcs::QInst));
	if (e == cudaSuccess) e = cudaMalloc(&b->d_order, count * sizeof(uint32_t));
	if (e == cudaSuccess) e = cudaMalloc(&b->d_tabs, b->tab_entries * ab);
	if (e == cudaSuccess) e = cudaMalloc(&b->d_etab, b->etab_entries * sizeof(double));
	if (e == cudaSuccess) e = cudaMalloc(&b->d_kltab, b->kl_entries * sizeof(int16_t));
	// K over the low group's internal edges for every low-group pattern
	if (e == cudaSuccess) {
		std::vector<int16_t> kl(b->kl_entries);
		for (size_t i = 0; i < count; ++i) {
			const qcs::QInst& I = b->inst[i];
			for (uint32_t x = 0; x < (1u << I.g0); ++x) {
				int k = 0;
				for (uint32_t q = 0; q < I.nlow; ++q) k += (((x >> I.ei[q]) ^ (x >> I.ej[q])) & 1u) ? -I.J[q] : I.J[q];
				kl[I.kl + x] = static_cast<int16_t>(k);
			}
		}
		e = cudaMemcpy(b->d_kltab, kl.data(), kl.size() * sizeof(int16_t), cudaMemcpyHostToDevice);
	}
	if (e == cudaSuccess) e = cudaMalloc(&b->d_layers, count * p * sizeof(qcs::QLayer));
	if (e == cudaSuccess) e = cudaMalloc(&b->d_parts, std::max<uint64_t>(1, b->total_parts) * sizeof(double));
	if (e == cudaSuccess) e = cudaMalloc(&b->d_energies, count * sizeof(double));
	if (e == cudaSuccess) e = cudaMalloc(&b->d_scale2, count * sizeof(double));
	if (e == cudaSuccess) e = cudaMallocHost(&b->h_energies, count * sizeof(double));
	if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_inst, b->inst.data(), count * sizeof(qcs::QInst), cudaMemcpyHostToDevice, b->stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_order, b->order.data(), count * sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream);
	// field energy tables: sum over the group's qubits of h_q s_q
	if (e == cudaSuccess) {
		std::vector<double> et(b->etab_entries);
		for (size_t i = 0; i < count; ++i) {
			const qcs::QInst& I = b->inst[i];
			const uint32_t g1 = I.n - I.g0;
			for (uint32_t x = 0; x < (1u << I.g0); ++x) {
				double s = 0;
				for (uint32_t q = 0; q < I.g0; ++q) s += b->h[i][q] * (((x >> q) & 1u) ? -1.0 : 1.0);
				et[I.eh + x] = s;
			}
			for (uint32_t x = 0; x < (1u << g1); ++x) {
				double s = 0;
				for (uint32_t q = 0; q < g1; ++q) s += b->h[i][I.g0 + q] * (((x >> q) & 1u) ? -1.0 : 1.0);
				et[I.eh + (1u << I.g0) + x] = s;
			}
		}
		e = cudaMemcpy(b->d_etab, et.data(), et.size() * sizeof(double), cudaMemcpyHostToDevice);
	}
	if (e != cudaSuccess) {
		qcs_qaoa_batch_destroy(b);
		cudaGetLastError();
		return e == cudaErrorMemoryAllocation ? QCS_OUT_OF_MEMORY : QCS_CUDA_ERROR;
	}
	*out = b;
	return QCS_OK;
}

int qcs_qaoa_batch_set_angles(qcs_qaoa_batch_handle b, const double* gammas, const double* betas) {
	if (!b || !gammas || !betas) return QCS_INVALID_ARGUMENT;
	const size_t ab = b->prec == QCS_FP64 ? 16 : 8;
	std::vector<unsigned char> tabs(b->tab_entries * ab);
	std::vector<qcs::QLayer> layers(b->count * b->p);
	std::vector<double> s2(b->count);
	auto put = [&](size_t idx, const cd& v) {
		if (b->prec == QCS_FP64) {
			const double2 x = make_double2(v.real(), v.imag());
			std::memcpy(&tabs[idx * ab], &x, ab);
		} else {
			const float2 x = make_float2(static_cast<float>(v.real()), static_cast<float>(v.imag()));
			std::memcpy(&tabs[idx * ab], &x, ab);
		}
	};
	for (size_t i = 0; i < b->count; ++i) {
		const qcs::QInst& I = b->inst[i];
		cd scale(1, 0);  // H^n is in the initial amplitudes; the mixers' factored scalars accumulate here
		for (uint32_t l = 0; l < b->p; ++l) {
			const double g = gammas[i * b->p + l], be = betas[i * b->p + l];
			const size_t base = I.tab + static_cast<size_t>(l) * I.tab_stride;
			// exp(-i g K) for K in [-kmax, kmax]: each edge contributes exp(-i g J s_i s_j) (the CNOT-RZ-CNOT
			// sandwich, RZ angle 2 g J)
			for (int k = -static_cast<int>(I.kmax); k <= static_cast<int>(I.kmax); ++k)
				put(base + static_cast<size_t>(k + static_cast<int>(I.kmax)), std::polar(1.0, -g * k));
			// field factors: RZ(g h_q) gives exp(-i g h_q s_q / 2)
			const uint32_t g1 = I.n - I.g0;
			for (uint32_t x = 0; x < (1u << I.g0); ++x) {
				cd f(1, 0);
				for (uint32_t q = 0; q < I.g0; ++q) {
					const double hq = b->h[i][q];
					if (hq == 0.) continue;  // the reference skips zero fields (IsingModel.h:522)
					f *= std::polar(1.0, (((x >> q) & 1u) ? 0.5 : -0.5) * g * hq);
				}
				put(base + 2 * I.kmax + 1 + x, f);
			}
			for (uint32_t x = 0; x < (1u << g1); ++x) {
				cd f(1, 0);
				for (uint32_t q = 0; q < g1; ++q) {
					const double hq = b->h[i][I.g0 + q];
					if (hq == 0.) continue;
					f *= std::polar(1.0, (((x >> q) & 1u) ? 0.5 : -0.5) * g * hq);
				}
				put(base + 2 * I.kmax + 1 + (1u << I.g0) + x, f);
			}
			// mixer RX(2 beta) = [[c, -is], [-is, c]] with c = cos(beta), s = sin(beta) (SimpleGates.h:840-848),
			// factored like the per-gate kernels
			const double c = std::cos(be), s = std::sin(be);
			qcs::QLayer& L = layers[i * b->p + l];
			std::memset(&L, 0, sizeof(L));
			if (std::abs(c) >= std::abs(s)) {
				L.form = 0;
				L.x0 = -s / c;
				L.x1 = -s / c;
				for (uint32_t q = 0; q < I.n; ++q) scale *= c;
			} else {
				L.form = 1;
				L.x0 = c / s;
				L.x1 = c / s;
				for (uint32_t q = 0; q < I.n; ++q) scale *= cd(0, -s);
			}
		}
		b->scale[i] = scale;
		s2[i] = std::norm(scale);
	}
	cudaError_t e = cudaMemcpy(b->d_tabs, tabs.data(), tabs.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(b->d_layers, layers.data(), layers.size() * sizeof(qcs::QLayer), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(b->d_scale2, s2.data(), s2.size() * sizeof(double), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return qfail(b, QCS_CUDA_ERROR, std::string("set angles: ") + cudaGetErrorString(e));
	return QCS_OK;
}

namespace {
// the captured graph holds the launch configuration: drop it when the schedule changes
void reset_graph(qcs_qaoa_batch* b) {
	if (b->exec) {
		cudaGraphExecDestroy(b->exec);
		b->exec = nullptr;
	}
	if (b->graph) {
		cudaGraphDestroy(b->graph);
		b->graph = nullptr;
	}
}
}  // namespace

int qcs_qaoa_batch_set_cluster(qcs_qaoa_batch_handle b, int ctas) {
	if (!b || ctas < 1 || ctas > 16 || (ctas & (ctas - 1))) return QCS_INVALID_ARGUMENT;
	b->cluster = ctas;
	reset_graph(b);
	return QCS_OK;
}

int qcs_qaoa_batch_set_tile(qcs_qaoa_batch_handle b, int low, int high) {
	if (!b) return QCS_INVALID_ARGUMENT;
	if (low < 3 || high < 1 || low + high > qcs::kGroupBits) return qfail(b, QCS_INVALID_ARGUMENT, "tile: low >= 3, high >= 1, low + high <= 12");
	b->stage_low = low;
	b->stage_high = high;
	reset_graph(b);
	return QCS_OK;
}

int qcs_qaoa_batch_run(qcs_qaoa_batch_handle b, double* energies_out) {
	if (!b) return QCS_INVALID_ARGUMENT;
	cudaError_t e = cudaSuccess;
	if (!b->exec) {
		e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
		if (e == cudaSuccess) {
			cudaError_t r = record(b);
			e = cudaStreamEndCapture(b->stream, &b->graph);
			if (r != cudaSuccess) e = r;
		}
		if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
		if (e != cudaSuccess) {
			cudaGetLastError();
			return qfail(b, QCS_CUDA_ERROR, std::string("graph capture: ") + cudaGetErrorString(e));
		}
	}
	e = cudaGraphLaunch(b->exec, b->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
	if (e != cudaSuccess) return qfail(b, QCS_CUDA_ERROR, std::string("run: ") + cudaGetErrorString(e));
	if (energies_out) std::memcpy(energies_out, b->h_energies, b->count * sizeof(double));
	return QCS_OK;
}

int qcs_qaoa_batch_state(qcs_qaoa_batch_handle b, size_t index, double* host_state) {
	if (!b || !host_state || index >= b->count) return QCS_INVALID_ARGUMENT;
	const qcs::QInst& I = b->inst[index];
	const uint64_t N = 1ULL << I.n;
	const cd sc = b->scale[index];
	cudaError_t e;
	if (b->prec == QCS_FP64) {
		e = cudaMemcpy(host_state, static_cast<double2*>(b->d_amps) + I.offset, N * 16, cudaMemcpyDeviceToHost);
		for (uint64_t i = 0; i < N && e == cudaSuccess; ++i) {
			const cd v = sc * cd(host_state[2 * i], host_state[2 * i + 1]);
			host_state[2 * i] = v.real();
			host_state[2 * i + 1] = v.imag();
		}
	} else {
		std::vector<float> tmp(2 * N);
		e = cudaMemcpy(tmp.data(), static_cast<float2*>(b->d_amps) + I.offset, N * 8, cudaMemcpyDeviceToHost);
		for (uint64_t i = 0; i < N && e == cudaSuccess; ++i) {
			const cd v = sc * cd(tmp[2 * i], tmp[2 * i + 1]);
			host_state[2 * i] = v.real();
			host_state[2 * i + 1] = v.imag();
		}
	}
	if (e != cudaSuccess) return qfail(b, QCS_CUDA_ERROR, std::string("state: ") + cudaGetErrorString(e));
	return QCS_OK;
}

uint64_t qcs_qaoa_batch_amplitudes(qcs_qaoa_batch_handle b) { return b ? b->total_amps : 0; }

const char* qcs_qaoa_batch_last_error(qcs_qaoa_batch_handle b) { return b ? b->err.c_str() : "null handle"; }

int qcs_qaoa_batch_destroy(qcs_qaoa_batch_handle b) {
	if (!b) return QCS_INVALID_ARGUMENT;
	if (b->stream) cudaStreamSynchronize(b->stream);
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->graph) cudaGraphDestroy(b->graph);
	cudaFree(b->d_amps);
	cudaFree(b->d_inst);
	cudaFree(b->d_order);
	cudaFree(b->d_tabs);
	cudaFree(b->d_etab);
	cudaFree(b->d_kltab);
	cudaFree(b->d_layers);
	cudaFree(b->d_parts);
	cudaFree(b->d_energies);
	cudaFree(b->d_scale2);
	if (b->h_energies) cudaFreeHost(b->h_energies);
	if (b->stream) cudaStreamDestroy(b->stream);
	delete b;
	return QCS_OK;
}

}  // extern "C"
