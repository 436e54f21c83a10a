// Dense operator on chosen qubits: a 2^k x 2^k matrix (k <= 10) on k target qubits, applied where
// every control qubit is one.  This is the work of QCSim's SubAlgo::NQubitsQuantumGate
// (NQubitsQuantumGate.h:20-46) and SubAlgo::NQubitsControlledQuantumGate
// (NQubitsControlledQuantumGate.h:20-60).  Those build the 2^n x 2^n extended matrix on the host and
// hand it to QubitRegister::ApplyOperatorMatrix (QubitRegister.h:499-505), which is O(4^n).  Here only
// the 2^k x 2^k operator travels, and each amplitude it touches is read and written once.
//
// The touched amplitudes split into groups of 2^k: one group per assignment of the other qubits, with
// the controls forced to one.  A CTA loads G groups into shared memory as a 2^k x G block X, forms
// Y = U X with U read from global memory (transposed, so that the threads of a warp read neighbouring
// entries; at most 16 MiB for k = 10 in FP64, L2-resident) and writes Y in place.  Every output
// amplitude belongs to one thread, and the CTA has read all of its groups before any write.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "batch.cuh"
#include "compile.cuh"
#include "engine.cuh"
#include "gate_math.cuh"

namespace qcs {
namespace {

int fail(qcs_handle h, int status, const std::string& msg) {
	h->err = msg;
	return status;
}

int cuda_fail(qcs_handle h, cudaError_t e, const char* where) {
	cudaGetLastError();
	return fail(h, e == cudaErrorMemoryAllocation ? QCS_OUT_OF_MEMORY : QCS_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
}

constexpr int kOpThreads = 256;
constexpr uint32_t kMaxOpQubits = 10;
constexpr size_t kOpSmem = 96 * 1024;  // two CTAs per SM

struct OpGeom {
	uint32_t k;                    // target qubits; matrix bit j is target j
	uint32_t nins;                 // positions a group number skips (targets and controls)
	uint64_t set_mask;             // controls: forced to one
	uint64_t tbit[kMaxOpQubits];   // register bit of matrix bit j
	uint8_t ins[64];               // the skipped positions, ascending
	int col_fastest;               // 1: neighbouring threads take neighbouring columns of one group
};

// shared memory: D column offsets, G group bases, then X (2^k x G amplitudes) on a 16-byte boundary
__host__ __device__ constexpr size_t x_offset(uint32_t D, uint64_t G) { return ((static_cast<size_t>(D) + G) * 8 + 15) / 16 * 16; }

template <typename T>
__global__ void __launch_bounds__(kOpThreads) k_dense_op(cplx_t<T>* __restrict__ s, const cplx_t<T>* __restrict__ Ut, const OpGeom geo,
                                                         uint64_t groups, uint32_t G) {
	extern __shared__ __align__(16) unsigned char smem[];
	const uint32_t D = 1u << geo.k;
	uint64_t* coff = reinterpret_cast<uint64_t*>(smem);  // column c -> offset of its amplitude in a group
	uint64_t* gbase = coff + D;                           // group of this batch -> its base index
	cplx_t<T>* X = reinterpret_cast<cplx_t<T>*>(smem + x_offset(D, G));
	for (uint32_t c = threadIdx.x; c < D; c += blockDim.x) {
		uint64_t o = 0;
		for (uint32_t j = 0; j < geo.k; ++j)
			if ((c >> j) & 1u) o |= geo.tbit[j];
		coff[c] = o;
	}
	for (uint64_t g0 = static_cast<uint64_t>(blockIdx.x) * G; g0 < groups; g0 += static_cast<uint64_t>(gridDim.x) * G) {
		const uint32_t ng = static_cast<uint32_t>(groups - g0 < G ? groups - g0 : G);
		__syncthreads();  // the previous batch's readers of X and gbase are done (and coff is ready)
		for (uint32_t g = threadIdx.x; g < ng; g += blockDim.x) {
			uint64_t p = g0 + g;
			for (uint32_t j = 0; j < geo.nins; ++j) {
				const uint32_t b = geo.ins[j];
				p = ((p >> b) << (b + 1)) | (p & ((1ULL << b) - 1));
			}
			gbase[g] = p | geo.set_mask;
		}
		__syncthreads();
		const uint32_t items = D * ng;
		for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
			const uint32_t c = geo.col_fastest ? i % D : i / ng, g = geo.col_fastest ? i / D : i % ng;
			X[c * G + g] = s[gbase[g] | coff[c]];
		}
		__syncthreads();
		for (uint32_t i = threadIdx.x; i < items; i += blockDim.x) {
			const uint32_t r = geo.col_fastest ? i % D : i / ng, g = geo.col_fastest ? i / D : i % ng;
			T re = 0, im = 0;
			for (uint32_t c = 0; c < D; ++c) {
				const cplx_t<T> u = Ut[static_cast<size_t>(c) * D + r], x = X[c * G + g];
				re = fma(u.x, x.x, re);
				re = fma(-u.y, x.y, re);
				im = fma(u.x, x.y, im);
				im = fma(u.y, x.x, im);
			}
			cplx_t<T> y;
			y.x = re;
			y.y = im;
			s[gbase[g] | coff[r]] = y;
		}
	}
}

template <typename T>
cudaError_t launch_dense_op(cplx_t<T>* s, const cplx_t<T>* Ut, const OpGeom& geo, uint64_t groups, int sms, cudaStream_t st) {
	const uint32_t D = 1u << geo.k;
	const size_t per_group = D * sizeof(cplx_t<T>) + sizeof(uint64_t);
	const size_t avail = kOpSmem - D * sizeof(uint64_t) - 16;
	uint64_t G = std::max<uint64_t>(1, std::min<uint64_t>(avail / per_group, std::max<uint32_t>(1, 4096 / D)));
	G = std::min<uint64_t>(G, groups);
	const size_t smem = x_offset(D, G) + G * D * sizeof(cplx_t<T>);
	if (smem > kOpSmem) return cudaErrorInvalidValue;
	cudaError_t e = cudaFuncSetAttribute(k_dense_op<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kOpSmem));
	if (e != cudaSuccess) return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dense_op<T>, kOpThreads, smem);
	if (e != cudaSuccess) return e;
	const uint64_t batches = (groups + G - 1) / G;
	const int grid = static_cast<int>(std::min<uint64_t>(batches, static_cast<uint64_t>(sms) * std::max(1, per_sm)));
	k_dense_op<T><<<grid, kOpThreads, smem, st>>>(s, Ut, geo, groups, static_cast<uint32_t>(G));
	note_launches(1);
	return cudaGetLastError();
}

template <typename T>
int apply(qcs_handle h, const double* m, uint32_t k, const OpGeom& geo, uint64_t groups) {
	const uint32_t D = 1u << k;
	std::vector<cplx_t<T>> ut(static_cast<size_t>(D) * D);
	for (uint32_t r = 0; r < D; ++r)
		for (uint32_t c = 0; c < D; ++c) {
			const double* e = m + 2 * (static_cast<size_t>(r) * D + c);
			ut[static_cast<size_t>(c) * D + r].x = static_cast<T>(e[0]);
			ut[static_cast<size_t>(c) * D + r].y = static_cast<T>(e[1]);
		}
	const size_t bytes = ut.size() * sizeof(cplx_t<T>);
	void* d = nullptr;
	cudaError_t e = cudaMallocAsync(&d, bytes, h->stream);
	if (e != cudaSuccess) return cuda_fail(h, e, "operator on qubits");
	// pageable source: the call returns once the entries are staged, so ut may go out of scope
	e = cudaMemcpyAsync(d, ut.data(), bytes, cudaMemcpyHostToDevice, h->stream);
	if (e == cudaSuccess) {
		const double touched = std::ldexp(1.0, -static_cast<int>(geo.nins - geo.k));
		prof_begin(h, "dense_op", 2.0 * h->amp_bytes() * static_cast<double>(h->N) * touched);
		e = launch_dense_op<T>(static_cast<cplx_t<T>*>(h->d_state), static_cast<const cplx_t<T>*>(d), geo, groups, h->sms, h->stream);
		prof_end(h);
	}
	const cudaError_t ef = cudaFreeAsync(d, h->stream);
	if (e == cudaSuccess) e = ef;
	if (e != cudaSuccess) return cuda_fail(h, e, "operator on qubits");
	return QCS_OK;
}

// a diagonal operator's entries on the device, in the register's precision (cudaMallocAsync on the
// register's stream; release with cudaFreeAsync on the same stream)
template <typename T>
cudaError_t upload_diagonal(qcs_handle h, const double* d, void** out) {
	std::vector<cplx_t<T>> v(h->N);
	for (uint64_t i = 0; i < h->N; ++i) {
		v[i].x = static_cast<T>(d[2 * i]);
		v[i].y = static_cast<T>(d[2 * i + 1]);
	}
	cudaError_t e = cudaMallocAsync(out, v.size() * sizeof(cplx_t<T>), h->stream);
	if (e != cudaSuccess) return e;
	// pageable source: the call returns once the entries are staged
	return cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(cplx_t<T>), cudaMemcpyHostToDevice, h->stream);
}

cudaError_t upload_diagonal_any(qcs_handle h, const double* d, void** out) {
	return h->prec == QCS_FP64 ? upload_diagonal<double>(h, d, out) : upload_diagonal<float>(h, d, out);
}

}  // namespace

template <typename T>
__global__ void k_table_diag(cplx_t<T>* __restrict__ s, const cplx_t<T>* __restrict__ d, uint64_t N) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) s[i] = cmul<T>(s[i], d[i]);
}

template <typename T>
cudaError_t launch_table_diag(cplx_t<T>* s, uint64_t N, const cplx_t<T>* d, int sms, cudaStream_t st) {
	k_table_diag<T><<<grid_for(N, 256, sms), 256, 0, st>>>(s, d, N);
	note_launches(1);
	return cudaGetLastError();
}
template cudaError_t launch_table_diag<double>(double2*, uint64_t, const double2*, int, cudaStream_t);
template cudaError_t launch_table_diag<float>(float2*, uint64_t, const float2*, int, cudaStream_t);

}  // namespace qcs

extern "C" int qcs_apply_diagonal(qcs_handle h, const double* d) {
	if (!h || !d) return QCS_INVALID_ARGUMENT;
	void* dd = nullptr;
	cudaError_t e = qcs::upload_diagonal_any(h, d, &dd);
	if (e == cudaSuccess) {
		qcs::prof_begin(h, "table_diag", 3.0 * h->amp_bytes() * static_cast<double>(h->N));
		e = h->prec == QCS_FP64
		        ? qcs::launch_table_diag<double>(static_cast<double2*>(h->d_state), h->N, static_cast<const double2*>(dd), h->sms, h->stream)
		        : qcs::launch_table_diag<float>(static_cast<float2*>(h->d_state), h->N, static_cast<const float2*>(dd), h->sms, h->stream);
		qcs::prof_end(h);
	}
	if (dd) {
		const cudaError_t ef = cudaFreeAsync(dd, h->stream);
		if (e == cudaSuccess) e = ef;
	}
	if (e != cudaSuccess) return qcs::cuda_fail(h, e, "diagonal operator");
	return QCS_OK;
}

extern "C" int qcs_schrodinger_evolve(qcs_handle h, const double* potential_op, const double* kinetic_op, uint64_t steps) {
	if (!h || !potential_op || !kinetic_op) return QCS_INVALID_ARGUMENT;
	void *dv = nullptr, *dk = nullptr;
	cudaError_t e = qcs::upload_diagonal_any(h, potential_op, &dv);
	if (e == cudaSuccess) e = qcs::upload_diagonal_any(h, kinetic_op, &dk);
	int st = QCS_OK;
	if (e == cudaSuccess) st = qcs::schrodinger_apply(h, dv, dk, steps);
	for (void* p : {dv, dk})
		if (p) {
			const cudaError_t ef = cudaFreeAsync(p, h->stream);
			if (e == cudaSuccess) e = ef;
		}
	if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
	if (e != cudaSuccess) return qcs::cuda_fail(h, e, "schrodinger");
	return st;
}

extern "C" int qcs_apply_operator_on_qubits(qcs_handle h, const double* m, uint32_t k, const uint32_t* qubits, uint64_t ctrl_mask) {
	if (!h || !m || !qubits) return QCS_INVALID_ARGUMENT;
	if (k < 1 || k > qcs::kMaxOpQubits || k > h->n) return qcs::fail(h, QCS_INVALID_ARGUMENT, "operator on qubits: 1 to 10 target qubits");
	if (h->n < 64 && (ctrl_mask >> h->n) != 0) return qcs::fail(h, QCS_INVALID_ARGUMENT, "operator on qubits: control qubit out of range");
	qcs::OpGeom geo;
	std::memset(&geo, 0, sizeof(geo));
	geo.k = k;
	uint64_t tmask = 0;
	for (uint32_t j = 0; j < k; ++j) {
		if (qubits[j] >= h->n) return qcs::fail(h, QCS_INVALID_ARGUMENT, "operator on qubits: target qubit out of range");
		const uint64_t b = 1ULL << qubits[j];
		if (tmask & b) return qcs::fail(h, QCS_INVALID_ARGUMENT, "operator on qubits: repeated target qubit");
		tmask |= b;
		geo.tbit[j] = b;
	}
	if (tmask & ctrl_mask) return qcs::fail(h, QCS_INVALID_ARGUMENT, "operator on qubits: a qubit is both target and control");
	const uint64_t skip = tmask | ctrl_mask;
	for (uint32_t q = 0; q < h->n; ++q)
		if ((skip >> q) & 1ULL) geo.ins[geo.nins++] = static_cast<uint8_t>(q);
	geo.set_mask = ctrl_mask;
	geo.col_fastest = (tmask & 1ULL) ? 1 : 0;
	const uint64_t groups = h->N >> geo.nins;
	return h->prec == QCS_FP64 ? qcs::apply<double>(h, m, k, geo, groups) : qcs::apply<float>(h, m, k, geo, groups);
}
