// GetQubitProbability through a fixed device array: qcs_qubit_probability_noalloc.
//
// qcs_qubit_probability reduces through scratch that the register allocates on its first
// observation.  Not every caller can let that happen.  A register sized to fill the GPU leaves no
// room for it; an application that hands device memory out from its own pool or budget cannot have a
// library take memory behind its back; and cudaFree, which releases such scratch, waits for the whole
// device, which a caller keeping other streams busy cannot accept.  This variant reduces through a
// file-scope device array instead and allocates nothing.
//
// Limits and rules:
//  * The array holds kPartials = 2^15 doubles (256 KiB) and is resident on every GPU that loads the
//    library, for the life of the process.  Each block folds kChunk = 2^16 amplitudes with the
//    qubit set, so registers of at most 2^32 amplitudes (32 qubits) are accepted; larger ones are
//    rejected with QCS_UNSUPPORTED and a message.
//  * The first call on a device does the set-up: it looks the array's address up with that device
//    current and makes sure the kernels are loaded there.  Make that first call before any stream
//    capture on the device.
//  * Every call is synchronous: it copies the one-double result to the host and synchronises the
//    register's stream before it returns.
//  * All calls share the one array.  Calls whose kernels can overlap on the GPU (two registers on
//    two streams, two host threads) race on it; serialise them.
//  * Nothing has to start at zero: every slot a call reads was written earlier by the same call.
#include <mutex>
#include <string>

#include "engine.cuh"

namespace qcs {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr uint64_t kChunk = 1ULL << 16;     // amplitudes (with the qubit set) folded per block
constexpr uint64_t kPartials = 1ULL << 15;  // blocks, one partial sum each
constexpr uint64_t kMaxAmps = 2 * kChunk * kPartials;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kPartials];

double* g_scratch[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// block b sums |a_i|^2 over the amplitudes i with bit q set whose rank among them lies in
// [b * kChunk, (b + 1) * kChunk); the order of the additions is fixed by the launch shape
template <typename T>
__global__ void __launch_bounds__(kNoAllocThreads) k_qprob_chunks(const cplx_t<T>* __restrict__ s, uint64_t half, uint32_t q,
                                                                double* __restrict__ partials) {
	__shared__ double red[kNoAllocThreads];
	const uint64_t lo = static_cast<uint64_t>(blockIdx.x) * kChunk;
	const uint64_t hi = min(half, lo + kChunk);
	const uint64_t low_mask = (1ULL << q) - 1;
	double acc = 0;
#pragma unroll 4
	for (uint64_t j = lo + threadIdx.x; j < hi; j += kNoAllocThreads) {
		const uint64_t i = ((j & ~low_mask) << 1) | (1ULL << q) | (j & low_mask);
		const cplx_t<T> a = s[i];
		const double x = static_cast<double>(a.x), y = static_cast<double>(a.y);
		acc += x * x + y * y;
	}
	red[threadIdx.x] = acc;
	__syncthreads();
	for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
		if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// one block folds partials[0, nblocks) in a fixed order into partials[0]
__global__ void __launch_bounds__(kNoAllocThreads) k_qprob_fold(double* __restrict__ partials, uint32_t nblocks) {
	__shared__ double red[kNoAllocThreads];
	double acc = 0;
	for (uint32_t i = threadIdx.x; i < nblocks; i += kNoAllocThreads) acc += partials[i];
	red[threadIdx.x] = acc;
	__syncthreads();
	for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
		if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x == 0) partials[0] = red[0];
}

// the array's address on the current device; the first call per device also loads the kernels there
cudaError_t scratch_for_device(int dev, double** out) {
	if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
	std::lock_guard<std::mutex> lock(g_scratch_mutex);
	if (!g_scratch[dev]) {
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
		if (e != cudaSuccess) return e;
		cudaFuncAttributes attr;
		if ((e = cudaFuncGetAttributes(&attr, k_qprob_chunks<double>)) != cudaSuccess) return e;
		if ((e = cudaFuncGetAttributes(&attr, k_qprob_chunks<float>)) != cudaSuccess) return e;
		if ((e = cudaFuncGetAttributes(&attr, k_qprob_fold)) != cudaSuccess) return e;
		g_scratch[dev] = static_cast<double*>(p);
	}
	*out = g_scratch[dev];
	return cudaSuccess;
}

}  // namespace
}  // namespace qcs

extern "C" int qcs_qubit_probability_noalloc(qcs_handle h, uint32_t qubit, double* p_out) {
	if (!h || !p_out) return QCS_INVALID_ARGUMENT;
	if (qubit >= 63) {
		h->err = "qubit out of range";
		return QCS_INVALID_ARGUMENT;
	}
	if (h->N > qcs::kMaxAmps) {
		h->err = "qcs_qubit_probability_noalloc accepts registers of at most 32 qubits: its fixed device array holds 2^15 "
		         "partial sums of 2^16 amplitudes; use qcs_qubit_probability";
		return QCS_UNSUPPORTED;
	}
	*p_out = 0;
	if (qubit >= h->n) return QCS_OK;  // no amplitude has the bit set, as in qcs_qubit_probability
	int dev = -1;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess && dev != h->device) {
		h->err = "qcs_qubit_probability_noalloc: make the register's device current first";
		return QCS_INVALID_ARGUMENT;
	}
	double* scratch = nullptr;
	if (e == cudaSuccess) e = qcs::scratch_for_device(dev, &scratch);
	if (e != cudaSuccess) {
		h->err = std::string("qcs_qubit_probability_noalloc: set-up of the device array failed: ") + cudaGetErrorString(e);
		return QCS_CUDA_ERROR;
	}
	const uint64_t half = h->N / 2;
	const uint32_t nblocks = static_cast<uint32_t>((half + qcs::kChunk - 1) / qcs::kChunk);
	if (h->prec == QCS_FP64)
		qcs::k_qprob_chunks<double>
		    <<<nblocks, qcs::kNoAllocThreads, 0, h->stream>>>(static_cast<const double2*>(h->d_state), half, qubit, scratch);
	else
		qcs::k_qprob_chunks<float>
		    <<<nblocks, qcs::kNoAllocThreads, 0, h->stream>>>(static_cast<const float2*>(h->d_state), half, qubit, scratch);
	qcs::k_qprob_fold<<<1, qcs::kNoAllocThreads, 0, h->stream>>>(scratch, nblocks);
	qcs::note_launches(2);
	double raw = 0;
	e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaMemcpyAsync(&raw, scratch, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
	if (e != cudaSuccess) {
		h->err = std::string("qcs_qubit_probability_noalloc: ") + cudaGetErrorString(e);
		return QCS_CUDA_ERROR;
	}
	// the stored amplitudes may carry a pending global factor: amplitude = scale x stored value
	*p_out = raw * std::norm(h->scale);
	return QCS_OK;
}
