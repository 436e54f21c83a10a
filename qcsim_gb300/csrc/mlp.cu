// Learned cost model: a 3-layer MLP (F inputs -> 64 -> 64 -> 1, ReLU, FP32) that predicts the log of a
// fused block's device time from its features.  Forward, backward and the Adam update are hand-written
// kernels; the partition choice (costmodel.cu) runs the inference kernel on every block of each
// candidate partition in one batch.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace qcs {
namespace {

constexpr int kH = 64;        // hidden width
constexpr int kMaxF = 32;     // largest input width
constexpr int kMThreads = 128;

// parameter layout: W1[H][F], b1[H], W2[H][H], b2[H], W3[H], b3
__host__ __device__ inline int off_w1() { return 0; }
__host__ __device__ inline int off_b1(int F) { return kH * F; }
__host__ __device__ inline int off_w2(int F) { return kH * F + kH; }
__host__ __device__ inline int off_b2(int F) { return kH * F + kH + kH * kH; }
__host__ __device__ inline int off_w3(int F) { return kH * F + 2 * kH + kH * kH; }
__host__ __device__ inline int off_b3(int F) { return kH * F + 3 * kH + kH * kH; }
__host__ __device__ inline int nparams(int F) { return kH * F + 3 * kH + kH * kH + 1; }

// one thread per sample: y = W3 relu(W2 relu(W1 x + b1) + b2) + b3; activations kept for backward
__global__ void __launch_bounds__(kMThreads) k_forward(const float* __restrict__ P, int F, const float* __restrict__ X, int B,
                                                       float* __restrict__ H1, float* __restrict__ H2, float* __restrict__ Y) {
	extern __shared__ float sp[];
	const int np = nparams(F);
	for (int i = threadIdx.x; i < np; i += blockDim.x) sp[i] = P[i];
	__syncthreads();
	const int s = blockIdx.x * blockDim.x + threadIdx.x;
	if (s >= B) return;
	float x[kMaxF];
	for (int f = 0; f < F; ++f) x[f] = X[static_cast<size_t>(s) * F + f];
	float h1[kH];
	for (int j = 0; j < kH; ++j) {
		float a = sp[off_b1(F) + j];
		for (int f = 0; f < F; ++f) a = fmaf(sp[off_w1() + j * F + f], x[f], a);
		h1[j] = fmaxf(a, 0.f);
		if (H1) H1[static_cast<size_t>(s) * kH + j] = h1[j];
	}
	float y = sp[off_b3(F)];
	for (int j = 0; j < kH; ++j) {
		float a = sp[off_b2(F) + j];
		for (int k = 0; k < kH; ++k) a = fmaf(sp[off_w2(F) + j * kH + k], h1[k], a);
		a = fmaxf(a, 0.f);
		if (H2) H2[static_cast<size_t>(s) * kH + j] = a;
		y = fmaf(sp[off_w3(F) + j], a, y);
	}
	Y[s] = y;
}

// gradients of L = mean((y - t)^2): per block, accumulated in shared memory, then one partial per block
__global__ void __launch_bounds__(kMThreads) k_backward(const float* __restrict__ P, int F, const float* __restrict__ X,
                                                        const float* __restrict__ T, int B, const float* __restrict__ H1,
                                                        const float* __restrict__ H2, const float* __restrict__ Y,
                                                        float* __restrict__ partials) {
	extern __shared__ float sm[];
	const int np = nparams(F);
	float* sp = sm;        // parameters
	float* sg = sm + np;   // gradient accumulators
	for (int i = threadIdx.x; i < np; i += blockDim.x) {
		sp[i] = P[i];
		sg[i] = 0.f;
	}
	__syncthreads();
	const int s = blockIdx.x * blockDim.x + threadIdx.x;
	if (s < B) {
		const float dy = 2.f * (Y[s] - T[s]) / static_cast<float>(B);
		const float* h1 = H1 + static_cast<size_t>(s) * kH;
		const float* h2 = H2 + static_cast<size_t>(s) * kH;
		atomicAdd(&sg[off_b3(F)], dy);
		float dh2[kH];
		for (int j = 0; j < kH; ++j) {
			atomicAdd(&sg[off_w3(F) + j], dy * h2[j]);
			dh2[j] = h2[j] > 0.f ? dy * sp[off_w3(F) + j] : 0.f;
		}
		float dh1[kH];
		for (int k = 0; k < kH; ++k) dh1[k] = 0.f;
		for (int j = 0; j < kH; ++j) {
			if (dh2[j] == 0.f) continue;
			atomicAdd(&sg[off_b2(F) + j], dh2[j]);
			for (int k = 0; k < kH; ++k) {
				atomicAdd(&sg[off_w2(F) + j * kH + k], dh2[j] * h1[k]);
				dh1[k] = fmaf(sp[off_w2(F) + j * kH + k], dh2[j], dh1[k]);
			}
		}
		for (int k = 0; k < kH; ++k) {
			if (h1[k] <= 0.f) continue;
			atomicAdd(&sg[off_b1(F) + k], dh1[k]);
			for (int f = 0; f < F; ++f) atomicAdd(&sg[off_w1() + k * F + f], dh1[k] * X[static_cast<size_t>(s) * F + f]);
		}
	}
	__syncthreads();
	for (int i = threadIdx.x; i < np; i += blockDim.x) partials[static_cast<size_t>(blockIdx.x) * np + i] = sg[i];
}

// fixed-order sum of the per-block partials
__global__ void k_sum_partials(const float* __restrict__ partials, int nblocks, int np, float* __restrict__ G) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	float a = 0.f;
	for (int b = 0; b < nblocks; ++b) a += partials[static_cast<size_t>(b) * np + i];
	G[i] = a;
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M, float* __restrict__ V, int np,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	const float g = G[i];
	const float m = b1 * M[i] + (1.f - b1) * g;
	const float v = b2 * V[i] + (1.f - b2) * g * g;
	M[i] = m;
	V[i] = v;
	P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

__global__ void k_sqerr(const float* __restrict__ Y, const float* __restrict__ T, int B, float* __restrict__ out) {
	__shared__ float red[256];
	float a = 0.f;
	for (int i = threadIdx.x; i < B; i += blockDim.x) {
		const float d = Y[i] - T[i];
		a += d * d;
	}
	red[threadIdx.x] = a;
	__syncthreads();
	for (int w = blockDim.x / 2; w > 0; w >>= 1) {
		if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x == 0) out[0] = red[0] / static_cast<float>(B);
}

}  // namespace
}  // namespace qcs

struct qcs_mlp {
	int F = 0;
	int np = 0;
	float* d_p = nullptr;
	float* d_g = nullptr;
	float* d_m = nullptr;
	float* d_v = nullptr;
	int step = 0;
	// work buffers
	float* d_x = nullptr;
	float* d_t = nullptr;
	float* d_h1 = nullptr;
	float* d_h2 = nullptr;
	float* d_y = nullptr;
	float* d_part = nullptr;
	float* d_loss = nullptr;
	int cap = 0;
	cudaStream_t stream = nullptr;
	std::string err;
};

namespace {

int mfail(qcs_mlp_handle m, cudaError_t e, const char* where) {
	if (m) m->err = std::string(where) + ": " + cudaGetErrorString(e);
	return e == cudaErrorMemoryAllocation ? QCS_OUT_OF_MEMORY : QCS_CUDA_ERROR;
}

cudaError_t ensure_cap(qcs_mlp_handle m, int B) {
	if (B <= m->cap) return cudaSuccess;
	cudaFree(m->d_x);
	cudaFree(m->d_t);
	cudaFree(m->d_h1);
	cudaFree(m->d_h2);
	cudaFree(m->d_y);
	cudaFree(m->d_part);
	const int nb = (B + qcs::kMThreads - 1) / qcs::kMThreads;
	cudaError_t e = cudaMalloc(&m->d_x, sizeof(float) * static_cast<size_t>(B) * m->F);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_t, sizeof(float) * B);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_h1, sizeof(float) * static_cast<size_t>(B) * qcs::kH);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_h2, sizeof(float) * static_cast<size_t>(B) * qcs::kH);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_y, sizeof(float) * B);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_part, sizeof(float) * static_cast<size_t>(nb) * m->np);
	if (e == cudaSuccess) m->cap = B;
	return e;
}

cudaError_t forward(qcs_mlp_handle m, int B) {
	const int nb = (B + qcs::kMThreads - 1) / qcs::kMThreads;
	qcs::k_forward<<<nb, qcs::kMThreads, sizeof(float) * m->np, m->stream>>>(m->d_p, m->F, m->d_x, B, m->d_h1, m->d_h2, m->d_y);
	qcs::note_launches(1);
	return cudaGetLastError();
}

cudaError_t gradients(qcs_mlp_handle m, int B) {
	const int nb = (B + qcs::kMThreads - 1) / qcs::kMThreads;
	cudaError_t e = forward(m, B);
	if (e != cudaSuccess) return e;
	qcs::k_backward<<<nb, qcs::kMThreads, 2 * sizeof(float) * m->np, m->stream>>>(m->d_p, m->F, m->d_x, m->d_t, B, m->d_h1, m->d_h2,
	                                                                                m->d_y, m->d_part);
	qcs::k_sum_partials<<<(m->np + 255) / 256, 256, 0, m->stream>>>(m->d_part, nb, m->np, m->d_g);
	qcs::note_launches(2);
	return cudaGetLastError();
}

}  // namespace

extern "C" {

int qcs_mlp_create(int inputs, uint64_t seed, qcs_mlp_handle* out) {
	if (!out || inputs < 1 || inputs > qcs::kMaxF) return QCS_INVALID_ARGUMENT;
	auto* m = new qcs_mlp;
	m->F = inputs;
	m->np = qcs::nparams(inputs);
	// He-style initialisation from a fixed-seed generator on the host
	std::vector<float> p(m->np, 0.f);
	uint64_t st = seed ? seed : 0x9E3779B97F4A7C15ULL;
	auto rnd = [&]() {
		st ^= st << 13;
		st ^= st >> 7;
		st ^= st << 17;
		return (static_cast<double>(st >> 11) / 9007199254740992.0) * 2.0 - 1.0;
	};
	const double a1 = std::sqrt(6.0 / inputs), a2 = std::sqrt(6.0 / qcs::kH);
	for (int i = 0; i < qcs::kH * inputs; ++i) p[qcs::off_w1() + i] = static_cast<float>(a1 * rnd());
	for (int i = 0; i < qcs::kH * qcs::kH; ++i) p[qcs::off_w2(inputs) + i] = static_cast<float>(a2 * rnd());
	for (int i = 0; i < qcs::kH; ++i) p[qcs::off_w3(inputs) + i] = static_cast<float>(a2 * rnd() * 0.5);
	cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_p, sizeof(float) * m->np);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_g, sizeof(float) * m->np);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_m, sizeof(float) * m->np);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_v, sizeof(float) * m->np);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_loss, sizeof(float));
	if (e == cudaSuccess) e = cudaMemcpy(m->d_p, p.data(), sizeof(float) * m->np, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, sizeof(float) * m->np);
	if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, sizeof(float) * m->np);
	if (e != cudaSuccess) {
		qcs_mlp_destroy(m);
		cudaGetLastError();
		return QCS_CUDA_ERROR;
	}
	*out = m;
	return QCS_OK;
}

int qcs_mlp_destroy(qcs_mlp_handle m) {
	if (!m) return QCS_INVALID_ARGUMENT;
	if (m->stream) cudaStreamSynchronize(m->stream);
	for (float* p : {m->d_p, m->d_g, m->d_m, m->d_v, m->d_x, m->d_t, m->d_h1, m->d_h2, m->d_y, m->d_part, m->d_loss}) cudaFree(p);
	if (m->stream) cudaStreamDestroy(m->stream);
	delete m;
	return QCS_OK;
}

int qcs_mlp_num_params(qcs_mlp_handle m) { return m ? m->np : 0; }

int qcs_mlp_get_params(qcs_mlp_handle m, float* out) {
	if (!m || !out) return QCS_INVALID_ARGUMENT;
	cudaError_t e = cudaMemcpy(out, m->d_p, sizeof(float) * m->np, cudaMemcpyDeviceToHost);
	return e == cudaSuccess ? QCS_OK : mfail(m, e, "get params");
}

int qcs_mlp_set_params(qcs_mlp_handle m, const float* in) {
	if (!m || !in) return QCS_INVALID_ARGUMENT;
	cudaError_t e = cudaMemcpy(m->d_p, in, sizeof(float) * m->np, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, sizeof(float) * m->np);
	if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, sizeof(float) * m->np);
	m->step = 0;
	return e == cudaSuccess ? QCS_OK : mfail(m, e, "set params");
}

int qcs_mlp_predict(qcs_mlp_handle m, const float* x, int count, float* y_out) {
	if (!m || !x || !y_out || count < 0) return QCS_INVALID_ARGUMENT;
	if (count == 0) return QCS_OK;
	cudaError_t e = ensure_cap(m, count);
	if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_x, x, sizeof(float) * static_cast<size_t>(count) * m->F, cudaMemcpyHostToDevice, m->stream);
	if (e == cudaSuccess) e = forward(m, count);
	if (e == cudaSuccess) e = cudaMemcpyAsync(y_out, m->d_y, sizeof(float) * count, cudaMemcpyDeviceToHost, m->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
	return e == cudaSuccess ? QCS_OK : mfail(m, e, "predict");
}

int qcs_mlp_gradient(qcs_mlp_handle m, const float* x, const float* t, int count, float* grad_out, float* loss_out) {
	if (!m || !x || !t || !grad_out || count <= 0) return QCS_INVALID_ARGUMENT;
	cudaError_t e = ensure_cap(m, count);
	if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_x, x, sizeof(float) * static_cast<size_t>(count) * m->F, cudaMemcpyHostToDevice, m->stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_t, t, sizeof(float) * count, cudaMemcpyHostToDevice, m->stream);
	if (e == cudaSuccess) e = gradients(m, count);
	if (e == cudaSuccess && loss_out) {
		qcs::k_sqerr<<<1, 256, 0, m->stream>>>(m->d_y, m->d_t, count, m->d_loss);
		qcs::note_launches(1);
		e = cudaMemcpyAsync(loss_out, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(grad_out, m->d_g, sizeof(float) * m->np, cudaMemcpyDeviceToHost, m->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
	return e == cudaSuccess ? QCS_OK : mfail(m, e, "gradient");
}

// full-batch Adam steps on (x, t); returns the loss after the last step
int qcs_mlp_train(qcs_mlp_handle m, const float* x, const float* t, int count, int steps, float lr, float* loss_out) {
	if (!m || !x || !t || count <= 0 || steps < 0) return QCS_INVALID_ARGUMENT;
	cudaError_t e = ensure_cap(m, count);
	if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_x, x, sizeof(float) * static_cast<size_t>(count) * m->F, cudaMemcpyHostToDevice, m->stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(m->d_t, t, sizeof(float) * count, cudaMemcpyHostToDevice, m->stream);
	const float b1 = 0.9f, b2 = 0.999f;
	for (int s = 0; s < steps && e == cudaSuccess; ++s) {
		e = gradients(m, count);
		++m->step;
		const float c1 = 1.f - std::pow(b1, static_cast<float>(m->step)), c2 = 1.f - std::pow(b2, static_cast<float>(m->step));
		if (e == cudaSuccess) {
			qcs::k_adam<<<(m->np + 255) / 256, 256, 0, m->stream>>>(m->d_p, m->d_g, m->d_m, m->d_v, m->np, lr, b1, b2, 1e-8f, c1, c2);
			qcs::note_launches(1);
			e = cudaGetLastError();
		}
	}
	if (e == cudaSuccess) e = forward(m, count);
	if (e == cudaSuccess) {
		qcs::k_sqerr<<<1, 256, 0, m->stream>>>(m->d_y, m->d_t, count, m->d_loss);
		qcs::note_launches(1);
		e = cudaGetLastError();
	}
	float loss = 0;
	if (e == cudaSuccess) e = cudaMemcpyAsync(&loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
	if (e != cudaSuccess) return mfail(m, e, "train");
	if (loss_out) *loss_out = loss;
	return QCS_OK;
}

}  // extern "C"
