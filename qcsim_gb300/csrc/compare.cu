// Cross-register comparison (either precision): <a|b>, |a|^2, |b|^2 and max |a_i - b_i|, for the
// fidelity and the max amplitude error that the FP32 path reports against an FP64 run.
#include <cmath>
#include <string>
#include <vector>

#include "engine.cuh"

namespace qcs {
namespace {

constexpr int kThreads = 256;

template <typename A, typename B>
__global__ void __launch_bounds__(kThreads) k_compare(const A* __restrict__ a, const B* __restrict__ b, uint64_t N, double2 sa,
                                                      double2 sb, double* part) {
	__shared__ double sh[5][kThreads];
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	double re = 0, im = 0, na = 0, nb = 0, mx = 0;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
		// amplitude = pending factor x stored value, in double
		const double sx = a[i].x, sy = a[i].y, tx = b[i].x, ty = b[i].y;
		const double ax = sa.x * sx - sa.y * sy, ay = sa.x * sy + sa.y * sx;
		const double bx = sb.x * tx - sb.y * ty, by = sb.x * ty + sb.y * tx;
		re = fma(ay, by, fma(ax, bx, re));
		im = fma(-ay, bx, fma(ax, by, im));
		na = fma(ay, ay, fma(ax, ax, na));
		nb = fma(by, by, fma(bx, bx, nb));
		const double dx = ax - bx, dy = ay - by;
		mx = fmax(mx, fma(dy, dy, dx * dx));  // squared; one square root at the end (FP64 pipe)
	}
	sh[0][threadIdx.x] = re;
	sh[1][threadIdx.x] = im;
	sh[2][threadIdx.x] = na;
	sh[3][threadIdx.x] = nb;
	sh[4][threadIdx.x] = mx;
	__syncthreads();
	for (int w = blockDim.x / 2; w > 0; w >>= 1) {
		if (threadIdx.x < w) {
			for (int c = 0; c < 4; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
			sh[4][threadIdx.x] = fmax(sh[4][threadIdx.x], sh[4][threadIdx.x + w]);
		}
		__syncthreads();
	}
	if (threadIdx.x == 0)
		for (int c = 0; c < 5; ++c) part[5 * blockIdx.x + c] = sh[c][0];
}

template <typename A, typename B>
cudaError_t run(const void* a, const void* b, uint64_t N, double2 sa, double2 sb, int sms, cudaStream_t st, double out[5]) {
	const int g = grid_for(N, kThreads, sms, 4);
	double* d = nullptr;
	cudaError_t e = cudaMalloc(&d, sizeof(double) * 5 * g);
	if (e != cudaSuccess) return e;
	k_compare<A, B><<<g, kThreads, 0, st>>>(static_cast<const A*>(a), static_cast<const B*>(b), N, sa, sb, d);
	note_launches(1);
	std::vector<double> h(5 * static_cast<size_t>(g));
	e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	cudaFree(d);
	if (e != cudaSuccess) return e;
	for (int c = 0; c < 5; ++c) out[c] = 0;
	for (int i = 0; i < g; ++i) {
		for (int c = 0; c < 4; ++c) out[c] += h[5 * i + c];
		out[4] = std::fmax(out[4], h[5 * i + 4]);
	}
	return cudaSuccess;
}

}  // namespace
}  // namespace qcs

extern "C" int qcs_compare(qcs_handle h, qcs_handle other, double* fidelity_out, double* max_abs_diff_out) {
	if (!h || !other || !fidelity_out || !max_abs_diff_out) return QCS_INVALID_ARGUMENT;
	if (h->N != other->N) {
		h->err = "registers differ in size";
		return QCS_INVALID_ARGUMENT;
	}
	// each register's pending global factor is applied inside the sweep (the stored values stay as they are);
	// the other register's queued work finishes first, the comparison runs on this register's stream
	cudaError_t e = cudaStreamSynchronize(other->stream);
	double r[5] = {0, 0, 0, 0, 0};
	const double2 sa = make_double2(h->scale.real(), h->scale.imag());
	const double2 sb = make_double2(other->scale.real(), other->scale.imag());
	if (e == cudaSuccess) {
		const bool a64 = h->prec == QCS_FP64, b64 = other->prec == QCS_FP64;
		if (a64 && b64) e = qcs::run<double2, double2>(h->d_state, other->d_state, h->N, sa, sb, h->sms, h->stream, r);
		else if (a64) e = qcs::run<double2, float2>(h->d_state, other->d_state, h->N, sa, sb, h->sms, h->stream, r);
		else if (b64) e = qcs::run<float2, double2>(h->d_state, other->d_state, h->N, sa, sb, h->sms, h->stream, r);
		else e = qcs::run<float2, float2>(h->d_state, other->d_state, h->N, sa, sb, h->sms, h->stream, r);
	}
	if (e != cudaSuccess) {
		h->err = std::string("compare: ") + cudaGetErrorString(e);
		return QCS_CUDA_ERROR;
	}
	const double den = r[2] * r[3];
	*fidelity_out = den > 0 ? (r[0] * r[0] + r[1] * r[1]) / den : 0.0;
	*max_abs_diff_out = std::sqrt(r[4]);
	return QCS_OK;
}
