// State setters, probability reductions, sampling, collapse and conversions.
//
// Reductions are deterministic: a fixed grid (a function of the register size and the SM count)
// sums in a fixed order, then a single block folds the per-block partials.  Probabilities are
// computed as re*re + im*im in FP64 with explicit round-to-nearest operations (no contraction),
// so every path sees the same |a_i|^2 values.
#include <cstring>

#include "engine.cuh"

#include <vector>

namespace qcs {
namespace {

constexpr int kRedThreads = 256;
constexpr uint64_t kChunk = 2048;  // amplitudes per sampling chunk

template <typename T> __device__ __forceinline__ double probd(const cplx_t<T>& a) {
	const double x = static_cast<double>(a.x), y = static_cast<double>(a.y);
	return __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
}

template <typename T> __global__ void k_fill(cplx_t<T>* s, uint64_t N, T re, T im) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
		cplx_t<T> v;
		v.x = re;
		v.y = im;
		s[i] = v;
	}
}

template <typename T> __global__ void k_set_one(cplx_t<T>* s, uint64_t idx, T re, T im) {
	cplx_t<T> v;
	v.x = re;
	v.y = im;
	s[idx] = v;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
	sh[threadIdx.x] = v;
	__syncthreads();
	for (int w = blockDim.x / 2; w > 0; w >>= 1) {
		if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
		__syncthreads();
	}
	const double r = sh[0];
	__syncthreads();
	return r;
}

// per-block partial of sum |a_i|^2 over (i & mask) == value
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_masked_prob(const cplx_t<T>* __restrict__ s, uint64_t N, uint64_t mask, uint64_t value, double* part) {
	__shared__ double sh[kRedThreads];
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	const uint64_t t0 = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	// four independent loads and sums in flight per thread (one dependent sum chain per thread leaves the
	// memory system idle); the four sums are folded in a fixed order, so the result is repeatable.  |a|^2
	// accumulates by two FMAs (the FP64 pipe bounds this kernel on GB300); these sums serve
	// GetQubitProbability, Normalize and the collapse factor, whose results the reference's own
	// summation order already leaves equal only to rounding -- the sampling scans keep probd.
	double acc[4] = {0, 0, 0, 0};
	auto add = [](double a, const cplx_t<T>& v) {
		const double x = static_cast<double>(v.x), y = static_cast<double>(v.y);
		return fma(y, y, fma(x, x, a));
	};
	if (mask && !(mask & (mask - 1)) && mask < N && (value & ~mask) == 0) {
		// one qubit of the register (GetQubitProbability): enumerate only the amplitudes with that bit at
		// `value` (j < N/2 with the bit inserted stays below N; a bit above the register takes the general
		// loop, which finds no amplitude)
		const uint64_t M = N >> 1, low = mask - 1;
		auto at = [&](uint64_t j) { return s[((j & ~low) << 1) | (j & low) | value]; };
		uint64_t j = t0;
		for (; j + 3 * stride < M; j += 4 * stride) {
			const cplx_t<T> a0 = at(j), a1 = at(j + stride), a2 = at(j + 2 * stride), a3 = at(j + 3 * stride);
			acc[0] = add(acc[0], a0);
			acc[1] = add(acc[1], a1);
			acc[2] = add(acc[2], a2);
			acc[3] = add(acc[3], a3);
		}
		for (; j < M; j += stride) acc[0] = add(acc[0], at(j));
	} else {
		uint64_t i = t0;
		for (; i + 3 * stride < N; i += 4 * stride) {
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				const uint64_t k = i + u * stride;
				if ((k & mask) == value) acc[u] = add(acc[u], s[k]);
			}
		}
		for (; i < N; i += stride)
			if ((i & mask) == value) acc[0] = add(acc[0], s[i]);
	}
	const double r = block_sum(__dadd_rn(__dadd_rn(acc[0], acc[1]), __dadd_rn(acc[2], acc[3])), sh);
	if (threadIdx.x == 0) part[blockIdx.x] = r;
}

// single block: fold `n` partials (stride `ncomp` components) in a fixed order
__global__ void __launch_bounds__(kRedThreads) k_fold(const double* part, int n, int ncomp, double* out) {
	__shared__ double sh[kRedThreads];
	for (int c = 0; c < ncomp; ++c) {
		double acc = 0;
		for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i * ncomp + c];
		const double r = block_sum(acc, sh);
		if (threadIdx.x == 0) out[c] = r;
	}
}

template <typename T>
__global__ void k_scale_masked(cplx_t<T>* s, uint64_t N, uint64_t mask, uint64_t value, double f) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
		cplx_t<T> a = s[i];
		if ((i & mask) == value) {
			a.x = static_cast<T>(static_cast<double>(a.x) * f);
			a.y = static_cast<T>(static_cast<double>(a.y) * f);
		} else {
			a.x = static_cast<T>(static_cast<double>(a.x) * 0.0);
			a.y = static_cast<T>(static_cast<double>(a.y) * 0.0);
		}
		s[i] = a;
	}
}

// a_i /= v (complex division, AdjustPhaseAndNormalize)
template <typename T>
__global__ void k_div_complex(cplx_t<T>* s, uint64_t N, double vr, double vi) {
	const double den = vr * vr + vi * vi;
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
		const double x = static_cast<double>(s[i].x), y = static_cast<double>(s[i].y);
		cplx_t<T> r;
		r.x = static_cast<T>((x * vr + y * vi) / den);
		r.y = static_cast<T>((y * vr - x * vi) / den);
		s[i] = r;
	}
}

template <typename T>
__global__ void k_probs(const cplx_t<T>* __restrict__ s, uint64_t N, double* __restrict__ out) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) out[i] = probd<T>(s[i]);
}

// per-block partial of sum conj(a_i) * b_i
template <typename T, typename U>
__global__ void __launch_bounds__(kRedThreads) k_inner(const cplx_t<T>* __restrict__ a, const U* __restrict__ b, uint64_t N, double* part) {
	__shared__ double sh[kRedThreads];
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	double re = 0, im = 0;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
		const double ax = a[i].x, ay = a[i].y, bx = b[i].x, by = b[i].y;
		re += ax * bx + ay * by;
		im += ax * by - ay * bx;
	}
	const double r0 = block_sum(re, sh);
	const double r1 = block_sum(im, sh);
	if (threadIdx.x == 0) {
		part[2 * blockIdx.x] = r0;
		part[2 * blockIdx.x + 1] = r1;
	}
}

// sampling, step 1: serial sum of |a|^2 inside each chunk (one thread per chunk keeps the order of
// the reference's running sum within the chunk)
template <typename T>
__global__ void k_chunk_sums(const cplx_t<T>* __restrict__ s, uint64_t N, uint64_t nchunks, double* __restrict__ sums) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t c = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; c < nchunks; c += stride) {
		const uint64_t lo = c * kChunk, hi = min(N, lo + kChunk);
		double acc = 0;
		for (uint64_t i = lo; i < hi; ++i) acc = __dadd_rn(acc, probd<T>(s[i]));
		sums[c] = acc;
	}
}

// sampling, step 2: exclusive running sum over chunk sums (excl[c] = probability before chunk c,
// excl[nchunks] = total), single block, serial within each thread's segment
__global__ void __launch_bounds__(1024) k_chunk_scan(const double* __restrict__ sums, uint64_t nchunks, double* __restrict__ excl) {
	__shared__ double seg[1024];
	const uint64_t per = (nchunks + blockDim.x - 1) / blockDim.x;
	const uint64_t lo = min(nchunks, per * threadIdx.x), hi = min(nchunks, lo + per);
	double acc = 0;
	for (uint64_t c = lo; c < hi; ++c) acc = __dadd_rn(acc, sums[c]);
	seg[threadIdx.x] = acc;
	__syncthreads();
	if (threadIdx.x == 0) {
		double run = 0;
		for (int t = 0; t < static_cast<int>(blockDim.x); ++t) {
			const double v = seg[t];
			seg[t] = run;
			run = __dadd_rn(run, v);
		}
		excl[nchunks] = run;
	}
	__syncthreads();
	double run = seg[threadIdx.x];
	for (uint64_t c = lo; c < hi; ++c) {
		excl[c] = run;
		run = __dadd_rn(run, sums[c]);
	}
}

// first index i whose running probability reaches the threshold: `strict` selects > instead of >=.
// Returns N when no index does.
template <typename T>
__device__ uint64_t find_first(const cplx_t<T>* __restrict__ s, uint64_t N, const double* __restrict__ excl, uint64_t nchunks,
                               double thr, bool strict) {
	// last chunk whose starting running sum is still below the threshold
	uint64_t lo = 0, hi = nchunks;  // invariant: answer chunk in [lo, hi)
	while (hi - lo > 1) {
		const uint64_t mid = (lo + hi) / 2;
		const bool below = strict ? (excl[mid] <= thr) : (excl[mid] < thr);
		if (below) lo = mid;
		else hi = mid;
	}
	double acc = excl[lo];
	for (uint64_t i = lo * kChunk; i < N; ++i) {
		acc = __dadd_rn(acc, probd<T>(s[i]));
		if (strict ? (acc > thr) : (thr <= acc)) return i;
	}
	return N;
}

// sampling, step 3: one thread per shot
template <typename T>
__global__ void k_sample(const cplx_t<T>* __restrict__ s, uint64_t N, const double* __restrict__ excl, uint64_t nchunks,
                         const double* __restrict__ probs, uint64_t nshots, int mode, uint64_t fallback,
                         unsigned long long* __restrict__ out) {
	const uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	if (k > nshots) return;
	if (k == nshots) {
		// RepeatedMeasure's table stops at the first entry above 1 - epsilon (QubitRegister.h:250)
		if (mode == 1) {
			const uint64_t t = find_first<T>(s, N, excl, nchunks, 1.0 - 2.220446049250313e-16, true);
			out[nshots] = (t == N) ? N - 1 : t;
		}
		return;
	}
	const uint64_t i = find_first<T>(s, N, excl, nchunks, probs[k], false);
	out[k] = (i == N) ? fallback : i;
}

// one measurement of a register of at most kChunk amplitudes in one launch of one block: the sampled
// state by the reference's running sum (the semantics of find_first with a single chunk), then
//   kind 0 (Measure):          collapse onto the sampled value of the masked qubits, renormalised;
//   kind 1 (MeasureAll):       the basis state sampled (all amplitudes rewritten);
//   kind 2 (MeasureNoCollapse): nothing written.
// out[0] = the sampled state (fallback when the running sum never reaches prob)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_measure_small(cplx_t<T>* __restrict__ s, uint64_t N, double prob, uint64_t mask, int kind,
                                                             uint64_t fallback, unsigned long long* __restrict__ out) {
	__shared__ double sh[kRedThreads];
	__shared__ unsigned long long picked;
	if (threadIdx.x == 0) {
		double acc = 0;
		uint64_t st = fallback;
		for (uint64_t i = 0; i < N; ++i) {
			acc = __dadd_rn(acc, probd<T>(s[i]));
			if (prob <= acc) {
				st = i;
				break;
			}
		}
		picked = st;
		out[0] = st;
	}
	__syncthreads();
	const uint64_t st = picked;
	if (kind == 2) return;
	if (kind == 1) {
		for (uint64_t i = threadIdx.x; i < N; i += blockDim.x) {
			cplx_t<T> v;
			v.x = static_cast<T>(i == st ? 1 : 0);
			v.y = static_cast<T>(0);
			s[i] = v;
		}
		return;
	}
	const uint64_t value = st & mask;
	double acc = 0;
	for (uint64_t i = threadIdx.x; i < N; i += blockDim.x)
		if ((i & mask) == value) {
			const double x = static_cast<double>(s[i].x), y = static_cast<double>(s[i].y);
			acc = fma(y, y, fma(x, x, acc));
		}
	const double total = block_sum(acc, sh);
	const double f = 1.0 / sqrt(total);
	for (uint64_t i = threadIdx.x; i < N; i += blockDim.x) {
		const double g = ((i & mask) == value) ? f : 0.0;
		cplx_t<T> v = s[i];
		v.x = static_cast<T>(static_cast<double>(v.x) * g);
		v.y = static_cast<T>(static_cast<double>(v.y) * g);
		s[i] = v;
	}
}

template <typename T>
__global__ void k_from_f64(cplx_t<T>* __restrict__ d, const double2* __restrict__ s, uint64_t N) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
		cplx_t<T> v;
		v.x = static_cast<T>(s[i].x);
		v.y = static_cast<T>(s[i].y);
		d[i] = v;
	}
}

template <typename T>
__global__ void k_to_f64(double2* __restrict__ d, const cplx_t<T>* __restrict__ s, uint64_t N) {
	const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
	for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride)
		d[i] = make_double2(static_cast<double>(s[i].x), static_cast<double>(s[i].y));
}

// out = M * in, one warp per output row (ApplyOperatorMatrix, QubitRegister.h:499-505)
template <typename T>
__global__ void k_opmat(const double2* __restrict__ M, const cplx_t<T>* __restrict__ in, cplx_t<T>* __restrict__ out, uint64_t N) {
	const uint64_t warp = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
	const int lane = threadIdx.x & 31;
	const uint64_t nw = static_cast<uint64_t>(gridDim.x) * blockDim.x / 32;
	for (uint64_t r = warp; r < N; r += nw) {
		double re = 0, im = 0;
		for (uint64_t c = lane; c < N; c += 32) {
			const double2 m = M[r * N + c];
			const double x = in[c].x, y = in[c].y;
			re += m.x * x - m.y * y;
			im += m.x * y + m.y * x;
		}
		for (int o = 16; o > 0; o >>= 1) {
			re += __shfl_down_sync(0xffffffffu, re, o);
			im += __shfl_down_sync(0xffffffffu, im, o);
		}
		if (lane == 0) {
			cplx_t<T> v;
			v.x = static_cast<T>(re);
			v.y = static_cast<T>(im);
			out[r] = v;
		}
	}
}

cudaError_t ensure_red(Scratch& sc, size_t n) {
	if (sc.red_cap >= n) return cudaSuccess;
	if (sc.d_red) cudaFree(sc.d_red);
	sc.d_red = nullptr;
	sc.red_cap = 0;
	cudaError_t e = cudaMalloc(&sc.d_red, n * sizeof(double));
	if (e == cudaSuccess) sc.red_cap = n;
	return e;
}

cudaError_t ensure_pinned(Scratch& sc, size_t n) {
	if (sc.pinned_cap >= n) return cudaSuccess;
	if (sc.h_pinned) cudaFreeHost(sc.h_pinned);
	sc.h_pinned = nullptr;
	sc.pinned_cap = 0;
	cudaError_t e = cudaMallocHost(&sc.h_pinned, n * sizeof(double));
	if (e == cudaSuccess) sc.pinned_cap = n;
	return e;
}

int red_grid(uint64_t N, int sms) { return grid_for(N, kRedThreads, sms, 4); }

}  // namespace

template <typename T> cudaError_t launch_fill_zero(cplx_t<T>* s, uint64_t N, cudaStream_t st) {
	return cudaMemsetAsync(s, 0, N * sizeof(cplx_t<T>), st);
}

template <typename T> cudaError_t launch_fill_const(cplx_t<T>* s, uint64_t N, double re, double im, cudaStream_t st) {
	int dev = 0, sms = 148;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	k_fill<T><<<grid_for(N, 256, sms), 256, 0, st>>>(s, N, static_cast<T>(re), static_cast<T>(im));
	note_launches(1);
	return cudaGetLastError();
}

template <typename T> cudaError_t launch_set_one(cplx_t<T>* s, uint64_t idx, double re, double im, cudaStream_t st) {
	k_set_one<T><<<1, 1, 0, st>>>(s, idx, static_cast<T>(re), static_cast<T>(im));
	note_launches(1);
	return cudaGetLastError();
}

template <typename T>
cudaError_t reduce_masked_prob(const cplx_t<T>* s, uint64_t N, uint64_t mask, uint64_t value, Scratch& sc, int sms, cudaStream_t st,
                               double* result_host) {
	const int g = red_grid(N, sms);
	cudaError_t e = ensure_red(sc, static_cast<size_t>(g) + 4);
	if (e != cudaSuccess) return e;
	if ((e = ensure_pinned(sc, 4)) != cudaSuccess) return e;
	k_masked_prob<T><<<g, kRedThreads, 0, st>>>(s, N, mask, value, sc.d_red + 4);
	note_launches(1);
	k_fold<<<1, kRedThreads, 0, st>>>(sc.d_red + 4, g, 1, sc.d_red);
	note_launches(1);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	if ((e = cudaMemcpyAsync(sc.h_pinned, sc.d_red, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
	if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
	*result_host = sc.h_pinned[0];
	return cudaSuccess;
}

template <typename T>
cudaError_t launch_scale_masked(cplx_t<T>* s, uint64_t N, uint64_t mask, uint64_t value, double f, int sms, cudaStream_t st) {
	k_scale_masked<T><<<grid_for(N, 256, sms), 256, 0, st>>>(s, N, mask, value, f);
	note_launches(1);
	return cudaGetLastError();
}

template <typename T>
cudaError_t launch_div_complex(cplx_t<T>* s, uint64_t N, double re, double im, int sms, cudaStream_t st) {
	k_div_complex<T><<<grid_for(N, 256, sms), 256, 0, st>>>(s, N, re, im);
	note_launches(1);
	return cudaGetLastError();
}

template <typename T>
cudaError_t launch_probabilities(const cplx_t<T>* s, uint64_t N, double* out, int sms, cudaStream_t st) {
	k_probs<T><<<grid_for(N, 256, sms), 256, 0, st>>>(s, N, out);
	note_launches(1);
	return cudaGetLastError();
}

template <typename T, typename U>
static cudaError_t inner_impl(const cplx_t<T>* a, const U* b, uint64_t N, Scratch& sc, int sms, cudaStream_t st, double* re_im_host) {
	const int g = red_grid(N, sms);
	cudaError_t e = ensure_red(sc, 2 * static_cast<size_t>(g) + 4);
	if (e != cudaSuccess) return e;
	if ((e = ensure_pinned(sc, 4)) != cudaSuccess) return e;
	k_inner<T, U><<<g, kRedThreads, 0, st>>>(a, b, N, sc.d_red + 4);
	note_launches(1);
	k_fold<<<1, kRedThreads, 0, st>>>(sc.d_red + 4, g, 2, sc.d_red);
	note_launches(1);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	if ((e = cudaMemcpyAsync(sc.h_pinned, sc.d_red, 2 * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
	if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
	re_im_host[0] = sc.h_pinned[0];
	re_im_host[1] = sc.h_pinned[1];
	return cudaSuccess;
}

template <typename T>
cudaError_t inner_product(const cplx_t<T>* a, const cplx_t<T>* b, uint64_t N, Scratch& sc, int sms, cudaStream_t st, double* re_im_host) {
	return inner_impl<T, cplx_t<T>>(a, b, N, sc, sms, st, re_im_host);
}

template <typename T>
cudaError_t inner_product_f64b(const cplx_t<T>* a, const double2* b, uint64_t N, Scratch& sc, int sms, cudaStream_t st, double* re_im_host) {
	return inner_impl<T, double2>(a, b, N, sc, sms, st, re_im_host);
}

template <typename T>
cudaError_t sample(const cplx_t<T>* s, uint64_t N, const double* probs_host, size_t nshots, int mode, uint64_t fallback,
                   Scratch& sc, int sms, cudaStream_t st, uint64_t* out_host) {
	const uint64_t nchunks = (N + kChunk - 1) / kChunk;
	cudaError_t e;
	if (sc.chunk_cap < 2 * nchunks + 2) {
		if (sc.d_chunk) cudaFree(sc.d_chunk);
		sc.d_chunk = nullptr;
		sc.chunk_cap = 0;
		if ((e = cudaMalloc(&sc.d_chunk, (2 * nchunks + 2) * sizeof(double))) != cudaSuccess) return e;
		sc.chunk_cap = 2 * nchunks + 2;
	}
	if (sc.shot_cap < nshots + 1) {
		if (sc.d_probs) cudaFree(sc.d_probs);
		if (sc.d_out) cudaFree(sc.d_out);
		sc.d_probs = nullptr;
		sc.d_out = nullptr;
		sc.shot_cap = 0;
		if ((e = cudaMalloc(&sc.d_probs, (nshots + 1) * sizeof(double))) != cudaSuccess) return e;
		if ((e = cudaMalloc(&sc.d_out, (nshots + 1) * sizeof(unsigned long long))) != cudaSuccess) return e;
		sc.shot_cap = nshots + 1;
	}
	double* sums = sc.d_chunk;
	double* excl = sc.d_chunk + nchunks + 1;
	k_chunk_sums<T><<<grid_for(nchunks, 128, sms, 16), 128, 0, st>>>(s, N, nchunks, sums);
	note_launches(1);
	k_chunk_scan<<<1, 1024, 0, st>>>(sums, nchunks, excl);
	note_launches(1);
	if (nshots) {
		if ((e = cudaMemcpyAsync(sc.d_probs, probs_host, nshots * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
	}
	const uint64_t threads = nshots + 1;
	k_sample<T><<<static_cast<unsigned>((threads + 127) / 128), 128, 0, st>>>(s, N, excl, nchunks, sc.d_probs, nshots, mode, fallback, sc.d_out);
	note_launches(1);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	std::vector<unsigned long long> tmp(nshots + 1);
	if ((e = cudaMemcpyAsync(tmp.data(), sc.d_out, (nshots + (mode == 1 ? 1 : 0)) * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
		return e;
	if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
	if (mode == 1) {
		const uint64_t T_ = tmp[nshots];
		for (size_t k = 0; k < nshots; ++k) out_host[k] = (tmp[k] > T_) ? T_ + 1 : tmp[k];
	} else {
		for (size_t k = 0; k < nshots; ++k) out_host[k] = tmp[k];
	}
	return cudaSuccess;
}

template <typename T>
cudaError_t measure_small(cplx_t<T>* s, uint64_t N, double prob, uint64_t mask, int kind, uint64_t fallback, Scratch& sc,
                          cudaStream_t st, uint64_t* out_host) {
	if (N > kChunk) return cudaErrorInvalidValue;
	cudaError_t e = ensure_red(sc, 4);
	if (e == cudaSuccess) e = ensure_pinned(sc, 4);
	if (e != cudaSuccess) return e;
	auto* dv = reinterpret_cast<unsigned long long*>(sc.d_red);
	k_measure_small<T><<<1, kRedThreads, 0, st>>>(s, N, prob, mask, kind, fallback, dv);
	note_launches(1);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	if ((e = cudaMemcpyAsync(sc.h_pinned, dv, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
	if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
	std::memcpy(out_host, sc.h_pinned, sizeof(uint64_t));
	return cudaSuccess;
}

template <typename T>
cudaError_t convert_from_f64(cplx_t<T>* dst, const double2* src, uint64_t N, int sms, cudaStream_t st) {
	k_from_f64<T><<<grid_for(N, 256, sms), 256, 0, st>>>(dst, src, N);
	note_launches(1);
	return cudaGetLastError();
}

template <typename T>
cudaError_t convert_to_f64(double2* dst, const cplx_t<T>* src, uint64_t N, int sms, cudaStream_t st) {
	k_to_f64<T><<<grid_for(N, 256, sms), 256, 0, st>>>(dst, src, N);
	note_launches(1);
	return cudaGetLastError();
}

template <typename T>
cudaError_t launch_operator_matrix(const double2* M, const cplx_t<T>* in, cplx_t<T>* out, uint64_t N, int sms, cudaStream_t st) {
	k_opmat<T><<<grid_for(N * 32, 256, sms), 256, 0, st>>>(M, in, out, N);
	note_launches(1);
	return cudaGetLastError();
}

#define QCS_INST(T)                                                                                                   \
	template cudaError_t launch_fill_zero<T>(cplx_t<T>*, uint64_t, cudaStream_t);                                    \
	template cudaError_t launch_fill_const<T>(cplx_t<T>*, uint64_t, double, double, cudaStream_t);                   \
	template cudaError_t launch_set_one<T>(cplx_t<T>*, uint64_t, double, double, cudaStream_t);                      \
	template cudaError_t reduce_masked_prob<T>(const cplx_t<T>*, uint64_t, uint64_t, uint64_t, Scratch&, int, cudaStream_t, double*); \
	template cudaError_t launch_scale_masked<T>(cplx_t<T>*, uint64_t, uint64_t, uint64_t, double, int, cudaStream_t); \
	template cudaError_t launch_div_complex<T>(cplx_t<T>*, uint64_t, double, double, int, cudaStream_t);             \
	template cudaError_t launch_probabilities<T>(const cplx_t<T>*, uint64_t, double*, int, cudaStream_t);            \
	template cudaError_t inner_product<T>(const cplx_t<T>*, const cplx_t<T>*, uint64_t, Scratch&, int, cudaStream_t, double*); \
	template cudaError_t inner_product_f64b<T>(const cplx_t<T>*, const double2*, uint64_t, Scratch&, int, cudaStream_t, double*); \
	template cudaError_t sample<T>(const cplx_t<T>*, uint64_t, const double*, size_t, int, uint64_t, Scratch&, int, cudaStream_t, uint64_t*); \
	template cudaError_t measure_small<T>(cplx_t<T>*, uint64_t, double, uint64_t, int, uint64_t, Scratch&, cudaStream_t, uint64_t*); \
	template cudaError_t convert_from_f64<T>(cplx_t<T>*, const double2*, uint64_t, int, cudaStream_t);              \
	template cudaError_t convert_to_f64<T>(double2*, const cplx_t<T>*, uint64_t, int, cudaStream_t);                \
	template cudaError_t launch_operator_matrix<T>(const double2*, const cplx_t<T>*, cplx_t<T>*, uint64_t, int, cudaStream_t);

QCS_INST(double)
QCS_INST(float)

}  // namespace qcs
