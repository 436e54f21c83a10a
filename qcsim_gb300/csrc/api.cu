// C ABI of the GB300 statevector engine: register lifetime, QubitRegister::ApplyGate's trait
// dispatch, measurements and snapshots (declared in include/qcs_gpu.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "engine.cuh"
#include "batch.cuh"
#include "compile.cuh"

using qcs::BitPlan;
using qcs::DenseArgs;
using qcs::Mat2;
using qcs::Op1;
using qcs::SwapKind;

namespace {

using cd = std::complex<double>;

int fail(qcs_handle h, int status, const std::string& msg) {
	if (h) h->err = msg;
	return status;
}

int cuda_fail(qcs_handle h, cudaError_t e, const char* where) {
	if (e == cudaErrorMemoryAllocation) {
		cudaGetLastError();
		return fail(h, QCS_OUT_OF_MEMORY, std::string(where) + ": " + cudaGetErrorString(e));
	}
	return fail(h, QCS_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
}

#define QCS_CK(h, expr, where)                                  \
	do {                                                        \
		cudaError_t e_ = (expr);                                \
		if (e_ != cudaSuccess) return cuda_fail((h), e_, where); \
	} while (0)





// QubitRegister::CheckQubits (QubitRegister.h:677-690)
int check_qubits(qcs_handle h, uint32_t k, uint64_t q, uint64_t c1, uint64_t c2) {
	const uint64_t n = h->n;
	if (n == 0) return fail(h, QCS_INVALID_ARGUMENT, "Qubit number is zero");
	if (n <= q) return fail(h, QCS_INVALID_ARGUMENT, "Qubit number is too high");
	if (k == 2) {
		if (n <= c1) return fail(h, QCS_INVALID_ARGUMENT, "Controlling qubit number is too high");
		if (q == c1) return fail(h, QCS_INVALID_ARGUMENT, "Qubit and controlling qubit are the same");
	} else if (k == 3) {
		if (n <= c1 || n <= c2) return fail(h, QCS_INVALID_ARGUMENT, "Controlling qubit number is too high");
		if (q == c1 || q == c2 || c1 == c2) return fail(h, QCS_INVALID_ARGUMENT, "Qubits must be different");
	}
	if (k < 1 || k > 3) return fail(h, QCS_UNSUPPORTED, "gates act on 1, 2 or 3 qubits");
	return QCS_OK;
}

// scale factors taken out of gates are kept on the host and folded into the amplitudes before the
// state is read, measured or copied (and when their magnitude leaves a safe range)
int materialize(qcs_handle h) {
	if (h->scale == cd(1, 0)) return QCS_OK;
	cudaError_t e = h->prec == QCS_FP64
	                    ? qcs::launch_scale_complex<double>(static_cast<double2*>(h->d_state), h->N, h->scale.real(), h->scale.imag(), h->sms, h->stream)
	                    : qcs::launch_scale_complex<float>(static_cast<float2*>(h->d_state), h->N, h->scale.real(), h->scale.imag(), h->sms, h->stream);
	QCS_CK(h, e, "scale");
	h->scale = cd(1, 0);
	return QCS_OK;
}

// QubitRegister::ApplyGate (QubitRegister.h:434-486) through the compiled trait dispatch
cudaError_t dispatch_one(qcs_handle h, const qcs_gate& g) {
	const qcs::CompiledGate c = qcs::compile_gate(g, true);
	if (c.kind != qcs::GKind::Identity)
		qcs::prof_begin(h, qcs::kernel_name(c), 2.0 * h->amp_bytes() * static_cast<double>(h->N) * qcs::touched_fraction(c));
	cudaError_t e = h->prec == QCS_FP64 ? qcs::launch_compiled<double>(static_cast<double2*>(h->d_state), h->N, c, h->sms, h->stream)
	                                    : qcs::launch_compiled<float>(static_cast<float2*>(h->d_state), h->N, c, h->sms, h->stream);
	qcs::prof_end(h);
	if (e != cudaSuccess) return e;
	h->scale *= c.scale;
	const double mag = std::abs(h->scale);
	if (mag > h->scale_limit() || mag < 1.0 / h->scale_limit()) {
		if (materialize(h) != QCS_OK) return cudaErrorUnknown;
	}
	return cudaSuccess;
}

cudaError_t dispatch_any(qcs_handle h, const double* m, uint32_t k, uint32_t q0, uint32_t q1, uint32_t q2, uint32_t tr) {
	qcs_gate g;
	g.k = k;
	g.q0 = q0;
	g.q1 = q1;
	g.q2 = q2;
	g.traits = tr;
	g.reserved = 0;
	const int dim = 1 << k;
	std::memcpy(g.m, m, sizeof(double) * 2 * dim * dim);
	return dispatch_one(h, g);
}

int apply_checked(qcs_handle h, const double* m, uint32_t k, uint32_t q0, uint32_t q1, uint32_t q2, uint32_t tr) {
	const int st = check_qubits(h, k, q0, q1, q2);
	if (st != QCS_OK) return st;
	QCS_CK(h, dispatch_any(h, m, k, q0, q1, q2, tr), "apply gate");
	return QCS_OK;
}

// sum of |a_i|^2 over (i & mask) == value
int masked_prob(qcs_handle h, uint64_t mask, uint64_t value, double* out) {
	if (int st = materialize(h)) return st;
	cudaError_t e = h->prec == QCS_FP64
	                    ? qcs::reduce_masked_prob<double>(static_cast<double2*>(h->d_state), h->N, mask, value, h->sc, h->sms, h->stream, out)
	                    : qcs::reduce_masked_prob<float>(static_cast<float2*>(h->d_state), h->N, mask, value, h->sc, h->sms, h->stream, out);
	QCS_CK(h, e, "probability reduction");
	return QCS_OK;
}

int scale_masked(qcs_handle h, uint64_t mask, uint64_t value, double f) {
	cudaError_t e = h->prec == QCS_FP64
	                    ? qcs::launch_scale_masked<double>(static_cast<double2*>(h->d_state), h->N, mask, value, f, h->sms, h->stream)
	                    : qcs::launch_scale_masked<float>(static_cast<float2*>(h->d_state), h->N, mask, value, f, h->sms, h->stream);
	QCS_CK(h, e, "scale");
	return QCS_OK;
}

int sample_any(qcs_handle h, const double* probs, size_t n, int mode, uint64_t fallback, uint64_t* out) {
	if (int st = materialize(h)) return st;
	cudaError_t e = h->prec == QCS_FP64
	                    ? qcs::sample<double>(static_cast<double2*>(h->d_state), h->N, probs, n, mode, fallback, h->sc, h->sms, h->stream, out)
	                    : qcs::sample<float>(static_cast<float2*>(h->d_state), h->N, probs, n, mode, fallback, h->sc, h->sms, h->stream, out);
	QCS_CK(h, e, "sampling");
	return QCS_OK;
}

// a register of at most kSmallMeasure amplitudes: sampling and collapse in one launch (measure_small)
int measure_small_any(qcs_handle h, double prob, uint64_t mask, int kind, uint64_t fallback, uint64_t* out) {
	if (int st = materialize(h)) return st;
	cudaError_t e = h->prec == QCS_FP64
	                    ? qcs::measure_small<double>(static_cast<double2*>(h->d_state), h->N, prob, mask, kind, fallback, h->sc, h->stream, out)
	                    : qcs::measure_small<float>(static_cast<float2*>(h->d_state), h->N, prob, mask, kind, fallback, h->sc, h->stream, out);
	QCS_CK(h, e, "measurement");
	return QCS_OK;
}

int set_basis_impl(qcs_handle h, uint64_t state) {
	if (state < h->N) h->scale = cd(1, 0);
	if (state >= h->N) return QCS_OK;
	QCS_CK(h, cudaMemsetAsync(h->d_state, 0, h->state_bytes(), h->stream), "clear");
	cudaError_t e = h->prec == QCS_FP64 ? qcs::launch_set_one<double>(static_cast<double2*>(h->d_state), state, 1.0, 0.0, h->stream)
	                                    : qcs::launch_set_one<float>(static_cast<float2*>(h->d_state), state, 1.0, 0.0, h->stream);
	QCS_CK(h, e, "set basis");
	return QCS_OK;
}

int read_amp(qcs_handle h, uint64_t idx, cd* out) {
	if (int st = materialize(h)) return st;
	if (h->prec == QCS_FP64) {
		double v[2];
		QCS_CK(h, cudaMemcpyAsync(v, static_cast<char*>(h->d_state) + idx * 16, 16, cudaMemcpyDeviceToHost, h->stream), "read amplitude");
		QCS_CK(h, cudaStreamSynchronize(h->stream), "read amplitude");
		*out = cd(v[0], v[1]);
	} else {
		float v[2];
		QCS_CK(h, cudaMemcpyAsync(v, static_cast<char*>(h->d_state) + idx * 8, 8, cudaMemcpyDeviceToHost, h->stream), "read amplitude");
		QCS_CK(h, cudaStreamSynchronize(h->stream), "read amplitude");
		*out = cd(v[0], v[1]);
	}
	return QCS_OK;
}

int normalize_impl(qcs_handle h) {
	double ss = 0;
	int st = masked_prob(h, 0, 0, &ss);
	if (st) return st;
	const double nrm = std::sqrt(ss);
	if (nrm < 1E-20) return QCS_OK;
	return scale_masked(h, 0, 0, 1. / nrm);
}

constexpr uint64_t kStageAmps = 1ULL << 26;  // host<->device staging granularity for FP32 registers

void free_register(qcs_handle h) {
	if (!h) return;
	if (h->d_state) cudaFree(h->d_state);
	if (h->d_saved) cudaFree(h->d_saved);
	if (h->sc.d_red) cudaFree(h->sc.d_red);
	if (h->sc.d_chunk) cudaFree(h->sc.d_chunk);
	if (h->sc.d_probs) cudaFree(h->sc.d_probs);
	if (h->sc.d_out) cudaFree(h->sc.d_out);
	if (h->sc.h_pinned) cudaFreeHost(h->sc.h_pinned);
	qcs::batch_release(h);
	qcs::prof_release(h);
	qcs::release_cost_model(h);
	if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
	delete h;
}

}  // namespace

extern "C" {

const char* qcs_status_string(int status) {
	switch (status) {
	case QCS_OK: return "ok";
	case QCS_INVALID_ARGUMENT: return "invalid argument";
	case QCS_OUT_OF_MEMORY: return "out of memory";
	case QCS_CUDA_ERROR: return "CUDA error";
	case QCS_UNSUPPORTED: return "unsupported";
	}
	return "unknown status";
}

int qcs_create(uint32_t nqubits, int precision, qcs_handle* out) {
	if (!out) return QCS_INVALID_ARGUMENT;
	*out = nullptr;
	if (nqubits == 0) return QCS_INVALID_ARGUMENT;  // QubitRegister ctor asserts N > 0 (QubitRegister.h:22)
	if (nqubits > 36) return QCS_UNSUPPORTED;
	if (precision != QCS_FP64 && precision != QCS_FP32) return QCS_INVALID_ARGUMENT;
	auto* h = new (std::nothrow) qcs_register;
	if (!h) return QCS_OUT_OF_MEMORY;
	h->n = nqubits;
	h->N = 1ULL << nqubits;
	h->prec = precision;
	cudaError_t e = cudaGetDevice(&h->device);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
	if (e != cudaSuccess) {
		cudaGetLastError();
		delete h;
		return QCS_CUDA_ERROR;
	}
	h->own_stream = true;
	e = cudaMalloc(&h->d_state, h->state_bytes());
	if (e != cudaSuccess) {
		cudaGetLastError();
		h->d_state = nullptr;
		free_register(h);
		return e == cudaErrorMemoryAllocation ? QCS_OUT_OF_MEMORY : QCS_CUDA_ERROR;
	}
	if (set_basis_impl(h, 0) != QCS_OK || cudaStreamSynchronize(h->stream) != cudaSuccess) {
		free_register(h);
		return QCS_CUDA_ERROR;
	}
	*out = h;
	return QCS_OK;
}

int qcs_destroy(qcs_handle h) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (h->stream) cudaStreamSynchronize(h->stream);
	free_register(h);
	return QCS_OK;
}

int qcs_clone(qcs_handle h, qcs_handle* out) {
	if (h) {
		if (int st = materialize(h)) return st;
	}
	if (!h || !out) return QCS_INVALID_ARGUMENT;
	qcs_handle c = nullptr;
	int st = qcs_create(h->n, h->prec, &c);
	if (st) return fail(h, st, "clone: allocation failed");
	QCS_CK(h, cudaStreamSynchronize(h->stream), "clone");
	cudaError_t e = cudaMemcpyAsync(c->d_state, h->d_state, h->state_bytes(), cudaMemcpyDeviceToDevice, c->stream);
	if (e == cudaSuccess && h->has_saved) {
		e = cudaMalloc(&c->d_saved, h->state_bytes());
		if (e == cudaSuccess) {
			e = cudaMemcpyAsync(c->d_saved, h->d_saved, h->state_bytes(), cudaMemcpyDeviceToDevice, c->stream);
			c->has_saved = true;
		}
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
	if (e != cudaSuccess) {
		qcs_destroy(c);
		return cuda_fail(h, e, "clone");
	}
	*out = c;
	return QCS_OK;
}

int qcs_set_stream(qcs_handle h, void* cuda_stream) {
	if (!h) return QCS_INVALID_ARGUMENT;
	QCS_CK(h, cudaStreamSynchronize(h->stream), "set stream");
	if (cuda_stream) {
		if (h->own_stream) cudaStreamDestroy(h->stream);
		h->own_stream = false;
		h->stream = static_cast<cudaStream_t>(cuda_stream);
	} else if (!h->own_stream) {
		QCS_CK(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "set stream");
		h->own_stream = true;
	}
	return QCS_OK;
}

int qcs_set_option(qcs_handle h, int option, int value) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (option == QCS_OPT_PASSES) {
		h->batch_mode = value ? 1 : 0;
		return QCS_OK;
	}
	if (option == QCS_OPT_FUSION) {
		if (value < 0 || value > 2) return fail(h, QCS_INVALID_ARGUMENT, "fusion mode must be 0, 1 or 2");
		h->fusion = value;
		return QCS_OK;
	}
	if (option == QCS_OPT_FUSION_MAX_QUBITS) {
		if (value < 1 || value > 5) return fail(h, QCS_INVALID_ARGUMENT, "fused blocks hold 1 to 5 qubits");
		h->fusion_max = value;
		return QCS_OK;
	}
	if (option == QCS_OPT_TENSOR_CORES) {
		h->tensor_cores = value ? 1 : 0;
		return QCS_OK;
	}
	return fail(h, QCS_INVALID_ARGUMENT, "unknown option");
}

int qcs_synchronize(qcs_handle h) {
	if (!h) return QCS_INVALID_ARGUMENT;
	QCS_CK(h, cudaStreamSynchronize(h->stream), "synchronize");
	return QCS_OK;
}

const char* qcs_last_error(qcs_handle h) { return h ? h->err.c_str() : "null handle"; }
uint32_t qcs_nqubits(qcs_handle h) { return h ? h->n : 0; }
uint64_t qcs_nstates(qcs_handle h) { return h ? h->N : 0; }
int qcs_precision_of(qcs_handle h) { return h ? h->prec : -1; }
void* qcs_device_state(qcs_handle h) { return h ? h->d_state : nullptr; }

int qcs_set_basis(qcs_handle h, uint64_t state) {
	if (!h) return QCS_INVALID_ARGUMENT;
	return set_basis_impl(h, state);
}

int qcs_set_qubit_state(qcs_handle h, uint64_t q) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (q >= h->n) return QCS_OK;
	return set_basis_impl(h, 1ULL << q);
}

int qcs_set_cat(qcs_handle h) {
	if (h) h->scale = cd(1, 0);
	if (!h) return QCS_INVALID_ARGUMENT;
	QCS_CK(h, cudaMemsetAsync(h->d_state, 0, h->state_bytes(), h->stream), "cat");
	const double v = 1. / std::sqrt(2.);
	cudaError_t e;
	if (h->prec == QCS_FP64) {
		e = qcs::launch_set_one<double>(static_cast<double2*>(h->d_state), 0, v, 0, h->stream);
		if (e == cudaSuccess) e = qcs::launch_set_one<double>(static_cast<double2*>(h->d_state), h->N - 1, v, 0, h->stream);
	} else {
		e = qcs::launch_set_one<float>(static_cast<float2*>(h->d_state), 0, v, 0, h->stream);
		if (e == cudaSuccess) e = qcs::launch_set_one<float>(static_cast<float2*>(h->d_state), h->N - 1, v, 0, h->stream);
	}
	QCS_CK(h, e, "cat");
	return QCS_OK;
}

int qcs_set_equal(qcs_handle h) {
	if (h) h->scale = cd(1, 0);
	if (!h) return QCS_INVALID_ARGUMENT;
	const double v = 1. / std::sqrt(static_cast<double>(h->N));
	cudaError_t e = h->prec == QCS_FP64 ? qcs::launch_fill_const<double>(static_cast<double2*>(h->d_state), h->N, v, 0, h->stream)
	                                    : qcs::launch_fill_const<float>(static_cast<float2*>(h->d_state), h->N, v, 0, h->stream);
	QCS_CK(h, e, "equal superposition");
	return QCS_OK;
}

int qcs_clear(qcs_handle h) {
	if (h) h->scale = cd(1, 0);
	if (!h) return QCS_INVALID_ARGUMENT;
	QCS_CK(h, cudaMemsetAsync(h->d_state, 0, h->state_bytes(), h->stream), "clear");
	return QCS_OK;
}

int qcs_set_amplitude(qcs_handle h, uint64_t state, double re, double im) {
	if (h) {
		if (int st = materialize(h)) return st;
	}
	if (!h) return QCS_INVALID_ARGUMENT;
	if (state >= h->N) return QCS_OK;
	cudaError_t e = h->prec == QCS_FP64 ? qcs::launch_set_one<double>(static_cast<double2*>(h->d_state), state, re, im, h->stream)
	                                    : qcs::launch_set_one<float>(static_cast<float2*>(h->d_state), state, re, im, h->stream);
	QCS_CK(h, e, "set amplitude");
	return QCS_OK;
}

int qcs_get_amplitude(qcs_handle h, uint64_t state, double* re_im) {
	if (!h || !re_im) return QCS_INVALID_ARGUMENT;
	if (state >= h->N) {
		re_im[0] = re_im[1] = 0;
		return QCS_OK;
	}
	cd v;
	int st = read_amp(h, state, &v);
	if (st) return st;
	re_im[0] = v.real();
	re_im[1] = v.imag();
	return QCS_OK;
}

int qcs_get_state(qcs_handle h, double* host_out) {
	if (h && h->scale != cd(1, 0)) {
		if (int st = materialize(h)) return st;
	}
	if (!h || !host_out) return QCS_INVALID_ARGUMENT;
	if (h->prec == QCS_FP64) {
		QCS_CK(h, cudaMemcpyAsync(host_out, h->d_state, h->state_bytes(), cudaMemcpyDeviceToHost, h->stream), "get state");
		QCS_CK(h, cudaStreamSynchronize(h->stream), "get state");
		return QCS_OK;
	}
	const uint64_t chunk = std::min<uint64_t>(h->N, kStageAmps);
	double2* tmp = nullptr;
	QCS_CK(h, cudaMalloc(&tmp, chunk * sizeof(double2)), "get state");
	cudaError_t e = cudaSuccess;
	for (uint64_t off = 0; off < h->N && e == cudaSuccess; off += chunk) {
		const uint64_t n = std::min(chunk, h->N - off);
		e = qcs::convert_to_f64<float>(tmp, static_cast<float2*>(h->d_state) + off, n, h->sms, h->stream);
		if (e == cudaSuccess) e = cudaMemcpyAsync(host_out + 2 * off, tmp, n * sizeof(double2), cudaMemcpyDeviceToHost, h->stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
	}
	cudaFree(tmp);
	QCS_CK(h, e, "get state");
	return QCS_OK;
}

int qcs_set_state(qcs_handle h, const double* host_in) {
	if (h) h->scale = cd(1, 0);
	if (!h || !host_in) return QCS_INVALID_ARGUMENT;
	if (h->prec == QCS_FP64) {
		QCS_CK(h, cudaMemcpyAsync(h->d_state, host_in, h->state_bytes(), cudaMemcpyHostToDevice, h->stream), "set state");
		QCS_CK(h, cudaStreamSynchronize(h->stream), "set state");
		return QCS_OK;
	}
	const uint64_t chunk = std::min<uint64_t>(h->N, kStageAmps);
	double2* tmp = nullptr;
	QCS_CK(h, cudaMalloc(&tmp, chunk * sizeof(double2)), "set state");
	cudaError_t e = cudaSuccess;
	for (uint64_t off = 0; off < h->N && e == cudaSuccess; off += chunk) {
		const uint64_t n = std::min(chunk, h->N - off);
		e = cudaMemcpyAsync(tmp, host_in + 2 * off, n * sizeof(double2), cudaMemcpyHostToDevice, h->stream);
		if (e == cudaSuccess) e = qcs::convert_from_f64<float>(static_cast<float2*>(h->d_state) + off, tmp, n, h->sms, h->stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
	}
	cudaFree(tmp);
	QCS_CK(h, e, "set state");
	return QCS_OK;
}

int qcs_normalize(qcs_handle h) {
	if (!h) return QCS_INVALID_ARGUMENT;
	return normalize_impl(h);
}

// AdjustPhaseAndNormalize (QubitRegister.h:133-167): divide by the first of a_0, a_{N/2}, a_{N-1}
// whose magnitude is at least 1e-5, then Normalize
int qcs_adjust_phase_normalize(qcs_handle h) {
	if (!h) return QCS_INVALID_ARGUMENT;
	const uint64_t cand[3] = {0, h->N >> 1, h->N - 1};
	for (uint64_t c : cand) {
		cd v;
		int st = read_amp(h, c, &v);
		if (st) return st;
		if (std::abs(v) >= 1E-5) {
			cudaError_t e = h->prec == QCS_FP64
			                    ? qcs::launch_div_complex<double>(static_cast<double2*>(h->d_state), h->N, v.real(), v.imag(), h->sms, h->stream)
			                    : qcs::launch_div_complex<float>(static_cast<float2*>(h->d_state), h->N, v.real(), v.imag(), h->sms, h->stream);
			QCS_CK(h, e, "adjust phase");
			break;
		}
	}
	return normalize_impl(h);
}

int qcs_apply_gate(qcs_handle h, const double* m, uint32_t k, uint32_t q0, uint32_t q1, uint32_t q2, uint32_t traits) {
	if (!h || !m) return QCS_INVALID_ARGUMENT;
	return apply_checked(h, m, k, q0, q1, q2, traits);
}

int qcs_apply_gates(qcs_handle h, const qcs_gate* gates, size_t count) {
	if (!h || (!gates && count)) return QCS_INVALID_ARGUMENT;
	for (size_t i = 0; i < count; ++i) {
		const qcs_gate& g = gates[i];
		const int st = check_qubits(h, g.k, g.q0, g.q1, g.q2);
		if (st != QCS_OK) return st;
	}
	return qcs::batch_apply(h, gates, count);
}

int qcs_apply_operator_matrix(qcs_handle h, const double* m) {
	if (h) {
		if (int st = materialize(h)) return st;
	}
	if (!h || !m) return QCS_INVALID_ARGUMENT;
	if (h->n > 13) return fail(h, QCS_UNSUPPORTED, "dense operators are limited to 13 qubits (a 2^n x 2^n matrix)");
	double2* dM = nullptr;
	void* tmp = nullptr;
	const size_t mbytes = static_cast<size_t>(h->N) * h->N * sizeof(double2);
	QCS_CK(h, cudaMalloc(&dM, mbytes), "operator matrix");
	cudaError_t e = cudaMalloc(&tmp, h->state_bytes());
	if (e == cudaSuccess) e = cudaMemcpyAsync(dM, m, mbytes, cudaMemcpyHostToDevice, h->stream);
	if (e == cudaSuccess)
		e = h->prec == QCS_FP64
		        ? qcs::launch_operator_matrix<double>(dM, static_cast<double2*>(h->d_state), static_cast<double2*>(tmp), h->N, h->sms, h->stream)
		        : qcs::launch_operator_matrix<float>(dM, static_cast<float2*>(h->d_state), static_cast<float2*>(tmp), h->N, h->sms, h->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
	if (e == cudaSuccess) std::swap(h->d_state, tmp);
	cudaFree(dM);
	if (tmp) cudaFree(tmp);
	QCS_CK(h, e, "operator matrix");
	return QCS_OK;
}

int qcs_qft(qcs_handle h, uint32_t start, uint32_t end, int inverse, int do_swap) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (end >= h->n || start > end) return fail(h, QCS_INVALID_ARGUMENT, "QFT qubit range out of the register");
	return qcs::qft_apply(h, start, end, inverse != 0, do_swap != 0);
}

int qcs_one_qubit_transform(qcs_handle h, const double* m, uint32_t traits, uint32_t start, uint32_t end) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (!m) return fail(h, QCS_INVALID_ARGUMENT, "one-qubit transform: no gate matrix");
	// the range is checked before the list is built: end < n also keeps q <= end from wrapping
	if (end >= h->n || start > end) return fail(h, QCS_INVALID_ARGUMENT, "one-qubit transform: qubit range out of the register");
	std::vector<qcs_gate> gs;
	gs.reserve(end - start + 1);
	for (uint32_t q = start; q <= end; ++q) {
		qcs_gate g;
		std::memset(&g, 0, sizeof(g));
		g.k = 1;
		g.q0 = q;
		g.traits = traits;
		std::memcpy(g.m, m, 8 * sizeof(double));
		gs.push_back(g);
	}
	return qcs_apply_gates(h, gs.data(), gs.size());
}

int qcs_measure_all(qcs_handle h, double prob, uint64_t* state_out) {
	if (!h || !state_out) return QCS_INVALID_ARGUMENT;
	if (h->N <= qcs::kSmallMeasure) return measure_small_any(h, prob, 0, 1, h->N - 1, state_out);
	uint64_t st = 0;
	int r = sample_any(h, &prob, 1, 0, h->N - 1, &st);
	if (r) return r;
	if ((r = set_basis_impl(h, st))) return r;
	*state_out = st;
	return QCS_OK;
}

int qcs_measure(qcs_handle h, uint32_t first, uint32_t second, double prob, uint64_t* value_out) {
	if (!h || !value_out) return QCS_INVALID_ARGUMENT;
	if (second >= 63 || first >= 63) return fail(h, QCS_INVALID_ARGUMENT, "measured qubit out of range");
	const uint64_t firstMask = (1ULL << first) - 1;
	const uint64_t mask = (1ULL << (second + 1)) - 1 - firstMask;
	uint64_t st = 0;
	if (h->N <= qcs::kSmallMeasure) {
		if (int r = measure_small_any(h, prob, mask, 0, 0, &st)) return r;
		*value_out = (st & mask) >> first;
		return QCS_OK;
	}
	int r = sample_any(h, &prob, 1, 0, 0, &st);
	if (r) return r;
	const uint64_t picked = st & mask;
	double acc = 0;
	if ((r = masked_prob(h, mask, picked, &acc))) return r;
	if ((r = scale_masked(h, mask, picked, 1. / std::sqrt(acc)))) return r;
	*value_out = picked >> first;
	return QCS_OK;
}

int qcs_measure_no_collapse(qcs_handle h, double prob, uint64_t* state_out) {
	if (!h || !state_out) return QCS_INVALID_ARGUMENT;
	if (h->N <= qcs::kSmallMeasure) return measure_small_any(h, prob, 0, 2, 0, state_out);
	return sample_any(h, &prob, 1, 0, 0, state_out);
}

int qcs_sample(qcs_handle h, const double* probs, size_t nshots, uint64_t* states_out) {
	if (!h || (nshots && (!probs || !states_out))) return QCS_INVALID_ARGUMENT;
	return sample_any(h, probs, nshots, 1, h->N, states_out);
}

int qcs_qubit_probability(qcs_handle h, uint32_t qubit, double* p_out) {
	if (!h || !p_out) return QCS_INVALID_ARGUMENT;
	if (qubit >= 63) return fail(h, QCS_INVALID_ARGUMENT, "qubit out of range");
	// the pending global factor stays pending: amplitudes = scale x stored values, so the probability
	// is |scale|^2 times the stored values' sum (no sweep folding the factor into the amplitudes)
	cudaError_t e = h->prec == QCS_FP64 ? qcs::reduce_masked_prob<double>(static_cast<double2*>(h->d_state), h->N, 1ULL << qubit,
	                                                                      1ULL << qubit, h->sc, h->sms, h->stream, p_out)
	                                    : qcs::reduce_masked_prob<float>(static_cast<float2*>(h->d_state), h->N, 1ULL << qubit,
	                                                                     1ULL << qubit, h->sc, h->sms, h->stream, p_out);
	QCS_CK(h, e, "probability reduction");
	*p_out *= std::norm(h->scale);
	return QCS_OK;
}

int qcs_probabilities(qcs_handle h, double* host_out) {
	if (h && h->scale != cd(1, 0)) {
		if (int st = materialize(h)) return st;
	}
	if (!h || !host_out) return QCS_INVALID_ARGUMENT;
	const uint64_t chunk = std::min<uint64_t>(h->N, kStageAmps);
	double* tmp = nullptr;
	QCS_CK(h, cudaMalloc(&tmp, chunk * sizeof(double)), "probabilities");
	cudaError_t e = cudaSuccess;
	for (uint64_t off = 0; off < h->N && e == cudaSuccess; off += chunk) {
		const uint64_t n = std::min(chunk, h->N - off);
		e = h->prec == QCS_FP64 ? qcs::launch_probabilities<double>(static_cast<double2*>(h->d_state) + off, n, tmp, h->sms, h->stream)
		                        : qcs::launch_probabilities<float>(static_cast<float2*>(h->d_state) + off, n, tmp, h->sms, h->stream);
		if (e == cudaSuccess) e = cudaMemcpyAsync(host_out + off, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
	}
	cudaFree(tmp);
	QCS_CK(h, e, "probabilities");
	return QCS_OK;
}

// stateFidelity (QubitRegister.h:527-534): the host vector is staged in chunks; partial inner
// products are added in chunk order
int qcs_fidelity_host(qcs_handle h, const double* host_state, double* f_out) {
	if (h && h->scale != cd(1, 0)) {
		if (int st = materialize(h)) return st;
	}
	if (!h || !host_state || !f_out) return QCS_INVALID_ARGUMENT;
	const uint64_t chunk = std::min<uint64_t>(h->N, kStageAmps);
	double2* tmp = nullptr;
	QCS_CK(h, cudaMalloc(&tmp, chunk * sizeof(double2)), "fidelity");
	cudaError_t e = cudaSuccess;
	double re = 0, im = 0;
	for (uint64_t off = 0; off < h->N && e == cudaSuccess; off += chunk) {
		const uint64_t n = std::min(chunk, h->N - off);
		double part[2] = {0, 0};
		e = cudaMemcpyAsync(tmp, host_state + 2 * off, n * sizeof(double2), cudaMemcpyHostToDevice, h->stream);
		if (e == cudaSuccess)
			e = h->prec == QCS_FP64
			        ? qcs::inner_product_f64b<double>(static_cast<double2*>(h->d_state) + off, tmp, n, h->sc, h->sms, h->stream, part)
			        : qcs::inner_product_f64b<float>(static_cast<float2*>(h->d_state) + off, tmp, n, h->sc, h->sms, h->stream, part);
		re += part[0];
		im += part[1];
	}
	cudaFree(tmp);
	QCS_CK(h, e, "fidelity");
	*f_out = re * re + im * im;
	return QCS_OK;
}

int qcs_inner(qcs_handle h, qcs_handle other, double* re_im_out) {
	if (h && other) {
		if (int st = materialize(h)) return st;
		if (int st = materialize(other)) return st;
	}
	if (!h || !other || !re_im_out) return QCS_INVALID_ARGUMENT;
	if (other->N != h->N || other->prec != h->prec) return fail(h, QCS_INVALID_ARGUMENT, "registers differ in size or precision");
	QCS_CK(h, cudaStreamSynchronize(other->stream), "inner product");
	cudaError_t e = h->prec == QCS_FP64
	                    ? qcs::inner_product<double>(static_cast<double2*>(h->d_state), static_cast<double2*>(other->d_state), h->N, h->sc, h->sms, h->stream, re_im_out)
	                    : qcs::inner_product<float>(static_cast<float2*>(h->d_state), static_cast<float2*>(other->d_state), h->N, h->sc, h->sms, h->stream, re_im_out);
	QCS_CK(h, e, "inner product");
	return QCS_OK;
}

int qcs_save_state(qcs_handle h) {
	if (h) {
		if (int st = materialize(h)) return st;
	}
	if (!h) return QCS_INVALID_ARGUMENT;
	if (!h->d_saved) QCS_CK(h, cudaMalloc(&h->d_saved, h->state_bytes()), "save state");
	QCS_CK(h, cudaMemcpyAsync(h->d_saved, h->d_state, h->state_bytes(), cudaMemcpyDeviceToDevice, h->stream), "save state");
	h->has_saved = true;
	return QCS_OK;
}

int qcs_restore_state(qcs_handle h) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (!h->has_saved) return QCS_OK;
	h->scale = cd(1, 0);
	QCS_CK(h, cudaMemcpyAsync(h->d_state, h->d_saved, h->state_bytes(), cudaMemcpyDeviceToDevice, h->stream), "restore state");
	return QCS_OK;
}

int qcs_restore_state_destructive(qcs_handle h) {
	if (!h) return QCS_INVALID_ARGUMENT;
	if (!h->has_saved) return QCS_OK;
	QCS_CK(h, cudaStreamSynchronize(h->stream), "restore state");
	h->scale = cd(1, 0);
	std::swap(h->d_state, h->d_saved);
	cudaFree(h->d_saved);
	h->d_saved = nullptr;
	h->has_saved = false;
	return QCS_OK;
}

// ExpectationValue (QubitRegister.h:646-660)
int qcs_expectation(qcs_handle h, const qcs_gate* gates, size_t count, double* re_im_out) {
	if (h) {
		if (int st = materialize(h)) return st;
	}
	if (!h || !re_im_out || (count && !gates)) return QCS_INVALID_ARGUMENT;
	if (count == 0) {
		re_im_out[0] = 1;
		re_im_out[1] = 0;
		return QCS_OK;
	}
	void* copy = nullptr;
	QCS_CK(h, cudaMalloc(&copy, h->state_bytes()), "expectation");
	cudaError_t e = cudaMemcpyAsync(copy, h->d_state, h->state_bytes(), cudaMemcpyDeviceToDevice, h->stream);
	if (e != cudaSuccess) {
		cudaFree(copy);
		return cuda_fail(h, e, "expectation");
	}
	int st = qcs_apply_gates(h, gates, count);
	if (st == QCS_OK) st = materialize(h);
	if (st == QCS_OK) {
		e = h->prec == QCS_FP64
		        ? qcs::inner_product<double>(static_cast<double2*>(copy), static_cast<double2*>(h->d_state), h->N, h->sc, h->sms, h->stream, re_im_out)
		        : qcs::inner_product<float>(static_cast<float2*>(copy), static_cast<float2*>(h->d_state), h->N, h->sc, h->sms, h->stream, re_im_out);
		if (e != cudaSuccess) st = cuda_fail(h, e, "expectation");
	}
	cudaStreamSynchronize(h->stream);
	std::swap(h->d_state, copy);  // restore the state
	cudaFree(copy);
	return st;
}

struct qcs_rng {
	std::mt19937_64 g;
	std::uniform_real_distribution<double> u{0, 1};
};

int qcs_rng_create(uint64_t seed, qcs_rng_handle* out) {
	if (!out) return QCS_INVALID_ARGUMENT;
	*out = new (std::nothrow) qcs_rng;
	if (!*out) return QCS_OUT_OF_MEMORY;
	(*out)->g.seed(seed);
	return QCS_OK;
}

int qcs_rng_destroy(qcs_rng_handle g) {
	delete g;
	return QCS_OK;
}

int qcs_rng_uniform(qcs_rng_handle g, double* out, size_t n) {
	if (!g || (n && !out)) return QCS_INVALID_ARGUMENT;
	for (size_t i = 0; i < n; ++i) out[i] = g->u(g->g);
	return QCS_OK;
}

}  // extern "C"

namespace qcs {
static std::atomic<uint64_t> g_launches{0};
void note_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace qcs

extern "C" uint64_t qcs_launch_count(void) { return qcs::g_launches.load(); }

extern "C" int qcs_scratch_bytes(qcs_handle h, uint64_t* device_bytes, uint64_t* pinned_bytes) {
	if (!h || !device_bytes || !pinned_bytes) return QCS_INVALID_ARGUMENT;
	const qcs::Scratch& sc = h->sc;
	*device_bytes = sizeof(double) * (sc.red_cap + sc.chunk_cap) + (sizeof(double) + sizeof(unsigned long long)) * sc.shot_cap;
	*pinned_bytes = sizeof(double) * sc.pinned_cap;
	return QCS_OK;
}

// exported for the batch planner: one gate through the per-gate kernels, and the scale fold
namespace qcs {
cudaError_t apply_one(qcs_handle h, const qcs_gate& g) { return dispatch_one(h, g); }
int fold_scale(qcs_handle h) { return materialize(h); }
}  // namespace qcs
