// Internal declarations of the GB300 statevector engine (behind include/qcs_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <complex>
#include <cstddef>
#include <string>
#include <vector>

#include "qcs_gpu.h"

namespace qcs {

// ---------------------------------------------------------------------------------------------
// amplitude types
// ---------------------------------------------------------------------------------------------
template <typename T> struct cplx;
template <> struct cplx<double> { using type = double2; };
template <> struct cplx<float> { using type = float2; };
template <typename T> using cplx_t = typename cplx<T>::type;

// a gate's matrix entries in the register's precision
template <typename T> struct Mat2 { cplx_t<T> m00, m01, m10, m11; };

// 1-qubit (or controlled 1-qubit) arithmetic chosen on the host from the trait dispatch and the
// values of the entries the reference reads
enum class Op1 : int {
	Diag = 0,        // a0 *= d0, a1 *= d1
	Phase,           // a1 *= d1 (d0 == 1)
	PhaseNeg,        // a1 = -a1 (d0 == 1, d1 == -1)
	PhaseI,          // a1 *= +-i (d0 == 1, d1 == +-i; sign in m11.y)
	Antidiag,        // (a0, a1) <- (m01 a1, m10 a0)
	Swap,            // (a0, a1) <- (a1, a0)
	Real,            // real 2x2
	RxLike,          // real diagonal, imaginary off-diagonal
	Generic,         // complex 2x2
	AntidiagUnit,    // (a0, a1) <- (u01 a1, u10 a0), u in {1, i, -1, -i}
	UnitRe01,        // factored rotations: one +-1 entry per row, the other real or imaginary
	UnitRe10,
	UnitIm01,
	UnitIm10
};

enum class SwapKind : int { Plain = 0, ISwap, ISwapDag };

constexpr int kMaxInsert = 3;

// positions of the bits that a work item does not enumerate (sorted ascending), the bits forced to
// one (controls), and the gate qubits
struct BitPlan {
	int nins = 0;
	int ins[kMaxInsert] = {0, 0, 0};
	uint64_t set_mask = 0;
};

struct DenseArgs {
	int k = 0;            // 2 or 3 qubits in the dense block
	uint64_t bit[3] = {0, 0, 0};  // bit masks of matrix bit 0, 1, 2
	double m[128];        // 2^k x 2^k complex, row-major interleaved
};

// ---------------------------------------------------------------------------------------------
// the register object behind qcs_handle
// ---------------------------------------------------------------------------------------------
struct Scratch {
	double* d_red = nullptr;      // reduction partials
	size_t red_cap = 0;           // in doubles
	double* d_chunk = nullptr;    // chunk sums / exclusive prefix for sampling
	size_t chunk_cap = 0;         // in doubles
	double* d_probs = nullptr;    // sampling inputs
	unsigned long long* d_out = nullptr;  // sampling outputs
	size_t shot_cap = 0;
	double* h_pinned = nullptr;   // small pinned host buffer
	size_t pinned_cap = 0;        // in doubles
};

// the bound on a register's pending global factor: it is folded into the amplitudes once its magnitude
// leaves [1/limit, limit], so that stored values (amplitude / scale) stay far inside the precision's range
inline double scale_limit_of(int prec) { return prec == QCS_FP64 ? 1e100 : 1e15; }

}  // namespace qcs

struct qcs_register {
	uint32_t n = 0;
	uint64_t N = 0;
	int prec = QCS_FP64;
	void* d_state = nullptr;
	void* d_saved = nullptr;
	bool has_saved = false;
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	int device = 0;
	int sms = 148;
	qcs::Scratch sc;
	std::complex<double> scale{1.0, 0.0};  // amplitudes = scale * stored values
	void* batch = nullptr;                 // planner buffers (batch.cu)
	int batch_mode = 1;                    // QCS_OPT_PASSES
	int fusion = -1;                       // QCS_OPT_FUSION (-1: by precision)
	int fusion_max = 0;                    // QCS_OPT_FUSION_MAX_QUBITS (0: by precision and size, fusion_limit)
	int tensor_cores = 1;                  // QCS_OPT_TENSOR_CORES
	void* cost_ctx = nullptr;              // learned partition choice (costmodel.cu)
	double last_predicted_ms = 0;          // its prediction for the last fused gate list
	size_t last_blocks = 0;                // blocks of the last fused gate list
	void* prof = nullptr;                  // launch timing records (profile.cu), when enabled
	std::string err;
	size_t amp_bytes() const { return prec == QCS_FP64 ? 16 : 8; }
	double scale_limit() const { return qcs::scale_limit_of(prec); }
	size_t state_bytes() const { return static_cast<size_t>(N) * amp_bytes(); }
	// the largest fused block: the option when set; otherwise 4 for FP32 registers of at least 26 qubits
	// with the tensor cores on (tensor-core passes of 4-qubit blocks were the fastest greedy partitions
	// there, ahead of 5-qubit blocks and of blocks of at most 3 on the CUDA cores), else 3
	int fusion_limit() const {
		if (fusion_max > 0) return fusion_max;
		return prec == QCS_FP32 && tensor_cores && n >= 26 ? 4 : 3;
	}
};

namespace qcs {

// launch timing (profile.cu): no-ops unless profiling is enabled on the register; fp_ops = the
// floating-point instructions the launch's gate arithmetic issues, where the launcher counts them
void prof_begin(qcs_handle h, const char* name, double bytes, double fp_ops = 0);
void prof_end(qcs_handle h);
void prof_release(qcs_handle h);

// ---- kernel launchers (gate_kernels.cu) ----
template <typename T>
cudaError_t launch_ctrl1q(cplx_t<T>* s, uint64_t N, Op1 op, const Mat2<T>& m, uint64_t tbit, const BitPlan& plan,
                          int sms, cudaStream_t st);
template <typename T>
cudaError_t launch_swap(cplx_t<T>* s, uint64_t N, SwapKind kind, uint64_t bitA, uint64_t bitB, const BitPlan& plan,
                        int sms, cudaStream_t st);
template <typename T>
cudaError_t launch_dense(cplx_t<T>* s, uint64_t N, const DenseArgs& a, const BitPlan& plan, int sms, cudaStream_t st);

// ---- state / measurement kernels (measure_kernels.cu) ----
template <typename T> cudaError_t launch_fill_zero(cplx_t<T>* s, uint64_t N, cudaStream_t st);
template <typename T> cudaError_t launch_fill_const(cplx_t<T>* s, uint64_t N, double re, double im, cudaStream_t st);
template <typename T> cudaError_t launch_set_one(cplx_t<T>* s, uint64_t idx, double re, double im, cudaStream_t st);
// sum of |a_i|^2 over i with (i & mask) == value, deterministic order
template <typename T>
cudaError_t reduce_masked_prob(const cplx_t<T>* s, uint64_t N, uint64_t mask, uint64_t value, Scratch& sc, int sms,
                               cudaStream_t st, double* result_host);
// a_i *= ((i & mask) == value) ? f : 0
template <typename T>
cudaError_t launch_scale_masked(cplx_t<T>* s, uint64_t N, uint64_t mask, uint64_t value, double f, int sms, cudaStream_t st);
template <typename T>
cudaError_t launch_div_complex(cplx_t<T>* s, uint64_t N, double re, double im, int sms, cudaStream_t st);
template <typename T>
cudaError_t launch_probabilities(const cplx_t<T>* s, uint64_t N, double* out, int sms, cudaStream_t st);
// <a|b> (b may be complex<double> host-staged data converted on the device)
template <typename T>
cudaError_t inner_product(const cplx_t<T>* a, const cplx_t<T>* b, uint64_t N, Scratch& sc, int sms, cudaStream_t st,
                          double* re_im_host);
template <typename T>
cudaError_t inner_product_f64b(const cplx_t<T>* a, const double2* b, uint64_t N, Scratch& sc, int sms, cudaStream_t st,
                               double* re_im_host);
// sampling: mode 0 = first index with running sum >= prob (fallback per query),
// mode 1 = RepeatedMeasure semantics (truncated table + lower_bound)
template <typename T>
cudaError_t sample(const cplx_t<T>* s, uint64_t N, const double* probs_host, size_t nshots, int mode,
                   uint64_t fallback, Scratch& sc, int sms, cudaStream_t st, uint64_t* out_host);
// registers of at most 2048 amplitudes: one measurement in one launch (kind 0: Measure with collapse onto
// the sampled value of the `mask` qubits; 1: MeasureAll; 2: MeasureNoCollapse); *out_host = the sampled
// state, `fallback` when the running sum never reaches prob
constexpr uint64_t kSmallMeasure = 2048;
template <typename T>
cudaError_t measure_small(cplx_t<T>* s, uint64_t N, double prob, uint64_t mask, int kind, uint64_t fallback, Scratch& sc,
                          cudaStream_t st, uint64_t* out_host);
template <typename T>
cudaError_t convert_from_f64(cplx_t<T>* dst, const double2* src, uint64_t N, int sms, cudaStream_t st);
template <typename T>
cudaError_t convert_to_f64(double2* dst, const cplx_t<T>* src, uint64_t N, int sms, cudaStream_t st);

// dense 2^n x 2^n operator (row-major complex<double>) applied out of place: out = M * in
template <typename T>
cudaError_t launch_operator_matrix(const double2* M, const cplx_t<T>* in, cplx_t<T>* out, uint64_t N, int sms, cudaStream_t st);

// kernels launched by this library (qcs_launch_count)
void note_launches(uint64_t n);

inline int grid_for(uint64_t work, int threads, int sms, int per_sm = 8) {
	uint64_t b = (work + threads - 1) / threads;
	const uint64_t cap = static_cast<uint64_t>(sms) * per_sm;
	if (b > cap) b = cap;
	if (b < 1) b = 1;
	return static_cast<int>(b);
}

}  // namespace qcs
