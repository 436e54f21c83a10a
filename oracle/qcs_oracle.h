/*
 * CPU oracle for the statevector hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++17 (+OpenMP) restatement of QCSim's QubitRegister / QubitRegisterCalculator behaviour:
 * the gate matrices and traits (QCSim/SimpleGates.h, QCSim/QuantumGate.h), the trait-based ApplyGate
 * dispatch (QCSim/QubitRegister.h:434-486), every gate-application loop
 * (QCSim/QubitRegisterCalculator.h:39-939), the measurement scans, norms and collapses
 * (QubitRegister.h:169-429, QubitRegisterCalculator.h:948-1254), the QFT gate sequence
 * (QCSim/QuantumFourierTransform.h:35-87, QCSim/QubitsSwapper.h:23-34) and the QAOA circuit and
 * Ising energy (QCSim/IsingModel.h:106-119, 203-206, 491-567).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this library, and
 * only as the checker or the timed CPU baseline.  Nothing in the product links or calls it.
 *
 * Parity pin: the restatement is checked against the compiled reference itself (QCSim's own headers
 * built against a small Eigen stand-in, see oracle/Makefile target `ref`) through golden fixtures
 * in tests/golden/, generated by tests/golden/make_golden.py.
 *
 * Matrices cross the boundary row-major with interleaved (re, im) doubles: m[2*(r*dim+c)+{0,1}].
 */
#ifndef QCS_ORACLE_H
#define QCS_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gate codes: one per gate class of QCSim/SimpleGates.h and QCSim/QuantumGate.h, plus
 * matrix-only gates that behave like QC::Gates::AppliedGate (no trait overrides). */
enum qo_gate_code {
	QO_H = 0, QO_HY = 1, QO_S = 2, QO_SDG = 3, QO_T = 4, QO_TDG = 5, QO_P = 6, QO_X = 7, QO_Y = 8, QO_Z = 9,
	QO_SX = 10, QO_SXDG = 11, QO_SPLITTER = 12, QO_RX = 13, QO_RY = 14, QO_RZ = 15, QO_U = 16,
	QO_SWAP = 20, QO_ISWAP = 21, QO_ISWAPDG = 22, QO_DECREMENT = 23, QO_CX = 24, QO_CY = 25, QO_CZ = 26,
	QO_CH = 27, QO_CSX = 28, QO_CSXDG = 29, QO_CS = 30, QO_CP = 31, QO_CU = 32, QO_CRX = 33, QO_CRY = 34,
	QO_CRZ = 35,
	QO_CCX = 40, QO_CSWAP = 41, QO_CCZ = 42,
	QO_CUSTOM1 = 50, QO_CUSTOM2 = 51, QO_CUSTOM3 = 52
};

/* Trait bits, one per virtual of QC::Gates::QuantumGate (SimpleGates.h:27-60). */
enum qo_trait {
	QO_TR_DIAGONAL = 1, QO_TR_ANTIDIAGONAL = 2, QO_TR_SWAP = 4, QO_TR_ISWAP = 8, QO_TR_ISWAPDAG = 16,
	QO_TR_CONTROLLED = 32, QO_TR_CONTROLQ1 = 64
};

typedef struct qo_gate {
	int32_t code;
	int32_t q0, q1, q2;   /* ApplyGate(gate, q0, q1, q2): q0 = target, q1 = controllingQubit1, q2 = controllingQubit2 */
	double p[4];          /* angle parameters (theta, phi, lambda, gamma) */
	double m[128];        /* matrix for QO_CUSTOM*, row-major interleaved complex */
} qo_gate;

/* gate matrix + traits exactly as the reference gate class builds them */
int qo_gate_matrix(int32_t code, const double* params, const double* custom, double* m_out, uint32_t* k_out, uint32_t* traits_out);

void* qo_create(uint32_t nqubits);
void qo_destroy(void* r);
void qo_set_multithreading(void* r, int enable);
void qo_set_threads(int nthreads);
int qo_max_threads(void);

/* ApplyGate for each gate in order; returns 0, or 1 for an invalid-argument error (message via qo_last_error) */
int qo_apply(void* r, const qo_gate* gates, size_t count);
const char* qo_last_error(void* r);

void qo_get_state(void* r, double* out);
void qo_set_state(void* r, const double* in);
uint64_t qo_nstates(void* r);

void qo_set_basis(void* r, uint64_t state);
void qo_set_qubit_state(void* r, uint64_t q);
void qo_set_cat(void* r);
void qo_set_equal(void* r);
void qo_clear(void* r);
void qo_set_raw(void* r, uint64_t state, double re, double im);
void qo_normalize(void* r);
void qo_adjust_phase_normalize(void* r);

uint64_t qo_measure_all(void* r, double prob);
uint64_t qo_measure(void* r, uint32_t first, uint32_t second, double prob);
uint64_t qo_measure_no_collapse(void* r, double prob);
uint64_t qo_measure_no_collapse_sub(void* r, uint32_t first, uint32_t second, double prob);
/* RepeatedMeasure: truncated cumulative distribution + lower_bound per shot (QubitRegister.h:243-271) */
void qo_sample(void* r, const double* probs, size_t nshots, uint64_t* out);
double qo_qubit_probability(void* r, uint32_t q);
double qo_fidelity(void* r, const double* other);
void qo_inner(void* r, const double* other, double* re, double* im);

/* QuantumFourierTransform::QFT / IQFT on qubits [start, end] */
int qo_qft(void* r, uint32_t start, uint32_t end, int inverse, int do_swap);

/* QAOA: QAOAIsingSubalgorithm::Exec for one instance; edges as (i, j) pairs with i < j.
 * Edge order is the order the reference would visit (site i ascending here, then j). */
int qo_qaoa_exec(void* r, uint32_t nedges, const uint32_t* edges, const double* J, const double* h,
                 uint32_t p, const double* gammas, const double* betas);
double qo_ising_energy(uint32_t n, uint32_t nedges, const uint32_t* edges, const double* J, const double* h, uint64_t state);
double qo_expected_energy(void* r, uint32_t nedges, const uint32_t* edges, const double* J, const double* h);

/* std::mt19937_64 seeded with one value, and std::uniform_real_distribution<double>(0,1) on it
 * (restated from the C++ standard's definitions, as libstdc++ implements generate_canonical). */
void* qo_rng_create(uint64_t seed);
void qo_rng_destroy(void* g);
uint64_t qo_rng_next(void* g);
double qo_rng_uniform(void* g);

/* bench inputs and checks at full size (OpenMP over all host threads):
 * a random state a_x = (g1 + i g2) / norm, g iid N(0, 1) from std::normal_distribution<double> on
 * std::mt19937_64; the 2^n amplitudes are drawn in blocks of 2^20, block b from the generator seeded
 * with seed * 1000003 + b, so that the blocks can be drawn in parallel.  out: 2^n complex<double>. */
void qo_random_normal_state(uint64_t seed, uint32_t n, double* out);
/* max over i of |a_i - b_i| for `count` complex<double> entries */
double qo_max_abs_diff(const double* a, const double* b, uint64_t count);

#ifdef __cplusplus
}
#endif

#endif
