/*
 * qcs_gpu.h — C ABI of the GB300 statevector engine (libqcs_gpu.so).
 *
 * The engine replaces the statevector hot path of QCSim: QC::QubitRegister (QCSim/QubitRegister.h)
 * and the static gate/measurement loops of QC::QubitRegisterCalculator
 * (QCSim/QubitRegisterCalculator.h).  Each entry point below names the reference member it
 * replaces.  Plain pointers and sizes only; no C++ or CUDA types cross the boundary.
 *
 * Conventions
 *  - A register of n qubits holds 2^n amplitudes; bit q of a basis-state index is qubit q
 *    (QubitRegister.h:7).  Amplitudes are complex<double> (re, im interleaved, 16 bytes) in
 *    QCS_FP64 registers and complex<float> in QCS_FP32 registers; host buffers are always
 *    complex<double>.
 *  - Gate matrices are 2^k x 2^k complex, row-major, (re, im) interleaved: m[2*(r*2^k + c)].
 *    Row/column bit 0 is `q0` (the target), bit 1 is `q1` (controllingQubit1) and bit 2 is `q2`
 *    (controllingQubit2), as in SimpleGates.h:329 and :430.
 *  - Gate traits are the answers of the gate object's virtuals (SimpleGates.h:27-60), captured by the
 *    caller; the engine dispatches on them exactly as QubitRegister::ApplyGate does
 *    (QubitRegister.h:434-486), so only the matrix entries that the reference reads are used.
 *  - Measurement randomness stays with the caller: each sampling call takes `prob` values, which the
 *    reference computes as 1 - uniform(rng) (QubitRegister.h:171, 210, 267, 621, 707).
 *  - Every call is ordered on the register's CUDA stream.  Calls that return values to the host
 *    synchronise that stream.  A handle is not thread-safe (same as the reference object).
 *  - Errors: a non-zero status; qcs_last_error(h) gives the message.  For invalid qubit arguments
 *    the messages are those of QubitRegister::CheckQubits (QubitRegister.h:677-690).
 */
#ifndef QCS_GPU_H
#define QCS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qcs_register* qcs_handle;

enum qcs_status {
	QCS_OK = 0,
	QCS_INVALID_ARGUMENT = 1, /* reference: std::invalid_argument from CheckQubits */
	QCS_OUT_OF_MEMORY = 2,
	QCS_CUDA_ERROR = 3,
	QCS_UNSUPPORTED = 4
};

enum qcs_precision { QCS_FP64 = 0, QCS_FP32 = 1 };

/* trait bits: QuantumGate::isDiagonal, isAntidiagonal, isSwapGate, IsISwapGate, IsISwapDagGate,
 * isControlled and isControlQubit(1) (SimpleGates.h:27-60) */
enum qcs_trait {
	QCS_TRAIT_DIAGONAL = 1,
	QCS_TRAIT_ANTIDIAGONAL = 2,
	QCS_TRAIT_SWAP = 4,
	QCS_TRAIT_ISWAP = 8,
	QCS_TRAIT_ISWAPDAG = 16,
	QCS_TRAIT_CONTROLLED = 32,
	QCS_TRAIT_CONTROLQ1 = 64
};

/* one gate application: ApplyGate(gate, q0, q1, q2) (QubitRegister.h:434) */
typedef struct qcs_gate {
	uint32_t k;        /* gate qubits: 1, 2 or 3 */
	uint32_t q0;       /* qubit */
	uint32_t q1;       /* controllingQubit1 (ignored when k == 1) */
	uint32_t q2;       /* controllingQubit2 (ignored when k < 3) */
	uint32_t traits;   /* qcs_trait bits */
	uint32_t reserved; /* must be 0 */
	double m[128];     /* 2^k x 2^k complex matrix, row-major interleaved */
} qcs_gate;

/* ---- lifetime (QubitRegister ctor QubitRegister.h:17-37, Clone :662-674) ---- */
/* allocates 2^n amplitudes on the current CUDA device, set to basis state 0 */
int qcs_create(uint32_t nqubits, int precision, qcs_handle* out);
int qcs_destroy(qcs_handle h);
/* copies state, saved state and qubit count into a new register (Clone, QubitRegister.h:662-674) */
int qcs_clone(qcs_handle h, qcs_handle* out);
/* orders this register's work on `cuda_stream` (a cudaStream_t; NULL = the engine's own stream) */
int qcs_set_stream(qcs_handle h, void* cuda_stream);
int qcs_synchronize(qcs_handle h);
const char* qcs_last_error(qcs_handle h);
const char* qcs_status_string(int status);
uint32_t qcs_nqubits(qcs_handle h);                 /* getNrQubits, QubitRegister.h:59 */
uint64_t qcs_nstates(qcs_handle h);                 /* getNrBasisStates, QubitRegister.h:60 */
int qcs_precision_of(qcs_handle h);
/* device pointer of the amplitude array (for callers that bring their own kernels) */
void* qcs_device_state(qcs_handle h);

/* ---- state setters (QubitRegister.h:74-122) ---- */
int qcs_set_basis(qcs_handle h, uint64_t state);     /* setToBasisState :74-80 (out of range: no-op) */
int qcs_set_qubit_state(qcs_handle h, uint64_t q);   /* setToQubitState :82-88 */
int qcs_set_cat(qcs_handle h);                       /* setToCatState :91-98 */
int qcs_set_equal(qcs_handle h);                     /* setToEqualSuperposition :106-109 */
int qcs_clear(qcs_handle h);                         /* Clear :119-122 */
int qcs_set_amplitude(qcs_handle h, uint64_t state, double re, double im); /* setRawAmplitude :112-117 */
int qcs_get_amplitude(qcs_handle h, uint64_t state, double* re_im);        /* getBasisStateAmplitude :62-66 (0 if out of range) */
/* whole vector, host complex<double>[2^n] (getRegisterStorage :507-510, setRegisterStorageFastNoNormalize :521-524) */
int qcs_get_state(qcs_handle h, double* host_out);
int qcs_set_state(qcs_handle h, const double* host_in);
int qcs_normalize(qcs_handle h);                     /* Normalize :124-130 */
int qcs_adjust_phase_normalize(qcs_handle h);        /* AdjustPhaseAndNormalize :133-167 */

/* ---- gates ---- */
/* ApplyGate (QubitRegister.h:434-486) with the trait dispatch of QubitRegisterCalculator.h:39-939 */
int qcs_apply_gate(qcs_handle h, const double* m, uint32_t k, uint32_t q0, uint32_t q1, uint32_t q2, uint32_t traits);
/* ApplyGates (QubitRegister.h:493-497): applies the list in order, with the same per-gate results;
 * consecutive gates may share one pass over the amplitudes (staged in shared memory) */
int qcs_apply_gates(qcs_handle h, const qcs_gate* gates, size_t count);
/* ApplyOperatorMatrix (QubitRegister.h:499-505): dense 2^n x 2^n operator, row-major interleaved */
int qcs_apply_operator_matrix(qcs_handle h, const double* m);
/* The work of SubAlgo::NQubitsQuantumGate (NQubitsQuantumGate.h:20-46) and
 * SubAlgo::NQubitsControlledQuantumGate (NQubitsControlledQuantumGate.h:20-60) without their 2^n x 2^n
 * extended matrix: a dense 2^k x 2^k operator m (row-major, interleaved; 1 <= k <= 10) on the target
 * qubits qubits[0..k-1] (matrix bit j = qubits[j]), applied to the amplitudes whose control qubits
 * (the set bits of ctrl_mask) are all one; the others are unchanged. */
int qcs_apply_operator_on_qubits(qcs_handle h, const double* m, uint32_t k, const uint32_t* qubits, uint64_t ctrl_mask);
/* ApplyOperatorMatrix (QubitRegister.h:499-505) of a diagonal operator: amplitude i *= d[i], d = the
 * 2^n diagonal entries (interleaved).  QCSim's SchrodingerSimulation applies its potential and kinetic
 * operators this way (Schrodinger.h:335-347). */
int qcs_apply_diagonal(qcs_handle h, const double* d);
/* SchrodingerSimulation::Execute (Schrodinger.h:32-45) after its Init (:291-315): `steps` times the
 * potential diagonal, the IQFT of the whole register (with the swaps), the kinetic diagonal and the
 * QFT.  potential_op and kinetic_op are the operators' 2^n diagonal entries (interleaved), sent to the
 * device once; the diagonals run inside the transforms' shared-memory passes. */
int qcs_schrodinger_evolve(qcs_handle h, const double* potential_op, const double* kinetic_op, uint64_t steps);
/* QuantumFourierTransform::QFT / IQFT on qubits [start, end] (QuantumFourierTransform.h:35-87) with
 * the mirror swaps of QubitsSwapper::Swap (QubitsSwapper.h:23-34) when do_swap != 0 */
int qcs_qft(qcs_handle h, uint32_t start, uint32_t end, int inverse, int do_swap);
/* OneQubitGateTransform (HadamardTransform.h:9-41): the same 1-qubit gate on every qubit in [start, end].
 * m is the gate's 2x2 matrix (row-major, interleaved) and traits its QCS_TRAIT_* bits.  start > end,
 * end >= n or a null m return QCS_INVALID_ARGUMENT and leave the register unchanged (the reference's
 * loop over an empty range does nothing; its callers clamp end to n - 1 first, QuantumAlgorithm.h:228-231). */
int qcs_one_qubit_transform(qcs_handle h, const double* m, uint32_t traits, uint32_t start, uint32_t end);

/* ---- measurement (QubitRegister.h:169-429, QubitRegisterCalculator.h:948-1254) ---- */
/* MeasureAll :169-195 — the first state whose running probability reaches prob (the last state if
 * none), then collapse to it */
int qcs_measure_all(qcs_handle h, double prob, uint64_t* state_out);
/* Measure(first, second) / MeasureQubit :198-224 — collapse and renormalise; returns the measured
 * sub-register value */
int qcs_measure(qcs_handle h, uint32_t first, uint32_t second, double prob, uint64_t* value_out);
/* MeasureNoCollapse() :619-642 — the first state whose running probability reaches prob (state 0 if none) */
int qcs_measure_no_collapse(qcs_handle h, double prob, uint64_t* state_out);
/* RepeatedMeasure :243-271 — for each prob, the lower_bound in the running-probability table that
 * stops at the first entry above 1 - epsilon; an index equal to the table size is possible, as in the
 * reference.  Results are full basis-state indices (callers mask sub-registers). */
int qcs_sample(qcs_handle h, const double* probs, size_t nshots, uint64_t* states_out);
/* GetQubitProbability :592-598 */
int qcs_qubit_probability(qcs_handle h, uint32_t qubit, double* p_out);
/* |a_i|^2 for all states into a host double[2^n] */
int qcs_probabilities(qcs_handle h, double* host_out);
/* stateFidelity :527-534 against a host complex<double>[2^n] vector: |<psi|v>|^2 */
int qcs_fidelity_host(qcs_handle h, const double* host_state, double* f_out);
/* <h|other> between two registers of the same size (the product inside stateFidelity / ExpectationValue) */
int qcs_inner(qcs_handle h, qcs_handle other, double* re_im_out);

/* two registers of the same size and any precisions: the normalised fidelity
 * |<h|other>|^2 / (|h|^2 |other|^2) and the largest |h_i - other_i|.  No reference counterpart: it
 * reports the FP32 path's accuracy against an FP64 run of the same circuit. */
int qcs_compare(qcs_handle h, qcs_handle other, double* fidelity_out, double* max_abs_diff_out);

/* ---- snapshots (SaveState / RestoreState / RestoreStateDestructive, QubitRegister.h:600-616) ---- */
int qcs_save_state(qcs_handle h);
int qcs_restore_state(qcs_handle h);                 /* no-op when nothing was saved */
int qcs_restore_state_destructive(qcs_handle h);
/* ExpectationValue (QubitRegister.h:646-660): <psi| G_n..G_1 |psi> for a gate list, state unchanged */
int qcs_expectation(qcs_handle h, const qcs_gate* gates, size_t count, double* re_im_out);

/* ---- batched QAOA (no reference counterpart as one call: the reference runs
 * QAOAIsingSubalgorithm::Exec (IsingModel.h:557-567) on one register at a time, and samples <H>
 * with RepeatedMeasure (IsingModel.h:569-578); here many instances of different sizes run in one
 * persistent launch captured in a CUDA graph, and <H> is the exact sum over basis states) ---- */
typedef struct qcs_qaoa_instance {
	uint32_t n;             /* qubits (spins) */
	uint32_t nedges;        /* couplings */
	const uint32_t* edges;  /* 2 * nedges qubit indices (i, j), i != j */
	const double* J;        /* nedges couplings (small integers) */
	const double* h;        /* n fields */
} qcs_qaoa_instance;
typedef struct qcs_qaoa_batch* qcs_qaoa_batch_handle;
/* allocates every instance's statevector (2^n amplitudes each) in one device buffer */
int qcs_qaoa_batch_create(const qcs_qaoa_instance* instances, size_t count, uint32_t p, int precision, qcs_qaoa_batch_handle* out);
/* gammas and betas: count x p, row per instance */
int qcs_qaoa_batch_set_angles(qcs_qaoa_batch_handle b, const double* gammas, const double* betas);
/* CTAs per thread-block cluster sharing one instance (1, 2, 4, 8 or 16; 0 before the first call: 8) */
int qcs_qaoa_batch_set_cluster(qcs_qaoa_batch_handle b, int ctas);
/* tile shape of the mixer passes over the high qubits: runs of 2^low contiguous amplitudes times
 * `high` further qubits per pass (low >= 3, high >= 1, low + high <= 12; default 6 and 6) */
int qcs_qaoa_batch_set_tile(qcs_qaoa_batch_handle b, int low, int high);
/* runs every instance from |0..0>: H on all qubits, then p layers; energies_out (count doubles) gets
 * <H> = sum_x |psi_x|^2 E(x), E(x) = -(sum h_i s_i + sum J_ij s_i s_j) (IsingModel.h:106-119) */
int qcs_qaoa_batch_run(qcs_qaoa_batch_handle b, double* energies_out);
/* the final statevector of one instance, host complex<double>[2^n] */
int qcs_qaoa_batch_state(qcs_qaoa_batch_handle b, size_t index, double* host_state);
uint64_t qcs_qaoa_batch_amplitudes(qcs_qaoa_batch_handle b);
const char* qcs_qaoa_batch_last_error(qcs_qaoa_batch_handle b);
int qcs_qaoa_batch_destroy(qcs_qaoa_batch_handle b);

/* ---- one fused block (no reference counterpart): a dense 2^k x 2^k operator applied as one operation of a
 * shared-memory pass, the form the fused path gives its blocks (the learned cost model times blocks
 * through it) ----
 * m: 2^k x 2^k complex, row-major interleaved; matrix bit j is qubits[j] (any order, distinct);
 * k <= 5 (FP32 registers) or 4 (FP64 registers).  General dense operators (up to 10 qubits, with
 * controls) go through qcs_apply_operator_on_qubits. */
int qcs_apply_matrix(qcs_handle h, const uint32_t* qubits, uint32_t k, const double* m);

/* ---- learned cost model (no reference counterpart): a 3-layer MLP, F inputs -> 64 -> 64 -> 1 with
 * ReLU, FP32, trained and evaluated by the engine's own kernels.  It predicts the log of a fused
 * block's device time; a register in fusion mode 2 scores candidate partitions with it. ---- */
typedef struct qcs_mlp* qcs_mlp_handle;
int qcs_mlp_create(int inputs, uint64_t seed, qcs_mlp_handle* out);
int qcs_mlp_destroy(qcs_mlp_handle m);
int qcs_mlp_num_params(qcs_mlp_handle m);
/* parameters as W1[64][F], b1[64], W2[64][64], b2[64], W3[64], b3 */
int qcs_mlp_get_params(qcs_mlp_handle m, float* out);
int qcs_mlp_set_params(qcs_mlp_handle m, const float* in);
/* x: count x F row-major */
int qcs_mlp_predict(qcs_mlp_handle m, const float* x, int count, float* y_out);
/* gradient of mean((y - t)^2) over the batch, and that loss */
int qcs_mlp_gradient(qcs_mlp_handle m, const float* x, const float* t, int count, float* grad_out, float* loss_out);
/* `steps` full-batch Adam steps with learning rate lr; the loss after the last step */
int qcs_mlp_train(qcs_mlp_handle m, const float* x, const float* t, int count, int steps, float lr, float* loss_out);
/* the model's input vector for a block: register qubits, the block's qubits (ascending), gate count */
int qcs_block_features(uint32_t nqubits, const uint32_t* qubits, uint32_t k, uint32_t ngates, float* out);
/* the greedy fuser's partition of a gate list (host only, no GPU): per block its qubit mask and the
 * number of gates folded in; nblocks_out may exceed capacity (then only capacity entries are written) */
int qcs_fusion_plan(uint32_t nqubits, const qcs_gate* gates, size_t count, int max_qubits, uint64_t* block_masks,
                    uint32_t* block_gates, size_t capacity, size_t* nblocks_out);
/* the shared-memory passes the engine forms for that partition (host only, no GPU): tiles of
 * `tile_qubits` qubits, the tensor-core matrix budget applied when tensor_cores != 0; pass_of_block[i]
 * is block i's pass (blocks as numbered by qcs_fusion_plan, global-factor blocks get UINT32_MAX) */
int qcs_fusion_passes(uint32_t nqubits, const qcs_gate* gates, size_t count, int max_qubits, int tile_qubits, int tensor_cores,
                      uint32_t* pass_of_block, size_t capacity, size_t* nblocks_out, size_t* npasses_out);
/* the shared-memory passes qcs_apply_gates plans for an unfused gate list on a register of this size and
 * precision (host only, no GPU): per pass its number of operations and, of those, the TileFactor ones
 * (diagonal gates outside the pass's tile merged into one factor per tile).  A list that runs one kernel
 * per gate (fewer than tile + 2 qubits, or a single gate) reports no passes; npasses_out may exceed
 * capacity (then only capacity entries are written) */
int qcs_plan_gate_passes(uint32_t nqubits, int precision, const qcs_gate* gates, size_t count, uint32_t* pass_ops,
                         uint32_t* pass_factors, size_t capacity, size_t* npasses_out);
/* attach a trained model (kept by the caller) and the measured time of one pass per register size
 * (pass_ms[n], milliseconds; with len >= 128, pass_ms[64 + n] is that of a tensor-core pass); NULL detaches */
int qcs_set_cost_model(qcs_handle h, qcs_mlp_handle mlp, const double* pass_ms, size_t len);

/* ---- engine options ---- */
enum qcs_option {
	QCS_OPT_PASSES = 1,          /* 1 (default): gate lists run as shared-memory passes; 0: one kernel per gate */
	QCS_OPT_FUSION = 2,          /* gate lists fused into dense blocks: 0 off (FP64 default), 1 greedy (FP32
	                                default), 2 partition chosen by the learned cost model when one is loaded */
	QCS_OPT_FUSION_MAX_QUBITS = 3, /* largest fused block (1..5; FP64 registers use at most 4).  Default: 4 on FP32
	                                  registers of 26 or more qubits with the tensor cores on (4-qubit blocks on
	                                  tcgen05 beat 5-qubit ones and blocks of at most 3 on the CUDA cores there),
	                                  else 3; the learned partition chooses per gate list */
	QCS_OPT_TENSOR_CORES = 4       /* FP32 registers: 1 (default) fused blocks of 4 and 5 qubits run as 3xTF32
	                                  products on the tensor cores (tcgen05); 0: FP32 FMAs on the CUDA cores */
};
int qcs_set_option(qcs_handle h, int option, int value);

/* ---- launch timing (no reference counterpart: the reference has no profiler) ----
 * When enabled, every kernel the register launches is bracketed by CUDA events on its stream.
 * qcs_profile_read synchronises the stream, returns per kernel family the launch count, the summed
 * device milliseconds, the summed algorithmic bytes (2 x amplitude bytes x amplitudes the launch
 * must read and write) and the summed floating-point instructions of the launches' gate arithmetic
 * (FMA, multiply or add on an amplitude component: one each, in the register's precision; counted for
 * the shared-memory passes on the CUDA cores, 0 for the other families), and clears the records. */
typedef struct qcs_profile_entry {
	char name[48];
	uint64_t launches;
	double milliseconds;
	double bytes;
	double fp_ops;
} qcs_profile_entry;
int qcs_profile_enable(qcs_handle h, int enable);
int qcs_profile_read(qcs_handle h, qcs_profile_entry* out, int capacity, int* count_out);

/* ---- engine statistics ---- */
/* number of CUDA kernels this library has launched since it was loaded (all registers) */
uint64_t qcs_launch_count(void);
/* bytes of scratch the register has allocated for reductions and sampling so far: device memory
 * (reduction partials, chunk sums, shot buffers) and pinned host memory.  Scratch is allocated on
 * the register's first observation that needs it and kept until qcs_destroy. */
int qcs_scratch_bytes(qcs_handle h, uint64_t* device_bytes, uint64_t* pinned_bytes);

/* ---- host random stream: std::mt19937_64 + std::uniform_real_distribution<double>(0,1), the
 * generator and distribution of QubitRegister.h:723-724, for callers without a C++ runtime ---- */
typedef struct qcs_rng* qcs_rng_handle;
int qcs_rng_create(uint64_t seed, qcs_rng_handle* out);
int qcs_rng_destroy(qcs_rng_handle g);
/* n uniforms in [0, 1) */
int qcs_rng_uniform(qcs_rng_handle g, double* out, size_t n);

/* ---- qubit probability without device allocation ----
 * No counterpart in the reference.  This variant of qcs_qubit_probability gives the same value (to
 * rounding) but reduces through one fixed file-scope device array (256 KiB per GPU, resident while
 * the library is loaded) instead of scratch the register allocates, for callers that cannot let the
 * library allocate: a register that fills the GPU, device memory owned by the application's own
 * pool, or a loop that cannot take the device-wide wait of cudaFree.
 *  - registers of at most 32 qubits; larger ones return QCS_UNSUPPORTED with a message;
 *  - call with the register's device current; the first call on a device sets the array up
 *    (address lookup, kernel loading), so make it before any stream capture on that device;
 *  - every call uses the same array: calls that can overlap on the GPU (registers on different
 *    streams, several host threads) race and must be serialised by the caller;
 *  - nothing needs zeroing first;
 *  - synchronous: it returns once the value has reached the host (a one-double device-to-host copy
 *    and a synchronisation of the register's stream). */
int qcs_qubit_probability_noalloc(qcs_handle h, uint32_t qubit, double* p_out);

#ifdef __cplusplus
}
#endif

#endif /* QCS_GPU_H */
