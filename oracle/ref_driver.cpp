// Driver around QCSim's own statevector code — TEST INFRASTRUCTURE ONLY.
//
// Compiled (oracle/Makefile target `ref`) against QCSim's unmodified headers where they lie in the
// reference checkout, with oracle/eigen_shim standing in for Eigen.  It exposes a small C API over
// QC::QubitRegister so that tests/golden/make_golden.py can record the reference's own outputs
// (statevectors, measurement outcomes, probabilities) as fixtures.  Output goes to oracle/_ref/.
//
// Gates are built from the reference's own gate classes (QC::Gates::*), so their matrices and trait
// overrides, and QubitRegister::ApplyGate's dispatch, are the reference's.
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>

#include "QubitRegister.h"
#include "QuantumGate.h"
#include "QuantumFourierTransform.h"
#include "IsingModel.h"
#include "NQubitsQuantumGate.h"
#include "NQubitsControlledQuantumGate.h"
#include "PauliStringSimulation.h"
#include "Oracle.h"

// GroverAlgorithm.h asserts unitarity with the name of QCSim's test-suite helper; this is the driver's own version
bool checkUnitary(const Eigen::MatrixXcd& m) {
	const Eigen::MatrixXcd r = m.adjoint() * m;
	for (Eigen::Index i = 0; i < r.rows(); ++i)
		for (Eigen::Index j = 0; j < r.cols(); ++j)
			if (std::abs(r(i, j) - std::complex<double>(i == j ? 1. : 0., 0.)) > 1e-10) return false;
	return true;
}
#include "GroverAlgorithm.h"
#include "DraperAdder.h"
#include "PhaseEstimation.h"
#include "VQE.h"
#include "ShorAlgorithm.h"
#include "QuantumCountingAlgorithm.h"

#include "qcs_oracle.h"  // gate codes and the qo_gate record layout

namespace {

using Reg = QC::QubitRegister<>;
using Mat = Eigen::MatrixXcd;

// QubitRegister with a deterministic generator and access to the protected no-collapse measures
class SeededRegister : public Reg {
public:
	explicit SeededRegister(size_t n) : Reg(n, 1) {}
	void seed(uint64_t s) { rng.seed(s); }
	size_t NoCollapseSub(size_t a, size_t b) { return MeasureNoCollapse(a, b); }
	std::string err;
};

// QAOA sub-algorithm with its protected circuit builder exposed
class QaoaProbe : public Models::QAOAIsingSubalgorithm<> {
public:
	void Run(Reg& r, const std::vector<double>& g, const std::vector<double>& b) { Exec(r, g, b); }
};

std::shared_ptr<QC::Gates::QuantumGateWithOp<>> make_ref_gate(const qo_gate& g) {
	using namespace QC::Gates;
	const double th = g.p[0], ph = g.p[1], la = g.p[2], ga = g.p[3];
	switch (g.code) {
	case QO_H: return std::make_shared<HadamardGate<>>();
	case QO_HY: return std::make_shared<HyGate<>>();
	case QO_S: return std::make_shared<SGate<>>();
	case QO_SDG: return std::make_shared<SDGGate<>>();
	case QO_T: return std::make_shared<TGate<>>();
	case QO_TDG: return std::make_shared<TDGGate<>>();
	case QO_P: return std::make_shared<PhaseShiftGate<>>(th);
	case QO_X: return std::make_shared<PauliXGate<>>();
	case QO_Y: return std::make_shared<PauliYGate<>>();
	case QO_Z: return std::make_shared<PauliZGate<>>();
	case QO_SX: return std::make_shared<SquareRootNOTGate<>>();
	case QO_SXDG: return std::make_shared<SquareRootNOTDagGate<>>();
	case QO_SPLITTER: return std::make_shared<SplitterGate<>>();
	case QO_RX: return std::make_shared<RxGate<>>(th);
	case QO_RY: return std::make_shared<RyGate<>>(th);
	case QO_RZ: return std::make_shared<RzGate<>>(th);
	case QO_U: return std::make_shared<UGate<>>(th, ph, la, ga);
	case QO_SWAP: return std::make_shared<SwapGate<>>();
	case QO_ISWAP: return std::make_shared<iSwapGate<>>();
	case QO_ISWAPDG: return std::make_shared<iSwapDagGate<>>();
	case QO_DECREMENT: return std::make_shared<DecrementGate<>>();
	case QO_CX: return std::make_shared<CNOTGate<>>();
	case QO_CY: return std::make_shared<ControlledYGate<>>();
	case QO_CZ: return std::make_shared<ControlledZGate<>>();
	case QO_CH: return std::make_shared<ControlledHadamardGate<>>();
	case QO_CSX: return std::make_shared<ControlledSquareRootNOTGate<>>();
	case QO_CSXDG: return std::make_shared<ControlledSquareRootNOTDagGate<>>();
	case QO_CS: return std::make_shared<ControlledPhaseGate<>>();
	case QO_CP: return std::make_shared<ControlledPhaseShiftGate<>>(th);
	case QO_CU: return std::make_shared<ControlledUGate<>>(th, ph, la, ga);
	case QO_CRX: return std::make_shared<ControlledRxGate<>>(th);
	case QO_CRY: return std::make_shared<ControlledRyGate<>>(th);
	case QO_CRZ: return std::make_shared<ControlledRzGate<>>(th);
	case QO_CCX: return std::make_shared<ToffoliGate<>>();
	case QO_CSWAP: return std::make_shared<FredkinGate<>>();
	case QO_CCZ: return std::make_shared<CCZGate<>>();
	case QO_CUSTOM1: case QO_CUSTOM2: case QO_CUSTOM3: {
		const int k = g.code - QO_CUSTOM1 + 1;
		const int d = 1 << k;
		Mat m(d, d);
		for (int r = 0; r < d; ++r)
			for (int c = 0; c < d; ++c) m(r, c) = std::complex<double>(g.m[2 * (r * d + c)], g.m[2 * (r * d + c) + 1]);
		return std::make_shared<AppliedGate<>>(m, g.q0, g.q1, g.q2);
	}
	default: return nullptr;
	}
}

unsigned traits_of(const QC::Gates::QuantumGate<>& g) {
	unsigned t = 0;
	if (g.isDiagonal()) t |= QO_TR_DIAGONAL;
	if (g.isAntidiagonal()) t |= QO_TR_ANTIDIAGONAL;
	if (g.isSwapGate()) t |= QO_TR_SWAP;
	if (g.IsISwapGate()) t |= QO_TR_ISWAP;
	if (g.IsISwapDagGate()) t |= QO_TR_ISWAPDAG;
	if (g.isControlled()) t |= QO_TR_CONTROLLED;
	if (g.isControlQubit(1)) t |= QO_TR_CONTROLQ1;
	return t;
}

// the algorithms' protected ExecuteWithoutMeasurement exposed
class GroverProbe : public Grover::GroverAlgorithm<> {
public:
	using Grover::GroverAlgorithm<>::GroverAlgorithm;
	void Run() { ExecuteWithoutMeasurement(); }
};
template <class Adder> class AdderProbe : public Adder {
public:
	using Adder::Adder;
	void Run() { this->ExecuteWithoutMeasurement(); }
};
class ShorPhaseEstimationProbe : public QC::SubAlgo::ShorPhaseEstimation<> {
public:
	using QC::SubAlgo::ShorPhaseEstimation<>::ShorPhaseEstimation;
	void Run(Reg& r) { ExecuteWithoutMeasurement(r); }
};
class PhaseEstimationProbe : public QC::SubAlgo::PhaseEstimation<> {
public:
	using QC::SubAlgo::PhaseEstimation<>::PhaseEstimation;
	void Run(Reg& r) { ExecuteWithoutMeasurement(r); }
};

void to_vector(const double* in, Eigen::Index nb, Eigen::VectorXcd& v) {
	v.resize(nb);
	for (Eigen::Index i = 0; i < nb; ++i) v(i) = std::complex<double>(in[2 * i], in[2 * i + 1]);
}
void from_vector(const Eigen::VectorXcd& v, double* out) {
	for (Eigen::Index i = 0; i < v.size(); ++i) {
		out[2 * i] = v(i).real();
		out[2 * i + 1] = v(i).imag();
	}
}

// function objects for the gate-built oracles: a table of values over the oracle's input qubits
struct TableFunction {
	std::vector<size_t> values;
	size_t operator()(size_t state) const { return values[state]; }
};
struct BoolTableFunction {
	std::vector<size_t> values;
	bool operator()(size_t state) const { return values[state] != 0; }
};

}  // namespace

extern "C" {

void* qr_create(uint32_t n, uint64_t seed) {
	auto* r = new SeededRegister(n);
	r->seed(seed);
	r->SetMultithreading(true);
	return r;
}
void qr_destroy(void* r) { delete static_cast<SeededRegister*>(r); }
void qr_seed(void* r, uint64_t s) { static_cast<SeededRegister*>(r)->seed(s); }
void qr_set_multithreading(void* r, int e) { static_cast<SeededRegister*>(r)->SetMultithreading(e != 0); }

int qr_gate_matrix(const qo_gate* g, double* m_out, uint32_t* k_out, uint32_t* traits_out) {
	auto gate = make_ref_gate(*g);
	if (!gate) return 1;
	const Mat& m = gate->getRawOperatorMatrix();
	const int d = static_cast<int>(m.rows());
	for (int r = 0; r < d; ++r)
		for (int c = 0; c < d; ++c) {
			m_out[2 * (r * d + c)] = m(r, c).real();
			m_out[2 * (r * d + c) + 1] = m(r, c).imag();
		}
	*k_out = static_cast<uint32_t>(gate->getQubitsNumber());
	*traits_out = traits_of(*gate);
	return 0;
}

int qr_apply(void* rp, const qo_gate* gates, size_t count) {
	auto* r = static_cast<SeededRegister*>(rp);
	for (size_t i = 0; i < count; ++i) {
		auto gate = make_ref_gate(gates[i]);
		if (!gate) { r->err = "Unknown gate code"; return 1; }
		try {
			r->ApplyGate(*gate, gates[i].q0, gates[i].q1, gates[i].q2);
		} catch (const std::invalid_argument& e) {
			r->err = e.what();
			return 1;
		}
	}
	return 0;
}
const char* qr_last_error(void* r) { return static_cast<SeededRegister*>(r)->err.c_str(); }

void qr_get_state(void* r, double* out) {
	const auto& v = static_cast<SeededRegister*>(r)->getRegisterStorage();
	for (Eigen::Index i = 0; i < v.size(); ++i) { out[2 * i] = v(i).real(); out[2 * i + 1] = v(i).imag(); }
}
void qr_set_state(void* r, const double* in) {
	auto* R = static_cast<SeededRegister*>(r);
	Eigen::VectorXcd v(static_cast<Eigen::Index>(R->getNrBasisStates()));
	for (Eigen::Index i = 0; i < v.size(); ++i) v(i) = std::complex<double>(in[2 * i], in[2 * i + 1]);
	R->setRegisterStorageFastNoNormalize(v);
}

uint64_t qr_measure_all(void* r) { return static_cast<SeededRegister*>(r)->MeasureAll(); }
uint64_t qr_measure(void* r, uint32_t a, uint32_t b) { return static_cast<SeededRegister*>(r)->Measure(a, b); }
uint64_t qr_measure_qubit(void* r, uint32_t q) { return static_cast<SeededRegister*>(r)->MeasureQubit(q); }
uint64_t qr_measure_no_collapse(void* r) { return static_cast<SeededRegister*>(r)->MeasureNoCollapse(); }
uint64_t qr_measure_no_collapse_sub(void* r, uint32_t a, uint32_t b) { return static_cast<SeededRegister*>(r)->NoCollapseSub(a, b); }

// RepeatedMeasure: histogram as parallel arrays (state, count); returns the number of entries
size_t qr_repeated_measure(void* r, size_t shots, uint64_t* states, uint64_t* counts) {
	const auto res = static_cast<SeededRegister*>(r)->RepeatedMeasure(shots);
	size_t i = 0;
	for (const auto& kv : res) { states[i] = kv.first; counts[i] = kv.second; ++i; }
	return i;
}
size_t qr_repeated_measure_sub(void* r, uint32_t a, uint32_t b, size_t shots, uint64_t* states, uint64_t* counts) {
	const auto res = static_cast<SeededRegister*>(r)->RepeatedMeasure(a, b, shots);
	size_t i = 0;
	for (const auto& kv : res) { states[i] = kv.first; counts[i] = kv.second; ++i; }
	return i;
}

double qr_qubit_probability(void* r, uint32_t q) { return static_cast<SeededRegister*>(r)->GetQubitProbability(q); }
void qr_normalize(void* r) { static_cast<SeededRegister*>(r)->Normalize(); }
void qr_adjust_phase_normalize(void* r) { static_cast<SeededRegister*>(r)->AdjustPhaseAndNormalize(); }
void qr_set_basis(void* r, uint64_t s) { static_cast<SeededRegister*>(r)->setToBasisState(s); }
void qr_set_equal(void* r) { static_cast<SeededRegister*>(r)->setToEqualSuperposition(); }
void qr_set_cat(void* r) { static_cast<SeededRegister*>(r)->setToCatState(); }
void qr_set_raw(void* r, uint64_t s, double re, double im) { static_cast<SeededRegister*>(r)->setRawAmplitude(s, {re, im}); }

double qr_fidelity(void* r, const double* other) {
	auto* R = static_cast<SeededRegister*>(r);
	Eigen::VectorXcd v(static_cast<Eigen::Index>(R->getNrBasisStates()));
	for (Eigen::Index i = 0; i < v.size(); ++i) v(i) = std::complex<double>(other[2 * i], other[2 * i + 1]);
	return R->stateFidelity(v);
}

// ExpectationValue of a list of matrix-only gates (QubitRegister.h:646-660)
void qr_expectation(void* r, const qo_gate* gates, size_t count, double* re, double* im) {
	std::vector<QC::Gates::AppliedGate<>> list;
	for (size_t i = 0; i < count; ++i) {
		auto g = make_ref_gate(gates[i]);
		list.emplace_back(g->getRawOperatorMatrix(), gates[i].q0, gates[i].q1, gates[i].q2);
	}
	const auto v = static_cast<SeededRegister*>(r)->ExpectationValue(list);
	*re = v.real();
	*im = v.imag();
}

// record gates, then replay (Compute) or undo (Uncompute) them (QubitRegister.h:536-590)
int qr_record_and_replay(void* rp, const qo_gate* gates, size_t count, int mode) {
	auto* r = static_cast<SeededRegister*>(rp);
	r->ComputeStart();
	if (qr_apply(rp, gates, count)) return 1;
	r->ComputeEnd();
	if (mode == 1) r->Compute();
	else if (mode == 2) r->Uncompute();
	return 0;
}

int qr_qft(void* rp, uint32_t n, uint32_t start, uint32_t end, int inverse, int do_swap) {
	auto* r = static_cast<SeededRegister*>(rp);
	QC::SubAlgo::QuantumFourierTransform<> qft(n, start, end);
	if (inverse) qft.IQFT(*r, do_swap != 0);
	else qft.QFT(*r, do_swap != 0);
	return 0;
}

// QAOA circuit (IsingModel.h:557-567) for one instance; edges as (i, j) pairs
int qr_qaoa_exec(void* rp, uint32_t n, uint32_t nedges, const uint32_t* edges, const double* J, const double* h,
                 uint32_t p, const double* gammas, const double* betas) {
	auto* r = static_cast<SeededRegister*>(rp);
	QaoaProbe q;
	std::vector<Models::IsingModel::Interaction> ints;
	for (uint32_t e = 0; e < nedges; ++e) ints.push_back({edges[2 * e], edges[2 * e + 1], J[e]});
	std::vector<double> hv(h, h + n);
	q.Set(ints, hv);
	std::vector<double> g(gammas, gammas + p), b(betas, betas + p);
	q.Run(*r, g, b);
	return 0;
}

double qr_ising_energy(uint32_t n, uint32_t nedges, const uint32_t* edges, const double* J, const double* h, uint64_t state) {
	QaoaProbe q;
	std::vector<Models::IsingModel::Interaction> ints;
	for (uint32_t e = 0; e < nedges; ++e) ints.push_back({edges[2 * e], edges[2 * e + 1], J[e]});
	std::vector<double> hv(h, h + n);
	q.Set(ints, hv);
	return q.Energy(state);
}

// SubAlgo::NQubitsQuantumGate (ctrl < 0) or NQubitsControlledQuantumGate (controlling qubit ctrl) of the
// 2^k x 2^k operator op (row-major interleaved) at startQubit on an n-qubit register: its extended
// matrix (getOperatorMatrix, row-major interleaved into ext_out) and, when r is given, Execute on r
// (QubitRegister::ApplyOperatorMatrix of that matrix)
int qr_nqubits_gate(void* r, uint32_t n, const double* op, uint32_t k, uint32_t start, int ctrl, double* ext_out) {
	const Eigen::Index D = Eigen::Index(1) << k, NB = Eigen::Index(1) << n;
	Mat U(D, D);
	for (Eigen::Index i = 0; i < D; ++i)
		for (Eigen::Index j = 0; j < D; ++j) U(i, j) = std::complex<double>(op[2 * (i * D + j)], op[2 * (i * D + j) + 1]);
	Mat ext;
	if (ctrl < 0) {
		QC::SubAlgo::NQubitsQuantumGate<> g(n, U, start);
		ext = g.getOperatorMatrix();
		if (r) g.Execute(*static_cast<SeededRegister*>(r));
	} else {
		QC::SubAlgo::NQubitsControlledQuantumGate<> g(n, U, start, static_cast<size_t>(ctrl));
		ext = g.getOperatorMatrix();
		if (r) g.Execute(*static_cast<SeededRegister*>(r));
	}
	if (ext_out)
		for (Eigen::Index i = 0; i < NB; ++i)
			for (Eigen::Index j = 0; j < NB; ++j) {
				ext_out[2 * (i * NB + j)] = ext(i, j).real();
				ext_out[2 * (i * NB + j) + 1] = ext(i, j).imag();
			}
	return 0;
}

// QuantumSimulation::PauliDecomposedHamiltonianSimulation on n qubits from the state in (interleaved) with
// nterms Pauli strings (ops: nterms x n codes, 0 = Z, 1 = X, 2 = Y) and coefficients, simulation time t in
// steps Trotter steps; the state after Execute into out
int qr_pauli_simulation(uint32_t n, const double* in, uint32_t nterms, const uint8_t* ops, const double* coeffs, double t,
                        uint32_t steps, double* out) {
	using PauliOp = PauliString::PauliString::PauliOp;
	QuantumSimulation::PauliDecomposedHamiltonianSimulation<> sim(n, t, steps);
	const Eigen::Index NB = Eigen::Index(1) << n;
	Eigen::VectorXcd v(NB);
	for (Eigen::Index i = 0; i < NB; ++i) v(i) = std::complex<double>(in[2 * i], in[2 * i + 1]);
	sim.setRegisterStorage(v);
	for (uint32_t k = 0; k < nterms; ++k) {
		QuantumSimulation::PauliStringSimulation<> term(0., n);
		for (uint32_t q = 0; q < n; ++q) term.setOperatorForQubit(q, static_cast<PauliOp>(ops[k * n + q]));
		sim.AddTerm(coeffs[k], term);
	}
	sim.Execute();
	const Eigen::VectorXcd& s = sim.getRegisterStorage();
	for (Eigen::Index i = 0; i < NB; ++i) {
		out[2 * i] = s(i).real();
		out[2 * i + 1] = s(i).imag();
	}
	return 0;
}

// QC::Oracles::OracleWithGatesSimpleFunction (simple != 0; f(x) != 0 flips the target) or OracleWithGates (f(x) xored
// into the qubits from target up) over the input qubits [start, end] with ancillas from anc, f given as a table of
// 2^(end - start + 1) values; Execute on the n-qubit state inout (interleaved), in place
int qr_oracle_with_gates(uint32_t n, uint32_t start, uint32_t end, uint32_t target, uint32_t anc, int simple,
                         const uint64_t* table, double* inout) {
	SeededRegister reg(n);
	const Eigen::Index NB = Eigen::Index(1) << n;
	Eigen::VectorXcd v(NB);
	for (Eigen::Index i = 0; i < NB; ++i) v(i) = std::complex<double>(inout[2 * i], inout[2 * i + 1]);
	reg.setRegisterStorage(v);
	const size_t nv = size_t(1) << (end - start + 1);
	if (simple) {
		BoolTableFunction f{std::vector<size_t>(table, table + nv)};
		QC::Oracles::OracleWithGatesSimpleFunction<BoolTableFunction> oracle(n, start, end, target, anc);
		oracle.setFunction(f);
		oracle.Execute(reg);
	} else {
		TableFunction f{std::vector<size_t>(table, table + nv)};
		QC::Oracles::OracleWithGates<TableFunction> oracle(n, start, end, target, anc);
		oracle.setFunction(f);
		oracle.Execute(reg);
	}
	const Eigen::VectorXcd& s = reg.getRegisterStorage();
	for (Eigen::Index i = 0; i < NB; ++i) {
		inout[2 * i] = s(i).real();
		inout[2 * i + 1] = s(i).imag();
	}
	return 0;
}

// Grover::GroverAlgorithm on n qubits with the marked state: the state after ExecuteWithoutMeasurement into out
int qr_grover(uint32_t n, uint64_t marked, double* out) {
	GroverProbe g(n);
	g.setCorrectQuestionState(marked);
	g.Run();
	from_vector(g.getRegisterStorage(), out);
	return 0;
}

// Adders::DraperAdder (carry == 0, 2N qubits) or DraperAdderWithCarry (2N + 1 qubits) from the state in: the state
// after ExecuteWithoutMeasurement into out
int qr_draper(uint32_t N, int carry, const double* in, double* out) {
	Eigen::VectorXcd v;
	if (carry) {
		AdderProbe<Adders::DraperAdderWithCarry<>> a(N);
		to_vector(in, a.getNrBasisStates(), v);
		a.setRegisterStorage(v);
		a.Run();
		from_vector(a.getRegisterStorage(), out);
	} else {
		AdderProbe<Adders::DraperAdder<>> a(N);
		to_vector(in, a.getNrBasisStates(), v);
		a.setRegisterStorage(v);
		a.Run();
		from_vector(a.getRegisterStorage(), out);
	}
	return 0;
}

// QC::SubAlgo::PhaseEstimation of the 2^k x 2^k operator op (row-major interleaved) on an N-qubit register with L
// precision qubits, starting from the state in: the state after ExecuteWithoutMeasurement into out
int qr_phase_estimation(const double* op, uint32_t k, uint32_t N, uint32_t L, const double* in, double* out) {
	const Eigen::Index D = Eigen::Index(1) << k;
	Mat U(D, D);
	for (Eigen::Index i = 0; i < D; ++i)
		for (Eigen::Index j = 0; j < D; ++j) U(i, j) = std::complex<double>(op[2 * (i * D + j)], op[2 * (i * D + j) + 1]);
	PhaseEstimationProbe pe(U, N, L);
	SeededRegister reg(N);
	Eigen::VectorXcd v;
	to_vector(in, reg.getNrBasisStates(), v);
	reg.setRegisterStorage(v);
	pe.Run(reg);
	from_vector(reg.getRegisterStorage(), out);
	return 0;
}

// VQE::PauliStringVQE on n qubits with the operator codes ops (0 = Z, 1 = X, 2 = Y): from |0>, Ansatz with the
// parameters, then Execute (the rotation into the measured basis); the state into out
int qr_vqe_term(uint32_t n, const uint8_t* ops, uint32_t nparams, const double* params, double* out) {
	using PauliOp = PauliString::PauliString::PauliOp;
	VQE::PauliStringVQE<> term(static_cast<int>(n));
	for (uint32_t q = 0; q < n; ++q) term.setOperatorForQubit(q, static_cast<PauliOp>(ops[q]));
	SeededRegister reg(n);
	reg.setToBasisState(0);
	term.Ansatz(reg, std::vector<double>(params, params + nparams));
	term.Execute(reg);
	from_vector(reg.getRegisterStorage(), out);
	return 0;
}

// Shor's period finding: QC::SubAlgo::ShorPhaseEstimation of Shor::Fx (number C, base a) on N qubits with L x qubits;
// the state after ExecuteWithoutMeasurement into out
int qr_shor_period_finding(uint32_t C, uint32_t a, uint32_t N, uint32_t L, double* out) {
	Shor::Fx<> f(L, N - L, C);
	f.setParam(a);
	ShorPhaseEstimationProbe pe(f, N, L);
	SeededRegister reg(N);
	pe.Run(reg);
	from_vector(reg.getRegisterStorage(), out);
	return 0;
}

// QuantumCounting::QuantumCountingAlgorithm with P precision and G Grover qubits and the marked states: its
// (private) ExecuteWithoutMeasurement runs inside ExecuteWithMultipleMeasurements, whose sampling does not collapse,
// so the register then holds the pre-measurement state, copied into out
int qr_counting(uint32_t P, uint32_t G, uint32_t nmarked, const uint64_t* marked, double* out) {
	QuantumCounting::QuantumCountingAlgorithm<> qc(P, G);
	std::vector<size_t> m(marked, marked + nmarked);
	qc.SetMarkedStates(m);
	qc.ExecuteWithMultipleMeasurements(1);
	from_vector(qc.getRegisterStorage(), out);
	return 0;
}

// one draw of std::uniform_real_distribution<double>(0,1) on std::mt19937_64(seed), as the register uses it
void qr_uniforms(uint64_t seed, size_t n, double* out) {
	std::mt19937_64 g(seed);
	std::uniform_real_distribution<double> u(0, 1);
	for (size_t i = 0; i < n; ++i) out[i] = u(g);
}

}  // extern "C"
