#pragma once

// Drop-in replacement for QCSim's QubitRegister.h: the same class template, namespace, constructor
// arguments and public members (QCSim/QubitRegister.h:11-728), with the amplitudes on a GB300 GPU.
// Every member forwards to libqcs_gpu.so through the C ABI of qcs_gpu.h.
//
// Use: put this directory ahead of the QCSim sources on the include path and link libqcs_gpu.so.
// QCSim's gate classes (QuantumGate.h, SimpleGates.h), QubitRegisterCalculator.h and every algorithm
// header are used unchanged; QubitRegisterDebug.h from this directory replaces the reference one
// (it reads amplitudes through getRegisterStorage()).
//
// Semantics kept from the reference:
//  - gate dispatch on the gate's trait virtuals (isDiagonal, isControlled, ...), captured here and
//    passed with the raw matrix (QubitRegister.h:434-486);
//  - std::invalid_argument from CheckQubits with the reference's messages (QubitRegister.h:677-690);
//  - the random stream: std::mt19937_64 seeded from the clock plus `addseed`, and prob = 1 - U[0,1)
//    per measurement (QubitRegister.h:26-34, 171, 210, 267, 621, 707);
//  - silent no-ops for out-of-range setters and reads (QubitRegister.h:63, 69, 76, 84, 114, 514, 607).
// Differences: the state has one device copy (gates run in place), and getRegisterStorage() returns a
// host mirror that is refreshed when the device state changed (a 16 * 2^n byte copy).

#include <cassert>
#include <chrono>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "QubitRegisterCalculator.h"
#include "qcs_gpu.h"

namespace QC {

	namespace detail {
		inline void qcs_check(int status, qcs_handle h)
		{
			if (status == QCS_OK) return;
			const std::string msg = h ? qcs_last_error(h) : qcs_status_string(status);
			if (status == QCS_INVALID_ARGUMENT) throw std::invalid_argument(msg);
			if (status == QCS_OUT_OF_MEMORY) throw std::bad_alloc();
			throw std::runtime_error("libqcs_gpu: " + msg);
		}

		template<class MatrixClass> void to_row_major(const MatrixClass& m, double* out)
		{
			const size_t d = static_cast<size_t>(m.rows());
			for (size_t r = 0; r < d; ++r)
				for (size_t c = 0; c < d; ++c)
				{
					const std::complex<double> v = m(r, c);
					out[2 * (r * d + c)] = v.real();
					out[2 * (r * d + c) + 1] = v.imag();
				}
		}

		template<class GateClass> uint32_t traits_of(const GateClass& g)
		{
			uint32_t t = 0;
			if (g.isDiagonal()) t |= QCS_TRAIT_DIAGONAL;
			if (g.isAntidiagonal()) t |= QCS_TRAIT_ANTIDIAGONAL;
			if (g.isSwapGate()) t |= QCS_TRAIT_SWAP;
			if (g.IsISwapGate()) t |= QCS_TRAIT_ISWAP;
			if (g.IsISwapDagGate()) t |= QCS_TRAIT_ISWAPDAG;
			if (g.isControlled()) t |= QCS_TRAIT_CONTROLLED;
			if (g.isControlQubit(1)) t |= QCS_TRAIT_CONTROLQ1;
			return t;
		}
	}

	template<class VectorClass = Eigen::VectorXcd, class MatrixClass = Eigen::MatrixXcd> class QubitRegister : public QubitRegisterCalculator<VectorClass, MatrixClass>
	{
	public:
		using GateClass = Gates::QuantumGateWithOp<MatrixClass>;
		using BaseClass = QubitRegisterCalculator<VectorClass, MatrixClass>;

		QubitRegister(size_t N = 3, unsigned int addseed = 0)
			: NrQubits(N), NrBasisStates(1ULL << NrQubits), uniformZeroOne(0, 1), recordGates(false)
		{
			assert(N > 0);
			detail::qcs_check(qcs_create(static_cast<uint32_t>(N), QCS_FP64, &handle), nullptr);
			Seed(addseed);
		}

		// swaps the caller's vector in, as the reference's special constructor (QubitRegister.h:40-57)
		QubitRegister(size_t N, VectorClass& v, unsigned int addseed = 0)
			: QubitRegister(N, addseed)
		{
			if (static_cast<size_t>(v.size()) == NrBasisStates)
				detail::qcs_check(qcs_set_state(handle, reinterpret_cast<const double*>(v.data())), handle);
			VectorClass empty;
			v.swap(empty);
			dirty = true;
		}

		QubitRegister(const QubitRegister& other)
			: BaseClass(other), NrQubits(other.NrQubits), NrBasisStates(other.NrBasisStates), rng(other.rng),
			uniformZeroOne(0, 1), computeGates(other.computeGates), recordGates(other.recordGates)
		{
			detail::qcs_check(qcs_clone(other.handle, &handle), other.handle);
		}

		QubitRegister& operator=(const QubitRegister& other)
		{
			if (this == &other) return *this;
			qcs_handle c = nullptr;
			detail::qcs_check(qcs_clone(other.handle, &c), other.handle);
			if (handle) qcs_destroy(handle);
			handle = c;
			NrQubits = other.NrQubits;
			NrBasisStates = other.NrBasisStates;
			rng = other.rng;
			computeGates = other.computeGates;
			recordGates = other.recordGates;
			dirty = true;
			return *this;
		}

		~QubitRegister()
		{
			if (handle) qcs_destroy(handle);
		}

		size_t getNrQubits() const { return NrQubits; };
		size_t getNrBasisStates() const { return NrBasisStates; };

		std::complex<double> getBasisStateAmplitude(size_t State) const {
			if (State >= NrBasisStates) return 0;
			double v[2];
			detail::qcs_check(qcs_get_amplitude(handle, State, v), handle);
			return std::complex<double>(v[0], v[1]);
		}

		double getBasisStateProbability(size_t State) const {
			if (State >= NrBasisStates) return 0;
			return std::norm(getBasisStateAmplitude(State));
		}

		void setToBasisState(size_t State) { detail::qcs_check(qcs_set_basis(handle, State), handle); dirty = true; }
		void setToQubitState(size_t q) { detail::qcs_check(qcs_set_qubit_state(handle, q), handle); dirty = true; }
		void setToCatState() { detail::qcs_check(qcs_set_cat(handle), handle); dirty = true; }
		void Reset() { setToBasisState(0); }
		void setToEqualSuperposition() { detail::qcs_check(qcs_set_equal(handle), handle); dirty = true; }

		void setRawAmplitude(size_t State, std::complex<double> val)
		{
			if (State >= NrBasisStates) return;
			detail::qcs_check(qcs_set_amplitude(handle, State, val.real(), val.imag()), handle);
			dirty = true;
		}

		void Clear() { detail::qcs_check(qcs_clear(handle), handle); dirty = true; }
		void Normalize() { detail::qcs_check(qcs_normalize(handle), handle); dirty = true; }
		void AdjustPhaseAndNormalize() { detail::qcs_check(qcs_adjust_phase_normalize(handle), handle); dirty = true; }

		size_t MeasureAll()
		{
			const double prob = 1. - uniformZeroOne(rng);
			uint64_t state = 0;
			detail::qcs_check(qcs_measure_all(handle, prob, &state), handle);
			dirty = true;
			return static_cast<size_t>(state);
		}

		size_t MeasureQubit(size_t qubit) { return Measure(qubit, qubit); }

		size_t Measure(size_t firstQubit, size_t secondQubit)
		{
			const double prob = 1. - uniformZeroOne(rng);
			uint64_t v = 0;
			detail::qcs_check(qcs_measure(handle, static_cast<uint32_t>(firstQubit), static_cast<uint32_t>(secondQubit), prob, &v), handle);
			dirty = true;
			return static_cast<size_t>(v);
		}

		std::map<size_t, size_t> RepeatedMeasure(size_t nrTimes = 1000)
		{
			std::map<size_t, size_t> m;
			Histogram(nrTimes, 0, NrQubits - 1, false, m);
			return m;
		}

		std::unordered_map<size_t, size_t> RepeatedMeasureUnordered(size_t nrTimes = 1000)
		{
			std::unordered_map<size_t, size_t> m;
			Histogram(nrTimes, 0, NrQubits - 1, false, m);
			return m;
		}

		std::map<size_t, size_t> RepeatedMeasure(size_t firstQubit, size_t secondQubit, size_t nrTimes = 1000)
		{
			std::map<size_t, size_t> m;
			Histogram(nrTimes, firstQubit, secondQubit, true, m);
			return m;
		}

		std::unordered_map<size_t, size_t> RepeatedMeasureUnordered(size_t firstQubit, size_t secondQubit, size_t nrTimes = 1000)
		{
			std::unordered_map<size_t, size_t> m;
			Histogram(nrTimes, firstQubit, secondQubit, true, m);
			return m;
		}

		void ApplyGate(const GateClass& gate, size_t qubit, size_t controllingQubit1 = 0, size_t controllingQubit2 = 0)
		{
			const size_t gateQubits = gate.getQubitsNumber();
			CheckQubits(gate, qubit, controllingQubit1, controllingQubit2, gateQubits);
			assert(gateQubits > 0 && gateQubits <= 3);
			double m[128];
			detail::to_row_major(gate.getRawOperatorMatrix(), m);
			detail::qcs_check(qcs_apply_gate(handle, m, static_cast<uint32_t>(gateQubits), static_cast<uint32_t>(qubit),
				static_cast<uint32_t>(controllingQubit1), static_cast<uint32_t>(controllingQubit2), detail::traits_of(gate)), handle);
			dirty = true;
			if (recordGates)
				computeGates.emplace_back(Gates::AppliedGate<MatrixClass>(gate.getRawOperatorMatrix(), qubit, controllingQubit1, controllingQubit2));
		}

		void ApplyGate(const Gates::AppliedGate<MatrixClass>& gate)
		{
			ApplyGate(gate, gate.getQubit1(), gate.getQubit2(), gate.getQubit3());
		}

		// one engine call for the whole list: consecutive gates can share a pass over the amplitudes
		void ApplyGates(const std::vector<Gates::AppliedGate<MatrixClass>>& gates)
		{
			std::vector<qcs_gate> recs(gates.size());
			for (size_t i = 0; i < gates.size(); ++i)
			{
				const auto& g = gates[i];
				const size_t k = g.getQubitsNumber();
				CheckQubits(g, g.getQubit1(), g.getQubit2(), g.getQubit3(), k);
				std::memset(&recs[i], 0, sizeof(qcs_gate));
				recs[i].k = static_cast<uint32_t>(k);
				recs[i].q0 = static_cast<uint32_t>(g.getQubit1());
				recs[i].q1 = static_cast<uint32_t>(g.getQubit2());
				recs[i].q2 = static_cast<uint32_t>(g.getQubit3());
				recs[i].traits = detail::traits_of(g);
				detail::to_row_major(g.getRawOperatorMatrix(), recs[i].m);
			}
			detail::qcs_check(qcs_apply_gates(handle, recs.data(), recs.size()), handle);
			dirty = true;
			if (recordGates)
				for (const auto& g : gates) computeGates.emplace_back(g);
		}

		// a diagonal matrix (every non-zero entry on the diagonal, as the Grover oracle and the Schrodinger
		// operators are) runs as one multiply per amplitude (qcs_apply_diagonal)
		void ApplyOperatorMatrix(const MatrixClass& m)
		{
			const size_t rows = static_cast<size_t>(m.rows()), cols = static_cast<size_t>(m.cols());
			if (rows != NrBasisStates || cols != NrBasisStates) throw std::invalid_argument("The operator matrix does not match the register size");
			bool diagonal = true;
			for (size_t c = 0; c < cols && diagonal; ++c)
				for (size_t r = 0; r < rows; ++r)
					if (r != c && m(r, c) != std::complex<double>(0, 0))
					{
						diagonal = false;
						break;
					}
			if (diagonal)
			{
				std::vector<double> d(2 * rows);
				for (size_t i = 0; i < rows; ++i)
				{
					d[2 * i] = std::complex<double>(m(i, i)).real();
					d[2 * i + 1] = std::complex<double>(m(i, i)).imag();
				}
				detail::qcs_check(qcs_apply_diagonal(handle, d.data()), handle);
			}
			else
			{
				std::vector<double> rm(2 * rows * cols);
				detail::to_row_major(m, rm.data());
				detail::qcs_check(qcs_apply_operator_matrix(handle, rm.data()), handle);
			}
			dirty = true;
			if (recordGates)
				computeGates.emplace_back(Gates::AppliedGate<MatrixClass>(m));
		}

		// A dense 2^k x 2^k operator U on the target qubits (matrix bit j = qubits[j], k <= 10), applied
		// where every qubit of ctrlMask is one: the device path of the dense operator gates
		// (NQubitsQuantumGate.h, NQubitsControlledQuantumGate.h of this directory).  A recording register
		// applies and logs the 2^n x 2^n extended matrix instead, as the reference's gates do through
		// ApplyOperatorMatrix (NQubitsQuantumGate.h:20-25).
		void ApplyOperatorOnQubits(const MatrixClass& U, const std::vector<uint32_t>& qubits, uint64_t ctrlMask = 0)
		{
			if (recordGates)
			{
				ApplyOperatorMatrix(ExtendedOperator(NrQubits, U, qubits, ctrlMask));
				return;
			}
			std::vector<double> rm(2 * static_cast<size_t>(U.rows()) * static_cast<size_t>(U.cols()));
			detail::to_row_major(U, rm.data());
			detail::qcs_check(qcs_apply_operator_on_qubits(handle, rm.data(), static_cast<uint32_t>(qubits.size()), qubits.data(), ctrlMask),
			                  handle);
			dirty = true;
		}

		// the 2^n x 2^n matrix of ApplyOperatorOnQubits on an n-qubit register: U between states that agree
		// off the targets and have every control set, the identity where a control is clear
		static MatrixClass ExtendedOperator(size_t n, const MatrixClass& U, const std::vector<uint32_t>& qubits, uint64_t ctrlMask)
		{
			const size_t NrBasisStates = 1ULL << n;
			MatrixClass ext = MatrixClass::Zero(NrBasisStates, NrBasisStates);
			size_t tmask = 0;
			for (uint32_t q : qubits) tmask |= 1ULL << q;
			auto sub = [&](size_t i) {
				size_t r = 0;
				for (size_t j = 0; j < qubits.size(); ++j) r |= ((i >> qubits[j]) & 1ULL) << j;
				return r;
			};
			for (size_t i = 0; i < NrBasisStates; ++i)
			{
				if ((i & ctrlMask) != ctrlMask)
				{
					ext(i, i) = 1;
					continue;
				}
				for (size_t c = 0; c < static_cast<size_t>(U.cols()); ++c)
				{
					size_t j = i & ~tmask;
					for (size_t b = 0; b < qubits.size(); ++b)
						if ((c >> b) & 1ULL) j |= 1ULL << qubits[b];
					ext(i, j) = U(sub(i), c);
				}
			}
			return ext;
		}

		const VectorClass& getRegisterStorage() const
		{
			if (dirty || static_cast<size_t>(registerStorage.size()) != NrBasisStates)
			{
				registerStorage.resize(NrBasisStates);
				detail::qcs_check(qcs_get_state(handle, reinterpret_cast<double*>(registerStorage.data())), handle);
				dirty = false;
			}
			return registerStorage;
		}

		void setRegisterStorage(const VectorClass& vals)
		{
			if (static_cast<size_t>(vals.size()) != NrBasisStates) return;
			detail::qcs_check(qcs_set_state(handle, reinterpret_cast<const double*>(vals.data())), handle);
			Normalize();
		}

		// swaps the caller's vector with the register's (QubitRegister.h:521-524)
		void setRegisterStorageFastNoNormalize(VectorClass& vals)
		{
			VectorClass old = getRegisterStorage();
			detail::qcs_check(qcs_set_state(handle, reinterpret_cast<const double*>(vals.data())), handle);
			vals.swap(old);
			dirty = true;
		}

		double stateFidelity(const VectorClass& state) const
		{
			if (static_cast<size_t>(state.size()) != NrBasisStates) return 0;
			double f = 0;
			detail::qcs_check(qcs_fidelity_host(handle, reinterpret_cast<const double*>(state.data()), &f), handle);
			return f;
		}

		void ComputeStart() { recordGates = true; computeGates.clear(); }
		void ComputeEnd() { recordGates = false; }
		void ComputeClear() { computeGates.clear(); }

		void Compute()
		{
			const bool recordSave = recordGates;
			recordGates = false;
			Replay(computeGates);
			recordGates = recordSave;
		}

		void Uncompute()
		{
			const bool recordSave = recordGates;
			recordGates = false;
			std::vector<Gates::AppliedGate<MatrixClass>> inv;
			for (auto it = computeGates.crbegin(); it != computeGates.crend(); ++it)
				inv.emplace_back(it->getRawOperatorMatrix().adjoint(), it->getQubit1(), it->getQubit2(), it->getQubit3());
			Replay(inv);
			recordGates = recordSave;
		}

		double GetQubitProbability(size_t qubit) const
		{
			double p = 0;
			detail::qcs_check(qcs_qubit_probability(handle, static_cast<uint32_t>(qubit), &p), handle);
			return p;
		}

		void SaveState() { detail::qcs_check(qcs_save_state(handle), handle); }
		void RestoreState() { detail::qcs_check(qcs_restore_state(handle), handle); dirty = true; }
		void RestoreStateDestructive() { detail::qcs_check(qcs_restore_state_destructive(handle), handle); dirty = true; }

		size_t MeasureNoCollapse()
		{
			const double prob = 1. - uniformZeroOne(rng);
			uint64_t s = 0;
			detail::qcs_check(qcs_measure_no_collapse(handle, prob, &s), handle);
			return static_cast<size_t>(s);
		}

		std::complex<double> ExpectationValue(const std::vector<Gates::AppliedGate<MatrixClass>>& gates)
		{
			if (gates.empty()) return 1.;
			std::vector<qcs_gate> recs(gates.size());
			for (size_t i = 0; i < gates.size(); ++i)
			{
				const auto& g = gates[i];
				std::memset(&recs[i], 0, sizeof(qcs_gate));
				recs[i].k = static_cast<uint32_t>(g.getQubitsNumber());
				recs[i].q0 = static_cast<uint32_t>(g.getQubit1());
				recs[i].q1 = static_cast<uint32_t>(g.getQubit2());
				recs[i].q2 = static_cast<uint32_t>(g.getQubit3());
				recs[i].traits = detail::traits_of(g);
				detail::to_row_major(g.getRawOperatorMatrix(), recs[i].m);
			}
			double v[2];
			detail::qcs_check(qcs_expectation(handle, recs.data(), recs.size(), v), handle);
			return std::complex<double>(v[0], v[1]);
		}

		std::unique_ptr<QubitRegister<VectorClass, MatrixClass>> Clone() const
		{
			auto qr = std::make_unique<QubitRegister<VectorClass, MatrixClass>>(1);
			qcs_destroy(qr->handle);
			qr->handle = nullptr;
			detail::qcs_check(qcs_clone(handle, &qr->handle), handle);
			qr->NrQubits = NrQubits;
			qr->NrBasisStates = NrBasisStates;
			qr->computeGates = computeGates;
			qr->recordGates = recordGates;
			qr->dirty = true;
			return qr;
		}

		// the engine handle, for callers that use the C ABI directly
		qcs_handle GetHandle() const { return handle; }

	protected:
		inline void CheckQubits(const GateClass& /*gate*/, size_t qubit, size_t controllingQubit1, size_t controllingQubit2, size_t gateQubits) const
		{
			if (NrQubits == 0) throw std::invalid_argument("Qubit number is zero");
			else if (NrQubits <= qubit) throw std::invalid_argument("Qubit number is too high");
			else if (gateQubits == 2) {
				if (NrQubits <= controllingQubit1) throw std::invalid_argument("Controlling qubit number is too high");
				else if (qubit == controllingQubit1) throw std::invalid_argument("Qubit and controlling qubit are the same");
			}
			else if (gateQubits == 3)
			{
				if (NrQubits <= controllingQubit1 || NrQubits <= controllingQubit2) throw std::invalid_argument("Controlling qubit number is too high");
				else if (qubit == controllingQubit1 || qubit == controllingQubit2 || controllingQubit1 == controllingQubit2) throw std::invalid_argument("Qubits must be different");
			}
		}

		size_t MeasureNoCollapse(size_t qubit) { return MeasureNoCollapse(qubit, qubit); }

		size_t MeasureNoCollapse(size_t firstQubit, size_t secondQubit)
		{
			const size_t s = MeasureNoCollapse();
			return (s & SubMask(firstQubit, secondQubit)) >> firstQubit;
		}

		static size_t SubMask(size_t firstQubit, size_t secondQubit)
		{
			return (1ULL << (secondQubit + 1)) - 1 - ((1ULL << firstQubit) - 1);
		}

		void Seed(unsigned int addseed)
		{
			if (addseed == 0)
			{
				std::random_device rdl;
				addseed = rdl();
			}
			const uint64_t timeSeed = std::chrono::high_resolution_clock::now().time_since_epoch().count() + addseed;
			std::seed_seq seed{ uint32_t(timeSeed & 0xffffffff), uint32_t(timeSeed >> 32) };
			rng.seed(seed);
		}

		template<class MapClass> void Histogram(size_t nrTimes, size_t firstQubit, size_t secondQubit, bool sub, MapClass& out)
		{
			if (nrTimes == 0) return;
			if (nrTimes == 1)
			{
				const size_t s = MeasureNoCollapse();
				++out[sub ? (s & SubMask(firstQubit, secondQubit)) >> firstQubit : s];
				return;
			}
			std::vector<double> probs(nrTimes);
			for (size_t i = 0; i < nrTimes; ++i) probs[i] = 1. - uniformZeroOne(rng);
			std::vector<uint64_t> states(nrTimes);
			detail::qcs_check(qcs_sample(handle, probs.data(), nrTimes, states.data()), handle);
			const size_t mask = SubMask(firstQubit, secondQubit);
			for (uint64_t s : states) ++out[sub ? (static_cast<size_t>(s) & mask) >> firstQubit : static_cast<size_t>(s)];
		}

		void Replay(const std::vector<Gates::AppliedGate<MatrixClass>>& gates)
		{
			std::vector<Gates::AppliedGate<MatrixClass>> run;
			for (const auto& g : gates)
			{
				if (g.getQubitsNumber() > 3)
				{
					if (!run.empty()) { ApplyGates(run); run.clear(); }
					ApplyOperatorMatrix(g.getRawOperatorMatrix());
				}
				else run.push_back(g);
			}
			if (!run.empty()) ApplyGates(run);
		}

		size_t NrQubits;
		size_t NrBasisStates;

		// host mirror of the device amplitudes (refreshed by getRegisterStorage when stale)
		mutable VectorClass registerStorage;
		mutable bool dirty = true;

		std::mt19937_64 rng;
		std::uniform_real_distribution<double> uniformZeroOne;

		std::vector<Gates::AppliedGate<MatrixClass>> computeGates;
		bool recordGates;

		qcs_handle handle = nullptr;
	};

}
