#pragma once

// Drop-in replacement for QCSim's NQubitsControlledQuantumGate.h: QC::SubAlgo::NQubitsControlledQuantumGate
// with the same template, constructor and public members (QCSim/NQubitsControlledQuantumGate.h:9-97).
// Execute sends the 2^k x 2^k operator and the controlling qubit to the device
// (QubitRegister::ApplyOperatorOnQubits of this directory) instead of building the 2^n x 2^n extended
// matrix (NQubitsControlledQuantumGate.h:20-25); placement as in NQubitsQuantumGate.h of this directory.

#include <cstdint>
#include <vector>

#include "QuantumAlgorithm.h"

namespace QC {

	namespace SubAlgo {

		template<class VectorClass = Eigen::VectorXcd, class MatrixClass = Eigen::MatrixXcd> class NQubitsControlledQuantumGate : public QuantumSubAlgorithmOnSubregister<VectorClass, MatrixClass>
		{
		public:
			using BaseClass = QuantumSubAlgorithmOnSubregister<VectorClass, MatrixClass>;
			using RegisterClass = QubitRegister<VectorClass, MatrixClass>;

			NQubitsControlledQuantumGate(size_t N, const MatrixClass& op, size_t startQubit = 1, size_t controllingQubit = 0)
				: BaseClass(N, startQubit, startQubit + getOperatorQubitsNumber(op)), U(op), nrQubits(N), ctrlQubit(controllingQubit)
			{
			}

			size_t Execute(RegisterClass& reg) override
			{
				reg.ApplyOperatorOnQubits(U, targets(), 1ULL << ctrlQubit);
				return 0;  // no measurement
			}

			// the extended matrix on a 2^N register: U where the controlling qubit is one, the identity
			// where it is zero
			MatrixClass getOperatorMatrix() const
			{
				return RegisterClass::ExtendedOperator(nrQubits, U, targets(), 1ULL << ctrlQubit);
			}

			const MatrixClass& getRawOperatorMatrix() const { return U; }

			size_t getRawOperatorQubitsNumber() const { return getOperatorQubitsNumber(U); }

			size_t getNrQubits() const { return nrQubits; }

		protected:
			std::vector<uint32_t> targets() const
			{
				std::vector<uint32_t> q;
				for (size_t j = 0; j < getRawOperatorQubitsNumber(); ++j) q.push_back(static_cast<uint32_t>(BaseClass::getStartQubit() + j));
				return q;
			}

			// the bit length of rows - 1 (k for a 2^k x 2^k operator)
			static size_t getOperatorQubitsNumber(const MatrixClass& op)
			{
				size_t res = 0;
				for (size_t sz = static_cast<size_t>(op.rows() - 1); sz; sz >>= 1) ++res;
				return res;
			}

			MatrixClass U;
			size_t nrQubits;
			size_t ctrlQubit;
		};

	}

}
