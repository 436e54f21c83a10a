#pragma once

// Drop-in replacement for QCSim's NQubitsQuantumGate.h: QC::SubAlgo::NQubitsQuantumGate with the same
// template, constructor and public members (QCSim/NQubitsQuantumGate.h:9-78).  Execute sends the
// 2^k x 2^k operator to the device (QubitRegister::ApplyOperatorOnQubits of this directory) instead
// of building the 2^n x 2^n extended matrix for ApplyOperatorMatrix (NQubitsQuantumGate.h:20-25).
//
// The operator acts on qubits startQubit .. startQubit + k - 1.  The reference's end qubit is
// startQubit + k clamped to N - 1 (QuantumAlgorithm.h:228-231), so its extended matrix stays within
// the operator's bounds only when the operator reaches the top qubit; there the two agree exactly.

#include <cstdint>
#include <vector>

#include "QuantumAlgorithm.h"

namespace QC {

	namespace SubAlgo {

		template<class VectorClass = Eigen::VectorXcd, class MatrixClass = Eigen::MatrixXcd> class NQubitsQuantumGate : public QuantumSubAlgorithmOnSubregister<VectorClass, MatrixClass>
		{
		public:
			using BaseClass = QuantumSubAlgorithmOnSubregister<VectorClass, MatrixClass>;
			using RegisterClass = QubitRegister<VectorClass, MatrixClass>;

			NQubitsQuantumGate(size_t N, const MatrixClass& op, size_t startQubit = 0)
				: BaseClass(N, startQubit, startQubit + getOperatorQubitsNumber(op)), U(op), nrQubits(N)
			{
			}

			size_t Execute(RegisterClass& reg) override
			{
				reg.ApplyOperatorOnQubits(U, targets(), 0);
				return 0;  // no measurement
			}

			// the extended matrix on a 2^N register: U on the operator's qubits, the identity elsewhere
			MatrixClass getOperatorMatrix() const
			{
				return RegisterClass::ExtendedOperator(nrQubits, U, targets(), 0);
			}

			const MatrixClass& getRawOperatorMatrix() const { return U; }

			size_t getRawOperatorQubitsNumber() const { return getOperatorQubitsNumber(U); }

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
		};

	}

}
