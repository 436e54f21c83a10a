// Compile check of the C++ drop-in against the rest of QCSim's statevector algorithms: every header
// below is the reference's own, unmodified, and each algorithm's Execute (and its helpers) is
// instantiated over the GPU-backed QubitRegister of qcsim_gb300/cpp, so every register member the
// algorithms call has to exist with a compatible signature.  main() runs each one once on a GPU.
#include <cstdio>
#include <iostream>

#include "QubitRegister.h"
#include "QuantumGate.h"

bool checkUnitary(const Eigen::MatrixXcd& m)
{
	const Eigen::MatrixXcd r = m.adjoint() * m;
	for (Eigen::Index i = 0; i < r.rows(); ++i)
		for (Eigen::Index j = 0; j < r.cols(); ++j)
			if (std::abs(r(i, j) - std::complex<double>(i == j ? 1. : 0., 0.)) > 1e-10) return false;
	return true;
}

// ShorAlgorithm.h uses NControlledGatesWithAncilla without including its header (QCSim's test driver
// includes it earlier)
#include "NControlledGateWithAncilla.h"
#include "ShorAlgorithm.h"
#include "VQE.h"
#include "ErrorCorrection3Qubits.h"
#include "ShorCode.h"
#include "BernsteinVazirani.h"
#include "DeutschJozsa.h"
#include "SimonAlgorithm.h"
#include "SuperdenseCoding.h"
#include "Teleportation.h"
#include "EntanglementSwapping.h"
#include "TeleportedCNOT.h"
#include "QuantumCountingAlgorithm.h"
#include "QuantumAdder.h"
#include "QMeansClustering2D.h"
#include "CheckCHSHInequality.h"
#include "QuantumCryptograpy.h"

int main()
{
	Shor::ShorAlgorithm<> shor(15, 7, 3, 4);
	size_t p1 = 0, p2 = 0;
	const bool used = shor.factorize(p1, p2);
	std::cout << "shor " << used << " " << p1 << " " << p2 << "\n";

	VQE::VariationalQuantumEigensolver<> vqe(2);
	std::cout << "vqe " << vqe.Execute() << "\n";

	ErrorCorrection::ErrorCorrection3QubitsFlip<> flip;
	ErrorCorrection::ErrorCorrection3QubitsSign<> sign;
	ErrorCorrection::ShorCode<> shorCode;
	std::cout << "error correction " << flip.Execute() << " " << sign.Execute() << " " << shorCode.Execute() << "\n";

	BernsteinVazirani::BernsteinVaziraniAlgorithm<> bv(4);
	bv.setString(5);
	BernsteinVazirani::BernsteinVaziraniAlgorithmWithGatesOracle<> bvg(4);
	bvg.setString(5);
	std::cout << "bernstein-vazirani " << bv.Execute() << " " << bvg.Execute() << "\n";

	DeutschJozsa::DeutschJozsaAlgorithm<> dj(3);
	DeutschJozsa::DeutschJozsaAlgorithmWithGatesOracle<> djg(3);
	std::cout << "deutsch-jozsa " << dj.Execute() << " " << djg.Execute() << "\n";

	Simon::SimonAlgorithm<> simon(3);
	simon.setString(3);
	Simon::SimonAlgorithmWithGatesOracle<> simong(3);
	simong.setString(3);
	std::cout << "simon " << simon.Execute() << " " << simong.Execute() << "\n";

	Coding::SuperdenseCoding<> coding;
	Teleportation::QuantumTeleportationRealization<> teleport;
	Teleportation::EntanglementSwapping<> swapping;
	Distributed::TeleportedCNOT<> tcnot;
	std::cout << "coding/teleportation " << coding.Execute() << " " << teleport.Execute() << " " << swapping.Execute() << " "
	          << tcnot.Execute() << "\n";

	QuantumCounting::QuantumCountingAlgorithm<> counting(4, 3);
	std::cout << "counting " << counting.Execute() << "\n";

	Adders::NQubitsAdderAlgorithm<> adder(2);
	std::cout << "adder " << adder.Execute() << "\n";

	MachineLearning::QMeansClustering2D<> qmeans;
	BellInequalities::CheckCHSHInequality<> chsh;
	QuantumCryptograpy::BB84Protocol<> bb84;
	std::cout << "qmeans/chsh/bb84 " << qmeans.Execute() << " " << chsh.Execute() << " " << bb84.Execute() << "\n";
	return 0;
}
