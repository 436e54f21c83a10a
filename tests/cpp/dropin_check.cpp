// Compile check of the C++ drop-in (qcsim_gb300/cpp/QubitRegister.h): QCSim's own algorithm headers,
// unmodified, built against the GPU-backed QubitRegister.  main() runs a few of them when a GPU is
// present and prints a digest.
#include <cstdio>
#include <iostream>

#include "QubitRegister.h"
#include "QuantumGate.h"

// GroverAlgorithm.h asserts unitarity with the test-suite helper of the same name
bool checkUnitary(const Eigen::MatrixXcd& m)
{
	const Eigen::MatrixXcd r = m.adjoint() * m;
	for (Eigen::Index i = 0; i < r.rows(); ++i)
		for (Eigen::Index j = 0; j < r.cols(); ++j)
			if (std::abs(r(i, j) - std::complex<double>(i == j ? 1. : 0., 0.)) > 1e-10) return false;
	return true;
}

#include "QuantumFourierTransform.h"
#include "HadamardTransform.h"
#include "IsingModel.h"
#include "GroverAlgorithm.h"
#include "DraperAdder.h"
#include "PhaseEstimation.h"
#include "NQubitsQuantumGate.h"

int main()
{
	QC::QubitRegister<> reg(6, 7);
	QC::Gates::HadamardGate<> h;
	QC::Gates::CNOTGate<> cx;
	QC::Gates::RzGate<> rz(0.3);
	QC::Gates::ToffoliGate<> ccx;
	QC::Gates::FredkinGate<> cswap;
	reg.ApplyGate(h, 0);
	reg.ApplyGate(cx, 1, 0);
	reg.ApplyGate(rz, 2);
	reg.ApplyGate(ccx, 3, 0, 1);
	reg.ApplyGate(cswap, 4, 5, 0);
	try { reg.ApplyGate(cx, 1, 1); } catch (const std::invalid_argument& e) { std::cout << "caught: " << e.what() << "\n"; }
	QC::SubAlgo::QuantumFourierTransform<> qft(6);
	qft.QFT(reg);
	qft.IQFT(reg);
	QC::SubAlgo::OneQubitGateTransform<> ht(6, 0, 5);
	ht.Execute(reg);
	reg.ComputeStart();
	reg.ApplyGate(h, 2);
	reg.ComputeEnd();
	reg.Uncompute();
	const auto& v = reg.getRegisterStorage();
	auto hist = reg.RepeatedMeasure(100);
	std::cout << "p(q0)=" << reg.GetQubitProbability(0) << " |a0|=" << std::abs(v(0)) << " outcomes=" << hist.size()
	          << " measured=" << reg.MeasureAll() << "\n";
	auto clone = reg.Clone();
	std::cout << "clone states " << clone->getNrBasisStates() << "\n";

	Grover::GroverAlgorithm<> grover(4);
	grover.setCorrectQuestionState(5);
	std::cout << "grover " << grover.Execute() << "\n";

	Adders::DraperAdder<> adder(6);
	adder.setToBasisState(2 | (3 << 3));
	std::cout << "draper " << adder.Execute() << "\n";

	Models::QAOAIsingSubalgorithm<> qaoa;
	qaoa.Set({ { 0, 1, 1. }, { 1, 2, -1. } }, { 0.1, 0.2, 0.3 });
	qaoa.SetDeltaE(1.);
	std::cout << "qaoa energy(3) " << qaoa.Energy(3) << "\n";

	// phase estimation (its controlled powers of U run through NQubitsControlledQuantumGate.h of the
	// drop-in directory) and a dense operator gate on the top qubits
	QC::Gates::PhaseShiftGate<> ps(0.75 * 2. * std::acos(-1.));
	QC::SubAlgo::PhaseEstimation<> pe(ps.getRawOperatorMatrix(), 4, 3);
	QC::QubitRegister<> per(4);
	per.setToQubitState(3);
	std::cout << "phase estimation outcomes " << pe.ExecuteWithMultipleMeasurements(per, 1000).size() << "\n";
	QC::SubAlgo::NQubitsQuantumGate<> ng(6, Eigen::MatrixXcd::Identity(4, 4), 4);
	ng.Execute(reg);
	std::cout << "nqubits extended " << ng.getOperatorMatrix().rows() << "\n";
	return 0;
}
