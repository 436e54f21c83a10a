// QCSim's own statevector test suite run over the GPU drop-in register -- TEST INFRASTRUCTURE ONLY.
//
// Linked with QCSim's unmodified test sources (Tests.cpp, GatesTests.cpp, MeasurementsTests.cpp, ...,
// compiled with qcsim_gb300/cpp ahead of the QCSim directory on the include path, oracle/Makefile
// target `dropin`), so every QC::QubitRegister those tests create is the GPU-backed one.  main() calls
// the test functions in the order of QCSim's tests(0) chain (Tests.cpp:761-785) and prints one line per
// function: "@@ <name> <1|0> <seconds>".  SimulationTests is left out: its Schrodinger part needs FFTW,
// which is not installed (the Pauli-string simulation it also covers is checked through ref_driver.cpp
// on the drop-in instead).  The exit status is 0 only if every function returned true.
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "Tests.h"

// Tests.cpp's tests(option) refers to the non-statevector simulators' suites (MPS, Clifford, Pauli
// propagation, path integral, extended stabilizer) and to SimulationTests; none of them is linked here
// and main() never calls tests(), so these definitions only satisfy the linker.
static bool not_linked(const char* name)
{
	std::cout << name << ": not part of the statevector suite run on the drop-in" << std::endl;
	return false;
}
bool MPSSimulatorTests() { return not_linked("MPSSimulatorTests"); }
bool CliffordSimulatorTests() { return not_linked("CliffordSimulatorTests"); }
bool CliffordExpectationValuesTests() { return not_linked("CliffordExpectationValuesTests"); }
bool TestPauliPropagator() { return not_linked("TestPauliPropagator"); }
bool TestPathIntegral() { return not_linked("TestPathIntegral"); }
bool TestExtStabilizer() { return not_linked("TestExtStabilizer"); }
bool SimulationTests() { return not_linked("SimulationTests"); }

// defined in Tests.cpp without a declaration in Tests.h
bool basicTests();
bool ShorTests();
bool GroverTests();
bool SimonTests();
bool BernsteinVaziraniTests();
bool SuperdenseCodingTests();
bool QuantumCryptograpyTests();
bool CountingTests();

int main(int argc, char** argv)
{
	struct Entry { const char* name; bool (*fn)(); };
	const Entry chain[] = {
		{ "basicTests", basicTests }, { "quantumAdderTests", quantumAdderTests }, { "DeutschJozsaTests", DeutschJozsaTests },
		{ "SimonTests", SimonTests }, { "BernsteinVaziraniTests", BernsteinVaziraniTests }, { "GroverTests", GroverTests },
		{ "PhaseEstimationTests", PhaseEstimationTests }, { "ShorTests", ShorTests }, { "TeleportationTests", TeleportationTests },
		{ "SuperdenseCodingTests", SuperdenseCodingTests }, { "QuantumCryptograpyTests", QuantumCryptograpyTests },
		{ "ParadoxesTests", ParadoxesTests }, { "GamesTests", GamesTests }, { "distributedTests", distributedTests },
		{ "CountingTests", CountingTests }, { "QMLTests", QMLTests }, { "IsingTests", IsingTests }, { "VQETests", VQETests },
	};
	// optional arguments: names of the functions to run (default: the whole chain)
	bool ok = true;
	int ran = 0;
	for (const Entry& e : chain)
	{
		if (argc > 1)
		{
			bool wanted = false;
			for (int i = 1; i < argc; ++i) wanted = wanted || std::strcmp(argv[i], e.name) == 0;
			if (!wanted) continue;
		}
		const auto t0 = std::chrono::steady_clock::now();
		const bool r = e.fn();
		const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
		std::cout << "@@ " << e.name << " " << (r ? 1 : 0) << " " << s << std::endl;
		ok = ok && r;
		++ran;
	}
	return ok && ran > 0 ? EXIT_SUCCESS : EXIT_FAILURE;
}
