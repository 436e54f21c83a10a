// CPU oracle for the statevector hot path — TEST INFRASTRUCTURE ONLY (see qcs_oracle.h).
//
// Every routine below restates the behaviour of a QCSim routine, cited as file:line within the
// QCSim project.  The loops are written for clarity, with the reference's OpenMP split
// (parallel when multithreading is on and the register has at least 8192 basis states,
// QubitRegisterCalculator.h:1276-1278) so the same code doubles as the timed CPU baseline.
#include "qcs_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cd = std::complex<double>;
constexpr size_t kOmpLimit = 8192;  // QubitRegisterCalculator.h:1276

// ---------------------------------------------------------------------------------------------
// Gate matrices and traits (SimpleGates.h:582-919, QuantumGate.h:10-469)
// ---------------------------------------------------------------------------------------------
struct GateDef {
	unsigned k = 1;
	unsigned traits = 0;
	std::vector<cd> m;  // row-major dim x dim
	cd& at(unsigned r, unsigned c) { return m[r * (1u << k) + c]; }
	cd get(unsigned r, unsigned c) const { return m[r * (1u << k) + c]; }
};

GateDef zero_gate(unsigned k) {
	GateDef g;
	g.k = k;
	g.m.assign((1u << k) * (1u << k), cd(0, 0));
	return g;
}

GateDef identity_gate(unsigned k) {
	GateDef g = zero_gate(k);
	for (unsigned i = 0; i < (1u << k); ++i) g.at(i, i) = 1;
	return g;
}

bool make_gate(int code, const double* p, const double* custom, GateDef& g) {
	const double th = p ? p[0] : 0, ph = p ? p[1] : 0, la = p ? p[2] : 0, ga = p ? p[3] : 0;
	const double t2 = th * 0.5;
	const double r2 = 1. / std::sqrt(2.);
	const cd I(0, 1);
	switch (code) {
	// single qubit gates start as a zero 2x2 (SimpleGates.h:140-143)
	case QO_H: g = zero_gate(1); g.at(0, 0) = r2; g.at(0, 1) = r2; g.at(1, 0) = r2; g.at(1, 1) = -r2; break;       // :588-596
	case QO_HY: g = zero_gate(1); g.at(0, 0) = r2; g.at(0, 1) = cd(0, -r2); g.at(1, 0) = cd(0, r2); g.at(1, 1) = -r2; break;  // :608-616
	case QO_S: g = zero_gate(1); g.at(0, 0) = 1; g.at(1, 1) = I; g.traits = QO_TR_DIAGONAL; break;              // :626-635
	case QO_SDG: g = zero_gate(1); g.at(0, 0) = 1; g.at(1, 1) = -I; g.traits = QO_TR_DIAGONAL; break;           // :644-653
	case QO_T: g = zero_gate(1); g.at(0, 0) = 1; g.at(1, 1) = std::polar<double>(1, M_PI / 4.); g.traits = QO_TR_DIAGONAL; break;   // :663-672
	case QO_TDG: g = zero_gate(1); g.at(0, 0) = 1; g.at(1, 1) = std::polar<double>(1, -M_PI / 4.); g.traits = QO_TR_DIAGONAL; break; // :681-690
	case QO_P: g = zero_gate(1); g.at(0, 0) = 1; g.at(1, 1) = std::polar(1., th); g.traits = QO_TR_DIAGONAL; break;  // :699-713
	case QO_X: g = zero_gate(1); g.at(0, 1) = 1; g.at(1, 0) = 1; g.traits = QO_TR_ANTIDIAGONAL; break;           // :723-732
	case QO_Y: g = zero_gate(1); g.at(0, 1) = -I; g.at(1, 0) = I; g.traits = QO_TR_ANTIDIAGONAL; break;          // :741-750
	case QO_Z: g = zero_gate(1); g.at(0, 0) = 1; g.at(1, 1) = -1; g.traits = QO_TR_DIAGONAL; break;              // :760-769
	case QO_SX: g = zero_gate(1); g.at(0, 0) = cd(0.5, 0.5); g.at(0, 1) = cd(0.5, -0.5); g.at(1, 0) = g.at(0, 1); g.at(1, 1) = g.at(0, 0); break;   // :779-785
	case QO_SXDG: g = zero_gate(1); g.at(0, 0) = cd(0.5, -0.5); g.at(0, 1) = cd(0.5, 0.5); g.at(1, 0) = g.at(0, 1); g.at(1, 1) = g.at(0, 0); break; // :794-800
	case QO_SPLITTER: g = zero_gate(1); g.at(0, 0) = r2; g.at(0, 1) = cd(0, r2); g.at(1, 0) = g.at(0, 1); g.at(1, 1) = r2; break;             // :809-816
	case QO_RX: g = zero_gate(1); g.at(0, 0) = cd(std::cos(t2), 0); g.at(0, 1) = cd(0, -std::sin(t2)); g.at(1, 0) = g.at(0, 1); g.at(1, 1) = g.at(0, 0); break;  // :840-848
	case QO_RY: g = zero_gate(1); g.at(0, 0) = cd(std::cos(t2), 0); g.at(0, 1) = cd(-std::sin(t2), 0); g.at(1, 0) = cd(std::sin(t2), 0); g.at(1, 1) = g.at(0, 0); break; // :862-870
	case QO_RZ: g = zero_gate(1); g.at(0, 0) = std::polar(1., -t2); g.at(1, 1) = std::polar(1., t2); g.traits = QO_TR_DIAGONAL; break;     // :884-895
	case QO_U:  // :910-918
		g = zero_gate(1);
		g.at(0, 0) = std::polar(1., ga) * cd(std::cos(t2), 0.);
		g.at(0, 1) = -std::polar(1., ga + la) * std::sin(t2);
		g.at(1, 0) = std::polar(1., ga + ph) * std::sin(t2);
		g.at(1, 1) = std::polar(1., ga + ph + la) * std::cos(t2);
		break;
	// two qubit gates start as identity (SimpleGates.h:240-243)
	case QO_SWAP: g = identity_gate(2); g.at(1, 1) = 0; g.at(2, 2) = 0; g.at(1, 2) = 1; g.at(2, 1) = 1; g.traits = QO_TR_SWAP; break;        // QuantumGate.h:16-27
	case QO_ISWAP: g = identity_gate(2); g.at(1, 1) = 0; g.at(2, 2) = 0; g.at(1, 2) = I; g.at(2, 1) = I; g.traits = QO_TR_ISWAP; break;    // :36-47
	case QO_ISWAPDG: g = identity_gate(2); g.at(1, 1) = 0; g.at(2, 2) = 0; g.at(1, 2) = -I; g.at(2, 1) = -I; g.traits = QO_TR_ISWAPDAG; break; // :56-67
	case QO_DECREMENT:  // :76-88
		g = identity_gate(2);
		for (unsigned i = 0; i < 4; ++i) g.at(i, i) = 0;
		g.at(3, 0) = 1; g.at(0, 1) = 1; g.at(1, 2) = 1; g.at(2, 3) = 1;
		break;
	case QO_CX: g = identity_gate(2); g.at(2, 2) = 0; g.at(3, 3) = 0; g.at(2, 3) = 1; g.at(3, 2) = 1; g.traits = QO_TR_CONTROLLED | QO_TR_ANTIDIAGONAL; break;   // :124-146
	case QO_CY: g = identity_gate(2); g.at(2, 2) = 0; g.at(3, 3) = 0; g.at(2, 3) = -I; g.at(3, 2) = I; g.traits = QO_TR_CONTROLLED | QO_TR_ANTIDIAGONAL; break;  // :155-167
	case QO_CZ: g = identity_gate(2); g.at(3, 3) = -1; g.traits = QO_TR_CONTROLLED | QO_TR_DIAGONAL; break;   // :176-184
	case QO_CH: g = identity_gate(2); g.at(2, 2) = r2; g.at(2, 3) = r2; g.at(3, 2) = r2; g.at(3, 3) = -r2; g.traits = QO_TR_CONTROLLED; break;  // :193-200
	case QO_CSX: g = identity_gate(2); g.at(2, 2) = cd(0.5, 0.5); g.at(2, 3) = cd(0.5, -0.5); g.at(3, 2) = g.at(2, 3); g.at(3, 3) = g.at(2, 2); g.traits = QO_TR_CONTROLLED; break;   // :209-215
	case QO_CSXDG: g = identity_gate(2); g.at(2, 2) = cd(0.5, -0.5); g.at(2, 3) = cd(0.5, 0.5); g.at(3, 2) = g.at(2, 3); g.at(3, 3) = g.at(2, 2); g.traits = QO_TR_CONTROLLED; break; // :224-230
	case QO_CS: g = identity_gate(2); g.at(3, 3) = I; g.traits = QO_TR_CONTROLLED | QO_TR_DIAGONAL; break;   // :240-248
	case QO_CP: g = identity_gate(2); g.at(3, 3) = std::polar(1., th); g.traits = QO_TR_CONTROLLED | QO_TR_DIAGONAL; break;  // :257-270
	case QO_CU:  // :284-292
		g = identity_gate(2);
		g.at(2, 2) = std::polar(1., ga) * std::cos(t2);
		g.at(2, 3) = -std::polar(1., ga + la) * std::sin(t2);
		g.at(3, 2) = std::polar(1., ga + ph) * std::sin(t2);
		g.at(3, 3) = std::polar(1., ga + ph + la) * std::cos(t2);
		g.traits = QO_TR_CONTROLLED;
		break;
	case QO_CRX: g = identity_gate(2); g.at(2, 2) = cd(std::cos(t2), 0); g.at(2, 3) = cd(0, -std::sin(t2)); g.at(3, 2) = g.at(2, 3); g.at(3, 3) = g.at(2, 2); g.traits = QO_TR_CONTROLLED; break;  // :316-324
	case QO_CRY: g = identity_gate(2); g.at(2, 2) = cd(std::cos(t2), 0); g.at(2, 3) = cd(-std::sin(t2), 0); g.at(3, 2) = cd(std::sin(t2), 0); g.at(3, 3) = g.at(2, 2); g.traits = QO_TR_CONTROLLED; break; // :338-346
	case QO_CRZ: g = identity_gate(2); g.at(2, 2) = std::polar(1., -t2); g.at(3, 3) = std::polar(1., t2); g.traits = QO_TR_CONTROLLED | QO_TR_DIAGONAL; break;  // :360-371
	// three qubit gates start as identity (SimpleGates.h:341-344)
	case QO_CCX: g = identity_gate(3); g.at(6, 6) = 0; g.at(7, 7) = 0; g.at(6, 7) = 1; g.at(7, 6) = 1; g.traits = QO_TR_CONTROLLED | QO_TR_CONTROLQ1 | QO_TR_ANTIDIAGONAL; break;  // :408-425
	case QO_CSWAP: g = identity_gate(3); g.at(5, 5) = 0; g.at(6, 6) = 0; g.at(5, 6) = 1; g.at(6, 5) = 1; g.traits = QO_TR_CONTROLLED | QO_TR_SWAP; break;  // :435-446
	case QO_CCZ: g = identity_gate(3); g.at(7, 7) = -1; g.traits = QO_TR_CONTROLLED | QO_TR_CONTROLQ1 | QO_TR_DIAGONAL; break;  // :455-468
	case QO_CUSTOM1: case QO_CUSTOM2: case QO_CUSTOM3: {
		const unsigned k = static_cast<unsigned>(code - QO_CUSTOM1 + 1);
		g = zero_gate(k);
		const unsigned d = 1u << k;
		for (unsigned i = 0; i < d * d; ++i) g.m[i] = cd(custom[2 * i], custom[2 * i + 1]);
		g.traits = 0;  // AppliedGate overrides no trait (SimpleGates.h:439-578)
		break;
	}
	default:
		return false;
	}
	return true;
}

// ---------------------------------------------------------------------------------------------
// std::mt19937_64 and generate_canonical<double, 53> (the algorithms of the C++ standard)
// ---------------------------------------------------------------------------------------------
struct Mt64 {
	uint64_t mt[312];
	int idx = 312;
	explicit Mt64(uint64_t seed) {
		mt[0] = seed;
		for (int i = 1; i < 312; ++i) mt[i] = 6364136223846793005ULL * (mt[i - 1] ^ (mt[i - 1] >> 62)) + static_cast<uint64_t>(i);
	}
	uint64_t next() {
		if (idx >= 312) {
			for (int i = 0; i < 312; ++i) {
				const uint64_t y = (mt[i] & 0xFFFFFFFF80000000ULL) | (mt[(i + 1) % 312] & 0x7FFFFFFFULL);
				uint64_t v = mt[(i + 156) % 312] ^ (y >> 1);
				if (y & 1ULL) v ^= 0xB5026F5AA96619E9ULL;
				mt[i] = v;
			}
			idx = 0;
		}
		uint64_t z = mt[idx++];
		z ^= (z >> 29) & 0x5555555555555555ULL;
		z ^= (z << 17) & 0x71D67FFFEDA60000ULL;
		z ^= (z << 37) & 0xFFF7EEE000000000ULL;
		z ^= z >> 43;
		return z;
	}
	double uniform() {
		// one 64-bit draw covers 53 mantissa bits: sum / 2^64, clamped below 1
		const double r = static_cast<double>(next()) / 18446744073709551616.0;
		return r >= 1.0 ? std::nextafter(1.0, 0.0) : r;
	}
};

// probability of an amplitude as re*re + im*im, without contraction
inline double prob_of(const cd& a) {
	const volatile double x2 = a.real() * a.real();
	const volatile double y2 = a.imag() * a.imag();
	return x2 + y2;
}

// ---------------------------------------------------------------------------------------------
// Register
// ---------------------------------------------------------------------------------------------
struct Reg {
	unsigned n = 0;
	size_t N = 0;
	std::vector<cd> s;    // registerStorage
	std::vector<cd> res;  // resultsStorage
	bool mt = true;
	std::string err;

	bool par() const { return mt && N >= kOmpLimit; }
};

// ApplyOneQubitGate[Omp] (QubitRegisterCalculator.h:39-135)
void apply1(Reg& R, const GateDef& g, size_t qb, bool& swapStorage) {
	const size_t N = R.N;
	cd* s = R.s.data();
	cd* out = R.res.data();
	const long long NN = static_cast<long long>(N);
	if (g.traits & QO_TR_DIAGONAL) {
		swapStorage = false;
		const cd v0 = g.get(0, 0), v1 = g.get(1, 1);
#pragma omp parallel for if (R.par())
		for (long long st = 0; st < NN; ++st) s[st] *= (static_cast<size_t>(st) & qb) ? v1 : v0;
		return;
	}
	const size_t nq = ~qb;
	if (g.traits & QO_TR_ANTIDIAGONAL) {
		const cd v10 = g.get(1, 0), v01 = g.get(0, 1);
#pragma omp parallel for if (R.par())
		for (long long st = 0; st < NN; ++st) {
			const size_t u = static_cast<size_t>(st);
			out[u] = (u & qb) ? v10 * s[u & nq] : v01 * s[u | qb];
		}
		return;
	}
#pragma omp parallel for if (R.par())
	for (long long st = 0; st < NN; ++st) {
		const size_t u = static_cast<size_t>(st);
		const unsigned row = (u & qb) ? 1 : 0;
		out[u] = g.get(row, 0) * s[u & nq] + g.get(row, 1) * s[u | qb];
	}
}

// ApplyTwoQubitsGate[Omp] (QubitRegisterCalculator.h:137-177) and its helpers (:230-597)
void apply2(Reg& R, const GateDef& g, size_t qb, size_t cb, bool& swapStorage) {
	const size_t N = R.N;
	cd* s = R.s.data();
	cd* out = R.res.data();
	const long long NN = static_cast<long long>(N);
	const size_t both = qb | cb;
	if (g.traits & (QO_TR_SWAP | QO_TR_ISWAP | QO_TR_ISWAPDAG)) {
		// swap / iSwap / iSwap-dagger in place: exchange |q=0,c=1> with |q=1,c=0> (:230-355)
		swapStorage = false;
		const bool isw = (g.traits & QO_TR_SWAP) == 0;
		const cd f = (g.traits & QO_TR_SWAP) ? cd(1, 0) : ((g.traits & QO_TR_ISWAP) ? cd(0, 1) : cd(0, -1));
#pragma omp parallel for if (R.par())
		for (long long st = 0; st < NN; ++st) {
			const size_t u = static_cast<size_t>(st);
			if ((u & qb) != 0 || (u & cb) == 0) continue;
			const size_t o = u ^ both;
			std::swap(s[u], s[o]);
			if (isw) { s[u] *= f; s[o] *= f; }
		}
		return;
	}
	if (g.traits & QO_TR_CONTROLLED) {
		if (g.traits & QO_TR_DIAGONAL) {  // :357-371, in place on the control=1 half
			swapStorage = false;
			const cd v2 = g.get(2, 2), v3 = g.get(3, 3);
#pragma omp parallel for if (R.par())
			for (long long st = 0; st < NN; ++st) {
				const size_t u = static_cast<size_t>(st);
				if ((u & cb) == 0) continue;
				s[u] *= (u & qb) ? v3 : v2;
			}
			return;
		}
		const size_t nq = ~qb;
		if (g.traits & QO_TR_ANTIDIAGONAL) {  // :373-393
			const cd v32 = g.get(3, 2), v23 = g.get(2, 3);
#pragma omp parallel for if (R.par())
			for (long long st = 0; st < NN; ++st) {
				const size_t u = static_cast<size_t>(st);
				if ((u & cb) == 0) { out[u] = s[u]; continue; }
				out[u] = (u & qb) ? v32 * s[u & nq] : v23 * s[u | qb];
			}
			return;
		}
#pragma omp parallel for if (R.par())
		for (long long st = 0; st < NN; ++st) {  // :395-417
			const size_t u = static_cast<size_t>(st);
			if ((u & cb) == 0) { out[u] = s[u]; continue; }
			const unsigned row = 2u | ((u & qb) ? 1u : 0u);
			out[u] = g.get(row, 2) * s[(u & nq) | cb] + g.get(row, 3) * s[u | both];
		}
		return;
	}
	// dense 4x4 (:419-465); matrix row = (c ? 2 : 0) | (q ? 1 : 0)
	const size_t nq = ~qb, nc = ~cb;
#pragma omp parallel for if (R.par())
	for (long long st = 0; st < NN; ++st) {
		const size_t u = static_cast<size_t>(st);
		const unsigned row = ((u & cb) ? 2u : 0u) | ((u & qb) ? 1u : 0u);
		const size_t b = u & nq & nc;
		out[u] = g.get(row, 0) * s[b] + g.get(row, 1) * s[b | qb] + g.get(row, 2) * s[b | cb] + g.get(row, 3) * s[b | both];
	}
}

// ApplyThreeQubitsGate[Omp] (QubitRegisterCalculator.h:179-227) and helpers (:599-939)
void apply3(Reg& R, const GateDef& g, size_t qb, size_t qb2, size_t cb, bool& swapStorage) {
	const size_t N = R.N;
	cd* s = R.s.data();
	cd* out = R.res.data();
	const long long NN = static_cast<long long>(N);
	if (g.traits & QO_TR_SWAP) {
		// Fredkin: exchange |c=1,q2=1,q=0> with |c=1,q2=0,q=1> (:181-194)
		swapStorage = false;
		const size_t both = qb | qb2;
#pragma omp parallel for if (R.par())
		for (long long st = 0; st < NN; ++st) {
			const size_t u = static_cast<size_t>(st);
			if ((u & cb) == 0 || (u & qb2) == 0 || (u & qb) != 0) continue;
			std::swap(s[u], s[u ^ both]);
		}
		return;
	}
	if (g.traits & QO_TR_CONTROLLED) {
		if (g.traits & QO_TR_CONTROLQ1) {
			const size_t cc = cb | qb2;  // both controls
			if (g.traits & QO_TR_DIAGONAL) {  // :642-656
				swapStorage = false;
				const cd v6 = g.get(6, 6), v7 = g.get(7, 7);
#pragma omp parallel for if (R.par())
				for (long long st = 0; st < NN; ++st) {
					const size_t u = static_cast<size_t>(st);
					if ((u & cc) != cc) continue;
					s[u] *= (u & qb) ? v7 : v6;
				}
				return;
			}
			const size_t nq = ~qb;
			if (g.traits & QO_TR_ANTIDIAGONAL) {  // :658-680
				const cd v76 = g.get(7, 6), v67 = g.get(6, 7);
#pragma omp parallel for if (R.par())
				for (long long st = 0; st < NN; ++st) {
					const size_t u = static_cast<size_t>(st);
					if ((u & cc) != cc) { out[u] = s[u]; continue; }
					out[u] = (u & qb) ? v76 * s[u & nq] : v67 * s[u | qb];
				}
				return;
			}
#pragma omp parallel for if (R.par())
			for (long long st = 0; st < NN; ++st) {  // :682-707
				const size_t u = static_cast<size_t>(st);
				if ((u & cc) != cc) { out[u] = s[u]; continue; }
				const unsigned row = 6u | ((u & qb) ? 1u : 0u);
				out[u] = g.get(row, 6) * s[(u & nq) | cc] + g.get(row, 7) * s[u | cc | qb];
			}
			return;
		}
		// single control on controllingQubit2: the 4x4 block of rows/cols 4..7 (:610-638)
		const size_t nq = ~qb, nq2 = ~qb2;
#pragma omp parallel for if (R.par())
		for (long long st = 0; st < NN; ++st) {
			const size_t u = static_cast<size_t>(st);
			if ((u & cb) == 0) { out[u] = s[u]; continue; }
			const unsigned row = 4u | ((u & qb2) ? 2u : 0u) | ((u & qb) ? 1u : 0u);
			const size_t b = (u & nq & nq2) | cb;
			out[u] = g.get(row, 4) * s[b] + g.get(row, 5) * s[b | qb] + g.get(row, 6) * s[b | qb2] + g.get(row, 7) * s[b | qb | qb2];
		}
		return;
	}
	// dense 8x8 (:710-762); row = (c ? 4 : 0) | (q2 ? 2 : 0) | (q ? 1 : 0)
	const size_t clr = ~(qb | qb2 | cb);
#pragma omp parallel for if (R.par())
	for (long long st = 0; st < NN; ++st) {
		const size_t u = static_cast<size_t>(st);
		const unsigned row = ((u & cb) ? 4u : 0u) | ((u & qb2) ? 2u : 0u) | ((u & qb) ? 1u : 0u);
		const size_t b = u & clr;
		cd acc = g.get(row, 0) * s[b];
		acc += g.get(row, 1) * s[b | qb];
		acc += g.get(row, 2) * s[b | qb2];
		acc += g.get(row, 3) * s[b | qb | qb2];
		acc += g.get(row, 4) * s[b | cb];
		acc += g.get(row, 5) * s[b | cb | qb];
		acc += g.get(row, 6) * s[b | cb | qb2];
		acc += g.get(row, 7) * s[b | cb | qb | qb2];
		out[u] = acc;
	}
}

// QubitRegister::CheckQubits (QubitRegister.h:677-690)
bool check_qubits(Reg& R, unsigned k, size_t q, size_t c1, size_t c2) {
	const size_t n = R.n;
	if (n == 0) { R.err = "Qubit number is zero"; return false; }
	if (n <= q) { R.err = "Qubit number is too high"; return false; }
	if (k == 2) {
		if (n <= c1) { R.err = "Controlling qubit number is too high"; return false; }
		if (q == c1) { R.err = "Qubit and controlling qubit are the same"; return false; }
	} else if (k == 3) {
		if (n <= c1 || n <= c2) { R.err = "Controlling qubit number is too high"; return false; }
		if (q == c1 || q == c2 || c1 == c2) { R.err = "Qubits must be different"; return false; }
	}
	return true;
}

// QubitRegister::ApplyGate (QubitRegister.h:434-486)
bool apply_gate(Reg& R, const GateDef& g, size_t q, size_t c1, size_t c2) {
	if (!check_qubits(R, g.k, q, c1, c2)) return false;
	if (g.k < 1 || g.k > 3) { R.err = "Unsupported gate size"; return false; }
	bool swapStorage = true;
	const size_t qb = 1ULL << q;
	if (g.k == 1) apply1(R, g, qb, swapStorage);
	else if (g.k == 2) apply2(R, g, qb, 1ULL << c1, swapStorage);
	else apply3(R, g, qb, 1ULL << c1, 1ULL << c2, swapStorage);
	if (swapStorage) R.s.swap(R.res);
	return true;
}

// first index whose running sum of |a|^2 reaches prob; `fallback` when none does
// (the scans of QubitRegister.h:171-190, 621-639 and QubitRegisterCalculator.h:955-970)
size_t scan(const Reg& R, double prob, size_t fallback) {
	double acc = 0;
	for (size_t i = 0; i < R.N; ++i) {
		acc += prob_of(R.s[i]);
		if (prob <= acc) return i;
	}
	return fallback;
}

void set_basis(Reg& R, size_t st) {
	if (st >= R.N) return;
	std::fill(R.s.begin(), R.s.end(), cd(0, 0));
	R.s[st] = 1;
}

}  // namespace

extern "C" {

int qo_gate_matrix(int32_t code, const double* params, const double* custom, double* m_out, uint32_t* k_out, uint32_t* traits_out) {
	GateDef g;
	if (!make_gate(code, params, custom, g)) return 1;
	const unsigned d = 1u << g.k;
	for (unsigned i = 0; i < d * d; ++i) { m_out[2 * i] = g.m[i].real(); m_out[2 * i + 1] = g.m[i].imag(); }
	*k_out = g.k;
	*traits_out = g.traits;
	return 0;
}

void* qo_create(uint32_t nqubits) {
	Reg* R = new Reg;
	R->n = nqubits;
	R->N = 1ULL << nqubits;
	R->s.assign(R->N, cd(0, 0));
	R->res.assign(R->N, cd(0, 0));
	R->s[0] = 1;
	return R;
}

void qo_destroy(void* r) { delete static_cast<Reg*>(r); }
void qo_set_multithreading(void* r, int enable) { static_cast<Reg*>(r)->mt = enable != 0; }

void qo_set_threads(int nthreads) {
#ifdef _OPENMP
	omp_set_num_threads(nthreads);
#else
	(void)nthreads;
#endif
}

int qo_max_threads(void) {
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

int qo_apply(void* r, const qo_gate* gates, size_t count) {
	Reg& R = *static_cast<Reg*>(r);
	GateDef g;
	for (size_t i = 0; i < count; ++i) {
		if (!make_gate(gates[i].code, gates[i].p, gates[i].m, g)) { R.err = "Unknown gate code"; return 1; }
		if (gates[i].q0 < 0 || gates[i].q1 < 0 || gates[i].q2 < 0) { R.err = "Qubit number is too high"; return 1; }
		if (!apply_gate(R, g, static_cast<size_t>(gates[i].q0), static_cast<size_t>(gates[i].q1), static_cast<size_t>(gates[i].q2))) return 1;
	}
	return 0;
}

const char* qo_last_error(void* r) { return static_cast<Reg*>(r)->err.c_str(); }

void qo_get_state(void* r, double* out) {
	Reg& R = *static_cast<Reg*>(r);
	std::memcpy(out, R.s.data(), R.N * sizeof(cd));
}

void qo_set_state(void* r, const double* in) {
	Reg& R = *static_cast<Reg*>(r);
	std::memcpy(static_cast<void*>(R.s.data()), in, R.N * sizeof(cd));
}

uint64_t qo_nstates(void* r) { return static_cast<Reg*>(r)->N; }

// state setters (QubitRegister.h:74-122)
void qo_set_basis(void* r, uint64_t state) { set_basis(*static_cast<Reg*>(r), state); }
void qo_set_qubit_state(void* r, uint64_t q) {
	Reg& R = *static_cast<Reg*>(r);
	if (q >= R.n) return;
	set_basis(R, 1ULL << q);
}
void qo_set_cat(void* r) {
	Reg& R = *static_cast<Reg*>(r);
	std::fill(R.s.begin(), R.s.end(), cd(0, 0));
	const double v = 1. / std::sqrt(2.);
	R.s[0] = v;
	R.s[R.N - 1] = v;
}
void qo_set_equal(void* r) {
	Reg& R = *static_cast<Reg*>(r);
	std::fill(R.s.begin(), R.s.end(), cd(1. / std::sqrt(static_cast<double>(R.N)), 0));
}
void qo_clear(void* r) {
	Reg& R = *static_cast<Reg*>(r);
	std::fill(R.s.begin(), R.s.end(), cd(0, 0));
}
void qo_set_raw(void* r, uint64_t state, double re, double im) {
	Reg& R = *static_cast<Reg*>(r);
	if (state >= R.N) return;
	R.s[state] = cd(re, im);
}

// Normalize (QubitRegister.h:124-130)
void qo_normalize(void* r) {
	Reg& R = *static_cast<Reg*>(r);
	double ss = 0;
	for (const cd& a : R.s) ss += prob_of(a);
	const double nrm = std::sqrt(ss);
	if (nrm < 1E-20) return;
	const double f = 1. / nrm;
	for (cd& a : R.s) a *= f;
}

// AdjustPhaseAndNormalize (QubitRegister.h:133-167)
void qo_adjust_phase_normalize(void* r) {
	Reg& R = *static_cast<Reg*>(r);
	const size_t cand[3] = {0, R.N >> 1, R.N - 1};
	for (size_t c : cand) {
		const cd v0 = R.s[c];
		if (std::abs(v0) >= 1E-5) {
			for (cd& a : R.s) a /= v0;
			break;
		}
	}
	qo_normalize(r);
}

// MeasureAll (QubitRegister.h:169-195): fallback is the last basis state; collapse to it
uint64_t qo_measure_all(void* r, double prob) {
	Reg& R = *static_cast<Reg*>(r);
	const size_t st = scan(R, prob, R.N - 1);
	set_basis(R, st);
	return st;
}

// Measure / MeasureQubit (QubitRegister.h:198-224 -> QubitRegisterCalculator.h:948-1059, 1124-1225)
uint64_t qo_measure(void* r, uint32_t first, uint32_t second, double prob) {
	Reg& R = *static_cast<Reg*>(r);
	const size_t firstMask = (1ULL << first) - 1;
	const size_t mask = (1ULL << (second + 1)) - 1 - firstMask;
	const size_t picked = scan(R, prob, 0) & mask;
	double acc = 0;
	const long long NN = static_cast<long long>(R.N);
#pragma omp parallel for reduction(+ : acc) if (R.par())
	for (long long st = 0; st < NN; ++st)
		if ((static_cast<size_t>(st) & mask) == picked) acc += prob_of(R.s[st]);
	const double f = 1. / std::sqrt(acc);
	cd* s = R.s.data();
#pragma omp parallel for if (R.par())
	for (long long st = 0; st < NN; ++st) s[st] *= ((static_cast<size_t>(st) & mask) == picked) ? f : 0.;
	return picked >> first;
}

// MeasureNoCollapse() (QubitRegister.h:619-642): fallback is state 0
uint64_t qo_measure_no_collapse(void* r, double prob) { return scan(*static_cast<Reg*>(r), prob, 0); }

// MeasureNoCollapse(first, second) (QubitRegister.h:705-713 -> QubitRegisterCalculator.h:1061-1086, 1227-1254)
uint64_t qo_measure_no_collapse_sub(void* r, uint32_t first, uint32_t second, double prob) {
	Reg& R = *static_cast<Reg*>(r);
	const size_t firstMask = (1ULL << first) - 1;
	const size_t mask = (1ULL << (second + 1)) - 1 - firstMask;
	return (scan(R, prob, 0) & mask) >> first;
}

// RepeatedMeasure (QubitRegister.h:243-271): the running sum is kept up to the first entry above
// 1 - epsilon; each shot is the lower_bound of its probability in that truncated table.
void qo_sample(void* r, const double* probs, size_t nshots, uint64_t* out) {
	Reg& R = *static_cast<Reg*>(r);
	std::vector<double> cdf;
	cdf.reserve(R.N);
	double acc = 0;
	for (size_t i = 0; i < R.N; ++i) {
		acc += prob_of(R.s[i]);
		cdf.push_back(acc);
		if (acc > 1.0 - std::numeric_limits<double>::epsilon()) break;
	}
	for (size_t k = 0; k < nshots; ++k)
		out[k] = static_cast<uint64_t>(std::lower_bound(cdf.begin(), cdf.end(), probs[k]) - cdf.begin());
}

// GetQubitProbability[Omp] (QubitRegisterCalculator.h:1088-1122)
double qo_qubit_probability(void* r, uint32_t q) {
	Reg& R = *static_cast<Reg*>(r);
	const size_t qb = 1ULL << q;
	double acc = 0;
	const long long NN = static_cast<long long>(R.N);
#pragma omp parallel for reduction(+ : acc) if (R.par())
	for (long long st = 0; st < NN; ++st)
		if (static_cast<size_t>(st) & qb) acc += prob_of(R.s[st]);
	return acc;
}

// stateFidelity (QubitRegister.h:527-534): |<psi|other>|^2
double qo_fidelity(void* r, const double* other) {
	double re, im;
	qo_inner(r, other, &re, &im);
	return re * re + im * im;
}

void qo_inner(void* r, const double* other, double* re, double* im) {
	Reg& R = *static_cast<Reg*>(r);
	cd acc(0, 0);
	for (size_t i = 0; i < R.N; ++i) acc += std::conj(R.s[i]) * cd(other[2 * i], other[2 * i + 1]);
	*re = acc.real();
	*im = acc.imag();
}

// QuantumFourierTransform::QFT / IQFT (QuantumFourierTransform.h:35-87) with the mirror swaps of
// QubitsSwapper::Swap (QubitsSwapper.h:23-34)
int qo_qft(void* r, uint32_t start, uint32_t end, int inverse, int do_swap) {
	Reg& R = *static_cast<Reg*>(r);
	GateDef h, cp, sw;
	make_gate(QO_H, nullptr, nullptr, h);
	make_gate(QO_SWAP, nullptr, nullptr, sw);
	const int sq = static_cast<int>(start), eq = static_cast<int>(end);
	auto swaps = [&]() {
		size_t a = start, b = end;
		while (a < b) {
			if (!apply_gate(R, sw, a, b, 0)) return false;
			++a; --b;
		}
		return true;
	};
	auto set_cp = [&](double phase) { double p[4] = {phase, 0, 0, 0}; make_gate(QO_CP, p, nullptr, cp); };
	if (!inverse) {
		if (!apply_gate(R, h, eq, 0, 0)) return 1;
		for (int cur = eq; cur > sq; --cur) {
			double phase = M_PI_2;
			for (int c = cur - 1; c >= sq; --c) {
				set_cp(phase);
				if (!apply_gate(R, cp, cur, c, 0)) return 1;
				phase *= 0.5;
			}
			if (!apply_gate(R, h, cur - 1, 0, 0)) return 1;
		}
		if (do_swap && !swaps()) return 1;
	} else {
		if (do_swap && !swaps()) return 1;
		for (int cur = sq + 1; cur <= eq; ++cur) {
			if (!apply_gate(R, h, cur - 1, 0, 0)) return 1;
			double phase = -M_PI_2;
			for (int c = cur - 1; c >= sq; --c) {
				set_cp(phase);
				if (!apply_gate(R, cp, cur, c, 0)) return 1;
				phase *= 0.5;
			}
		}
		if (!apply_gate(R, h, eq, 0, 0)) return 1;
	}
	return 0;
}

// QAOAIsingSubalgorithm::Exec (IsingModel.h:557-567) with ApplyIsingOperator (:491-531) and
// ApplyMixingOperator (:533-554, plain mixing)
int qo_qaoa_exec(void* r, uint32_t nedges, const uint32_t* edges, const double* J, const double* h,
                 uint32_t p, const double* gammas, const double* betas) {
	Reg& R = *static_cast<Reg*>(r);
	GateDef H, cx, rz, rx;
	make_gate(QO_H, nullptr, nullptr, H);
	make_gate(QO_CX, nullptr, nullptr, cx);
	set_basis(R, 0);
	for (unsigned q = 0; q < R.n; ++q) if (!apply_gate(R, H, q, 0, 0)) return 1;
	for (uint32_t l = 0; l < p; ++l) {
		const double gamma = gammas[l];
		for (uint32_t e = 0; e < nedges; ++e) {
			const size_t q1 = edges[2 * e], q2 = edges[2 * e + 1];
			double prm[4] = {2 * gamma * J[e], 0, 0, 0};
			make_gate(QO_RZ, prm, nullptr, rz);
			if (!apply_gate(R, cx, q1, q2, 0)) return 1;
			if (!apply_gate(R, rz, q1, 0, 0)) return 1;
			if (!apply_gate(R, cx, q1, q2, 0)) return 1;
		}
		for (unsigned q = 0; q < R.n; ++q) {
			if (h[q] == 0.) continue;
			double prm[4] = {gamma * h[q], 0, 0, 0};
			make_gate(QO_RZ, prm, nullptr, rz);
			if (!apply_gate(R, rz, q, 0, 0)) return 1;
		}
		double prm[4] = {2 * betas[l], 0, 0, 0};
		make_gate(QO_RX, prm, nullptr, rx);
		for (unsigned q = 0; q < R.n; ++q) if (!apply_gate(R, rx, q, 0, 0)) return 1;
	}
	return 0;
}

// IsingModel::Energy(state) (IsingModel.h:106-119 with SetState :121-128 and GetTrueSpin :203-206):
// spin +1 for a 0 bit and -1 for a 1 bit, E = -(sum h_i s_i + sum J_ij s_i s_j)
double qo_ising_energy(uint32_t n, uint32_t nedges, const uint32_t* edges, const double* J, const double* h, uint64_t state) {
	double e = 0;
	for (uint32_t i = 0; i < n; ++i) e += h[i] * (((state >> i) & 1ULL) ? -1 : 1);
	for (uint32_t k = 0; k < nedges; ++k) {
		const int si = ((state >> edges[2 * k]) & 1ULL) ? -1 : 1;
		const int sj = ((state >> edges[2 * k + 1]) & 1ULL) ? -1 : 1;
		e += J[k] * si * sj;
	}
	return -e;
}

// exact <H> = sum_x |psi_x|^2 E(x) (the quantity EnergyExpectationValue, IsingModel.h:569-578, samples)
double qo_expected_energy(void* r, uint32_t nedges, const uint32_t* edges, const double* J, const double* h) {
	Reg& R = *static_cast<Reg*>(r);
	double acc = 0;
	const long long NN = static_cast<long long>(R.N);
#pragma omp parallel for reduction(+ : acc) if (R.par())
	for (long long x = 0; x < NN; ++x)
		acc += prob_of(R.s[x]) * qo_ising_energy(R.n, nedges, edges, J, h, static_cast<uint64_t>(x));
	return acc;
}

void* qo_rng_create(uint64_t seed) { return new Mt64(seed); }
void qo_rng_destroy(void* g) { delete static_cast<Mt64*>(g); }
uint64_t qo_rng_next(void* g) { return static_cast<Mt64*>(g)->next(); }
double qo_rng_uniform(void* g) { return static_cast<Mt64*>(g)->uniform(); }

void qo_random_normal_state(uint64_t seed, uint32_t n, double* out) {
	const uint64_t N = 1ULL << n;
	const uint64_t block = std::min<uint64_t>(N, 1ULL << 20);
	const long long nblocks = static_cast<long long>(N / block);
	double norm2 = 0;
#pragma omp parallel for reduction(+ : norm2) schedule(static)
	for (long long b = 0; b < nblocks; ++b) {
		std::mt19937_64 gen(seed * 1000003ULL + static_cast<uint64_t>(b));
		std::normal_distribution<double> g(0.0, 1.0);
		double acc = 0;
		double* o = out + 2 * static_cast<uint64_t>(b) * block;
		for (uint64_t i = 0; i < 2 * block; ++i) {
			o[i] = g(gen);
			acc += o[i] * o[i];
		}
		norm2 += acc;
	}
	const double inv = 1.0 / std::sqrt(norm2);
#pragma omp parallel for schedule(static)
	for (long long i = 0; i < static_cast<long long>(2 * N); ++i) out[i] *= inv;
}

double qo_max_abs_diff(const double* a, const double* b, uint64_t count) {
	double worst = 0;
#pragma omp parallel for reduction(max : worst) schedule(static)
	for (long long i = 0; i < static_cast<long long>(count); ++i) {
		const double dx = a[2 * i] - b[2 * i], dy = a[2 * i + 1] - b[2 * i + 1];
		worst = std::max(worst, std::sqrt(dx * dx + dy * dy));
	}
	return worst;
}

}  // extern "C"
