#pragma once

// Drop-in replacement for QCSim's QubitRegisterDebug.h (QubitRegisterDebug.h:11-94): the same
// members, reading the amplitudes through getRegisterStorage() (the host mirror of the GPU state)
// instead of the reference's in-object vector.

#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>

#include "QubitRegister.h"

namespace QC {

	template<class VectorClass = Eigen::VectorXcd, class MatrixClass = Eigen::MatrixXcd> class QubitRegisterDebug : public QubitRegister<VectorClass, MatrixClass>
	{
	public:
		using BaseClass = QubitRegister<VectorClass, MatrixClass>;

		QubitRegisterDebug(size_t N = 3, unsigned int addseed = 0)
			: BaseClass(N, addseed)
		{
		}

		// one line per basis state: index, then |amplitude| or the complex amplitude
		bool writeToFile(const std::string& name, bool amplitude = true, bool append = false) const
		{
			try {
				std::ofstream thefile;
				thefile.open(name, std::ios::out | (append ? std::ios::app : std::ios::trunc));
				if (!thefile.is_open()) return false;
				if (append) thefile << std::endl << std::endl;
				const VectorClass& v = BaseClass::getRegisterStorage();
				for (size_t i = 0; i < BaseClass::getNrBasisStates(); ++i)
				{
					thefile << i << "\t";
					if (amplitude) thefile << std::abs(v(i));
					else thefile << v(i);
					thefile << std::endl;
				}
				return true;
			}
			catch (...) {};
			return false;
		}

		void displayState(size_t state) const
		{
			const size_t nQubits = BaseClass::getNrQubits();
			std::cout << "|";
			size_t mask = 1ULL << (nQubits - 1);
			for (size_t qubit = 0; qubit < nQubits; ++qubit)
			{
				std::cout << ((state & mask) ? "1" : "0");
				mask >>= 1;
			}
			std::cout << ">    ";
		}

		void displayRegister() const
		{
			const size_t nQubits = BaseClass::getNrQubits();
			const size_t nStates = BaseClass::getNrBasisStates();
			const VectorClass& v = BaseClass::getRegisterStorage();
			std::cout << std::setprecision(4);
			for (size_t state = 0; state < nStates; ++state)
			{
				const std::complex<double> val = v(state);
				if (std::abs(std::real(val)) < 1E-10 && std::abs(std::imag(val)) < 1E-10) continue;
				bool r = false;
				if (std::abs(std::real(val)) > 1E-10) {
					std::cout << std::real(val) << " ";
					r = true;
				}
				if (std::abs(std::imag(val)) > 1E-10) {
					if (r && std::imag(val) > 0) std::cout << "+ ";
					if (std::imag(val) < 0) {
						std::cout << "-";
						if (r) std::cout << " ";
					}
					std::cout << std::abs(std::imag(val)) << "i ";
				}
				displayState(nQubits);
			}
		}
	};

}
