"""CPU oracle (test infrastructure): see oracle/qcs_oracle.h."""
