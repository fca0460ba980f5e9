"""CPU oracle of the SBM hot path (test infrastructure only; see sbm_oracle.h)."""
