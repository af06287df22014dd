"""CPU oracle of the hot path -- test infrastructure only (see phasta_oracle.h)."""
