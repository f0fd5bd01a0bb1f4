"""CPU oracle (test infrastructure only; see toucan_oracle.h)."""
