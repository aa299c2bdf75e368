"""CPU oracle for the NRG hot path (test infrastructure only; see nrg_oracle.py)."""
