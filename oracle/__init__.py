"""CPU oracle for the PEEC plane-current solve: test infrastructure only (see peec_oracle.py)."""
