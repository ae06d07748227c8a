"""CPU oracle (test infrastructure only; see marie_oracle.py)."""
