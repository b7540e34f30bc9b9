"""CPU oracle for the TARA 2D path -- test infrastructure only (see oracle.py)."""
