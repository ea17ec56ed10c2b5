"""CPU oracle for dtFFT's execute path -- test infrastructure only (see oracle.py)."""
