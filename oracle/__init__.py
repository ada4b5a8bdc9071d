"""CPU oracle of the VNEC mxv path — test infrastructure only (see oracle.py)."""
