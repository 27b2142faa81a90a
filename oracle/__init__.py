"""CPU oracle for the BioFVM step (test infrastructure, see oracle/oracle.py)."""
