"""ORACLE -- test infrastructure only (see oracle/fdtd_oracle.py)."""
