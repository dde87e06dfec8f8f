"""Parity checker for the GB300 engine: test infrastructure only (see oracle.py)."""
