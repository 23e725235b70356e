"""ORACLE — test infrastructure only (see oracle/brute.c)."""
