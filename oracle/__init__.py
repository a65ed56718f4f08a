"""ORACLE — test infrastructure only.

CPU restatement of the reference prover's hot path (C, in this directory),
loaded through ctypes by tests/, the smoke check and bench.py's CPU-baseline
leg, where it is the checker. The product package never imports it.
"""
