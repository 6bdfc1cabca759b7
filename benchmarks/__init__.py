"""Measurement harnesses behind bench.py's sections (served stream, batched
solves, orbital optimisation, determinant lists, DOCI, single kernels). They
drive the library through its public API; only their CPU-baseline legs load the
oracle. Not part of the ciflow_gb300 package."""
