"""Measurement scripts of the library (run from the repository root as
``python -m benchmarks.<name>``): GEMM throughput, (T), whole solves in both
precisions and formulations, and the complex branch.  They call the library
through its Python front end and are not part of the package."""
