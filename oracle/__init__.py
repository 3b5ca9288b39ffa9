"""CPU oracle for the resident advection path (test infrastructure only).

Only tests, the smoke check and the CPU-baseline leg of the benchmark import
this package. The product path never does.
"""
