"""CPU checker for the CUDA kernels (test infrastructure only).

oracle.py is the numpy front end; build.py compiles the C restatement
(oracle/*.c) and, where the reference checkout exists, the reference's own
kernels through oracle/ref_shim.
"""
