"""CPU oracle for the reconstruction hot path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
import this package, and only to check results or to time the CPU baseline.
The product path (libfbp) never calls into it.

Modules:
  cpu      ctypes binding of the plain-C restatement (fbp_oracle.c, FP64)
  numpy_ref FP64 NumPy restatements of filter_H and the LCT pipeline
  harness  the reference's own CUDA kernels, compiled from its sources
"""
