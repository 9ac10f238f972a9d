"""GB300-native PairHMM (CUDA_LOGLESS) for GATK's read-likelihood step.

Modules:
  native    ctypes binding of libghmm.so (include/ghmm*.h)
  pairhmm   the PairHMM plugin mirror (CudaLoglessPairHMM) and the batched Engine
  workload  flat region workloads and the deterministic synthetic generator
  build     in-tree build of libghmm.so for sm_103a
"""
__all__ = ["native", "pairhmm", "workload", "build"]
