"""GB300-native PhyloCSF likelihood engine.

The compute path is the native library built from ``csrc/`` (CUDA for
sm_103a plus a C++ host runtime) behind the C-ABI in ``include/``; this
package is the host-side mirror of the reference's model interface.
"""
from .engine import (FIXED, MLE, MARGINALIZE, PREC, Batch, Engine, EngineError, Tree, candidate_regions,
                     load_library, make, pack_regions, read_ecm, score)

__all__ = ["FIXED", "MLE", "MARGINALIZE", "PREC", "Batch", "Engine", "EngineError", "Tree", "candidate_regions",
           "load_library", "make", "pack_regions", "read_ecm", "score"]
