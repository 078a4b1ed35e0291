"""GB300-native (sm_103a) implementation of OLCAO's per-SCF-iteration hot path.

The product is the C-ABI library ``libolcao_gb300.so`` (include/olcao_gpu.h);
``olcao_gb300.api`` is its Python front end and ``olcao_gb300.system`` builds
the seeded input sets.
"""

__all__ = ["api", "system", "build"]
