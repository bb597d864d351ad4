"""GB300-native neural-radiance-cache hot path.

The product is the C-ABI library libnrc.so (include/nrc.h, sources in csrc/):
record encoding, the fused MLP query, the fused training step and the Adam
update as sm_103a kernels. This package builds it in-tree (build.py), binds it
for Python callers (nrc.py) and generates the synthetic benchmark records
(synthetic.py).
"""
from .nrc import (P, TRAIN_BATCH_COUNT, TRAIN_BATCH_SIZE, WEIGHTS_TRAIN, WEIGHTS_USE, Cache, Config, NRCError,
                  default_config, he_init_host, lib)

__all__ = ["P", "TRAIN_BATCH_COUNT", "TRAIN_BATCH_SIZE", "WEIGHTS_TRAIN", "WEIGHTS_USE", "Cache", "Config",
           "NRCError", "default_config", "he_init_host", "lib"]
