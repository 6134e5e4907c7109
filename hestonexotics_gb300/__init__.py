"""GB300-native Monte Carlo engine for hexo's Heston exotic-option pricer.

The compute path is libhexo_mc.so (hand-written sm_103a CUDA behind a C ABI,
include/hexo_mc.h); this package is its Python face:

  engine      Engine / Params / Options / Config / Server: typed wrapper of the C ABI
  shard       path-range shards merged exactly across ranks (torch.distributed)
  paramsdb    the reference's HParams.db parameter store as a request source
  workloads   seeded synthetic workloads with the configurations' shapes
  build       in-tree build of libhexo_mc.so
"""
from .engine import (ASIAN, EUROPEAN, FP32, FP64, STEP_GRID, STEP_REFERENCE, Batch, Config, Engine, Options,
                     Params, Request, Server, finalize_limbs)
from ._lib import EngineUnavailable, HexoError

__all__ = ["ASIAN", "EUROPEAN", "FP32", "FP64", "STEP_GRID", "STEP_REFERENCE", "Batch", "Config", "Engine",
           "Options", "Params", "Request", "Server", "finalize_limbs", "EngineUnavailable", "HexoError"]
