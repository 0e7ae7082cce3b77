"""GB300-native batched candidate-evaluation engine for sampling-based system identification.

Drop-in for the replay-evaluation path of SPI-Active (scripts/eval.py): a batch of
parameter samples theta is evaluated against a batch of logged state windows in one
launch of hand-written sm_103a CUDA kernels behind a C ABI (include/spi_engine.h).
"""
from .robot import SimConfig, THETA_DIM, STATE_DIM, N_COMP, THETA_NAMES  # noqa: F401
from ._lib import SpiError  # noqa: F401

__all__ = ["SimConfig", "THETA_DIM", "STATE_DIM", "N_COMP", "THETA_NAMES", "SpiError"]
