"""GB300-native Universal Beta Splatting rasteriser: native library loader
and the batched / fused interfaces built on it."""
from . import build
from ._lib import call, last_error, lib, library_path

__all__ = ["build", "call", "last_error", "lib", "library_path"]
