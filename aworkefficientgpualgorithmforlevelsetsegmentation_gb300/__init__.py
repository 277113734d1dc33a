"""GB300-native sparse level-set segmentation (LSS).

A from-scratch sm_103a implementation of the work-efficient sparse level-set
solver of Roberts et al. (HPG 2010) behind a C ABI (include/lss.h, built into
_build/liblss.so by build.py).  `Segmenter` mirrors the reference's solver
object; `Batch` runs many volumes in one persistent launch; `phantoms` makes
the seeded synthetic workloads.
"""
from ._lib import LssError, library_path, load  # noqa: F401
from .segmenter import (ALPHA_CURVATURE, ALPHA_DATA, DATA_LITERAL, DATA_NORMALISED,  # noqa: F401
                        MODE_NS, MODE_REF, Batch, Segmenter, config, default_params)

__all__ = ["Segmenter", "Batch", "LssError", "MODE_REF", "MODE_NS", "ALPHA_CURVATURE",
           "ALPHA_DATA", "DATA_NORMALISED", "DATA_LITERAL", "config", "default_params", "load",
           "library_path"]
