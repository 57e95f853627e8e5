"""ennemi_gb300 -- GB300 (sm_103a) nearest-neighbour estimators of mutual
information and entropy with ennemi's API.

Drop-in for ``ennemi``'s public functions.  The nearest-neighbour work (KSG
MI, Frenzel-Pompe conditional MI, Ross semidiscrete MI, Kozachenko-Leonenko
entropy) runs in hand-written CUDA kernels of ``libennemi_gb.so``, reached
through a ctypes C ABI (``include/ennemi_gb.h``); every call batches all of
its estimation tasks into one launch sequence on one GPU.  There is no CPU
fallback: without the library or a CUDA device the estimators raise.
"""

from ._driver import (estimate_corr, estimate_entropy, estimate_mi, normalize_mi,
                      pairwise_corr, pairwise_mi)
from ._build import build

__all__ = ["estimate_entropy", "estimate_mi", "estimate_corr",
           "pairwise_mi", "pairwise_corr", "normalize_mi", "build"]
__version__ = "0.1.0"
