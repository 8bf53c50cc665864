"""GB300-native (sm_103a) affine-gap score-only pairwise alignment.

A drop-in for rrahn/pairwise_aligner's affine global/local score DP: the same
``cfg`` rule names (``cfg.configure_aligner``, ``cfg.method_global``,
``cfg.method_local``, ``cfg.gap_model_affine``, ``cfg.score_model_unitary*``)
and ``compute(...)`` results with ``score()``, computed by hand-written CUDA
kernels through the C ABI of include/pairwise_aligner_gb300.h.
"""
from . import cfg, seqio
from .aligner import ALIGNMENT_DTYPE, Aligner, AlignerResult, AlignmentResult, Context, RESULT_DTYPE, cigar, pack
from ._lib import PaError

__all__ = ["cfg", "seqio", "Aligner", "AlignerResult", "AlignmentResult", "Context", "RESULT_DTYPE",
           "ALIGNMENT_DTYPE", "cigar", "pack", "PaError"]
__version__ = "0.1.0"
