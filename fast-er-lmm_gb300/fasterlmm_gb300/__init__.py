"""
fasterlmm_gb300: the FaST-ER-LMM batched LMM association scan (fastlmm-compat LOCO path) on one GB300.

Drop-in modules: ``fasterlmm_gb300.core`` mirrors ``fasterlmm.core``'s compat scan functions and
``fasterlmm_gb300.perms`` mirrors ``fasterlmm.perms.perm_threshold``; ``fasterlmm_gb300.post`` holds the post-scan
statistics (-log10 p, permutation thresholds).  All compute runs in the CUDA library built from ``csrc/`` for
sm_103a (``build()``); nothing falls back to the CPU.
"""

from ._build import build  # noqa: F401

__version__ = "1.0.0"
