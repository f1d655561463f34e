"""The oracle: a CPU restatement of splatter's per-frame splat pipeline (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import this package, as the
checker or as the timed CPU baseline.  The product (splatter_gb300) never imports it.

PARITY UNPINNED: the reference (Rust + wgpu) cannot be built or run here and has no tests or golden
vectors; see the header of oracle.cpp for the assumptions this restatement makes.
"""
from .oracle import *  # noqa: F401,F403
