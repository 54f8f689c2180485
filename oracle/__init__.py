"""CPU oracle for cutrialdive's trial-factoring hot path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
import this package.  The product (``cutrialdive_gb300``) never does.
"""
from .ctd_oracle import *  # noqa: F401,F403
