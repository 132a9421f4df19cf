"""Oracle package: CPU restatement of the reference tiled-SVD path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package, and only as the parity reference
(or, for the reference arm of the benchmark, as the timed CPU restatement).
The product library never loads it.
"""
from .oracle import *  # noqa: F401,F403
