"""CPU oracle for the Mallard hot path (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this package.  The product package ``mallard_gb300`` never does.
"""

from .pyoracle import Oracle, OracleMesh, OracleCase, load  # noqa: F401
