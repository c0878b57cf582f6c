"""CPU oracle for the K-SVD path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs may import this
package, as the checker.  The product library (``ksvd_gb300``) never imports it.
"""
from .oracle import *  # noqa: F401,F403
from . import adjoint  # noqa: F401
