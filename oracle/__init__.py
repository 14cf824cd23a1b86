"""CPU oracle for the DMRG/TDVP inner loop of FiniteMPTools (numpy, float64/complex128).

TEST INFRASTRUCTURE ONLY.  This package is the checker: only the tests, the
smoke check in ``__graft_entry__`` and the CPU-baseline leg of ``bench.py``
may import it.  The product (``finitemptools_gb300``) never imports or calls
anything here, and it fails loudly instead of falling back to this code.

Every function restates the reference's own algorithm and cites the Julia
file:line it follows (paths relative to the FiniteMPTools project root).
Tensors keep the reference's index order; a numpy array ``x`` of shape
(D_l, d, D_r) is the Julia tensor ``x[a, s, b]`` and ``x.ravel(order='F')`` is
its column-major storage.

Pinning: the reference is Julia and cannot run here, and it ships no golden
vectors.  Its own tests pin DMRG and TDVP only against exact diagonalisation
and exact time evolution (test/runtests.jl:773-790); ``oracle.ed`` restates
those checks and ``tests/test_oracle_pins.py`` runs them.
"""

from .core import *  # noqa: F401,F403
from .algorithms import *  # noqa: F401,F403
