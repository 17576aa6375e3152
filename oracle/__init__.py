"""CPU oracle for the 3x3 block ILU(0)-PCG path: TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, as the checker. The product package (delfem2_gb300) never imports it.
"""
from .oracle import Oracle, build, port, reference, HAVE_REFERENCE_BUILD  # noqa: F401
