"""CPU oracle for the apply_A hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import, link or run anything in this folder, and only as the checker.  The product (the CUDA
library in ``dg-sparsegrid_gb300/``) never routes through it.
"""
