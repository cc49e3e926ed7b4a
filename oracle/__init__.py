"""CPU oracle for the acoustic hot path - test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package, and only as the checker; the product path
(``wavefield_imaging_gb300``) never does.
"""
