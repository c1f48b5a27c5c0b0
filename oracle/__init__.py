"""Test infrastructure — the CPU oracle for psd_projection_gb300.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs import this package, and only as the checker.  Nothing in the library
(psd_projection_gb300/) depends on it.
"""
