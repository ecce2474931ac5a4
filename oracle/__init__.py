"""ORACLE -- test infrastructure, not product code.

CPU restatements of the reference's permutation-inference path
(TFCE sweep, OLS/SE/t, Sobel z, per-permutation max, FWER lookup).  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this package; the product (``tfce_mediation_gb300``) never does.
"""
