"""GB300-native permutation-inference path of TFCE_mediation.

Drop-in modules for the reference's operator API (``tfce``, ``cynumstats``,
``pyfunc``, ``tm_func``) backed by hand-written sm_103a CUDA kernels through
the C-ABI in ``include/tfce_gb300.h``, plus a batched permutation engine
(``engine``).
"""
__version__ = "0.1.0"
