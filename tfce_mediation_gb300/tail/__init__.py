"""Learned null-tail surrogate for FWER p-values.

A small MLP (hand-written CUDA kernels: csrc/mlp.cu) maps summary statistics
of a few hundred permutation maxima to the generalised-Pareto tail of the
max-TFCE null, so tail p-values need far fewer permutations; vertices whose
surrogate p-value lies within a margin of alpha are sent back for more
permutations (the full permutation run stays the fallback and the yardstick).
"""
