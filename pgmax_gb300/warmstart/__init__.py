"""Learned warm start for loopy BP: a conv net predicts initial log-messages, plain BP finishes.

`potts` generates the spin-glass Potts family (toroidal grids, per-edge couplings) and its
wiring; `convnet` is the network (BF16 weights and activations, FP32 accumulation) on the
library's own CUDA kernels; `evaluate` runs warm and cold starts to a residual tolerance.
"""
