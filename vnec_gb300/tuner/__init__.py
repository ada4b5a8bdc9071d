"""Learned kernel selection: training data (``dataset``) and training (``train``).

The model itself — features, the MLP and its kernels — lives in the C ABI
library (``csrc/features.cu``, ``csrc/mlp.cu``, ``csrc/tuner.cpp``); these
modules generate its training data with the library's exhaustive autotuner
and train it with the library's own forward/backward/Adam kernels.
"""
