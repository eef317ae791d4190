"""GB300-native exact distance evaluators (dense and sparse Rank DP, completion tables).

The package mirrors the `cdist` evaluator API of tropidist for the Rank DP hot path:
`trellis` (host planning), `kernel` (plan executor on the GPU), `auto` (dense front end),
`sparse_dp` (weight-truncated sweep with a GPU table backend) and `search.Table`
(completion tables built and probed on the GPU).  Every evaluator runs through the
hand-written CUDA library `libtropigpu.so` (C-ABI, loaded with ctypes); there is no
CPU fallback.
"""
__version__ = "0.1.0"
