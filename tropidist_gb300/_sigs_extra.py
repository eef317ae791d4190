"""ctypes signatures of the sparse-DP, completion-table and batching entry points."""
SIGNATURES = {}
