"""CPU oracle for the GPU evaluators: TEST INFRASTRUCTURE ONLY.

Restatements of the reference's algorithms on the Rank DP hot path, used by tests/, by the
smoke check of __graft_entry__ and by bench.py's CPU baseline leg as the checker.  Nothing in
the tropidist_gb300 package imports this directory; the product path runs on the GPU only.

  dense.py        numpy executor of a trellis plan and its traceback  (cdist/kernel.py:72-91,
                  cdist/auto.py:126-182), brute force (tests/test_dp.py:12-23)
  dense_port.c    C/OpenMP port of the dense kernels (cdist/viterbi.c:73-193) plus a whole-plan
                  loop (cdist/kernel.py:94-138); the timed CPU baseline ("port")
  sparse.py       numpy sparse tables (cdist/sparse_dp.py:300-455) and the lookahead bound
                  (cdist/sparse_dp.py:148-217)
  table.py        completion tables (cdist/gmitm.c:61-186, cdist/search.py:83-142)
  table_port.c    the completion table in C with a native probe for the search: the timed CPU
                  baseline of the weight-bounded search
  tree.py         tree DP join over all pairs and the post-order executor (cdist/tree_dp.c:13-39,
                  cdist/tree_dp.py:442-501), brute force; run_port drives tree_port.c
  tree_port.c     the reference's Gray-code tree join in C: the timed CPU baseline of the tree DP
  Makefile        builds dense_port.so, tree_port.so, table_port.so, and oracle/_ref/ from the
                  reference C sources when the reference tree is present

Parity is pinned against golden vectors produced by the reference itself (tests/golden/).
"""
