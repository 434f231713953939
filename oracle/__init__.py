"""Oracle package: CPU restatement of gratopy's kernels and solvers.

Test infrastructure only (tests/, bench.py's CPU baseline, smoke()); the
product path never imports it.
"""
