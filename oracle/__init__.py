"""CPU oracle for the GridNeighborhoodSearch + FullGridCellList hot path.

TEST INFRASTRUCTURE ONLY: a restatement of the reference's CPU algorithm that tests/,
__graft_entry__.smoke() and the CPU-baseline leg of bench.py compare the CUDA path with.
"""
