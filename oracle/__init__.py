"""ORACLE — test infrastructure, not product code.

CPU restatement of NetworkDynamics.jl's network RHS (SequentialExecution +
SequentialAggregator, and the threaded PolyesterExecution + PolyesterAggregator), a CPU
Tsit5, a dense Newton fixpoint solver and a numpy MPNN, used only by tests/,
__graft_entry__.smoke() and bench.py's CPU baseline, to check the GPU results against;
no product code imports it.
"""
