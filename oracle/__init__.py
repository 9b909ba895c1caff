"""Oracle package: the CPU restatement of the reference EMC kernels and the
FP64 form of the fused iteration.  Test infrastructure only -- imported by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the
emc_gb300 package."""
