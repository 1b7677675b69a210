"""Test-only oracles: an FP64 numpy restatement of the reference's SIM
reconstruction and makeotf, and a harness that runs the reference's own CUDA
kernels.  Nothing in the product imports this package."""
