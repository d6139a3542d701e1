"""CPU oracle: an FP64 C restatement of mcvine/acc's propagation chain.
Test infrastructure only (the checker and the CPU baseline)."""
