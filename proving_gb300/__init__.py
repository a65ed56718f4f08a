"""GB300-native CUDA backend for the Stwo Circle-STARK prover hot path."""
