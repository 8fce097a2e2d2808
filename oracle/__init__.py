"""CPU checkers for the GPU engine (test infrastructure)."""
