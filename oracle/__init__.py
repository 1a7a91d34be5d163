"""FP64 CPU oracle of the scalar-propagation hot path (test infrastructure only)."""
