"""CPU oracle of the nBounce path-tracing pass (test infrastructure only)."""
