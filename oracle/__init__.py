"""CPU oracle of the GB300 state-vector engine (test infrastructure only)."""
