"""CPU oracle of the finite-volume hot path: test infrastructure only."""
