"""CPU oracle of the HoughLine path (test infrastructure only)."""
