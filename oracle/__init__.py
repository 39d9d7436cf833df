"""CPU oracle of the thin-wire MoM fill-and-solve path (test infrastructure only)."""
