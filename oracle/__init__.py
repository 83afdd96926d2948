"""CPU oracle of the LASSIE integrator: test infrastructure (the checker)."""
