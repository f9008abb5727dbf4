"""CPU oracle of the thermal Monte Carlo and ray tracer (test infrastructure only)."""
