"""RHS builders for the suite's equations (wave, Euler, Maxwell)."""
