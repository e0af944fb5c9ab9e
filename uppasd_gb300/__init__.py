"""GB300-native spin-update hot path for UppASD (LLG + Monte Carlo)."""
