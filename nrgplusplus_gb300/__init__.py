"""GB300-native NRG iteration engine (package root)."""
