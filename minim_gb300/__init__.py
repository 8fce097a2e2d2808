"""GB300-native minimisation engine (package stub)."""
