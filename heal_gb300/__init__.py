"""GB300-native HEAL vendor backend (package root)."""
