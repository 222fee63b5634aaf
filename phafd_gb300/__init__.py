"""GB300-native PHAFD particle-field hot path."""
