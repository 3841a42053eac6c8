"""GB300-native RocfluMP explicit residual-and-update path."""
