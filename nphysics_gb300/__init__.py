"""GB300-native rigid-body step for nphysics3d (package root)."""
