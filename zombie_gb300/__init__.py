"""zombie_gb300: GB300-native Walk on Spheres / Walk on Stars engine."""
