"""GB300-native VBM3D (placeholder; filled in below)."""
