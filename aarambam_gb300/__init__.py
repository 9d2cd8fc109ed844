"""GB300-native Aarambam initial-condition path (white noise -> modal
non-Gaussian potential -> 2LPT displacements -> particles)."""
