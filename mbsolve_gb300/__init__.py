"""mbsolve_gb300: GB300-native Maxwell-Bloch time loop (see README.md)."""
