"""GB300-native plane-wave H.psi and eigensolver path behind QimPy's operator API."""
