"""GB300-native method-of-lines right-hand side of PeleC (getMOLSrcTerm) for
one AMR level without embedded boundaries."""
