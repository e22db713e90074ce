"""GB300-native RHS path of the high-order curvilinear compressible solver."""
