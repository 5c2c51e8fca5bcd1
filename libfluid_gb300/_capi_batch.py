"""ctypes signatures of the batched and served entry points of include/sph_c.h."""
SIGNATURES: list = []
