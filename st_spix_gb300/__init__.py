"""st_spix_gb300 — GB300-native streaming BASS ("BIST") superpixels.

Drop-in for the reference's `bist_cuda` extension: see st_spix_gb300.bist_cuda.
"""
__version__ = "0.1.0"
