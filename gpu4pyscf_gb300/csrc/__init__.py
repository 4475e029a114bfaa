"""CUDA sources of the J/K engine and their build script."""
