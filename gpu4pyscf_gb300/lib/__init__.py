"""Native library loader (libgb300jk.so)."""
