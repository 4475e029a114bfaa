"""SCF layer: J/K builds (jk) and the restricted Hartree-Fock driver (hf)."""
