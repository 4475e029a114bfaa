from .mole import Mole, M, BOHR, cart2sph_coeff, gto_norm, cart_components, ncart, nsph
from . import basis
