"""Resolution of (omega, lr_factor, sr_factor) as gpu4pyscf/scf/jk.py:1122-1168
does it, and the operator each combination selects (host logic, no GPU)."""
import pytest

from gpu4pyscf_gb300 import gto
from gpu4pyscf_gb300.scf.jk import _check_rsh_factors, _env_operator


def _mol(omega=0.):
    mol = gto.M(atom='H 0 0 0; H 0 0 0.74', basis='sto-3g')
    mol.omega = omega
    return mol


@pytest.mark.parametrize('args, want', [
    ((None, None, None), (0, 1, 1)),          # mol.omega = 0: full range
    ((0.3, None, None), (0.3, 1, 0)),         # libcint: omega > 0 is long range
    ((-0.3, None, None), (-0.3, 0, 1)),       # omega < 0 is short range
    ((0.3, None, 0.5), (-0.3, 0, 0.5)),       # sr only: short range, omega made negative
    ((0.3, 0.7, None), (0.3, 0.7, 0)),        # lr only
    ((0.3, 0.6, 0.2), (-0.3, 0.6, 0.2)),      # both parts: omega negative marks the sr part
    ((0.3, 0.4, 0.4), (0, 0.4, 0.4)),         # lr == sr: full range
    ((0., None, 0.5), (0., 0.5, 0.5)),
])
def test_resolution(args, want):
    assert _check_rsh_factors(_mol(), *args) == want


def test_mol_omega_default():
    assert _check_rsh_factors(_mol(0.25), None, None, None) == (0.25, 1, 0)
    assert _check_rsh_factors(_mol(-0.25), None, None, None) == (-0.25, 0, 1)


def test_long_range_needs_positive_omega():
    with pytest.raises(AssertionError):
        _check_rsh_factors(_mol(), -0.3, 0.7, None)


def test_env_operator():
    assert _env_operator(0.) == (0., 1., 1.)
    assert _env_operator(0.2) == (0.2, 1., 0.)
    assert _env_operator(-0.2) == (0.2, 0., 1.)
