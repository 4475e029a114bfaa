"""Extract the golden J/K fingerprints from the reference's own tests.

Reads (as text) gpu4pyscf/scf/tests/test_rhf.py (molecule ``mol1`` with its
inline uncontracted basis, test_get_jk1 / test_get_jk1_hermi0 fingerprints)
and gpu4pyscf/scf/tests/test_scf_jk.py (test_jk_get_k_hermi2 on O2/STO-3G)
and writes reference_fingerprints.json beside this script.

Run in a tree where the reference is present:
    python tests/golden/make_golden.py /path/to/reference
"""
import json
import os
import re
import sys


def main(ref_root):
    t_rhf = open(os.path.join(ref_root, 'gpu4pyscf/scf/tests/test_rhf.py')).read()
    t_jk = open(os.path.join(ref_root, 'gpu4pyscf/scf/tests/test_scf_jk.py')).read()
    m = re.search(r"mol1 = pyscf\.M\(\s*atom='''(.*?)''',\s*basis='''(.*?)''',", t_rhf, re.S)
    atom1, basis1 = m.group(1), m.group(2)

    def body(src, name):
        return src.split('def ' + name)[1].split('\n    def ')[0].split('\ndef ')[0]

    def fps(txt):
        return [float(x) for x in re.findall(r"lib\.fp\([^)]*\)\)?,\s*([-\d.e]+)", txt)]

    h1 = fps(body(t_rhf, 'test_get_jk1(self)'))
    h0 = fps(body(t_rhf, 'test_get_jk1_hermi0(self)'))
    b2 = body(t_jk, 'test_jk_get_k_hermi2')
    atom2 = re.search(r"atom='''(.*?)'''", b2, re.S).group(1)
    fp2 = float(re.search(r"lib\.fp\(vk\.get\(\)\) - ([-\d.e]+)\)", b2).group(1))
    out = {
        'source': 'gpu4pyscf/scf/tests/test_rhf.py (mol1, test_get_jk1, test_get_jk1_hermi0); '
                  'gpu4pyscf/scf/tests/test_scf_jk.py (test_jk_get_k_hermi2)',
        'mol1': {'atom': atom1, 'basis': basis1, 'unit': 'Angstrom', 'seed': 1, 'n_dm': 2,
                 'hermi1': {'fp_vj': h1[0], 'fp_vk': h1[1], 'places': 7},
                 'hermi0': {'fp_vj': h0[0], 'fp_vk': h0[1], 'places': 7}},
        'o2_sto3g_hermi2': {'atom': atom2, 'basis': 'sto-3g', 'seed': 1, 'n_dm': 2,
                            'fp_vk': fp2, 'tol': 1e-12},
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'reference_fingerprints.json')
    with open(path, 'w') as f:
        json.dump(out, f, indent=1)
    print('wrote', path)


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden.py <root of the gpu4pyscf source tree>')
    main(sys.argv[1])
