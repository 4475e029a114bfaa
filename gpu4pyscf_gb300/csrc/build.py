"""Build libgb300jk.so (sm_103a) in-tree with nvcc.

The per-class kernels are compiled from jk_classes.cu once per bra pair
class (-DJK_BRA_CLASS=0..9) so the translation units compile in parallel,
then linked with the host driver into gpu4pyscf_gb300/lib/libgb300jk.so.
"""
import concurrent.futures
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, '_build')
LIB_DIR = os.path.join(PKG, 'lib')
LIB = os.path.join(LIB_DIR, 'libgb300jk.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC = os.environ.get('NVCC', 'nvcc')
FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '-diag-suppress', '1444',
         '-I' + HERE, '-I' + os.path.join(ROOT, 'include')]
NBRA = 10

# every file of this directory that can reach the library: a change to any
# of them forces a rebuild
SOURCE_EXTS = ('.cu', '.cuh', '.h', '.inc', '.py')


def _sources():
    return sorted(f for f in os.listdir(HERE) if f.endswith(SOURCE_EXTS))


def _digest():
    h = hashlib.sha256()
    for f in _sources():
        h.update(f.encode())
        with open(os.path.join(HERE, f), 'rb') as fh:
            h.update(fh.read())
    for hdr in ('gb300jk.h', 'gb300mlp.h'):
        with open(os.path.join(ROOT, 'include', hdr), 'rb') as fh:
            h.update(fh.read())
    h.update(' '.join(ARCH + FLAGS).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('build failed: %s\n%s\n%s' % (' '.join(cmd), r.stdout, r.stderr))
    return r.stderr


def build(force=False, verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    stamp = os.path.join(BUILD, 'stamp')
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB
    cmds = []
    objs = []
    for b in range(NBRA):
        o = os.path.join(BUILD, 'jk_classes_%d.o' % b)
        cmds.append([NVCC] + ARCH + FLAGS + ['-DJK_BRA_CLASS=%d' % b, '-c',
                                             os.path.join(HERE, 'jk_classes.cu'), '-o', o])
        objs.append(o)
    for src in ('jk_engine.cu', 'jk_generic.cu', 'jk_grad.cu', 'int1e.cu', 'mlp.cu'):
        o = os.path.join(BUILD, src.replace('.cu', '.o'))
        cmds.append([NVCC] + ARCH + FLAGS + ['-c', os.path.join(HERE, src), '-o', o])
        objs.append(o)
    # largest classes first so the long compiles start early
    order = list(reversed(range(NBRA))) + list(range(NBRA, len(cmds)))
    jobs = jobs or min(len(cmds), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_run, cmds[i]) for i in order]
        for f in futs:
            msg = f.result()
            if verbose and msg:
                sys.stderr.write(msg)
    tmp = LIB + '.tmp'
    _run([NVCC] + ARCH + ['-shared', '-o', tmp] + objs)
    os.replace(tmp, LIB)
    with open(stamp, 'w') as f:
        f.write(dig)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
