"""Build the CUDA library libsclbm.so for sm_103a (in-tree, no cmake).

Every translation unit under ``idea.deploy_gb300/csrc`` is compiled in parallel
with ``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into
``sclbm/_lib/libsclbm.so`` (static CUDA runtime).  Rebuilds only when a
source or header is newer than the library.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), 'csrc')
INCLUDE = os.path.join(os.path.dirname(os.path.dirname(HERE)), 'include')
OUT_DIR = os.path.join(HERE, '_lib')
LIB = os.path.join(OUT_DIR, 'libsclbm.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-std=c++17', '-O3', '-lineinfo', '--expt-relaxed-constexpr', '-Xcompiler', '-fPIC',
              '-Xcompiler', '-fvisibility=hidden', '-I', INCLUDE]


def nvcc():
    for c in [os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc']:
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return 'nvcc'


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')) + glob.glob(os.path.join(CSRC, '*.cpp')))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(CSRC, '*.h')) + \
        glob.glob(os.path.join(INCLUDE, '*.h'))


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(verbose=False, force=False):
    """Compile and link libsclbm.so; returns its path."""
    if not force and up_to_date():
        return LIB
    obj_dir = os.path.join(OUT_DIR, 'obj')
    os.makedirs(obj_dir, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.basename(src) + '.o')
        cmd = [cc] + ARCH + NVCC_FLAGS + ['-c', src, '-o', obj]
        if src.endswith('.cpp'):
            cmd = [cc] + NVCC_FLAGS + ['-x', 'c++', '-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed on %s:\n%s%s' % (src, r.stdout, r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    srcs = _sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + '.%d.tmp' % os.getpid()
    cmd = [cc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart_static', '-lrt', '-ldl', '-lpthread']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s%s' % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(verbose=True, force='--force' in sys.argv))
