"""Build the engine's CUDA library in-tree (nvcc, sm_103a only).

``build()`` compiles every ``csrc/*.cu`` translation unit in parallel and links
``libmpdo_gb300.so`` next to this file.  Rebuilds only when a source is newer
than the library.  No cmake, no torch extension machinery: one nvcc per file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = ROOT / 'csrc'
INCLUDE = ROOT.parent / 'include'
BUILD = ROOT / '_build'
LIB = PKG / 'libmpdo_gb300.so'

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
         '-Xptxas', '-O3']


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError('nvcc not found: the MPDO engine needs the CUDA toolkit to build')


def _sources():
    return sorted(CSRC.glob('*.cu'))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(_sources()) + list(CSRC.glob('*.cuh')) + list(INCLUDE.glob('*.h')) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src: Path):
        obj = BUILD / (src.stem + '.o')
        cmd = [cc, *ARCH, *FLAGS, *extra_flags, f'-I{INCLUDE}', f'-I{CSRC}', '-c', str(src), '-o', str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'nvcc failed on {src.name}:\n{r.stderr}')
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB.with_suffix('.so.tmp')
    cmd = [cc, *ARCH, '-shared', '-Xcompiler', '-fPIC', *map(str, objs), '-o', str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'link failed:\n{r.stderr}')
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    import sys
    print(build(force='-f' in sys.argv, verbose='-v' in sys.argv))
