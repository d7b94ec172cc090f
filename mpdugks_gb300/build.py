"""Build libdugks_gpu.so in-tree for sm_103a (nvcc, one -gencode, parallel TUs)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / 'csrc'
BUILD = PKG / '_build'
LIB = BUILD / 'libdugks_gpu.so'
INCLUDE = PKG.parent / 'include'
HOST = PKG / 'host'
RUNNER = BUILD / 'dugks_run'

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
# host code: no FMA contraction, so the host-side initial states are the same
# doubles on x86-64 and aarch64 (and equal the reference's)
NVFLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
           '-Xcompiler', '-ffp-contract=off', '--expt-relaxed-constexpr', f'-I{INCLUDE}']


# the reference-exact FP64 step keeps every multiply and add separately rounded
PER_FILE = {'fp64_exact.cu': ['-fmad=false']}


def sources() -> list[Path]:
    # the serving loop writes FlowField files with the host driver's writer
    return sorted(CSRC.glob('*.cu')) + sorted(CSRC.glob('*.cpp')) + [HOST / 'flowfield.cpp']


def nvcc() -> str:
    exe = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not Path(exe).exists():
        raise RuntimeError('nvcc not found')
    return exe


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    deps = srcs + sorted(CSRC.glob('*.cuh')) + sorted(CSRC.glob('*.h')) + sorted(INCLUDE.glob('*.h')) + \
        sorted(HOST.glob('*.hpp'))
    newest = max(p.stat().st_mtime for p in deps)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest and not extra:
        build_host()
        return LIB
    exe = nvcc()
    flags = NVFLAGS + (extra or [])

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.name + '.o')
        cmd = [exe] + ARCH + flags + PER_FILE.get(src.name, []) + ['-x', 'cu', '-c', str(src), '-o', str(obj)]
        if verbose:
            cmd.insert(1, '-Xptxas=-v')
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'nvcc failed on {src.name}:\n{r.stderr}')
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix('.so.tmp')
    r = subprocess.run([exe] + ARCH + ['-shared', '-cudart=static', '-o', str(tmp)] + [str(o) for o in objs],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'nvcc link failed:\n{r.stderr}')
    tmp.replace(LIB)
    build_host(force=True)
    return LIB


def build_host(force: bool = False) -> Path:
    """The host driver dugks_run (C++, links libdugks_gpu.so)."""
    srcs = sorted(HOST.glob('*.cpp'))
    deps = srcs + sorted(HOST.glob('*.hpp')) + sorted(INCLUDE.glob('*.h')) + [LIB]
    if not force and RUNNER.exists() and RUNNER.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return RUNNER
    gxx = shutil.which('g++') or 'g++'
    tmp = RUNNER.with_suffix('.tmp')
    cmd = [gxx, '-O2', '-std=c++17', '-ffp-contract=off', f'-I{INCLUDE}'] + [str(x) for x in srcs] + \
          [f'-L{BUILD}', '-ldugks_gpu', "-Wl,-rpath,$ORIGIN", '-o', str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'g++ failed on the host driver:\n{r.stderr}')
    tmp.replace(RUNNER)
    return RUNNER


if __name__ == '__main__':
    import sys
    print(build(force=True, verbose='-v' in sys.argv))
