"""Compile the CPU restatement (test infrastructure) into oracle/_build/libdugks_oracle.so.

gcc -O2 -ffp-contract=off keeps the reference's operation order and rounding
(no fused multiply-add), on x86-64 and aarch64 alike.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / '_build'
LIB = BUILD / 'libdugks_oracle.so'
SOURCES = [HERE / 'dugks_oracle.c', HERE / 'dugks_oracle_d2v16.c']


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES + [HERE / 'dugks_oracle.h'])
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix('.so.tmp')
    subprocess.run(['gcc', '-O2', '-ffp-contract=off', '-fopenmp', '-fPIC', '-shared', '-std=c11',
                    '-Wall', '-Wno-unused-function', '-o', str(tmp)] + [str(s) for s in SOURCES] + ['-lm'],
                   check=True)
    tmp.replace(LIB)
    return LIB


if __name__ == '__main__':
    print(build(force=True))
