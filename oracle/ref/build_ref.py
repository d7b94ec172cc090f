"""Build and run the unmodified reference solver for the oracle (test infrastructure).

Recipe, per variant of ``variants.py``:

1. read Ark/Constant/{ZeroFlip,ZeroReference,ZeroNamespace}.h and
   Ark/Lib/nonidealEoS.h from the reference tree, apply exact-substring
   substitutions (constants, switches, mesh name) and write the results to
   ``oracle/_ref/<variant>/include``; that directory comes first on the
   include path, so no reference Constant header is opened;
2. when gravity is on, write a copy of Ark/Cpp/SourceM.cpp with its
   commented gravity line (Ark/Cpp/SourceM.cpp:32) enabled to
   ``oracle/_ref/<variant>/src``;
3. compile every Ark/Cpp/*.cpp, Ark/Cpp/Mesh/*.cpp and Ark/Lib/<model>.cpp
   where they lie, with g++ -O2 -ffp-contract=off -fopenmp (main.cpp with
   -Dmain=reference_main), plus ``ref_driver.cpp``, into
   ``oracle/_ref/<variant>/ref_driver``;
4. write the mesh to ``oracle/_ref/<variant>/home/Mesh/<name>.cas`` (the
   reference reads ``$HOME/Mesh``) and, with ``--run``, run the driver there.

Nothing here is copied into the repository; ``oracle/_ref`` is git-ignored.
Usage: python oracle/ref/build_ref.py [variant ...] [--run STEPS] [--every N]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from mesh_cas import write_cas  # noqa: E402
from variants import VARIANTS  # noqa: E402

# the reference tree: DUGKS_REFERENCE, else where the build container mounts it
REF_ROOT = Path(os.environ.get('DUGKS_REFERENCE', '/root/reference'))
REF = REF_ROOT / 'Ark'
OUT = HERE.parent / '_ref'


def available() -> bool:
    """Whether the reference sources are present (they are not on the GPU machines)."""
    return (REF / 'Cpp').is_dir()


def _sub(text: str, old: str, new: str, what: str) -> str:
    n = text.count(old)
    if n != 1:
        raise RuntimeError(f'{what}: expected exactly one {old!r}, found {n}')
    return text.replace(old, new)


def mesh_name(v: dict) -> str:
    return f"{v['nx']}_{v['ny']}_Car_{'Wall' if v['walls'] else 'Periodic'}_oracle"


def gen_headers(name: str, v: dict, inc: Path) -> None:
    c = v['consts']
    nx, ny = v['nx'], v['ny']
    inc.mkdir(parents=True, exist_ok=True)
    # --- ZeroReference.h: mesh size and viscosity
    t = (REF / 'Constant/ZeroReference.h').read_text()
    t = _sub(t, 'Nx = 128,', f'Nx = {nx},', 'Nx')
    t = _sub(t, 'Ny = 128,', f'Ny = {ny},', 'Ny')
    t = _sub(t, 'NL = 128;', f'NL = {nx};', 'NL')
    t = _sub(t, 'ChLength = 128.0,', f'ChLength = {float(nx)!r},', 'ChLength')
    t = _sub(t, 'X_End = 128,', f'X_End = {nx},', 'X_End')
    t = _sub(t, 'Y_End = 128.0,', f'Y_End = {float(ny)!r},', 'Y_End')
    if 'Mu0' in c:
        t = _sub(t, 'Mu0 = 0.1,', f"Mu0 = {c['Mu0']!r},", 'Mu0')
    (inc / 'ZeroReference.h').write_text(t)
    # --- ZeroNamespace.h: phase-field and pseudopotential parameters
    t = (REF / 'Constant/ZeroNamespace.h').read_text()
    if 'M_Phi' in c:
        t = _sub(t, 'M_Phi = 0.1,', f"M_Phi = {c['M_Phi']!r},", 'M_Phi')
    if 'W' in c:
        t = _sub(t, 'Cn = 5/ChLength,', f"Cn = {c['W']!r}/ChLength,", 'Cn')
    if 'Sigma' in c:
        t = _sub(t, 'Sigma = 1E-2,', f"Sigma = {c['Sigma']!r},", 'Sigma')
    if 'RhoL' in c or 'RhoV' in c:
        t = _sub(t, 'RhoL = 10.0,RhoV = 1.0,',
                 f"RhoL = {c.get('RhoL', 10.0)!r},RhoV = {c.get('RhoV', 1.0)!r},", 'RhoL/RhoV')
    if 'Gy' in c:
        t = _sub(t, 'Gx = 0.0, Gy = 0.0,', f"Gx = 0.0, Gy = {c['Gy']!r},", 'Gy')
    if 'radius' in c:
        t = _sub(t, 'radius = 0.36*ChLength,', f"radius = {c['radius']!r},", 'radius')
    if 'PP_RhoL' in c:
        t = _sub(t, 'RhoL = 2.4806E-1, RhoV = 4.5435E-2;',
                 f"RhoL = {c['PP_RhoL']!r}, RhoV = {c['PP_RhoV']!r};", 'PP rho')
    if 'Tr' in c:
        t = _sub(t, 'Tr = 0.85,', f"Tr = {c['Tr']!r},", 'Tr')
    (inc / 'ZeroNamespace.h').write_text(t)
    # --- ZeroFlip.h: mesh name, model family, walls
    t = (REF / 'Constant/ZeroFlip.h').read_text()
    t = _sub(t, '"128_128_Car_Periodic_Square_LBM"', f'"{mesh_name(v)}"', 'mesh name')
    extra = []
    if v.get('scheme', 'CD').startswith('UW'):
        t = _sub(t, '#ifndef _FLUX_SCHEME_CD_ARK\n#define _FLUX_SCHEME_CD_ARK "CD"\n'
                    '#define _FLUX_SCHEME_ARK _FLUX_SCHEME_CD_ARK\n#endif',
                 '#define _FLUX_SCHEME_UW_ARK "UW"\n#define _FLUX_SCHEME_ARK _FLUX_SCHEME_UW_ARK', 'flux scheme')
        # the cell gradient of the UW reconstruction (read by ref_driver.cpp)
        if v['scheme'] == 'UW_LS':
            extra.append('#define REF_UW_GRAD_LS')
        elif v['scheme'] == 'UW_4P':
            extra.append('#define REF_UW_GRAD_4P')
    if v['model'] == 'D2Q9PP':
        t = _sub(t, '#ifndef _ARK_ALLENCAHN_FLIP\n#define _ARK_ALLENCAHN_FLIP\n#endif', '', 'AC flip')
        extra.append('#define _ARK_PSEUDOPSI_FLIP')
    if v['walls']:
        extra += ['#define _Wall_3_BCs_FLIP 3',
                  '#define _Wall_3_BCs_NEE' if v.get('wall') == 'NEE' else '#define _Wall_3_BCs_BB']
    if extra:
        idx = t.rfind('#endif')
        t = t[:idx] + '\n'.join(extra) + '\n' + t[idx:]
    (inc / 'ZeroFlip.h').write_text(t)
    # --- ZeroCondition.h is included by the reference main (renamed); keep it
    (inc / 'ZeroCondition.h').write_text((REF / 'Constant/ZeroCondition.h').read_text())
    # --- nonidealEoS.h: Carnahan-Starling attraction and critical temperature
    t = (REF / 'Lib/nonidealEoS.h').read_text()
    if 'aCS' in c:
        t = _sub(t, 'aCS = 1.0,', f"aCS = {c['aCS']!r},", 'aCS')
    if 'Tc_CS' in c:
        t = _sub(t, 'Tc_CS = 0.0943,', f"Tc_CS = {c['Tc_CS']!r},", 'Tc_CS')
    (inc / 'nonidealEoS.h').write_text(t)


def build(name: str, jobs: int = 8) -> Path:
    v = VARIANTS[name]
    vdir = OUT / name
    inc = vdir / 'include'
    src = vdir / 'src'
    obj = vdir / 'obj'
    gen_headers(name, v, inc)
    src.mkdir(parents=True, exist_ok=True)
    obj.mkdir(parents=True, exist_ok=True)
    sources = sorted((REF / 'Cpp').glob('*.cpp')) + sorted((REF / 'Cpp/Mesh').glob('*.cpp'))
    sources.append(REF / 'Lib' / f"{v['model']}.cpp")
    if v['consts'].get('Gy', 0.0) != 0.0:
        t = (REF / 'Cpp/SourceM.cpp').read_text()
        t = _sub(t, '//\tcellptr->msq->Fy -= Gy*(cellptr->msq->Rho-RhoL);',
                 '\tcellptr->msq->Fy -= Gy*(cellptr->msq->Rho-RhoL);', 'gravity line')
        (src / 'SourceM.cpp').write_text(t)
        sources = [s for s in sources if s.name != 'SourceM.cpp'] + [src / 'SourceM.cpp']
    sources.append(HERE / 'ref_driver.cpp')
    common = ['g++', '-O2', '-ffp-contract=off', '-fopenmp', '-w',
              f'-I{inc}', f'-I{REF / "Header"}', f'-I{REF / "Lib"}', f'-I{REF / "Constant"}']

    def compile_one(s: Path) -> Path:
        o = obj / (s.stem + '.o')
        cmd = common + (['-std=c++14'] if s.name == 'ref_driver.cpp' else ['-std=c++11'])
        if s.name == 'main.cpp':
            cmd.append('-Dmain=reference_main')
        subprocess.run(cmd + ['-c', str(s), '-o', str(o)], check=True)
        return o

    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_one, sources))
    exe = vdir / 'ref_driver'
    subprocess.run(['g++', '-fopenmp', '-o', str(exe)] + [str(o) for o in objs], check=True)
    home = vdir / 'home'
    write_cas(str(home / 'Mesh' / (mesh_name(v) + '.cas')), v['nx'], v['ny'], v['walls'])
    # the reference writes to ../FlowField/{global,Convergence} relative to its cwd
    (vdir / 'run').mkdir(exist_ok=True)
    for d in ('FlowField/global', 'FlowField/Convergence'):
        (vdir / d).mkdir(parents=True, exist_ok=True)
    return exe


def run(name: str, steps: int, every: int = 0, threads: int | None = None,
        dump: str | None = None, extra_env: dict | None = None) -> tuple[Path, str]:
    v = VARIANTS[name]
    vdir = OUT / name
    env = dict(os.environ, HOME=str(vdir / 'home'))
    if threads:
        env['OMP_NUM_THREADS'] = str(threads)
    if extra_env:
        env.update(extra_env)
    out = Path(dump) if dump else vdir / f'dump_{steps}.bin'
    cmd = [str(vdir / 'ref_driver'), v['init'], str(steps), str(out)]
    if every:
        cmd.append(str(every))
    r = subprocess.run(cmd, cwd=vdir / 'run', env=env, stdin=subprocess.DEVNULL,
                       capture_output=True, text=True, check=True)
    return out, r.stdout


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('variants', nargs='*')
    ap.add_argument('--run', type=int, default=0)
    ap.add_argument('--every', type=int, default=0)
    ap.add_argument('--threads', type=int, default=0)
    a = ap.parse_args()
    names = a.variants or list(VARIANTS)
    for nm in names:
        exe = build(nm)
        print('built', exe)
        if a.run:
            out, log = run(nm, a.run, a.every, a.threads or None)
            tail = [ln for ln in log.splitlines() if ln.startswith(('step', 'done'))]
            print('\n'.join(tail[-5:]))
            print('dump', out)
