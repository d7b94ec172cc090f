"""Golden Case.ark and FlowField files written by the reference's own writers.

OutputCase (Ark/Cpp/Output.cpp:65-141) and Output_Flowfield
(Ark/Cpp/Output.cpp:541-606) run inside the reference driver
(oracle/ref/ref_driver.cpp, with REF_FLOWFIELD set) for a few steps of two
small cases: the reference's AC_Drop init on a 32x24 periodic grid (ac_ff, and
uw_ff with the UW flux scheme) and a 16x64 Rayleigh-Taylor box with walls
(hcz_rt, and nee_rt with NEE walls).  The files land in
tests/golden/flowfield/<case>/ (FlowField .dat files gzip-compressed), with the
reference's MidX / MidY / Diag profile files after the last step
(Ark/Cpp/Output.cpp:312-532, under Convergence/) and, for the AC_Drop cases,
AC_Drop_L2Norm (Ark/Cpp/Output.cpp:226-238) in l2.json.
Needs the reference sources, so it runs only where they are present:

    python tests/golden/make_flowfield_golden.py
"""
import gzip
import json
import shutil
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / 'oracle' / 'ref'))

import build_ref  # noqa: E402

STEPS = {'ac_ff': 20, 'hcz_rt': 20, 'uw_ff': 20, 'nee_rt': 20}


def main(names=None) -> None:
    for name, steps in STEPS.items():
        if names and name not in names:
            continue
        build_ref.build(name)
        vdir = build_ref.OUT / name
        ff = vdir / 'FlowField'
        shutil.rmtree(ff, ignore_errors=True)
        (ff / 'global').mkdir(parents=True)
        (ff / 'Convergence').mkdir(parents=True)
        _, log = build_ref.run(name, steps, threads=1, extra_env={"REF_FLOWFIELD": "1"})
        out = ROOT / 'tests' / 'golden' / 'flowfield' / name
        shutil.rmtree(out, ignore_errors=True)
        out.mkdir(parents=True)
        shutil.copy(ff / 'Case.ark', out / 'Case.ark')
        for f in sorted((ff / 'global').glob('*.dat')):
            with open(f, 'rb') as src, gzip.GzipFile(out / (f.name + '.gz'), 'wb', mtime=0) as dst:
                shutil.copyfileobj(src, dst)
        conv = out / 'Convergence'
        conv.mkdir()
        for f in sorted((ff / 'Convergence').glob('*.dat')):
            shutil.copy(f, conv / f.name)
        l2 = [ln.split()[1] for ln in log.splitlines() if ln.startswith('L2_phi ')]
        if l2:
            (out / 'l2.json').write_text(json.dumps({'steps': steps, 'L2_phi': l2[0]}) + '\n')
        print(name, sorted(p.name for p in out.iterdir()))


if __name__ == '__main__':
    main(sys.argv[1:] or None)
