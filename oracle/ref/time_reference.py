"""Time the unmodified reference solver against the CPU restatement on the same cores
-- TEST INFRASTRUCTURE ONLY (a calibration of the CPU baseline, run where the
reference sources are; the reference cannot be built on the aarch64 GPU machines,
whose CPU baseline is the restatement).

Both run the 512 x 2048 Rayleigh-Taylor workload (HCZ, walls, the case constants of
bench.py's rt512x2048) for the same steps with the same OpenMP thread count, after
one untimed step; the reference reports its own loop time (ref_driver's
"done ... seconds"), the restatement is timed around Oracle.step.  The two final
states are compared bit for bit.  Prints one JSON line.

Usage: python oracle/ref/time_reference.py [--steps N] [--threads T] [--out FILE]
(the committed oracle/ref/reference_timing.json is its output; bench.py reports it beside the
CPU baseline)
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))

import build_ref  # noqa: E402
from variants import VARIANTS  # noqa: E402

NAME = 'rt512x2048'


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--threads', type=int, default=os.cpu_count() or 1)
    ap.add_argument('--out', default=None)
    a = ap.parse_args()
    import bench
    from oracle.oracle import Oracle, read_dump
    wl = bench.WORKLOADS[NAME]
    kw = bench.case_kw(wl)
    VARIANTS[NAME] = dict(model='D2Q9HCZ', nx=wl['nx'], ny=wl['ny'], walls=True, init='ac_rt', consts=kw)
    build_ref.build(NAME)
    # the reference: 1 + steps steps; its printed loop time covers all of them (dumps in a
    # temporary directory: ~300 MB each)
    tmp = tempfile.TemporaryDirectory()
    _, log1 = build_ref.run(NAME, 1, threads=a.threads, dump=f'{tmp.name}/d1.bin')
    out, log = build_ref.run(NAME, 1 + a.steps, threads=a.threads, dump=f'{tmp.name}/d.bin')
    secs = lambda text: float(next(ln for ln in text.splitlines() if ln.startswith('done')).split()[6])
    ref_s = secs(log) - secs(log1)
    o = Oracle('HCZ', wl['nx'], wl['ny'], True, 'ac_rt', **kw)
    o.step(1, a.threads)
    t0 = time.perf_counter()
    o.step(a.steps, a.threads)
    port_s = time.perf_counter() - t0
    _, ref = read_dump(out)
    tmp.cleanup()
    same = all(bool((o.get(k) == v).all()) for k, v in ref.items() if k in ('rho', 'u', 'v', 'p', 'phi'))
    cells = wl['nx'] * wl['ny']
    res = {'workload': wl['name'], 'threads': a.threads, 'steps': a.steps,
           'reference_mlups': round(cells * a.steps / ref_s / 1e6, 3),
           'port_mlups': round(cells * a.steps / port_s / 1e6, 3),
           'port_over_reference': round(ref_s / port_s, 3), 'final_states_bit_identical': same}
    print(json.dumps(res))
    if a.out:
        res['where'] = ('the x86-64 build container (the reference cannot be built on the aarch64 GPU host: '
                        'its sources are not there and there is no cross compiler)')
        res['recipe'] = f'python oracle/ref/time_reference.py --steps {a.steps} --out {a.out}'
        Path(a.out).write_text(json.dumps(res, indent=1) + '\n')
    return 0


if __name__ == '__main__':
    sys.exit(main())
