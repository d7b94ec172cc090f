"""Generate the golden fixtures in tests/golden from the UNMODIFIED reference.

Runs the reference solver built by oracle/ref/build_ref.py (this container
only: it needs the reference sources) for the variants of
oracle/ref/variants.py and stores its binary FP64 dumps as compressed .npz.
Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / 'oracle' / 'ref'))
sys.path.insert(0, str(ROOT))
import build_ref  # noqa: E402
from variants import VARIANTS  # noqa: E402
from oracle.oracle import read_dump  # noqa: E402

OUT = Path(__file__).resolve().parent

# variant -> (steps, dump_every, fields to keep)
PLAN = {
    'ac_small': (500, 500, 'all'),
    'hcz_drop': (200, 200, 'all'),
    'hcz_rt': (300, 300, 'all'),
    'pp_drop': (200, 200, 'all'),
    'ac_c1': (2000, 0, ['rho', 'p', 'phi']),
    'ac_default': (2000, 0, ['rho', 'p', 'phi']),
    'uw_small': (500, 500, 'all'),
    'uw_hcz': (200, 200, 'all'),
    'uwls_small': (500, 500, 'all'),
    'uwls_hcz': (200, 200, 'all'),
    'uw4p_hcz': (200, 200, 'all'),
    'nee_rt': (300, 300, 'all'),
    'nee_ac': (300, 300, 'all'),
}


def main(names=None) -> None:
    meta_path = OUT / 'golden_meta.json'
    meta = json.loads(meta_path.read_text()) if names and meta_path.exists() else {}
    for name, (steps, every, keep) in PLAN.items():
        if names and name not in names:
            continue
        build_ref.build(name)
        dump = f'/tmp/golden_{name}.bin'
        out, log = build_ref.run(name, steps, every, threads=8, dump=dump)
        paths = [Path(dump + f'.{s}') for s in range(0, steps, every)] if every else []
        paths.append(Path(dump))
        arrays = {}
        for p in paths:
            st, fields = read_dump(p)
            for k, v in fields.items():
                if keep == 'all' or k in keep:
                    arrays[f'{k}@{st}'] = v
        np.savez_compressed(OUT / f'{name}.npz', **arrays)
        lines = [ln.split() for ln in log.splitlines() if ln.startswith('step ')]
        meta[name] = dict(variant=VARIANTS[name], steps=steps,
                          log={int(l[1]): dict(sumrho=float(l[3]), residual=float(l[5])) for l in lines})
        print(name, 'fields', len(arrays), 'size', (OUT / f'{name}.npz').stat().st_size)
    (OUT / 'golden_meta.json').write_text(json.dumps(meta, indent=1, sort_keys=True))


if __name__ == '__main__':
    main(sys.argv[1:] or None)
