"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / 'include' / 'dugks_gpu.h').read_text()
    return sorted(set(re.findall(r'\b(dugks_(?:gpu|srv|slabs)_\w+)\s*\(', text)))


def test_header_declares_abi():
    syms = declared_symbols()
    for s in ('dugks_gpu_create', 'dugks_gpu_upload', 'dugks_gpu_step', 'dugks_gpu_reduce',
              'dugks_gpu_download', 'dugks_gpu_destroy', 'dugks_gpu_last_error'):
        assert s in syms


def test_library_builds_and_exports_all_symbols():
    import ctypes
    from mpdugks_gb300 import build, capi
    lib_path = build.build()
    lib = ctypes.CDLL(str(lib_path))
    for s in declared_symbols():
        assert hasattr(lib, s), f'{s} not exported'
    # the binding's signature table covers the whole header
    assert set(capi.SIGNATURES) == set(declared_symbols())


def test_create_fails_cleanly_without_valid_grid():
    import ctypes
    from mpdugks_gb300 import capi
    lib = capi.load(build_if_missing=True)
    case = capi.make_case('AC')
    grid = capi.GridT(2, 2, 0)  # too small: rejected before any CUDA call
    h = ctypes.c_void_p()
    rc = lib.dugks_gpu_create(ctypes.byref(case), ctypes.byref(grid), ctypes.byref(h))
    assert rc == capi.DUGKS_EINVAL
    buf = ctypes.create_string_buffer(256)
    lib.dugks_gpu_last_error(None, buf, 256)
    assert b'nx' in buf.value


def test_serving_create_reports_missing_gpu():
    """Without a GPU the server is not created: an error code, no fallback."""
    import ctypes
    import torch
    from mpdugks_gb300 import capi
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    lib = capi.load(build_if_missing=True)
    h = ctypes.c_void_p()
    rc = lib.dugks_srv_create(None, ctypes.byref(h))
    assert rc == capi.DUGKS_ECUDA and not h.value


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes structure has the size and field offsets the C compiler gives the header's."""
    import ctypes
    import shutil
    import subprocess
    from mpdugks_gb300 import capi
    gcc = shutil.which('gcc') or shutil.which('cc')
    if gcc is None:
        pytest.skip('no C compiler')
    structs = {'dugks_case_t': capi.CaseT, 'dugks_grid_t': capi.GridT, 'dugks_reductions_t': capi.ReductionsT,
               'dugks_srv_config_t': capi.SrvConfigT, 'dugks_srv_request_t': capi.SrvRequestT,
               'dugks_srv_status_t': capi.SrvStatusT, 'dugks_srv_stats_t': capi.SrvStatsT}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dugks_gpu.h"', 'int main(void) {']
    want = []
    for cname, py in structs.items():
        lines.append(f'    printf("%zu\\n", sizeof({cname}));')
        want.append(ctypes.sizeof(py))
        for fname, *_ in py._fields_:
            lines.append(f'    printf("%zu\\n", offsetof({cname}, {fname}));')
            want.append(getattr(py, fname).offset)
    lines += ['    return 0;', '}']
    src = tmp_path / 'layout.c'
    src.write_text('\n'.join(lines) + '\n')
    exe = tmp_path / 'layout'
    subprocess.run([gcc, f'-I{ROOT / "include"}', str(src), '-o', str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == want


@pytest.mark.parametrize('model,precision,walls', [('AC', 'fp32dev', True), ('HCZ', 'fp64', True),
                                                   ('PP9', 'fp64', False), ('PP16', 'fp32dev', False),
                                                   ('AC', 'fp64fused', False)])
def test_uw_flux_scheme_rejected_where_not_supported(model, precision, walls):
    """UW runs with the plain FP64 precisions and FP32 storage, the Allen-Cahn models and
    periodic y; other combinations are refused before any device work, with the reason."""
    import ctypes
    from mpdugks_gb300 import capi
    lib = capi.load(build_if_missing=True)
    case = capi.make_case(model, precision, scheme='UW')
    grid = capi.GridT(16, 16, int(walls))
    h = ctypes.c_void_p()
    rc = lib.dugks_gpu_create(ctypes.byref(case), ctypes.byref(grid), ctypes.byref(h))
    assert rc == capi.DUGKS_EINVAL and not h.value
    buf = ctypes.create_string_buffer(256)
    lib.dugks_gpu_last_error(None, buf, 256)
    assert b'UW' in buf.value


# FP32 storage takes NEE walls on grids of at least 8 rows (its streaming step)
@pytest.mark.parametrize('model,precision,walls,ny', [('AC', 'fp32dev', 1, 6), ('PP9', 'fp64', 0, 16),
                                                      ('HCZ', 'fp64fused', 1, 16)])
def test_nee_walls_rejected_where_not_supported(model, precision, walls, ny):
    import ctypes
    from mpdugks_gb300 import capi
    lib = capi.load(build_if_missing=True)
    case = capi.make_case(model, precision, wall='NEE')
    grid = capi.GridT(16, ny, walls)
    h = ctypes.c_void_p()
    rc = lib.dugks_gpu_create(ctypes.byref(case), ctypes.byref(grid), ctypes.byref(h))
    assert rc == capi.DUGKS_EINVAL and not h.value
    buf = ctypes.create_string_buffer(256)
    lib.dugks_gpu_last_error(None, buf, 256)
    assert b'NEE' in buf.value
