"""The .cas mesh reader of the host driver (mpdugks_gb300/host/mesh_cas.cpp):
meshes in the layout the reference's MeshConstruct reads (Ark/Cpp/Mesh/
MeshConstruct.cpp:69-123), with cells, faces and nodes numbered in any order,
mapped to the GPU's row-major grid; meshes the GPU path does not take are
rejected with the reason."""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / 'oracle' / 'ref'))


def runner() -> Path:
    from mpdugks_gb300 import build
    build.build()
    return build.RUNNER


def mesh_info(path):
    r = subprocess.run([runner(), 'mesh-info', str(path)], capture_output=True, text=True)
    if r.returncode != 0:
        return None, r.stderr
    lines = r.stdout.split('\n')
    nx, ny, walls = (int(v) for v in lines[0].split())
    return (nx, ny, walls, [int(v) for v in lines[1].split()]), ''


def write_permuted_cas(path, nx, ny, walls, seed, bc_top=None, dx=1.0, mixed=False):
    """A Cartesian mesh with its nodes, cells and faces numbered in a seeded
    random order.  Returns cell_index: mesh cell k -> j*nx + i."""
    from mesh_cas import cartesian_faces
    rng = np.random.default_rng(seed)
    faces = cartesian_faces(nx, ny, walls)  # (bc, zone, n0, n1, c0, c1), 1-based ids
    nn, nc = (nx + 1) * (ny + 1), nx * ny
    node_new = rng.permutation(nn) + 1    # old id - 1 -> new id
    cell_new = rng.permutation(nc) + 1
    order = rng.permutation(len(faces))   # new face position -> old face index
    if bc_top is not None:
        faces = [(bc_top if f[1] == 7 else f[0],) + f[1:] for f in faces]
    # faces keep their zone runs contiguous: sort the shuffled faces by zone
    order = sorted(order, key=lambda k: faces[k][1])
    new_pos = {old: k for k, old in enumerate(order)}
    out = ['(0 "permuted Cartesian mesh")', '(2 2)', f'(10 (0 1 {nn:x} 0 2))', f'(12 (0 1 {nc:x} 0))',
           f'(13 (0 1 {len(faces):x} 0))', f'(10 (1 1 {nn:x} 1 2)(']
    xy = [None] * nn
    for j in range(ny + 1):
        for i in range(nx + 1):
            xy[node_new[j * (nx + 1) + i] - 1] = (i * dx, j * dx)
    out += [f'{x!r} {y!r}' for x, y in xy]
    out.append('))')
    out.append(f'(12 (2 1 {nc:x} 1 3))')
    start = 0
    while start < len(order):
        f0 = faces[order[start]]
        end = start
        while end < len(order) and faces[order[end]][:2] == f0[:2]:
            end += 1
        ft = 0 if mixed else 2
        out.append(f'(13 ({f0[1]:x} {start + 1:x} {end:x} {f0[0]:x} {ft})(')
        for k in range(start, end):
            bc, zone, n0, n1, c0, c1 = faces[order[k]]
            ids = [node_new[n0 - 1], node_new[n1 - 1], cell_new[c0 - 1], cell_new[c1 - 1] if c1 else 0]
            out.append(('2 ' if mixed else '') + ' '.join(f'{v:x}' for v in ids))
        out.append('))')
        start = end
    # periodic pairs, in the generator's own face numbering mapped to the new one
    first_left = (nx - 1) * ny + nx * (ny - 1)
    pairs = [(first_left + j, first_left + ny + j) for j in range(ny)]
    if not walls:
        fb = first_left + 2 * ny
        pairs += [(fb + i, fb + nx + i) for i in range(nx)]
    out.append(f'(18 (1 {len(pairs):x} 4 5)(')
    out += [f'{new_pos[a] + 1:x} {new_pos[b] + 1:x}' for a, b in pairs]
    out.append('))')
    Path(path).write_text('\n'.join(out) + '\n')
    index = np.empty(nc, dtype=int)
    index[cell_new - 1] = np.arange(nc)
    return index.tolist()


@pytest.mark.parametrize('nx,ny,walls', [(8, 6, False), (7, 5, True), (32, 24, False)])
def test_generated_mesh_maps_to_the_identity(nx, ny, walls, tmp_path):
    from mesh_cas import write_cas
    write_cas(str(tmp_path / 'm.cas'), nx, ny, walls)
    info, err = mesh_info(tmp_path / 'm.cas')
    assert info is not None, err
    assert info[:3] == (nx, ny, int(walls)) and info[3] == list(range(nx * ny))


@pytest.mark.parametrize('nx,ny,walls,seed,mixed', [(8, 6, False, 1, False), (9, 7, True, 2, True),
                                                    (32, 24, False, 3, False)])
def test_any_numbering_is_mapped_back(nx, ny, walls, seed, mixed, tmp_path):
    want = write_permuted_cas(tmp_path / 'm.cas', nx, ny, walls, seed, mixed=mixed)
    info, err = mesh_info(tmp_path / 'm.cas')
    assert info is not None, err
    assert info[:3] == (nx, ny, int(walls)) and info[3] == want


@pytest.mark.parametrize('kw,msg', [
    (dict(bc_top=4), 'pressure inlet'),
    (dict(bc_top=10), 'velocity inlet'),
    (dict(dx=0.5), 'length 1'),
])
def test_meshes_the_gpu_path_does_not_take_are_rejected(kw, msg, tmp_path):
    write_permuted_cas(tmp_path / 'm.cas', 6, 5, True, 4, **kw)
    info, err = mesh_info(tmp_path / 'm.cas')
    assert info is None and msg in err, err


def test_reference_built_meshes_are_read(tmp_path):
    """The meshes written for the reference's own oracle builds, where present."""
    meshes = sorted((ROOT / 'oracle' / '_ref').glob('*/home/Mesh/*.cas'))
    if not meshes:
        pytest.skip('no reference build here')
    for m in meshes[:4]:
        info, err = mesh_info(m)
        assert info is not None, (m, err)
        assert info[3] == list(range(info[0] * info[1]))


@pytest.mark.gpu
def test_driver_writes_flowfield_cells_in_mesh_order(tmp_path):
    """dugks_run with a renumbered mesh of the reference's AC_Drop 32x24 case:
    the FlowField file at step 20 holds the reference's cell lines, reordered
    to the mesh's cell numbering."""
    import gzip
    gold = ROOT / 'tests' / 'golden' / 'flowfield' / 'ac_ff'
    index = write_permuted_cas(tmp_path / 'm.cas', 32, 24, False, 11)
    out = tmp_path / 'FlowField'
    subprocess.run([runner(), 'run', gold / 'Case.ark', '--out', out, '--steps', '20', '--mesh', tmp_path / 'm.cas'],
                   check=True, capture_output=True)
    f = next(gold.glob('step20Ma*.dat.gz'))
    ref = gzip.decompress(f.read_bytes()).decode().split('\n')
    got = (out / 'global' / f.name[:-3]).read_text().split('\n')
    assert len(got) == len(ref)
    cells, k = 32 * 24, 0
    while k < len(ref) and ref[k].startswith('(300'):
        assert got[k] == ref[k]
        body_ref, body_got = ref[k + 1:k + 1 + cells], got[k + 1:k + 1 + cells]
        assert body_got == [body_ref[c] for c in index]
        k += cells + 2
    assert k > 0
