"""Fluent-style ``.cas`` writer for uniform Cartesian meshes (test infrastructure).

The reference solver reads its mesh from ``$HOME/Mesh/<name>.cas``
(Ark/Cpp/Mesh/MeshConstruct.cpp:69-123) and ships no mesh, so the oracle
build writes one with this module.  The text layout is the subset that the
reference parser accepts:

* a header line whose last non-blank character is ``(`` opens a body
  (Ark/Cpp/Mesh/MeshConstruct.cpp:16-35); declaration lines without a body
  allocate the arrays (Ark/Lib/MeshConstructFunc.h:27-54);
* ``(10 …)`` nodes as decimal ``x y`` pairs, ``(12 …)`` cells declared as
  quads by the trailing element type 3 (Ark/Lib/MeshConstructFunc.h:83-112),
  ``(13 (zone first last bc_type 2)(`` faces as four hex ids
  ``n0 n1 c0 c1`` (Ark/Lib/MeshConstructFunc.h:181-215) and ``(18 …)``
  periodic face pairs (Ark/Lib/MeshConstructFunc.h:344-358);
* ``bc_type`` 2 = interior, 12/8 = periodic/periodic-shadow, 3 = wall
  (Ark/Lib/MeshConstructFunc.h:216-275);
* the normal ``(dy, -dx)/|S|`` of ``n0 -> n1`` points from owner to
  neighbour (Ark/Cpp/Mesh/Face_2D.cpp:339-345, checked by
  Ark/Cpp/Mesh/MeshCartesian.cpp:131-248).

Only this module's own face order is used by the product's geometry builder
(``mpdugks_gb300`` replicates it in memory), so the two agree cell by cell.

Zones: interior 3, left 4, right 5, bottom 6, top 7 (the zone numbers of the
reference's sample ``FlowField/Case.ark``).
"""
from __future__ import annotations

import os


def cartesian_faces(nx: int, ny: int, y_walls: bool):
    """Return the face list in file order as (bc_type, zone, n0, n1, c0, c1).

    Node (i, j) has 1-based id j*(nx+1)+i+1, cell (i, j) has id j*nx+i+1,
    and c1 = 0 marks a boundary face.
    """
    def nid(i, j):
        return j * (nx + 1) + i + 1

    def cid(i, j):
        return j * nx + i + 1

    faces = []
    # interior x-faces (normal +x): owner (i, j), neighbour (i+1, j)
    for j in range(ny):
        for i in range(nx - 1):
            faces.append((2, 3, nid(i + 1, j), nid(i + 1, j + 1), cid(i, j), cid(i + 1, j)))
    # interior y-faces (normal +y): owner (i, j), neighbour (i, j+1)
    for j in range(ny - 1):
        for i in range(nx):
            faces.append((2, 3, nid(i + 1, j + 1), nid(i, j + 1), cid(i, j), cid(i, j + 1)))
    # left (normal -x) and right (normal +x) boundaries, periodic in x
    for j in range(ny):
        faces.append((12, 4, nid(0, j + 1), nid(0, j), cid(0, j), 0))
    for j in range(ny):
        faces.append((8, 5, nid(nx, j), nid(nx, j + 1), cid(nx - 1, j), 0))
    # bottom (normal -y) and top (normal +y) boundaries
    bb, bt = (3, 3) if y_walls else (12, 8)
    for i in range(nx):
        faces.append((bb, 6, nid(i, 0), nid(i + 1, 0), cid(i, 0), 0))
    for i in range(nx):
        faces.append((bt, 7, nid(i + 1, ny), nid(i, ny), cid(i, ny - 1), 0))
    return faces


def write_cas(path: str, nx: int, ny: int, y_walls: bool = False,
              dx: float = 1.0, dy: float = 1.0, x0: float = 0.0, y0: float = 0.0) -> None:
    faces = cartesian_faces(nx, ny, y_walls)
    nnodes = (nx + 1) * (ny + 1)
    ncells = nx * ny
    nfaces = len(faces)
    out = []
    w = out.append
    w('(0 "uniform Cartesian mesh written by oracle/ref/mesh_cas.py")')
    w('(2 2)')
    w(f'(10 (0 1 {nnodes:x} 0 2))')
    w(f'(12 (0 1 {ncells:x} 0))')
    w(f'(13 (0 1 {nfaces:x} 0))')
    w(f'(10 (1 1 {nnodes:x} 1 2)(')
    for j in range(ny + 1):
        y = y0 + j * dy
        for i in range(nx + 1):
            w(f'{x0 + i * dx!r} {y!r}')
    w('))')
    w(f'(12 (2 1 {ncells:x} 1 3))')
    # one (13 …) section per (zone, bc_type) run, in file order
    start = 0
    while start < nfaces:
        bc, zone = faces[start][0], faces[start][1]
        end = start
        while end < nfaces and faces[end][0] == bc and faces[end][1] == zone:
            end += 1
        w(f'(13 ({zone:x} {start + 1:x} {end:x} {bc:x} 2)(')
        for f in faces[start:end]:
            w(f'{f[2]:x} {f[3]:x} {f[4]:x} {f[5]:x}')
        w('))')
        start = end
    # periodic pairs: left j <-> right j, and bottom i <-> top i when periodic in y
    first_left = (nx - 1) * ny + nx * (ny - 1) + 1
    first_right = first_left + ny
    first_bottom = first_right + ny
    first_top = first_bottom + nx
    pairs = [(first_left + j, first_right + j) for j in range(ny)]
    if not y_walls:
        pairs += [(first_bottom + i, first_top + i) for i in range(nx)]
    w(f'(18 (1 {len(pairs):x} 4 5)(')
    for a, b in pairs:
        w(f'{a:x} {b:x}')
    w('))')
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, 'w') as fh:
        fh.write('\n'.join(out) + '\n')


if __name__ == '__main__':
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument('path')
    ap.add_argument('nx', type=int)
    ap.add_argument('ny', type=int)
    ap.add_argument('--walls', action='store_true')
    a = ap.parse_args()
    write_cas(a.path, a.nx, a.ny, a.walls)
