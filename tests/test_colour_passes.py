"""Race freedom of the in-place red-black passes, checked on the index arithmetic the kernels
use (no GPU): a colour pass writes only cells of its colour and reads only the opposite colour
plus the cell itself, so no cell a pass writes is read by another thread of the same pass; and
each kernel's thread mapping covers every interior cell of the colour exactly once.

Mappings (kernels_pressure.cu / stage_bodies.cuh body_sweep; kernels_group.cu grouped passes):
  block:      x = 1 + ((1 + y + z + c) & 1) + 2 * (bx * 64 + tx), y = 1 + by * 4 + ty, z = 1 + bz
  flattened:  f = tile * 256 + tid in a plane, H = (nx - 1) // 2, y = 1 + f // H,
              x = 1 + 2 * (f % H) + ((1 + y + z + c) & 1)
  z-slab:     the flattened (k, y) column walks z0..z1, x alternating between xa and xa + 1
"""
import itertools

import numpy as np
import pytest

SIZES = [(3, 3, 3), (13, 10, 11), (32, 32, 32), (70, 9, 5), (5, 66, 7)]


def _interior_colour(nx, ny, nz, c):
    return {(x, y, z) for z in range(1, nz - 1) for y in range(1, ny - 1) for x in range(1, nx - 1)
            if (x + y + z) % 2 == c}


def _block_mapping(nx, ny, nz, c):
    half = (nx - 2 + 1) // 2
    out = []
    for z in range(1, nz - 1):
        for by in range((ny - 2 + 3) // 4):
            for ty in range(4):
                y = 1 + by * 4 + ty
                for bx in range((half + 63) // 64):
                    for tx in range(64):
                        x = 1 + ((1 + y + z + c) & 1) + 2 * (bx * 64 + tx)
                        if x <= nx - 2 and y <= ny - 2:
                            out.append((x, y, z))
    return out


def _flattened_mapping(nx, ny, nz, c, zslab):
    H = (nx - 1) // 2
    rows = ny - 2
    tpp = -(-(H * rows) // 256) if nx > 2 and ny > 2 else 0
    out = []
    slabs = -(-(nz - 2) // zslab) if nz > 2 else 0
    for local in range(tpp * slabs):
        z0 = 1 + (local // tpp) * zslab
        z1 = min(z0 + zslab, nz - 1)
        for tid in range(256):
            f = (local % tpp) * 256 + tid
            if f >= H * rows:
                continue
            y = 1 + f // H
            xa = 1 + 2 * (f % H)
            par = (1 + y + z0 + c) & 1
            for z in range(z0, z1):
                if xa + par <= nx - 2:
                    out.append((xa + par, y, z))
                par ^= 1
    return out


@pytest.mark.parametrize("nx,ny,nz", SIZES)
@pytest.mark.parametrize("c", [0, 1])
def test_mappings_cover_the_colour_once(nx, ny, nz, c):
    want = _interior_colour(nx, ny, nz, c)
    for cells in (_block_mapping(nx, ny, nz, c), _flattened_mapping(nx, ny, nz, c, 1),
                  _flattened_mapping(nx, ny, nz, c, 4), _flattened_mapping(nx, ny, nz, c, 7)):
        assert len(cells) == len(set(cells)) == len(want)
        assert set(cells) == want


@pytest.mark.parametrize("nx,ny,nz", SIZES)
@pytest.mark.parametrize("c", [0, 1])
def test_write_set_disjoint_from_read_set(nx, ny, nz, c):
    writes = _interior_colour(nx, ny, nz, c)
    reads = set()
    for (x, y, z) in writes:
        for dx, dy, dz in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
            reads.add((x + dx, y + dy, z + dz))
    assert not (writes & reads)
    # the reads stay inside the allocated cell range [0, n-1]
    a = np.array(sorted(reads)) if reads else np.zeros((0, 3), int)
    if len(a):
        assert a.min() >= 0 and (a.max(axis=0) <= np.array([nx - 1, ny - 1, nz - 1])).all()
