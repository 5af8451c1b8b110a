"""The staged kernel's copy segments (lbm_stage_segments, the host list the kernel's bulk copies
follow), checked on the CPU: staging a tile by those segments and reading each cell's populations at
the staged kernel's positions gives exactly the pull sources x - c_q of the double-buffer step
(src/lbm/kernels/ops/load_and_store.mojo:164-221), with the periodic wrap, for every lattice and
stageable tile shape; the segments cover each stage byte once, stay inside the source tile's
population block and are 16-byte aligned."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from mojo_lbm_gb300 import _capi
from mojo_lbm_gb300.lattice import get_lattice

T = 256


def segments(lattice_id: int, tile, esz: int):
    lib = _capi.lib()
    out = np.zeros(4 * 4096, np.uint32)
    sb = C.c_uint32(0)
    n = lib.lbm_stage_segments(lattice_id, *tile, esz, out.ctypes.data, 4096, C.byref(sb))
    assert n <= 4096
    return out[:4 * n].reshape(n, 4).astype(np.int64), int(sb.value)


def stage_regions(dirs):
    sizes = [T if c[0] == 0 else 2 * T for c in dirs]
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)


CASES = [(lat, tile, esz) for lat, tiles in
         {0: [(16, 16, 1), (8, 32, 1), (32, 8, 1), (4, 64, 1)],
          1: [(8, 8, 4), (16, 4, 4), (4, 8, 8), (8, 4, 8), (32, 8, 1)],
          2: [(8, 8, 4), (4, 8, 8), (16, 16, 1)]}.items()
         for tile in tiles for esz in (2, 4)]


@pytest.mark.parametrize("lat,tile,esz", CASES, ids=[f"{c[0]}-{'x'.join(map(str, c[1]))}-{c[2]}" for c in CASES])
def test_stage_segments_reproduce_the_pull(lat, tile, esz):
    segs, stage_bytes = segments(lat, tile, esz)
    if tile[0] * esz % 16:
        assert len(segs) == 0 and stage_bytes == 0  # rows shorter than 16 bytes are not staged
        return
    L = get_lattice(lat)
    dirs = np.asarray(L.directions, np.int64)
    Q, D = len(dirs), L.D
    dirs3 = np.zeros((Q, 3), np.int64)
    dirs3[:, :D] = dirs
    reg = stage_regions(dirs3)
    assert stage_bytes == reg[-1] * esz
    # the segments: aligned, inside the source block, covering the stage once
    src, dst, nbytes, nbr = segs.T
    assert (dst % 16 == 0).all() and (nbytes % 16 == 0).all() and (nbytes > 0).all()
    assert ((src * esz) % 16 == 0).all() and (src >= 0).all() and (src * esz + nbytes <= Q * T * esz).all()
    assert ((nbr >= 0) & (nbr < 27)).all()
    cover = np.zeros(stage_bytes, np.int64)
    for d, b in zip(dst, nbytes):
        cover[d:d + b] += 1
    assert (cover == 1).all()

    tx, ty, tz = tile
    shape = (2 * tx, 3 * ty, (2 * tz) if D == 3 else 1)  # several tiles per axis; x pairs wrap onto each other
    for grid_shape in (shape, (tx, ty, tz)):             # and a single tile, every neighbour itself
        nx, ny, nz = grid_shape
        ntx, nty, ntz = nx // tx, ny // ty, nz // tz
        N = nx * ny * nz
        f = np.arange(Q * N, dtype=np.int64)  # element e holds e

        def element(x, y, z, q):
            bx, lx = divmod(x, tx)
            by, ly = divmod(y, ty)
            bz, lz = divmod(z, tz)
            return (lx + tx * (ly + ty * lz)) + T * (q + Q * (bx + ntx * (by + nty * bz)))

        for tid in range(ntx * nty * ntz):
            byz, bx = divmod(tid, ntx)
            bz, by = divmod(byz, nty)
            stage = np.full(reg[-1], -1, np.int64)
            for s, d, b, code in segs:
                ox, oy, oz = code % 3 - 1, (code // 3) % 3 - 1, code // 9 - 1
                nt = ((bx + ox) % ntx) + ntx * (((by + oy) % nty) + nty * ((bz + oz) % ntz))
                n = b // esz
                stage[d // esz:d // esz + n] = f[nt * T * Q + s:nt * T * Q + s + n]
            for t in range(T):
                lx, rest = t % tx, t // tx
                ly, lz = rest % ty, rest // ty
                x, y, z = bx * tx + lx, by * ty + ly, bz * tz + lz
                bm = t - 1 if lx >= 1 else t + T + tx - 1
                bp = t + 1 if lx + 2 <= tx else t + T - tx + 1
                for q in range(Q):
                    cx, cy, cz = dirs3[q]
                    b = t if cx == 0 else (bm if cx > 0 else bp)
                    want = element((x - cx) % nx, (y - cy) % ny, (z - cz) % nz, q)
                    assert stage[reg[q] + b] == want, (tid, t, q)


def test_unstageable_shapes():
    assert segments(1, (1, 16, 16), 2)[0].shape[0] == 0
    assert segments(1, (4, 8, 8), 2)[0].shape[0] == 0    # 8-byte rows of Float16C
    assert segments(1, (4, 8, 8), 4)[0].shape[0] > 0     # 16-byte rows of float32
