"""The tile partition every SpMV of the engine runs over (sg_build_tiles, host only): each row
is covered exactly once, by the kind its length calls for, within the shape's limits, with
warp teams that follow the split (CPU only)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from samaya_gb300 import _native


def _tiles(ptr, cap, cap_rows, warp_min, split):
    lib = _native.load(build_if_missing=True)
    rows = len(ptr) - 1
    ptr = np.ascontiguousarray(ptr, dtype=np.int32)
    ntiles, nlong = ctypes.c_int(0), ctypes.c_int(0)
    p32 = ctypes.POINTER(ctypes.c_int32)
    rc = lib.sg_build_tiles(rows, ptr.ctypes.data_as(p32), cap, cap_rows, warp_min, split, None,
                            0, ctypes.byref(ntiles), ctypes.byref(nlong))
    assert rc in (0, -5)
    out = np.zeros(max(ntiles.value, 1) * 9, dtype=np.int32)
    rc = lib.sg_build_tiles(rows, ptr.ctypes.data_as(p32), cap, cap_rows, warp_min, split,
                            out.ctypes.data_as(p32), ntiles.value, ctypes.byref(ntiles),
                            ctypes.byref(nlong))
    assert rc == 0
    return out[:ntiles.value * 9].reshape(-1, 9), nlong.value


def _team_of(length, split):
    t = 1
    if split > 0:
        while t < 8 and length > t * split:
            t *= 2
    return t


@pytest.mark.parametrize("cap,cap_rows,split", [(256, 256, 0), (1024, 512, 0), (4096, 1024, 0),
                                                (4096, 1024, 300), (2048, 1024, 1000),
                                                (8192, 1024, 366)])
def test_tiles_cover_every_row_once(cap, cap_rows, split):
    rng = np.random.default_rng(cap + split)
    kinds = rng.integers(0, 6, size=3000)
    lengths = np.where(kinds == 0, 0, np.where(
        kinds <= 2, rng.integers(1, 33, size=3000), np.where(
            kinds == 3, rng.integers(33, 129, size=3000), np.where(
                kinds == 4, rng.integers(129, 4097, size=3000),
                rng.integers(4097, 20000, size=3000)))))
    lengths[rng.random(3000) < 0.9] //= 7  # mostly short, as sparse LPs are
    ptr = np.concatenate([[0], np.cumsum(lengths)])
    warp_min = 128
    tiles, nlong = _tiles(ptr, cap, cap_rows, warp_min, split)
    long_len = max(cap, warp_min)
    nxt = 0
    lrow_seen = []
    covered = 0
    i = 0
    while i < len(tiles):
        r0, r1, k0, k1, kind, team, seg, nseg, lrow = (int(v) for v in tiles[i])
        assert r0 == nxt, (i, r0, nxt)
        if kind == 1:
            length = lengths[r0]
            assert r1 == r0 + 1 and length > long_len
            assert nseg == (length + cap - 1) // cap
            for s in range(nseg):
                t = tiles[i + s]
                assert t[4] == 1 and t[0] == r0 and t[6] == s and t[7] == nseg and t[8] == lrow
                assert t[2] == ptr[r0] + s * cap and t[3] == min(ptr[r0 + 1], t[2] + cap)
                covered += int(t[3] - t[2])
            lrow_seen.append(lrow)
            i += nseg
        else:
            assert r1 > r0 and k0 == ptr[r0] and k1 == ptr[r1]
            seglen = lengths[r0:r1]
            if kind == 0:
                assert team == 1 and np.all(seglen <= warp_min)
                assert r1 - r0 <= cap_rows
                assert k1 - k0 <= cap or r1 - r0 == 1
            else:
                assert kind == 2
                assert np.all((seglen > warp_min) & (seglen <= long_len))
                assert team in (1, 2, 4, 8) and r1 - r0 <= 8 // team
                assert all(_team_of(int(x), split) == team for x in seglen)
            covered += k1 - k0
            i += 1
        nxt = r1
    assert nxt == len(lengths)
    assert covered == ptr[-1]
    assert lrow_seen == list(range(nlong))
    assert nlong == int(np.sum(lengths > long_len))


def test_build_tiles_argument_checks():
    lib = _native.load(build_if_missing=True)
    ptr = np.array([0, 3, 2], dtype=np.int32)  # decreasing
    n, nl = ctypes.c_int(0), ctypes.c_int(0)
    p32 = ctypes.POINTER(ctypes.c_int32)
    assert lib.sg_build_tiles(2, ptr.ctypes.data_as(p32), 256, 256, 128, 0, None, 0,
                              ctypes.byref(n), ctypes.byref(nl)) == -1
    ptr = np.array([0, 3, 5], dtype=np.int32)
    assert lib.sg_build_tiles(2, ptr.ctypes.data_as(p32), 0, 256, 128, 0, None, 0,
                              ctypes.byref(n), ctypes.byref(nl)) == -1
    assert lib.sg_build_tiles(2, ptr.ctypes.data_as(p32), 256, 256, 128, 0, None, 0,
                              ctypes.byref(n), ctypes.byref(nl)) == -5 and n.value == 1


def _group_tiles(ptr, neighbours, cap, cap_rows, warp_min, split):
    lib = _native.load(build_if_missing=True)
    rows = len(ptr) - 1
    ptr = np.ascontiguousarray(ptr, dtype=np.int32)
    nb = np.ascontiguousarray(neighbours, dtype=np.uint8)
    ntiles, nlong = ctypes.c_int(0), ctypes.c_int(0)
    p32 = ctypes.POINTER(ctypes.c_int32)
    p8 = ctypes.POINTER(ctypes.c_uint8)
    rc = lib.sg_build_group_tiles(rows, ptr.ctypes.data_as(p32), nb.ctypes.data_as(p8), cap,
                                  cap_rows, warp_min, split, None, 0, ctypes.byref(ntiles),
                                  ctypes.byref(nlong))
    assert rc in (0, -5)
    out = np.zeros(max(ntiles.value, 1) * 9, dtype=np.int32)
    rc = lib.sg_build_group_tiles(rows, ptr.ctypes.data_as(p32), nb.ctypes.data_as(p8), cap,
                                  cap_rows, warp_min, split, out.ctypes.data_as(p32),
                                  ntiles.value, ctypes.byref(ntiles), ctypes.byref(nlong))
    assert rc == 0
    return out[:ntiles.value * 9].reshape(-1, 9), nlong.value


@pytest.mark.parametrize("cap", [2048, 4096, 8192])
def test_row_groups_cover_runs_of_neighbour_rows(cap):
    """sg_build_group_tiles (the dual steps' partition with row groups): every row once; a
    kind-3 tile holds 8-32 consecutive rows longer than warp_min, each a neighbour of the next,
    its segments cover positions [0, longest row) in steps of the group segment length; the
    other rows are partitioned as sg_build_tiles would (kinds 0-2), and the counters of split
    rows and multi-segment groups are numbered in order."""
    rng = np.random.default_rng(cap)
    rows = 4000
    lengths = np.where(rng.random(rows) < 0.5, rng.integers(0, 100, size=rows),
                       rng.integers(129, 3000, size=rows))
    # Runs of neighbour rows of various lengths (some shorter than 8, some longer than 32).
    neighbours = np.zeros(rows, dtype=np.uint8)
    r = 0
    while r < rows:
        run = int(rng.integers(1, 70))
        if rng.random() < 0.6:
            end = min(rows, r + run)
            neighbours[r:end - 1] = 1
            # Mostly long rows inside a run, a few short ones breaking it.
            lengths[r:end] = np.where(rng.random(end - r) < 0.95,
                                      rng.integers(129, 3000, size=end - r), 50)
        r += run
    ptr = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    warp_min = 128
    tiles, nlong = _group_tiles(ptr, neighbours, cap, 1024, warp_min, 0)
    gp = max(128, (cap // 32) // 128 * 128)
    long_len = max(cap, warp_min)
    covered = np.zeros(int(ptr[-1]), dtype=np.int32)
    rows_seen = np.zeros(rows, dtype=np.int32)
    counters = []
    groups = 0
    i = 0
    while i < len(tiles):
        r0, r1, k0, k1, kind, team, seg, nseg, lrow = (int(v) for v in tiles[i])
        if kind == 3:
            g = r1 - r0
            assert 8 <= g <= 32
            assert np.all(lengths[r0:r1] > warp_min) and np.all(neighbours[r0:r1 - 1] == 1)
            maxlen = int(lengths[r0:r1].max())
            assert nseg == (maxlen + gp - 1) // gp
            for s in range(nseg):
                t = tiles[i + s]
                assert t[4] == 3 and t[0] == r0 and t[1] == r1 and t[6] == s and t[7] == nseg
                assert t[2] == s * gp and t[3] == min(maxlen, (s + 1) * gp)
                for q in range(r0, r1):
                    a, b = ptr[q] + t[2], min(ptr[q + 1], ptr[q] + t[3])
                    if b > a:
                        covered[a:b] += 1
            if nseg > 1:
                counters.append(lrow)
            rows_seen[r0:r1] += 1
            groups += 1
            i += nseg
        elif kind == 1:
            assert lengths[r0] > long_len
            for s in range(nseg):
                t = tiles[i + s]
                covered[t[2]:t[3]] += 1
            counters.append(lrow)
            rows_seen[r0] += 1
            i += nseg
        else:
            assert kind in (0, 2) and k0 == ptr[r0] and k1 == ptr[r1]
            if kind == 2:
                # A row group would have started inside a kind-2 tile: never.
                for q in range(r0 + 1, r1):
                    run = 1
                    while run < 32 and q + run < rows and neighbours[q + run - 1] and \
                            lengths[q + run] > warp_min:
                        run += 1
                    assert run < 8 or lengths[q] <= warp_min
            covered[k0:k1] += 1
            rows_seen[r0:r1] += 1
            i += 1
    assert np.all(rows_seen == 1)
    assert np.all(covered == 1)
    assert counters == list(range(nlong))
    assert groups > 10


def test_group_tiles_need_the_neighbours():
    lib = _native.load(build_if_missing=True)
    ptr = np.array([0, 3, 5], dtype=np.int32)
    n, nl = ctypes.c_int(0), ctypes.c_int(0)
    p32 = ctypes.POINTER(ctypes.c_int32)
    assert lib.sg_build_group_tiles(2, ptr.ctypes.data_as(p32), None, 256, 256, 128, 0, None, 0,
                                    ctypes.byref(n), ctypes.byref(nl)) == -1
