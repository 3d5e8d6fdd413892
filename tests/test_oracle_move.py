"""moveParticle known answers, restating share/picongpu/unit/MoveParticle.cpp:98-258.

Supercell 8x8x4 (param/memory.param:51); localCellIdx linearised x fastest.
"""
import numpy as np
import pytest

G = dict(nx=16, ny=16, nz=8, sx=8, sy=8, sz=4, dx=1, dy=1, dz=1, dt=0.5, c=1, eps0=1)
EPS = np.finfo(np.float32).eps


def close(a, b):
    return np.all(np.abs(np.asarray(a, np.float32) - np.asarray(b, np.float32)) <= 100 * EPS)


def test_unchanged_position(orc):
    pos, lc, mm, _ = orc.move_particle(G, [0, 0, 0], 0)
    assert close(pos, [0, 0, 0]) and lc == 0 and mm == 1


@pytest.mark.parametrize("i", [0, 1, 2])
def test_moves_trivially_inside_cell(orc, i):
    p = [0.0, 0.0, 0.0]
    p[i] = 0.42
    pos, lc, mm, _ = orc.move_particle(G, p, 0)
    assert close(pos, p) and lc == 0 and mm == 1


@pytest.mark.parametrize("i,expected", [(0, 1), (1, 8), (2, 64)])
def test_moves_out_of_cell_positive(orc, i, expected):
    p = [0.0, 0.0, 0.0]
    p[i] = 1.1
    pos, lc, mm, _ = orc.move_particle(G, p, 0)
    e = [0.0, 0.0, 0.0]
    e[i] = 0.1
    assert close(pos, e) and lc == expected and mm == 1


@pytest.mark.parametrize("i", [0, 1, 2])
def test_moves_out_of_cell_negative(orc, i):
    last = 8 * 8 * 4 - 1
    expected = [last - 1, last - 8, 191][i]
    p = [0.0, 0.0, 0.0]
    p[i] = -0.3
    pos, lc, mm, _ = orc.move_particle(G, p, last)
    e = [0.0, 0.0, 0.0]
    e[i] = 0.7
    assert close(pos, e) and lc == expected and mm == 1


def test_moves_diagonally(orc):
    pos, lc, mm, _ = orc.move_particle(G, [1.4, 1.6, 0.0], 0)
    assert close(pos, [0.4, 0.6, 0.0]) and lc == 9 and mm == 1


def test_moves_out_of_supercell(orc):
    pos, lc, mm, d = orc.move_particle(G, [-0.9, 0.0, 0.0], 0)
    assert close(pos, [0.1, 0, 0]) and lc == 7 and mm == 3 and list(d) == [-1, 0, 0]


def test_rounding_near_zero(orc):
    pos, lc, mm, _ = orc.move_particle(G, [-EPS / 4, 0.0, 0.0], 0)
    assert pos[0] == 0.0 and lc == 0 and mm == 1


@pytest.mark.parametrize("d", [(1, 0, 0), (0, -1, 0), (0, 0, 1), (1, 1, 1), (-1, -1, -1), (1, -1, 0)])
def test_multimask_encodes_direction(orc, d):
    """multiMask = 1 + sum(dir_i' * 3^i) with dir' = 2 for -1 (MoveParticle.hpp:138-149)."""
    scs = (8, 8, 4)
    lc3 = [scs[a] - 1 if d[a] > 0 else 0 for a in range(3)]
    lcell = lc3[0] + 8 * (lc3[1] + 8 * lc3[2])
    p = [0.5 + 0.7 * d[a] for a in range(3)]
    pos, lc, mm, dd = orc.move_particle(G, p, lcell)
    expect = 1 + sum((2 if d[a] == -1 else d[a]) * 3 ** a for a in range(3))
    assert mm == expect and list(dd) == list(d)
    new3 = [(lc3[a] + d[a]) % scs[a] for a in range(3)]
    assert lc == new3[0] + 8 * (new3[1] + 8 * new3[2])
