"""Index arithmetic of the two-phase ray update's mark phase, on the CPU.

The mark kernel (bonxai_gb300/csrc/bxg_mark.cuh) sets one bit per visited
cell in a leaf-blocked bitmap over a cube of leaves around the scan's origin:
block b = bx + S*(by + S*bz) of 16 words, bit getLeafIndex (x fastest,
bonxai.hpp:441-447) of the cell in its 8^3 leaf. A ray's first 8*NB + 1
cells go through a shared-memory copy of the (2 NB + 1)^3 leaves around the
origin's leaf, the rest straight to the bitmap; a block's touched flag sits at
a scattered bit (b * kTouchMul) mod 2^k. These tests restate that arithmetic
and check, for random rays walked as RayIterator does
(probabilistic_map.hpp:162-203, in its closed form):

* every cell k <= 8 NB of a ray lies inside the shared neighbourhood;
* the shared word of a near cell maps back to the same bitmap word and bit as
  the direct (far) mapping, so both routes set the bit getLeafIndex names;
* every cell of a ray whose end lies in the cube lies in the cube;
* the touched-bit permutation is a bijection whose inverse is the listed
  block.
"""
from __future__ import annotations

import numpy as np

K_TOUCH_MUL = 0x9E3779B1
K_TOUCH_INV = 0x0E8B2F51
M32 = 0xFFFFFFFF


def ray_cells(d, m):
    """Cells k = 0..m-1 of a ray with offset d (closed form of RayIterator)."""
    k = np.arange(m, dtype=np.int64)[:, None]
    a = np.abs(np.asarray(d, np.int64))[None, :]
    n = (2 * k * a + m) // (2 * m)
    return np.where(np.asarray(d)[None, :] < 0, -n, n)


def far_word(c, S):
    cx, cy, cz = c[:, 0], c[:, 1], c[:, 2]
    return ((cx >> 3) + S * (cy >> 3) + S * S * (cz >> 3)) * 16 + ((cy >> 2) & 1) + ((cz & 7) << 1)


def bit_of(c):
    return (c[:, 0] & 7) | ((c[:, 1] & 3) << 3)


def touched_mask(S):
    p = 32
    while p < S ** 3:
        p <<= 1
    return p - 1


def test_near_and_far_routes_set_the_leaf_index_bit():
    rng = np.random.default_rng(5)
    for NB in (2, 3):
        NS = 2 * NB + 1
        near = 8 * NB + 1
        for S, reach in ((2 * 6 + 1, 30), (2 * 20 + 1, 150)):
            HL = (S - 1) // 2
            checked = 0
            for _ in range(200):
                o = rng.integers(-3000, 3000, 3)
                x0 = ((o >> 3) - HL) * 8
                d = rng.integers(-reach, reach + 1, 3)
                m = int(np.abs(d).max())
                if m == 0:
                    continue
                e = o + d
                if np.any(e - x0 < 0) or np.any(e - x0 >= 8 * S):
                    continue
                cells = ray_cells(d, m) + (o - x0)  # cube-relative
                assert cells.min() >= 0 and cells.max() < 8 * S
                # reference: getLeafIndex bit of each cell in its leaf block
                li = (cells[:, 0] & 7) | ((cells[:, 1] & 7) << 3) | ((cells[:, 2] & 7) << 6)
                blk = (cells[:, 0] >> 3) + S * (cells[:, 1] >> 3) + S * S * (cells[:, 2] >> 3)
                want_w, want_b = blk * 16 + (li >> 5), li & 31
                got_w, got_b = far_word(cells, S), bit_of(cells)
                nl = ((o - x0) >> 3) - NB
                k = np.arange(m)
                sel = k < near
                u = cells[sel] - 8 * nl
                assert u.min() >= 0 and u.max() < 8 * NS  # inside the neighbourhood
                sw = (((u[:, 2] >> 3) * NS + (u[:, 1] >> 3)) * NS + (u[:, 0] >> 3)) * 16 + \
                    ((u[:, 1] >> 2) & 1) + ((u[:, 2] & 7) << 1)
                q = sw >> 4
                qb = (nl[0] + q % NS) + S * (nl[1] + (q // NS) % NS) + S * S * (nl[2] + q // (NS * NS))
                got_w = got_w.copy()
                got_w[sel] = qb * 16 + (sw & 15)
                assert np.array_equal(got_w, want_w) and np.array_equal(got_b, want_b)
                checked += 1
            assert checked > 100


def test_touched_permutation_is_inverted_by_the_list_pass():
    assert (K_TOUCH_MUL * K_TOUCH_INV) & M32 == 1
    for S in (1, 3, 9, 17, 33):
        mask = touched_mask(S)
        b = np.arange(S ** 3, dtype=np.uint64)
        t = (b * K_TOUCH_MUL) & M32 & mask
        assert len(np.unique(t)) == len(b)  # one bit per block
        assert t.max() < mask + 1
        back = (t * K_TOUCH_INV) & M32 & mask
        assert np.array_equal(back, b)
