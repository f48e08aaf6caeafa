"""Reader of the reference's serialization format (serialization.hpp:77-199),
for tests: header line, uint32 root count, per root the key, inner mask words,
per inner bit the leaf mask words and on-cell values."""
import struct

import numpy as np


def parse(data: bytes, value_bytes: int, inner_bits: int = 2, leaf_bits: int = 3):
    """(header str, coords int32 [n,3] sorted, values bytes [n] as uint8 rows)."""
    nl = data.index(b"\n")
    header = data[:nl].decode()
    p = nl + 1
    (nroots,) = struct.unpack_from("<I", data, p)
    p += 4
    iw = max((1 << (3 * inner_bits)) // 64, 1)
    lw = max((1 << (3 * leaf_bits)) // 64, 1)
    im, lm = (1 << inner_bits) - 1, (1 << leaf_bits) - 1
    coords, vals = [], []
    for _ in range(nroots):
        kx, ky, kz = struct.unpack_from("<iii", data, p)
        p += 12
        inner = struct.unpack_from(f"<{iw}Q", data, p)
        p += 8 * iw
        for a, word in enumerate(inner):
            while word:
                b = (word & -word).bit_length() - 1
                word &= word - 1
                ii = a * 64 + b
                xb = kx | ((ii & im) << leaf_bits)
                yb = ky | (((ii >> inner_bits) & im) << leaf_bits)
                zb = kz | (((ii >> (2 * inner_bits)) & im) << leaf_bits)
                leaf = struct.unpack_from(f"<{lw}Q", data, p)
                p += 8 * lw
                for c, lword in enumerate(leaf):
                    while lword:
                        cb = (lword & -lword).bit_length() - 1
                        lword &= lword - 1
                        ci = c * 64 + cb
                        coords.append((xb | (ci & lm), yb | ((ci >> leaf_bits) & lm),
                                       zb | ((ci >> (2 * leaf_bits)) & lm)))
                        vals.append(data[p:p + value_bytes])
                        p += value_bytes
    assert p == len(data), (p, len(data))
    xyz = np.array(coords, np.int32).reshape(-1, 3)
    order = np.lexsort((xyz[:, 2], xyz[:, 1], xyz[:, 0]))
    v = np.frombuffer(b"".join(vals), np.uint8).reshape(-1, value_bytes) if value_bytes else None
    return header, xyz[order], (v[order] if v is not None else None)
