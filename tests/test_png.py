"""PNG writer of the package (no GPU): the file decodes to the image written."""
import struct
import zlib

import numpy as np


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(kind + body) & 0xFFFFFFFF
        chunks.setdefault(kind, b"")
        chunks[kind] += body
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    raw = zlib.decompress(chunks[b"IDAT"])
    rows = [raw[y * (1 + 4 * w):(y + 1) * (1 + 4 * w)] for y in range(h)]
    assert all(r[0] == 0 for r in rows) and depth == 8 and ctype == 6 and b"IEND" in chunks
    return np.frombuffer(b"".join(r[1:] for r in rows), dtype=np.uint8).reshape(h, w, 4)


def test_png_round_trip(ifl, tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, size=(37, 53, 4), dtype=np.uint8)
    path = str(tmp_path / "frame.png")
    ifl.write_png(path, img)
    assert np.array_equal(_read_png(path), img)
