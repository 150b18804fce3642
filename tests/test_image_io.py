"""PNG writer (SavePNG / SavePNG16 / SavePNG16Alpha replacement) and string settings.

The files are decoded here with Python's zlib and checked chunk by chunk (CRC-32 of every
chunk, IHDR fields, filter bytes, the samples in big-endian order)."""
import ctypes
import struct
import zlib

import numpy as np
import pytest

import mandelbulber_gb300 as mb


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF, typ
        chunks.append((typ, body))
        pos += 12 + n
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    raw = zlib.decompress(chunks[1][1])
    ch = 4 if ctype == 6 else 3
    bps = depth // 8
    row = w * ch * bps
    rows = []
    for y in range(h):
        line = raw[y * (row + 1):(y + 1) * (row + 1)]
        assert line[0] == 0
        rows.append(line[1:])
    buf = b"".join(rows)
    arr = np.frombuffer(buf, dtype=">u2" if depth == 16 else np.uint8).reshape(h, w, ch)
    return (w, h, depth, ctype, comp, filt, inter), arr


@pytest.mark.parametrize("depth,channels,shape", [(8, 3, (5, 7)), (16, 3, (33, 300)), (16, 4, (260, 257))])
def test_png_round_trip(mblib, tmp_path, depth, channels, shape):
    rng = np.random.default_rng(depth * 10 + channels)
    h, w = shape
    dt = np.uint8 if depth == 8 else np.uint16
    img = rng.integers(0, 2 ** depth, (h, w, channels), dtype=np.uint64).astype(dt)
    path = str(tmp_path / "x.png").encode()
    assert mblib.mbgb_write_png(path, w, h, depth, channels, img.ctypes.data) == 0
    hdr, arr = _read_png(path)
    assert hdr == (w, h, depth, 6 if channels == 4 else 2, 0, 0, 0)
    np.testing.assert_array_equal(arr.astype(np.uint64), img.astype(np.uint64))


def test_png_rejects_bad_arguments(mblib, tmp_path):
    img = np.zeros((2, 2, 3), np.uint8)
    assert mblib.mbgb_write_png(str(tmp_path / "y.png").encode(), 2, 2, 12, 3, img.ctypes.data) != 0
    assert mblib.mbgb_write_png(b"/nonexistent-dir/z.png", 2, 2, 8, 3, img.ctypes.data) != 0


def test_settings_string(mblib, tmp_path):
    f = tmp_path / "s.fract"
    f.write_text("file_destination images/image;\nimage_width 320;\nfile_keyframes keyframes/key;\n")
    out = ctypes.create_string_buffer(1000)
    assert mblib.mbgb_settings_string(None, str(f).encode(), None, 0, b"file_destination", out, 1000) == 0
    assert out.value == b"images/image"
    ov = (ctypes.c_char_p * 1)(b"file_destination=other/frame")
    assert mblib.mbgb_settings_string(None, str(f).encode(), ov, 1, b"file_destination", out, 1000) == 0
    assert out.value == b"other/frame"
    assert mblib.mbgb_settings_string(None, str(f).encode(), None, 0, b"file_animation_path", out, 1000) != 0
