"""imwrite (PNG) on the CPU: the reference's preprocessing (normalise,
clamp, gamma on colour channels only, 8-bit) and a valid PNG file, read
back with a minimal decoder of the unfiltered 8-bit images it writes."""
import struct
import zlib

import numpy as np
import pytest
import torch

import diffvg_gb300 as dvg


def _read_png(path):
    data = open(path, 'rb').read()
    assert data[:8] == b'\x89PNG\r\n\x1a\n'
    i, idat, ihdr = 8, b'', None
    while i < len(data):
        n, = struct.unpack('>I', data[i:i + 4])
        kind, body = data[i + 4:i + 8], data[i + 8:i + 8 + n]
        crc, = struct.unpack('>I', data[i + 8 + n:i + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xffffffff
        if kind == b'IHDR':
            ihdr = struct.unpack('>IIBBBBB', body)
        elif kind == b'IDAT':
            idat += body
        i += 12 + n
    w, h, depth, ctype = ihdr[:4]
    c = {0: 1, 4: 2, 2: 3, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + w * c)
    assert depth == 8 and (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, c)


def test_imwrite_rgba_gamma_and_clamp(tmp_path):
    img = torch.rand(5, 7, 4) * 1.2 - 0.1
    f = str(tmp_path / 'sub' / 'a.png')
    dvg.imwrite(img, f, gamma=2.2)
    ref = np.clip(img.numpy(), 0, 1)
    ref[:, :, :3] = ref[:, :, :3] ** (1 / 2.2)
    assert np.array_equal(_read_png(f), (ref * 255).astype(np.uint8))


def test_imwrite_grey_normalised(tmp_path):
    img = np.linspace(2.0, 4.0, 12, dtype=np.float32).reshape(3, 4)
    f = str(tmp_path / 'g.png')
    dvg.imwrite(img, f, gamma=1.0, normalize=True)
    got = _read_png(f)
    assert got.shape == (3, 4, 1)
    assert got[0, 0, 0] == 0 and got[-1, -1, 0] == 255


def test_imwrite_other_formats_raise(tmp_path):
    with pytest.raises(NotImplementedError):
        dvg.imwrite(np.zeros((2, 2, 3), np.float32), str(tmp_path / 'x.jpg'))
