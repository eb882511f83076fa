"""imwrite(img, filename, gamma=2.2, normalize=False) with pydiffvg's
behaviour (pydiffvg/image.py): optional min-max normalisation, clamping to
[0, 1], gamma on the colour channels (not alpha), 8-bit quantisation.

The reference writes through scikit-image; here PNG files are encoded
directly (8-bit greyscale, grey + alpha, RGB or RGBA by channel count, no
filtering, zlib-compressed) and other formats raise NotImplementedError.
"""
import os
import struct
import zlib

import numpy as np

__all__ = ['imwrite']

_COLOR_TYPE = {1: 0, 2: 4, 3: 2, 4: 6}   # channels -> PNG colour type


def _chunk(kind, data):
    body = kind + data
    return struct.pack('>I', len(data)) + body + struct.pack('>I', zlib.crc32(body) & 0xffffffff)


def _png_bytes(pixels):
    """8-bit H x W x C array (C in 1..4) -> PNG file contents."""
    h, w, c = pixels.shape
    rows = np.concatenate([np.zeros((h, 1), np.uint8), pixels.reshape(h, w * c)], axis=1)  # filter type 0
    ihdr = struct.pack('>IIBBBBB', w, h, 8, _COLOR_TYPE[c], 0, 0, 0)
    return (b'\x89PNG\r\n\x1a\n' + _chunk(b'IHDR', ihdr) + _chunk(b'IDAT', zlib.compress(rows.tobytes(), 6)) +
            _chunk(b'IEND', b''))


def imwrite(img, filename, gamma=2.2, normalize=False):
    directory = os.path.dirname(filename)
    if directory != '' and not os.path.exists(directory):
        os.makedirs(directory)
    if not isinstance(img, np.ndarray):
        img = img.detach().cpu().numpy()
    if normalize:
        rng = np.max(img) - np.min(img)
        if rng > 0:
            img = (img - np.min(img)) / rng
    img = np.clip(img, 0.0, 1.0)
    if img.ndim == 2:
        img = np.expand_dims(img, 2)
    img[:, :, :3] = np.power(img[:, :, :3], 1.0 / gamma)
    pixels = (img * 255).astype(np.uint8)
    if not filename.lower().endswith('.png'):
        raise NotImplementedError('imwrite: only PNG files are written here (%s)' % filename)
    if pixels.shape[2] not in _COLOR_TYPE:
        raise ValueError('imwrite: 1 to 4 channels expected, got %d' % pixels.shape[2])
    with open(filename, 'wb') as f:
        f.write(_png_bytes(np.ascontiguousarray(pixels)))
