"""Device selection, mirroring pydiffvg/device.py.

The GB300 path has one device kind (CUDA).  ``set_use_gpu(False)`` is
accepted for source compatibility but rendering then raises: there is no CPU
fallback in this library.
"""
import torch

_use_gpu = True
_device = torch.device('cuda')


def set_use_gpu(v):
    global _use_gpu, _device
    _use_gpu = bool(v)
    if not _use_gpu:
        _device = torch.device('cpu')
    elif _device.type != 'cuda':
        _device = torch.device('cuda')


def get_use_gpu():
    return _use_gpu


def set_device(d):
    global _device, _use_gpu
    _device = torch.device(d)
    _use_gpu = _device.type == 'cuda'


def get_device():
    return _device
