"""Pixel filter record (pydiffvg/pixel_filter.py:4-9).

``type`` is a FilterType (box, tent, parabolic, hann: filter.h:6-11);
``radius`` a scalar tensor, differentiable.
"""
import torch


class PixelFilter:
    def __init__(self, type, radius=torch.tensor(0.5)):
        self.type = type
        self.radius = radius
