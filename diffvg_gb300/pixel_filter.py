"""Pixel filter record (pydiffvg/pixel_filter.py:4-9).

``type`` is a FilterType (box, tent, parabolic, hann: filter.h:6-11; and
gaussian, which the reference lacks: a separable Gaussian of standard
deviation radius / 2, shifted to reach 0 at the edge of the support);
``radius`` a scalar tensor, differentiable.
"""
import torch


class PixelFilter:
    def __init__(self, type, radius=torch.tensor(0.5)):
        self.type = type
        self.radius = radius
