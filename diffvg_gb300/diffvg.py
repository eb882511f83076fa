"""Enumerations of the native diffvg module, for code written against it.

pydiffvg code refers to ``diffvg.ShapeType``, ``diffvg.ColorType`` and
``diffvg.FilterType`` (reference: diffvg.cpp:1683-1687, 1710-1713, 1764-1768).
``from diffvg_gb300 import diffvg`` provides the same names with the same
integer values, which are also the values of the C ABI (include/diffvg_gb300.h).
"""
from enum import IntEnum


class ShapeType(IntEnum):
    circle = 0
    ellipse = 1
    path = 2
    rect = 3


class ColorType(IntEnum):
    constant = 0
    linear_gradient = 1
    radial_gradient = 2


class FilterType(IntEnum):
    box = 0
    tent = 1
    parabolic = 2
    hann = 3
    gaussian = 4  # not in the reference: separable Gaussian, sigma = radius / 2, zero at the support's edge
