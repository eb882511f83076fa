"""diffvg_gb300: a GB300-native (sm_103a) implementation of diffvg's render
hot path behind pydiffvg's API.

``import diffvg_gb300 as pydiffvg`` gives the scene classes (Circle,
Ellipse, Path, Polygon, Rect, ShapeGroup), paints (LinearGradient,
RadialGradient), PixelFilter, the device switches and RenderFunction with
pydiffvg's signatures, the SVG scene I/O (svg_to_scene, save_svg,
from_svg_path) and imwrite (PNG).  Rendering runs the hand-written CUDA kernels of
libdiffvg_gb300.so through its C ABI (include/diffvg_gb300.h); there is no
CPU fallback.
"""
from .device import set_use_gpu, get_use_gpu, set_device, get_device
from .shape import Circle, Ellipse, Path, Polygon, Rect, ShapeGroup, from_svg_path
from .color import LinearGradient, RadialGradient
from .pixel_filter import PixelFilter
from .diffvg import ShapeType, ColorType, FilterType
from .render_pytorch import (RenderFunction, OutputType, set_print_timing, clear_scene_cache, fuse_parameters,
                             set_fragment_cache, get_fragment_cache)
from .parse_svg import svg_to_scene
from .save_svg import save_svg
from .image import imwrite
from . import diffvg

__version__ = '0.1.0'
