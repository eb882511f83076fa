"""The CUDA path (through the C ABI) against the reference at the full sizes
of the three plain-method workloads: the single circle with its MSE loss
(256x256, 2x2 spp), the stroke-heavy scene (512x512, 2048 open cubic paths,
2x2 spp) and the fill-heavy prefiltered scene (1024x1024, 512 closed paths
with gradient fills, 1 spp): tests/golden/full_*.npz."""
import pytest

import full_golden_check as fg
import golden_util as gu

pytestmark = pytest.mark.gpu


def _render(packed, params, w, h, nsx, nsy, seed, d_image=None):
    import native_util as nu
    if d_image is None:
        return nu.render(packed, params, w, h, nsx, nsy, seed)['image']
    return nu.render(packed, params, w, h, nsx, nsy, seed, d_out=d_image)['d_params']


@pytest.mark.parametrize('name', gu.full_names())
def test_cuda_matches_reference_full_size(name):
    fg.check(name, _render)
