"""The CPU oracle against the reference at the full sizes of the three
plain-method workloads (single circle with its MSE loss, stroke-heavy 512x512,
fill-heavy prefiltered 1024x1024): tests/golden/full_*.npz."""
import os

import pytest

import full_golden_check as fg
import golden_util as gu
import oracle

THREADS = max(1, min(16, os.cpu_count() or 1))


def _render(packed, params, w, h, nsx, nsy, seed, d_image=None):
    if d_image is None:
        return oracle.render(packed, params, w, h, nsx, nsy, seed, num_threads=THREADS)['image']
    return oracle.render(packed, params, w, h, nsx, nsy, seed, forward=False, d_image=d_image,
                         num_threads=THREADS)['d_params']


@pytest.mark.parametrize('name', gu.full_names())
def test_oracle_matches_reference_full_size(name):
    fg.check(name, _render)
