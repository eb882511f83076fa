"""__graft_entry__.smoke(): one small forward + backward on cuda:0 checked
against the oracle."""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu


def test_smoke_runs():
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__
    __graft_entry__.smoke()
