"""The driver-facing entry points that run without a GPU: the smoke check's comparison."""
import numpy as np

import __graft_entry__ as entry


def test_smoke_comparison_handles_zero_components():
    r = np.array([[1.0, 2.0, 0.0], [3.0, -4.0, 0.0]])
    assert entry.normwise_max(r.copy(), r) == 0.0
    a = r.copy()
    a[1, 1] += 4e-12
    assert abs(entry.normwise_max(a, r) - 1e-12) < 1e-15
    a = r.copy()
    a[0, 2] = 1e-3          # a component that must stay zero and does not
    assert entry.normwise_max(a, r) == 1e-3
    a = r.copy()
    a[0, 0] = np.nan
    assert np.isnan(entry.normwise_max(a, r))
