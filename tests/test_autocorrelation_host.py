"""The autocorrelation solve's host-side steps on CPU, against the reference's own outputs:
the Fourier antisupport mask (autocorrelation.py:66-85)."""
import numpy as np

from cmtip_gb300 import autocorrelation


def test_antisupport_matches_reference_fixture(golden):
    g = golden("autocorrelation")
    for m in (9, 21, 22):  # odd and even grids
        mask = autocorrelation.gen_F_antisupport(m)
        assert mask.shape == (m,) * 3 and mask.dtype == bool
        assert np.array_equal(mask, g[f"anti{m}"])
    # the corners lie outside the pi-ball, the centre inside
    mask = autocorrelation.gen_F_antisupport(21)
    assert mask[0, 0, 0] and not mask[10, 10, 10]
