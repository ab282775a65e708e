"""Host-side logic of the GPU phasing module that needs no GPU: the Gaussian taps handed to
the filter kernels reproduce scipy.ndimage.gaussian_filter (cmtip/phasing/phase.py:160-161,
186-187), and the module exposes the reference's function names."""
import numpy as np
import pytest
from scipy.ndimage import gaussian_filter

from cmtip_gb300 import phasing


@pytest.mark.parametrize("sigma", [0.5, 1.0, 1.5, 2.0])
@pytest.mark.parametrize("mode", ["wrap", "constant"])
def test_gauss_taps_match_ndimage(sigma, mode):
    # one axis pass with the taps (outermost first, as the kernel adds them) equals ndimage
    w, r = phasing._gauss_taps(sigma, 2.0)
    assert r == int(2.0 * sigma + 0.5) and w.shape == (2 * r + 1,) and abs(w.sum() - 1.0) < 1e-15
    rng = np.random.default_rng(1)
    x = rng.random(23) ** 2
    n = x.size

    def sample(p):
        if mode == "wrap":
            return x[p % n]
        return x[p] if 0 <= p < n else 0.0

    out = np.empty(n)
    for i in range(n):
        t = sample(i) * w[r]
        for d in range(r, 0, -1):
            t += (sample(i - d) + sample(i + d)) * w[r + d]
        out[i] = t
    ref = gaussian_filter(x, sigma=sigma, mode=mode, truncate=2)
    assert np.array_equal(out, ref)


def test_reference_names_exported():
    for name in ("center_of_mass", "recenter", "create_support_", "ER_loop", "HIO_loop", "ER", "HIO",
                 "step_phase", "shrink_wrap", "phase"):
        assert callable(getattr(phasing, name))
    assert phasing.DEFAULT_PREC == 32
