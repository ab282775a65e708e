"""The alignment's host-side steps on CPU: pixel weights (align.py:11-24, against the
reference's own outputs) and the reference-orientation set (align.py:96-111)."""
import numpy as np

from cmtip_gb300 import alignment, geometry


def test_generate_weights_match_reference_fixture(golden):
    g = golden("alignment")
    for order, key in ((0, "w0"), (-2, "w2"), (1, "w1")):
        w = alignment.generate_weights(g["ppr"], order)
        assert np.allclose(w, g[key], rtol=1e-12, atol=0)
        assert np.isclose(w.sum(), 1.0, rtol=1e-12)


def test_reference_orientations_rounding_and_splicing():
    # n_ref rounds up to a multiple of nbatches; uniform quaternions as float32
    refs = alignment.reference_orientations(101, nbatches=4)
    assert refs.shape == (104, 4) and refs.dtype == np.float32
    assert np.array_equal(refs, geometry.uniform_quaternions(104).astype(np.float32))
    # true orientations replace the tail, then the set is shuffled (np.random, as the reference)
    true = geometry.random_quaternions(7, np.random.default_rng(4)).astype(np.float32)
    np.random.seed(0)
    spliced = alignment.reference_orientations(50, true_orientations=true)
    assert spliced.shape == (50, 4)
    kept = geometry.uniform_quaternions(50).astype(np.float32)[:43]
    rows = {tuple(r) for r in spliced}
    assert rows == {tuple(r) for r in kept} | {tuple(r) for r in true}
    # given orientations are used as they are
    given = np.eye(4, dtype=np.float64)
    assert np.array_equal(alignment.reference_orientations(4, ref_orientations=given), given.astype(np.float32))
