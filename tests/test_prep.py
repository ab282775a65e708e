"""Data preparation (cmtip/prep_data.py) against fixtures made by the unmodified reference:
host-side index logic on the CPU, the device pass on the GPU (bit-exact: block means in
numpy's summation order, gathers)."""
import numpy as np
import pytest


def test_index_logic_matches_reference(golden):
    from cmtip_gb300 import prep
    g = golden("prep")
    det_shape = (4, 32, 32)
    assert np.array_equal(prep.bin_pixel_index_map(g["index_map"], 2), g["index_map_bin2"])
    idx = prep.kept_indices(g["ppr"], float(g["res_limit"]))
    assert np.array_equal(g["ppr"][:, :, idx], g["clip_ppr"])
    keep = prep.trim_indices(g["index_map"], g["ppr"], det_shape, float(g["res_limit"]))
    assert np.array_equal(g["ppr"].reshape(3, -1)[:, keep][:, None, :], g["trim_ppr"])
    assert np.array_equal(g["imgs"].reshape(5, -1)[:, keep][:, None, :].astype(np.float64), g["trim_img"])


@pytest.mark.gpu
def test_device_binning_clipping_trimming_bit_exact(golden):
    import torch
    from cmtip_gb300 import prep
    g = golden("prep")
    det_shape = (4, 32, 32)
    rl = float(g["res_limit"])
    for b, key in ((2, "bin2"), (4, "bin4"), (8, "bin8")):
        out = prep.bin_data(g["imgs"], b, det_shape)
        assert out.dtype == np.float32 and np.array_equal(out, g[key])
    assert np.array_equal(prep.bin_data(g["ppr"], 2, det_shape), g["ppr_bin2"])  # float64
    assert np.array_equal(prep.clip_data(g["imgs"], g["ppr"], rl), g["clip_img"])
    q, x = prep.clip_dataset(g["ppr"], g["imgs"], rl)
    assert np.array_equal(q, g["clip_ppr"]) and np.array_equal(x, g["clip_img"])
    q, x = prep.trim_dataset(g["index_map"], g["ppr"], g["imgs"], det_shape, rl)
    assert np.array_equal(q, g["trim_ppr"]) and x.dtype == np.float64 and np.array_equal(x, g["trim_img"])
    # fused binning + clipping equals the two steps; device tensors stay on the device
    q2, x2 = prep.bin_clip(torch.from_numpy(g["imgs"]).cuda(), g["ppr"], 2, det_shape, rl)
    ref = prep.clip_data(g["bin2"], g["ppr_bin2"], rl)
    assert x2.is_cuda and np.array_equal(x2.cpu().numpy(), ref)
    assert np.array_equal(q2, prep.clip_data(g["ppr_bin2"], g["ppr_bin2"], rl))
    # indices outside the binned range are refused (no out-of-range read)
    from cmtip_gb300.prep import _bin_clip_dev
    with pytest.raises(ValueError):
        _bin_clip_dev(torch.zeros(2, 64, device="cuda"), 1, 8, 8, 1, np.array([0, 64]))
