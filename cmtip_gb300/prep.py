"""Data preparation on the device, mirroring ``cmtip.prep_data``.

``bin_data`` (prep_data.py:181-212), ``clip_data`` / ``clip_dataset`` (:149-178) and
``trim_dataset`` (:96-146) keep the reference's signatures and shapes; the pixel work is one
pass of ``cmt_bin_clip`` over the image stack (block means in numpy's summation order, so
results equal the reference's bit for bit, then a gather of the kept pixels).  The index
bookkeeping (which pixels a resolution limit keeps, the assembled-detector crop) is
detector-sized and stays on the host.  numpy inputs give numpy outputs; CUDA tensors stay
on the device.  ``bin_clip`` fuses binning and clipping for the reconstruction loop's
alignment data.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .nufft import _stream_ptr


def _dev(a):
    t = a if torch.is_tensor(a) else torch.from_numpy(np.ascontiguousarray(a))
    if t.dtype not in (torch.float32, torch.float64):
        t = t.to(torch.float64)
    return t.to("cuda").contiguous()


def _bin_clip_dev(x, n_panels, px, py, bin_factor, keep=None):
    """x: (n, n_panels * px * py) device tensor -> (n, n_keep)."""
    n = x.shape[0]
    prec = 64 if x.dtype == torch.float64 else 32
    n_binned = n_panels * (px // bin_factor) * (py // bin_factor)
    kp = None
    n_keep = n_binned
    if keep is not None:
        kp = torch.as_tensor(np.asarray(keep, dtype=np.int64) if not torch.is_tensor(keep) else keep,
                             device="cuda").to(torch.int64).contiguous()
        n_keep = kp.numel()
    out = torch.empty((n, n_keep), dtype=x.dtype, device="cuda")
    if n_keep == 0 or n == 0:
        return out
    _lib.call("cmt_bin_clip", prec, ctypes.c_void_p(x.data_ptr()), n, n_panels, px, py, int(bin_factor),
              ctypes.c_void_p(kp.data_ptr()) if kp is not None else None, n_keep, ctypes.c_void_p(out.data_ptr()),
              _stream_ptr())
    return out


def bin_data(arr, bin_factor, det_shape=None):
    """prep_data.py:181-212: bin detector data by block means.  arr (n, n_panels, nx, ny), or
    (n, 1, n_pixels) with det_shape = (n_panels, nx, ny); returns the same layout binned."""
    numpy_io = not torch.is_tensor(arr)
    if det_shape is not None:
        n_panels, px, py = (int(v) for v in det_shape)
    else:
        n_panels, px, py = (int(v) for v in arr.shape[1:4])
    assert px % bin_factor == 0
    assert py % bin_factor == 0
    x = _dev(arr).reshape(arr.shape[0], -1)
    out = _bin_clip_dev(x, n_panels, px, py, int(bin_factor))
    bx, by = px // bin_factor, py // bin_factor
    out = out.reshape(arr.shape[0], 1, n_panels * bx * by) if det_shape is not None else \
        out.reshape(arr.shape[0], n_panels, bx, by)
    return out.cpu().numpy() if numpy_io else out


def kept_indices(pixel_position_reciprocal, res_limit):
    """Indices of the pixels of clip_data (prep_data.py:160-161): resolution 1e10 / |q| above
    res_limit, taken from the first panel row of the q-vectors."""
    p = pixel_position_reciprocal.cpu().numpy() if torch.is_tensor(pixel_position_reciprocal) else \
        np.asarray(pixel_position_reciprocal)
    resolution = 1.0 / np.linalg.norm(p, axis=0) * 1e10
    return np.where(resolution[0] > res_limit)[0]


def clip_data(arr, pixel_position_reciprocal, res_limit):
    """prep_data.py:149-163: keep the pixels beyond the resolution limit, arr (n, n_panels,
    n_pixels) -> (n, n_panels, n_retained)."""
    numpy_io = not torch.is_tensor(arr)
    idx = kept_indices(pixel_position_reciprocal, res_limit)
    n, n_panels, n_pix = (int(v) for v in arr.shape)
    x = _dev(arr).reshape(n * n_panels, n_pix)
    out = _bin_clip_dev(x, 1, 1, n_pix, 1, idx).reshape(n, n_panels, len(idx))
    return out.cpu().numpy() if numpy_io else out


def clip_dataset(pixel_position_reciprocal, intensities, res_limit):
    """prep_data.py:165-178."""
    if res_limit == 0:
        return pixel_position_reciprocal, intensities
    intensities = clip_data(intensities, pixel_position_reciprocal, res_limit)
    pixel_position_reciprocal = clip_data(pixel_position_reciprocal, pixel_position_reciprocal, res_limit)
    return pixel_position_reciprocal, intensities


def bin_clip(intensities, pixel_position_reciprocal, bin_factor, det_shape, res_limit=0):
    """bin_data of the images and q-vectors followed by clip_data at res_limit (0: none), the
    images in one device pass.  intensities (n, 1, n_pixels), q-vectors (3, 1, n_pixels);
    returns (q-vectors, intensities) in the reference's shapes."""
    numpy_io = not torch.is_tensor(intensities)
    ppr_b = bin_data(np.asarray(pixel_position_reciprocal.cpu() if torch.is_tensor(pixel_position_reciprocal)
                                else pixel_position_reciprocal), bin_factor, det_shape)
    n_panels, px, py = (int(v) for v in det_shape)
    keep = None if res_limit == 0 else kept_indices(ppr_b, res_limit)
    x = _dev(intensities).reshape(intensities.shape[0], -1)
    out = _bin_clip_dev(x, n_panels, px, py, int(bin_factor), keep)
    out = out.reshape(intensities.shape[0], 1, -1)
    if keep is not None:
        ppr_b = ppr_b[:, :, keep]
    return ppr_b, (out.cpu().numpy() if numpy_io else out)


def bin_pixel_index_map(arr, bin_factor):
    """prep_data.py:215-229 (host: detector-sized)."""
    arr = np.moveaxis(arr, -1, 0)
    arr = np.minimum(arr[..., ::bin_factor, :], arr[..., 1::bin_factor, :])
    arr = np.minimum(arr[..., ::bin_factor], arr[..., 1::bin_factor])
    arr = arr // bin_factor
    return np.moveaxis(arr, 0, -1)


def assemble_image_stack_batch(image_stack, index_map):
    """prep_data.py:232-255: panels -> 2D detector images through the index map."""
    numpy_io = not torch.is_tensor(image_stack)
    x = _dev(image_stack)
    nx = int(index_map[:, :, :, 0].max()) + 1
    ny = int(index_map[:, :, :, 1].max()) + 1
    img = torch.zeros((x.shape[0], nx, ny), dtype=torch.float64, device="cuda")
    im = torch.as_tensor(np.asarray(index_map), device="cuda").long()
    for lp in range(x.shape[1]):
        img[:, im[lp, :, :, 0], im[lp, :, :, 1]] = x[:, lp].to(torch.float64)
    return img.cpu().numpy() if numpy_io else img


def trim_indices(pixel_index_map, pixel_position_reciprocal, det_shape, res_limit):
    """The flattened detector pixels trim_dataset keeps (prep_data.py:96-146), in its output
    order (row-major over the centred square of the assembled detector), or None when the
    data are returned untrimmed."""
    ppr = np.asarray(pixel_position_reciprocal)
    if res_limit == 0:
        return None
    data_max_res = 1e10 / np.linalg.norm(ppr, axis=0).max()
    if res_limit < data_max_res:
        print("Warning: requested resolution exceeds data resolution.")
        return None
    im = np.asarray(pixel_index_map)
    nx, ny = int(im[:, :, :, 0].max()) + 1, int(im[:, :, :, 1].max()) + 1
    src = -np.ones((nx, ny), dtype=np.int64)  # assembled pixel -> flattened source pixel
    n_panels, px, py = (int(v) for v in det_shape)
    flat = np.arange(n_panels * px * py).reshape(n_panels, px, py)
    for lp in range(n_panels):
        src[im[lp, :, :, 0], im[lp, :, :, 1]] = flat[lp]
    q = ppr.reshape((3,) + tuple(det_shape))
    qa = np.zeros((3, nx, ny))
    for lp in range(n_panels):
        qa[:, im[lp, :, :, 0], im[lp, :, :, 1]] = q[:, lp]
    center = np.array(0.5 * np.array([nx, ny])).astype(int)
    min_pix = 20
    norms = np.linalg.norm(qa, axis=0)
    res = np.array([1e10 / norms[center[0] - i, center[1] - i] for i in range(min_pix, np.min(center))])
    nkeep = np.argmin(np.abs(res - res_limit)) + min_pix
    crop = src[center[0] - nkeep:center[0] + nkeep, center[1] - nkeep:center[1] + nkeep]
    return crop[crop >= 0]


def trim_dataset(pixel_index_map, pixel_position_reciprocal, intensities, det_shape, res_limit):
    """prep_data.py:96-146: keep the centred square of the assembled detector whose corner
    pixel has the requested resolution; the images' pixels are gathered on the device."""
    keep = trim_indices(pixel_index_map, pixel_position_reciprocal, det_shape, res_limit)
    if keep is None:
        return pixel_position_reciprocal, intensities
    numpy_io = not torch.is_tensor(intensities)
    n = intensities.shape[0]
    x = _dev(intensities).reshape(n, -1)
    # the reference assembles into a float64 image (prep_data.py:247), so its output is float64
    out = _bin_clip_dev(x, 1, 1, x.shape[1], 1, keep).reshape(n, 1, -1).to(torch.float64)
    ppr = np.asarray(pixel_position_reciprocal, dtype=np.float64).reshape(3, -1)[:, keep][:, None, :]
    return ppr, (out.cpu().numpy() if numpy_io else out)
