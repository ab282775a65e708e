"""The MTIP generation loop of cmtip/reconstruct.py:29-96 (``run_mtip``) on the GPU.

Generation 0 solves the autocorrelation with the given (``aligned``) or random orientations
and phases it; every later generation matches the images, clipped to ``res_limit``, against
``n_ref`` model slices of the last phased autocorrelation (unless ``aligned``), solves the
autocorrelation from all pixels with the phased one as estimate and support source, and
phases it again from the previous support and density.  The hand-offs are the reference's:
the phased autocorrelation as a float32 estimate (:82-83), the matched orientations as
float32 (:80), the phasing's support and density carried to the next phasing (:85-88).

The stages are this package's: ``solve_ac`` (autocorrelation.py), ``match_orientations``
(alignment.py), ``phase`` (phasing.py) and ``clip_data`` (prep.py).  Images stay on the
device across generations when ``data['intensities']`` is a CUDA tensor.  The reference's
per-generation h5 checkpoint and MRC density (prep_data.py:271-294) need h5py / mrcfile;
here ``on_generation(generation, checkpoint)`` is called at that point instead, and
``output`` (optional) receives ``checkpoint_g{generation}.npz``.
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

from . import alignment, autocorrelation, phasing, prep
from .nufft import DEFAULT_EPS


def load_checkpoint(input_file=None):
    """prep_data.py:297-324: generation 0 and no orientations, or the arrays of a checkpoint
    written by ``run_mtip`` (generation parsed from ``checkpoint_g<generation>.npz``)."""
    if input_file is None:
        return {"generation": 0, "orientations": None}
    with np.load(input_file, allow_pickle=False) as f:
        ck = {k: f[k] for k in f.files}
    ck["generation"] = int(os.path.basename(input_file).split("g")[1].split(".")[0])
    if "reciprocal_extent" in ck:
        ck["reciprocal_extent"] = float(ck["reciprocal_extent"])
    return ck


def _to_numpy(a):
    return a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)


def _save(output, generation, checkpoint):
    arrays = {k: _to_numpy(v) for k, v in checkpoint.items()
              if k != "generation" and v is not None}
    np.savez(os.path.join(output, f"checkpoint_g{generation}.npz"), **arrays)


def run_mtip(data, M, output=None, aligned=True, n_iterations=10, use_gpu=True, checkpoint=None, *,
             n_ref=5000, res_limit=9, cg_maxiter=100, cg_rtol=1e-5, phase_iterations=10, nER=50, nHIO=25,
             prec=32, match_mode="bf16", phase_prec=None, eps=DEFAULT_EPS, rng=None, on_generation=None,
             verbose=True):
    """reconstruct.py:29-96.  ``data``: 'pixel_position_reciprocal' (3, n_panels, n_pix),
    'reciprocal_extent', 'intensities' (n_images, n_panels, n_pix; numpy or a CUDA tensor),
    and 'orientations' when ``aligned``.  The reference's hard-coded n_ref = 5000,
    res_limit = 9 (:45), solve_ac's maxiter 100 / rtol 1e-5 and phase()'s schedule (10 cycles
    of ER 50, HIO 25, ER 50) are the defaults.  ``prec`` / ``match_mode`` / ``phase_prec``
    select the forms of the solve, the distance GEMM and the phasing (``prec=64``,
    ``match_mode='fp64'``, ``phase_prec=64``: the reference's arithmetic); ``rng`` draws the
    random generation-0 orientations when they are not given.  Returns the checkpoint dict
    of the last generation (orientations, ac, ac_phased, support_, rho_, generation)."""
    t0 = time.perf_counter()
    say = print if verbose else (lambda *a, **k: None)
    say("Running MTIP")
    checkpoint = load_checkpoint() if checkpoint is None else checkpoint
    ppr = data["pixel_position_reciprocal"]
    rext = data["reciprocal_extent"]
    intens = data["intensities"]
    solve_kw = dict(prec=prec, eps=eps, maxiter=cg_maxiter, rtol=cg_rtol, verbose=verbose)
    phase_kw = dict(n_iterations=phase_iterations, nER=nER, nHIO=nHIO)
    if phase_prec is not None:
        phase_kw["prec"] = phase_prec
    if aligned:
        say("Using ground truth quaternions")
        checkpoint["orientations"] = data["orientations"]

    def done(generation):
        checkpoint["generation"] = generation
        if output is not None:
            os.makedirs(output, exist_ok=True)
            _save(output, generation, checkpoint)
        if on_generation is not None:
            on_generation(generation, checkpoint)

    # generation 0: no estimate of the autocorrelation yet
    if checkpoint["generation"] == 0:
        ac = autocorrelation.solve_ac(0, ppr, rext, intens, M, orientations=checkpoint["orientations"], rng=rng,
                                      **solve_kw)
        checkpoint["ac"] = ac
        checkpoint["ac_phased"], checkpoint["support_"], checkpoint["rho_"] = phasing.phase(0, ac, **phase_kw)
        checkpoint["reciprocal_extent"] = rext
        done(0)

    clipped = None
    for generation in range(checkpoint["generation"] + 1, n_iterations):
        ac_phased = checkpoint["ac_phased"]
        est32 = ac_phased.to(torch.float32) if torch.is_tensor(ac_phased) else ac_phased.astype(np.float32)
        if not aligned:
            if clipped is None:  # the resolution clip depends on the detector only
                clipped = (prep.clip_data(ppr, ppr, res_limit), prep.clip_data(intens, ppr, res_limit))
            checkpoint["orientations"] = alignment.match_orientations(generation, clipped[0], rext, clipped[1],
                                                                      est32, n_ref, mode=match_mode, eps=eps)
        q = checkpoint["orientations"]
        q32 = q.to(torch.float32) if torch.is_tensor(q) else np.asarray(q).astype(np.float32)
        est = est32.clone() if torch.is_tensor(est32) else est32.copy()
        checkpoint["ac"] = autocorrelation.solve_ac(generation, ppr, rext, intens, M, orientations=q32,
                                                    ac_estimate=est, **solve_kw)
        checkpoint["ac_phased"], checkpoint["support_"], checkpoint["rho_"] = phasing.phase(
            generation, checkpoint["ac"], checkpoint["support_"], checkpoint["rho_"], **phase_kw)
        done(generation)

    say("elapsed time is %.2f" % ((time.perf_counter() - t0) / 60.0))
    return checkpoint
