"""Generate the golden fixtures in this folder by running the UNMODIFIED reference.

This script is the only place that imports the reference (cmtip) itself, from a
read-only checkout named by ``--reference PATH`` or the ``CMTIP_REFERENCE`` environment
variable (the directory that holds the ``cmtip`` package); it runs in the development
container only.
Third-party modules the reference needs but that are absent here are replaced by
stubs in ``sys.modules`` before import:

* ``finufft``  -> ``oracle.nufft`` (FP64 ES-kernel NUFFT with finufft's signatures);
* ``skopi``    -> ``quaternion2rot3d`` (cmtip/eval/geom.py:25-46 convention),
                  ``get_uniform_quat`` / ``get_random_quat`` (seeded project generators);
* ``np.infty`` -> ``np.inf`` (numpy 2 removed the alias; cmtip/phasing/phase.py:203).

The package ``cmtip`` is registered without executing ``cmtip/__init__.py`` (which
pulls in h5py/mrcfile/skopi-GPU drivers); only the hot-path submodules are loaded.
Outputs: small ``.npz`` files holding inputs and the reference's outputs.

Run:  python tests/golden/make_golden.py --reference PATH [--only NAME ...]
      (NAME: core, phasing, sweep, loop; default: all)
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("CMTIP_REFERENCE", "")
sys.path.insert(0, REPO)

from cmtip_gb300 import geometry  # noqa: E402
from oracle import nufft as onufft  # noqa: E402


def _install_stubs(rng_seed=1234):
    np.infty = np.inf
    sys.modules["finufft"] = onufft
    sk = types.ModuleType("skopi")
    sk.quaternion2rot3d = geometry.quaternion2rot3d
    sk.get_uniform_quat = lambda n, avoid_symmetric=True: geometry.uniform_quaternions(n)
    _rng = np.random.default_rng(rng_seed)
    sk.get_random_quat = lambda n: geometry.random_quaternions(n, _rng)
    sys.modules["skopi"] = sk
    pkg = types.ModuleType("cmtip")
    pkg.__path__ = [os.path.join(REF, "cmtip")]
    sys.modules["cmtip"] = pkg


def _load_reference():
    _install_stubs()
    import importlib
    nufft = importlib.import_module("cmtip.nufft")
    ac = importlib.import_module("cmtip.autocorrelation.autocorrelation")
    al = importlib.import_module("cmtip.alignment.align")
    return nufft, ac, al


def synthetic_case(M, n_img, P, n_atoms, radius, seed):
    """Seeded particle, AC, detector, orientations and FP64 intensities (small)."""
    rng = np.random.default_rng(seed)
    rho = geometry.gaussian_particle(M, n_atoms, radius, rng)
    ac = geometry.autocorrelation_of(rho)
    ppr, rext = geometry.ewald_detector(P)
    rext = rext / 0.9
    quats = geometry.random_quaternions(n_img, rng).astype(np.float32)
    rot = np.array([np.linalg.inv(geometry.quaternion2rot3d(q)) for q in quats])
    H, K, L = np.einsum("ijk,klm->jilm", rot, ppr)
    x = [(a.astype(np.float32).ravel() / rext * np.pi).astype(np.float64) for a in (H, K, L)]
    intens = onufft.type2(x[0], x[1], x[2], ac.astype(np.complex128), eps=1e-12, isign=-1).real
    return dict(ac=ac.astype(np.float32), ppr=ppr, rext=np.float64(rext), quats=quats,
                slices=intens.reshape(n_img, 1, -1).astype(np.float32))


def main():
    nufft, ref_ac, ref_al = _load_reference()
    out = {}

    # 1. NUFFT wrappers (forward/adjoint, support, recip-sym, /M^3) on random points.
    rng = np.random.default_rng(7)
    M = 15
    N = 3000
    H_, K_, L_ = [rng.uniform(-0.95 * np.pi, 0.95 * np.pi, N).astype(np.float32) for _ in range(3)]
    ugrid = rng.standard_normal((M,) * 3).astype(np.float32)
    support = (rng.random((M,) * 3) > 0.3).astype(np.float32)
    nuvect = (rng.standard_normal(N) + 1j * rng.standard_normal(N)).astype(np.complex64)
    fwd = nufft.forward_cpu(ugrid.copy(), H_, K_, L_, support, True)
    adj = nufft.adjoint_cpu(nuvect, H_, K_, L_, M, True, support)
    adj_c = nufft.adjoint_cpu(nuvect, H_, K_, L_, M, False, None)
    np.savez_compressed(os.path.join(HERE, "nufft_wrappers.npz"), H=H_, K=K_, L=L_, ugrid=ugrid,
                        support=support, nuvect=nuvect, forward=fwd, adjoint=adj, adjoint_complex=adj_c, M=M)
    out["nufft_wrappers"] = (fwd.shape, adj.shape)

    # 2. positions, antisupport, linops, CG on a small seeded reconstruction.
    case = synthetic_case(M=21, n_img=12, P=8, n_atoms=20, radius=4.0, seed=11)
    H, K, L = ref_ac.gen_nonuniform_positions(case["quats"], case["ppr"])
    anti = {m: ref_ac.gen_F_antisupport(m) for m in (9, 21, 22)}
    Mg = 21
    Mtot = Mg ** 3
    slices = case["slices"]
    N = np.prod(slices.shape)  # numpy integer, as in autocorrelation.py:201 (makes rlambda float64)
    Hf, Kf, Lf = H.astype(np.float32), K.astype(np.float32), L.astype(np.float32)
    data = slices.flatten().astype(np.float32)
    est = (case["ac"] + 0.05 * rng.standard_normal(case["ac"].shape)).astype(np.float32)
    from scipy.ndimage import gaussian_filter
    ac_support = (gaussian_filter(est, 0.5) > 1e-12).astype(np.float32)
    x0 = (est * ac_support).flatten()
    weights = np.ones(N, dtype=np.float32)
    alambda, rlambda, flambda = 1, Mtot / N / 1000, 1e3
    W, d = ref_ac.setup_linops(Hf, Kf, Lf, data, ac_support, weights, x0, Mg, Mtot, N, case["rext"],
                               alambda, rlambda, flambda, use_gpu=False, use_recip_sym=True)
    probe = rng.standard_normal((3, Mtot))
    Wp = np.stack([W.matvec(p.astype(np.complex128)) for p in probe])
    from scipy.sparse.linalg import cg
    x10, _ = cg(W, d, x0=x0, maxiter=10, rtol=0.0)
    ac_solved = ref_ac.solve_ac(1, case["ppr"], case["rext"], slices, Mg,
                                orientations=case["quats"], ac_estimate=est.copy(), use_gpu=False)
    ac_gen0 = ref_ac.solve_ac(0, case["ppr"], case["rext"], slices, Mg,
                              orientations=case["quats"], ac_estimate=None, use_gpu=False)
    np.savez_compressed(os.path.join(HERE, "autocorrelation.npz"),
                        quats=case["quats"], ppr=case["ppr"], rext=case["rext"], slices=slices,
                        ac_true=case["ac"], estimate=est, H=H, K=K, L=L,
                        anti9=anti[9], anti21=anti[21], anti22=anti[22],
                        ac_support=ac_support, x0=x0, d=d, probe=probe, W_probe=Wp,
                        x_cg10=x10, ac_solved=ac_solved, ac_gen0=ac_gen0, M=Mg)
    out["autocorrelation"] = (d.dtype, x10.dtype, ac_solved.dtype)

    # 3. alignment: weights, slices, distances and the reference's own match test
    #    (true orientations spliced into 100 refs, nbatches=2; cmtip/tests/test_align.py:44-61).
    case = synthetic_case(M=21, n_img=3, P=8, n_atoms=20, radius=4.0, seed=21)
    w0 = ref_al.generate_weights(case["ppr"], order=0)
    w2 = ref_al.generate_weights(case["ppr"], order=-2)
    w1 = ref_al.generate_weights(case["ppr"], order=1)
    sl = ref_al.compute_slices(case["quats"], case["ppr"], case["rext"], case["ac"], use_gpu=False)
    ref_q = geometry.uniform_quaternions(40).astype(np.float32)
    model = ref_al.compute_slices(ref_q, case["ppr"], case["rext"], case["ac"]).reshape(40, -1)
    data2 = case["slices"].reshape(3, -1)
    dist = ref_al.calc_eudist(model * w2, data2 * w2)
    np.random.seed(5)
    matched = ref_al.match_orientations(0, case["ppr"], case["rext"], case["slices"], case["ac"], 100,
                                        nbatches=2, order=0, use_gpu=False,
                                        true_orientations=case["quats"])
    np.random.seed(5)
    ref_list = geometry.uniform_quaternions(100).astype(np.float32)
    ref_list = np.vstack((ref_list[:-3], case["quats"]))
    np.random.shuffle(ref_list)
    np.savez_compressed(os.path.join(HERE, "alignment.npz"),
                        quats=case["quats"], ppr=case["ppr"], rext=case["rext"], ac=case["ac"],
                        slices=case["slices"], w0=w0, w2=w2, w1=w1, slices_model=sl,
                        ref_q=ref_q, dist=dist, matched=matched, shuffled_refs=ref_list)
    out["alignment"] = (matched.shape,)

    # 4. multi-conformation alignment (align.py:135-213): images of two particles, each
    #    matched against both volumes; true orientations spliced into the references
    ca = synthetic_case(M=21, n_img=4, P=8, n_atoms=20, radius=4.0, seed=31)
    cb = synthetic_case(M=21, n_img=4, P=8, n_atoms=25, radius=5.0, seed=32)
    slices_m = np.concatenate([ca["slices"], cb["slices"]])
    quats_m = np.concatenate([ca["quats"], cb["quats"]])
    ac_mult = np.stack([ca["ac"], cb["ac"]])
    np.random.seed(7)
    q_mult, conf = ref_al.match_orientations_mult(0, ca["ppr"], ca["rext"], slices_m.copy(), ac_mult, 60,
                                                  nbatches=2, order=0, use_gpu=False,
                                                  true_orientations=quats_m)
    np.random.seed(7)
    ref_m = geometry.uniform_quaternions(60).astype(np.float32)
    ref_m = np.vstack((ref_m[:-len(quats_m)], quats_m))
    np.random.shuffle(ref_m)
    np.savez_compressed(os.path.join(HERE, "alignment_mult.npz"),
                        ppr=ca["ppr"], rext=ca["rext"], slices=slices_m, quats=quats_m, ac_mult=ac_mult,
                        shuffled_refs=ref_m, matched=q_mult, conformations=conf)
    out["alignment_mult"] = (q_mult.shape, conf.tolist())

    # 5. data preparation (prep_data.py:96-229): binning, clipping and trimming of a
    #    4-panel detector assembled as 2 x 2 quadrants
    import importlib
    sys.modules["h5py"] = types.ModuleType("h5py")
    sys.modules["cmtip.phasing"] = types.ModuleType("cmtip.phasing")
    ref_prep = importlib.import_module("cmtip.prep_data")
    P = 32  # trim_dataset needs an assembled detector wider than 2 x 20 pixels
    ppr_d, _ = geometry.ewald_detector(P)
    det_shape = (4, P, P)
    index_map = np.zeros((4, P, P, 2), dtype=np.int64)
    xx, yy = np.meshgrid(np.arange(P), np.arange(P), indexing="ij")
    for lp in range(4):
        index_map[lp, :, :, 0] = (lp // 2) * P + xx
        index_map[lp, :, :, 1] = (lp % 2) * P + yy
    rng = np.random.default_rng(51)
    imgs = (rng.random((5, 1, 4 * P * P)) * 1e3).astype(np.float32)
    res = 1e10 / np.linalg.norm(ppr_d, axis=0)
    res_limit = float(np.quantile(res, 0.5))
    b2 = ref_prep.bin_data(imgs, 2, det_shape)
    b4 = ref_prep.bin_data(imgs, 4, det_shape)
    b8 = ref_prep.bin_data(imgs, 8, det_shape)
    q2 = ref_prep.bin_data(ppr_d, 2, det_shape)
    c_img = ref_prep.clip_data(imgs, ppr_d, res_limit)
    c_ppr = ref_prep.clip_data(ppr_d, ppr_d, res_limit)
    t_ppr, t_img = ref_prep.trim_dataset(index_map, ppr_d, imgs, det_shape, res_limit)
    im2 = ref_prep.bin_pixel_index_map(index_map, 2)
    np.savez_compressed(os.path.join(HERE, "prep.npz"), ppr=ppr_d, index_map=index_map, imgs=imgs,
                        res_limit=res_limit, bin2=b2, bin4=b4, bin8=b8, ppr_bin2=q2, clip_img=c_img,
                        clip_ppr=c_ppr, trim_ppr=t_ppr, trim_img=t_img, index_map_bin2=im2)
    out["prep"] = (b2.shape, c_img.shape, t_img.shape, t_img.dtype)
    print(out)


def phasing_fixtures():
    """6. phasing (cmtip/phasing/phase.py): seeded phase() runs (short, medium, with a given
    support and density, even M, the full default schedule) and each function on random
    inputs, including an asymmetric amplitude mask and a finite rho_max."""
    import importlib
    _install_stubs()
    pk = sys.modules.get("cmtip.phasing") or types.ModuleType("cmtip.phasing")
    pk.__path__ = [os.path.join(REF, "cmtip", "phasing")]  # skip __init__ (maps.py needs mrcfile/h5py)
    sys.modules["cmtip.phasing"] = pk
    ph = importlib.import_module("cmtip.phasing.phase")
    from oracle import reference_port as rp

    def particle(M, n_atoms, radius, seed):
        rng = np.random.default_rng(seed)
        rho = geometry.gaussian_particle(M, n_atoms, radius, rng)
        return rho, geometry.autocorrelation_of(rho)

    M = 25
    rho_true, ac = particle(M, 30, 4.0, 61)
    res = dict(M=M, ac=ac, rho_true=rho_true)
    for tag, seed, kw in (("a", 21, dict(n_iterations=1, nER=5, nHIO=5)),
                          ("b", 22, dict(n_iterations=2, nER=20, nHIO=10)),
                          ("e", 23, dict())):
        np.random.seed(seed)
        a, s, r = ph.phase(0, ac.copy(), **kw)
        res.update({tag + "_seed": seed, tag + "_ac": a, tag + "_sup": s, tag + "_rho": r})
    rng = np.random.default_rng(62)
    sup_in = res["b_sup"].copy()
    rho_in = sup_in * rng.random((M, M, M))
    res.update(c_sup_in=sup_in.copy(), c_rho_in=rho_in.copy())
    a, s, r = ph.phase(1, ac.copy(), support_=sup_in, rho_=rho_in, n_iterations=1, nER=4, nHIO=4)
    res.update(c_ac=a, c_sup=s, c_rho=r)
    M2 = 20
    _, ac2 = particle(M2, 20, 3.0, 63)
    np.random.seed(24)
    a, s, r = ph.phase(0, ac2.copy(), n_iterations=1, nER=3, nHIO=3)
    res.update(f_ac_in=ac2, f_ac=a, f_sup=s, f_rho=r, f_seed=24)

    # single functions on random inputs
    ac_filt_, amp = rp.phase_amplitudes(ac)
    rho0 = rng.standard_normal((M, M, M)) * 0.1 + np.fft.ifftshift(rho_true)
    sup0 = rng.random((M, M, M)) > 0.4
    mask_sym = np.ones((M, M, M), dtype=np.bool_)
    mask_sym[0, 0, 0] = False
    mask_rand = rng.random((M, M, M)) > 0.2
    amp_rand = amp * (1 + 0.3 * rng.random((M, M, M)))
    rmod, star = ph.step_phase(rho0, amp_rand, mask_rand, sup0)
    rho_max = 0.5 * float(ph.step_phase(rho0, amp, mask_sym, sup0)[0].max())  # exercises the over-maximum branch
    er = rho0.copy()
    ph.ER(er, amp, mask_sym, sup0, rho_max)
    hio = rho0.copy()
    ph.HIO(0.3, hio, amp, mask_sym, sup0, rho_max)
    sw1 = sup0.copy()
    ph.shrink_wrap(5e-2, 1, rho0, sw1)
    sw15 = sup0.copy()
    ph.shrink_wrap(0.2, 1.5, rho0, sw15)
    cs = ph.create_support_(ac_filt_, M, int((M - 1) / 4), 0)
    hkl = rp.phase_recenter_grid(M)
    com = ph.center_of_mass(rho0, hkl, M)
    rc_rho, rc_sup = np.roll(rho0, (3, -2, 5), (0, 1, 2)), sup0.copy()
    ph.recenter(rc_rho, rc_sup, M)
    res.update(ac_filt_=ac_filt_, amplitudes_=amp, rho0=rho0, sup0=sup0, mask_rand=mask_rand,
               amp_rand=amp_rand, step_rmod=rmod, step_star=star, rho_max=rho_max, er=er, hio=hio,
               sw1=sw1, sw15=sw15, create_support=cs, com=com,
               rc_in=np.roll(rho0, (3, -2, 5), (0, 1, 2)), rc_rho=rc_rho, rc_sup=rc_sup)
    np.savez_compressed(os.path.join(HERE, "phasing.npz"), **res)
    print("phasing", {k: getattr(v, "shape", v) for k, v in res.items() if k.endswith("_ac")})


class _RankComm:
    """Rank ``rank`` of a ``size``-rank communicator in which every rank holds the whole data
    set, for running the reference's MPI lambda scan (autocorrelation_mpi.py:99-190) one rank
    after another in one process: Reduce keeps the rank's own grid (the data are that rank's),
    the broadcasts of reduced grids are no-ops, and rank 0 -- run last -- gathers the
    summaries the other ranks recorded and receives the kept rank's solution by Bcast."""

    def __init__(self, rank, size, book):
        self.rank, self.size, self.book = rank, size, book

    def Reduce(self, send, recv, op=None, root=0):
        recv[...] = send

    def Bcast(self, buf, root=0):
        if self.rank == 0 and root != 0:
            buf[...] = self.book["ac"][root]

    def bcast(self, obj, root=0):
        return obj if self.rank == root else -1

    def gather(self, obj, root=0):
        self.book["summary"][self.rank] = obj
        if self.rank != root:
            return None
        return [self.book["summary"][r] for r in range(self.size)]


def sweep_fixture():
    """7. the lambda scan of autocorrelation_mpi.py:99-190 on n ranks, generations 0 and 1."""
    import contextlib
    import importlib
    import io
    import re
    _install_stubs()
    mpi = types.ModuleType("mpi4py")
    mpi.MPI = types.SimpleNamespace(SUM="sum")
    sys.modules["mpi4py"] = mpi
    acm = importlib.import_module("cmtip.autocorrelation.autocorrelation_mpi")
    solved = []
    scipy_cg = acm.cg

    def recording_cg(*args, **kwargs):  # scipy's cg unchanged; keeps each rank's own solution
        ret = scipy_cg(*args, **kwargs)
        solved.append(np.ascontiguousarray(ret[0].real))
        return ret

    acm.cg = recording_cg
    case = synthetic_case(M=21, n_img=12, P=8, n_atoms=20, radius=4.0, seed=71)
    rng = np.random.default_rng(72)
    est = (case["ac"] * (1.0 + 0.05 * rng.standard_normal(case["ac"].shape))).astype(np.float32)
    size, M = 6, 21
    out = dict(quats=case["quats"], ppr=case["ppr"], rext=case["rext"], slices=case["slices"], estimate=est,
               M=M, size=size)
    for gen in (0, 1):
        book = {"summary": {}, "ac": {}}
        its, own = {}, {}
        for rank in list(range(1, size)) + [0]:
            buf = io.StringIO()
            with contextlib.redirect_stdout(buf):
                ac = acm.solve_ac_mpi(_RankComm(rank, size, book), gen, case["ppr"], case["rext"],
                                      case["slices"], M, orientations=case["quats"],
                                      ac_estimate=None if gen == 0 else est.copy(), use_gpu=False)
            its[rank] = int(re.search(r"got AC in (\d+) iterations", buf.getvalue()).group(1))
            own[rank] = solved[-1].reshape((M,) * 3)
            if rank != 0:
                book["ac"][rank] = ac.copy()
            else:
                kept = re.search(r"Keeping result from rank (\d+)", buf.getvalue())
                out[f"g{gen}_keep"] = int(kept.group(1))
                out[f"g{gen}_ac"] = ac
        ranks, lambdas, v1s, v2s = [np.array(el) for el in zip(*[book["summary"][r] for r in range(size)])]
        out.update({f"g{gen}_rlambdas": lambdas, f"g{gen}_v1": v1s, f"g{gen}_v2": v2s,
                    f"g{gen}_iterations": np.array([its[r] for r in range(size)]),
                    f"g{gen}_solutions": np.stack([own[r] for r in range(size)])})
    acm.cg = scipy_cg
    np.savez_compressed(os.path.join(HERE, "lambda_sweep.npz"), **out)
    print("lambda_sweep", {k: out[k] for k in ("g0_keep", "g1_keep")}, out["g0_iterations"], out["g1_iterations"])
    for gen in (0, 1):
        print(gen, out[f"g{gen}_v1"], out[f"g{gen}_v2"], np.mean(out[f"g{gen}_v1"]))


LOOP = dict(M=21, n_img=30, P=8, n_atoms=20, radius=4.0, seed=81, generations=3, np_seed=17,
            phase=dict(n_iterations=1, nER=5, nHIO=5))


def loop_fixture():
    _loop_fixture(aligned=False, name="mtip_loop")
    _loop_fixture(aligned=True, name="mtip_loop_aligned")


def _loop_fixture(aligned, name):
    """8. the MTIP generation loop (reconstruct.py:29-96, run_mtip) on a small case, not
    aligned (random generation-0 orientations from the skopi stub's seeded generator, then
    matching against the reference's hard-coded 5000 references at its 9 A resolution
    limit) and aligned (the true orientations throughout).
    Two stand-ins: save_checkpoint (h5py / mrcfile) records each generation's checkpoint in
    memory, and phase() runs a short schedule (LOOP['phase']) -- ER / HIO from a random start
    are chaotic over the default 1300 iterations, so only short schedules can be compared."""
    import functools
    import importlib
    _install_stubs()
    sys.modules["h5py"] = types.ModuleType("h5py")
    pk = types.ModuleType("cmtip.phasing")
    pk.__path__ = [os.path.join(REF, "cmtip", "phasing")]  # skip __init__ (maps.py needs mrcfile)
    sys.modules["cmtip.phasing"] = pk
    ph = importlib.import_module("cmtip.phasing.phase")
    pk.phase = functools.partial(ph.phase, **LOOP["phase"])
    rec = importlib.import_module("cmtip.reconstruct")
    saved = {}

    def record(generation, output, checkpoint):
        saved[generation] = {k: (np.array(v, copy=True) if isinstance(v, np.ndarray) else v)
                             for k, v in checkpoint.items()}

    rec.save_checkpoint = record
    solves = []
    ref_solve = rec.autocorrelation.solve_ac

    def recording_solve(*args, **kwargs):  # the reference's solve_ac, unchanged; keeps its output
        ac = ref_solve(*args, **kwargs)
        solves.append(np.array(ac, copy=True))
        return ac

    rec.autocorrelation.solve_ac = recording_solve
    case = synthetic_case(M=LOOP["M"], n_img=LOOP["n_img"], P=LOOP["P"], n_atoms=LOOP["n_atoms"],
                          radius=LOOP["radius"], seed=LOOP["seed"])
    data = {"pixel_position_reciprocal": case["ppr"], "reciprocal_extent": case["rext"],
            "intensities": case["slices"], "orientations": case["quats"]}
    np.random.seed(LOOP["np_seed"])
    rec.run_mtip(data, LOOP["M"], "unused", aligned=aligned, n_iterations=LOOP["generations"], use_gpu=False,
                 checkpoint=rec.load_checkpoint())
    out = dict(ppr=case["ppr"], rext=case["rext"], slices=case["slices"], quats_true=case["quats"],
               ac_true=case["ac"], M=LOOP["M"], np_seed=LOOP["np_seed"], stub_seed=1234,
               generations=LOOP["generations"], **{"phase_" + k: v for k, v in LOOP["phase"].items()})
    rec.autocorrelation.solve_ac = ref_solve
    out["g0_ac"] = solves[0]
    out["aligned"] = aligned
    for g, ck in saved.items():
        for k in ("orientations", "ac", "ac_phased", "support_", "rho_"):
            if ck.get(k) is not None:
                out[f"g{g}_{k}"] = ck[k]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, sorted(k for k in out if k.startswith("g")))


FIXTURES = {"core": lambda: main(), "phasing": lambda: phasing_fixtures(), "sweep": lambda: sweep_fixture(),
            "loop": lambda: loop_fixture()}


def _cli():
    import argparse
    global REF
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference", default=REF,
                    help="checkout of the reference project (holds cmtip/); default $CMTIP_REFERENCE")
    ap.add_argument("--only", nargs="*", choices=sorted(FIXTURES), default=None,
                    help="fixtures to regenerate (default: all)")
    a = ap.parse_args()
    if not a.reference or not os.path.isdir(os.path.join(a.reference, "cmtip")):
        ap.error("give the reference checkout with --reference PATH or CMTIP_REFERENCE")
    REF = a.reference
    for name in (a.only or list(FIXTURES)):
        FIXTURES[name]()


if __name__ == "__main__":
    _cli()
