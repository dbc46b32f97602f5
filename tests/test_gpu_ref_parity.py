"""Reference-mode parity on the GPU: the CUDA path through the C ABI against the
CPU oracle (fr_oracle.c, op-order matched), bit for bit."""
import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N
from oracle import oracle as O
from tests.helpers import assert_bitexact, images, random_state, rel_err

pytestmark = pytest.mark.gpu


def _to(dev, a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _params(dims, **kw):
    base = dict(volume_dims=dims, no_labels=4, max_iter=8, alpha=0.05, tau=0.2, w_reg=0.2, rho_0=1.0, p=2.0, C=0.25,
                reset_iter=-1, max_update_norm=-1e-10)
    base.update(kw)
    return Params(**base)


STAGINGS = [1, 2]  # STAGING: per-thread cp.async, TMA tensor copies


@pytest.mark.parametrize("staging", STAGINGS)
@pytest.mark.parametrize("dims", [(4, 4, 4), (5, 6, 4), (7, 9, 11), (33, 17, 20), (40, 36, 30)])
@pytest.mark.parametrize("iter_no", [1, 2, 7])
def test_one_iteration_from_random_state(cuda, dims, iter_no, staging):
    """One iteration (L, pass A, pass B) from a random mid-registration state, with
    either staging of the stencil operands."""
    seed = 10 * dims[0] + iter_no
    d = images(dims, seed)
    st = random_state(dims, seed + 1, disp=1.5, vel=0.3)
    P = _params(dims, staging=staging)
    fr = FastReg(P)
    tens = [_to(cuda, d[k]) for k in ("T", "labT", "S", "labS")]
    fr.begin([tuple(tens)])
    fr.set_field(N.FR_FIELD_RHO, _to(cuda, st["rho"]))
    fr.set_field(N.FR_FIELD_V, _to(cuda, st["v"]))
    fr.set_field(N.FR_FIELD_PSI, _to(cuda, st["psi"]))
    fr.set_field(N.FR_FIELD_PSI_INV, _to(cuda, st["psi_inv"]))
    t = P.alpha * iter_no
    fr.step(iter_no, t)
    rho_g = fr.get_field(N.FR_FIELD_RHO).cpu().numpy()
    v_g = fr.get_field(N.FR_FIELD_V).cpu().numpy()
    psi_g = fr.get_field(N.FR_FIELD_PSI).cpu().numpy()
    pinv_g = fr.get_field(N.FR_FIELD_PSI_INV).cpu().numpy()
    norms, vox = fr.trace()

    k = O.ref_coef(P.alpha, np.float32(t), P.p, P.C, P.tau, P.w_reg)
    L = O.ref_laplacian(st["psi"])
    rho_o, v_o, pinv_o = O.ref_pass_a(k, d["S"], d["T"], iter_no == 1, st["rho"], st["v"], st["psi_inv"], L)
    psi_o, mx, am = O.ref_pass_b(P.alpha, v_o, st["psi"])

    assert_bitexact(rho_g, rho_o, "rho")
    assert_bitexact(v_g, v_o, "v")
    assert_bitexact(pinv_g, pinv_o, "psi_inv")
    assert_bitexact(psi_g, psi_o, "psi")
    assert np.float32(norms[iter_no - 1]) == np.float32(mx)
    assert int(vox[iter_no - 1]) == am
    fr.close()


@pytest.mark.parametrize("staging", STAGINGS)
@pytest.mark.parametrize("dims,iters", [((4, 5, 4), 20), ((12, 10, 9), 30), ((24, 20, 18), 60), ((64, 64, 64), 200)])
def test_full_registration(cuda, dims, iters, staging):
    """A whole registration through FastReg::operator() semantics (in place), with either
    staging of the stencil operands."""
    import torch
    d = images(dims, 7 + dims[0])
    P = _params(dims, max_iter=iters, alpha=0.02, staging=staging)
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, d[k]) for k in ("T", "labT", "S", "labS"))
    assert fr(iT, lT, iS, lS)
    st = fr.stats()
    psi_g = fr.get_field(N.FR_FIELD_PSI).cpu().numpy()
    pinv_g = fr.get_field(N.FR_FIELD_PSI_INV).cpu().numpy()
    norms, vox = fr.trace()

    o = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
    assert st.iterations == o["iterations"] == iters
    assert fr.tile_staging()[0] == ("tma" if staging == 2 else "cp.async")
    assert_bitexact(psi_g, o["psi"], "psi")
    assert_bitexact(pinv_g, o["psi_inv"], "psi_inv")
    assert_bitexact(iT.cpu().numpy(), o["out_T"], "T o psi_inv")
    assert_bitexact(iS.cpu().numpy(), o["out_S"], "S o psi")
    assert_bitexact(lT.cpu().numpy(), o["out_labT"], "labels T o psi_inv")
    assert_bitexact(lS.cpu().numpy(), o["out_labS"], "labels S o psi")
    assert_bitexact(norms, o["trace_norm"], "max update norms")
    assert_bitexact(vox, o["trace_idx"], "max update voxels")

    os_ = O.stats(d["T"], d["labT"], o["out_S"], o["out_labS"], o["psi"], P.no_labels)
    assert rel_err(st.e_data, os_["e_data"]) < 1e-12
    assert rel_err(st.e_reg, os_["e_reg"]) < 1e-12
    assert st.folds == os_["folds"]
    assert st.dice_inter == list(os_["dice_inter"][:P.no_labels])
    assert st.dice_count == list(os_["dice_count"][:P.no_labels])
    assert st.dice_out_of_range == os_["dice_out_of_range"]
    # FP32 rounding drift against the FP64 oracle, in voxels (positions are O(dims),
    # so a relative bound on them would say little about the displacement)
    o64 = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"], prec=64)
    err = float(np.abs(psi_g.astype(np.float64) - o64["psi"]).max())
    err_inv = float(np.abs(pinv_g.astype(np.float64) - o64["psi_inv"]).max())
    assert err < 1e-3 and err_inv < 1e-3, f"FP32 vs FP64 drift: psi {err}, psi_inv {err_inv} voxels"
    fr.close()


def test_warp_standalone(cuda):
    """fr_warp (apply_kernel) on random positions, including positions outside the
    grid and NaN, against the oracle: intensities and floor-corner labels bit-exact."""
    import torch
    from fastreg_gb300 import warp
    r = np.random.Generator(np.random.PCG64(5))
    for dims in [(7, 9, 11), (33, 17, 20), (64, 64, 64)]:
        X, Y, Z = dims
        img = r.normal(0, 1, (Z, Y, X)).astype(np.float32)
        lab = r.integers(0, 8, (Z, Y, X)).astype(np.int16)
        pos = np.stack([r.uniform(-2, X + 1, (Z, Y, X)), r.uniform(-2, Y + 1, (Z, Y, X)),
                        r.uniform(-2, Z + 1, (Z, Y, X))]).astype(np.float32)
        pos[:, 0, 0, :3] = np.nan
        pos[0, 1, 1, 1] = X - 1  # exactly on the upper face
        out, out_lab = warp(_to(cuda, pos), _to(cuda, img), _to(cuda, lab))
        o_img, o_lab = O.warp(pos, img, lab)
        assert_bitexact(out.cpu().numpy(), o_img, f"warp {dims}")
        assert_bitexact(out_lab.cpu().numpy(), o_lab, f"warp labels {dims}")


def test_convergence_stops_on_device(cuda):
    """MAX_UPDATE_NORM reached -> the solver stops at that iteration, on the device
    (graph path), with the same state as the oracle's break (solver.cu:418-421)."""
    dims = (24, 20, 18)
    d = images(dims, 99)
    P0 = _params(dims, max_iter=40, alpha=0.02)
    o_full = O.ref_register(P0, d["T"], d["labT"], d["S"], d["labS"])
    thr = float(np.float32(o_full["trace_norm"][12]))  # stop where the norm first drops to this
    P = _params(dims, max_iter=40, alpha=0.02, max_update_norm=thr)
    o = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
    assert o["converged"] and o["iterations"] < 40
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, d[k]) for k in ("T", "labT", "S", "labS"))
    fr(iT, lT, iS, lS)
    st = fr.stats()
    assert st.converged and st.iterations == o["iterations"]
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), o["psi"], "psi")
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI_INV).cpu().numpy(), o["psi_inv"], "psi_inv")
    assert_bitexact(iS.cpu().numpy(), o["out_S"], "S o psi")
    assert_bitexact(iT.cpu().numpy(), o["out_T"], "T o psi_inv")


def test_reset_iter_schedule(cuda):
    """RESET_ITER restarts t (solver.cu:428-432)."""
    dims = (16, 14, 12)
    d = images(dims, 3)
    P = _params(dims, max_iter=25, alpha=0.03, reset_iter=7)
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, d[k]) for k in ("T", "labT", "S", "labS"))
    fr(iT, lT, iS, lS)
    o = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), o["psi"], "psi")
    assert_bitexact(iS.cpu().numpy(), o["out_S"], "S o psi")


def test_keep_state_carries_fields_over(cuda):
    """KEEP_STATE=1 continues from the previous call's psi/psi_inv/v like a reused
    FastReg instance (fastreg.cpp:58-75 never clears the solver)."""
    dims = (16, 14, 12)
    d = images(dims, 4)
    P = _params(dims, max_iter=9, alpha=0.03, keep_state=1)
    fr = FastReg(P)
    bufs = [_to(cuda, d[k]) for k in ("T", "labT", "S", "labS")]
    fr(*bufs)
    bufs = [_to(cuda, d[k]) for k in ("T", "labT", "S", "labS")]
    fr(*bufs)
    o1 = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
    state = dict(rho=o1["rho"], v=o1["v"], psi=o1["psi"], psi_inv=o1["psi_inv"])
    o2 = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"], state=state)
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), o2["psi"], "psi after 2 calls")
    assert_bitexact(bufs[2].cpu().numpy(), o2["out_S"], "S o psi after 2 calls")


GOLDEN = sorted((__import__("pathlib").Path(__file__).resolve().parent / "golden").glob("ref_*.npz"))


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_cuda_path_matches_reference_kernels(cuda, path):
    """The CUDA path against the outputs of the reference's own CUDA kernels
    (tests/golden, made by tests/golden/make_golden.py): bit for bit on psi,
    psi_inv, the warped images and the warped labels."""
    f = np.load(path)
    dims = tuple(int(v) for v in f["dims"])
    pv = f["params"]
    P = Params(volume_dims=dims, no_labels=4, max_iter=int(pv[0]), reset_iter=int(pv[1]),
               max_update_norm=float(pv[2]), rho_0=float(pv[3]), tau=float(pv[4]), w_reg=float(pv[5]),
               alpha=float(pv[6]), p=float(pv[7]), C=float(pv[8]))
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, f[k]) for k in ("T", "labT", "S", "labS"))
    fr(iT, lT, iS, lS)
    assert fr.stats().iterations == int(f["iterations"])
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), f["psi"], "psi")
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI_INV).cpu().numpy(), f["psi_inv"], "psi_inv")
    assert_bitexact(iT.cpu().numpy(), f["out_T"], "T o psi_inv")
    assert_bitexact(iS.cpu().numpy(), f["out_S"], "S o psi")
    assert_bitexact(lT.cpu().numpy(), f["out_labT"], "labels T o psi_inv")
    assert_bitexact(lS.cpu().numpy(), f["out_labS"], "labels S o psi")
    norms, vox = fr.trace()
    assert np.abs(norms.astype(np.float64) - f["trace_norm"]).max() <= 1e-6 * float(np.abs(f["trace_norm"]).max())
    assert_bitexact(vox, f["trace_idx"], "max update voxels")
    fr.close()


def test_verbose_mode_prints_and_matches_graph_mode(cuda, capfd):
    """verbosity 1 runs the host-driven loop with the reference's prints (energy at
    iteration 1, every 100 and the last; max update norm; Dice) and the same bits as the
    graph path (solver.cu:329-433)."""
    dims = (20, 18, 16)
    d = images(dims, 61)
    out = {}
    for verbosity in (0, 1):
        P = _params(dims, max_iter=12, alpha=0.03, verbosity=verbosity)
        fr = FastReg(P)
        bufs = [_to(cuda, d[k]) for k in ("T", "labT", "S", "labS")]
        fr(*bufs)
        out[verbosity] = (fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), bufs[2].cpu().numpy(), fr.stats())
        fr.close()
    text = capfd.readouterr().out
    assert "iter. no. 1" in text and "data energy + w_reg * reg energy" in text
    assert "max. update norm" in text and "DICE COEFFICIENT" in text
    assert_bitexact(out[1][0], out[0][0], "psi (verbose vs graph)")
    assert_bitexact(out[1][1], out[0][1], "S o psi (verbose vs graph)")
    assert out[1][2].e_data == out[0][2].e_data


def test_field_ops_vs_oracle_and_reference(cuda):
    """fr_estimate_inverse (one launch, all sweeps per thread) and fr_interpolate_field
    against the oracle bit for bit, on the golden inputs and on odd-sized random fields,
    and against the reference's own kernels run here when their cubins are present."""
    import torch
    from pathlib import Path
    from fastreg_gb300 import estimate_inverse, interpolate_field
    from oracle import ref_runner
    f = np.load(Path(__file__).resolve().parent / "golden" / "field_ops.npz")
    cases = {n: (f[f"{n}_psi"], f[f"{n}_psi_inv0"], f[f"{n}_field"], f[f"{n}_pos"])
             for n in sorted({k.split("_")[0] for k in f.files})}
    r = np.random.Generator(np.random.PCG64(9))
    Z, Y, X = 7, 10, 15
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    idn = np.stack([xx, yy, zz]).astype(np.float32)
    cen = np.array([(X - 1) / 2, (Y - 1) / 2, (Z - 1) / 2], np.float32).reshape(3, 1, 1, 1)
    cases["random"] = ((-(cen + 0.4 * (idn - cen)) + r.normal(0, 0.6, idn.shape)).astype(np.float32), idn,
                       r.normal(0, 1, idn.shape).astype(np.float32),
                       (idn + r.uniform(-3, 3, idn.shape)).astype(np.float32))
    for name, (psi, pinv0, field, pos) in cases.items():
        for sweeps in (1, 48):
            got = estimate_inverse(_to(cuda, psi), _to(cuda, pinv0.copy()), sweeps).cpu().numpy()
            assert_bitexact(got, O.estimate_inverse(psi, pinv0, sweeps), f"estimate_inverse {name} x{sweeps}")
            if sweeps == 48 and ref_runner.available():
                assert_bitexact(got, ref_runner.estimate_inverse(psi, pinv0, 48), f"vs reference {name}")
        got = interpolate_field(_to(cuda, field), _to(cuda, pos)).cpu().numpy()
        assert_bitexact(got, O.interpolate_field(field, pos), f"interpolate_field {name}")
        if ref_runner.available():
            assert_bitexact(got, ref_runner.interpolate_gradient(field, pos), f"interpolate vs reference {name}")


@pytest.mark.parametrize("kw", [dict(p=1.5, C=0.5, tau=0.1, rho_0=0.8, w_reg=0.05, alpha=0.03),
                                dict(p=3.0, C=0.1, tau=0.35, rho_0=1.3, w_reg=0.6, alpha=0.01)])
def test_nondefault_solver_constants(cuda, kw):
    """Other values of the params.ini constants (the t^(p-2) factor below and above 1,
    density start, diffusion and regularisation weights): a registration bit for bit."""
    dims = (21, 19, 17)
    d = images(dims, 77)
    P = _params(dims, max_iter=30, **kw)
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, d[k]) for k in ("T", "labT", "S", "labS"))
    fr(iT, lT, iS, lS)
    o = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
    norms, vox = fr.trace()
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), o["psi"], "psi")
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI_INV).cpu().numpy(), o["psi_inv"], "psi_inv")
    assert_bitexact(fr.get_field(N.FR_FIELD_RHO).cpu().numpy(), o["rho"], "rho")
    assert_bitexact(iS.cpu().numpy(), o["out_S"], "S o psi")
    assert_bitexact(iT.cpu().numpy(), o["out_T"], "T o psi_inv")
    assert_bitexact(norms, o["trace_norm"], "max update norms")
    fr.close()


def test_two_handles_interleaved(cuda):
    """Two handles of different sizes and solvers used alternately, each on its own
    stream: every call gives the oracle's bits (no state, graph or tuned shape leaks
    between handles)."""
    import torch
    da, db = (19, 13, 11), (26, 22, 14)
    pa, pb = images(da, 501), images(db, 502)
    Pa = _params(da, max_iter=12, alpha=0.02)
    Pb = Params(volume_dims=db, no_labels=4, max_iter=10, solver="sobolev", smooth_sigma=1.5, smooth_width=7,
                damping=0.9, step=0.5)
    oa = O.ref_register(Pa, pa["T"], pa["labT"], pa["S"], pa["labS"])
    ob = O.sob_register(Pb, pb["T"], pb["S"])
    fa, fb = FastReg(Pa), FastReg(Pb)
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(2):
        ba = [_to(cuda, pa[k]) for k in ("T", "labT", "S", "labS")]
        bb = [_to(cuda, pb[k]) for k in ("T", "labT", "S", "labS")]
        torch.cuda.synchronize()
        fa(*ba, stream=sa)
        fb(*bb, stream=sb)
        torch.cuda.synchronize()
        assert_bitexact(fa.get_field(N.FR_FIELD_PSI).cpu().numpy(), oa["psi"], "reference handle psi")
        assert_bitexact(ba[2].cpu().numpy(), oa["out_S"], "reference handle S o psi")
        assert_bitexact(fb.get_field(N.FR_FIELD_PSI).cpu().numpy(), ob["phi"], "sobolev handle phi")
    fa.close()
    fb.close()
