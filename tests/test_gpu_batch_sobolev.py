"""Batched cohorts and the sobolev solver on the GPU against the CPU oracle."""
import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N
from oracle import oracle as O
from tests.helpers import assert_bitexact, images, rel_err

pytestmark = pytest.mark.gpu


def _to(dev, a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("staging", [1, 2])
@pytest.mark.parametrize("solver", ["reference", "sobolev"])
def test_batch_equals_pairs_alone(cuda, solver, staging):
    """A cohort of uneven pairs in one set of launches gives, pair by pair, the bits
    of each pair registered alone (and of the oracle), with either staging."""
    dims_list = [(20, 18, 16), (33, 17, 21), (16, 24, 12), (40, 9, 10), (4, 4, 5)]
    kw = dict(no_labels=4, max_iter=25, alpha=0.02, solver=solver, step=0.5, damping=0.9, staging=staging)
    pairs_np = [images(d, 50 + k) for k, d in enumerate(dims_list)]
    P = Params(volume_dims=dims_list[0], **kw)
    fr = FastReg(P)
    bufs = [tuple(_to(cuda, p[k]) for k in ("T", "labT", "S", "labS")) for p in pairs_np]
    fr.register_batch(bufs)
    for k, (d, p) in enumerate(zip(dims_list, pairs_np)):
        psi_b = fr.get_field(N.FR_FIELD_PSI, pair=k).cpu().numpy()
        Pk = Params(volume_dims=d, **kw)
        if solver == "reference":
            o = O.ref_register(Pk, p["T"], p["labT"], p["S"], p["labS"])
            assert_bitexact(psi_b, o["psi"], f"pair {k} psi")
            assert_bitexact(bufs[k][2].cpu().numpy(), o["out_S"], f"pair {k} S o psi")
            assert_bitexact(bufs[k][3].cpu().numpy(), o["out_labS"], f"pair {k} labels")
            assert_bitexact(bufs[k][0].cpu().numpy(), o["out_T"], f"pair {k} T o psi_inv")
        else:
            o = O.sob_register(Pk, p["T"], p["S"])
            assert_bitexact(psi_b, o["phi"], f"pair {k} phi")
            w = O.warp(o["phi"], p["S"])
            assert_bitexact(bufs[k][2].cpu().numpy(), w, f"pair {k} S o phi")
            lab = O.warp_nearest_label(o["phi"], p["labS"])
            assert_bitexact(bufs[k][3].cpu().numpy(), lab, f"pair {k} nearest labels")
        st = fr.stats(pair=k)
        assert st.iterations == 25


@pytest.mark.parametrize("staging", [1, 2])
@pytest.mark.parametrize("dims", [(4, 5, 4), (12, 10, 9), (33, 17, 20)])
def test_sobolev_registration(cuda, dims, staging):
    d = images(dims, 11 + dims[0])
    P = Params(volume_dims=dims, no_labels=4, max_iter=30, solver="sobolev", smooth_sigma=1.5, smooth_width=7,
               damping=0.9, step=0.5, staging=staging)
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, d[k]) for k in ("T", "labT", "S", "labS"))
    fr(iT, lT, iS, lS)
    phi = fr.get_field(N.FR_FIELD_PSI).cpu().numpy()
    m = fr.get_field(N.FR_FIELD_V).cpu().numpy()
    o = O.sob_register(P, d["T"], d["S"])
    assert_bitexact(phi, o["phi"], "phi")
    assert_bitexact(m, o["m"], "momentum")
    norms, vox = fr.trace()
    assert_bitexact(norms, o["trace_norm"], "update norms")
    assert_bitexact(vox, o["trace_idx"], "update voxels")
    # targets are left as they are by the sobolev solver
    assert_bitexact(iT.cpu().numpy(), d["T"], "T unchanged")
    st = fr.stats()
    W = O.warp(o["phi"], d["S"])
    e = 0.5 * float(((d["T"].astype(np.float64) - W.astype(np.float64)) ** 2).sum())
    assert rel_err(st.e_data, e) < 1e-12
    o64 = O.sob_register(P, d["T"], d["S"], prec=64)
    err = np.abs(phi - o64["phi"]).max()
    assert err < 1e-3, f"phi vs FP64 oracle: max abs err {err} voxels"


@pytest.mark.parametrize("staging", [1, 2])
@pytest.mark.parametrize("width", [1, 3, 5, 7, 9, 11, 13, 15])
def test_sobolev_smoothing_widths(cuda, width, staging):
    """Every smoothing radius with either staging (one kernel instance per radius and
    staging: cp.async or TMA copies, an x halo of 4 or 8 columns, 2 to 4 staging buffers,
    clamped rows and columns at the volume's edges) gives the oracle's bits; odd sizes put
    most tiles on an x edge."""
    dims = (37, 19, 23)
    d = images(dims, 300 + width)
    P = Params(volume_dims=dims, no_labels=4, max_iter=6, solver="sobolev", smooth_sigma=0.4 + 0.3 * width,
               smooth_width=width, damping=0.9, step=0.5, staging=staging)
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, d[k]) for k in ("T", "labT", "S", "labS"))
    fr(iT, lT, iS, lS)
    o = O.sob_register(P, d["T"], d["S"])
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), o["phi"], f"phi (width {width})")
    assert_bitexact(fr.get_field(N.FR_FIELD_V).cpu().numpy(), o["m"], f"momentum (width {width})")


@pytest.mark.parametrize("solver", ["reference", "sobolev"])
def test_autotuned_shapes_do_not_change_results(cuda, solver):
    """AUTOTUNE=1 times tile depths and blocks per SM per kernel and keeps the fastest;
    the fields are bit-identical to AUTOTUNE=0's default shapes, and the chosen shapes
    are among the candidates."""
    dims_list = [(41, 23, 29), (20, 18, 16)]
    # the depth candidates: a fixed ladder and ceil(Zmax / k), k = 1..32 (Zmax = 29 here)
    zmax = max(d[2] for d in dims_list)
    candidates = {1, 2, 4, 8, 12, 16, 24, 32, 48, 64, 96} | {-(-zmax // k) for k in range(1, 33)}
    kw = dict(no_labels=4, max_iter=12, alpha=0.02, solver=solver, step=0.5, damping=0.9)
    pairs_np = [images(d, 700 + k) for k, d in enumerate(dims_list)]
    fields = []
    for tune in (0, 1):
        fr = FastReg(Params(volume_dims=dims_list[0], autotune=tune, **kw))
        bufs = [tuple(_to(cuda, p[k]) for k in ("T", "labT", "S", "labS")) for p in pairs_np]
        fr.register_batch(bufs)
        fields.append([fr.get_field(N.FR_FIELD_PSI, pair=k).cpu().numpy() for k in range(len(dims_list))])
        shapes = fr.tile_shapes()
        assert all(d in candidates and (b >= 1 or b == -1) for d, b in shapes), shapes
        if not tune:
            default = (16, 24, 24) if solver == "reference" else (12, 32, 8)
            assert tuple(d for d, _ in shapes) == default, shapes
        fr.close()
    for k in range(len(dims_list)):
        assert_bitexact(fields[1][k], fields[0][k], f"pair {k} psi, autotuned vs default shapes")


@pytest.mark.parametrize("solver", ["reference", "sobolev"])
def test_per_pair_w_reg(cuda, solver):
    """fr_set_pair_w_reg: one batched registration with a regularisation weight per pair
    gives, pair by pair, the oracle's bits for that pair's W_REG; the energy uses it."""
    dims_list = [(20, 18, 16), (33, 17, 21), (16, 24, 12)]
    weights = [0.05, 0.2, 0.6]
    kw = dict(no_labels=4, max_iter=20, alpha=0.02, solver=solver, step=0.5, damping=0.9)
    pairs_np = [images(d, 900 + k) for k, d in enumerate(dims_list)]
    fr = FastReg(Params(volume_dims=dims_list[0], w_reg=0.3, **kw))
    fr.set_pair_w_reg(weights)
    bufs = [tuple(_to(cuda, p[k]) for k in ("T", "labT", "S", "labS")) for p in pairs_np]
    fr.register_batch(bufs)
    for k, (d, p) in enumerate(zip(dims_list, pairs_np)):
        Pk = Params(volume_dims=d, w_reg=weights[k], **kw)
        psi = fr.get_field(N.FR_FIELD_PSI, pair=k).cpu().numpy()
        if solver == "reference":
            o = O.ref_register(Pk, p["T"], p["labT"], p["S"], p["labS"])
            assert_bitexact(psi, o["psi"], f"pair {k} psi (w_reg {weights[k]})")
        else:
            o = O.sob_register(Pk, p["T"], p["S"])
            assert_bitexact(psi, o["phi"], f"pair {k} phi (w_reg {weights[k]})")
        st = fr.stats(pair=k)
        assert abs(st.energy - (st.e_data + float(np.float32(weights[k])) * st.e_reg)) <= 1e-12 * abs(st.energy)
    fr.set_pair_w_reg([0.1])  # one weight for three pairs
    with pytest.raises(N.FastRegError):
        fr.register_batch(bufs)
    fr.set_pair_w_reg(None)  # back to W_REG = 0.3 for every pair
    fr.register_batch([tuple(_to(cuda, pairs_np[0][k]) for k in ("T", "labT", "S", "labS"))])  # fresh inputs
    o = (O.ref_register(Params(volume_dims=dims_list[0], w_reg=0.3, **kw), *(pairs_np[0][k] for k in
                                                                                ("T", "labT", "S", "labS")))
         if solver == "reference" else O.sob_register(Params(volume_dims=dims_list[0], w_reg=0.3, **kw),
                                                       pairs_np[0]["T"], pairs_np[0]["S"]))
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), o["psi" if solver == "reference" else "phi"], "W_REG")
    fr.close()


@pytest.mark.parametrize("solver", ["reference", "sobolev"])
def test_batched_convergence_and_keep_state(cuda, solver):
    """One MAX_UPDATE_NORM for a cohort whose pairs converge at different iterations (the
    graph keeps launching; a stopped pair's tiles are skipped): each pair stops where the
    oracle's loop breaks, with the oracle's fields.  For the reference solver a second
    call with KEEP_STATE=1 then continues every pair from its own final state, whatever
    the parity of the iteration it stopped at."""
    dims_list = [(24, 20, 18), (20, 18, 16), (16, 24, 12), (18, 15, 21)]
    pairs_np = [images(d, 1300 + k) for k, d in enumerate(dims_list)]
    kw = dict(no_labels=4, max_iter=40, alpha=0.02, solver=solver, step=0.5, damping=0.9)

    def oracle(dims, p, P, state=None):
        if solver == "reference":
            return O.ref_register(P, p["T"], p["labT"], p["S"], p["labS"], state=state)
        o = O.sob_register(P, p["T"], p["S"])
        o["psi"] = o["phi"]
        return o

    # thresholds inside the pairs' update-norm traces: the reference solver's norms halve at
    # iteration 2 and then grow (stops at 1, 2, 2 and none); the sobolev solver's rise and
    # decay (stops at 40, 24, 1 and none)
    kw["max_update_norm"] = 3e-6 if solver == "reference" else 2.7e-3
    expect = [oracle(d, p, Params(volume_dims=d, **kw)) for d, p in zip(dims_list, pairs_np)]
    stops = [o["iterations"] if o["converged"] else None for o in expect]
    assert None in stops and len(set(stops)) >= 3, stops

    fr = FastReg(Params(volume_dims=dims_list[0], keep_state=1 if solver == "reference" else 0, **kw))
    bufs = [tuple(_to(cuda, p[k]) for k in ("T", "labT", "S", "labS")) for p in pairs_np]
    fr.register_batch(bufs)
    for k, o in enumerate(expect):
        st = fr.stats(pair=k)
        assert st.iterations == o["iterations"] and st.converged == o["converged"], (k, st.iterations, o["iterations"])
        assert_bitexact(fr.get_field(N.FR_FIELD_PSI, pair=k).cpu().numpy(), o["psi"], f"pair {k} psi")
        if solver == "reference":
            assert_bitexact(fr.get_field(N.FR_FIELD_PSI_INV, pair=k).cpu().numpy(), o["psi_inv"], f"pair {k} psi_inv")
            assert_bitexact(bufs[k][2].cpu().numpy(), o["out_S"], f"pair {k} S o psi")
            assert_bitexact(bufs[k][0].cpu().numpy(), o["out_T"], f"pair {k} T o psi_inv")
    if solver != "reference":
        return
    bufs = [tuple(_to(cuda, p[k]) for k in ("T", "labT", "S", "labS")) for p in pairs_np]
    fr.register_batch(bufs)
    for k, (d, p, o1) in enumerate(zip(dims_list, pairs_np, expect)):
        state = dict(rho=o1["rho"], v=o1["v"], psi=o1["psi"], psi_inv=o1["psi_inv"])
        o2 = oracle(d, p, Params(volume_dims=d, keep_state=1, **kw), state=state)
        assert fr.stats(pair=k).iterations == o2["iterations"]
        assert_bitexact(fr.get_field(N.FR_FIELD_PSI, pair=k).cpu().numpy(), o2["psi"], f"pair {k} psi, 2nd call")
        assert_bitexact(bufs[k][2].cpu().numpy(), o2["out_S"], f"pair {k} S o psi, 2nd call")
