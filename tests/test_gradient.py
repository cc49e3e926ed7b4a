"""The engine's misfit gradient (awe_gradient: hand-written adjoint step,
checkpointed forward, FP64 accumulation) against the FP64 adjoint oracle and
against finite differences through the torch.autograd harness."""
import numpy as np
import pytest

from helpers import desc_from_par, grad_case, rel_l2, tapered_direction

pytestmark = pytest.mark.gpu


def _plan(par, vel, sou, rec):
    import wavefield_imaging_gb300 as awe

    p = awe.Plan(desc_from_par(par, precision=awe.FAST))
    p.set_model(vel)
    p.set_geometry(sou, rec)
    return p


def _observed(par, vtrue, wav, sou, rec):
    from oracle import oracle

    dobs, _ = oracle.cart_cpu(par, vtrue, wav, sou, rec)
    return dobs


@pytest.mark.parametrize("nd,fsrf", [(2, 0), (2, 1), (3, 0), (3, 1)])
def test_gradient_matches_fp64_oracle(nd, fsrf):
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = grad_case(nd, fsrf=fsrf, nt=200 if nd == 2 else 110)
    dobs = _observed(par, vtrue, wav, sou, rec)
    gref, Jref, dref = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs)
    T = int(np.ceil(np.sqrt(par["nt"])))
    with _plan(par, vel, sou, rec) as p:
        g32, J32, d32 = p.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32, return_dsyn=True)
        gb, Jb = p.gradient(wav, dobs, ckpt_format=awe.CKPT_BF16)
        gh, Jh = p.gradient(wav, dobs, ckpt_format=awe.CKPT_FP16)
        gf, Jf = p.gradient(wav, dobs, ckpt_format=awe.CKPT_BFP16)
    assert rel_l2(d32, dref) <= 1e-5
    assert abs(J32 - Jref) <= 1e-5 * abs(Jref)
    assert Jb == J32 and Jh == J32 and Jf == J32  # the misfit comes from the forward pass, not the checkpoints
    # FP32 checkpoints: only the FP32 arithmetic differs from the FP64 oracle
    assert rel_l2(g32, gref) <= 1e-4
    # 16-bit checkpoints: the recomputed segments start from levels rounded to
    # 8 (BF16) or 11 (FP16) significant bits, or to 16-bit integers with a
    # scale per 64 cells (BFP16, emulated as ckpt_bits=-1).  The oracle
    # emulates the same rounding in FP64; the engine must match that, and the
    # error it leaves against the exact gradient is the checkpoint format's,
    # not the kernels'.  BFP16 meets the 1e-3 gradient bound at 2 bytes/cell.
    for g16, bits, bound in ((gb, 8, 3e-2), (gh, 11, 4e-3), (gf, -1, 1e-3)):
        gq, _, _ = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, ckpt_every=T, ckpt_bits=bits)
        assert rel_l2(g16, gq) <= 0.5 * rel_l2(gq, gref) + 1e-4
        assert rel_l2(g16, gref) <= bound


@pytest.mark.parametrize("every", [1, 7, 1000])
def test_checkpoint_interval_does_not_change_fp32_gradient(every):
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = grad_case(3, nt=60)
    dobs = _observed(par, vtrue, wav, sou, rec)
    with _plan(par, vel, sou, rec) as p:
        ref, Jr = p.gradient(wav, dobs, ckpt_every=0, ckpt_format=awe.CKPT_FP32)
        g, J = p.gradient(wav, dobs, ckpt_every=every, ckpt_format=awe.CKPT_FP32)
    assert J == Jr
    # recompute from FP32 checkpoints repeats the forward exactly; only the
    # order of coincident receiver-corner atomics may differ
    assert rel_l2(g, ref) <= 1e-6


def test_gradient_with_decimated_data():
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = grad_case(2, nt=180)
    par["jdata"] = 4
    dobs = _observed(par, vtrue, wav, sou, rec)[::4]
    gref, Jref, _ = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, jdata=4)
    with _plan(par, vel, sou, rec) as p:
        g, J = p.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32)
    assert abs(J - Jref) <= 1e-5 * abs(Jref)
    assert rel_l2(g, gref) <= 1e-4


@pytest.mark.parametrize("nd", [2, 3])
def test_autograd_harness_against_finite_differences(nd):
    """8 seeded directions, relative step 1e-3, through torch.autograd."""
    torch = pytest.importorskip("torch")
    import wavefield_imaging_gb300 as awe
    from wavefield_imaging_gb300.autograd import misfit

    par, vel, wav, sou, rec, vtrue = grad_case(nd, nt=200 if nd == 2 else 110)
    dobs = _observed(par, vtrue, wav, sou, rec)
    m0 = torch.tensor(1.0 / vel.astype(np.float64) ** 2, dtype=torch.float64, device="cuda")
    with _plan(par, vel, sou, rec) as p:
        m = m0.clone().requires_grad_(True)
        J = misfit(m, p, wav, dobs, ckpt_format=awe.CKPT_FP32)
        J.backward()
        g = m.grad.detach().cpu().numpy()
        rng = np.random.default_rng(2024)
        errs = []
        for _ in range(8):
            dm = tapered_direction(vel.shape, rng) * m0.cpu().numpy()
            h = 1e-3
            Jp = float(misfit(m0 + h * torch.tensor(dm, device="cuda"), p, wav, dobs))
            Jm = float(misfit(m0 - h * torch.tensor(dm, device="cuda"), p, wav, dobs))
            fd = (Jp - Jm) / (2 * h)
            an = float((g * dm).sum())
            errs.append(abs(fd - an) / abs(an))
    # FP32 forward: J carries ~1e-7 relative rounding, amplified by 1/h in the
    # difference quotient
    assert max(errs) <= 1e-2, errs


def test_gradient_rejects_unsupported_plans():
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = grad_case(2, nt=20)
    dobs = np.zeros((20, rec.shape[0]), np.float32)
    with awe.Plan(desc_from_par(par, precision=awe.EXACT)) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        with pytest.raises(awe.AweError):
            p.gradient(wav, dobs)
    par_h = dict(par, hybrid=1)
    with awe.Plan(desc_from_par(par_h, precision=awe.FAST)) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        with pytest.raises(awe.AweError):
            p.gradient(wav, dobs)


@pytest.mark.gpu
@pytest.mark.parametrize("nd", [2, 3])
def test_repeated_gradient_replays_the_captured_graph(nd):
    """The first call with given buffers runs directly, the second captures
    the gradient as a CUDA graph and replays it, later calls replay: all
    give the same gradient, misfit and synthetic data (the 2D adjoint adds
    receivers from per-cell lists, so bit for bit; 3D within float atomics)."""
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = grad_case(nd, nt=80 if nd == 2 else 40)
    dobs = _observed(par, vtrue, wav, sou, rec)
    with _plan(par, vel, sou, rec) as p:
        runs = [p.gradient(wav, dobs, ckpt_format=awe.CKPT_BFP16, return_dsyn=True) for _ in range(4)]
        p.set_model((vel * 1.01).astype(np.float32))  # drops the graph: direct run, then capture again
        again = [p.gradient(wav, dobs, ckpt_format=awe.CKPT_BFP16, return_dsyn=True) for _ in range(3)]
    for runs_ in (runs, again):
        g0, J0, d0 = runs_[0]
        for g, J, d in runs_[1:]:
            assert J == J0
            np.testing.assert_array_equal(d, d0)
            if nd == 2:
                np.testing.assert_array_equal(g, g0)
            else:
                assert rel_l2(g, g0) <= 1e-6
    assert again[0][1] != runs[0][1]


@pytest.mark.gpu
@pytest.mark.parametrize("nd", [2, 3])
def test_empty_point_sets(nd):
    """No receivers: zero misfit and gradient; no sources: zero wavefield,
    so a zero gradient while the misfit is the data's energy."""
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = grad_case(nd, nt=40)
    with _plan(par, vel, sou, np.zeros((0, nd), np.float32)) as p:
        g, J = p.gradient(wav, np.zeros((40, 0), np.float32), ckpt_format=awe.CKPT_FP32)
        assert J == 0.0 and not g.any()
    with _plan(par, vel, np.zeros((0, nd), np.float32), rec) as p:
        dobs = np.ones((40, rec.shape[0]), np.float32)
        g, J = p.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32)
        assert J == pytest.approx(0.5 * dobs.size) and not g.any()


@pytest.mark.parametrize("fsrf,n", [(0, None), (1, None), (0, [120, 40, 30]), (1, [120, 40, 30])])
def test_single_boundary_launch_matches_separate_launches(monkeypatch, fsrf, n):
    """3D gradient on the TMA path: the one boundary launch per adjoint step
    (kappa fold, transposed ABC of the six faces, g = I vel2 nu: k_bnd3_adj)
    against the separate launches it replaces (AWE_BND3=0), for the gradient
    and both images; the larger grid has several axis-1 and axis-2 ranges of
    face blocks.  The fold moves from after the adjoint step to the next
    step's launch, so only its order against the receiver term may differ."""
    import wavefield_imaging_gb300 as awe

    # the larger grid needs the steps for the wave to reach its receivers
    par, vel, wav, sou, rec, vtrue = grad_case(3, fsrf=fsrf, nt=70 if n is None else 260, n=n)
    dobs = _observed(par, vtrue, wav, sou, rec)
    out = {}
    for env in ("0", "1"):
        monkeypatch.setenv("AWE_BND3", env)
        with _plan(par, vel, sou, rec) as p:
            assert p.step_kernel == "tma3d"
            g, J = p.gradient(wav, dobs, ckpt_every=9, ckpt_format=awe.CKPT_FP32)
            xc = p.rtm(wav, dobs, condition=awe.IMAGE_XCORR, ckpt_format=awe.CKPT_FP32)
            bo = p.rtm(wav, dobs, condition=awe.IMAGE_BORN, ckpt_format=awe.CKPT_FP32)
        out[env] = (g, J, xc, bo)
    (g0, J0, x0, b0), (g1, J1, x1, b1) = out["0"], out["1"]
    assert np.abs(g0).max() > 0 and np.abs(x0).max() > 0
    assert J1 == J0
    assert rel_l2(g1, g0) <= 1e-6
    assert rel_l2(x1, x0) <= 1e-6
    assert rel_l2(b1, b0) <= 1e-6
