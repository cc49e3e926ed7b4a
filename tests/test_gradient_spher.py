"""Misfit gradient of the spherical GPU-program scheme (sfAWEFDspher3Dgpu's
step, the scheme of the spherical-shell workload) on the engine's discrete adjoint,
against the FP64 adjoint oracle (oracle/awe_adjoint_sph.c), which is pinned
by finite differences of its own FP64 misfit."""
import numpy as np
import pytest

from helpers import rel_l2, spher_desc, spher_grad_case


def _dobs(par, vtrue, wav, sou, rec):
    from oracle import oracle

    _, _, d = oracle.spher3d_gradient(par, vtrue, wav, sou, rec, np.zeros((par["nt"], rec.shape[0])))
    return d.astype(np.float32)


@pytest.mark.parametrize("fsrf", [0, 1])
def test_oracle_gradient_matches_finite_differences(fsrf):
    """Centred differences of the FP64 misfit in m = 1/v^2 (double model
    path), Richardson-extrapolated over steps 1e-3 and 5e-4, along 3 seeded
    directions."""
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = spher_grad_case(fsrf=fsrf)
    dobs = _dobs(par, vtrue, wav, sou, rec)
    m = 1.0 / vel.astype(np.float64) ** 2
    g, J, _ = oracle.spher3d_gradient(par, vel, wav, sou, rec, dobs, m=m)
    assert J > 0
    rng = np.random.default_rng(5)
    for _ in range(3):
        dm = rng.standard_normal(m.shape) * m
        fd = []
        for h in (1e-3, 5e-4):
            jp = oracle.spher3d_gradient(par, vel, wav, sou, rec, dobs, m=m + h * dm)[1]
            jm = oracle.spher3d_gradient(par, vel, wav, sou, rec, dobs, m=m - h * dm)[1]
            fd.append((jp - jm) / (2 * h))
        rich = (4 * fd[1] - fd[0]) / 3
        assert abs(float(np.sum(g * dm)) - rich) <= 1e-7 * abs(rich)


def test_oracle_checkpoint_emulation_fp32_is_exact():
    """Rounding the checkpoints to 24 bits (FP32) changes the FP64 oracle
    gradient by no more than float rounding of the restart levels."""
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = spher_grad_case()
    dobs = _dobs(par, vtrue, wav, sou, rec)
    g, J, _ = oracle.spher3d_gradient(par, vel, wav, sou, rec, dobs)
    g24, J24, _ = oracle.spher3d_gradient(par, vel, wav, sou, rec, dobs, ckpt_every=13, ckpt_bits=24)
    assert J24 == J
    assert rel_l2(g24, g) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("fsrf,nr", [(0, 45), (1, 45), (0, 46), (1, 46), (0, 48), (1, 48)])
def test_gradient_matches_fp64_oracle(fsrf, nr):
    """nr = 45: odd padded radius count (one radius per thread); 46: even
    (two radii per thread, packed arithmetic); 48: padded count a multiple of
    4 (the TMA-staged forward, recompute and adjoint kernels)."""
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = spher_grad_case(fsrf=fsrf, n=(nr, 20, 20))
    dobs = _dobs(par, vtrue, wav, sou, rec)
    gref, Jref, dref = oracle.spher3d_gradient(par, vel, wav, sou, rec, dobs)
    T = int(np.ceil(np.sqrt(par["nt"])))
    with awe.Plan(spher_desc(par)) as p:
        assert p.step_kernel == ("tma_sph" if (nr + 2 * par["nb"]) % 4 == 0 else "simple")
        p.set_model(vel)
        p.set_geometry(sou, rec)
        g32, J32, d32 = p.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32, return_dsyn=True)
        gf, Jf = p.gradient(wav, dobs, ckpt_format=awe.CKPT_BFP16)
        gb, Jb = p.gradient(wav, dobs, ckpt_format=awe.CKPT_BF16)
    assert rel_l2(d32, dref) <= 1e-5
    # the residual is a small difference of close trace sets (the true model
    # differs by 5 % in one layer), so the FP32 trace error weighs more in J
    assert abs(J32 - Jref) <= 2e-4 * abs(Jref)
    assert Jf == J32 and Jb == J32  # the misfit comes from the forward pass
    assert rel_l2(g32, gref) <= 1e-4
    # 16-bit checkpoints: the oracle emulates the same rounding in FP64
    for g16, bits, bound in ((gf, -1, 1e-3), (gb, 8, 3e-2)):
        gq, _, _ = oracle.spher3d_gradient(par, vel, wav, sou, rec, dobs, ckpt_every=T, ckpt_bits=bits)
        assert rel_l2(g16, gq) <= 0.5 * rel_l2(gq, gref) + 1e-4
        assert rel_l2(g16, gref) <= bound


@pytest.mark.gpu
@pytest.mark.parametrize("every", [1, 7, 1000])
@pytest.mark.parametrize("nr", [45, 48])
def test_checkpoint_interval_does_not_change_fp32_gradient(every, nr):
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = spher_grad_case(nt=60, n=(nr, 20, 20))
    dobs = _dobs(par, vtrue, wav, sou, rec)
    with awe.Plan(spher_desc(par)) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        ref, Jr = p.gradient(wav, dobs, ckpt_every=0, ckpt_format=awe.CKPT_FP32)
        g, J = p.gradient(wav, dobs, ckpt_every=every, ckpt_format=awe.CKPT_FP32)
    assert J == Jr
    # the recompute repeats the forward exactly; only the order of coincident
    # receiver-corner atomics may differ
    assert rel_l2(g, ref) <= 1e-6


@pytest.mark.gpu
def test_reflectivity_injection_is_refused():
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = spher_grad_case(nt=20)
    par["expl"] = 1
    with awe.Plan(spher_desc(par)) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        with pytest.raises(awe.AweError):
            p.gradient(wav, np.zeros((par["nt"], rec.shape[0]), np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("nr", [46, 48])
def test_several_shots_sum_the_single_shot_gradients(nr):
    """awe_set_shots (the spherical track's layout): the gradient of three shots
    is the sum of the three single-shot gradients, the misfit the sum of
    theirs, the synthetic data each shot's own columns; awe_set_geometry
    afterwards goes back to one shot."""
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = spher_grad_case(n=(nr, 20, 20), nt=80)
    d = par["d"]
    shots = [(sou + np.array([[0.0, k * 3 * d[2], 0.0]], np.float32), rec[: 7 - k]) for k in range(3)]
    dobs = [_dobs(par, vtrue, wav, s_, r_) for s_, r_ in shots]
    with awe.Plan(spher_desc(par)) as p:
        p.set_model(vel)
        gsum, Jsum, dsyn = np.zeros_like(vel, np.float64), 0.0, []
        for (s_, r_), d_ in zip(shots, dobs):
            p.set_geometry(s_, r_)
            g, J, ds = p.gradient(wav, d_, ckpt_format=awe.CKPT_FP32, return_dsyn=True)
            gsum += g
            Jsum += J
            dsyn.append(ds)
        p.set_shots(shots)
        gm, Jm, dsm = p.gradient(wav, np.concatenate(dobs, axis=1), ckpt_format=awe.CKPT_FP32, return_dsyn=True)
        p.set_geometry(*shots[1])
        d1 = p.forward(wav)
    assert rel_l2(gm, gsum) <= 1e-6  # coincident receiver corners add by atomics
    assert abs(Jm - Jsum) <= 1e-9 * Jsum
    np.testing.assert_array_equal(dsm, np.concatenate(dsyn, axis=1))
    np.testing.assert_array_equal(d1, dsyn[1])


@pytest.mark.gpu
def test_empty_point_sets():
    """No receivers: zero misfit and gradient; no sources: zero wavefield,
    so a zero gradient while the misfit is the data's energy."""
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = spher_grad_case(n=(46, 20, 20), nt=40)
    with awe.Plan(spher_desc(par)) as p:
        p.set_model(vel)
        p.set_geometry(sou, np.zeros((0, 3), np.float32))
        g, J = p.gradient(wav, np.zeros((par["nt"], 0), np.float32), ckpt_format=awe.CKPT_FP32)
        assert J == 0.0 and not g.any()
        p.set_geometry(np.zeros((0, 3), np.float32), rec)
        dobs = np.ones((par["nt"], rec.shape[0]), np.float32)
        g, J = p.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32)
        assert J == pytest.approx(0.5 * dobs.size) and not g.any()


@pytest.mark.gpu
@pytest.mark.parametrize("nr", [45, 46, 48])
def test_rtm_images_match_fp64_oracle(nr):
    """awe_rtm on the spherical scheme: zero-lag cross-correlation and Born
    images of recorded data against the FP64 adjoint oracle, and the
    gradient as the Born image of the residual (linearity in the data)."""
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = spher_grad_case(n=(nr, 20, 20), nt=120)
    data = _dobs(par, vtrue, wav, sou, rec)
    with awe.Plan(spher_desc(par)) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        xc = p.rtm(wav, data, condition=awe.IMAGE_XCORR, ckpt_format=awe.CKPT_FP32)
        bo = p.rtm(wav, data, condition=awe.IMAGE_BORN, ckpt_format=awe.CKPT_FP32)
        g, J, dsyn = p.gradient(wav, data, ckpt_format=awe.CKPT_FP32, return_dsyn=True)
        bs = p.rtm(wav, dsyn, condition=awe.IMAGE_BORN, ckpt_format=awe.CKPT_FP32)
    assert rel_l2(xc, oracle.spher3d_image(par, vel, wav, sou, rec, data, 0)) <= 1e-4
    assert rel_l2(bo, oracle.spher3d_image(par, vel, wav, sou, rec, data, 1)) <= 1e-4
    # the two Born images are about 20x larger than their difference (the
    # true model differs by 5 % in one layer), so their FP32 rounding weighs
    # that much more here (the FP64 oracle gives 9e-6 on the same check)
    assert rel_l2(bs - bo, g) <= 5e-4


@pytest.mark.gpu
@pytest.mark.parametrize("fsrf", [0, 1])
def test_tma_kernels_match_register_kernels(monkeypatch, fsrf):
    """The TMA-staged forward, recompute and adjoint (k_stepA_sph_tma,
    k_adjA_sph_tma) against the register-march kernels they replace
    (AWE_STEP_KERNEL=simple): gradient, misfit, synthetic traces and both
    images.  The kernels evaluate the same packed FP32x2 expressions, so the
    bar is rel-L2 1e-6 (float rounding of the order of coincident receiver
    atomics), with 5-plane phi chunks across the grid."""
    import wavefield_imaging_gb300 as awe

    par, vel, wav, sou, rec, vtrue = spher_grad_case(fsrf=fsrf, n=(48, 20, 20), nt=90)
    dobs = _dobs(par, vtrue, wav, sou, rec)
    out = {}
    for kern in ("simple", "tma_sph"):
        if kern == "simple":
            monkeypatch.setenv("AWE_STEP_KERNEL", "simple")
        else:
            monkeypatch.delenv("AWE_STEP_KERNEL", raising=False)
            monkeypatch.setenv("AWE_TMA_CHUNK", "5")
        with awe.Plan(spher_desc(par)) as p:
            assert p.step_kernel == kern
            p.set_model(vel)
            p.set_geometry(sou, rec)
            g, J, d = p.gradient(wav, dobs, ckpt_every=7, ckpt_format=awe.CKPT_FP32, return_dsyn=True)
            xc = p.rtm(wav, dobs, condition=awe.IMAGE_XCORR, ckpt_format=awe.CKPT_FP32)
            bo = p.rtm(wav, dobs, condition=awe.IMAGE_BORN, ckpt_format=awe.CKPT_FP32)
        out[kern] = (g, J, d, xc, bo)
    (g0, J0, d0, x0, b0), (g1, J1, d1, x1, b1) = out["simple"], out["tma_sph"]
    assert np.abs(g0).max() > 0 and np.abs(x0).max() > 0
    assert rel_l2(d1, d0) <= 1e-6
    assert abs(J1 - J0) <= 1e-5 * abs(J0)
    assert rel_l2(g1, g0) <= 1e-6
    assert rel_l2(x1, x0) <= 1e-6
    assert rel_l2(b1, b0) <= 1e-6
