"""The FP64 adjoint oracle (oracle/awe_adjoint.c) against finite differences
of its own misfit, and its forward data against the float restatement of the
reference scheme.  CPU only."""
import numpy as np
import pytest

from helpers import grad_case, tapered_direction


@pytest.mark.parametrize("nd,fsrf", [(2, 0), (2, 1), (3, 0), (3, 1)])
def test_oracle_gradient_matches_finite_differences(nd, fsrf):
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = grad_case(nd, fsrf=fsrf, nt=160 if nd == 2 else 90)
    dobs, _ = oracle.cart_cpu(par, vtrue, wav, sou, rec)
    g, J, dsyn = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs)
    d32, _ = oracle.cart_cpu(par, vel, wav, sou, rec)
    # FP64 run of the same scheme against the float restatement
    assert np.linalg.norm(dsyn - d32) / np.linalg.norm(dsyn) < 1e-5
    rng = np.random.default_rng(11)
    m = 1.0 / vel.astype(np.float64) ** 2
    gm, _, _ = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, m=m)
    # the float-velocity and double-slowness models differ only by rounding
    assert np.linalg.norm(gm - g) <= 1e-5 * np.linalg.norm(g)
    for _ in range(2):
        dm = tapered_direction(vel.shape, rng) * m
        an = float((gm * dm).sum())
        fds = []
        for h in (1e-3, 5e-4):
            Jp = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, m=m + h * dm)[1]
            Jm = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, m=m - h * dm)[1]
            fds.append((Jp - Jm) / (2 * h))
        # central differences converge as h^2: Richardson-extrapolate the pair
        fd = (4 * fds[1] - fds[0]) / 3
        assert abs(fd - an) <= 1e-7 * abs(an)


def test_oracle_gradient_with_decimated_data():
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = grad_case(2, nt=150)
    dobs_full, _ = oracle.cart_cpu(par, vtrue, wav, sou, rec)
    dobs = dobs_full[::3]
    g, J, dsyn = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, jdata=3)
    assert dsyn.shape == dobs.shape
    rng = np.random.default_rng(12)
    m = 1.0 / vel.astype(np.float64) ** 2
    g, _, _ = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, jdata=3, m=m)
    dm = tapered_direction(vel.shape, rng) * m
    fds = []
    for h in (1e-3, 5e-4):
        Jp = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, jdata=3, m=m + h * dm)[1]
        Jm = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, jdata=3, m=m - h * dm)[1]
        fds.append((Jp - Jm) / (2 * h))
    an = float((g * dm).sum())
    assert abs((4 * fds[1] - fds[0]) / 3 - an) <= 1e-7 * abs(an)


def test_checkpoint_rounding_emulation_converges():
    """Recompute from rounded checkpoints: the gradient error falls as the
    stored precision rises (8, 11, 24 significant bits)."""
    from oracle import oracle
    from helpers import rel_l2

    par, vel, wav, sou, rec, vtrue = grad_case(2, nt=150)
    dobs, _ = oracle.cart_cpu(par, vtrue, wav, sou, rec)
    g, _, _ = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs)
    errs = [rel_l2(oracle.misfit_gradient(par, vel, wav, sou, rec, dobs, ckpt_every=13, ckpt_bits=b)[0], g)
            for b in (8, 11, 24)]
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 1e-6


def test_oracle_born_image_is_linear_in_the_data():
    """The FP64 Born image (the gradient formula with the data as residual)
    satisfies grad(dobs) = born(dsyn) - born(dobs); the cross-correlation
    image is nonzero and finite."""
    from oracle import oracle

    par, vel, wav, sou, rec, vtrue = grad_case(2, nt=120)
    dobs, _ = oracle.cart_cpu(par, vtrue, wav, sou, rec)
    g, _, dsyn = oracle.misfit_gradient(par, vel, wav, sou, rec, dobs)
    b_syn = oracle.rtm_image(par, vel, wav, sou, rec, dsyn.astype(np.float32), 1)
    b_obs = oracle.rtm_image(par, vel, wav, sou, rec, dobs, 1)
    assert np.linalg.norm(g - (b_syn - b_obs)) <= 1e-6 * np.linalg.norm(g)
    x = oracle.rtm_image(par, vel, wav, sou, rec, dobs, 0)
    assert np.isfinite(x).all() and np.abs(x).max() > 0
