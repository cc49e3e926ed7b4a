"""Multi-rank path on CPU (gloo, world size 2): shot sharding, the single
end-of-run gradient reduction, and bench.py's max-over-ranks timing helper.
The per-shot gradients come from the FP64 oracle, so no GPU is needed."""
import os
import socket

import numpy as np
import pytest

from helpers import ricker

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _survey():
    rng = np.random.default_rng(6)
    nz, nxm, nt = 40, 120, 120
    vel = (150.0 + 30.0 * rng.random((nxm, nz))).astype(np.float32)
    vtrue = (vel * (1 + 0.04 * rng.standard_normal(vel.shape))).astype(np.float32)
    shots = []
    for i in range(5):
        nx = int(rng.integers(40, 60))
        x0 = int(rng.integers(0, nxm - nx))
        xs = (x0 + nx / 2) * 5.0
        sou = np.array([[xs, 40.0]], np.float32)
        rec = np.stack([np.linspace(xs - 60, xs + 60, 7), np.full(7, 30.0)], 1).astype(np.float32)
        shots.append((x0, nx, sou, rec))
    return vel, vtrue, shots, nz, nt


def _shot_gradient(vel, vtrue, shot, nz, nt):
    from oracle import oracle

    x0, nx, sou, rec = shot
    par = dict(n=[nz, nx], d=[5.0, 5.0], o=[0.0, x0 * 5.0], nb=8, nt=nt, dt=0.005, fdorder=8, dabc=1, expl=1)
    wav = ricker(nt, 0.005)
    dobs, _ = oracle.cart_cpu(par, vtrue[x0:x0 + nx], wav, sou, rec)
    g, J, _ = oracle.misfit_gradient(par, vel[x0:x0 + nx], wav, sou, rec, dobs)
    full = np.zeros(vel.shape, np.float64)
    full[x0:x0 + nx] = g
    return full, J


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    from wavefield_imaging_gb300.replicas import reduce_gradient, shard

    d, r, w, _ = bench.dist_init()
    assert (r, w) == (rank, world) and d is not None
    vel, vtrue, shots, nz, nt = _survey()
    grad = np.zeros(vel.shape, np.float64)
    J = 0.0
    for shot in shard(shots, rank, world):
        g, j = _shot_gradient(vel, vtrue, shot, nz, nt)
        grad += g
        J += j
    grad, J = reduce_gradient(grad, J, d)
    bench.barrier(d)
    t = bench.allmax(d, float(rank + 1))
    if rank == 0:
        np.save(out, grad)
        with open(out + ".txt", "w") as f:
            f.write("%r %r" % (J, t))
    d.destroy_process_group()


def test_two_ranks_sum_to_the_single_process_gradient(tmp_path):
    out = str(tmp_path / "g.npy")
    mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    grad = np.load(out)
    J2, tmax = map(float, open(out + ".txt").read().split())
    vel, vtrue, shots, nz, nt = _survey()
    ref = np.zeros(vel.shape, np.float64)
    Jref = 0.0
    for shot in shots:
        g, j = _shot_gradient(vel, vtrue, shot, nz, nt)
        ref += g
        Jref += j
    np.testing.assert_allclose(grad, ref, rtol=1e-12, atol=1e-30)
    assert abs(J2 - Jref) <= 1e-12 * Jref
    assert tmax == 2.0  # bench.allmax: the slowest rank's time


def test_shard_covers_every_shot_once():
    from wavefield_imaging_gb300.replicas import shard

    items = list(range(11))
    parts = [shard(items, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == items


def _engine_survey():
    import bench

    nt, nz = 300, 96
    vtrue, shots = bench.batch_survey(nshots=12, nxm=700, nz=nz, seed=9)
    shots = [(x0, min(nx, 200), sou, rec) for x0, nx, sou, rec in shots]
    shots = [(max(0, min(700 - nx, int(sou[0, 0] / 5.0) - nx // 2)), nx, sou, rec) for _, nx, sou, rec in shots]
    v0 = bench.smooth(vtrue, 4.0)
    wav = bench.ricker(nt, 0.005, 5.0)
    return vtrue, v0, shots, wav, nt, nz


def _engine_desc(awe, vel, nt, nz):
    return awe.make_desc(2, (nz, vel.shape[0]), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=16, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)


def _engine_rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    import wavefield_imaging_gb300 as awe
    from wavefield_imaging_gb300.replicas import survey_gradient

    d, _, _, _ = bench.dist_init()
    vtrue, v0, shots, wav, nt, nz = _engine_survey()
    desc = _engine_desc(awe, vtrue, nt, nz)
    with awe.Batch(desc, shots) as b:  # observed data, every shot on every rank
        b.set_model(vtrue)
        dobs = b.forward(wav)
    # both ranks share the one GPU: their kernels never wait on each other;
    # the gradients meet only in the host-side gloo sum
    grad, J = survey_gradient(desc, shots, v0, wav, dobs, dist=d, device=0)
    if rank == 0:
        np.save(out, grad)
        with open(out + ".txt", "w") as f:
            f.write("%r" % J)
    d.destroy_process_group()


@pytest.mark.gpu
def test_two_ranks_through_the_engine_match_one_process(tmp_path):
    """The shot split through the engine: two ranks (gloo) each run the
    batched gradient of half the shots; the reduced gradient and misfit equal
    one process's batched gradient of all shots (up to the order of the FP64
    sums)."""
    import wavefield_imaging_gb300 as awe
    from wavefield_imaging_gb300.replicas import survey_gradient

    out = str(tmp_path / "g.npy")
    mp.spawn(_engine_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    grad2 = np.load(out)
    J2 = float(open(out + ".txt").read())
    vtrue, v0, shots, wav, nt, nz = _engine_survey()
    desc = _engine_desc(awe, vtrue, nt, nz)
    with awe.Batch(desc, shots) as b:
        b.set_model(vtrue)
        dobs = b.forward(wav)
    grad1, J1 = survey_gradient(desc, shots, v0, wav, dobs)
    assert J1 > 0 and np.abs(grad1).max() > 0
    np.testing.assert_allclose(grad2, grad1, rtol=1e-9, atol=1e-12 * np.abs(grad1).max())
    assert abs(J2 - J1) <= 1e-9 * J1
