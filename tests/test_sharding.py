"""Row-block sharding of computeGreensFunction over CPU ranks (gloo, world size 2).

The ranks run the product orchestration (partition, status exchange, gather) with the oracle as the
per-rank row computation and epilogue, so the test needs no GPU; the GPU entry points behind the
default callables are covered by the GPU tests."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from multimodenonlinearoptics_gb300 import sharding

CFG = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, beta1s=2, beta3s=0.1, tMax=20, tPrecision=32,
           zPrecision=10, poling=np.ones(4))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def oracle_rows(med):
    """Raw rows of impulse propagations [lo, hi) (instance 2 (im N + bin) + {0: 1, 1: i})."""
    n = med.n_freqs

    def rows(lo, hi):
        idx = np.arange(lo, hi)
        prof = np.zeros((idx.size, n), dtype=np.complex128)
        prof[np.arange(idx.size), (idx // 2) % n] = np.where(idx % 2 == 0, 1.0, 1.0j)
        f, _ = med.propagate(prof, False, 0)
        return f[:, 0]
    return rows


def oracle_finish(raw):
    n = raw.shape[1]
    o1, oi = raw[0::2], raw[1::2]
    c = (0.5 * o1 - 0.5j * oi).T
    s = (0.5 * o1 + 0.5j * oi).T
    return np.fft.fftshift(c), np.fft.fftshift(s)


def _worker(rank, world, port, fail_rank, silent_rank, outdir):
    import torch.distributed as dist
    from oracle import nlm_oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    med = O.Chi2PDC(**CFG)
    med.run_pump_simulation()
    rows = oracle_rows(med)
    if rank == fail_rank:
        def rows(lo, hi):  # noqa: F811 - this rank's propagation fails
            raise MemoryError("simulated device failure")
    if rank == silent_rank:
        os._exit(0)          # leaves between steps without reporting
    try:
        res = sharding.green_sharded(med, 2 * med.n_freqs, med.n_freqs, rows, oracle_finish, timeout=5.0)
        if rank == 0:
            np.savez(os.path.join(outdir, "res.npz"), C=res[0], S=res[1])
        open(os.path.join(outdir, "ok%d" % rank), "w").close()
    except sharding.RankFailure as exc:
        open(os.path.join(outdir, "fail%d" % rank), "w").write(str(exc))
    dist.destroy_process_group() if silent_rank < 0 else None


def _run(tmp_path, fail_rank=-1, silent_rank=-1, world=2):
    port = _free_port()
    mp.spawn(_worker, args=(world, port, fail_rank, silent_rank, str(tmp_path)), nprocs=world, join=True)


def test_partition_matches_reference_split():
    for n, w in ((2048, 1), (2048, 3), (64, 7), (5, 8)):
        parts = sharding.partition(n, w)
        assert parts[0][0] == 0 and parts[-1][1] == n
        assert all(parts[k][1] == parts[k + 1][0] for k in range(w - 1))
        assert sum(b - a for a, b in parts) == n


def test_sharded_gather_equals_single_rank(tmp_path):
    from oracle import nlm_oracle as O
    _run(tmp_path)
    res = np.load(os.path.join(tmp_path, "res.npz"))
    med = O.Chi2PDC(**CFG)
    C, S = med.compute_greens_function()
    assert np.abs(res["C"] - C).max() < 1e-13 and np.abs(res["S"] - S).max() < 1e-13
    assert os.path.exists(os.path.join(tmp_path, "ok1"))


def test_failed_rank_raises_everywhere(tmp_path):
    _run(tmp_path, fail_rank=1)
    for r in range(2):
        msg = open(os.path.join(tmp_path, "fail%d" % r)).read()
        assert "rank 1 failed" in msg and "MemoryError" in msg


def test_silent_rank_times_out(tmp_path):
    _run(tmp_path, silent_rank=1)
    msg = open(os.path.join(tmp_path, "fail0")).read()
    assert "did not report" in msg


def test_media_assignment_is_balanced_and_deterministic():
    costs = [5.0, 1.0, 9.0, 3.0, 3.0, 7.0, 2.0]
    owned = sharding.assign_media(costs, 3)
    assert sorted(k for o in owned for k in o) == list(range(len(costs)))
    loads = [sum(costs[k] for k in o) for o in owned]
    assert max(loads) - min(loads) <= max(costs)
    assert owned == sharding.assign_media(costs, 3)
    assert sharding.assign_media(costs, 1) == [list(range(len(costs)))]
    assert sharding.assign_media([], 2) == [[], []]


class _OracleBatchMedium:
    """The engine medium's batch interface on the oracle (for CPU ranks)."""

    def __init__(self, med):
        self.med = med
        self._dims = {"nSignalModes": med.n_signal_modes, "nFreqs": med.n_freqs}

    def batchSignalSimulation(self, x, **kw):
        return self.med.batch_signal_simulation(x, kw.get("inTimeDomain", False), False)


SFG = dict(relativeLength=1, nlLength=1, nlLengthOrig=1, beta2=0.3, beta2s=-0.2, beta2o=0, beta1s=1.1, beta3s=0.05,
           tMax=10, zPrecision=6)


def _ragged_media(O):
    media, inputs = [], []
    rng = np.random.default_rng(7)
    for n, doms in ((32, [1, 2, 1]), (64, [2, 1]), (16, [1, 1, 1, 1]), (32, [3, 1]), (64, [1, 2, 2])):
        m = O.Chi2SFG(tPrecision=n, poling=doms, **SFG)
        m.run_pump_simulation()
        media.append(m)
        inputs.append((rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 1e-3)
    return media, inputs


def _oracle_ragged_run(ms, xs):
    return [m.propagate(np.asarray(x)[None, :], False, 0)[0][0] for m, x in zip(ms, xs)]


def _worker_rows(rank, world, port, outdir):
    import torch.distributed as dist
    from oracle import nlm_oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    med = O.Chi2PDC(**CFG)
    med.run_pump_simulation()
    x = (np.random.default_rng(3).standard_normal((7, med.n_freqs)) + 0j)
    out = sharding.batch_sharded(_OracleBatchMedium(med), x, timeout=5.0, inTimeDomain=False)
    media, inputs = _ragged_media(O)
    costs = [m.n_z_steps * m.n_freqs * np.log2(m.n_freqs) * m.n_signal_modes for m in media]
    shapes = [(m.n_signal_modes, m.n_freqs) for m in media]
    rag = sharding.ragged_sharded(media, inputs, group=None, timeout=5.0, run=_oracle_ragged_run, costs=costs,
                                  out_shapes=shapes)
    if rank == 0:
        np.savez(os.path.join(outdir, "rows.npz"), batch=out, *rag)
    dist.destroy_process_group()


def test_batch_and_ragged_sharding_equal_single_rank(tmp_path):
    from oracle import nlm_oracle as O
    port = _free_port()
    mp.spawn(_worker_rows, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = np.load(os.path.join(tmp_path, "rows.npz"))
    med = O.Chi2PDC(**CFG)
    med.run_pump_simulation()
    x = (np.random.default_rng(3).standard_normal((7, med.n_freqs)) + 0j)
    assert np.array_equal(res["batch"], med.batch_signal_simulation(x, False, False))
    media, inputs = _ragged_media(O)
    ref = _oracle_ragged_run(media, inputs)
    for k, r in enumerate(ref):
        assert np.array_equal(res["arr_%d" % k], r)
