"""computeGreensFunction split over several GPUs, one process per GPU.

The 2·N·nModes impulse propagations of a Green's function are independent.  The reference splits
them over std::threads in contiguous ranges (src/_NonlinearMedium.cpp:350-353); here each rank
propagates one contiguous range on its own GPU (nlm_green_rows: every rank regenerates the pump
locally, nothing is exchanged during the propagation), the raw rows are gathered once to rank 0 and
rank 0 builds C and S (nlm_green_finish: transpose, block fftshift, normalisation).

Failure handling: before the only collective, every rank publishes its status in the process
group's store; a rank whose propagation raised, or that never reports within `timeout` seconds, makes
every other rank raise RankFailure instead of entering a collective that would never complete.
"""

import ctypes
import itertools

import numpy as np


class RankFailure(RuntimeError):
    """Another rank of the sharded computation failed or did not report."""


def partition(n_units, world):
    """Contiguous ranges [r n / w, (r + 1) n / w) for r = 0..w-1 (src/_NonlinearMedium.cpp:350-353)."""
    return [((r * n_units) // world, ((r + 1) * n_units) // world) for r in range(world)]


def engine_rows(medium, in_time_domain, run_pump):
    """Row computation on this rank's GPU: raw outputs of impulse propagations [lo, hi)."""
    from . import nonlinearmedium as nlm

    def rows(lo, hi):
        d = medium._dims
        out = np.empty((hi - lo, d["nSignalModes"] * d["nFreqs"]), dtype=np.complex128)
        nlm._check(nlm._lib.nlm_green_rows(medium._h(), int(bool(in_time_domain)), int(bool(run_pump)), lo, hi - lo,
                                           nlm._dptr(out.view(np.float64))))
        return out
    return rows


def engine_finish(medium, normalize):
    """C and S from the gathered raw rows, on rank 0's GPU."""
    from . import nonlinearmedium as nlm

    def finish(raw):
        d = medium._dims
        size = d["nSignalModes"] * d["nFreqs"]
        raw = np.ascontiguousarray(raw, dtype=np.complex128)
        C = np.empty((size, size), dtype=np.complex128)
        S = np.empty_like(C)
        nlm._check(nlm._lib.nlm_green_finish(medium._h(), nlm._dptr(raw.view(np.float64)), int(bool(normalize)),
                                             nlm._dptr(C.view(np.float64)), nlm._dptr(S.view(np.float64))))
        return C, S
    return finish


_CALLS = itertools.count()


def green_sharded(medium, n_units, row_width, compute_rows, finish, group=None, timeout=60.0):
    """Run the row blocks of one Green's function over the ranks of `group`.

    compute_rows(lo, hi) -> (hi - lo, row_width) complex rows of this rank; finish(raw) -> (C, S) on
    rank 0.  Returns (C, S) on rank 0 and None elsewhere.
    """
    import datetime

    import torch
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    store = dist.distributed_c10d._get_default_store()
    call = next(_CALLS)
    lo, hi = partition(n_units, world)[rank]
    status, rows = "ok", None
    try:
        rows = np.asarray(compute_rows(lo, hi), dtype=np.complex128).reshape(hi - lo, row_width)
    except Exception as exc:  # reported to every rank below
        status = "error: %s: %s" % (type(exc).__name__, exc)
    store.set("nlm-green/%d/%d" % (call, rank), status)
    store.set_timeout(datetime.timedelta(seconds=timeout))
    for r in range(world):
        try:
            other = store.get("nlm-green/%d/%d" % (call, r)).decode()
        except Exception as exc:
            raise RankFailure("rank %d did not report within %.0f s (%s)" % (r, timeout, exc)) from exc
        if other != "ok":
            raise RankFailure("rank %d failed: %s" % (r, other))
    # one gather of the row blocks (padded to the largest block)
    counts = [b - a for a, b in partition(n_units, world)]
    width = max(counts)
    use_cuda = dist.get_backend(group) == "nccl"
    dev = torch.device("cuda", torch.cuda.current_device()) if use_cuda else torch.device("cpu")
    block = torch.zeros((width, row_width, 2), dtype=torch.float64, device=dev)
    block[: hi - lo] = torch.view_as_real(torch.from_numpy(rows)).to(dev)
    parts = [torch.empty_like(block) for _ in range(world)]
    dist.all_gather(parts, block, group=group)
    if rank != 0:
        return None
    raw = np.concatenate([torch.view_as_complex(p[:c].cpu()).numpy() for p, c in zip(parts, counts)], axis=0)
    return finish(raw)


def compute_greens_function_sharded(medium, inTimeDomain=False, runPump=True, normalize=False, group=None,
                                    timeout=60.0):
    """computeGreensFunction of `medium` with its propagations split over the ranks of `group`
    (all modes as inputs and outputs).  Returns (C, S) on rank 0, None elsewhere."""
    d = medium._dims
    n_units = 2 * d["nSignalModes"] * d["nFreqs"]
    width = d["nSignalModes"] * d["nFreqs"]
    return green_sharded(medium, n_units, width, engine_rows(medium, inTimeDomain, runPump),
                         engine_finish(medium, normalize), group, timeout)


del ctypes
