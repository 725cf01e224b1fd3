"""computeGreensFunction, batchSignalSimulation and ragged batches split over several GPUs, one
process per GPU.

The 2·N·nModes impulse propagations of a Green's function are independent.  The reference splits
them over std::threads in contiguous ranges (src/_NonlinearMedium.cpp:350-353); here each rank
propagates one contiguous range on its own GPU (nlm_green_rows_device: every rank regenerates the
pump locally, nothing is exchanged during the propagation), the raw rows are gathered once to rank 0
(one NCCL gather of device buffers) and rank 0 builds C and S in place (nlm_green_finish_device:
transpose, block fftshift, normalisation).  The rows of a
batch are split the same way.  The media of a ragged set are assigned to ranks by cost (longest
processing time first), each rank running its media in one ragged launch.

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
    """Row computation on this rank's GPU: raw outputs of impulse propagations [lo, hi) (host rows)."""
    from . import nonlinearmedium as nlm

    def rows(lo, hi):
        d = medium._dims
        out = np.empty((hi - lo, d["nSignalModes"] * d["nFreqs"]), dtype=np.complex128)
        nlm._check(nlm._lib.nlm_green_rows(medium._h(), int(bool(in_time_domain)), int(bool(run_pump)), lo, hi - lo,
                                           nlm._dptr(out.view(np.float64))))
        return out
    return rows


def engine_rows_device(medium, in_time_domain, run_pump):
    """Row computation on this rank's GPU into a CUDA tensor (nlm_green_rows_device): the rows stay in
    device memory for the NCCL gather."""
    import torch
    from . import nonlinearmedium as nlm

    def rows(lo, hi):
        d = medium._dims
        out = torch.empty((hi - lo, d["nSignalModes"] * d["nFreqs"]), dtype=torch.complex128, device="cuda")
        nlm._check(nlm._lib.nlm_green_rows_device(medium._h(), int(bool(in_time_domain)), int(bool(run_pump)), lo,
                                                  hi - lo, ctypes.c_void_p(out.data_ptr())))
        return out
    return rows


def engine_finish(medium, normalize):
    """C and S from the gathered raw rows, on rank 0's GPU.  Rows in a CUDA tensor are read in place
    (nlm_green_finish_device); host rows are uploaded (nlm_green_finish).  Returns numpy C and S."""
    from . import nonlinearmedium as nlm

    def finish(raw):
        d = medium._dims
        size = d["nSignalModes"] * d["nFreqs"]
        if not isinstance(raw, np.ndarray):
            import torch
            raw = raw.contiguous()
            C = torch.empty((size, size), dtype=torch.complex128, device=raw.device)
            S = torch.empty_like(C)
            nlm._check(nlm._lib.nlm_green_finish_device(medium._h(), ctypes.c_void_p(raw.data_ptr()),
                                                        int(bool(normalize)), ctypes.c_void_p(C.data_ptr()),
                                                        ctypes.c_void_p(S.data_ptr())))
            return C.cpu().numpy(), S.cpu().numpy()
        raw = np.ascontiguousarray(raw, dtype=np.complex128)
        C = np.empty((size, size), dtype=np.complex128)
        S = np.empty_like(C)
        nlm._check(nlm._lib.nlm_green_finish(medium._h(), nlm._dptr(raw.view(np.float64)), int(bool(normalize)),
                                             nlm._dptr(C.view(np.float64)), nlm._dptr(S.view(np.float64))))
        return C, S
    return finish


_CALLS = itertools.count()


def _publish_and_check(store, call, rank, world, status, timeout):
    """Every rank writes its status, then reads all others; raises RankFailure on a failed or silent rank."""
    import datetime
    store.set("nlm-shard/%d/%d" % (call, rank), status)
    store.set_timeout(datetime.timedelta(seconds=timeout))
    for r in range(world):
        try:
            other = store.get("nlm-shard/%d/%d" % (call, r)).decode()
        except Exception as exc:
            raise RankFailure("rank %d did not report within %.0f s (%s)" % (r, timeout, exc)) from exc
        if other != "ok":
            raise RankFailure("rank %d failed: %s" % (r, other))


def _gather_to_root(rows, counts, group):
    """Gather of every rank's leading-axis block (counts[r] entries on rank r) to rank 0, in one
    collective: rows is a torch tensor (complex) on the backend's device (CUDA for NCCL, so that the
    rows never leave device memory) or a numpy array (moved there).  The blocks are padded to the
    longest.  Returns the concatenation on rank 0 (a tensor on that device) and None elsewhere."""
    import torch
    import torch.distributed as dist
    rank = dist.get_rank(group)
    use_cuda = dist.get_backend(group) == "nccl"
    dev = torch.device("cuda", torch.cuda.current_device()) if use_cuda else torch.device("cpu")
    if isinstance(rows, np.ndarray):
        rows = torch.from_numpy(np.ascontiguousarray(rows, dtype=np.complex128))
    rows = rows.to(dev)
    longest = max(max(counts), 1)
    block = torch.zeros((longest,) + tuple(rows.shape[1:]) + (2,), dtype=torch.float64, device=dev)
    if rows.shape[0]:
        block[: rows.shape[0]] = torch.view_as_real(rows.contiguous())
    parts = [torch.empty_like(block) for _ in counts] if rank == 0 else None
    dst = 0 if group is None else dist.get_global_rank(group, 0)
    dist.gather(block, gather_list=parts, dst=dst, group=group)
    if rank != 0:
        return None
    return torch.view_as_complex(torch.cat([p[:c] for p, c in zip(parts, counts)]).contiguous())


def sharded_rows(n_units, row_width, compute_rows, group=None, timeout=60.0, keep_device=False):
    """Rows [lo, hi) of n_units independent units per rank (contiguous ranges), gathered to rank 0.

    compute_rows(lo, hi) -> (hi - lo, row_width) complex rows of this rank (numpy, or a torch tensor
    on the backend's device).  Returns the (n_units, row_width) rows on rank 0 (numpy; the gathered
    tensor when keep_device) and None elsewhere.
    """
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    store = dist.distributed_c10d._get_default_store()
    call = next(_CALLS)
    lo, hi = partition(n_units, world)[rank]
    status, rows = "ok", np.zeros((hi - lo, row_width), dtype=np.complex128)
    try:
        out = compute_rows(lo, hi)
        rows = out.reshape(hi - lo, row_width) if not isinstance(out, np.ndarray) else \
            np.asarray(out, dtype=np.complex128).reshape(hi - lo, row_width)
    except Exception as exc:  # reported to every rank below
        status = "error: %s: %s" % (type(exc).__name__, exc)
    _publish_and_check(store, call, rank, world, status, timeout)
    counts = [b - a for a, b in partition(n_units, world)]
    raw = _gather_to_root(rows, counts, group)
    if raw is None:
        return None
    return raw if keep_device else raw.cpu().numpy()


def green_sharded(medium, n_units, row_width, compute_rows, finish, group=None, timeout=60.0):
    """Run the row blocks of one Green's function over the ranks of `group`.

    compute_rows(lo, hi) -> (hi - lo, row_width) complex rows of this rank; finish(raw) -> (C, S) on
    rank 0.  Returns (C, S) on rank 0 and None elsewhere.
    """
    raw = sharded_rows(n_units, row_width, compute_rows, group, timeout, keep_device=True)
    if raw is None:
        return None
    return finish(raw if raw.is_cuda else raw.numpy())


def batch_sharded(medium, inputProfs, group=None, timeout=60.0, **kwargs):
    """batchSignalSimulation of `medium` with its rows split over the ranks (contiguous ranges), each
    rank propagating its rows on its own GPU.  Returns the output rows on rank 0, None elsewhere."""
    x = np.asarray(inputProfs, dtype=np.complex128)
    if x.ndim == 1:
        x = x.reshape(1, -1)
    d = medium._dims
    out_modes = kwargs.get("useOutput") or [1] * d["nSignalModes"]
    width = sum(1 for u in out_modes if u) * d["nFreqs"]

    def rows(lo, hi):
        if hi == lo:
            return np.zeros((0, width), dtype=np.complex128)
        return medium.batchSignalSimulation(x[lo:hi], **kwargs)
    return sharded_rows(x.shape[0], width, rows, group, timeout)


def assign_media(costs, world):
    """Longest-processing-time assignment of media (by cost) to ranks: each medium in decreasing cost
    goes to the least loaded rank (ties to the lowest rank).  Returns one index list per rank."""
    load = [0.0] * world
    owned = [[] for _ in range(world)]
    for k in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        owned[r].append(k)
        load[r] += costs[k]
    return [sorted(o) for o in owned]


def media_cost(medium):
    """Propagation cost of one medium: nZSteps x modes x N log2 N."""
    d = medium._dims
    n = d["nFreqs"]
    return float(d["nZSteps"] * d["nSignalModes"] * n * max(1.0, np.log2(n)))


def ragged_sharded(media, inputs, inTimeDomain=False, group=None, timeout=60.0, run=None, costs=None,
                   out_shapes=None):
    """nlm_ragged_batch over the ranks: media assigned by cost (assign_media), each rank running its
    media in one ragged launch on its own GPU, outputs gathered.  Returns the list of outputs (one
    (modes, N) array per medium, in input order) on rank 0, None elsewhere.  `run(media, inputs)`,
    `costs` and `out_shapes` replace the engine call and the engine's cost and shape queries (tests)."""
    import torch.distributed as dist
    from . import nonlinearmedium as nlm_mod

    media = list(media)
    inputs = list(inputs)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    store = dist.distributed_c10d._get_default_store()
    call = next(_CALLS)
    if costs is None:
        costs = [media_cost(m) for m in media]
    owned = assign_media(costs, world)
    if out_shapes is None:
        out_shapes = [(m._dims["nSignalModes"], m._dims["nFreqs"]) for m in media]
    shapes = [tuple(sh) for sh in out_shapes]
    run = run or (lambda ms, xs: nlm_mod.ragged_batch(ms, xs, inTimeDomain))
    status, flat = "ok", np.zeros(0, dtype=np.complex128)
    try:
        mine = owned[rank]
        outs = run([media[k] for k in mine], [inputs[k] for k in mine]) if mine else []
        flat = np.concatenate([np.asarray(o, dtype=np.complex128).ravel() for o in outs]) if outs else flat
    except Exception as exc:
        status = "error: %s: %s" % (type(exc).__name__, exc)
    _publish_and_check(store, call, rank, world, status, timeout)
    counts = [sum(int(np.prod(shapes[k])) for k in owned[r]) for r in range(world)]
    gathered = _gather_to_root(flat, counts, group)
    if gathered is None:
        return None
    gathered = gathered.cpu().numpy()
    result = [None] * len(media)
    off = 0
    for r in range(world):
        for k in owned[r]:
            size = int(np.prod(shapes[k]))
            result[k] = gathered[off: off + size].reshape(shapes[k])
            off += size
    return result


def green_sharded_device(medium, C, S, inTimeDomain=False, runPump=True, normalize=False, group=None,
                         timeout=60.0):
    """computeGreensFunction of `medium` split over the ranks of an NCCL group with nothing on the
    host: each rank's rows in device memory, one gather of device buffers to rank 0, and C and S
    written in place into rank 0's CUDA tensors C and S (ignored elsewhere).  Returns True on rank 0."""
    d = medium._dims
    n_units = 2 * d["nSignalModes"] * d["nFreqs"]
    width = d["nSignalModes"] * d["nFreqs"]
    raw = sharded_rows(n_units, width, engine_rows_device(medium, inTimeDomain, runPump), group, timeout,
                       keep_device=True)
    if raw is None:
        return False
    from . import nonlinearmedium as nlm
    raw = raw.contiguous()
    nlm._check(nlm._lib.nlm_green_finish_device(medium._h(), ctypes.c_void_p(raw.data_ptr()), int(bool(normalize)),
                                                ctypes.c_void_p(C.data_ptr()), ctypes.c_void_p(S.data_ptr())))
    return True


def compute_greens_function_sharded(medium, inTimeDomain=False, runPump=True, normalize=False, group=None,
                                    timeout=60.0):
    """computeGreensFunction of `medium` with its propagations split over the ranks of `group`
    (all modes as inputs and outputs).  Returns (C, S) on rank 0, None elsewhere."""
    import torch.distributed as dist
    d = medium._dims
    n_units = 2 * d["nSignalModes"] * d["nFreqs"]
    width = d["nSignalModes"] * d["nFreqs"]
    on_device = dist.get_backend(group) == "nccl"
    rows = (engine_rows_device if on_device else engine_rows)(medium, inTimeDomain, runPump)
    return green_sharded(medium, n_units, width, rows, engine_finish(medium, normalize), group, timeout)

