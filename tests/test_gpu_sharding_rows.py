"""The GPU half of the sharded Green's function (sharding.py), on one GPU: the impulse propagations
computed in three contiguous row blocks (nlm_green_rows, and nlm_green_rows_device into device
memory) and finished once (nlm_green_finish, nlm_green_finish_device) must equal the one-call
computeGreensFunction bit for bit (src/_NonlinearMedium.cpp:312-356 splits the same ranges over
threads).  The autotuner is off so that every block runs the same kernel variant."""
import numpy as np
import pytest

import cases
from multimodenonlinearoptics_gb300 import sharding

pytestmark = pytest.mark.gpu


def _medium(nlm):
    med = nlm.Chi2PDC(**dict(cases.CASES["Chi2PDC"], tPrecision=1024, tMax=40))
    med._set_schedule(cta_per_sm=-1)
    return med


def test_row_blocks_equal_green_host(nlm):
    med = _medium(nlm)
    C, S = med.computeGreensFunction()
    n = med._dims["nFreqs"]
    rows = sharding.engine_rows(med, False, False)
    raw = np.concatenate([rows(lo, hi) for lo, hi in sharding.partition(2 * n, 3)])
    C2, S2 = sharding.engine_finish(med, False)(raw)
    assert np.array_equal(C2, C) and np.array_equal(S2, S)


def test_row_blocks_equal_green_device(nlm):
    torch = pytest.importorskip("torch")
    med = _medium(nlm)
    C, S = med.computeGreensFunction()
    n = med._dims["nFreqs"]
    rows = sharding.engine_rows_device(med, False, False)
    blocks = [rows(lo, hi) for lo, hi in sharding.partition(2 * n, 3)]
    assert all(b.is_cuda for b in blocks)
    C2, S2 = sharding.engine_finish(med, False)(torch.cat(blocks))
    assert np.array_equal(C2, C) and np.array_equal(S2, S)
    # an empty block is allowed (more ranks than rows)
    assert rows(5, 5).shape == (0, n)
