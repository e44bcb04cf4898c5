"""Failure detection without a GPU fault: every wait in the library's kernels
is bounded. A self-test kernel waits on an mbarrier phase that never completes
and on a device flag that nothing sets, and the persistent Life and
multi-pass 2D kernels are started at pass 1 of runs whose pass 0 never ran
(their real dependency waits);
each gives up after a few polls and latches the timeout in the device error
word; the host reads it as PSKEL_ERR_DEVICE and the next call on the same
context succeeds."""
from __future__ import annotations

import numpy as np
import pytest

import pskel_gb300 as P
from pskel_gb300 import synth as S
from tests.gpu_util import bits, run2d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which,word", [(0, "TMA/mbarrier wait timed out"), (1, "dependency wait"),
                                        (2, "dependency wait"), (3, "dependency wait")])
def test_bounded_wait_times_out_and_reports(cuda, oracle_mod, which, word):
    P._check(P.lib.pskel_selftest_bounded_wait(which, 1000, None))
    with pytest.raises(P.PskelError) as ei:
        P.sync()
    assert ei.value.status == P.PSKEL_ERR_DEVICE
    assert word in str(ei.value)
    # the error word is cleared and the context is usable
    P.sync()
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, "f32", S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    a, b = S.jacobi2d(300, 200, seed=3)
    got = run2d(cuda, st, a, b, 5)
    assert np.array_equal(bits(got), bits(oracle_mod.lin2d(a, b, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, 5)))

