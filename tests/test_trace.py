"""The opt-in push-kernel phase trace (gde_ctx_trace / gde_ctx_trace_read).

Checks the shape and ordering of the stamps and that the grid barrier is a
barrier in the timeline: no block leaves a phase barrier before the last
block has entered it.  Tracing must not change results.
"""
import numpy as np
import pytest

from gde import _lib as L
from gde import api, graphs

pytestmark = pytest.mark.gpu

TICK_NS = 2_000  # slack for %globaltimer granularity across SMs


@pytest.mark.parametrize("groups", [1, 8])
def test_trace_timeline_is_ordered_and_barriers_hold(groups):
    """One block group: the barrier holds over the whole grid.  Eight groups (one per served slot, the
    default for 8 queries): it holds within each group, blocks [ceil(g B / 8), ceil((g+1) B / 8))."""
    g = graphs.chung_lu(3000, 2.1, 8.0, 300.0, seed=3)
    Gd = api.Graph(g.indptr, g.indices)
    seeds = graphs.uniform_seeds(g, 8, seed=5)
    tun = {"groups": groups}
    ref = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp64", alpha=0.1, tuning=tun)
    api.trace(6)
    try:
        res = api.solve(Gd, L.PPR, L.LOCAL_GD, seeds, 1e-6, prec="fp64", alpha=0.1, tuning=tun)
        tr = api.trace_read()
    finally:
        api.trace(0)
    np.testing.assert_array_equal(res["oper"], ref["oper"])
    np.testing.assert_allclose(res["x"], ref["x"], rtol=0, atol=1e-14)
    iters, grid, points = tr.shape
    assert iters == 6 and points == 8 and grid > 0
    ran = tr[:, :, 0] != 0
    assert ran.all(), "every block stamps every traced iteration of a 6+ round solve"
    t = tr.astype(np.int64)
    # within a block and iteration the phase stamps never go back
    assert (np.diff(t, axis=2) >= 0).all()
    # iterations follow one another
    assert (t[1:, :, 0] >= t[:-1, :, 7]).all()
    # barriers: every block of a group leaves after the last block of the group entered
    member = (np.arange(grid) * groups) // grid
    for grp in range(groups):
        tg = t[:, member == grp, :]
        for enter, leave in ((2, 3), (6, 7)):
            last_in = tg[:, :, enter].max(axis=1)
            first_out = tg[:, :, leave].min(axis=1)
            assert (first_out + TICK_NS >= last_in).all(), grp
    assert api.trace_read().size == 0


def test_random_atomic_probe_reports_a_rate():
    """The random-access ceiling probe runs and gives a plausible positive rate."""
    small = api.probe_random_atomics(1 << 20)
    large = api.probe_random_atomics(64 << 20)
    assert 0.1 < large < 10_000 and 0.1 < small < 10_000
    # an L2-resident array is at least as fast as a 256 MB one
    assert small > 0.8 * large
    with pytest.raises(L.GDEError):
        api.probe_random_atomics(0)
