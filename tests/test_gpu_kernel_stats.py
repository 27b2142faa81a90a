"""Per-kernel statistics of a context (pcg_set_kernel_timing, pcg_get_kernel_stats).

Every kernel that ran with timing on must report its launches, a positive time and
positive algorithmic bytes: the cell kernels' bytes scale with counts that live on
the device (agents of shared voxels, agents that write a voxel), read after every
timed ballot and, for a ballot built before timing was switched on, when it is.
The apply kernel's bytes must equal its per-writer figure times the number of
agents that write a voxel (occupied voxels), counted here on the host.
"""
import numpy as np
import pytest

from physicore_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _problem():
    rng = np.random.default_rng(21)
    S, n, A = 4, (40, 36, 30), 20000
    pos = W.uniform_positions(rng, A, 3, 0.0, np.array(n, dtype=np.float64) * 20.0)
    pos[: A // 4] = pos[A // 4: A // 2]  # shared voxels
    ag = W.agents_block(rng, A, S, pos, net_export_hi=0.5)
    return dict(name="kernel_stats", dims=3, bbmin=(0, 0, 0), bbmax=tuple(v * 20 for v in n), voxel=(20, 20, 20),
                dt=0.01, D=np.geomspace(10.0, 1e4, S), decay=np.geomspace(1e-3, 0.5, S), initial=np.zeros(S),
                field=rng.random((n[2], n[1], n[0], S)), field_layout="interleaved", boundary=[], interior=None,
                bulk=None, agents=ag, compute_internalized=True)


def _check_all(stats):
    ran = {k: v for k, v in stats.items() if v["launches"]}
    assert ran, "no kernel ran"
    for name, v in ran.items():
        assert v["ms"] > 0, name
        assert v["bytes"] > 0, f"{name}: {v['launches']} launches, {v['ms']:.3f} ms but no bytes"
    return ran


@pytest.mark.parametrize("precision", [0, 1])
def test_kernel_stats_after_an_untimed_ballot(pcg, precision):
    p = _problem()
    s = W.apply(pcg.Solver(precision), p)
    s.solve(1)  # ballot built without timing
    s.set_kernel_timing(True)
    s.reset_kernel_stats()
    s.solve(3)
    ran = _check_all(s.kernel_stats())
    assert {"cells_apply", "cells_internalize"} <= set(ran)
    counts = s.get_counts()
    writers = int(np.count_nonzero(counts))
    S, w = 4, (4 if precision == 0 else 8)
    per_writer = 9 + 5 * S * w + 16 * S
    assert ran["cells_apply"]["bytes"] == pytest.approx(3 * writers * per_writer)
    s.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_kernel_stats_with_a_timed_ballot(pcg, precision):
    p = _problem()
    s = W.apply(pcg.Solver(precision), p)
    s.set_kernel_timing(True)
    s.reset_kernel_stats()  # launches of the initialisation were not timed
    s.solve(2)  # the first call rebuilds the ballot under timing
    s.recompute_positional_data()
    s.solve(1)
    ran = _check_all(s.kernel_stats())
    assert {"cells_locate", "cells_ballot", "cells_group", "cells_reduce", "cells_apply",
            "cells_internalize"} <= set(ran)
    s.close()
