"""The serving loop on the GPU: every request's result is the same served
alone (one synchronous launch) and in the batched mix (fused sweeps, several
streams), within the FP64 tolerance (1e-12 relative to the result's scale)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_mix(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim
    from tskit_gb300.serve import GpuBackend, Server, poisson_requests

    resident = {
        "small": tskit_gb300.TreeSequence(sim.simulate(600, 1e6, 3000, 3000, 91)),
        "large": tskit_gb300.TreeSequence(sim.simulate(70000, 1e6, 300, 2000, 92)),
    }
    reqs = poisson_requests(resident, 80, 1e6, 5, window_choices=(1, 4), set_range=(10, 200),
                            rv_columns=3)
    be = GpuBackend(resident, num_slots=4)
    mix = Server(be, num_slots=4).run(reqs)
    alone = Server(GpuBackend(resident, num_slots=1), num_slots=1).run(reqs, mode="plain")
    assert mix.launches < alone.launches == len(reqs)
    for r in reqs:
        a, b = alone.results[r.rid], mix.results[r.rid]
        assert a.shape == b.shape
        scale = max(np.nanmax(np.abs(a)), 1e-300) if a.size else 1.0
        np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-12 * scale, equal_nan=True,
                                   err_msg=f"{r.stat} {r.mode} {r.ts}")
