"""Served job stream on the GPU: each job's result is the same alone and in the mix.

A small stream of Lennard-Jones and Sutton-Chen jobs of different sizes and lengths runs
through the job server (continuous batching: several batches in flight on their own
streams, finished jobs retired from a running batch).  Then some of the jobs run again
alone, each as the only system of its batch, and their final positions and velocities must
match the in-mix results bit for bit (mixed precision: fixed-point force sums make every
per-system trajectory independent of what else shares the launches, and of the lane count the
server picks for the batch's size); thermo records match to FP32 summation order.
"""
import numpy as np
import pytest

from lpmd2_gb300 import inputs as I

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")
serve = pytest.importorskip("lpmd2_gb300.serve")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def stream():
    spec = [("lj", 4, 120, 0.00), ("lj", 6, 75, 0.00), ("sc", 5, 60, 0.00), ("lj", 5, 200, 0.00),
            ("sc", 6, 33, 0.00), ("lj", 7, 41, 0.02), ("sc", 5, 90, 0.03), ("lj", 4, 57, 0.03)]
    jobs = []
    for j, (kind, k, steps, t) in enumerate(spec):
        jobs.append(dict(id=j, kind=kind, k=k, steps=steps, arrival=t, rho_star=0.7 + 0.03 * j,
                         t_star=0.8 + 0.15 * j, seed=900 + j))
    return jobs


def alone(backend, job):
    system = I.materialize_job(job)
    b = backend.open(job["kind"], [system])
    backend.advance(b, job["steps"])
    out = backend.read(b, 0)
    backend.close(b)
    return out


def test_served_results_equal_alone():
    jobs = stream()
    backend = serve.GbmdBackend()
    srv = serve.Server(backend, budget_bytes=150e9, max_batches=3, max_systems=4, chunk_steps=50)
    res = srv.serve(jobs, I.materialize_job)
    assert all(r.error is None for r in res)
    by_batch = {}
    for r in res:
        by_batch.setdefault(r.batch, []).append(r)
    assert max(len(v) for v in by_batch.values()) > 1  # jobs shared a batch
    spans = [(min(r.admitted for r in v), max(r.finished for r in v)) for v in by_batch.values()]
    assert any(a0 < b1 and b0 < a1 for i, (a0, a1) in enumerate(spans) for (b0, b1) in spans[i + 1:])
    for j in (0, 2, 3, 6):
        pos, vel, th = alone(backend, jobs[j])
        np.testing.assert_array_equal(res[j].pos, pos)
        np.testing.assert_array_equal(res[j].vel, vel)
        # the lane count of the LJ force pass follows the batch's live atoms (serve.lanes_for):
        # forces, hence trajectories, are bitwise the same for every lane count; the per-atom
        # FP32 energy and stress sums, and the per-warp kinetic sums, are grouped differently
        np.testing.assert_allclose(res[j].thermo["raw"], th["raw"], rtol=1e-7, atol=1e-12)
        assert res[j].thermo["step"] == jobs[j]["steps"]
