"""Independent swimmers of uneven size: the seeded workload and the host
side of batch.SwimmerBatch (threads, ordering, errors), without a GPU.  The
swimmers in these tests are stand-ins with the Simulation interface."""
import threading

import numpy as np
import pytest

from generic_mobility_interface_class_gb300 import workloads
from generic_mobility_interface_class_gb300.batch import SwimmerBatch


def test_config4_sizes_follow_the_workload():
    sw = workloads.config4()
    assert len(sw) == 64
    r = np.array([s["body_radius"] for s in sw])
    nb = np.array([s["nblob"] for s in sw])
    nf = np.array([s["nfil"] for s in sw])
    assert r.min() >= 10.0 and r.max() <= 40.0
    assert nb.min() >= 642 and nb.max() <= 4096
    # the blob count grows with the radius
    order = np.argsort(r)
    assert np.all(np.diff(nb[order]) >= 0)
    assert nf.min() >= 16 and nf.max() <= 512
    for s in sw:
        assert s["nfil"] <= workloads.max_filaments(s["body_radius"])
        assert s["nseg"] == 20
        assert s["blob_refs"].shape == (s["nblob"], 3)
        assert np.allclose(np.linalg.norm(s["blob_refs"], axis=1), s["body_radius"])
    # uneven: the filament counts spread over more than a factor of four
    assert nf.max() >= 4 * nf.min()


def test_config4_filament_bases_keep_two_segment_lengths_apart():
    for s in workloads.config4(nswim=8):
        b = s["fil_refs"]
        d = np.linalg.norm(b[:, None, :] - b[None, :, :], axis=2)
        np.fill_diagonal(d, np.inf)
        # the angular separation on the base sphere is 2 DL, so the chords are
        # slightly shorter; the bases must not touch (segment radius 1)
        assert d.min() > 2.0 * 2.2 * 0.99


def test_config4_is_seeded():
    a, b = workloads.config4(nswim=4), workloads.config4(nswim=4)
    c = workloads.config4(seed=7, nswim=4)
    for x, y in zip(a, b):
        for k in ("blob_refs", "fil_refs", "perturbation1", "perturbation2"):
            assert np.array_equal(x[k], y[k])
    assert any(x["nfil"] != z["nfil"] or x["body_radius"] != z["body_radius"] for x, z in zip(a, c))


class FakeSim:
    """Stand-in with the Simulation interface: step() waits on a shared
    barrier, so a batch step completes only if every swimmer steps at once."""

    def __init__(self, *, name, barrier=None, fail_at=None, log=None, precision=0, device=0):
        self.name, self.barrier, self.fail_at, self.log = name, barrier, fail_at, log
        self.closed = False
        self.nt_seen = []

    def prepare(self):
        return self.name

    def step(self, nt):
        if self.barrier is not None:
            self.barrier.wait(timeout=10)
        self.nt_seen.append(nt)
        if self.log is not None:
            self.log.append((self.name, nt))
        if self.fail_at == nt:
            raise RuntimeError(f"swimmer {self.name} failed at step {nt}")
        return (self.name, 10 * nt)

    def state(self, name):
        return np.full((2, 3), float(self.name))

    @property
    def launches(self):
        return 5

    def close(self):
        self.closed = True


def test_batch_steps_every_swimmer_at_once():
    n = 6
    barrier = threading.Barrier(n)
    batch = SwimmerBatch([dict(name=i, barrier=barrier) for i in range(n)], sim_factory=FakeSim)
    assert batch.prepare() == list(range(n))
    for nt in range(3):
        assert batch.step() == [(i, 10 * nt) for i in range(n)]
    assert all(s.nt_seen == [0, 1, 2] for s in batch.sims)
    assert [float(a[0, 0]) for a in batch.state("body_v")] == list(range(n))
    assert batch.launches == 5 * n
    sims = list(batch.sims)
    batch.close()
    assert all(s.closed for s in sims)


def test_batch_with_one_thread_steps_in_order():
    log = []
    batch = SwimmerBatch([dict(name=i, log=log) for i in range(4)], sim_factory=FakeSim, threads=1)
    batch.step(0)
    batch.step(1)
    assert log == [(i, nt) for nt in (0, 1) for i in range(4)]
    batch.close()


@pytest.mark.parametrize("threads", [None, 1])
def test_batch_error_surfaces_after_every_swimmer_stepped(threads):
    log = []
    batch = SwimmerBatch([dict(name=i, log=log, fail_at=(1 if i == 2 else None)) for i in range(4)],
                         sim_factory=FakeSim, threads=threads)
    batch.step(0)
    with pytest.raises(RuntimeError, match="swimmer 2 failed at step 1"):
        batch.step(1)
    # the others still took their step: no swimmer is left behind mid-batch
    assert sorted(name for name, nt in log if nt == 1) == [0, 1, 2, 3]
    batch.close()


def test_batch_creation_failure_closes_the_batch():
    made = []

    def factory(**kw):
        if kw["name"] == 3:
            raise ValueError("bad swimmer")
        s = FakeSim(**kw)
        made.append(s)
        return s

    with pytest.raises(ValueError, match="bad swimmer"):
        SwimmerBatch([dict(name=i) for i in range(5)], sim_factory=factory)
    assert len(made) == 4 and all(s.closed for s in made)
    with pytest.raises(ValueError):
        SwimmerBatch([], sim_factory=FakeSim)


def test_batch_run_needs_no_batch_wide_barrier():
    """run(steps): a swimmer goes on to its next step while another is still
    in its first, which a per-step barrier would forbid."""
    first_done = threading.Event()

    class Slow(FakeSim):
        def step(self, nt):
            if self.name == 0 and nt == 0:
                # swimmer 0 finishes its first step only once swimmer 1 has
                # taken its second
                assert first_done.wait(timeout=10)
            if self.name == 1 and nt == 1:
                first_done.set()
            return super().step(nt)

    batch = SwimmerBatch([dict(name=i) for i in range(2)], sim_factory=Slow)
    out = batch.run(3)
    assert out == [[(i, 0), (i, 10), (i, 20)] for i in range(2)]
    assert batch.nt == 3 and all(s.nt_seen == [0, 1, 2] for s in batch.sims)
    assert batch.step() == [(0, 30), (1, 30)]
    batch.close()


def test_batch_run_stops_a_failing_swimmer_only():
    batch = SwimmerBatch([dict(name=i, fail_at=(1 if i == 0 else None)) for i in range(3)], sim_factory=FakeSim)
    with pytest.raises(RuntimeError, match="swimmer 0 failed at step 1"):
        batch.run(3)
    assert batch.sims[0].nt_seen == [0, 1]
    assert batch.sims[1].nt_seen == [0, 1, 2] and batch.sims[2].nt_seen == [0, 1, 2]
    # each swimmer's count is the steps it really took: the failed one is
    # still at step 1, and the batch no longer claims one step number
    assert batch.next_nt == [1, 3, 3]
    with pytest.raises(ValueError, match="different time steps"):
        batch.nt
    # stepping on continues each swimmer from its own step
    batch.sims[0].fail_at = None
    batch.step()
    assert batch.sims[0].nt_seen == [0, 1, 1] and batch.sims[1].nt_seen == [0, 1, 2, 3]
    assert batch.next_nt == [2, 4, 4]
    batch.close()


def test_batch_step_failure_keeps_per_swimmer_counts():
    batch = SwimmerBatch([dict(name=i, fail_at=(0 if i == 1 else None)) for i in range(3)], sim_factory=FakeSim)
    with pytest.raises(RuntimeError, match="swimmer 1 failed at step 0"):
        batch.step()
    assert batch.next_nt == [1, 0, 1]
    batch.close()
