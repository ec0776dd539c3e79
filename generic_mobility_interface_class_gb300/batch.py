"""Independent swimmers of uneven size stepped together on one GPU.

The reference runs every swimmer of a simulation through one mobility
solver, in one coupled system (cilia_sim_main.cpp:205-343); swimmers that do
not interact hydrodynamically are separate simulations.  ``SwimmerBatch``
keeps one device time step (``sim.Simulation``) per swimmer, each on its own
context, so on its own CUDA stream, and drives each from its own host thread:
the library's calls release the interpreter lock, so the swimmers' host-side
control (the Broyden loop, the refinement checks) runs in parallel and their
kernels overlap on the GPU.  A small swimmer's latency-bound GMRES kernels
then fill the SMs that a large swimmer's leave idle.

No swimmer reads another's memory, and the library serialises what would
otherwise collide across threads: stream captures and device-wide
synchronising calls take one process-wide lock, and a kernel's dynamic
shared-memory limit is only ever raised.  A batch of small swimmers steps
bit-identically to stepping them one by one.  Stepped one by one, the full
64-swimmer workload is bit-reproducible from run to run; stepped
concurrently, its GMRES iteration totals vary by up to 14 in 50,000 between
runs, an ordering effect not yet traced to its kernel.
"""
from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

from ._lib import GMI_FP64


class SwimmerBatch:
    """One ``Simulation`` per entry of ``swimmers`` (their keyword sets),
    all at one precision on one device.

    threads: host threads driving the swimmers; ``None`` gives one per
    swimmer, 1 steps them one after another.  sim_factory builds a swimmer
    from its keyword set (``sim.Simulation`` by default).
    """

    def __init__(self, swimmers, *, precision=GMI_FP64, device=0, threads=None, sim_factory=None):
        if sim_factory is None:
            from .sim import Simulation as sim_factory
        swimmers = list(swimmers)
        if not swimmers:
            raise ValueError("SwimmerBatch: no swimmers")
        self.threads = len(swimmers) if threads is None else max(1, int(threads))
        self._pool = ThreadPoolExecutor(max_workers=self.threads) if self.threads > 1 else None
        self.sims = []
        made = []  # list.append is atomic: the pool's threads share it

        def make(kw):
            s = sim_factory(**kw, precision=precision, device=device)
            made.append(s)
            return s

        try:
            self.sims = self._map(make, swimmers)
        except BaseException:
            self.sims = made  # close whatever was built
            self.close()
            raise
        # the next time step of each swimmer: advanced per swimmer as each of
        # its steps completes, so after a failure every swimmer's count is
        # the steps it really took
        self.next_nt = [0] * len(self.sims)

    @property
    def nt(self):
        """The next time step of the batch: every swimmer's, when they agree;
        after a failure that left them apart, a ValueError names them
        (``next_nt`` holds each swimmer's)."""
        if len(set(self.next_nt)) != 1:
            raise ValueError(f"swimmers are at different time steps: {self.next_nt}")
        return self.next_nt[0]

    def __len__(self):
        return len(self.sims)

    def _map(self, fn, items):
        """fn over items, in parallel on the pool; every call finishes before
        the first error (in item order) is raised."""
        items = list(items)
        if self._pool is None:
            results, first = [], None
            for it in items:
                try:
                    results.append(fn(it))
                except Exception as e:  # keep stepping the others, as the pool does
                    results.append(None)
                    if first is None:
                        first = e
            if first is not None:
                raise first
            return results
        futures = [self._pool.submit(fn, it) for it in items]
        errors = [f.exception() for f in futures]
        for e in errors:
            if e is not None:
                raise e
        return [f.result() for f in futures]

    def prepare(self):
        """Body reference matrices of every swimmer (gmi_sim_prepare)."""
        return self._map(lambda s: s.prepare(), self.sims)

    def step(self, nt=None):
        """One implicit time step of every swimmer (time step nt, or each
        swimmer's own next step); returns the per-swimmer (Broyden
        iterations, GMRES iterations).  A swimmer that fails keeps its step
        count; the others advance, and the first failure is raised."""

        def one(i):
            t = self.next_nt[i] if nt is None else nt
            r = self.sims[i].step(t)
            self.next_nt[i] = t + 1
            return r

        return self._map(one, range(len(self.sims)))

    def run(self, steps, nt=None):
        """steps time steps of every swimmer, each swimmer's thread going on
        to its next step without waiting for the others (no batch-wide
        barrier between steps, so the GPU keeps the large swimmers' work
        and the small swimmers' next steps in flight together).  Returns,
        per swimmer, its list of (Broyden iterations, GMRES iterations).
        A swimmer that fails stops there, with ``next_nt`` at the step that
        failed; the others finish their steps and the first failure (in
        swimmer order) is raised."""

        def advance(i):
            t0 = self.next_nt[i] if nt is None else nt
            out = []
            for k in range(steps):
                out.append(self.sims[i].step(t0 + k))
                self.next_nt[i] = t0 + k + 1
            return out

        return self._map(advance, range(len(self.sims)))

    def state(self, name):
        """The state field ``name`` of every swimmer (see ``Simulation.state``)."""
        return [s.state(name) for s in self.sims]

    @property
    def launches(self):
        return sum(s.launches for s in self.sims)

    def close(self):
        for s in self.sims:
            try:
                s.close()
            except Exception:
                pass
        self.sims = []
        if self._pool is not None:
            self._pool.shutdown(wait=True)
            self._pool = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
