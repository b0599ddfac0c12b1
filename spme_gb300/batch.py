"""Uneven batches of independent systems.

A batch holds systems of different N, box L, mesh K and order p (e.g. 64
systems with N between 500 and 50,000).  Each system is small: alone, its
kernels cover a few dozen tiles and leave most of the 152 SMs idle, and a
per-system loop pays ~20 launches per system.

``SystemBatch.run`` uses the native batch (:class:`spme_gb300.Batch`,
``spme_batch_*`` in include/spme_gb300.h): every stage of the position build
and of the apply is one persistent launch over a packed work list of all
systems' blocks, cuFFT runs one batched plan per distinct K, and the whole
step is one captured CUDA graph.  Two references run the same systems through
separate engines: ``run_loop`` one after the other, ``run_engines_graph`` as
independent branches of one captured graph.
"""
from __future__ import annotations

import math

import numpy as np

from . import TERM_ALL, Batch, Engine, next_smooth


def uneven_systems(count: int = 64, nmin: int = 500, nmax: int = 50_000, phi: float = 0.05,
                   radius: float = 1.0, xi: float = 0.3, rc: float = 10.0, orders=(4, 6, 8),
                   seed: int = 1234) -> list[dict]:
    """Systems with N log-uniform in [nmin, nmax], L for volume fraction phi,
    K the smallest 2^a 3^b 5^c >= 0.6 L and p drawn from `orders`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        L = (n * 4.0 / 3.0 * math.pi * radius ** 3 / phi) ** (1.0 / 3.0)
        K = next_smooth(int(math.ceil(0.6 * L)))
        p = int(rng.choice(orders))
        out.append(dict(N=n, L=L, K=max(K, p), p=p, xi=xi, rc=rc, radius=radius))
    return out


class SystemBatch:
    """Independent systems applied together.

    ``bind(pos, f, u)`` fixes the device buffers (lists of CUDA tensors:
    positions (N_i, 3) float64, right-hand sides (R, 3 N_i) and outputs of the
    batch precision) and packs them; ``run()`` is one native batched step
    (positions rebuilt, all systems applied, one graph launch) into the packed
    result, ``results()`` its per-system views; ``run_loop()`` and
    ``run_engines_graph()`` write the caller's ``u`` tensors through one engine
    per system."""

    def __init__(self, systems: list[dict], nrhs: int = 4, precision: str = "fp32",
                 terms: int = TERM_ALL, tune: bool = True):
        if terms != TERM_ALL:
            raise ValueError("a batch applies the full operator (TERM_ALL)")
        self.systems = systems
        self.nrhs = nrhs
        self.precision = precision
        self.tune = tune
        self.batch = Batch(systems, nrhs=nrhs, precision=precision)
        self.batch.set_graphs(True)
        self.engines = None
        self.graph = None
        self.tuned = None

    def _make_engines(self):
        if self.engines is None:
            self.engines = [Engine(s["N"], s["L"], s["xi"], s["K"], s["p"], radius=s["radius"],
                                   rcut=s["rc"], precision=self.precision, max_nrhs=self.nrhs,
                                   terms=TERM_ALL) for s in self.systems]

    def bind(self, pos, f, u):
        import torch
        self.pos, self.f, self.u = list(pos), list(f), list(u)
        self.pos_p = Batch.pack(self.pos).contiguous()
        self.f_p = Batch.pack(self.f).contiguous()
        self.u_p = torch.zeros_like(self.f_p)
        self.graph = None
        if self.tune:
            from .autotune import autotune_batch
            self.tuned, _ = autotune_batch(self.batch, self.pos_p, self.f_p, self.u_p)

    def run(self):
        """One batched step (one CUDA graph launch after the first call)."""
        self.batch.step(self.pos_p, self.f_p, self.u_p)

    def results(self):
        return self.batch.unpack(self.u_p)

    def _apply_one(self, k):
        self.engines[k].set_positions(self.pos[k])
        self.engines[k].apply(self.f[k], self.u[k])

    def run_loop(self):
        """Sequential per-system loop on the current stream."""
        self._make_engines()
        for k in range(len(self.engines)):
            self._apply_one(k)

    def capture_engines_graph(self):
        """Per-system engines as independent branches of one captured graph."""
        import torch
        self._make_engines()
        main = torch.cuda.Stream()
        streams = [torch.cuda.Stream() for _ in self.engines]
        # warm every engine on its stream (plans and TMA descriptors exist before capture)
        for k, s in enumerate(streams):
            with torch.cuda.stream(s):
                self._apply_one(k)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=main, capture_error_mode="thread_local"):
            fork = torch.cuda.Event()
            fork.record(main)
            joins = []
            for k, s in enumerate(streams):
                s.wait_event(fork)
                with torch.cuda.stream(s):
                    self._apply_one(k)
                    ev = torch.cuda.Event()
                    ev.record(s)
                joins.append(ev)
            for ev in joins:
                main.wait_event(ev)
        self.graph, self._streams, self._main = g, streams, main
        return g

    def run_engines_graph(self):
        if self.graph is None:
            self.capture_engines_graph()
        self.graph.replay()

    def close(self):
        self.graph = None
        if self.engines:
            for e in self.engines:
                e.close()
        self.batch.close()
