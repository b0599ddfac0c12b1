"""Uneven batches of independent systems in one CUDA-graph launch.

A batch holds systems of different N, box L, mesh K and order p (e.g. 64
systems with N between 500 and 50,000).  Each system is small: alone, its
spread launch may cover a few dozen tiles and leave most of the 152 SMs idle,
and a per-system loop pays ~20 launches per system.  Here every system keeps
its own engine (own streams, tiles picked by the autotuner) and the whole
batch — position builds and applies of all systems — is captured once into a
single CUDA graph in which the systems are independent branches; one graph
launch then runs them concurrently and fills the GPU.

cuFFT cannot run inside a persistent kernel, so the batch is a graph of
per-system kernels rather than one persistent kernel; the graph gives the
same single launch and concurrency.
"""
from __future__ import annotations

import math

import numpy as np

from . import TERM_ALL, Engine, next_smooth


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
    engine precision); ``capture()`` records one graph; ``run()`` replays it
    (positions rebuilt and all systems applied); ``run_loop()`` is the
    sequential per-system reference."""

    def __init__(self, systems: list[dict], nrhs: int = 4, precision: str = "fp32",
                 terms: int = TERM_ALL, tune: bool = True):
        self.systems = systems
        self.nrhs = nrhs
        self.tune = tune
        self.engines = [Engine(s["N"], s["L"], s["xi"], s["K"], s["p"], radius=s["radius"],
                               rcut=s["rc"], precision=precision, max_nrhs=nrhs, terms=terms)
                        for s in systems]
        self.graph = None
        self.tiles = [None] * len(systems)

    def bind(self, pos, f, u):
        self.pos, self.f, self.u = list(pos), list(f), list(u)
        self.graph = None
        if self.tune:
            from .autotune import autotune
            for k, eng in enumerate(self.engines):
                self.tiles[k], _ = autotune(eng, self.pos[k], self.f[k], reps=2)

    def _apply_one(self, k):
        self.engines[k].set_positions(self.pos[k])
        self.engines[k].apply(self.f[k], self.u[k])

    def run_loop(self):
        """Sequential per-system loop on the current stream."""
        for k in range(len(self.engines)):
            self._apply_one(k)

    def capture(self):
        import torch
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

    def run(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def close(self):
        self.graph = None
        for e in self.engines:
            e.close()
