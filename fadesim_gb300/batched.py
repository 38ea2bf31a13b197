"""Batches of crossbar tiles of uneven size, solved as one GPU job.

A layer (or any workload) can hold tiles of several sizes, each with its own
input vectors.  Tiles are grouped by shape; every group is one launch of a
persistent solver kernel -- shared-memory tile-per-CTA up to 128 x 128,
cluster-per-tile up to 512 x 512, or the layout the autotuner picked -- whose
CTAs (clusters) claim (tile, vector chunk) items from the call's device-side
queue, and the groups run concurrently on forked streams.
``TileBatch.capture()`` records the whole job as one CUDA graph for replay
(inputs updated in place between replays).  ``TileBatch.tune()`` runs the
project's autotuner (``fadesim_gb300.autotune``) on a sample of every group;
per-shape launch parameters come from its cache.
"""
import torch

from . import autotune
from . import cpp_ir_drop_accelerate as _acc


class TileGroup:
    """Tiles of one shape: G [T, n, m] and inputs vin [B, T, n] (contiguous, CUDA)."""

    def __init__(self, G, vin):
        if G.dim() != 3 or vin.dim() != 3 or vin.shape[1] != G.shape[0] or vin.shape[2] != G.shape[1]:
            raise ValueError("TileGroup wants G [T, n, m] and vin [B, T, n]")
        self.G = G.contiguous()
        self.vin = vin.contiguous()
        self.T, self.n, self.m = G.shape
        self.B = vin.shape[0]
        self.out = torch.empty((self.B, self.T, self.m), dtype=G.dtype, device=G.device)

    @property
    def solves(self):
        return self.B * self.T


class TileBatch:
    """Several TileGroups solved together (one group per shape)."""

    def __init__(self, groups, g_wire=1 / 2.93, method="line", tol_v=None, residual="ff", tuned=True,
                 concurrent=True):
        self.groups = list(groups)
        self.g_wire = g_wire
        self.method = method
        self.tol_v = tol_v  # None: the module-wide cpp_ir_drop_accelerate.options.tol_v
        self.residual = residual
        self.tuned = tuned
        # concurrent: one forked stream per group; else the groups run one after
        # another on the caller's stream, largest tiles first
        self.concurrent = concurrent
        self.streams = [torch.cuda.Stream() for _ in self.groups] if concurrent else None
        self.graph = None

    @property
    def solves(self):
        return sum(g.solves for g in self.groups)

    def _launch(self, g, stream, stats):
        kw = autotune.lookup(g.n, g.m, self.method) if self.tuned else {}
        method = kw.pop("method", self.method)  # the tuner may pick the two-level method
        with torch.cuda.stream(stream):
            _, st, _ = _acc.ir_drop_gs_ex(g.vin, g.G, g.B, g.n, g.m, g.T, 1, g_wire=self.g_wire, method=method,
                                          tol_v=self.tol_v, residual=self.residual, return_stats=stats,
                                          out=g.out, **kw)
        return st

    def run(self, stats=False):
        """Solve every group; returns the per-group stats when ``stats``."""
        main = torch.cuda.current_stream()
        if not self.concurrent:
            order = sorted(range(len(self.groups)), key=lambda i: -self.groups[i].n * self.groups[i].m)
            res = {i: self._launch(self.groups[i], main, stats) for i in order}
            return [res[i] for i in range(len(self.groups))] if stats else None
        ev = torch.cuda.Event()
        ev.record(main)
        # largest tiles first: the cluster kernels take whole clusters of SMs
        # (36 four-CTA clusters use 144 of 152), and the tile-per-CTA kernels
        # launched after them start on the SMs left over, their CTAs claiming
        # work items from the device queue as SMs free up
        order = sorted(range(len(self.groups)), key=lambda i: -self.groups[i].n * self.groups[i].m)
        res = {}
        for i in order:
            self.streams[i].wait_event(ev)
            res[i] = self._launch(self.groups[i], self.streams[i], stats)
        for s in self.streams:
            main.wait_stream(s)
        return [res[i] for i in range(len(self.groups))] if stats else None

    def tune(self, sample_tiles=304, reps=2):
        """Autotune every group's launch parameters (kernel layout, vectors per
        work item, precise-residual period, and on strongly coupled 128 x 128
        tiles the two-level method) on its first ``sample_tiles`` tiles
        and cache the winners; later runs use them when ``tuned``.  Returns
        {shape: (kwargs, ms)}."""
        out = {}
        for g in self.groups:
            k = min(g.T, sample_tiles)
            out["%dx%d" % (g.n, g.m)] = autotune.tune(g.G[:k].contiguous(), g.vin[:, :k].contiguous(),
                                                      g_wire=self.g_wire, method=self.method, reps=reps)
        return out

    def capture(self):
        """Record run() as a CUDA graph (warm-up launch first, as graph capture needs)."""
        self.run()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.run()
        return self.graph

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def outputs(self):
        return [g.out for g in self.groups]
