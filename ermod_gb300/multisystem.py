"""Several independent systems in one CUDA graph, and the batch-size autotuner.

`SystemGraph` records one step -- frame plus placements -- of every system into one
CUDA graph (ermod_graph_create) and replays it with one launch per step; the systems
run concurrently.  Inputs live in device buffers that the caller overwrites in place
between launches (`set_frame`, `set_placements`).

`autotune_tiles` picks, per system, the tile shape -- the number of placements per PME
launch (the batch B: the tile of placements that the spectrum, transform and gather
kernels work on together) and per molecule-energy block (the finish group G) -- by timing
one step at each candidate with CUDA events.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


class SystemGraph:
    def __init__(self, engines, frames, placements, tags, sws=None):
        """engines: EnergyRepresentation per system (mixed precision), each after one
        ordinary step; frames: (sitepos, cell) per system; placements: (n, nsite, 3)
        solute coordinates per system, or None (solution mode: the in-frame solute);
        tags: the solute molecule (1-based) per system."""
        import torch
        self.engines = list(engines)
        n = len(self.engines)
        dev = torch.device("cuda", self.engines[0].device)
        self._pos = [torch.from_numpy(np.ascontiguousarray(f[0], np.float64)).to(dev) for f in frames]
        self._pl = [None if p is None else torch.from_numpy(np.ascontiguousarray(p, np.float64)).to(dev)
                    for p in placements]
        self.nplace = [1 if p is None else len(p) for p in placements]
        self._tag = [torch.full((m,), int(t), dtype=torch.int32, device=dev) for m, t in zip(self.nplace, tags)]
        self._sws = None if sws is None else [
            None if s is None else torch.from_numpy(np.asarray(s, np.float64)).to(dev) for s in sws]
        torch.cuda.synchronize(dev)
        vp = C.c_void_p

        def arr(xs):
            return (vp * n)(*[None if x is None else x.data_ptr() for x in xs])

        cells = np.concatenate([np.asfortranarray(f[1], np.float64).ravel(order="F") for f in frames])
        ctxs = (vp * n)(*[e.ctx for e in self.engines])
        nplace = np.array(self.nplace, np.int32)
        mol = np.array(tags, np.int32)
        out = vp()
        check(_lib.load().ermod_graph_create(n, ctxs, arr(self._pos), _lib.dp(cells), None, _lib.ip(nplace),
                                             _lib.ip(mol), arr(self._tag), arr(self._pl),
                                             None if self._sws is None else arr(self._sws), C.byref(out)),
              "ermod_graph_create")
        self.g = out

    def set_frame(self, i: int, sitepos):
        self._pos[i].copy_(self._pos[i].new_tensor(np.ascontiguousarray(sitepos, np.float64)))

    def set_placements(self, i: int, solute_sitepos):
        self._pl[i].copy_(self._pl[i].new_tensor(np.ascontiguousarray(solute_sitepos, np.float64)))

    def frame_buffer(self, i: int):
        """System i's coordinate buffer on the device (the graph's input), for callers that
        write the next frame into it themselves."""
        return self._pos[i]

    def launch_ordered(self, stream_handle: int):
        """One step, asynchronous on stream_handle, ordered after what the caller queued on
        that stream (its input copies included); no host wait."""
        check(_lib.load().ermod_graph_launch(self.g, C.c_void_p(stream_handle or None)), "ermod_graph_launch")

    def launch(self, stream_handle: int = 0):
        """One step of every system, asynchronous on stream_handle (the input copies on
        torch's current stream are waited for first)."""
        import torch
        torch.cuda.current_stream().synchronize()
        check(_lib.load().ermod_graph_launch(self.g, C.c_void_p(stream_handle or None)), "ermod_graph_launch")

    def sync(self):
        check(_lib.load().ermod_graph_sync(self.g), "ermod_graph_sync")

    def close(self):
        if self.g:
            _lib.load().ermod_graph_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_tiles(params, topo, bins, frame, placements, tag, batches=(32, 64, 128, 256), groups=(4, 8),
                   device=0):
    """The tile shape of one system with the highest placements/s on one step, timed with
    CUDA events after a warm-up step: the batch B (placements per PME launch: the tile of
    placements the spectrum, transform and gather kernels work on together) and the finish
    group G (placements per molecule-energy block: the real-space and binning tile).
    Returns (B, G, {(B, G): placements/s})."""
    import torch
    from .engproc import EnergyRepresentation
    n = len(placements)
    tags = np.full(n, tag, np.int32)
    rates = {}
    for B in batches:
        if B > max(4, n):
            continue
        for G in groups:
            if B % G:
                continue
            eng = EnergyRepresentation(params, topo, bins, precision="mixed", device=device, batch=B,
                                       finish_group=G)
            eng.frame(frame[0], frame[1])
            eng.placements(tags, placements)
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            t0.record()
            eng.frame(frame[0], frame[1])
            eng.placements(tags, placements)
            t1.record()
            torch.cuda.synchronize()
            rates[(B, G)] = n / (t0.elapsed_time(t1) / 1e3)
            eng.close()
    (B, G) = max(rates, key=rates.get)
    return B, G, rates


def autotune_batch(params, topo, bins, frame, placements, tag, candidates=(32, 64, 128, 256), device=0):
    """The batch size alone (finish group automatic): autotune_tiles over batches."""
    return autotune_tiles(params, topo, bins, frame, placements, tag, batches=candidates, groups=(8,),
                          device=device)[0]
