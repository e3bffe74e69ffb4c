"""The reference's multi-slot DSP pipeline, GB300 style.

larsjoost/wgls-rs-fft examples/parallel_pipeline.rs runs, per slot, six
dispatch groups: H2D -> NOISE -> FFT (radix-4 passes) -> WINDOW -> IFFT
(radix-4 passes) -> SCALE -> D2H, with six slots in flight.  Here the
device part is two launches of this library's kernels: a forward transform
that adds the pipeline's noise as it loads each sample, and an inverse
transform that multiplies the Hann window over the bins as it loads and the
1/N scale as it stores.  The two launches of every slot are captured once into
a CUDA graph and replayed.
"""
from __future__ import annotations

import torch

from ._lib import FORWARD, INVERSE, WINDOW_HANN, WINDOW_NONE, Context


class SpectralPipeline:
    """noise -> FFT -> Hann over the bins -> IFFT for `slots` device batches."""

    def __init__(self, n: int, batch: int, slots: int = 2, seed: int = 42, sigma: float = 0.1,
                 device: int = 0):
        self.n, self.batch, self.slots = n, batch, slots
        self.seed, self.sigma = seed, sigma
        self.fwd = Context(device)       # one context per stage: their settings differ
        self.inv = Context(device)
        self.fwd.set_noise(seed, sigma)
        self.inv.set_window(WINDOW_HANN)
        dev = torch.device("cuda", device)
        self.inputs = [torch.zeros(batch, n, dtype=torch.complex64, device=dev) for _ in range(slots)]
        self.spectra = [torch.empty_like(t) for t in self.inputs]
        self.outputs = [torch.empty_like(t) for t in self.inputs]
        self.stream = torch.cuda.Stream(device=dev)
        self.graph = None

    def _enqueue(self, s):
        for i in range(self.slots):
            self.fwd.c2c_device(self.inputs[i], self.spectra[i], self.n, self.batch, FORWARD, stream=s)
            self.inv.c2c_device(self.spectra[i], self.outputs[i], self.n, self.batch, INVERSE, stream=s)

    def run_eager(self):
        s = self.stream.cuda_stream
        self._enqueue(s)

    def capture(self):
        """Build plans and tables eagerly, then capture every slot's launches."""
        self.run_eager()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._enqueue(self.stream.cuda_stream)
        return self

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def close(self):
        self.fwd.set_noise(0, 0.0)
        self.inv.set_window(WINDOW_NONE)
        self.fwd.close()
        self.inv.close()
