"""The reference's multi-slot DSP pipeline, GB300 style.

larsjoost/wgls-rs-fft examples/parallel_pipeline.rs runs, per slot, six
dispatch groups: H2D -> NOISE -> FFT (radix-4 passes) -> WINDOW -> IFFT
(radix-4 passes) -> SCALE -> D2H, with six slots in flight
(parallel_pipeline.rs:109, 644-735).  Here the device part is two launches of
this library's kernels: a forward transform that adds the pipeline's noise as
it loads each sample, and an inverse transform that multiplies the Hann window
over the bins as it loads and the 1/N scale as it stores.

Two ways to drive it:
  * run_frames(frames): the reference's loop -- each host frame goes through a
    slot (pinned staging, its own CUDA stream): host -> device copy, the two
    launches with the frame's index as the noise seed (the reference's
    frame_seed), device -> host copy; `slots` frames are in flight, and a
    slot's previous result is collected just before the slot is reused.
  * run_eager / capture / replay: device-resident batches only, the two
    launches of every slot captured once into a CUDA graph and replayed.
"""
from __future__ import annotations

import numpy as np
import torch

from ._lib import FORWARD, INVERSE, WINDOW_HANN, WINDOW_NONE, Context


class SpectralPipeline:
    """noise -> FFT -> Hann over the bins -> IFFT for `slots` device batches."""

    def __init__(self, n: int, batch: int, slots: int = 6, seed: int = 42, sigma: float = 0.1,
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

    def run_frames(self, frames, seed_base: int = 0):
        """Every host frame ([batch, n] complex64) through H2D -> noise + FFT ->
        window + IFFT (1/N) -> D2H, `slots` frames in flight; frame f uses noise
        seed seed_base + f.  Returns the outputs in frame order."""
        dev = self.inputs[0].device
        if not hasattr(self, "_pin_in"):
            self._pin_in = [torch.empty(self.batch, self.n, dtype=torch.complex64).pin_memory()
                            for _ in range(self.slots)]
            self._pin_out = [torch.empty_like(t).pin_memory() for t in self._pin_in]
            self._streams = [torch.cuda.Stream(device=dev) for _ in range(self.slots)]
            self._events = [torch.cuda.Event() for _ in range(self.slots)]
        busy = [None] * self.slots  # frame index in flight per slot
        results = [None] * len(frames)
        for f in range(len(frames) + self.slots):
            k = f % self.slots
            if busy[k] is not None:  # collect this slot's previous frame
                self._events[k].synchronize()
                results[busy[k]] = self._pin_out[k].numpy().copy()
                busy[k] = None
            if f >= len(frames):
                continue
            fr = np.ascontiguousarray(frames[f], dtype=np.complex64).reshape(self.batch, self.n)
            self._pin_in[k].numpy()[...] = fr
            st = self._streams[k]
            sp = st.cuda_stream
            with torch.cuda.stream(st):
                self.inputs[k].copy_(self._pin_in[k], non_blocking=True)
            self.fwd.set_noise(seed_base + f, self.sigma)  # read when the launch is enqueued
            self.fwd.c2c_device(self.inputs[k], self.spectra[k], self.n, self.batch, FORWARD, stream=sp)
            self.inv.c2c_device(self.spectra[k], self.outputs[k], self.n, self.batch, INVERSE, stream=sp)
            with torch.cuda.stream(st):
                self._pin_out[k].copy_(self.outputs[k], non_blocking=True)
                self._events[k].record(st)
            busy[k] = f
        self.fwd.set_noise(self.seed, self.sigma)
        return results

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
