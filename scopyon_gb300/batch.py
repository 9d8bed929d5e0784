"""Batched fields of view: many independent fields in one set of launches.

A study often simulates many small, independent fields of view, each with
its own image size, emitter count and diffusion coefficient; the reference
runs them one ``generate_images`` call at a time
(``src/scopyon/base.py:260-294``).  Here all fields are packed into one
canvas with a gap of 16 pixels (two tiles) between neighbours, and a frame
of every field is one frame of the canvas: one CUDA graph replay of the
record, binning, splat and camera kernels for the whole batch.

Why the canvas is exact: an emitter's footprint reaches at most
``ceil(999 nm / px) + 1`` pixels past its field (reflecting walls keep every
emitter inside its own field), which lands in the gap; the reference drops
those pixels at the image edge, and nothing reads the gap.  Each field keeps
its own diffusion coefficient (one diffusion class per field) and its own
walls.  ``field_image`` cuts a field's frame out of the canvas.

``autotune`` times a few (tile edge, warps per tile) choices of the splat on
the batch itself and keeps the fastest.
"""

import copy
import math

import numpy
import torch

from . import _lib
from .base import _psf_for
from .epifm import TILE_CANDIDATES, EngineConfig, FrameGraph, FramePipeline, tune_tiles
from .sampling import DeviceTrajectories

GAP = 16


def pack_fields(sizes, gap=GAP, width=8192):
    """Shelf packing of square fields (edge ``sizes[k]`` pixels, largest first)
    into rows of at most ``width`` pixels, ``gap`` pixels apart.  Returns the
    canvas (W, H) and each field's pixel origin (i0, j0)."""
    order = sorted(range(len(sizes)), key=lambda k: -sizes[k])
    origins = [None] * len(sizes)
    x = y = gap
    row_h = 0
    canvas_w = 0
    for k in order:
        s = int(sizes[k])
        if x + s + gap > width and x > gap:
            y += row_h + gap
            x, row_h = gap, 0
        origins[k] = (x, y)
        x += s + gap
        row_h = max(row_h, s)
        canvas_w = max(canvas_w, x)
    canvas_h = y + row_h + gap
    if canvas_w > 32767 or canvas_h > 32767:
        raise ValueError("fields do not fit a 32767-pixel canvas")
    return (canvas_w, canvas_h), origins


class BatchedFields:
    """Frames of many fields of view, one canvas frame per step.

    config: a ``Configuration`` for every field (image_size is replaced per
    field); sizes: field edges in pixels; counts: emitters per field; D:
    diffusion coefficient per field (m^2/s); frames: frames to simulate;
    substeps: sub-steps per exposure; frames_per_step: frames per ``step``
    (more than one pipelines them: each frame's records beside the previous
    frame's splat, see ``FrameGraph``).
    """

    def __init__(self, config, sizes, counts, D, frames, substeps, seed=0, device=None,
                 frames_per_step=1):
        self.device = torch.device(device or "cuda")
        self.sizes = [int(s) for s in sizes]
        self.counts = [int(c) for c in counts]
        self.D = numpy.asarray(D, dtype=float)
        self.canvas, self.origins = pack_fields(self.sizes)
        cfg = copy.deepcopy(config)
        cfg.update({"default": {"detector": {"image_size": list(self.canvas)}}})
        rng = numpy.random.RandomState(seed)
        self.eng = EngineConfig(cfg["default"], rng=rng)
        self.pipe = FramePipeline(self.eng, self.device, psf=_psf_for(self.eng, self.device))
        self.pipe.psf.ensure([0])  # two-dimensional inputs: every emitter at depth 0
        if self.pipe.camera_kind == _lib.CAM_SCMOS:
            self.pipe.scmos_sigma_map(rng)
        px = self.eng.px
        W, H = self.canvas
        pts, klass, boxes = [], [], []
        for k, (s, n) in enumerate(zip(self.sizes, self.counts)):
            i0, j0 = self.origins[k]
            lo = numpy.array([i0 * px - W * px / 2, j0 * px - H * px / 2, 0.0])
            hi = lo + numpy.array([s * px, s * px, 0.0])
            p = numpy.zeros((n, 4))
            p[:, 0] = rng.uniform(lo[0], hi[0], n)
            p[:, 1] = rng.uniform(lo[1], hi[1], n)
            pts.append(p)
            klass.append(numpy.full(n, k, dtype=numpy.int32))
            boxes.append(numpy.concatenate([lo, hi]))
        points = numpy.concatenate(pts)
        points[:, 2] = numpy.arange(len(points))
        points[:, 3] = 1.0
        self.n_emit = len(points)
        self.substeps = int(substeps)
        self.dt = self.eng.exposure_time / self.substeps
        times = numpy.arange(frames * self.substeps + 1) * self.dt
        Dk = numpy.repeat(self.D[:, None], 2, axis=1)
        self.traj = DeviceTrajectories(times, points, Dk, 2, int(rng.randint(0, 2 ** 31)),
                                       boundary="reflecting", klass=numpy.concatenate(klass),
                                       device=self.device, class_box=numpy.stack(boxes))
        self.pipe.ensure_slots(self.n_emit)
        if self.eng.bleaching:
            beta = self.eng.half_life / math.log(2.0)
            self.pipe.budget[:self.n_emit].copy_(torch.from_numpy(
                rng.exponential(beta, self.n_emit) * self.eng.n_emit0))
        self.graph = FrameGraph(self.pipe, self.traj, self.substeps, self.dt,
                                seed=int(rng.randint(0, 2 ** 31)), frames_per_step=frames_per_step)
        self.tuning = None

    # ------------------------------------------------------------------
    def autotune(self, candidates=TILE_CANDIDATES, frames=2):
        """Time whole batch frames (graph replays) for each (tile, warps)
        choice; keep the fastest.  Returns {(tile, warps): ms per frame}."""
        times = tune_tiles(self.graph, candidates, frames)
        name = "%dx%d tiles, %d warps, %d stages"
        self.tuning = {name % (t, t, w, st): ms for (t, w, st), ms in times.items()}
        self.tuning["chosen"] = name % (self.pipe.tile, self.pipe.tile, self.pipe.warps,
                                        self.pipe.stages)
        return times

    def step(self):
        """frames_per_step frames of every field (one graph replay once captured);
        field_image then shows the last of them."""
        self.graph.step()

    def field_image(self, k, what="adc"):
        """Frame of field k from the last step: 'adc' counts or 'expect' photons."""
        W, H = self.canvas
        src = self.pipe.adc32 if what == "adc" else self.pipe.expect
        i0, j0 = self.origins[k]
        s = self.sizes[k]
        return src.view(W, H)[i0:i0 + s, j0:j0 + s]
