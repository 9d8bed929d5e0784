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
CHUNK_PIXELS = 4096  # pixels of one camera work entry of the persistent frame


def batch_plan(canvas, tile, halo, origins, sizes, counts, chunk_pixels=CHUNK_PIXELS):
    """Work list of the persistent batched frame (``sc_batch_frame``).

    Fields are taken heaviest first (by emitters); each field contributes the
    tiles its pixels read that no earlier field queued, then its camera
    chunks, so every chunk comes after the tiles it waits for.  A pixel (i, j)
    reads the tile buffers (tx, ty) with tx * tile <= i < tx * tile + edge,
    edge = tile + halo (and the same along j).  Returns numpy arrays: work,
    tile_field_off, tile_field, field [n][4] (i0, j0, size, tiles read),
    chunk [m][2] (field, first pixel)."""
    W, H = canvas
    T, E = int(tile), int(tile) + int(halo)
    tiles_y = -(-H // T)
    n_tiles = (-(-W // T)) * tiles_y
    queued = numpy.zeros(n_tiles, dtype=bool)
    readers = [[] for _ in range(n_tiles)]
    work, chunks = [], []
    field = numpy.zeros((len(sizes), 4), dtype=numpy.int32)
    for f in sorted(range(len(sizes)), key=lambda k: -int(counts[k])):
        i0, j0 = origins[f]
        s = int(sizes[f])
        tx = numpy.arange(max(0, (i0 - E) // T + 1), (i0 + s - 1) // T + 1)
        ty = numpy.arange(max(0, (j0 - E) // T + 1), (j0 + s - 1) // T + 1)
        tiles = (tx[:, None] * tiles_y + ty[None, :]).ravel()
        for t in tiles.tolist():
            readers[t].append(f)
            if not queued[t]:
                queued[t] = True
                work.append(t)
        field[f] = (i0, j0, s, len(tiles))
        for first in range(0, s * s, chunk_pixels):
            chunks.append((f, first))
            work.append(-len(chunks))
    off = numpy.zeros(n_tiles + 1, dtype=numpy.int32)
    off[1:] = numpy.cumsum([len(r) for r in readers])
    flat = numpy.array([f for r in readers for f in r], dtype=numpy.int32)
    return (numpy.array(work, dtype=numpy.int32), off, flat, field,
            numpy.array(chunks, dtype=numpy.int32).reshape(-1, 2))


class _PersistentFrames(FrameGraph):
    """FrameGraph whose splat and camera are one persistent launch per frame
    (``sc_batch_frame``) over the batch's work list."""

    def __init__(self, batch, *args, **kwargs):
        self.batch = batch
        super().__init__(*args, **kwargs)

    def _image(self, recs, tag, frame_offset):
        pipe = self.pipe
        recs, bufs = recs
        sp = bufs[0]
        plan = self.batch.plan_for(pipe)
        sws_bytes = _lib.load().sc_splat_workspace_bytes(sp)
        sws = pipe._buf("splat_ws", (sws_bytes + 3) // 4, torch.float32)
        cp = pipe.camera_params(self.seed, frame_offset, self.frame)
        maps = pipe.pixel_maps
        expect, adc32 = self.outputs[frame_offset]
        with pipe.timed("batch_frame"):
            _lib.call("sc_batch_frame", _lib.ptr(recs), _lib.ptr(bufs[4]), _lib.ptr(bufs[3]),
                      _lib.ptr(pipe.psf.tables), _lib.ptr(pipe.psf.box), sp, plan, cp,
                      _lib.ptr(pipe.offset_f) if maps else None,
                      _lib.ptr(pipe.inv_gain_f) if maps else None, _lib.ptr(pipe.sigma),
                      _lib.ptr(pipe.table_value), _lib.ptr(pipe.table_cdf), _lib.ptr(sws),
                      sws_bytes, _lib.ptr(expect), _lib.ptr(adc32),
                      _lib.ptr(pipe.status), _lib.stream_ptr())


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
                 frames_per_step=1, persistent=False):
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
        graph_seed = int(rng.randint(0, 2 ** 31))
        self.persistent = bool(persistent)
        self._plan = None  # (tile, halo, ScBatchPlan, device arrays)
        self.spin_limit, self.target_extra = 0, 0  # test hooks of the persistent launch
        self.blocks_per_sm = 0  # persistent launch: resident blocks per SM (0: all that fit)
        if self.persistent:
            if not 12 <= self.pipe.psf.box_nq <= 16:
                raise ValueError("the persistent batched frame needs box tables with 12..16 "
                                 "pixel offsets per axis (160 nm pixels give 14)")
            self.graph = _PersistentFrames(self, self.pipe, self.traj, self.substeps, self.dt,
                                           seed=graph_seed, frames_per_step=frames_per_step)
        else:
            self.graph = FrameGraph(self.pipe, self.traj, self.substeps, self.dt,
                                    seed=graph_seed, frames_per_step=frames_per_step)
        self.tuning = None

    def plan_for(self, pipe):
        """The persistent launch's plan for the pipeline's current tile shape."""
        key = (pipe.tile, pipe.halo, self.spin_limit, self.target_extra, self.blocks_per_sm)
        if self._plan is None or self._plan[0] != key:
            work, off, flat, field, chunk = batch_plan(self.canvas, pipe.tile, pipe.halo,
                                                       self.origins, self.sizes, self.counts)
            dev = self.device

            def dt(a):
                return torch.from_numpy(numpy.ascontiguousarray(a, dtype=numpy.int32)
                                        .reshape(-1)).to(dev)

            arrays = dict(work=dt(work), off=dt(off), flat=dt(numpy.append(flat, 0)),
                          field=dt(field), chunk=dt(chunk),
                          counters=torch.zeros(2 + len(self.sizes), dtype=torch.int32,
                                               device=dev))
            plan = _lib.BatchPlan()
            plan.d_work, plan.d_tile_field_off = arrays["work"].data_ptr(), arrays["off"].data_ptr()
            plan.d_tile_field, plan.d_field = arrays["flat"].data_ptr(), arrays["field"].data_ptr()
            plan.d_chunk, plan.d_counters = arrays["chunk"].data_ptr(), arrays["counters"].data_ptr()
            plan.n_work, plan.n_fields = len(work), len(self.sizes)
            plan.n_chunks, plan.chunk_pixels = len(chunk), CHUNK_PIXELS
            plan.spin_limit, plan.target_extra = int(self.spin_limit), int(self.target_extra)
            plan.blocks_per_sm = int(self.blocks_per_sm)
            self._plan = (key, plan, arrays)
        return self._plan[1]

    # ------------------------------------------------------------------
    def autotune(self, candidates=TILE_CANDIDATES, frames=2, blocks_per_sm=(0, 4, 3, 2)):
        """Time whole batch frames (graph replays) for each (tile, warps,
        copies in flight) choice and keep the fastest; the persistent form then
        times the launch's resident blocks per SM (fewer leave room for the
        next frame's records on the side stream).  Returns {choice: ms per
        frame}, a choice being (tile, warps, stages) or ('blocks_per_sm', n)."""
        if self.persistent:  # its tiles always take the bulk-copy ring
            candidates = [cand for cand in candidates if cand[2] > 0]
        times = tune_tiles(self.graph, candidates, frames)
        name = "%dx%d tiles, %d warps, %d stages"
        self.tuning = {name % (t, t, w, st): ms for (t, w, st), ms in times.items()}
        self.tuning["chosen"] = name % (self.pipe.tile, self.pipe.tile, self.pipe.warps,
                                        self.pipe.stages)
        if self.persistent and len(blocks_per_sm) > 1:
            per = {}
            for n in blocks_per_sm:
                self.blocks_per_sm = n
                per[n] = tune_tiles(self.graph, [(self.pipe.tile, self.pipe.warps,
                                                  self.pipe.stages)], frames)[
                    (self.pipe.tile, self.pipe.warps, self.pipe.stages)]
                times[("blocks_per_sm", n)] = per[n]
            self.blocks_per_sm = min(per, key=per.get)
            self.tuning["blocks_per_sm"] = {str(k): v for k, v in per.items()}
            self.tuning["chosen_blocks_per_sm"] = self.blocks_per_sm
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
