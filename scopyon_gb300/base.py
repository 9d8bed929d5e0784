"""Public API, a drop-in for ``scopyon.form_image`` / ``scopyon.generate_images``.

Signatures, input layouts, return values and errors follow the reference
(src/scopyon/base.py:28-294).  Extensions, all keyword-only and optional:
``device`` (CUDA device), ``draws`` (an ``InjectedDraws`` replacing the
camera / bleaching random draws, the reference-parity mode).

Random numbers: the caller's ``rng`` (a numpy RandomState) supplies, in the
reference's order, the fixed-pattern-noise offsets and the photobleaching
budgets; the camera noise of each frame comes from on-device Philox streams
keyed by one 64-bit seed drawn from ``rng`` per frame.  Pixel statistics
match the reference's models; the individual draws differ unless ``draws``
is given.
"""

import collections.abc
import concurrent.futures
import math
import numbers
import os
import warnings

import numpy

from . import _lib
from . import config as _config
from .epifm import (EngineConfig, FramePipeline, HostRowsGraph, InjectedDraws, PSFTables,
                    frame_windows)
from .image import Image
from .sampling import DeviceTrajectories

__all__ = ["EPIFMSimulator", "create_simulator", "form_image", "generate_images",
           "EnvironSettings", "InjectedDraws"]


class EnvironSettings:
    """``environ`` sub-tree (reference base.py:20-26); ``processes`` is accepted and unused."""

    def __init__(self, config):
        self.processes = config.processes


def _as_config(config):
    if config is None:
        return _config.DefaultConfiguration()
    if isinstance(config, str):
        return _config.Configuration(filename=config)
    if isinstance(config, _config.Configuration):
        return config
    if hasattr(config, "yaml") and isinstance(getattr(config, "yaml"), dict):
        return _config.Configuration.from_reference(config)
    raise TypeError("Configuration or str must be given [{}].".format(type(config)))


# PSF tables and device buffers survive across calls with the same optics
_PSF_CACHE = {}


def _psf_for(cfg, device):
    key = (str(device), cfg.fluorophore_type, float(cfg.psf_wavelength), cfg.na,
           float(cfg.radial_width or 0.0), float(cfg.radial_cutoff), float(cfg.depth_cutoff),
           cfg.box_p)
    tables = _PSF_CACHE.get(key)
    if tables is None:
        tables = _PSF_CACHE[key] = PSFTables(cfg, device)
    return tables


class EPIFMSimulator:

    def __init__(self, config=None, method=None, rng=None, device=None):
        config = _as_config(config)
        if rng is None:
            warnings.warn("A random number generator is not given.")
            rng = numpy.random.RandomState()
        self.__config = config
        self.__method = (method or config.get("method", "default")).lower()
        self.__rng = rng
        self.__device = device or "cuda"

    @property
    def config(self):
        return self.__config

    @property
    def method(self):
        return self.__method

    def base(self):
        """Engine configuration of the method sub-tree (draws FPN offsets from rng)."""
        return EngineConfig(self.__config[self.__method], rng=self.__rng)

    def _format_data(self, inputs):
        """Columns -> [depth, x, y, m_id, p_state] (reference base.py:61-110)."""
        if not isinstance(inputs, numpy.ndarray):
            raise TypeError("a numpy.ndarray is expected")
        if inputs.ndim != 2:
            raise ValueError("The given 'inputs' has wrong dimension.")
        pre = self.__config.preprocessing
        k = inputs.shape[1]
        n = inputs.shape[0]
        if k == 2:
            data = numpy.hstack((numpy.zeros((n, 1)), inputs * pre.scale))
            data = numpy.hstack((data, numpy.zeros((n, 2))))
            data[:, 3] = numpy.arange(n)
            data[:, 4] = 1.0
        elif k in (3, 5):
            origin = numpy.array(pre.origin)
            pos = inputs[:, :3] * pre.scale - origin
            unit_z = numpy.cross(pre.unit_x, pre.unit_y)
            data = numpy.hstack((numpy.dot(pos, unit_z).reshape((-1, 1)),
                                 numpy.dot(pos, pre.unit_x).reshape((-1, 1)),
                                 numpy.dot(pos, pre.unit_y).reshape((-1, 1))))
            if k == 3:
                data = numpy.hstack((data, numpy.zeros((n, 2))))
                data[:, 3] = numpy.arange(n)
                data[:, 4] = 1.0
            else:
                data = numpy.hstack((data, inputs[:, 3:]))
        elif k == 4:
            data = numpy.hstack((numpy.zeros((n, 1)), inputs[:, :2] * pre.scale, inputs[:, 2:]))
        else:
            raise ValueError("The given 'inputs' has wrong shape.")
        return data

    def _format_inputs(self, inputs):
        if isinstance(inputs, DeviceTrajectories):
            return inputs
        if isinstance(inputs, numpy.ndarray):
            return ((0.0, self._format_data(inputs)),)
        if isinstance(inputs, collections.abc.Iterable):
            data = []
            for elem in inputs:
                if not (isinstance(elem, (tuple, list)) and len(elem) == 2
                        and isinstance(elem[0], numbers.Real) and isinstance(elem[1], numpy.ndarray)):
                    raise ValueError("The given 'inputs' has wrong type.")
                data.append((elem[0], self._format_data(elem[1])))
            return data
        raise TypeError("Invalid argument was given [{}]. A ndarray is expected.".format(type(inputs)))

    def form_image(self, inputs, start_time=0.0, exposure_time=None, full_output=False, *,
                   draws=None):
        """Form one image; returns ``Image`` or ``(Image, infodict)`` like scopyon."""
        data = self._format_inputs(inputs)
        cfg = self.base()
        img, info = next(_Frames(self, cfg, data, 1, start_time, exposure_time, False, draws,
                                 full_output))
        if full_output:
            return img, info
        return img

    def generate_images(self, inputs, num_frames, start_time=0.0, exposure_time=None,
                        full_output=False, *, draws=None):
        """Yield ``num_frames`` images (with infodicts if ``full_output``)."""
        data = self._format_inputs(inputs)
        cfg = self.base()
        for img, info in _Frames(self, cfg, data, num_frames, start_time, exposure_time,
                                 cfg.bleaching, draws, full_output):
            yield (img, info) if full_output else img

    # access for _Frames
    def _rng(self):
        return self.__rng

    def _device(self):
        return self.__device


_POOL = None


def _host_pool():
    """Threads for the per-sub-step host copies (numpy releases the GIL)."""
    global _POOL
    if _POOL is None:
        _POOL = concurrent.futures.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
    return _POOL


_AHEAD = None


def _ahead_pool():
    """One thread that stages the next frame's inputs (it fans out to
    _host_pool) while the current frame runs on the device."""
    global _AHEAD
    if _AHEAD is None:
        _AHEAD = concurrent.futures.ThreadPoolExecutor(max_workers=1)
    return _AHEAD


def _stage_known(arrays, slot_ids_f, staging):
    """Copies each sub-step's array into the pinned staging buffer, on the
    host threads, when every array has exactly the known ids in slot order;
    returns (depth min, depth max), or None when the ids differ (the caller
    then takes the general path).  Row-major float64 arrays go through
    ``sc_stage_rows`` (one native pass per sub-step, GIL released); others
    through numpy."""
    n = len(slot_ids_f)
    lib = _lib.load()
    ids = numpy.ascontiguousarray(slot_ids_f, dtype=numpy.float64)

    def one(k):
        a = arrays[k]
        if a.shape != (n, 5):
            return None
        if a.dtype == numpy.float64 and a.flags.c_contiguous:
            rng_ = numpy.empty(2)
            rc = lib.sc_stage_rows(a.ctypes.data, n, ids.ctypes.data, staging[k].ctypes.data,
                                   rng_.ctypes.data)
            if rc == 1:
                return None
            _lib.check(rc, "sc_stage_rows")
            return float(rng_[0]), float(rng_[1])
        if not numpy.array_equal(a[:, 3], slot_ids_f):
            return None
        numpy.copyto(staging[k], a)
        d = staging[k, :, 0]
        return float(d.min()), float(d.max())

    res = list(_host_pool().map(one, range(len(arrays))))
    if any(r is None for r in res):
        return None
    if any(math.isnan(r[0]) or math.isnan(r[1]) for r in res):
        return math.nan, math.nan  # refused by ensure_depth_range
    return min(r[0] for r in res), max(r[1] for r in res)


_PIN_LIMIT = 8 << 30  # bytes of formatted inputs kept in one pinned host block


class _PinnedInputs:
    """The formatted inputs of a frame sequence in one pinned host block, so
    that each frame's sub-steps are uploaded straight from it (one
    asynchronous copy, no host copy per frame).  Built once, on the host
    threads, when every array is (n, 5) with the same n and the block stays
    under _PIN_LIMIT bytes.  Per array it keeps the depth range and whether
    its ids equal the first array's, row for row."""

    def __init__(self, arrays):
        import torch
        n = arrays[0].shape[0]
        self.ids = numpy.ascontiguousarray(arrays[0][:, 3], dtype=numpy.float64)
        self._t = torch.empty(len(arrays) * n * 5, dtype=torch.float64, pin_memory=True)
        self.block = self._t.numpy().reshape(len(arrays), n, 5)
        self.lo = numpy.empty(len(arrays))
        self.hi = numpy.empty(len(arrays))
        self.same = numpy.zeros(len(arrays), dtype=bool)
        lib = _lib.load()

        def one(k):
            a = numpy.ascontiguousarray(arrays[k], dtype=numpy.float64)
            rng_ = numpy.empty(2)
            rc = lib.sc_stage_rows(a.ctypes.data, n, self.ids.ctypes.data,
                                   self.block[k].ctypes.data, rng_.ctypes.data)
            if rc == 1:  # other ids: copied without the check
                numpy.copyto(self.block[k], a)
                d = a[:, 0]
                rng_[:] = (d.min(), d.max())  # NaN when a depth is NaN
            else:
                _lib.check(rc, "sc_stage_rows")
                self.same[k] = True
            self.lo[k], self.hi[k] = rng_

        list(_host_pool().map(one, range(len(arrays))))

    @classmethod
    def build(cls, data):
        arrays = [a for _, a in data]
        if len(arrays) < 2:
            return None
        n = arrays[0].shape[0]
        if n == 0 or any(a.shape != (n, 5) for a in arrays) or len(arrays) * n * 40 > _PIN_LIMIT:
            return None
        return cls(arrays)

    def frame(self, idx):
        """(particles, depth min, depth max) of the arrays idx, a run of
        consecutive indices that all hold the first array's ids; None
        otherwise."""
        i0, i1 = idx[0], idx[-1] + 1
        if i1 - i0 != len(idx) or not self.same[i0:i1].all():
            return None
        return self.block[i0:i1], float(self.lo[i0:i1].min()), float(self.hi[i0:i1].max())


def _finish(pipe, out, nw, nh):
    """The Image of a frame whose counts frame_out is copying to the host:
    waits for the copy, raises what the frame's status words record."""
    ev, counts, status = out
    ev.synchronize()
    pipe.raise_for_status(status)
    return Image(counts.reshape(nw, nh).astype(numpy.float64)), {}


def _Frames(sim, cfg, data, num_frames, start_time, exposure_time, bleaching, draws,
            full_output=True):
    """Frame generator: host bookkeeping around FramePipeline.run_frame.

    When it ends or is closed, it waits for the device: the uploads and
    read-backs it issued through the library (one cudaMemcpyAsync each) are
    not known to torch's pinned-memory cache, which could otherwise hand a
    pinned buffer they still use to a new allocation."""
    import torch
    try:
        yield from _frames(sim, cfg, data, num_frames, start_time, exposure_time, bleaching,
                           draws, full_output)
    finally:
        if torch.cuda.is_initialized():
            torch.cuda.synchronize(torch.device(sim._device()))


def _frames(sim, cfg, data, num_frames, start_time, exposure_time, bleaching, draws,
            full_output):
    import torch
    rng = sim._rng()
    device = torch.device(sim._device())
    pipe = FramePipeline(cfg, device, psf=_psf_for(cfg, device))
    if pipe.camera_kind == _lib.CAM_SCMOS:
        pipe.scmos_sigma_map(rng)
    if isinstance(data, DeviceTrajectories):
        yield from _DeviceFrames(sim, cfg, pipe, data, num_frames, start_time, exposure_time,
                                 bleaching, draws, full_output)
        return
    exposure = exposure_time or cfg.exposure_time
    times = numpy.array([t for t, _ in data])
    shutter = (cfg.shutter_start, cfg.shutter_end) if cfg.shutter_switch else None
    slots = {}
    slot_ids = []
    slot_arr = numpy.zeros(0, dtype=numpy.int64)
    beta = cfg.half_life / numpy.log(2.0) if bleaching else None
    focal0 = cfg.focal_point[0]
    nw, nh = cfg.image_size
    slot_ids_f = None
    pending = None  # (frame, staging, future): the next frame's inputs, staged ahead
    # frames on the fast paths are yielded one frame late: frame f's counts
    # are read back while frame f + 1 runs on the device
    out = None
    pinned = _PinnedInputs.build(data) if num_frames > 1 and not full_output else None
    if pinned is not None and isinstance(data, list):
        for k in range(len(data)):  # the formatted arrays live on in the block only
            data[k] = (data[k][0], pinned.block[k])
    pinned_ok = None  # the slot order equals the pinned block's ids
    host_graph = None  # native frames from the pinned block: graph replays
    seq_seed = []

    def native_seed():
        """The camera's Philox key for the sequence's native frames (drawn
        from rng at the first; each frame's counter is its index)."""
        if not seq_seed:
            seq_seed.append(int(rng.randint(0, 2 ** 31 - 1)) << 31 | int(rng.randint(0, 2 ** 31 - 1)))
        return seq_seed[0]
    for f in range(num_frames):
        ahead = None
        if pending is not None:
            ahead = (pending[1], pending[2].result()) if pending[0] == f else None
            pending = None
        windows, exp_eff = frame_windows(times, len(data), start_time, exposure, f, shutter)
        uts = numpy.array([ut for _, ut in windows], dtype=float)
        if windows and slot_ids_f is not None and not full_output and pinned is not None:
            # the usual case: the same particles in the same order at every
            # sub-step, uploaded from the pinned block
            if pinned_ok is None:
                pinned_ok = numpy.array_equal(slot_ids_f, pinned.ids)
            got = pinned.frame([i for i, _ in windows]) if pinned_ok else None
            if got is not None:
                particles, lo, hi = got
                try:
                    pipe.ensure_slots(len(slot_ids_f))
                    pipe.psf.ensure_depth_range(lo - focal0, hi - focal0)
                    frame_draws = draws.next_frame() if draws is not None and draws.frames else None
                    if frame_draws is None:
                        n_sub = particles.shape[0]
                        if host_graph is None or (host_graph.n_sub, host_graph.n) != \
                                (n_sub, particles.shape[1]):
                            host_graph = HostRowsGraph(pipe, n_sub, particles.shape[1],
                                                       native_seed(), bleaching)
                        adc = host_graph.run(particles, uts, f)
                    else:
                        _, adc, _ = pipe.run_frame(particles, uts, with_optinfo=False,
                                                   draws=frame_draws, seed=0, counter=f,
                                                   present=None, bleaching=bleaching,
                                                   track_upload=False)
                    nxt = pipe.frame_out(adc, slot=f % 2)
                except Exception:
                    if out is not None:  # the frame before first, then the error
                        yield _finish(pipe, out, nw, nh)
                    raise
                if out is not None:
                    yield _finish(pipe, out, nw, nh)
                out = nxt
                continue
        arrays = [data[i][1] for i, _ in windows]
        if arrays and slot_ids_f is not None and not full_output:
            # the same particles in the same order at every sub-step; staged
            # on the host threads (while the previous frame ran), no per-frame
            # id scan
            if ahead is not None:
                staging, rng_ = ahead
            else:
                staging = pipe.host_staging((len(arrays), len(slot_ids_f), 5), slot=f % 2)
                rng_ = _stage_known(arrays, slot_ids_f, staging)
            if rng_ is not None:
                try:
                    pipe.ensure_slots(len(slot_ids_f))
                    pipe.psf.ensure_depth_range(rng_[0] - focal0, rng_[1] - focal0)
                    frame_draws = draws.next_frame() if draws is not None and draws.frames else None
                    seed = native_seed() if frame_draws is None else 0
                    _, adc, _ = pipe.run_frame(staging, uts, with_optinfo=False,
                                               draws=frame_draws, seed=seed, counter=f,
                                               present=None, bleaching=bleaching)
                except Exception:
                    if out is not None:  # the frame before first, then the error
                        yield _finish(pipe, out, nw, nh)
                    raise
                if f + 1 < num_frames:
                    w_next, _ = frame_windows(times, len(data), start_time, exposure, f + 1,
                                              shutter)
                    a_next = [data[i][1] for i, _ in w_next]
                    if a_next:
                        # the other slot's last upload (frame f - 1) is complete
                        st_next = pipe.host_staging((len(a_next), len(slot_ids_f), 5),
                                                    slot=(f + 1) % 2)
                        pending = (f + 1, st_next,
                                   _ahead_pool().submit(_stage_known, a_next, slot_ids_f, st_next))
                nxt = pipe.frame_out(adc, slot=f % 2)
                if out is not None:
                    yield _finish(pipe, out, nw, nh)
                out = nxt
                continue
        if out is not None:
            yield _finish(pipe, out, nw, nh)
            out = None
        new_ids = []
        id_cols = [a[:, 3].astype(numpy.int64) for a in arrays]
        same = len(arrays) > 0 and all(ids.shape == id_cols[0].shape and numpy.array_equal(ids, id_cols[0])
                                       for ids in id_cols)
        known = same and slot_arr.shape == id_cols[0].shape and numpy.array_equal(slot_arr, id_cols[0])
        if not known:
            for ids in (id_cols[:1] if same else id_cols):
                for m in ids.tolist():
                    if m not in slots:
                        slots[m] = len(slots)
                        slot_ids.append(m)
                        new_ids.append(m)
            slot_arr = numpy.array(slot_ids, dtype=numpy.int64)
        n_slots = len(slots)
        slot_ids_f = numpy.asarray(slot_ids, dtype=float) if same else None
        pinned_ok = None
        pipe.ensure_slots(n_slots)
        if bleaching and new_ids:
            times_b = numpy.empty(len(new_ids))
            todo = [k for k, m in enumerate(new_ids) if not (draws and m in draws.bleach)]
            if todo:
                times_b[todo] = rng.exponential(scale=beta, size=len(todo))
            for k, m in enumerate(new_ids):
                if draws and m in draws.bleach:
                    times_b[k] = draws.bleach[m]
            idx = torch.tensor([slots[m] for m in new_ids], dtype=torch.int64, device=device)
            pipe.budget.index_copy_(0, idx, torch.from_numpy(times_b * cfg.n_emit0).to(device))
        s_count = len(arrays)
        present = None
        if s_count == 0:
            particles = numpy.zeros((0, n_slots, 5))
        elif same and slot_arr.shape == id_cols[0].shape and numpy.array_equal(slot_arr, id_cols[0]):
            particles = pipe.host_staging((s_count, n_slots, 5))
            numpy.stack(arrays, out=particles)
        else:
            particles = numpy.zeros((s_count, n_slots, 5))
            present = numpy.zeros((s_count, n_slots), dtype=numpy.uint8)
            for s_i, a in enumerate(arrays):
                sl = numpy.array([slots[m] for m in id_cols[s_i].tolist()], dtype=numpy.int64)
                particles[s_i, sl] = a
                present[s_i, sl] = 1
        if s_count:
            depth = particles[:, :, 0]
            pipe.psf.ensure_depth_range(float(depth.min()) - focal0, float(depth.max()) - focal0)
        frame_draws = draws.next_frame() if draws is not None and draws.frames else None
        seed = native_seed() if frame_draws is None else 0
        expect, adc, opt = pipe.run_frame(particles, uts, with_optinfo=full_output,
                                          draws=frame_draws, seed=seed, counter=f,
                                          present=present, bleaching=bleaching)
        pipe.check_status()
        adc_np = adc.cpu().numpy().reshape(nw, nh).astype(numpy.float64)
        info = {}
        if full_output:
            info["expectation"] = expect.cpu().numpy().astype(float).reshape(nw, nh)
            info["true_data"] = _true_data(cfg, opt, slots, id_cols, exp_eff, nw, nh)
        if bleaching and full_output:
            b = pipe.budget[:n_slots].cpu().numpy()
            info["fluorescence_states"] = {m: float(b[slots[m]]) for m in slot_ids}
        yield Image(adc_np), info
    if out is not None:
        yield _finish(pipe, out, nw, nh)


def _DeviceFrames(sim, cfg, pipe, traj, num_frames, start_time, exposure_time, bleaching, draws,
                  full_output):
    """Frames from device-resident trajectories: diffusion, physics, splat and camera
    all on the GPU; the host only picks each frame's time window."""
    import torch
    rng = sim._rng()
    device = pipe.device
    pre = sim.config.preprocessing
    transform = {}
    if traj.ndim == 3:
        transform = dict(scale=pre.scale, origin=pre.origin, unit_x=pre.unit_x, unit_y=pre.unit_y)
    else:
        transform = dict(scale=pre.scale)
    exposure = exposure_time or cfg.exposure_time
    shutter = (cfg.shutter_start, cfg.shutter_end) if cfg.shutter_switch else None
    n = traj.n_particles
    ids = traj.ids().astype(numpy.int64)
    nw, nh = cfg.image_size
    pipe.ensure_slots(n)
    if bleaching:
        beta = cfg.half_life / numpy.log(2.0)
        times_b = numpy.empty(n)
        todo = [k for k in range(n) if not (draws and int(ids[k]) in draws.bleach)]
        if todo:
            times_b[todo] = rng.exponential(scale=beta, size=len(todo))
        for k in range(n):
            if draws and int(ids[k]) in draws.bleach:
                times_b[k] = draws.bleach[int(ids[k])]
        pipe.budget[:n].copy_(torch.from_numpy(times_b * cfg.n_emit0))
    slots = {int(m): k for k, m in enumerate(ids)}
    for f in range(num_frames):
        windows, exp_eff = frame_windows(traj.times, len(traj), start_time, exposure, f, shutter)
        if windows:
            g0, g1 = windows[0][0], windows[-1][0]
        else:
            g0 = g1 = None
        n_sub = 0 if g0 is None else g1 - g0 + 1
        uts = numpy.zeros(n_sub)
        for i, ut in windows:
            uts[i - g0] = ut
        # native trajectories with the identity transform: 16-byte FP32 rows
        layout = 1 if traj.compact_rows(transform) else 0
        width = 4 if layout else 5
        part = pipe._buf("particles32" if layout else "particles", max(n_sub, 1) * n * width,
                         torch.float32 if layout else torch.float64)
        if n_sub:
            traj.run(g0, n_sub, part, transform, layout=layout)
            if len(pipe.psf.slot_of) < pipe.psf.max_key + 2:
                pipe.psf.ensure(_device_depth_keys(
                    cfg, part[: n_sub * n * width].view(n_sub, n, width).double()))
        ut_dev = torch.from_numpy(uts).to(device)
        frame_draws = draws.next_frame() if draws is not None and draws.frames else None
        seed = int(rng.randint(0, 2 ** 31 - 1)) << 31 | int(rng.randint(0, 2 ** 31 - 1)) \
            if frame_draws is None else 0
        expect, adc, opt = pipe.run_frame_device(part, ut_dev, n_sub, n, with_optinfo=full_output,
                                                 draws=frame_draws, seed=seed, counter=f,
                                                 bleaching=bleaching, row_layout=layout)
        pipe.check_status()
        adc_np = adc.cpu().numpy().reshape(nw, nh).astype(numpy.float64)
        info = {}
        if full_output:
            info["expectation"] = expect.cpu().numpy().astype(float).reshape(nw, nh)
            info["true_data"] = _true_data(cfg, opt, slots, [ids] if n_sub else [], exp_eff, nw, nh)
            if bleaching:
                b = pipe.budget[:n].cpu().numpy()
                info["fluorescence_states"] = {int(m): float(b[k]) for k, m in enumerate(ids)}
        yield Image(adc_np), info


def _device_depth_keys(cfg, part):
    """Distinct PSF depth keys of formatted device particles (same rule as depth_keys)."""
    import torch
    d = (part[:, :, 0] - float(cfg.focal_point[0])).abs().reshape(-1)
    inside = d < cfg.depth_cutoff + 1e-9
    keys = torch.where(inside, torch.floor(d / 1e-9), torch.full_like(d, -1.0))
    return torch.unique(keys).cpu().numpy().astype(numpy.int64)


def _true_data(cfg, opt, slots, id_cols, exposure, nw, nh):
    """Per-molecule 8-vectors of the frame (_epifm.py:1207-1216, :1322-1333)."""
    if opt is None or not id_cols:
        return {}
    seen = []
    mark = set()
    for ids in id_cols:
        for m in ids.tolist():
            if m not in mark:
                mark.add(m)
                seen.append(m)
    o = opt.cpu().numpy()[[slots[m] for m in seen]].copy()
    p0 = cfg.focal_point
    px = cfg.px
    o[:, 1] /= exposure
    o[:, 2:6] /= o[:, 0:1]
    o[:, 2] = (o[:, 2] - p0[1]) / px + (nw - 1) * 0.5
    o[:, 3] = (o[:, 3] - p0[2]) / px + (nh - 1) * 0.5
    return {m: o[k] for k, m in enumerate(seen)}


def create_simulator(config=None, method=None, rng=None, device=None):
    """Return a simulator for ``config[method].type`` (reference base.py:203-225)."""
    config = _as_config(config)
    method = (method or config.get("method", "default")).lower()
    kind = str(config[method].type).lower()
    if kind in ("epifm", "epifm_gpu"):
        return EPIFMSimulator(config=config, method=method, rng=rng, device=device)
    raise ValueError(f"An unknown type [{kind}] was given.")


def form_image(inputs, start_time=0.0, exposure_time=None, *, method=None, config=None, rng=None,
               full_output=False, device=None, draws=None):
    """Form one image (reference base.py:227-258)."""
    sim = create_simulator(config, method=method, rng=rng, device=device)
    return sim.form_image(inputs, start_time, exposure_time, full_output=full_output, draws=draws)


def generate_images(inputs, num_frames, start_time=0.0, exposure_time=None, *, method=None,
                    config=None, rng=None, full_output=False, device=None, draws=None):
    """Generate images frame by frame (reference base.py:260-294)."""
    sim = create_simulator(config, method=method, rng=rng, device=device)
    return sim.generate_images(inputs, num_frames, start_time, exposure_time,
                               full_output=full_output, draws=draws)
