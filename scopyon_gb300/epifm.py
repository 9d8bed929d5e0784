"""Image-formation engine: configuration, PSF tables and the frame pipeline.

Host code mirrors the reference's ``EPIFMConfigs`` / ``_EPIFMSimulator``
(src/scopyon/_epifm.py:757-1225) for everything that is set-up or
bookkeeping (frame windows, molecule ids, random draws taken from the caller's
``rng``); every per-particle, per-pixel operation runs in the CUDA library.
Device buffers are torch CUDA tensors, reused across frames.
"""

import contextlib
import ctypes
import math
import os
import warnings

import numpy
import torch

from . import _catalog, _lib
from ._lib import call, ptr, stream_ptr
from .physics import absorption_terms, snells_law

__all__ = ["EngineConfig", "PSFTables", "FramePipeline", "InjectedDraws", "frame_windows"]

PSF_RES = 1e-9  # radial and depth resolution of the PSF tables (_epifm.py:61-62)


def _gpu_opt(tree, key, default=None):
    gpu = tree.get("gpu") if isinstance(tree, dict) else None
    if not isinstance(gpu, dict):
        return default
    v = gpu.get(key, default)
    return default if v is None else v


class EngineConfig:
    """Numbers of one method sub-tree (what ``EPIFMConfigs.initialize`` reads).

    ``conf`` is a ``Configuration`` of the method sub-tree; ``rng`` is used only
    for fixed-pattern-noise offsets, drawn exactly as the reference does
    (``_epifm.py:926-963``).
    """

    def __init__(self, conf, rng=None):
        if str(conf.type).lower() != "epifm":
            raise ValueError("An invalid type [%s] was given. 'epifm' is required." % conf.type)
        raw = conf.yaml
        fl = conf.fluorophore
        self.fluorophore_type = fl.type
        self.radius = fl.radius
        self.psf_normalization = fl.normalization
        self.radial_width = fl.radial_width if "radial_width" in fl else None
        self.radial_cutoff = fl.radial_cutoff
        self.depth_cutoff = fl.depth_cutoff
        min_wl, max_wl = fl.min_wave_length, fl.max_wave_length
        fl_wl = fl.wave_length if "wave_length" in fl else None
        self.psf_wavelength, fl_norm_sum = _catalog.psf_wavelength_and_norm(
            self.fluorophore_type, min_wl, max_wl, fl_wl,
            catalog_dir=_gpu_opt(raw, "catalog_dir"), override=_gpu_opt(raw, "psf_wavelength"))
        if self.fluorophore_type == "Gaussian" and self.radial_width is None:
            raise ValueError("fluorophore.radial_width must be given for Gaussian type fluorophore.")
        self.na = float(_gpu_opt(raw, "NA", 1.4))

        src = conf.light_source
        self.source_wavelength = src.wave_length
        self.flux_density = src.flux_density
        self.angle = src.angle
        self.amplitude0, self.penetration = snells_law(self.flux_density, self.source_wavelength,
                                                       self.angle)
        self.magnification = conf.magnification

        det = conf.detector
        self.detector_type = det.type
        if self.detector_type not in ("EMCCD", "CCD", "CMOS"):
            raise RuntimeError("Unknown detector type was given [%s]. Use either one of 'CMOS', "
                               "'CCD' or 'EMCCD'." % self.detector_type)
        self.image_size = tuple(int(v) for v in det.image_size)
        self.pixel_length = det.pixel_length
        self.exposure_time = det.exposure_time
        self.focal_point = numpy.asarray(det.focal_point, dtype=float)
        self.qe = det.QE
        self.readout_noise = det.readout_noise
        self.emgain = det.emgain

        adc = conf.analog_to_digital_converter
        self.bit = int(adc.bit)
        self.fullwell = adc.fullwell
        self._validate()
        self.fpn_type, self.fpn_count = adc.type, adc.count
        self.offset, self.gain = self._adc_maps(adc.offset, rng)

        eff = conf.effects
        self.background_switch = bool(eff.background.switch)
        self.background_mean = eff.background.mean
        self.qy = eff.fluorescence.quantum_yield
        self.abs_coeff = eff.fluorescence.abs_coefficient
        pb = eff.photo_bleaching
        self.bleaching = bool(pb.switch)
        self.half_life = pb.half_life
        self.x_sec, self.beer = absorption_terms(self.abs_coeff, self.radius)
        # photons per second at the unattenuated amplitude: the budget unit
        self.n_emit0 = self.qy * (self.amplitude0 * self.x_sec * 1.0) * self.beer

        sh = conf.shutter if "shutter" in conf else None
        self.shutter_switch = bool(sh.switch) if sh is not None else False
        self.shutter_start = sh.start_time if sh is not None else None
        self.shutter_end = sh.end_time if sh is not None else None

        norm = fl_norm_sum
        for name in ("dichroic_mirror", "emission_filter"):
            if name in conf and conf[name].switch:
                warnings.warn("%s is on: the spectral efficiency is applied once per configuration "
                              "(the reference compounds it per particle)" % name)
                norm = self._filtered_norm(conf, name, min_wl, max_wl)
        self.norm_coeff = norm * self.psf_normalization

        self.cmos_noise = str(_gpu_opt(raw, "cmos_noise", "table"))
        self.scmos_median = float(_gpu_opt(raw, "scmos_readout_median", 1.5))
        self.scmos_sigma = float(_gpu_opt(raw, "scmos_readout_sigma", 0.4))
        self.adc_rounding = str(_gpu_opt(raw, "adc_rounding", "none")) == "round"
        self.boundary = str(_gpu_opt(raw, "boundary", "none"))
        self.tile = int(_gpu_opt(raw, "tile", 0))
        self.l2_fetch_bytes = int(_gpu_opt(raw, "l2_fetch_bytes", 32))
        if self.l2_fetch_bytes not in (0, 32, 64, 128):
            raise ValueError("gpu.l2_fetch_bytes must be 0, 32, 64 or 128 (got %r)"
                             % self.l2_fetch_bytes)
        nvtx = _gpu_opt(raw, "nvtx", False)
        self.nvtx = (nvtx if isinstance(nvtx, bool) else str(nvtx).lower() in ("1", "true", "yes")) \
            or os.environ.get("SCOPYON_GB300_NVTX", "") not in ("", "0")
        self.use_box = bool(_gpu_opt(raw, "box_tables", True))
        self.catalog_dir = _gpu_opt(raw, "catalog_dir")
        table = _gpu_opt(raw, "cmos_table")
        self.cmos_table = None if table is None else numpy.asarray(table, dtype=float)

    def _validate(self):
        """Reject a corrupt detector or ADC section before anything reaches the
        device (the reference fails later, inside numpy, on the same values)."""
        def finite_pos(name, v):
            try:
                ok = math.isfinite(float(v)) and float(v) > 0
            except (TypeError, ValueError):
                ok = False
            if not ok:
                raise ValueError("%s must be a finite positive number (got %r)" % (name, v))
        if len(self.image_size) != 2 or not all(0 < v < 32767 for v in self.image_size):
            raise ValueError("detector.image_size must be two sizes in 1..32766 (got %r)"
                             % (self.image_size,))
        finite_pos("detector.pixel_length", self.pixel_length)
        finite_pos("magnification", self.magnification)
        finite_pos("detector.exposure_time", self.exposure_time)
        finite_pos("analog_to_digital_converter.fullwell", self.fullwell)
        if not 1 <= self.bit <= 32:
            raise ValueError("analog_to_digital_converter.bit must be in 1..32 (got %r)"
                             % self.bit)
        try:
            qe = float(self.qe)
        except (TypeError, ValueError):
            qe = float("nan")
        if not 0.0 <= qe <= 1.0:
            raise ValueError("detector.QE must be in [0, 1] (got %r)" % (self.qe,))

    @property
    def px(self):
        return self.pixel_length / self.magnification

    def _adc_maps(self, offset0, rng):
        nw, nh = self.image_size
        if self.fpn_type == "none":
            offset = numpy.full(nw * nh, offset0)
        elif self.fpn_type == "pixel":
            if rng is None:
                raise RuntimeError("A random number generator is required.")
            offset = numpy.rint(rng.normal(offset0, self.fpn_count, nw * nh))
        elif self.fpn_type == "column":
            if rng is None:
                raise RuntimeError("A random number generator is required.")
            column = rng.normal(offset0, self.fpn_count, nh)
            offset = numpy.rint(numpy.tile(column, (1, nw)).reshape(nh * nw))
        else:
            raise ValueError("FPN type [%s] is invalid ['pixel', 'column' or 'none']"
                             % self.fpn_type)
        gain = (self.fullwell - 0.0) / (pow(2.0, self.bit) - offset)
        return (numpy.asarray(offset, dtype=float).reshape(nw, nh),
                numpy.asarray(gain, dtype=float).reshape(nw, nh))

    def _filtered_norm(self, conf, name, min_wl, max_wl):
        cdir = _catalog.find_catalog_dir(self.catalog_dir)
        if cdir is None:
            raise FileNotFoundError("%s needs the scopyon catalog (gpu.catalog_dir)" % name)
        grid = numpy.arange(min_wl, max_wl, 1e-9, dtype=float)
        sections = _catalog.read_catalog(
            "%s/fluorophore/%s.csv" % (cdir, self.fluorophore_type))
        em = _catalog._efficiency(sections["Emission"], grid)
        em[int(em.argmax())] = 100
        em /= sum(em)
        sub = {"dichroic_mirror": "dichroic", "emission_filter": "emission"}[name]
        spec = _catalog.read_catalog("%s/%s/%s.csv" % (cdir, sub, conf[name].type))["wavedataset"]
        return float(numpy.sum(em * 0.01 * _catalog._efficiency(spec, grid)))

    # -- PSF geometry ----------------------------------------------------
    @property
    def n_r(self):
        return len(numpy.arange(0.0, self.radial_cutoff, PSF_RES, dtype=float))

    @property
    def box_p(self):
        """Grid rows per pixel when px / 1 nm is an integer P (box tables apply), else 0.

        The box path needs bound k = ceil(a) + P k for every bound of a
        footprint; with |px/res - P| * (bounds per footprint) below 1e-10 the
        drift stays far inside the 1e-9 margin the records test for.
        """
        if not self.use_box:
            return 0
        b = self.px / PSF_RES
        p = int(round(b))
        n_signal = 2 * self.n_r - 1
        if p < 1 or abs(b - p) * (n_signal / p + 3) >= 1e-10:
            return 0
        return p

    @property
    def max_key(self):
        return int((self.depth_cutoff + PSF_RES) / PSF_RES) + 1

    def depth_keys(self, depths):
        """Depth keys of ``PointSpreadingFunction.get`` (_epifm.py:76-88), vectorised."""
        d = numpy.abs(numpy.asarray(depths, dtype=float))
        inside = d < self.depth_cutoff + PSF_RES
        keys = numpy.full(d.shape, -1, dtype=numpy.int64)
        keys[inside] = (d[inside] / PSF_RES).astype(numpy.int64)
        return keys


class PSFTables:
    """Device cache of quadrant summed-area tables, one per 1-nm depth key."""

    def __init__(self, cfg, device):
        self.cfg = cfg
        self.device = device
        self.n_r = cfg.n_r
        self.pitch = ((self.n_r + 1 + 3) // 4) * 4
        self.table_floats = (self.n_r + 1) * self.pitch * 2
        self.max_key = cfg.max_key
        self.slot_of = {}
        self.key_slot_host = numpy.full(self.max_key + 2, -1, dtype=numpy.int32)
        self.key_slot = torch.full((self.max_key + 2,), -1, dtype=torch.int32, device=device)
        self.tables = torch.empty(0, dtype=torch.float32, device=device)
        self.capacity = 0
        self.box_p = cfg.box_p
        n_signal = 2 * self.n_r - 1
        self.box_nq = (n_signal + self.box_p - 1) // self.box_p + 1 if self.box_p else 0
        # floats from one phase block's start to the next, as the library was built
        self.box_block = _lib.load().sc_box_block_floats(self.box_nq) if self.box_p else 0
        self.box_floats = self.box_p ** 2 * self.box_block
        self.box = torch.empty(0, dtype=torch.float32, device=device) if self.box_p else None
        self._covered = None  # a depth range whose keys are all built

    def _depth_of_key(self, key):
        return self.cfg.depth_cutoff if key < 0 else key * PSF_RES

    def _grow(self, need):
        if need <= self.capacity:
            return
        cap = max(need, min(2 * self.capacity, self.max_key + 2), 1)
        new = torch.empty(cap * self.table_floats, dtype=torch.float32, device=self.device)
        if self.capacity:
            new[: self.capacity * self.table_floats].copy_(self.tables)
        if self.box_p:
            nbox = torch.empty(cap * self.box_floats, dtype=torch.float32, device=self.device)
            if self.capacity:
                nbox[: self.capacity * self.box_floats].copy_(self.box)
            self.box = nbox
        self.tables, self.capacity = new, cap

    def ensure(self, keys, stream=None):
        """Build the tables of any keys not cached yet."""
        keys = numpy.unique(numpy.asarray(keys, dtype=numpy.int64))
        missing = [int(k) for k in keys if int(k) not in self.slot_of]
        if not missing:
            return
        if any(k > self.max_key for k in missing):
            raise ValueError("depth key beyond the table range")
        self._grow(len(self.slot_of) + len(missing))
        kind = _lib.PSF_GAUSSIAN if self.cfg.fluorophore_type == "Gaussian" else _lib.PSF_BORN_WOLF
        sigma = float(self.cfg.radial_width or 0.0)
        batch = 64
        s = stream_ptr(stream)
        for b0 in range(0, len(missing), batch):
            chunk = missing[b0: b0 + batch]
            depths = torch.tensor([self._depth_of_key(k) for k in chunk], dtype=torch.float64,
                                  device=self.device)
            radial = torch.empty((len(chunk), self.n_r), dtype=torch.float64, device=self.device)
            call("sc_psf_radial", kind, float(self.cfg.psf_wavelength), self.cfg.na, sigma,
                 ptr(depths), len(chunk), self.n_r, PSF_RES, ptr(radial), s)
            first = len(self.slot_of)
            out = self.tables[first * self.table_floats: (first + len(chunk)) * self.table_floats]
            call("sc_psf_quadrant_sat", ptr(radial), len(chunk), self.n_r, PSF_RES, ptr(out),
                 self.pitch, s)
            if self.box_p:
                bout = self.box[first * self.box_floats: (first + len(chunk)) * self.box_floats]
                call("sc_psf_box_table", ptr(out), len(chunk), self.n_r, self.pitch, self.box_p,
                     ptr(bout), s)
            for j, k in enumerate(chunk):
                self.slot_of[k] = first + j
                self.key_slot_host[k if k >= 0 else self.max_key + 1] = first + j
        self.key_slot.copy_(torch.from_numpy(self.key_slot_host))

    def ensure_depth_range(self, dmin, dmax, stream=None):
        """Build every key a depth in [dmin, dmax] (relative to the focal
        plane) can map to.  Keys grow with |depth| up to the cutoff, so the
        keys of the two extreme |depths| bound them all: a contiguous range,
        checked against the built set without sorting the per-emitter keys."""
        cov = self._covered
        if cov is not None and cov[0] <= dmin and dmax <= cov[1]:
            return  # within a range already checked (keys are never dropped)
        if not (math.isfinite(dmin) and math.isfinite(dmax)):
            raise ValueError("non-finite emitter depth")
        lo = 0.0 if dmin <= 0.0 <= dmax else min(abs(dmin), abs(dmax))
        hi = max(abs(dmin), abs(dmax))
        k_lo, k_hi = (int(k) for k in self.cfg.depth_keys([lo, hi]))
        if k_lo < 0:  # every depth is past the cutoff
            wanted = [-1]
        else:
            top = self.max_key if k_hi < 0 else k_hi
            wanted = list(range(k_lo, top + 1)) + ([-1] if k_hi < 0 else [])
        have = self.key_slot_host
        if not (all(have[k if k >= 0 else self.max_key + 1] >= 0 for k in (wanted[0], wanted[-1]))
                and (have[k_lo: (self.max_key if k_hi < 0 else k_hi) + 1] >= 0).all()):
            self.ensure(wanted, stream)
        self._covered = (dmin, dmax)

    def ensure_all(self, stream=None):
        self.ensure(list(range(0, self.max_key + 1)) + [-1], stream)


class InjectedDraws:
    """Random draws supplied by the caller instead of the engine's Philox streams.

    ``bleach``: {m_id: bleaching time in seconds}, used at a molecule's first
    sight in place of ``rng.exponential``.  ``frames``: one dict per frame with
    ``noise`` (electrons, W x H) and ``signal`` (electrons, W x H), or for the
    EMCCD exact draw ``uniform`` (W x H) instead of ``signal``, or for the
    CMOS table ``uniform`` (noise index draw) and ``signal``.  This is the mode
    in which the engine reproduces the reference's output for recorded draws.
    """

    def __init__(self, bleach=None, frames=None):
        self.bleach = dict(bleach or {})
        self.frames = list(frames or [])
        self.index = 0

    def next_frame(self):
        d = self.frames[self.index]
        self.index += 1
        return d


def frame_windows(times, num, start_time, exposure_time, frame_index, shutter=None):
    """Sub-step slices and unit times of one frame (_epifm.py:1146-1193)."""
    t = start_time + exposure_time * frame_index
    if shutter is not None:
        t = max(t, shutter[0])
        exposure_time = max(0.0, min(t + exposure_time, shutter[1]))
    start = numpy.searchsorted(times, t, side="right")
    if start != 0:
        start -= 1
    stop = numpy.searchsorted(times, t + exposure_time, side="left")
    if len(times) and times[start] > t:
        warnings.warn("No data input for interval [{}, {}]".format(t, times[start]))
    idx = list(range(start, stop))
    out = []
    for k, i in enumerate(idx):
        current = times[i] if k != 0 else t
        nxt = times[idx[k + 1]] if k + 1 < len(idx) else t + exposure_time
        unit_time = nxt - current
        if unit_time < 1e-13:
            continue
        out.append((i, unit_time))
    return out, exposure_time


class FramePipeline:
    """Device buffers and kernel sequence for frames of one configuration."""

    def __init__(self, cfg, device=None, psf=None):
        self.cfg = cfg
        self.device = torch.device(device or "cuda")
        _lib.load()
        if cfg.l2_fetch_bytes:
            # the splat reads random 784-byte blocks and 32-byte record heads:
            # smaller L2 fetches read fewer bytes it does not use
            with torch.cuda.device(self.device):
                call("sc_set_l2_fetch_granularity", cfg.l2_fetch_bytes)
        self.psf = psf or PSFTables(cfg, self.device)
        nw, nh = cfg.image_size
        self.nw, self.nh = nw, nh
        self.n_pix = nw * nh
        dev = self.device
        self.status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
        self.image = torch.empty(self.n_pix, dtype=torch.float32, device=dev)
        self.expect = torch.empty(self.n_pix, dtype=torch.float32, device=dev)
        self.adc = torch.empty(self.n_pix, dtype=torch.float64, device=dev)  # injected draws
        self.adc32 = torch.empty(self.n_pix, dtype=torch.float32, device=dev)  # native draws
        self.poisson = _lib.poisson_table(dev)
        self.offset = torch.from_numpy(numpy.ascontiguousarray(cfg.offset, dtype=float)).to(dev).reshape(-1)
        self.gain = torch.from_numpy(numpy.ascontiguousarray(cfg.gain, dtype=float)).to(dev).reshape(-1)
        self.offset_f = self.offset.float()
        self.inv_gain_f = (1.0 / self.gain).float()
        # without fixed-pattern noise every pixel has the same offset and gain:
        # the camera takes them from its parameters instead of reading two maps
        self.pixel_maps = cfg.fpn_type != "none"
        self.sigma = None
        self.table_value = self.table_cdf = None
        n_signal = 2 * self.psf.n_r - 1
        # pixels a footprint reaches past its first one
        self.halo = int(math.ceil(PSF_RES * (n_signal - 1) / cfg.px)) + 1
        self.tile, self.warps = self._pick_tile()
        self.stages = 4
        if cfg.tile:
            self.tile = cfg.tile
        self.tiles_x = (nw + self.tile - 1) // self.tile
        self.tiles_y = (nh + self.tile - 1) // self.tile
        self._cap = {}
        self.budget = torch.zeros(0, dtype=torch.float64, device=dev)
        self.camera_kind = self._camera_kind()
        # name -> [(start, end) CUDA events]; set to a dict to time kernels in place
        self.kernel_events = None
        # native frames merge the splat's tile buffers inside the camera pass
        self.merge_camera = True
        # test hook: polls of each splat warp's first block wait (0: the normal
        # bound; -1: none, so that the wait runs out and the frame reports it)
        self.first_wait_polls = 0

    def graph_signature(self):
        """Every device address and launch shape a captured frame graph of
        this pipeline depends on: its own buffers, the PSF tables' and the
        tile shape.  A graph is replayed only while this is unchanged."""
        psf = self.psf
        ts = (self.status, self.image, self.expect, self.adc, self.adc32, self.budget,
              self.offset_f, self.inv_gain_f, self.sigma, self.table_value, self.table_cdf,
              psf.key_slot, psf.tables, psf.box, self.poisson)
        return (tuple(0 if t is None else t.data_ptr() for t in ts) +
                tuple(v.data_ptr() for v in self._cap.values() if isinstance(v, torch.Tensor)) +
                (psf.capacity, self.tile, self.warps, self.stages, self.merge_camera,
                 self.pixel_maps, self.first_wait_polls))

    def set_tiles(self, tile, warps, stages=4):
        """Use tiles of tile x tile pixels, `warps` warps per splat CTA and
        `stages` box-table block copies in flight per warp (0: the register
        kernel, which loads each block with 16-byte loads instead)."""
        if tile not in (8, 16, 32) or warps not in (1, 2, 4, 8) or not 0 <= stages <= 8:
            raise ValueError("tile must be 8, 16 or 32, warps 1, 2, 4 or 8, stages 0..8")
        nw, nh = self.nw, self.nh
        self.tile, self.warps, self.stages = int(tile), int(warps), int(stages)
        self.tiles_x = (nw + self.tile - 1) // self.tile
        self.tiles_y = (nh + self.tile - 1) // self.tile

    def _pick_tile(self):
        """(tile edge, warps per tile CTA) that fit shared memory; see tune_tiles."""
        for tile, warps in ((8, 4), (8, 2), (8, 1)):
            edge = tile + self.halo
            stride = ((edge * edge + 31) // 32) * 32 + 16
            if 2 * warps * stride * 4 + warps * 2 * (edge + 2) * 4 <= 200 * 1024:
                return tile, warps
        raise ValueError("pixel size %g m is too small for the splat's shared memory" % self.cfg.px)

    def _camera_kind(self):
        t = self.cfg.detector_type
        if t == "EMCCD":
            return _lib.CAM_EMCCD
        if t == "CCD":
            return _lib.CAM_CCD
        if self.cfg.cmos_noise == "scmos":
            return _lib.CAM_SCMOS
        return _lib.CAM_CMOS_TABLE

    def scmos_sigma_map(self, rng):
        """Per-pixel readout sigma ~ lognormal(log(median), sigma) (sCMOS mode)."""
        sig = rng.lognormal(math.log(self.cfg.scmos_median), self.cfg.scmos_sigma,
                            size=self.n_pix)
        self.sigma = torch.from_numpy(sig.astype(numpy.float32)).to(self.device)

    def load_cmos_table(self, table=None):
        if table is None:
            table = _catalog.cmos_noise_table(self.cfg.catalog_dir)
        table = numpy.asarray(table, dtype=float)
        prob = table[:, 1] / table[:, 1].sum()
        cdf = prob.cumsum()
        cdf /= cdf[-1]
        self.table_value = torch.from_numpy(numpy.ascontiguousarray(table[:, 0])).to(self.device)
        self.table_cdf = torch.from_numpy(cdf).to(self.device)

    # -- scratch buffers sized on demand, reused across frames -------------
    def _buf(self, name, numel, dtype):
        t = self._cap.get(name)
        if t is None or t.numel() < numel or t.dtype != dtype:
            t = torch.empty(max(numel, 1), dtype=dtype, device=self.device)
            self._cap[name] = t
        return t

    def host_staging(self, shape, slot=0):
        """A pinned host array of ``shape`` (float64) for an upload; two slots
        let one frame's inputs be staged while the other's are uploaded."""
        numel = int(numpy.prod(shape))
        name = "staging%d" % slot
        t = self._cap.get(name)
        if t is not None:
            ev = self._cap.get("upload_events", {}).get(t.data_ptr())
            if ev is not None:
                ev.synchronize()  # the previous upload from this buffer has finished
        if t is None or t.numel() < numel:
            t = torch.empty(max(numel, 1), dtype=torch.float64, pin_memory=True)
            self._cap[name] = t
        return t[:numel].numpy().reshape(shape)

    def _upload_small(self, values, ring=8):
        """A small float64 host array to a new device tensor through a ring of
        pinned buffers: each slot is refilled only after its previous upload
        has completed (the slot's event, recorded again at each use)."""
        n = values.size
        r = self._cap.get("small_ring")
        if r is None or r[0].shape[1] < n:
            host = torch.empty((ring, max(64, n)), dtype=torch.float64, pin_memory=True)
            r = (host.numpy(), host, [None] * ring, [0])
            self._cap["small_ring"] = r
        views, host, events, nxt = r
        k = nxt[0]
        nxt[0] = (k + 1) % len(events)
        ev = events[k]
        if ev is None:
            ev = events[k] = torch.cuda.Event()
        else:
            ev.synchronize()
        views[k, :n] = values
        out = torch.empty(n, dtype=torch.float64, device=self.device)
        call("sc_copy_async", ptr(out), ctypes.c_void_p(views[k].ctypes.data), n * 8,
             stream_ptr())
        ev.record()
        return out

    def ensure_slots(self, n_slots, initial=None):
        if self.budget.numel() < n_slots:
            grown = torch.zeros(n_slots, dtype=torch.float64, device=self.device)
            if self.budget.numel():
                grown[: self.budget.numel()].copy_(self.budget)
            self.budget = grown

    def step_params(self, n_sub, n_particles, with_optinfo):
        cfg = self.cfg
        p = _lib.StepParams()
        p.px, p.res, p.depth_cutoff = cfg.px, PSF_RES, cfg.depth_cutoff
        for k in range(3):
            p.focal[k] = float(cfg.focal_point[k])
        p.nw, p.nh = self.nw, self.nh
        p.n_signal = 2 * self.psf.n_r - 1
        p.n_sub, p.n_particles = n_sub, n_particles
        p.max_key = self.psf.max_key
        p.amplitude0, p.penetration = float(cfg.amplitude0), float(cfg.penetration)
        p.x_sec, p.qy, p.beer = float(cfg.x_sec), float(cfg.qy), float(cfg.beer)
        p.norm_coeff = float(cfg.norm_coeff)
        p.bleaching = 1 if cfg.bleaching else 0
        p.with_optinfo = 1 if with_optinfo else 0
        p.box_p, p.box_nq = self.psf.box_p, self.psf.box_nq
        return p

    def splat_params(self, n_images=1, rec_per_image=0):
        p = _lib.SplatParams()
        p.nw, p.nh, p.tile = self.nw, self.nh, self.tile
        p.halo, p.warps = self.halo, self.warps
        p.tiles_x, p.tiles_y = self.tiles_x, self.tiles_y
        p.n_r, p.sat_pitch = self.psf.n_r, self.psf.pitch
        p.n_images, p.rec_per_image = n_images, rec_per_image
        p.box_p, p.box_nq = self.psf.box_p, self.psf.box_nq
        p.n_slots = self.psf.capacity
        # stages 0: the register box kernel (the persistent batched frame,
        # which has no register form, then keeps 4 copies in flight)
        p.box_stages = self.stages if self.stages > 0 else 4
        p.box_kernel = 1 if self.stages == 0 else 0
        p.first_wait_polls = int(self.first_wait_polls)
        p.px, p.res = self.cfg.px, PSF_RES
        return p

    def bin_buffers(self, n_rec, n_images=1, rec_per_image=0, tag=""):
        """Splat parameters and the binning workspace, items and bin offsets
        (``tag`` names a second set, for a frame binned while another splats)."""
        sp = self.splat_params(n_images, rec_per_image)
        n_tiles = self.tiles_x * self.tiles_y * n_images
        ws_bytes = _lib.load().sc_bin_workspace_bytes(n_rec, n_tiles)
        ws = self._buf("ws" + tag, (ws_bytes + 3) // 4, torch.int32)
        items = self._buf("items" + tag, n_rec, torch.int32)
        tile_start = self._buf("tile_start" + tag, 2 * n_tiles + 1, torch.int32)
        return sp, ws, ws_bytes, items, tile_start

    def splat_records(self, recs, n_rec, image, n_images=1, rec_per_image=0, stream=None,
                      counted=False, tag="", binned=False, bufs=None):
        """Bin records by tile and splat them into ``image`` (n_images x W x H, float32).

        counted: the records' producer already counted them into the binning
        workspace (sc_native_records), so only sc_bin_finish runs here;
        binned: the bins are complete too (``finish_bins``), only the splat runs.
        bufs: the ``bin_buffers`` tuple when the caller has it."""
        s = stream_ptr(stream)
        sp, ws, ws_bytes, items, tile_start = bufs or self.bin_buffers(n_rec, n_images,
                                                                       rec_per_image, tag)
        if binned:
            pass
        elif counted:
            with self.timed("bins", stream):
                call("sc_bin_finish", n_rec, sp, ptr(ws), ws_bytes, ptr(tile_start), ptr(items), s)
        else:
            with self.timed("bins", stream):
                call("sc_bin_steps", ptr(recs), n_rec, sp, ptr(ws), ws_bytes, ptr(tile_start),
                     ptr(items), ptr(self.status), s)
        L = _lib.load()
        sws_bytes = L.sc_splat_workspace_bytes(sp)
        sws = self._buf("splat_ws", (sws_bytes + 3) // 4, torch.float32)
        with self.timed("splat", stream):
            call("sc_splat", ptr(recs), ptr(tile_start), ptr(items), ptr(self.psf.tables),
                 ptr(self.psf.box), sp, ptr(sws), sws_bytes, ptr(image), ptr(self.status), s)
        return sp, sws, sws_bytes

    def splat_camera(self, recs, n_rec, seed=0, counter=0, d_frame=None, stream=None, tag="",
                     binned=False, bufs=None, out=None):
        """A native frame's splat and camera into self.expect / self.adc32 (or
        the (expect, adc32) pair ``out``): the splat without its merge, then
        the merge and the camera in one pass (sc_merge_camera), equal bit for
        bit to splat_records into self.image followed by camera().  With
        merge_camera off, those two."""
        expect, adc32 = out if out is not None else (self.expect, self.adc32)
        if not self.merge_camera:
            self.splat_records(recs, n_rec, self.image, stream=stream, tag=tag, binned=binned,
                               bufs=bufs)
            self.camera(self.image, expect, None, adc32, seed=seed, counter=counter,
                        stream=stream, d_frame=d_frame)
            return
        sp, sws, sws_bytes = self.splat_records(recs, n_rec, None, stream=stream, tag=tag,
                                                binned=binned, bufs=bufs)
        cp = self.camera_params(seed, counter, d_frame)
        maps = self.pixel_maps
        with self.timed("camera", stream):
            call("sc_merge_camera", sp, ptr(sws), sws_bytes, cp,
                 ptr(self.offset_f) if maps else None, ptr(self.inv_gain_f) if maps else None,
                 ptr(self.sigma), ptr(self.table_value), ptr(self.table_cdf), ptr(expect),
                 ptr(adc32), ptr(self.status), stream_ptr(stream))

    def finish_bins(self, n_rec, tag="", stream=None, bufs=None):
        """Scan, placement and order of records already counted into the bin
        buffers named by ``tag`` (sc_bin_finish)."""
        sp, ws, ws_bytes, items, tile_start = bufs or self.bin_buffers(n_rec, tag=tag)
        with self.timed("bins", stream):
            call("sc_bin_finish", n_rec, sp, ptr(ws), ws_bytes, ptr(tile_start), ptr(items),
                 stream_ptr(stream))

    @contextlib.contextmanager
    def timed(self, name, stream=None):
        """CUDA events around the enclosed launches when kernel_events is a
        dict (appended under `name`), and an NVTX range ``scopyon/<name>``
        around them when the configuration turns NVTX ranges on (``gpu.nvtx``
        or ``SCOPYON_GB300_NVTX=1``); nothing otherwise."""
        nvtx = self.cfg.nvtx
        if nvtx:
            torch.cuda.nvtx.range_push("scopyon/" + name)
        try:
            ev = self.kernel_events
            if ev is None:
                yield
                return
            st = stream if stream is not None else torch.cuda.current_stream()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            yield
            e1.record(st)
            ev.setdefault(name, []).append((e0, e1))
        finally:
            if nvtx:
                torch.cuda.nvtx.range_pop()

    def camera_params(self, seed=0, counter=0, d_frame=None, exact=False):
        """The camera's parameter block (loads the CMOS noise table when needed)."""
        cfg = self.cfg
        if self.camera_kind == _lib.CAM_CMOS_TABLE and self.table_value is None:
            self.load_cmos_table(self.cfg.cmos_table)
        cp = _lib.CameraParams()
        cp.nw, cp.nh, cp.camera = self.nw, self.nh, self.camera_kind
        cp.exact = 1 if exact else 0
        cp.rounding = 1 if cfg.adc_rounding else 0
        cp.bit = cfg.bit
        cp.qe = float(cfg.qe)
        cp.background = float(cfg.background_mean) if cfg.background_switch else 0.0
        cp.readout_noise = float(cfg.readout_noise or 0.0)
        cp.emgain = float(cfg.emgain or 1.0)
        cp.fullwell = float(cfg.fullwell)
        cp.offset0, cp.gain0 = float(cfg.offset.flat[0]), float(cfg.gain.flat[0])
        cp.table_n = 0 if self.table_value is None else self.table_value.numel()
        cp.seed, cp.counter = int(seed) & (2 ** 64 - 1), int(counter) & (2 ** 64 - 1)
        cp.d_frame = None if d_frame is None else d_frame.data_ptr()
        cp.d_poisson_table = self.poisson.data_ptr()
        return cp

    def camera(self, photons, expect, adc64, adc32=None, seed=0, counter=0, draws=None,
               stream=None, d_frame=None, photons64=None, expect64=None):
        """Camera model + ADC on one frame (photons: float32 W*H on the device;
        with injected draws, photons64 / expect64 are the FP64 photons read and
        the FP64 expectation written in their place)."""
        cfg = self.cfg
        s = stream_ptr(stream)
        cp = self.camera_params(seed, counter, d_frame, exact=draws is not None)
        if draws is not None:
            cp.d_photons64 = None if photons64 is None else photons64.data_ptr()
            cp.d_expect64 = None if expect64 is None else expect64.data_ptr()
        inj_noise = inj_signal = inj_uniform = None
        if draws is not None:
            dev = self.device

            def dev64(a):
                return torch.from_numpy(numpy.ascontiguousarray(a, dtype=float).reshape(-1)).to(dev)

            inj_noise = dev64(draws["noise"]) if "noise" in draws else None
            if "signal" in draws:
                inj_signal = dev64(draws["signal"])
            if "uniform" in draws:
                inj_uniform = dev64(numpy.nan_to_num(numpy.asarray(draws["uniform"], float)))
            if inj_signal is None and self.camera_kind == _lib.CAM_EMCCD:
                inj_signal = self._buf("emccd_sig", self.n_pix, torch.float64)
                if photons64 is None:
                    photons64 = photons.double()
                call("sc_emccd_exact", ptr(photons64), float(cfg.qe), cp.background,
                     ptr(inj_uniform), self.n_pix, float(cfg.emgain), ptr(inj_signal),
                     ptr(self.status), s)
                inj_uniform = None
        with self.timed("camera", stream):
            maps = self.pixel_maps
            call("sc_camera", cp, ptr(photons), ptr(self.offset) if maps else None,
                 ptr(self.gain) if maps else None, ptr(self.offset_f) if maps else None,
                 ptr(self.inv_gain_f) if maps else None, ptr(self.sigma), ptr(self.table_value),
                 ptr(self.table_cdf), ptr(inj_noise), ptr(inj_signal), ptr(inj_uniform),
                 ptr(expect), ptr(adc64), ptr(adc32), ptr(self.status), s)

    def check_status(self):
        self.raise_for_status(self.status.cpu().numpy())

    def frame_out(self, adc, slot=0):
        """Enqueues on the current stream the device-to-host copies of a
        frame's ADC counts and of the status words into pinned buffers (two
        slots, so that one frame's are read while the next frame's are
        copied); returns (event, counts, status) with the host arrays valid
        once the event has completed."""
        name = "frame_out%d" % slot
        h = self._cap.get(name)
        if h is None or h[0].numel() < adc.numel() or h[0].dtype != adc.dtype:
            counts = torch.empty(adc.numel(), dtype=adc.dtype, pin_memory=True)
            status = torch.empty(self.status.numel(), dtype=torch.int32, pin_memory=True)
            # the slot's event is recorded again at each use: the caller has
            # read the slot's previous frame before it asks for the slot again
            h = (counts, status, counts.numpy(), status.numpy(), torch.cuda.Event())
            self._cap[name] = h
        counts, status, counts_np, status_np, ev = h
        if not adc.is_contiguous():
            adc = adc.contiguous()
        s = stream_ptr()
        call("sc_copy_async", ctypes.c_void_p(counts.data_ptr()), ptr(adc),
             adc.numel() * adc.element_size(), s)
        call("sc_copy_async", ctypes.c_void_p(status.data_ptr()), ptr(self.status),
             status.numel() * 4, s)
        ev.record()
        return ev, counts_np[: adc.numel()], status_np

    def raise_for_status(self, st):
        """Raises the error the status words ``st`` (read from the device)
        record, after clearing them on the device; nothing when clear."""
        if st[0]:
            self.status.zero_()
            bits = int(st[0])
            msgs = []
            if bits & 1:
                msgs.append("depth key beyond table range (particle %d, sub-step %d)" % (st[1], st[2]))
            if bits & 2:
                msgs.append("PSF table missing for key %d" % st[3])
            if bits & 4:
                msgs.append("footprint outside its tile buffer or EMCCD support empty "
                            "(%d, %d, %d)" % (st[1], st[2], st[3]))
            if bits & 8:
                msgs.append("random-variate loop bound reached")
            if bits & 16:
                msgs.append("bin capacity exceeded (%d entries)" % st[1])
            if bits & 32:
                msgs.append("bounded wait for an asynchronous copy ran out (tile %d)" % st[3])
            if bits & 64:
                msgs.append("record %d has a negative first pixel (%d, %d)" % (st[1], st[2], st[3]))
            if bits & 128:
                msgs.append("non-finite emitter position or normalisation (particle %d, "
                            "sub-step %d)" % (st[1], st[2]))
            if bits & 256:
                msgs.append("index %d out of range %d at check site %d (bounds-checked build)"
                            % (st[1], st[2], st[3]))
            if bits & ~(64 | 128) == 0:
                raise _lib.ScopyonInputError(
                    _lib.SC_ERR_NAN if bits & 128 else _lib.SC_ERR_ARG, "; ".join(msgs))
            code = _lib.SC_ERR_TIMEOUT if bits == 32 else _lib.SC_ERR_CAPACITY
            raise _lib.ScopyonGPUError(code, "; ".join(msgs))

    def run_frame(self, particles, unit_times, with_optinfo=True, draws=None, seed=0, counter=0,
                  present=None, bleaching=None, stream=None, track_upload=True):
        """One frame from host arrays.

        particles: (S, N, 5) float64 [depth, x, y, m_id, p_state] per sub-step,
        column n holding particle slot n; unit_times: (S,) float64.
        Returns device tensors (expect f32, adc f64, optinfo f64 (N, 8) or None).
        Pinned particles are uploaded asynchronously; with track_upload the
        upload's event is kept for ``host_staging`` (a staging buffer that
        will be refilled), without it the caller keeps the array unchanged.
        """
        n_sub, n = particles.shape[0], particles.shape[1]
        dev = self.device
        part = self._buf("particles", n_sub * n * 5, torch.float64)[: n_sub * n * 5]
        host = numpy.ascontiguousarray(particles, dtype=float)
        # one copy on the current stream (from pageable memory it returns once
        # the source has been read)
        call("sc_copy_async", ptr(part), ctypes.c_void_p(host.ctypes.data), host.nbytes,
             stream_ptr(stream))
        if track_upload and host.size and torch.from_numpy(host.reshape(-1)).is_pinned():
            ev = torch.cuda.Event()
            ev.record()
            self._cap.setdefault("upload_events", {})[host.ctypes.data] = ev
        # from a pinned buffer (a pageable upload would wait for all the work
        # queued before it), one of a ring allocated once: pinning per frame
        # calls the driver's host allocator whenever the cached blocks are
        # still in flight, which is slow while the OS reclaims memory
        ut = self._upload_small(numpy.ascontiguousarray(unit_times, dtype=float).reshape(-1))
        pres = None
        if present is not None:
            pres = torch.from_numpy(numpy.ascontiguousarray(present, dtype=numpy.uint8).reshape(-1)).to(dev)
        return self.run_frame_device(part, ut, n_sub, n, with_optinfo, draws, seed, counter, pres,
                                     bleaching, stream)

    def run_frame_device(self, part, ut, n_sub, n, with_optinfo=True, draws=None, seed=0,
                         counter=0, present=None, bleaching=None, stream=None, d_frame=None,
                         row_layout=0):
        """One frame from device tensors: part (n_sub*n*5 f64 rows, or with
        row_layout 1 n_sub*n*4 f32 rows of sc_diffuse_steps), ut (n_sub f64)."""
        s = stream_ptr(stream)
        self.ensure_slots(n)
        n_rec = n_sub * n
        recs = self._buf("recs", max(n_rec, 1) * (_lib.STEP_REC_BYTES // 4), torch.int32)
        optinfo = self._buf("optinfo", n * 8, torch.float64) if with_optinfo else None
        # injected draws: the reference-parity mode, with the expected image
        # accumulated in FP64 (sc_splat_fp64) so that draws taken from it are
        # the reference's
        exact = draws is not None
        norm = self._buf("norm64", max(n_rec, 1), torch.float64) if exact else None
        if n_rec:
            sp = self.step_params(n_sub, n, with_optinfo)
            sp.row_layout = row_layout
            if bleaching is not None:
                sp.bleaching = 1 if bleaching else 0
            with self.timed("records_from_rows", stream):
                call("sc_emitter_steps", sp, ptr(part), ptr(ut), ptr(present),
                     ptr(self.psf.key_slot), ptr(self.budget), ptr(optinfo), ptr(recs), ptr(norm),
                     ptr(self.status), s)
        opt = optinfo[: n * 8].view(n, 8) if with_optinfo else None
        if exact:
            image64 = self._buf("image64", self.n_pix, torch.float64)[: self.n_pix]
            expect64 = self._buf("expect64", self.n_pix, torch.float64)[: self.n_pix]
            image64.zero_()
            if n_rec:
                call("sc_splat_fp64", ptr(recs), ptr(norm), n_rec, ptr(self.psf.tables),
                     self.splat_params(), ptr(image64), ptr(self.status), s)
            self.camera(None, None, self.adc, seed=seed, counter=counter, draws=draws,
                        stream=stream, d_frame=d_frame, photons64=image64, expect64=expect64)
            return expect64, self.adc, opt
        self.splat_camera(recs, n_rec, seed=seed, counter=counter, d_frame=d_frame,
                          stream=stream)
        return self.expect, self.adc32, opt


# (tile edge, warps per splat CTA, block copies in flight per warp; 0: the
# register kernel)
TILE_CANDIDATES = ((8, 4, 4), (8, 4, 8), (8, 2, 6), (16, 4, 4), (16, 8, 4), (16, 4, 8),
                   (8, 4, 0), (8, 8, 0), (16, 8, 0))


def tune_tiles(graph, candidates=TILE_CANDIDATES, frames=3):
    """Autotuner of the splat launch: for each (tile edge, warps per splat CTA,
    block copies in flight per warp) choice, capture the frame graph of
    ``graph`` (a FrameGraph) and time
    ``frames`` replays of the whole frame (binning, splat and merge all depend
    on the tile); keep the fastest on its pipeline and return
    {(tile, warps, stages): ms per frame}.  Every choice runs the same frames
    from the same state (positions, photon budgets, frame counter), and that
    state is restored at the end: the simulation does not advance."""
    pipe = graph.pipe
    traj = graph.traj
    state = (traj._pos.clone(), pipe.budget.clone(), graph.frame.clone(), graph.frames_done,
             traj._cls.clone())

    def restore():
        traj._pos.copy_(state[0])
        pipe.budget.copy_(state[1])
        graph.frame.copy_(state[2])
        graph.frames_done = state[3]
        traj._cls.copy_(state[4])

    times = {}
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for cand in candidates:
        restore()
        try:
            pipe.set_tiles(*cand)
            graph.graph, graph.use_graph = None, True
            graph.step()  # one eager frame, then capture
            graph.step()
            torch.cuda.synchronize()
            a.record()
            for _ in range(frames):
                graph.step()
            b.record()
            torch.cuda.synchronize()
            times[tuple(cand)] = a.elapsed_time(b) / (frames * graph.frames_per_step)
        except (ValueError, _lib.ScopyonGPUError):
            continue
    graph.graph = None
    torch.cuda.synchronize()
    restore()
    if not times:
        raise RuntimeError("no tile configuration ran")
    pipe.set_tiles(*min(times, key=times.get))
    return times


class HostRowsGraph:
    """Native frames from host rows replayed from captured CUDA graphs.

    A frame's rows ((n_sub, n, 5) float64 [depth, x, y, m_id, p_state], in
    pinned host memory that stays unchanged) and unit times go to the device
    on a copy stream, into one of two input slots, while the frame before
    runs on the current stream; the current stream then waits for them and
    replays the slot's graph: the records (sc_emitter_steps), the binning,
    the splat and the merge with the camera, into ``pipe.expect`` and
    ``pipe.adc32``.  The camera's Philox key is ``seed`` and its counter the
    frame index, which travels with the slot's unit times.  Before each
    replay the pipeline's ``graph_signature`` is compared with the one the
    graphs were captured with; a change (a PSF table that grew, a buffer
    reallocated) runs that frame eagerly and captures the graphs again.
    """

    def __init__(self, pipe, n_sub, n, seed, bleaching):
        dev = pipe.device
        self.pipe, self.n_sub, self.n = pipe, int(n_sub), int(n)
        self.seed, self.bleaching = int(seed), bleaching
        self.part = [torch.empty(max(self.n_sub * self.n * 5, 1), dtype=torch.float64, device=dev)
                     for _ in range(2)]
        # per slot: the unit times (float64) then the frame index (int64)
        self.small = [torch.empty(self.n_sub + 1, dtype=torch.int64, device=dev) for _ in range(2)]
        self.h_small = torch.empty((2, self.n_sub + 1), dtype=torch.int64, pin_memory=True)
        self.h_small_np = self.h_small.numpy()
        self.copy_stream = torch.cuda.Stream(device=dev)
        for t in self.part + self.small:
            t.record_stream(self.copy_stream)  # freed only after the copies queued on it
        self.copied = [torch.cuda.Event(), torch.cuda.Event()]
        self.done = [torch.cuda.Event(), torch.cuda.Event()]
        self.used = [False, False]
        self.graphs = [None, None]
        self.sig = None
        self.k = 0
        self.captures = 0

    def _frame(self, k):
        """The frame's kernels on the current stream, from input slot k."""
        small = self.small[k]
        self.pipe.run_frame_device(self.part[k], small[: self.n_sub].view(torch.float64),
                                   self.n_sub, self.n, with_optinfo=False, seed=self.seed,
                                   counter=0, bleaching=self.bleaching,
                                   d_frame=small[self.n_sub:])

    def run(self, rows, unit_times, frame):
        """Frame ``frame`` from ``rows`` (pinned, C-contiguous, not changed
        afterwards) and ``unit_times`` (n_sub); returns ``pipe.adc32``."""
        k = self.k % 2
        self.k += 1
        main, cs = torch.cuda.current_stream(), self.copy_stream
        if self.used[k]:
            self.copied[k].synchronize()  # the slot's host values have been copied
            cs.wait_event(self.done[k])  # the slot's last frame has read its inputs
        else:
            cs.wait_stream(main)
        hs = self.h_small_np[k]
        hs[: self.n_sub].view(numpy.float64)[:] = unit_times
        hs[self.n_sub] = int(frame)
        s = stream_ptr(cs)
        call("sc_copy_async", ptr(self.part[k]), ctypes.c_void_p(rows.ctypes.data), rows.nbytes, s)
        call("sc_copy_async", ptr(self.small[k]), ctypes.c_void_p(hs.ctypes.data), hs.nbytes, s)
        self.copied[k].record(cs)
        main.wait_event(self.copied[k])
        self.used[k] = True
        sig = self.pipe.graph_signature()
        if self.graphs[k] is not None and sig == self.sig:
            self.graphs[k].replay()
        else:
            # eagerly (which allocates what the frame needs), then capture
            # both slots' graphs on the buffers as they now are
            self._frame(k)
            self.graphs = [None, None]
            for j in range(2):
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._frame(j)
                self.graphs[j] = g
            self.sig = self.pipe.graph_signature()
            self.captures += 1
        self.done[k].record(main)
        return self.pipe.adc32


class FrameGraph:
    """Frames of device trajectories replayed from one captured CUDA graph.

    Every frame runs the same kernel sequence -- Brownian sub-steps, emitter
    physics and footprints, tile binning, splat, camera -- on fixed buffers;
    the only per-frame quantity, the frame index that offsets the Philox
    counters, lives in device memory and is advanced by the graph itself.
    Launch cost per frame is one graph launch.  Outputs (``pipe.expect``,
    ``pipe.adc32``) are overwritten by each frame.

    frames_per_step=k > 1 runs k consecutive frames per step (per graph
    replay) as a pipeline: the records kernels (which need only the positions
    and budgets the previous frame left) and the binning run in frame order on
    a high-priority side stream, each into one of two record and bin buffer
    sets, while the main stream splats and images the frame before.  Frame i + 2's
    records wait for frame i's image to free its buffer set.  The frames and
    their results are those of k single steps.  Frame i of a step writes its
    expectation and ADC counts into ``outputs[i]``; the last frame's pair is
    ``pipe.expect`` / ``pipe.adc32``, so all k frames' images remain after
    the step.
    """

    def __init__(self, pipe, traj, n_sub, unit_time, first_frame=0, transform=None, seed=0,
                 use_graph=True, frames_per_step=1):
        if int(frames_per_step) < 1:
            raise ValueError("frames_per_step must be at least 1")
        self.frames_per_step = int(frames_per_step)
        self.pipe, self.traj, self.n_sub = pipe, traj, int(n_sub)
        self.n = traj.n_particles
        dev = pipe.device
        traj.prepare_uniform(self.n_sub)
        if traj._index != first_frame * self.n_sub:
            traj.advance_to(first_frame * self.n_sub, transform)
        self.frame = torch.full((1,), int(first_frame), dtype=torch.int64, device=dev)
        self.ut = torch.full((self.n_sub,), float(unit_time), dtype=torch.float64, device=dev)
        self.transform = transform
        self.seed = int(seed)
        pipe.ensure_slots(self.n)
        self.graph = None
        self.use_graph = use_graph
        self.frames_done = 0
        # the second frame's records: a side stream that the scheduler serves first
        self._side = torch.cuda.Stream(device=dev, priority=-1) if frames_per_step > 1 else None
        # record and bin buffer sets: the records run up to this many frames
        # ahead of the image
        self.record_sets = 2
        # (expect, adc32) of each frame of a step, the last one the pipeline's
        self.outputs = [(torch.empty_like(pipe.expect), torch.empty_like(pipe.adc32))
                        for _ in range(self.frames_per_step - 1)] + [(pipe.expect, pipe.adc32)]

    def _records(self, tag, first_step):
        """Records of one frame (sub-steps first_step .. + n_sub of the frame
        counter's frame), counted into the bin buffers named by ``tag``."""
        pipe, traj, s = self.pipe, self.traj, stream_ptr()
        n_rec = self.n_sub * self.n
        recs = pipe._buf("recs" + tag, max(n_rec, 1) * (_lib.STEP_REC_BYTES // 4), torch.int32)
        dp = traj.graph_params(first_step, self.n_sub, self.transform)
        dp.d_frame = self.frame.data_ptr()
        sp = pipe.step_params(self.n_sub, self.n, False)
        bufs = pipe.bin_buffers(n_rec, tag=tag)
        bsp, ws, ws_bytes, _, _ = bufs
        call("sc_bin_reset", bsp, ptr(ws), ws_bytes, s)
        with pipe.timed("records"):
            call("sc_native_records", dp, sp, ptr(traj._pos), ptr(traj._cls),
                 ptr(traj._g_sigma), None, ptr(self.ut), ptr(pipe.budget), ptr(pipe.psf.key_slot),
                 ptr(recs), bsp, ptr(ws), ws_bytes, ptr(pipe.status), s)
        pipe.finish_bins(n_rec, tag, bufs=bufs)
        return recs, bufs

    def _image(self, recs, tag, frame_offset):
        """Splat and camera of one frame's binned records."""
        pipe = self.pipe
        recs, bufs = recs
        pipe.splat_camera(recs, self.n_sub * self.n, seed=self.seed, counter=frame_offset,
                          d_frame=self.frame, tag=tag, binned=True, bufs=bufs,
                          out=self.outputs[frame_offset])

    def _launch(self):
        s = stream_ptr()
        if self.frames_per_step == 1:
            self._image(self._records("", 0), "", 0)
            call("sc_counter_add", ptr(self.frame), 1, s)
            return
        main, side, k = torch.cuda.current_stream(), self._side, self.frames_per_step
        n_sets = self.record_sets
        tags = ("",) + tuple("_%d" % j for j in range(1, n_sets))
        recs, ready, imaged = [None] * k, [None] * k, [None] * k

        def records(i):
            if i >= n_sets:  # frame i - n_sets is done with this buffer set
                side.wait_event(imaged[i - n_sets])
            with torch.cuda.stream(side):
                recs[i] = self._records(tags[i % n_sets], i * self.n_sub)
            ready[i] = torch.cuda.Event()
            ready[i].record(side)

        fork = torch.cuda.Event()
        fork.record(main)
        side.wait_event(fork)
        for i in range(min(n_sets, k)):
            records(i)
        for i in range(k):
            main.wait_event(ready[i])
            self._image(recs[i], tags[i % n_sets], i)
            imaged[i] = torch.cuda.Event()
            imaged[i].record(main)
            if i + n_sets < k:
                records(i + n_sets)
        call("sc_counter_add", ptr(self.frame), k, s)

    def state_dict(self):
        """Checkpoint: the trajectories' state, the photon budgets and the
        frame counter, as host arrays and numbers (picklable).  The frames
        after ``load_state_dict`` of it equal those that followed it."""
        n = self.n
        frame = int(self.frame.item())
        traj = self.traj.state_dict()
        traj["index"] = frame * self.n_sub  # the graph counts frames on the device
        return {"trajectories": traj,
                "budget": self.pipe.budget[:n].cpu().numpy().copy(),
                "frame": frame, "frames_done": int(self.frames_done),
                "seed": self.seed, "n_sub": self.n_sub}

    def load_state_dict(self, state):
        """Resume from ``state_dict()`` in place: the device buffers keep their
        addresses, so a captured graph replays from the restored state."""
        if int(state["seed"]) != self.seed or int(state["n_sub"]) != self.n_sub:
            raise ValueError("the state is of a frame graph with another seed or sub-step count")
        budget = numpy.asarray(state["budget"], dtype=numpy.float64)
        if budget.shape != (self.n,):
            raise ValueError("the state holds %d budgets for %d particles" % (budget.size, self.n))
        self.traj.load_state_dict(state["trajectories"])
        self.pipe.budget[: self.n].copy_(torch.from_numpy(budget))
        self.frame.fill_(int(state["frame"]))
        self.frames_done = int(state["frames_done"])

    def capture(self):
        """Run one frame eagerly (allocates every buffer), then capture the next."""
        self._launch()
        self.frames_done += self.frames_per_step
        if not self.use_graph:
            return
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._launch()
        self.graph = g

    def step(self):
        if self.graph is None and self.use_graph:
            self.capture()
            return
        if self.graph is not None:
            self.graph.replay()
        else:
            self._launch()
        self.frames_done += self.frames_per_step

    @property
    def launches_per_frame(self):
        # native records (counting into bins), bin scan, then place + sort +
        # long-list sort or, from 2^20 records on, three kernels per radix
        # digit pass; splat box (the bulk-copy kernel also adds the summed-area
        # records), summed-area pass otherwise; camera (with the merge),
        # counter (plus one memset)
        pipe = self.pipe
        fused = (pipe.stages > 0 and pipe.psf.box_p > 0 and 12 <= pipe.psf.box_nq <= 16 and
                 pipe.tile + 15 <= 32)
        # box kernel, summed-area pass unless fused, merge unless it runs in
        # the camera pass (sc_merge_camera, counted as the camera)
        splat = (1 if fused else 2) + (0 if pipe.merge_camera else 1)
        n_rec = self.n_sub * self.n
        if n_rec < (1 << 20):
            return 7 + splat
        n_bins = 2 * pipe.tiles_x * pipe.tiles_y
        bits = max(1, n_bins.bit_length())  # keys 0 .. n_bins
        return 4 + splat + 3 * (-(-bits // 9))
