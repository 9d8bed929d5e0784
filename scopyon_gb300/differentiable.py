"""Differentiable expected images (Gaussian and Born-Wolf PSFs) with hand-written adjoints.

The forward is the reference's Gaussian point-spread path, ``_epifm.py:133-134``
with the pixel sums of ``overlay_signal_`` (``_epifm.py:224-282``). Two
changes: each pixel is integrated analytically rather than on the 1-nm grid,
and the depth enters through the TIRF excitation ``exp(-|z - z_focal| / d)``
(``_epifm.py:1281-1289``)::

    mu[f, i, j] = bg[f] + sum_e I_e A(z_e) Gx_e(i) Gy_e(j)

``expected_image`` wraps the CUDA forward (``sc_gauss_forward``) and adjoint
(``sc_gauss_backward``) in a ``torch.autograd.Function``. It gives
gradients with respect to emitter x, y, z, intensity, background and the PSF
width sigma. ``poisson_nll`` reduces the Poisson negative log-likelihood in
FP64 on the GPU.

``diffusion_loss`` differentiates a summed frame through Brownian
trajectories with respect to the diffusion coefficient D, using the
reparameterisation ``dp_t/dD = (p_t - p0) / (2 D)``. The backward pass
regenerates the trajectories from their Philox counters instead of storing
them.

The reference has no gradients; this module extends it on the same geometry
and configuration.
"""

import math

import torch

from . import _lib
from ._lib import call, ptr, stream_ptr


_scratch = {}


def _reduce_scratch(seg_len, n_seg, device):
    """A cached device scratch large enough for one reduction of this shape."""
    n = _lib.load().sc_reduce_scratch_bytes(int(seg_len), int(n_seg))
    t = _scratch.get(device)
    if t is None or t.numel() < n:
        t = torch.empty(max(n, 8), dtype=torch.uint8, device=device)
        _scratch[device] = t
    return t, n


class GaussianImageModel:
    """Geometry of the differentiable image: W x H pixels of ``px`` metres.

    ``sigma_max`` bounds the PSF width the model will see (windows are
    ``2R + 1`` pixels with ``R = ceil(5.5 sigma_max / px)``, at most 15);
    ``penetration`` is the TIRF depth ``d`` (``math.inf`` for EPI).
    """

    def __init__(self, nw, nh, px, sigma_max, penetration=math.inf, z_focal=0.0, tile=8,
                 device=None):
        self.nw, self.nh, self.px = int(nw), int(nh), float(px)
        self.half_win = max(1, min(15, int(math.ceil(5.5 * float(sigma_max) / self.px))))
        self.inv_pen = 0.0 if math.isinf(penetration) else 1.0 / float(penetration)
        self.z_focal = float(z_focal)
        self.tile = int(tile)
        self.device = torch.device(device or "cuda")

    @classmethod
    def from_config(cls, config, sigma_max=None, device=None):
        """Geometry, sigma bound and illumination of a ``Configuration``."""
        from .epifm import EngineConfig
        eng = EngineConfig(config["default"] if "default" in config else config)
        width = eng.radial_width if eng.radial_width else 0.1e-6
        nw, nh = eng.image_size
        return cls(nw, nh, eng.px, sigma_max or 1.5 * width, eng.penetration,
                   float(eng.focal_point[2]), device=device)

    def params(self, n_frames, n_emit):
        p = _lib.GaussParams()
        p.nw, p.nh, p.n_frames, p.n_emit = self.nw, self.nh, int(n_frames), int(n_emit)
        p.half_win, p.tile = self.half_win, self.tile
        p.px, p.inv_pen, p.z_focal = self.px, self.inv_pen, self.z_focal
        return p

    def workspace(self, p):
        """A fresh forward workspace (records and tile bins); the backward pass
        of the same call reads it, so calls do not share one."""
        n = _lib.load().sc_gauss_workspace_bytes(p)
        return torch.empty(max(n, 1), dtype=torch.uint8, device=self.device), n


def _check_inputs(emitters, background, sigma, model):
    if emitters.dim() != 3 or emitters.shape[-1] != 4:
        raise ValueError("emitters must be (frames, emitters, 4): x, y, z, intensity")
    if emitters.dtype != torch.float32 or not emitters.is_cuda:
        raise TypeError("emitters must be a float32 CUDA tensor")
    if background.shape != (emitters.shape[0],):
        raise ValueError("background must have one value per frame")
    if sigma.numel() != 1:
        raise ValueError("sigma must be a scalar tensor")


class _ExpectedImage(torch.autograd.Function):

    @staticmethod
    def forward(ctx, emitters, background, sigma, model):
        emitters = emitters.contiguous()
        background = background.contiguous().float()
        sig = sigma.reshape(1).contiguous().float()
        _check_inputs(emitters, background, sig, model)
        F, N = emitters.shape[:2]
        p = model.params(F, N)
        ws, nbytes = model.workspace(p)
        mu = torch.empty(F, model.nw, model.nh, dtype=torch.float32, device=emitters.device)
        status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=emitters.device)
        call("sc_gauss_forward", p, ptr(emitters), ptr(sig), ptr(background), ptr(ws), nbytes,
             ptr(mu), ptr(status), stream_ptr())
        ctx.save_for_backward(emitters, sig, ws)
        ctx.model = model
        return mu

    @staticmethod
    def backward(ctx, grad_mu):
        emitters, sig, ws = ctx.saved_tensors
        model = ctx.model
        F, N = emitters.shape[:2]
        g = grad_mu.contiguous().float()
        p = model.params(F, N)
        g_emit = torch.empty_like(emitters)
        g_sig_e = torch.empty(F, N, dtype=torch.float32, device=emitters.device)
        s = stream_ptr()
        call("sc_gauss_backward", p, ptr(emitters), ptr(sig), ptr(ws), ws.numel(), ptr(g),
             ptr(g_emit), ptr(g_sig_e), s)
        dev = emitters.device
        g_bg = torch.empty(F, dtype=torch.float64, device=dev)
        scr, n = _reduce_scratch(model.nw * model.nh, F, dev)
        call("sc_segment_sum", ptr(g), model.nw * model.nh, F, ptr(scr), n, ptr(g_bg), s)
        g_sigma = torch.empty(1, dtype=torch.float64, device=dev)
        scr, n = _reduce_scratch(F * N, 1, dev)
        call("sc_segment_sum", ptr(g_sig_e), F * N, 1, ptr(scr), n, ptr(g_sigma), s)
        return g_emit, g_bg.float(), g_sigma.float().reshape(()), None


def expected_image(emitters, background, sigma, model):
    """Expected photons per pixel, (frames, W, H) float32, differentiable.

    emitters: (frames, emitters, 4) float32 CUDA tensor of x, y (metres from
    the image centre), z (metres) and intensity (photons); background:
    (frames,) photons per pixel; sigma: scalar tensor, the PSF width (metres).
    """
    return _ExpectedImage.apply(emitters, background, sigma, model)


class BornWolfImageModel:
    """The differentiable Born-Wolf image of a configuration: its geometry,
    illumination and 1-nm depth-keyed PSF tables (the engine's, built on
    demand for the depths the emitters reach).

    The image is the reference's Born-Wolf image made continuous
    (``sc_bw_forward``): each 1-nm grid value fills a cell and a pixel takes
    the exact integral over its extent, and the two depth keys around
    ``|z - z_focal|`` are blended linearly, so that x, y and z all have
    gradients.  It differs from the reference's rounded bounds by a fraction
    of one 1-nm cell at each pixel edge.  Intensities are the photons an
    emitter in focus puts on its whole 1999-nm grid (the grid keeps the
    reference's constant floor past the radial cutoff, _epifm.py:123).
    """

    def __init__(self, config, device=None):
        import numpy
        from .base import _psf_for
        from .epifm import EngineConfig
        conf = config["default"] if "default" in config else config
        self.eng = EngineConfig(conf, rng=numpy.random.RandomState(0))
        if self.eng.fluorophore_type == "Gaussian":
            raise ValueError("the Born-Wolf image needs a Born-Wolf fluorophore")
        self.device = torch.device(device or "cuda")
        self.psf = _psf_for(self.eng, self.device)
        self.nw, self.nh = self.eng.image_size
        self.px = float(self.eng.px)
        pen = float(self.eng.penetration)
        self.inv_pen = 0.0 if math.isinf(pen) else 1.0 / pen
        # depth is the first component of the focal point, as in the
        # reference's [depth, x, y] layout (_epifm.py:1277-1289)
        self.z_focal = float(self.eng.focal_point[0])
        self.res = 1e-9
        self.key_hi = int(round(self.eng.depth_cutoff / self.res))
        # intensity = photons of an emitter in focus over its whole 1999-nm
        # grid: cnorm is one over the in-focus grid's sum (the full-grid prefix
        # S(n_signal, n_signal) from the quadrant table, 4 G[n][n] - 2 G[n][1]
        # - 2 G[1][n] + G[1][1] with n = n_r)
        self.psf.ensure([0])
        n = self.psf.n_r
        slot = self.psf.slot_of[0]
        tab = self.psf.tables[slot * self.psf.table_floats: (slot + 1) * self.psf.table_floats]
        G = tab.view(n + 1, self.psf.pitch, 2).double().sum(-1)
        total = float(4 * G[n, n] - 2 * G[n, 1] - 2 * G[1, n] + G[1, 1])
        self.cnorm = 1.0 / total

    def ensure_keys(self, emitters):
        """Build the tables of every depth key the emitters' |z - z_focal| needs."""
        z = emitters[..., 2]
        zr = (z.double() - self.z_focal).abs()
        lo, hi = float(zr.min()), float(zr.max())
        k_lo = min(int(lo / self.res), self.key_hi - 1)
        k_hi = min(int(hi / self.res), self.key_hi - 1) + 1
        self.psf.ensure(list(range(k_lo, k_hi + 1)))

    def params(self, n_frames, n_emit):
        p = _lib.BWParams()
        p.nw, p.nh, p.n_frames, p.n_emit = self.nw, self.nh, int(n_frames), int(n_emit)
        p.n_r, p.sat_pitch, p.key_hi = self.psf.n_r, self.psf.pitch, self.key_hi
        p.px, p.res, p.inv_pen, p.z_focal = self.px, self.res, self.inv_pen, self.z_focal
        p.cnorm = self.cnorm
        p.d_key_slot = self.psf.key_slot.data_ptr()
        return p


class _BornWolfImage(torch.autograd.Function):

    @staticmethod
    def forward(ctx, emitters, background, model):
        emitters = emitters.contiguous()
        background = background.contiguous().float()
        if emitters.dim() != 3 or emitters.shape[-1] != 4:
            raise ValueError("emitters must be (frames, emitters, 4): x, y, z, intensity")
        if emitters.dtype != torch.float32 or not emitters.is_cuda:
            raise TypeError("emitters must be a float32 CUDA tensor")
        if background.shape != (emitters.shape[0],):
            raise ValueError("background must have one value per frame")
        F, N = emitters.shape[:2]
        if N:
            model.ensure_keys(emitters)
        p = model.params(F, N)
        dev = emitters.device
        nbytes = _lib.load().sc_bw_work_bytes(p)
        work = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=dev)
        mu = torch.empty(F, model.nw, model.nh, dtype=torch.float32, device=dev)
        status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
        call("sc_bw_forward", p, ptr(emitters), ptr(background), ptr(model.psf.tables),
             ptr(work), nbytes, ptr(mu), ptr(status), stream_ptr())
        if int(status[0].item()):
            raise _lib.ScopyonGPUError(_lib.SC_ERR_ARG, "born-wolf image: status %s"
                                       % status.cpu().tolist())
        ctx.save_for_backward(emitters)
        ctx.model = model
        return mu

    @staticmethod
    def backward(ctx, grad_mu):
        (emitters,) = ctx.saved_tensors
        model = ctx.model
        F, N = emitters.shape[:2]
        dev = emitters.device
        g = grad_mu.contiguous().float()
        g_emit = torch.zeros_like(emitters)
        s = stream_ptr()
        status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
        call("sc_bw_backward", model.params(F, N), ptr(emitters), ptr(model.psf.tables), ptr(g),
             ptr(g_emit), ptr(status), s)
        g_bg = torch.empty(F, dtype=torch.float64, device=dev)
        scr, n = _reduce_scratch(model.nw * model.nh, F, dev)
        call("sc_segment_sum", ptr(g), model.nw * model.nh, F, ptr(scr), n, ptr(g_bg), s)
        return g_emit, g_bg.float(), None


def born_wolf_image(emitters, background, model):
    """Expected photons per pixel, (frames, W, H) float32, of the continuous
    Born-Wolf image (``BornWolfImageModel``), differentiable in the emitters
    (x, y, z, intensity) and the per-frame background.

    emitters: (frames, emitters, 4) float32 CUDA tensor of x, y (metres from
    the image centre), z (metres) and intensity (photons of the emitter in
    focus); background: (frames,) photons per pixel."""
    return _BornWolfImage.apply(emitters, background, model)


class _PoissonNLL(torch.autograd.Function):

    @staticmethod
    def forward(ctx, mu, counts):
        mu = mu.contiguous().float()
        counts = counts.contiguous().float()
        if mu.shape != counts.shape:
            raise ValueError("mu and counts must have the same shape")
        F = mu.shape[0] if mu.dim() > 1 else 1
        seg = mu.numel() // F
        loss = torch.empty(F, dtype=torch.float64, device=mu.device)
        grad = torch.empty_like(mu)
        scr, n = _reduce_scratch(seg, F, mu.device)
        call("sc_poisson_nll", ptr(mu), ptr(counts), seg, F, ptr(scr), n, ptr(loss), ptr(grad),
             stream_ptr())
        ctx.save_for_backward(grad)
        return loss.sum()

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return grad * g.to(grad.dtype), None


def poisson_nll(mu, counts):
    """sum(mu - k log mu) over all pixels (FP64 on the GPU), differentiable in mu."""
    return _PoissonNLL.apply(mu, counts)


def _dgrad_scratch(n, device):
    nbytes = _lib.load().sc_dgrad_scratch_bytes(int(n))
    key = ("dgrad", device)
    t = _scratch.get(key)
    if t is None or t.numel() < nbytes:
        t = torch.empty(max(nbytes, 8), dtype=torch.uint8, device=device)
        _scratch[key] = t
    return t, nbytes


def diffusion_positions(D, emitters, T, dt, seed=0, normals=None):
    """(T, N, 4) float32 sub-step positions (x_t, y_t, z, I / T) of emitters
    (N, 4) diffusing with coefficient D (device scalar, m^2/s) for T steps of
    dt; normals (T, N, 2), if given, replace the Philox draws."""
    N = emitters.shape[0]
    out = torch.empty(T, N, 4, dtype=torch.float32, device=emitters.device)
    call("sc_diffusion_positions", ptr(emitters), N, int(T), ptr(D), float(dt),
         int(seed) & (2 ** 64 - 1), ptr(normals), ptr(out), stream_ptr())
    return out


class _DiffusionLoss(torch.autograd.Function):

    @staticmethod
    def forward(ctx, D, emitters, counts, sigma, model, T, dt, seed, background, var, var_map,
                normals):
        D = D.reshape(1).contiguous().float()
        emitters = emitters.contiguous().float()
        dev = emitters.device
        N = emitters.shape[0]
        pos = diffusion_positions(D, emitters, T, dt, seed, normals)
        sig = sigma.reshape(1).contiguous().float()
        p = model.params(1, N * T)
        ws, nbytes = model.workspace(p)
        mu = torch.empty(1, model.nw, model.nh, dtype=torch.float32, device=dev)
        bg = torch.full((1,), float(background), dtype=torch.float32, device=dev)
        status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
        s = stream_ptr()
        call("sc_gauss_forward", p, ptr(pos), ptr(sig), ptr(bg), ptr(ws), nbytes, ptr(mu),
             ptr(status), s)
        del pos  # trajectories are not kept for the backward pass
        grad_mu = torch.empty_like(mu)
        loss = torch.empty(1, dtype=torch.float64, device=dev)
        scr, n = _dgrad_scratch(mu.numel(), dev)
        call("sc_gauss_nll", ptr(mu), ptr(counts.contiguous().float()), mu.numel(), ptr(var_map),
             float(var), ptr(scr), n, ptr(loss), ptr(grad_mu), s)
        ctx.save_for_backward(D, emitters, grad_mu, sig, ws,
                              normals if normals is not None else D)
        ctx.has_normals = normals is not None
        ctx.model, ctx.T, ctx.dt, ctx.seed = model, T, dt, seed
        return loss.reshape(())

    @staticmethod
    def backward(ctx, g):
        D, emitters, grad_mu, sig, ws, normals = ctx.saved_tensors
        normals = normals if ctx.has_normals else None
        model, T = ctx.model, ctx.T
        N = emitters.shape[0]
        dev = emitters.device
        # regenerate the trajectories from their counters
        pos = diffusion_positions(D, emitters, T, ctx.dt, ctx.seed, normals)
        p = model.params(1, N * T)
        grad_pos = torch.empty_like(pos)
        s = stream_ptr()
        call("sc_gauss_backward", p, ptr(pos), ptr(sig), ptr(ws), ws.numel(), ptr(grad_mu),
             ptr(grad_pos), None, s)
        dD = torch.empty(1, dtype=torch.float64, device=dev)
        scr, n = _dgrad_scratch(N * T, dev)
        call("sc_diffusion_dD", ptr(pos), ptr(emitters), N, int(T), ptr(grad_pos), ptr(D),
             ptr(scr), n, ptr(dD), s)
        return (dD * g).float().reshape(()), None, None, None, None, None, None, None, None, \
            None, None, None


def diffusion_loss(D, emitters, counts, sigma, model, T, dt, seed=0, background=0.0,
                   readout_var=0.0, normals=None):
    """Gaussian-approximated negative log-likelihood of the frame summed over T
    sub-steps of Brownian motion, differentiable in D (a scalar tensor, m^2/s).

    emitters: (N, 4) float32 CUDA tensor of start x, y (metres from the image
    centre), z and photons per frame; counts: (W, H) observed frame; sigma:
    PSF width (scalar tensor, metres); model: a ``GaussianImageModel``;
    readout_var: scalar or (W, H) tensor, the variance added to the shot
    noise; normals: (T, N, 2) float32 in place of the Philox draws."""
    var_map = readout_var if torch.is_tensor(readout_var) else None
    var = 0.0 if var_map is not None else float(readout_var)
    if var_map is not None:
        var_map = var_map.contiguous().float()
    return _DiffusionLoss.apply(D, emitters, counts, sigma, model, int(T), float(dt), int(seed),
                                float(background), var, var_map, normals)
