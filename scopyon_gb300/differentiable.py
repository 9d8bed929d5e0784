"""Differentiable expected images (Gaussian PSF) with a hand-written adjoint.

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
        self._ws = None

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
        n = _lib.load().sc_gauss_workspace_bytes(p)
        if self._ws is None or self._ws.numel() < n:
            self._ws = torch.empty(max(n, 1), dtype=torch.uint8, device=self.device)
        return self._ws, n


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
        ctx.save_for_backward(emitters, sig)
        ctx.model = model
        return mu

    @staticmethod
    def backward(ctx, grad_mu):
        emitters, sig = ctx.saved_tensors
        model = ctx.model
        F, N = emitters.shape[:2]
        g = grad_mu.contiguous().float()
        p = model.params(F, N)
        g_emit = torch.empty_like(emitters)
        g_sig_e = torch.empty(F, N, dtype=torch.float32, device=emitters.device)
        s = stream_ptr()
        call("sc_gauss_backward", p, ptr(emitters), ptr(sig), ptr(g), ptr(g_emit), ptr(g_sig_e), s)
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
