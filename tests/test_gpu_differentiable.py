"""GPU: the differentiable expected image and its hand-written adjoint.

Checked against an FP64 torch model of the same analytic image (the same
(2R+1)^2 windows): the forward to 1e-5 relative per pixel, the gradients of a
Poisson negative log-likelihood with respect to x, y, z, intensity,
background and sigma against FP64 autograd, and against central finite
differences (h = 1e-3) of the FP64 loss.  A short Adam fit recovers emitter
positions from a Poisson-noisy image.
"""

import math

import numpy
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

PX = 160e-9


@pytest.fixture(scope="module")
def dm():
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import differentiable
    return differentiable


def reference_image(emit, bg, sigma, model):
    """FP64 torch model: mu = bg + sum_e I A(z) Gx Gy over each emitter's window."""
    F, N, _ = emit.shape
    x, y, z, inten = emit.unbind(-1)
    R = model.half_win
    d = torch.arange(-R, R + 1, dtype=torch.float64, device=emit.device)

    def axis(c, n):
        cr = (c + n * model.px * 0.5) / model.px
        ic = torch.floor(cr).detach()
        f = cr - ic
        s = model.px / sigma
        a = (d - f[..., None]) * s
        b = (d + 1.0 - f[..., None]) * s
        g = 0.5 * (torch.erf(b / math.sqrt(2)) - torch.erf(a / math.sqrt(2)))
        idx = (ic[..., None] + d).long()
        ok = (idx >= 0) & (idx < n)
        full = torch.zeros(F, N, n, dtype=torch.float64, device=emit.device)
        full = full.scatter_add(2, idx.clamp(0, n - 1), torch.where(ok, g, torch.zeros_like(g)))
        return full

    gx, gy = axis(x, model.nw), axis(y, model.nh)
    amp = torch.exp(-(z - model.z_focal).abs() * model.inv_pen) if model.inv_pen else 1.0
    c = inten * amp
    return bg[:, None, None] + torch.einsum("fn,fni,fnj->fij", c, gx, gy)


def make_case(dm, seed, F=3, N=60, nw=48, nh=40, pen=math.inf, sigma=1.3 * PX, tile=8):
    rng = numpy.random.RandomState(seed)
    model = dm.GaussianImageModel(nw, nh, PX, 1.5 * sigma, penetration=pen, tile=tile)
    e = numpy.zeros((F, N, 4))
    e[..., 0] = rng.uniform(-0.55, 0.55, (F, N)) * nw * PX  # some windows leave the image
    e[..., 1] = rng.uniform(-0.55, 0.55, (F, N)) * nh * PX
    e[..., 2] = rng.uniform(-0.5e-6, 0.5e-6, (F, N))
    e[..., 3] = rng.lognormal(math.log(2000.0), 0.3, (F, N))
    bg = numpy.full(F, 10.0)
    return model, e, bg, sigma


# (illumination, sigma in pixels, tile): sigma 1.3 px gives R = 11 (the per-pixel
# kernels), 0.8 px R = 7 and 0.45 px R = 4 (the tile kernels, buffers of 24 and
# 32 pixels a side)
CASES = [(math.inf, 1.3, 8), (300e-9, 1.3, 8), (math.inf, 0.8, 8), (300e-9, 0.8, 16),
         (math.inf, 0.45, 16), (300e-9, 0.45, 8)]


@pytest.mark.parametrize("pen,sigma_px,tile", CASES)
def test_forward_matches_fp64(dm, pen, sigma_px, tile):
    model, e, bg, sigma = make_case(dm, 1, pen=pen, sigma=sigma_px * PX, tile=tile)
    emit = torch.tensor(e, dtype=torch.float32, device="cuda")
    mu = dm.expected_image(emit, torch.tensor(bg, dtype=torch.float32, device="cuda"),
                           torch.tensor(sigma, dtype=torch.float32, device="cuda"), model)
    ref = reference_image(emit.double(), torch.tensor(bg, device="cuda"),
                          torch.tensor(float(torch.tensor(sigma, dtype=torch.float32)),
                                       dtype=torch.float64, device="cuda"), model)
    rel = ((mu.double() - ref).abs() / ref).max().item()
    assert rel <= 1e-5, rel
    # deterministic: the same inputs give the same bits
    mu2 = dm.expected_image(emit, torch.tensor(bg, dtype=torch.float32, device="cuda"),
                            torch.tensor(sigma, dtype=torch.float32, device="cuda"), model)
    assert torch.equal(mu, mu2)


def _loss64(emit, bg, sigma, model, counts):
    mu = reference_image(emit, bg, sigma, model)
    return (mu - counts * torch.log(mu)).sum()


@pytest.mark.parametrize("pen,sigma_px,tile", CASES)
def test_gradients_match_fp64_autograd_and_finite_differences(dm, pen, sigma_px, tile):
    model, e, bg, sigma = make_case(dm, 2, pen=pen, sigma=sigma_px * PX, tile=tile)
    dev = "cuda"
    emit = torch.tensor(e, dtype=torch.float32, device=dev)
    emit[..., 2] += 1e-9 * (emit[..., 2] == 0)  # keep |z - z_focal| differentiable
    bg_t = torch.tensor(bg, dtype=torch.float32, device=dev)
    sig_t = torch.tensor(sigma, dtype=torch.float32, device=dev)
    # noisy target from the model itself (shifted emitters, so gradients are not ~0)
    with torch.no_grad():
        shifted = emit.clone()
        shifted[..., 0] += 0.3 * PX
        shifted[..., 3] *= 1.2
        lam = dm.expected_image(shifted, bg_t, sig_t, model)
    counts = torch.poisson(lam.double(), generator=torch.Generator(dev).manual_seed(3)).float()

    emit_g = emit.clone().requires_grad_(True)
    bg_g = bg_t.clone().requires_grad_(True)
    sig_g = sig_t.clone().requires_grad_(True)
    loss = dm.poisson_nll(dm.expected_image(emit_g, bg_g, sig_g, model), counts)
    loss.backward()

    e64 = emit.double().requires_grad_(True)
    b64 = bg_t.double().requires_grad_(True)
    s64 = sig_t.double().requires_grad_(True)
    l64 = _loss64(e64, b64, s64, model, counts.double())
    l64.backward()
    assert abs(loss.item() - l64.item()) <= 1e-6 * abs(l64.item())

    scale = {0: PX, 1: PX, 2: 1e-6, 3: 1.0}  # gradients per pixel / micron / photon
    for k in range(4):
        g = emit_g.grad[..., k].double() * scale[k]
        r = e64.grad[..., k] * scale[k]
        if pen == math.inf and k == 2:
            assert g.abs().max().item() == 0.0
            continue
        err = (g - r).abs().max().item() / r.abs().max().item()
        assert err <= 2e-5, (k, err)
    assert abs(bg_g.grad - b64.grad).max().item() <= 1e-5 * b64.grad.abs().max().item()
    assert abs(sig_g.grad.item() - s64.grad.item()) <= 1e-4 * abs(s64.grad.item())

    # central finite differences of the FP64 loss, h = 1e-3 (pixels, microns, relative)
    rng = numpy.random.RandomState(5)
    for _ in range(6):
        f, n, k = rng.randint(3), rng.randint(emit.shape[1]), rng.randint(4)
        if pen == math.inf and k == 2:
            continue
        h = 1e-3 * {0: PX, 1: PX, 2: 1e-6, 3: e[f, n, 3]}[k]
        with torch.no_grad():
            ep, em = emit.double().clone(), emit.double().clone()
            ep[f, n, k] += h
            em[f, n, k] -= h
            fd = (_loss64(ep, b64, s64, model, counts.double()) -
                  _loss64(em, b64, s64, model, counts.double())).item() / (2 * h)
        got = emit_g.grad[f, n, k].item()
        assert abs(got - fd) <= 2e-3 * abs(fd) + 1e-6 * abs(e64.grad[..., k]).max().item(), (f, n, k)
    with torch.no_grad():
        hs = 1e-3 * sigma
        fd = (_loss64(emit.double(), b64, s64 + hs, model, counts.double()) -
              _loss64(emit.double(), b64, s64 - hs, model, counts.double())).item() / (2 * hs)
    assert abs(sig_g.grad.item() - fd) <= 2e-3 * abs(fd)


def test_interleaved_forwards_keep_their_own_workspace(dm):
    """Two forward calls before one backward: each backward pass reads the
    records and bins of its own forward call."""
    model, e, bg, sigma = make_case(dm, 4, sigma=0.8 * PX)
    dev = "cuda"
    bg_t = torch.tensor(bg, dtype=torch.float32, device=dev)
    sig_t = torch.tensor(sigma, dtype=torch.float32, device=dev)
    e1 = torch.tensor(e, dtype=torch.float32, device=dev)
    e2 = e1.flip(1).contiguous()
    e2[..., 0] += 0.4 * PX
    with torch.no_grad():
        counts = torch.poisson(dm.expected_image(e1, bg_t, sig_t, model).double(),
                               generator=torch.Generator(dev).manual_seed(2)).float()
    grads = []
    for pair in ((e1, e2), (e1, None), (None, e2)):
        leaves = [x.clone().requires_grad_(True) if x is not None else None for x in pair]
        loss = sum(dm.poisson_nll(dm.expected_image(x, bg_t, sig_t, model), counts)
                   for x in leaves if x is not None)
        loss.backward()
        grads.append([x.grad if x is not None else None for x in leaves])
    assert torch.equal(grads[0][0], grads[1][0])
    assert torch.equal(grads[0][1], grads[2][1])


def test_adam_localisation(dm):
    """Positions fitted by Adam on the Poisson NLL land near the truth."""
    model, e, bg, sigma = make_case(dm, 7, F=2, N=30, nw=64, nh=64)
    e[..., 0] *= 0.8  # keep emitters inside the image
    e[..., 1] *= 0.8
    dev = "cuda"
    truth = torch.tensor(e, dtype=torch.float32, device=dev)
    bg_t = torch.tensor(bg, dtype=torch.float32, device=dev)
    sig_t = torch.tensor(sigma, dtype=torch.float32, device=dev)
    with torch.no_grad():
        counts = torch.poisson(dm.expected_image(truth, bg_t, sig_t, model).double(),
                               generator=torch.Generator(dev).manual_seed(11)).float()
    rng = numpy.random.RandomState(8)
    start = truth.clone()
    start[..., :2] += torch.tensor(rng.uniform(-0.5, 0.5, (2, 30, 2)) * PX, dtype=torch.float32,
                                   device=dev)
    xy = (start[..., :2] / PX).clone().requires_grad_(True)  # optimise in pixel units
    opt = torch.optim.Adam([xy], lr=0.02)
    first = None
    for _ in range(200):
        opt.zero_grad()
        emit = torch.cat([xy * PX, truth[..., 2:]], dim=-1)
        loss = dm.poisson_nll(dm.expected_image(emit, bg_t, sig_t, model), counts)
        loss.backward()
        opt.step()
        first = loss.item() if first is None else first
    assert loss.item() < first
    err = (xy.detach() - truth[..., :2] / PX).abs()
    assert err.mean().item() < 0.06 and err.max().item() < 0.3, err.max().item()
