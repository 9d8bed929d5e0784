"""GPU: the differentiable Born-Wolf image and its adjoint.

The CUDA forward and adjoint (``born_wolf_image``) against an FP64 torch
model of the same continuous image (each 1-nm cell of the Born-Wolf grid a
constant, integrated exactly over each pixel; the two depth keys around
|z - z_focal| blended linearly; TIRF excitation), built here from the
oracle's grids, with torch autograd for its gradients:
* expected photons within 1e-5 relative per pixel (above 1e-6 of the max);
* dL/dx, dL/dy, dL/dz, dL/dI and dL/dbg within 1e-5 of each component's
  largest magnitude, for L = sum w mu with fixed random weights w (the
  adjoint itself, free of the cancellation in dL/dmu of a likelihood near its
  optimum);
* central differences of the same L on the GPU at positions inside one 1-nm
  cell (h = 0.25 nm): the image is linear in x, y and z inside a cell, so the
  differences are exact up to FP32 rounding, within 1e-3 of each
  component's scale;
* an Adam localisation of x, y, z on a Poisson likelihood.
"""

import math

import numpy
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

RES = 1e-9


@pytest.fixture(scope="module")
def dm():
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import differentiable
    return differentiable


def _model(dm, edge=24, angle=None):
    import scopyon_gb300 as sg
    cfg = sg.DefaultConfiguration()
    upd = {"magnification": 100, "fluorophore": {"type": "EGFP"},
           "detector": {"image_size": [edge, edge]}}
    if angle is not None:
        upd["light_source"] = {"angle": angle}
    cfg.update({"default": upd})
    return dm.BornWolfImageModel(cfg, device="cuda")


class _Prefix:
    """FP64 2-D prefix sums of the full 1999^2 Born-Wolf grid per depth key."""

    def __init__(self, model):
        self.model, self.cache = model, {}
        self.r = O.radial_grid()

    def __call__(self, key):
        if key not in self.cache:
            m = self.model
            psf_r = O.born_wolf_radial(self.r, key * RES, float(m.eng.psf_wavelength), m.eng.na)
            grid = O.radial_to_cartesian(self.r, psf_r)
            s = numpy.zeros((grid.shape[0] + 1, grid.shape[1] + 1))
            s[1:, 1:] = grid.cumsum(0).cumsum(1)
            self.cache[key] = torch.from_numpy(s)
        return self.cache[key]


def _bilinear(S, alpha, beta, ns):
    """Bilinear prefix at corner coordinates (alpha (nx+1,), beta (ny+1,)), clamped."""
    al = alpha.clamp(0.0, float(ns))
    be = beta.clamp(0.0, float(ns))
    a = torch.clamp(torch.floor(al.detach()).long(), max=ns - 1)
    b = torch.clamp(torch.floor(be.detach()).long(), max=ns - 1)
    fa = (al - a.double())[:, None]
    fb = (be - b.double())[None, :]
    s00, s10 = S[a[:, None], b[None, :]], S[a[:, None] + 1, b[None, :]]
    s01, s11 = S[a[:, None], b[None, :] + 1], S[a[:, None] + 1, b[None, :] + 1]
    return (1 - fa) * ((1 - fb) * s00 + fb * s01) + fa * ((1 - fb) * s10 + fb * s11)


def torch_image(model, prefix, emit, bg):
    """The same continuous image in FP64 torch (differentiable by autograd)."""
    F, N = emit.shape[:2]
    nw, nh, px = model.nw, model.nh, model.px
    n_r = model.psf.n_r
    ns = 2 * n_r - 1
    half_w, half_h, half_sig = nw * px * 0.5, nh * px * 0.5, RES * (ns - 1) * 0.5
    mu = [bg[f] + torch.zeros(nw, nh, dtype=torch.float64) for f in range(F)]
    for f in range(F):
        for n in range(N):
            x, y, z, I = emit[f, n]
            dz = z - model.z_focal
            zr = dz.abs()
            zq = zr / RES
            if float(zq.detach()) >= model.key_hi:
                k, t = model.key_hi - 1, torch.ones((), dtype=torch.float64)
            else:
                k = int(math.floor(float(zq.detach())))
                t = zq - k
            A = torch.exp(-zr * model.inv_pen) if model.inv_pen > 0 else 1.0
            x0 = (half_w + x) - half_sig
            y0 = (half_h + y) - half_sig
            span = RES * ns
            i_lo = max(0, int(math.floor(float((x0 - RES) / px))))
            i_hi = min(nw - 1, int(math.floor(float((x0 - RES + span) / px))))
            j_lo = max(0, int(math.floor(float((y0 - RES) / px))))
            j_hi = min(nh - 1, int(math.floor(float((y0 - RES + span) / px))))
            if i_hi < i_lo or j_hi < j_lo:
                continue
            ci = torch.arange(i_lo, i_hi + 2, dtype=torch.float64)
            cj = torch.arange(j_lo, j_hi + 2, dtype=torch.float64)
            alpha = (ci * px - x0) / RES + 1.0
            beta = (cj * px - y0) / RES + 1.0

            def box(S):
                Fc = _bilinear(S, alpha, beta, ns)
                return Fc[1:, 1:] - Fc[:-1, 1:] - Fc[1:, :-1] + Fc[:-1, :-1]

            B = (1 - t) * box(prefix(k)) + t * box(prefix(k + 1))
            mu[f] = mu[f].index_put((torch.arange(i_lo, i_hi + 1)[:, None],
                                     torch.arange(j_lo, j_hi + 1)[None, :]),
                                    I * A * model.cnorm * B, accumulate=True)
    return torch.stack(mu)


def _emitters(model, F, N, seed, mid_cell=False):
    rng = numpy.random.RandomState(seed)
    half = model.nw * model.px * 0.3
    e = numpy.zeros((F, N, 4))
    e[..., 0] = rng.uniform(-half, half, (F, N))
    e[..., 1] = rng.uniform(-half, half, (F, N))
    e[..., 2] = rng.uniform(0.05e-6, 0.7e-6, (F, N)) * rng.choice([-1, 1], (F, N))
    e[..., 3] = rng.lognormal(math.log(2000.0), 0.3, (F, N))
    if mid_cell:  # x, y, z in the middle of a 1-nm cell
        e[..., :3] = (numpy.floor(e[..., :3] / RES) + 0.5) * RES
    return e.astype(numpy.float32)


@pytest.mark.parametrize("angle", [0.0, None])  # EPI, and the default TIRF angle
def test_forward_and_gradients_match_fp64_autograd(dm, angle):
    model = _model(dm, angle=angle)
    prefix = _Prefix(model)
    e = _emitters(model, 2, 4, seed=3)
    bg = numpy.array([10.0, 4.0], dtype=numpy.float32)
    emit = torch.tensor(e, device="cuda").requires_grad_(True)
    bgt = torch.tensor(bg, device="cuda").requires_grad_(True)
    mu = dm.born_wolf_image(emit, bgt, model)
    w = torch.randn(mu.shape, generator=torch.Generator().manual_seed(5), dtype=torch.float64)
    (mu * w.float().cuda()).sum().backward()

    e64 = torch.tensor(e.astype(numpy.float64)).requires_grad_(True)
    b64 = torch.tensor(bg.astype(numpy.float64)).requires_grad_(True)
    mu64 = torch_image(model, prefix, e64, b64)
    (mu64 * w.float().double()).sum().backward()

    ref = mu64.detach().numpy()
    got = mu.detach().double().cpu().numpy()
    sig = ref - bg[:, None, None]
    big = sig > 1e-6 * sig.max()
    assert (numpy.abs(got - ref)[big] / ref[big]).max() <= 1e-5
    ge, gr = emit.grad.cpu().numpy(), e64.grad.numpy()
    for comp in range(4):
        scale = numpy.abs(gr[..., comp]).max()
        assert numpy.abs(ge[..., comp] - gr[..., comp]).max() <= 1e-5 * scale, comp
    numpy.testing.assert_allclose(bgt.grad.cpu().numpy(), b64.grad.numpy(), rtol=1e-5)


def test_gradients_match_central_differences(dm):
    model = _model(dm, angle=None)  # TIRF: z enters through the depth keys and A(z)
    e = _emitters(model, 1, 3, seed=11, mid_cell=True)
    bg = torch.tensor([6.0], device="cuda")
    w = torch.randn((1, model.nw, model.nh), generator=torch.Generator().manual_seed(2)).cuda()
    emit = torch.tensor(e, device="cuda").requires_grad_(True)
    (dm.born_wolf_image(emit, bg, model) * w).sum().backward()
    g = emit.grad.cpu().numpy()
    h = 0.25 * RES

    def loss(ep):
        with torch.no_grad():
            mu = dm.born_wolf_image(torch.tensor(ep, device="cuda"), bg, model)
            return float((mu.double() * w.double()).sum())

    for comp in range(3):
        scale = numpy.abs(g[0, :, comp]).max()
        for n in range(3):
            ep, em = e.copy(), e.copy()
            ep[0, n, comp] += h
            em[0, n, comp] -= h
            fd = (loss(ep) - loss(em)) / (2 * h)
            assert abs(fd - g[0, n, comp]) <= 1e-3 * scale, (n, comp, fd, g[0, n, comp])


def test_adam_localisation(dm):
    model = _model(dm, edge=32, angle=0.0)
    truth = _emitters(model, 1, 3, seed=21)
    truth[..., 2] = numpy.abs(truth[..., 2]) + 0.2e-6
    bg = torch.tensor([5.0], device="cuda")
    with torch.no_grad():
        mu = dm.born_wolf_image(torch.tensor(truth, device="cuda"), bg, model)
        counts = torch.poisson(mu.double() * 50,
                               generator=torch.Generator("cuda").manual_seed(1)).float() / 50
    start = truth.copy()
    rng = numpy.random.RandomState(4)
    start[..., :2] += rng.uniform(-60e-9, 60e-9, start[..., :2].shape)
    start[..., 2] += rng.uniform(-50e-9, 50e-9, start[..., 2].shape)
    pos = torch.tensor(start[..., :3] * 1e6, device="cuda").requires_grad_(True)  # um
    inten = torch.tensor(start[..., 3:], device="cuda")
    opt = torch.optim.Adam([pos], lr=5e-3)
    first = None
    for _ in range(150):
        opt.zero_grad()
        emit = torch.cat([pos * 1e-6, inten], -1)
        loss = dm.poisson_nll(dm.born_wolf_image(emit, bg, model), counts)
        first = float(loss) if first is None else first
        loss.backward()
        opt.step()
    err = numpy.abs(pos.detach().cpu().numpy() - truth[..., :3] * 1e6)
    assert float(loss) < first
    assert err[..., :2].max() < 0.01  # 10 nm in x and y
