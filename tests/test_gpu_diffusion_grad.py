"""GPU: the reparameterised gradient of a summed frame with respect to D.

1,000 emitters, 20 sub-steps: the GPU dL/dD against FP64 autograd of the
same model (same normals), and against central finite differences in D of
the GPU loss and of the FP64 loss; under Philox draws the loss is
deterministic and the backward pass (trajectories regenerated) agrees with
finite differences.
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


def reference_loss(D, p0, normals, T, dt, sigma, model, counts, bg, var):
    """FP64 torch: positions p0 + sqrt(2 D dt) Z_t, frame, Gaussian NLL."""
    N = p0.shape[0]
    Z = torch.cat([torch.zeros(1, N, 2, dtype=torch.float64, device=p0.device),
                   torch.cumsum(normals, 0)[:-1]], 0)  # Z_t = n_0 + ... + n_{t-1}
    s = torch.sqrt(2 * D * dt)
    xy = p0[None, :, :2] + s * Z
    R = model.half_win
    d = torch.arange(-R, R + 1, dtype=torch.float64, device=p0.device)

    def axis(c, n):
        cr = (c + n * model.px * 0.5) / model.px
        ic = torch.floor(cr).detach()
        f = cr - ic
        a = (d - f[..., None]) * (model.px / sigma)
        b = (d + 1.0 - f[..., None]) * (model.px / sigma)
        g = 0.5 * (torch.erf(b / math.sqrt(2)) - torch.erf(a / math.sqrt(2)))
        idx = (ic[..., None] + d).long()
        ok = (idx >= 0) & (idx < n)
        full = torch.zeros(*c.shape, n, dtype=torch.float64, device=p0.device)
        return full.scatter_add(-1, idx.clamp(0, n - 1), torch.where(ok, g, torch.zeros_like(g)))

    gx, gy = axis(xy[..., 0], model.nw), axis(xy[..., 1], model.nh)
    w = p0[:, 3] / T
    mu = bg + torch.einsum("n,tni,tnj->ij", w, gx, gy)
    r = counts - mu
    v = mu + var
    return (r * r / (2 * v) + 0.5 * torch.log(v)).sum()


def setup(dm, N=1000, T=20, nw=128, seed=4):
    rng = numpy.random.RandomState(seed)
    sigma = 120e-9
    model = dm.GaussianImageModel(nw, nw, PX, 1.5 * sigma)
    e = numpy.zeros((N, 4), dtype=numpy.float32)
    e[:, 0] = rng.uniform(-0.45, 0.45, N) * nw * PX
    e[:, 1] = rng.uniform(-0.45, 0.45, N) * nw * PX
    e[:, 3] = rng.lognormal(math.log(2000.0), 0.3, N)
    normals = rng.standard_normal((T, N, 2)).astype(numpy.float32)
    dt, D_true, D0 = 1e-3, 0.05e-12, 0.03e-12
    return model, e, normals, sigma, dt, D_true, D0


def test_dD_matches_fp64_and_finite_differences(dm):
    model, e, normals, sigma, dt, D_true, D0 = setup(dm)
    dev = "cuda"
    T = normals.shape[0]
    emit = torch.tensor(e, device=dev)
    nrm = torch.tensor(normals, device=dev)
    sig = torch.tensor(sigma, dtype=torch.float32, device=dev)
    bg, var = 10.0, 2.25
    # synthetic target: the frame at the true D, with Gaussian noise of the model's variance
    with torch.no_grad():
        p_true = dm.diffusion_positions(torch.tensor(D_true, dtype=torch.float32, device=dev),
                                        emit, T, dt, normals=nrm)
        mu_true = dm.expected_image(p_true.reshape(1, -1, 4), torch.full((1,), bg, device=dev),
                                    sig, model)[0]
        gen = torch.Generator(dev).manual_seed(2)
        counts = mu_true + torch.sqrt(mu_true + var) * torch.randn(mu_true.shape, device=dev,
                                                                   generator=gen)
    D = torch.tensor(D0, dtype=torch.float32, device=dev).requires_grad_(True)
    loss = dm.diffusion_loss(D, emit, counts, sig, model, T, dt, background=bg,
                             readout_var=var, normals=nrm)
    loss.backward()
    g_gpu = D.grad.item()

    D64 = torch.tensor(float(torch.tensor(D0, dtype=torch.float32)), dtype=torch.float64,
                       device=dev).requires_grad_(True)
    l64 = reference_loss(D64, emit.double(), nrm.double(), T, dt,
                         float(torch.tensor(sigma, dtype=torch.float32)), model, counts.double(),
                         bg, var)
    l64.backward()
    assert abs(loss.item() - l64.item()) <= 1e-6 * abs(l64.item())
    assert abs(g_gpu - D64.grad.item()) <= 1e-3 * abs(D64.grad.item()), (g_gpu, D64.grad.item())

    h = 1e-3 * D0
    with torch.no_grad():
        lp = reference_loss(D64 + h, emit.double(), nrm.double(), T, dt, sig.double(), model,
                            counts.double(), bg, var).item()
        lm = reference_loss(D64 - h, emit.double(), nrm.double(), T, dt, sig.double(), model,
                            counts.double(), bg, var).item()
        gp = dm.diffusion_loss(torch.tensor(D0 + h, device=dev), emit, counts, sig, model, T, dt,
                               background=bg, readout_var=var, normals=nrm).item()
        gm = dm.diffusion_loss(torch.tensor(D0 - h, device=dev), emit, counts, sig, model, T, dt,
                               background=bg, readout_var=var, normals=nrm).item()
    fd64 = (lp - lm) / (2 * h)
    fd32 = (gp - gm) / (2 * h)
    assert abs(g_gpu - fd64) <= 2e-3 * abs(fd64), (g_gpu, fd64)
    assert abs(g_gpu - fd32) <= 2e-2 * abs(fd64), (g_gpu, fd32)
    assert g_gpu < 0  # D0 below the true D: increasing D lowers the loss


def test_philox_path_regenerates_trajectories(dm):
    model, e, normals, sigma, dt, D_true, D0 = setup(dm, N=400, T=30, seed=9)
    dev = "cuda"
    emit = torch.tensor(e, device=dev)
    sig = torch.tensor(sigma, dtype=torch.float32, device=dev)
    with torch.no_grad():
        pos = dm.diffusion_positions(torch.tensor(D_true, device=dev), emit, 30, dt, seed=7)
        counts = dm.expected_image(pos.reshape(1, -1, 4), torch.full((1,), 5.0, device=dev), sig,
                                   model)[0]
    D = torch.tensor(D0, dtype=torch.float32, device=dev).requires_grad_(True)
    loss = dm.diffusion_loss(D, emit, counts, sig, model, 30, dt, seed=7, background=5.0,
                             readout_var=1.0)
    loss2 = dm.diffusion_loss(D.detach(), emit, counts, sig, model, 30, dt, seed=7,
                              background=5.0, readout_var=1.0)
    assert loss.item() == loss2.item()  # same counters, same trajectories, same bits
    loss.backward()
    h = 1e-3 * D0
    with torch.no_grad():
        lp = dm.diffusion_loss(torch.tensor(D0 + h, device=dev), emit, counts, sig, model, 30, dt,
                               seed=7, background=5.0, readout_var=1.0).item()
        lm = dm.diffusion_loss(torch.tensor(D0 - h, device=dev), emit, counts, sig, model, 30, dt,
                               seed=7, background=5.0, readout_var=1.0).item()
    fd = (lp - lm) / (2 * h)
    assert abs(D.grad.item() - fd) <= 2e-2 * abs(fd), (D.grad.item(), fd)
    # the start positions at t = 0 equal the emitters
    assert torch.equal(pos[0, :, :2], emit[:, :2])
