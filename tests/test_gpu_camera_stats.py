"""GPU: native (Philox) camera draws against the reference's laws.

The camera is called through the C ABI on frames of constant expectation, so
each pixel is one independent draw; counts are read back exactly (ADC gain
1, offset 0, 32-bit, no read noise unless stated).  Chi-square tests against
the oracle's laws (pinned to the reference's goldens) must not reject at
p = 1e-3:

* Poisson photo-electrons (CCD / CMOS signal, _epifm.py:348-353, :428-433)
  at means that cover the table (integer and fractional parts), its edge at
  256 and the PTRS fallback above it;
* EMCCD output electrons (_epifm.py:365-400) at E = 0.5, 5, 50, 500 and
  1000 e-, against the reference's truncated discrete law (log-shifted so
  that E > 709 e- has a law at all);
* the CMOS read noise (RNDist_F40 table, _epifm.py:332-345).

Then per-pixel mean and variance over many frames against the CMOS model's
moments (mean (E + mean noise) / gain + offset, variance (E + noise
variance) / gain^2).
"""

import numpy
import pytest

import oracle as O

torch = pytest.importorskip("torch")
stats = pytest.importorskip("scipy.stats")

pytestmark = pytest.mark.gpu

N = 1 << 20  # draws per law


@pytest.fixture(scope="module")
def lib():
    from scopyon_gb300 import _build, _lib
    _build.build()
    return _lib


def _draw(lib, kind, photons, *, readout=0.0, emgain=1.0, table=None, counter=3, seed=99,
          offset=0.0, gain=1.0, bit=32):
    from scopyon_gb300._lib import call, ptr, stream_ptr
    dev = torch.device("cuda")
    ph = torch.as_tensor(numpy.asarray(photons, dtype=numpy.float32), device=dev).reshape(-1)
    n = ph.numel()
    cp = lib.CameraParams()
    cp.nw, cp.nh = 1, n
    cp.camera = {"EMCCD": lib.CAM_EMCCD, "CCD": lib.CAM_CCD, "CMOS": lib.CAM_CMOS_TABLE}[kind]
    cp.exact, cp.rounding, cp.bit = 0, 0, bit
    cp.qe, cp.background, cp.readout_noise, cp.emgain = 1.0, 0.0, readout, emgain
    cp.fullwell, cp.offset0, cp.gain0 = 1e12, offset, gain
    cp.seed, cp.counter = seed, counter
    cp.d_poisson_table = lib.poisson_table(dev).data_ptr()
    tv = tc = None
    if table is not None:
        prob = table[:, 1] / table[:, 1].sum()
        cdf = prob.cumsum()
        cdf /= cdf[-1]
        tv = torch.as_tensor(numpy.ascontiguousarray(table[:, 0]), device=dev)
        tc = torch.as_tensor(cdf, device=dev)
        cp.table_n = len(table)
    adc = torch.empty(n, dtype=torch.float64, device=dev)
    status = torch.zeros(lib.STATUS_WORDS, dtype=torch.int32, device=dev)
    call("sc_camera", cp, ptr(ph), None, None, None, None, None, ptr(tv), ptr(tc), None, None,
         None, None, ptr(adc), None, ptr(status), stream_ptr())
    torch.cuda.synchronize()
    assert int(status[0]) == 0, status.cpu().numpy()
    return adc.cpu().numpy()


def _chi2_pvalue(samples, values, probs, min_expected=80.0):
    """Chi-square p-value of integer samples against a discrete law (values
    sorted, probs summing to 1); adjacent values are merged until each bin
    expects at least min_expected samples."""
    n = len(samples)
    cum = numpy.concatenate([[0.0], numpy.cumsum(probs)])
    edges = [0]
    acc = 0.0
    for i, p in enumerate(probs):
        acc += p
        if acc * n >= min_expected:
            edges.append(i + 1)
            acc = 0.0
    if edges[-1] != len(probs):
        edges[-1] = len(probs)
    edges = numpy.array(edges)
    expected = (cum[edges[1:]] - cum[edges[:-1]]) * n
    # sample -> value index -> bin
    vi = numpy.searchsorted(values, samples)
    ok = (vi < len(values)) & (values[numpy.minimum(vi, len(values) - 1)] == samples)
    assert ok.all(), "samples outside the law's support: %s" % samples[~ok][:5]
    b = numpy.searchsorted(edges, vi, side="right") - 1
    observed = numpy.bincount(b, minlength=len(expected))
    chi2 = ((observed - expected) ** 2 / expected).sum()
    return stats.chi2.sf(chi2, len(expected) - 1), len(expected)


@pytest.mark.parametrize("lam", [0.3, 3.7, 17.0, 40.5, 255.25, 256.5, 700.0])
def test_native_poisson_counts(lib, lam):
    k = numpy.rint(_draw(lib, "CCD", numpy.full(N, lam))).astype(numpy.int64)
    hi = int(lam + 12 * numpy.sqrt(lam) + 20)
    values = numpy.arange(hi)
    probs = stats.poisson.pmf(values, lam)
    probs[-1] += stats.poisson.sf(hi - 1, lam)
    assert k.max() < hi
    p, bins = _chi2_pvalue(k, values, probs / probs.sum())
    assert p > 1e-3, (lam, p, bins)


@pytest.mark.parametrize("e", [0.5, 5.0, 50.0, 500.0, 1000.0])
def test_native_emccd_matches_reference_law(lib, e):
    g = 300.0
    s = numpy.rint(_draw(lib, "EMCCD", numpy.full(N, e), emgain=g)).astype(numpy.int64)
    values, probs = O.emccd_distribution(e, int(g))
    p, bins = _chi2_pvalue(s, values, probs)
    assert p > 1e-3, (e, p, bins)


def test_native_cmos_table_noise(lib, golden):
    table = numpy.asarray(golden["cmos_table"])
    noise = _draw(lib, "CMOS", numpy.zeros(N), table=table)
    vals = numpy.unique(table[:, 0].astype(numpy.float32).astype(numpy.float64))
    assert len(vals) == len(table)
    prob = table[:, 1] / table[:, 1].sum()
    order = numpy.argsort(table[:, 0])
    p, bins = _chi2_pvalue(noise, table[order, 0].astype(numpy.float32).astype(numpy.float64),
                           prob[order])
    assert p > 1e-3, (p, bins)


def test_native_cmos_per_pixel_moments(lib, golden):
    """Per-pixel mean and variance over 400 frames of a 64 x 64 frame with
    expectations from 0 to 200 e-, against the CMOS model (table noise plus
    Poisson signal, gain 2.5 e-/ADU, offset 100)."""
    table = numpy.asarray(golden["cmos_table"])
    prob = table[:, 1] / table[:, 1].sum()
    mu_n = (table[:, 0] * prob).sum()
    var_n = ((table[:, 0] - mu_n) ** 2 * prob).sum()
    rng = numpy.random.RandomState(4)
    e = rng.uniform(0.0, 200.0, 64 * 64).astype(numpy.float32)
    gain, offset, frames = 2.5, 100.0, 400
    adc = numpy.array([_draw(lib, "CMOS", e, table=table, counter=f, offset=offset, gain=gain,
                             bit=16) for f in range(frames)])
    m = adc.mean(axis=0)
    v = adc.var(axis=0, ddof=1)
    mean_model = (e + mu_n) / gain + offset
    var_model = (e + var_n) / gain ** 2
    z = (m - mean_model) / numpy.sqrt(var_model / frames)
    assert abs(z.mean()) < 4.0 / numpy.sqrt(z.size)
    assert 0.9 < z.std() < 1.1
    ratio = v / var_model
    assert abs(ratio.mean() - 1.0) < 0.01
