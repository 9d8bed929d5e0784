"""GPU parity at the benchmark configurations' own shapes.

The CUDA path, driven through the public API (``generate_images`` with host
trajectories), against the vectorised FP64 oracle (oracle/frames.py, pinned
to the reference's frames) on the same inputs.

Each case runs twice on the GPU:
* native mode (Philox camera draws; bleaching times injected): the production
  FP32 path (box tables, tile bins, splat).  Expected photons within 1e-5
  relative per pixel for pixels above 1e-6 of the image maximum, and within
  1e-6 norm-wise (sum |e - e_ref| / sum e_ref);
* injected-draws mode: the parity path, expected photons accumulated in FP64
  (within 1e-10 per pixel above the same floor, 1e-11 norm-wise), then the
  camera on the caller's draws.  ADC: CMOS exact up to FP64 rounding (1e-9
  of the largest count); EMCCD, whose inverse-CDF draw runs on each side's
  own expectation, at most max(1, 1e-4 * pixels) pixels differ, each by at
  most 1 ADU.
true_data: rtol 1e-12; bleaching budgets: rtol 1e-12.
"""

import multiprocessing
import os

import numpy
import pytest

import oracle as O
from oracle import frames as F
import full_shape_cases as C

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

WORKERS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def pool():
    # spawned workers: the test process already holds a CUDA context
    with multiprocessing.get_context("spawn").Pool(WORKERS) as p:
        yield p


@pytest.fixture(scope="module")
def lib():
    from scopyon_gb300 import _build, _lib
    _build.build()
    return _lib


def _check_expectation(e, e_ref, exact):
    per_pixel, norm = C.expectation_errors(e, e_ref)
    assert per_pixel <= (1e-10 if exact else 1e-5), per_pixel
    assert norm <= (1e-11 if exact else 1e-6), norm
    return per_pixel, norm


def _check_adc(adc, adc_ref, emccd):
    diff = numpy.abs(adc - adc_ref)
    if emccd:
        bad = diff > 1e-9
        assert bad.sum() <= max(1, int(1e-4 * diff.size)), bad.sum()
        assert diff.max() <= 1.0, diff.max()
    else:
        assert diff.max() <= 1e-9 * max(1.0, adc_ref.max()), diff.max()


def _check_info(info, oinfo, bleaching):
    ids = list(oinfo["true_data"])
    got = numpy.array([info["true_data"][m] for m in ids])
    ref = numpy.array([oinfo["true_data"][m] for m in ids])
    numpy.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300)
    if bleaching:
        st = numpy.array([info["fluorescence_states"][m] for m in ids])
        st_ref = numpy.array([oinfo["fluorescence_states"][m] for m in ids])
        numpy.testing.assert_allclose(st, st_ref, rtol=1e-12, atol=0)


def test_config1_tirf_emccd_160px_1000_emitters(lib, pool):
    """Two frames: 1,000 emitters, 10 sub-steps of 3 ms, 100 photons/emitter/ms,
    EMCCD whose brightest pixels pass 709 e- (the exact draws run above it)."""
    import scopyon_gb300 as sg
    n_frames = 2
    cfg = C.config1()
    params = C.oracle_params(cfg)
    inputs = C.inputs1(n_frames)
    data = [(t, O.format_data(p)) for t, p in inputs]
    rng = numpy.random.RandomState(5)
    shape = (C.CFG1["edge"],) * 2
    frames = [{"noise": rng.normal(0, 100, shape), "uniform": rng.random_sample(shape)}
              for _ in range(n_frames)]
    exact = list(sg.generate_images(inputs, n_frames, config=cfg,
                                    rng=numpy.random.RandomState(1), full_output=True,
                                    device="cuda:0",
                                    draws=sg.InjectedDraws(frames=[dict(f) for f in frames])))
    native = list(sg.generate_images(inputs, n_frames, config=cfg,
                                     rng=numpy.random.RandomState(1), full_output=True,
                                     device="cuda:0"))
    peak = 0.0
    for f in range(n_frames):
        cam, oinfo = F.output_frame_fast(params, data, None, f, camera=False, pool=pool,
                                         workers=WORKERS)
        e_ref = cam[:, :, 0]
        peak = max(peak, e_ref.max())
        signal = C.emccd_signal(e_ref, params.emgain, frames[f]["uniform"], pool, WORKERS)
        adc_ref = O.adc_counts(signal + frames[f]["noise"], params.fullwell, params.gain,
                               params.offset, params.bit)
        img, info = exact[f]
        _check_expectation(info["expectation"], e_ref, exact=True)
        _check_adc(img.as_array(), adc_ref, emccd=True)
        _check_info(info, oinfo, bleaching=False)
        _, ninfo = native[f]
        _check_expectation(ninfo["expectation"], e_ref, exact=False)
        _check_info(ninfo, oinfo, bleaching=False)
    assert peak > 709.0  # the reference's EMCCD law would have overflowed here


def _config2_case(pool, n, n_frames, table, seed):
    import scopyon_gb300 as sg
    cfg = C.config2(table)
    params = C.oracle_params(cfg, rng=numpy.random.RandomState(seed), cmos_table=table)
    inputs = C.inputs2(n_frames, n=n)
    data = [(t, O.format_data(p)) for t, p in inputs]
    rng = numpy.random.RandomState(seed + 1)
    bleach = dict(zip(range(n), rng.exponential(2.0, n)))
    states = {}
    shape = (C.CFG2["edge"],) * 2
    refs, frames = [], []
    for f in range(n_frames):
        cam, oinfo = F.output_frame_fast(params, data, O.InjectedDraws(bleach, []), f,
                                         states=states, camera=False, pool=pool, workers=WORKERS)
        e_ref = cam[:, :, 0]
        u = rng.random_sample(shape)
        signal = rng.poisson(e_ref).astype(float)
        adc_ref = O.adc_counts(signal + O.cmos_table_draw(table, u), params.fullwell,
                               params.gain, params.offset, params.bit)
        refs.append((e_ref, adc_ref, oinfo))
        frames.append({"uniform": u, "signal": signal})
    exact = sg.generate_images(inputs, n_frames, config=cfg, rng=numpy.random.RandomState(seed),
                               full_output=True, device="cuda:0",
                               draws=sg.InjectedDraws(bleach=bleach, frames=frames))
    for f, (img, info) in enumerate(exact):
        e_ref, adc_ref, oinfo = refs[f]
        _check_expectation(info["expectation"], e_ref, exact=True)
        _check_adc(img.as_array(), adc_ref, emccd=False)
        _check_info(info, oinfo, bleaching=True)
    # native mode: Philox camera, the bleaching times injected
    native = sg.generate_images(inputs, n_frames, config=cfg, rng=numpy.random.RandomState(seed),
                                full_output=True, device="cuda:0",
                                draws=sg.InjectedDraws(bleach=bleach))
    out = []
    for f, (img, info) in enumerate(native):
        e_ref, _, oinfo = refs[f]
        out.append(_check_expectation(info["expectation"], e_ref, exact=False))
        _check_info(info, oinfo, bleaching=True)
    return out


def test_config2_epi_defocus_cmos_512px_20k_emitters(lib, pool, golden):
    """Two frames at 512^2 px: 20,000 emitters in +-1 um of depth (about 1,000
    depth keys on the box-table path), 20 sub-steps, bleaching carried over."""
    _config2_case(pool, C.CFG2["n"], 2, golden["cmos_table"], seed=31)


def test_dense_frame_radix_binning_60k_emitters(lib, pool, golden):
    """One frame of 60,000 emitters x 20 sub-steps: 1.2M records, so the tile
    lists are ordered by the radix sort, with bins of thousands of records."""
    _config2_case(pool, 60000, 1, golden["cmos_table"], seed=47)
