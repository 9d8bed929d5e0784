"""Multi-state sampler (the reference's sampling2.sample).

CPU: the oracle restatement against golden trajectories recorded from the
reference itself (tests/golden/make_sampling2_golden.py), and the host side of
``scopyon_gb300.sample``: initial points, states and the pre-drawn normals and
uniforms of the exact mode, replayed in numpy.  GPU: the exact mode's device
trajectories equal the goldens bit for bit; with Philox draws the state
occupancy relaxes to the chain's stationary distribution; the frame graph's
fused records kernel moves states as sc_diffuse_steps does.
"""

import os

import numpy
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {
    "a": dict(N=[5, 3, 2], lower=-2e-6, upper=2e-6, D=[4e-13, 1e-13, 0.0],
              transmat=[[0.0, 150.0, 0.0], [120.0, 0.0, 30.0], [0.0, 200.0, 0.0]], ndim=2,
              periodic=True, seed=3),
    "b": dict(N=4, lower=[-1e-6, -2e-6, -0.5e-6], upper=[1e-6, 2e-6, 0.5e-6], D=0.2e-12,
              transmat=None, ndim=3, periodic=False, seed=8),
    "c": dict(N=[30, 20], lower=[-3e-6, -3e-6, 0.0], upper=[3e-6, 3e-6, 0.0], D=[1e-12, 5e-14],
              transmat=[[0.0, 800.0], [600.0, 0.0]], ndim=3, periodic=True, seed=21),
}


@pytest.fixture(scope="module")
def golden():
    return numpy.load(os.path.join(HERE, "golden", "sampling2_goldens.npz"))


def _args(name):
    c = dict(CASES[name])
    return c.pop("seed"), c


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference(golden, name):
    seed, c = _args(name)
    out = O.sampling2_sample(golden["s2%s_t" % name], rng=numpy.random.RandomState(seed), **c)
    numpy.testing.assert_array_equal(numpy.array(out), golden["s2%s_pts" % name])


@pytest.mark.parametrize("name", sorted(CASES))
def test_host_draws_replay_the_reference(golden, name):
    """The exact mode's initial points and pre-drawn normals / uniforms,
    applied in numpy in the kernels' order, give the reference's points."""
    from scopyon_gb300 import sampling2
    seed, c = _args(name)
    t = golden["s2%s_t" % name]
    traj = sampling2.sample(t, rng=numpy.random.RandomState(seed), exact=True, **c)
    ndim = traj.ndim
    pos = traj.points0[:, :ndim].copy()
    cls = traj.klass.astype(int).copy()
    ref = golden["s2%s_pts" % name]
    numpy.testing.assert_array_equal(pos, ref[0][:, :ndim])
    numpy.testing.assert_array_equal(cls, ref[0][:, ndim])
    sigma_all = numpy.zeros((len(t) - 1, traj.D.shape[0], 3))
    for g in range(len(t) - 1):
        if t[g + 1] > t[g]:
            sigma_all[g, :, :ndim] = numpy.sqrt(2 * traj.D * (t[g + 1] - t[g]))
    for g in range(len(t) - 1):
        sg = sigma_all[g][cls]
        pos = pos + sg[:, :ndim] * traj.normals[g]
        if traj.boundary == "periodic":
            for d in range(ndim):
                lo, hi = traj.lower[d], traj.upper[d]
                pos[:, d] = (pos[:, d] - lo) % (hi - lo) + lo if hi > lo else lo
        if traj.transmat is not None:
            table = traj._transitions(g, 1)[0]
            cls = numpy.array([min(numpy.searchsorted(table[a], u, side="left"),
                                   table.shape[0] - 1)
                               for a, u in zip(cls, traj.uniforms[g])])
        numpy.testing.assert_array_equal(pos, ref[g + 1][:, :ndim])
        numpy.testing.assert_array_equal(cls, ref[g + 1][:, ndim])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_device_trajectories_match_reference(golden, name):
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import sampling2
    seed, c = _args(name)
    traj = sampling2.sample(golden["s2%s_t" % name], rng=numpy.random.RandomState(seed),
                            exact=True, **c)
    got = numpy.array(list(traj))
    numpy.testing.assert_array_equal(got, golden["s2%s_pts" % name])
    assert len(traj) == len(golden["s2%s_t" % name])
    numpy.testing.assert_array_equal(traj[3], golden["s2%s_pts" % name][3])


@pytest.mark.gpu
def test_philox_states_reach_the_stationary_distribution():
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300 import sampling2
    k01, k10 = 200.0, 300.0  # 1/s
    n, steps, dt = 20000, 400, 1e-3
    traj = sampling2.sample(numpy.arange(steps + 1) * dt, N=[n, 0], lower=-5e-6, upper=5e-6,
                            D=[1e-12, 0.0], transmat=[[0.0, k01], [k10, 0.0]], ndim=2,
                            periodic=True, rng=numpy.random.RandomState(4))
    last = traj[steps]
    frac0 = (last[:, 2] == 0).mean()
    pi0 = k10 / (k01 + k10)
    assert abs(frac0 - pi0) < 0.02, frac0
    # one step from all-in-state-0: about 1 - exp(-k01 dt) switch
    one = traj[1]
    switched = (one[:, 2] == 1).mean()
    assert abs(switched - (1 - numpy.exp(-k01 * dt))) < 0.006, switched
    assert (numpy.abs(last[:, :2]) <= 5e-6).all()  # periodic box


@pytest.mark.gpu
def test_fused_records_move_states_like_the_separate_pass():
    """Frames from the frame graph (states changed inside the records kernel)
    equal frames from generate_images on the same trajectories (states
    changed by sc_diffuse_steps), and so do the final states."""
    from scopyon_gb300 import _build
    _build.build()
    import torch
    import scopyon_gb300 as sg
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "detector": {"type": "EMCCD", "image_size": [40, 40], "exposure_time": 0.004},
        "effects": {"photo_bleaching": {"switch": False}}}})
    t = numpy.arange(4 * 4 + 1) * 1e-3
    traj = sg.sampling2.sample(t, N=[150, 100], lower=[-2.5e-6, -2.5e-6, -0.2e-6],
                               upper=[2.5e-6, 2.5e-6, 0.2e-6], D=[0.8e-12, 0.02e-12],
                               transmat=[[0.0, 400.0], [300.0, 0.0]], ndim=3, periodic=True,
                               rng=numpy.random.RandomState(12))
    eng = EngineConfig(cfg["default"])
    pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
    pipe.psf.ensure(list(range(0, 800)))
    fused_traj = traj.copy()
    fg = FrameGraph(pipe, fused_traj, 4, 1e-3, seed=3, use_graph=False)
    fused = []
    for _ in range(4):
        fg.step()
        fused.append(pipe.expect.cpu().numpy().copy())
    sep_traj = traj.copy()
    sim = sg.EPIFMSimulator(cfg, method="default", rng=numpy.random.RandomState(0))
    sep = [info["expectation"] for _, info in sim.generate_images(sep_traj, 4, full_output=True)]
    for a, b in zip(fused, sep):
        numpy.testing.assert_array_equal(a.reshape(40, 40).astype(float), b)
    numpy.testing.assert_array_equal(fused_traj.classes(), sep_traj.classes())
    assert 0 < (fused_traj.classes() == 1).mean() < 1
