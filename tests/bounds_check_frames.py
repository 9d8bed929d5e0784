"""Frames for the bounds-checked build's test, in a child process.

``tests/test_gpu_bounds_check.py`` runs this script twice, once with the
normal library and once with the one built with ``-DSC_BOUNDS_CHECK``
(chosen by ``SCOPYON_GB300_LIB``), and compares the arrays it writes:

- frames of device trajectories through the frame graph's kernels, with the
  bulk-copy ring and with the register splat (8x8 and 16x16 tiles), merged
  inside the camera pass;
- frames of host trajectories through ``generate_images`` (binning with
  ranks, the graph replays of host-row frames);
- bins of random records counted without rank storage (atomic cursors).

Any status bit a frame sets raises, so a check that fires fails the run.

usage: python tests/bounds_check_frames.py OUT.npz
"""

import os
import sys

import numpy

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def device_frames(sg, out):
    import torch
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {"magnification": 100,
                            "detector": {"type": "EMCCD", "image_size": [200, 136],
                                         "exposure_time": 0.004},
                            "light_source": {"angle": 0.0}}})
    t = numpy.arange(4 * 4 + 1) * 1e-3
    # emitters past the field's edges too (clipped footprints); reflecting
    # walls keep the depths within the keys built below
    traj = sg.sample_inputs(t, N=3000, lower=[-17e-6, -12e-6, -0.3e-6],
                            upper=[17e-6, 12e-6, 0.3e-6], D=0.4e-12, ndim=3,
                            rng=numpy.random.RandomState(12), boundary="reflecting")
    eng = EngineConfig(cfg["default"])
    for tile, warps, stages in ((8, 4, 4), (8, 4, 0), (16, 8, 4), (16, 8, 0)):
        pipe = FramePipeline(eng, "cuda", psf=_psf_for(eng, torch.device("cuda")))
        pipe.psf.ensure(list(range(0, 400)))
        pipe.set_tiles(tile, warps, stages)
        fg = FrameGraph(pipe, traj.copy(), 4, 1e-3, seed=3, use_graph=False)
        frames = []
        for _ in range(3):
            fg.step()
            frames.append(numpy.stack([pipe.expect.cpu().numpy(), pipe.adc32.cpu().numpy()]))
        pipe.check_status()
        out["device_%d_%d_%d" % (tile, warps, stages)] = numpy.array(frames)


def host_frames(sg, out):
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {"magnification": 100,
                            "detector": {"type": "EMCCD", "image_size": [64, 48],
                                         "exposure_time": 0.004}}})
    rng = numpy.random.RandomState(4)
    n = 400
    ids = numpy.arange(n, dtype=float)
    inputs = []
    for k in range(5 * 4 + 1):
        xyz = numpy.column_stack([rng.uniform(-5e-6, 5e-6, n), rng.uniform(-4e-6, 4e-6, n),
                                  rng.uniform(-0.3e-6, 0.3e-6, n)])
        inputs.append((k * 1e-3, numpy.hstack([xyz, ids[:, None], numpy.ones((n, 1))])))
    gen = sg.generate_images(inputs, 5, config=cfg, rng=numpy.random.RandomState(5))
    out["host"] = numpy.array([img.as_array() for img in gen])


def cursor_bins(out):
    """sc_bin_steps with a workspace for the counts only: records placed by
    atomic cursors, then each list sorted."""
    import ctypes
    import torch
    from scopyon_gb300 import _lib
    rng = numpy.random.RandomState(6)
    n, nw, nh, tile = 50000, 256, 192, 8
    rec = numpy.zeros(n, dtype=[("box_off", "<i8"), ("i_start", "<i2"), ("n_i", "<i2"),
                                ("j_start", "<i2"), ("n_j", "<i2"), ("w", "<f4"), ("slot", "<i4"),
                                ("box", "<i4"), ("box_local", "<i4"), ("rest", "V32")])
    rec["i_start"] = rng.randint(0, nw, n)
    rec["j_start"] = rng.randint(0, nh, n)
    rec["n_i"] = rng.randint(0, 15, n)
    rec["n_j"] = rng.randint(0, 15, n)
    rec["slot"] = rng.randint(-1, 4, n)
    rec["box"] = rng.randint(0, 3, n)
    assert rec.dtype.itemsize == _lib.STEP_REC_BYTES
    p = _lib.SplatParams()
    p.nw, p.nh, p.tile, p.halo, p.warps = nw, nh, tile, 14, 4
    p.tiles_x, p.tiles_y = nw // tile, nh // tile
    p.n_images = 1
    n_tiles = p.tiles_x * p.tiles_y
    dev = torch.device("cuda")
    d_rec = torch.from_numpy(rec.view(numpy.uint8)).to(dev)
    ws = torch.zeros(4 * n_tiles, dtype=torch.int32, device=dev)
    tile_start = torch.empty(2 * n_tiles + 1, dtype=torch.int32, device=dev)
    items = torch.empty(n, dtype=torch.int32, device=dev)
    status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
    _lib.call("sc_bin_steps", _lib.ptr(d_rec), n, ctypes.byref(p), _lib.ptr(ws), 16 * n_tiles,
              _lib.ptr(tile_start), _lib.ptr(items), _lib.ptr(status), _lib.stream_ptr())
    torch.cuda.synchronize()
    assert int(status[0]) == 0, status.cpu().numpy()
    ts = tile_start.cpu().numpy()
    out["cursor_tile_start"] = ts
    out["cursor_items"] = items.cpu().numpy()[: ts[-1]]


def main(path):
    import scopyon_gb300 as sg
    out = {}
    device_frames(sg, out)
    host_frames(sg, out)
    cursor_bins(out)
    numpy.savez(path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
