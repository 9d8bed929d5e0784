"""GPU: sc_bin_steps_static, the binning entry point with fixed scratch.

Called through the C ABI and compared with sc_bin_steps (caller workspace)
and with a numpy restatement of the sort, on two calls in a row with
different records, so that counts left over from the first call would show.
"""

import ctypes

import numpy
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

REC = numpy.dtype([("box_off", "<i8"), ("i_start", "<i2"), ("n_i", "<i2"), ("j_start", "<i2"),
                   ("n_j", "<i2"), ("w", "<f4"), ("slot", "<i4"), ("box", "<i4"), ("box_local", "<i4"),
                   ("x0", "<f8"), ("y0", "<f8"), ("ax_hi", "<f4"), ("ax_lo", "<f4"),
                   ("ay_hi", "<f4"), ("ay_lo", "<f4")])


@pytest.fixture(scope="module")
def lib():
    from scopyon_gb300 import _build, _lib
    _build.build()
    assert REC.itemsize == _lib.STEP_REC_BYTES
    return _lib


def params(lib, nw, nh, tile=8, n_images=1, rec_per_image=0):
    p = lib.SplatParams()
    p.nw, p.nh, p.tile, p.halo, p.warps = nw, nh, tile, 14, 4
    p.tiles_x, p.tiles_y = -(-nw // tile), -(-nh // tile)
    p.n_images, p.rec_per_image = n_images, rec_per_image
    return p


def random_records(rng, n, nw, nh, negative=False):
    """Records spread over the image; some past its edge (no bin), and with
    ``negative`` some with a negative first pixel (no bin, status bit 6)."""
    r = numpy.zeros(n, REC)
    lo = -20 if negative else 0
    r["i_start"] = rng.randint(lo, nw + 4, n)  # past the image: no bin
    r["j_start"] = rng.randint(lo, nh + 4, n)
    r["n_i"] = rng.randint(0, 30, n)  # fewer than 2 pixels: no bin
    r["n_j"] = rng.randint(0, 30, n)
    r["slot"] = numpy.where(rng.rand(n) < 0.05, -1, 0)
    r["box"] = rng.randint(0, 2, n)
    return r


def numpy_bins(r, p):
    """Bin of each record and the stable order by bin (the kernels' result)."""
    idx = numpy.arange(len(r))
    img = idx // p.rec_per_image if p.rec_per_image > 0 else numpy.zeros(len(r), int)
    n_tiles = p.tiles_x * p.tiles_y * p.n_images
    ok = ((r["n_i"] >= 2) & (r["n_j"] >= 2) & (r["slot"] >= 0) & (img < p.n_images)
          & (r["i_start"] >= 0) & (r["j_start"] >= 0)
          & (r["i_start"] < p.nw) & (r["j_start"] < p.nh))
    i0, j0 = r["i_start"].astype(numpy.int64), r["j_start"].astype(numpy.int64)
    t = img * p.tiles_x * p.tiles_y + (i0 // p.tile) * p.tiles_y + j0 // p.tile
    b = numpy.where(r["box"] != 0, t, t + n_tiles)
    b = numpy.where(ok, b, -1)
    counts = numpy.bincount(b[ok], minlength=2 * n_tiles)
    start = numpy.concatenate([[0], numpy.cumsum(counts)]).astype(numpy.int32)
    order = idx[ok][numpy.argsort(b[ok], kind="stable")].astype(numpy.int32)
    return start, order


def malformed(r):
    """Records the counting pass reports: pixels to splat, negative first pixel."""
    return ((r["n_i"] >= 2) & (r["n_j"] >= 2) & (r["slot"] >= 0)
            & ((r["i_start"] < 0) | (r["j_start"] < 0)))


def run(lib, fn, recs_h, p, counts_only=False):
    L = lib.load()
    n = len(recs_h)
    n_tiles = p.tiles_x * p.tiles_y * p.n_images
    recs = torch.from_numpy(recs_h.view(numpy.int32).copy()).cuda()
    start = torch.full((2 * n_tiles + 1,), -7, dtype=torch.int32, device="cuda")
    items = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    status = torch.zeros(4, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = ctypes.c_void_p
    if fn == "static":
        rc = L.sc_bin_steps_static(P(recs.data_ptr()), n, ctypes.byref(p), P(start.data_ptr()),
                                   P(items.data_ptr()), P(status.data_ptr()), s)
    else:
        ws_bytes = 16 * n_tiles if counts_only else L.sc_bin_workspace_bytes(n, n_tiles)
        ws = torch.empty((ws_bytes + 3) // 4, dtype=torch.int32, device="cuda")
        rc = L.sc_bin_steps(P(recs.data_ptr()), n, ctypes.byref(p), P(ws.data_ptr()), ws_bytes,
                            P(start.data_ptr()), P(items.data_ptr()), P(status.data_ptr()), s)
    assert rc == 0, L.sc_last_error().decode()
    torch.cuda.synchronize()
    start = start.cpu().numpy()
    st = status.cpu().numpy()
    bad = malformed(recs_h)
    assert bool(st[0] & 64) == bool(bad.any()), st
    if bad.any():
        assert bad[st[1]], st  # the flagged record is one of the malformed ones
    return start, items.cpu().numpy()[:start[-1]]


@pytest.mark.parametrize("shape", [(512, 512, 1), (96, 64, 2), (16, 16, 1)])
def test_static_matches_workspace_entry_point(lib, shape):
    nw, nh, n_images = shape
    rng = numpy.random.RandomState(11)
    for call in range(2):
        n = 20000 + 3001 * call
        rpi = -(-n // n_images) if n_images > 1 else 0
        p = params(lib, nw, nh, n_images=n_images, rec_per_image=rpi)
        r = random_records(rng, n, nw, nh, negative=call == 1)
        s_start, s_items = run(lib, "static", r, p)
        w_start, w_items = run(lib, "workspace", r, p)
        numpy.testing.assert_array_equal(s_start, w_start)
        numpy.testing.assert_array_equal(s_items, w_items)
        c_start, c_items = run(lib, "workspace", r, p, counts_only=True)
        numpy.testing.assert_array_equal(c_start, w_start)
        numpy.testing.assert_array_equal(c_items, w_items)
        e_start, e_items = numpy_bins(r, p)
        numpy.testing.assert_array_equal(s_start, e_start)
        numpy.testing.assert_array_equal(s_items, e_items)


def test_static_counts_only_fallback(lib):
    """With more records than the fixed array has room for (bins and ranks
    of every record), sc_bin_steps_static takes the counts-only path: atomic
    cursors, then a sort of each bin.  Same lists as the workspace path and
    numpy, two calls in a row."""
    L = lib.load()
    rng = numpy.random.RandomState(23)
    p = params(lib, 512, 512)
    n_tiles = p.tiles_x * p.tiles_y
    for call in range(2):
        n = 300000 + 17 * call
        assert L.sc_bin_workspace_bytes(n, n_tiles) > 1 << 20  # beyond the fixed array
        r = random_records(rng, n, 512, 512, negative=call == 0)
        s_start, s_items = run(lib, "static", r, p)
        e_start, e_items = numpy_bins(r, p)
        numpy.testing.assert_array_equal(s_start, e_start)
        numpy.testing.assert_array_equal(s_items, e_items)
        w_start, w_items = run(lib, "workspace", r, p)
        numpy.testing.assert_array_equal(s_items, w_items)


@pytest.mark.parametrize("shape", [(4096, 2048, 1), (256, 256, 1), (1024, 512, 3)])
def test_radix_path_matches_sort_path(lib, shape):
    """From 2^20 records on, sc_bin_steps orders the lists with a radix sort:
    the same start offsets and lists as the sort path and numpy, with 2 and 3
    digit passes, dense bins (over 700 records each) and records in no bin."""
    nw, nh, n_images = shape
    rng = numpy.random.RandomState(5)
    n = 1500000 + 77
    rpi = -(-n // n_images) if n_images > 1 else 0
    p = params(lib, nw, nh, n_images=n_images, rec_per_image=rpi)
    r = random_records(rng, n, nw, nh)
    w_start, w_items = run(lib, "workspace", r, p)
    e_start, e_items = numpy_bins(r, p)
    numpy.testing.assert_array_equal(w_start, e_start)
    numpy.testing.assert_array_equal(w_items, e_items)
    c_start, c_items = run(lib, "workspace", r, p, counts_only=True)
    numpy.testing.assert_array_equal(c_items, w_items)


def test_static_rejects_too_many_tiles(lib):
    L = lib.load()
    p = params(lib, 4096, 4096)  # 512 x 512 tiles > SC_BIN_STATIC_MAX_TILES
    rc = L.sc_bin_steps_static(None, 10, ctypes.byref(p), None, None, None, None)
    assert rc == -1
    assert "fixed scratch" in L.sc_last_error().decode()
