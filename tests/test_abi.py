"""The C ABI library builds for sm_103a, loads, and exports every declared symbol.

No compute call is made here (this runs without a GPU)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fname in os.listdir(os.path.join(ROOT, "include")):
        if fname.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fname)).read()
            names |= set(re.findall(r"^[A-Za-z_][\w \*]*?\b(sc_\w+)\s*\(", text, re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    from scopyon_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 10
    for name in sorted(names):
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from scopyon_gb300 import _lib
    assert set(_lib.declared_symbols()) == _declared()


def test_version_and_error_string(lib):
    lib.sc_get_version.restype = ctypes.c_int
    lib.sc_last_error.restype = ctypes.c_char_p
    assert lib.sc_get_version() >= 1
    assert isinstance(lib.sc_last_error(), bytes)


def test_host_side_validation_needs_no_gpu():
    # argument checks run before any CUDA call and return SC_ERR_ARG
    from scopyon_gb300 import _build, _lib
    _build.build()
    L = _lib.load()
    assert L.sc_psf_radial(0, 5e-7, 1.4, 0.0, None, 0, 1000, 1e-9, None, None) == _lib.SC_ERR_ARG
    assert b"n_keys" in L.sc_last_error()
    p = _lib.SplatParams(nw=64, nh=64, tile=12, halo=14, warps=4, tiles_x=6, tiles_y=6, n_r=1000,
                         sat_pitch=1004, n_images=1, rec_per_image=0, px=1.6e-7, res=1e-9)
    assert L.sc_splat(None, None, None, None, None, ctypes.byref(p), None, 0, None, None,
                      None) == _lib.SC_ERR_ARG
    assert b"tile=12" in L.sc_last_error()
    assert L.sc_bin_workspace_bytes(0, 16) == 0
    # counts, cursors; bins, ranks; long-bin list
    assert L.sc_bin_workspace_bytes(100, 16) == 16 * 16 + 8 * 100 + 4 * (2 * 16 + 1)
    # from 2^20 records on: + the radix sort's values, block digit counts and totals
    n = 1 << 20
    assert L.sc_bin_workspace_bytes(n, 16) == (16 * 16 + 8 * n + 4 * (2 * 16 + 1) + 16 +
                                               4 * (n + 512 * (n // 2048) + 512))
    p.tile, p.tiles_x, p.tiles_y = 16, 4, 4
    assert L.sc_splat_workspace_bytes(ctypes.byref(p)) == 16 * 30 * 30 * 4


def test_struct_sizes_match_c_layout():
    """The ctypes structs have the sizes the C compiler gave the header's."""
    from scopyon_gb300 import _build, _lib
    _build.build()
    out = (ctypes.c_size_t * 6)()
    assert _lib.load().sc_struct_sizes(ctypes.addressof(out), 6) == 0
    assert list(out) == [_lib.STEP_REC_BYTES, ctypes.sizeof(_lib.StepParams),
                         ctypes.sizeof(_lib.SplatParams), ctypes.sizeof(_lib.CameraParams),
                         ctypes.sizeof(_lib.DiffuseParams), ctypes.sizeof(_lib.GaussParams)]


def test_stage_rows_host_helper():
    """sc_stage_rows (host only): copies the rows, returns the depth range,
    flags the first id that differs, and propagates a NaN depth."""
    import numpy
    from scopyon_gb300 import _build, _lib
    _build.build()
    L = _lib.load()
    rng = numpy.random.RandomState(2)
    n = 1000
    a = numpy.column_stack([rng.uniform(-1e-6, 1e-6, (n, 3)), numpy.arange(n, dtype=float),
                            numpy.ones(n)])
    ids = numpy.arange(n, dtype=float)
    dst = numpy.zeros((n, 5))
    out = numpy.zeros(2)
    assert L.sc_stage_rows(a.ctypes.data, n, ids.ctypes.data, dst.ctypes.data, out.ctypes.data) == 0
    numpy.testing.assert_array_equal(dst, a)
    assert (out[0], out[1]) == (a[:, 0].min(), a[:, 0].max())
    b = a.copy()
    b[700, 3] = 5.0
    assert L.sc_stage_rows(b.ctypes.data, n, ids.ctypes.data, dst.ctypes.data, out.ctypes.data) == 1
    b = a.copy()
    b[3, 0] = numpy.nan
    assert L.sc_stage_rows(b.ctypes.data, n, ids.ctypes.data, dst.ctypes.data, out.ctypes.data) == 0
    assert numpy.isnan(out).all()
    assert L.sc_stage_rows(None, n, ids.ctypes.data, dst.ctypes.data, out.ctypes.data) == \
        _lib.SC_ERR_ARG


def test_stage_known_matches_numpy():
    """The host fast path's staging: native rows for row-major float64
    arrays, numpy for the rest, the same staging and range either way."""
    import numpy
    from scopyon_gb300 import _build
    _build.build()
    from scopyon_gb300.base import _stage_known
    rng = numpy.random.RandomState(5)
    n, S = 500, 6
    ids = numpy.arange(n, dtype=float)
    arrays = [numpy.column_stack([rng.uniform(-2e-6, 2e-6, (n, 3)), ids, numpy.ones(n)])
              for _ in range(S)]
    arrays[2] = numpy.asfortranarray(arrays[2])  # takes the numpy form
    staging = numpy.zeros((S, n, 5))
    rng_ = _stage_known(arrays, ids, staging)
    numpy.testing.assert_array_equal(staging, numpy.stack(arrays))
    allz = numpy.concatenate([a[:, 0] for a in arrays])
    assert rng_ == (allz.min(), allz.max())
    arrays[4] = arrays[4].copy()
    arrays[4][10, 3] = -1.0
    assert _stage_known(arrays, ids, staging) is None


def test_undersized_workspace_is_a_capacity_error():
    """A caller workspace smaller than the call needs: SC_ERR_CAPACITY, found
    before anything is launched (the pointers are never dereferenced)."""
    from scopyon_gb300 import _build, _lib
    _build.build()
    L = _lib.load()
    P = ctypes.c_void_p
    fake = P(1 << 20)  # non-NULL, never dereferenced: validation fails first
    p = _lib.SplatParams(nw=64, nh=64, tile=8, halo=14, warps=4, tiles_x=8, tiles_y=8, n_r=1000,
                         sat_pitch=1004, n_images=1, rec_per_image=0, px=1.6e-7, res=1e-9)
    need = L.sc_bin_workspace_bytes(1000, 64)
    rc = L.sc_bin_steps(fake, 1000, ctypes.byref(p), fake, 16, fake, fake, None, None)
    assert rc == _lib.SC_ERR_CAPACITY
    assert b"workspace" in L.sc_last_error()
    rc = L.sc_bin_finish(1000, ctypes.byref(p), fake, need - 4, fake, fake, None)
    assert rc == _lib.SC_ERR_CAPACITY
    rc = L.sc_splat(fake, fake, fake, fake, None, ctypes.byref(p), fake,
                    L.sc_splat_workspace_bytes(ctypes.byref(p)) - 4, fake, None, None)
    assert rc == _lib.SC_ERR_CAPACITY
    with pytest.raises(_lib.ScopyonGPUError) as err:
        _lib.call("sc_splat", fake, fake, fake, fake, None, ctypes.byref(p), fake, 0, fake,
                  None, None)
    assert err.value.code == _lib.SC_ERR_CAPACITY


def test_layout_and_kernel_choices_are_checked_on_the_host():
    """Row layouts, the box-kernel choice and the L2 fetch hint are checked
    before any CUDA call: SC_ERR_ARG with a message (pointers never read)."""
    from scopyon_gb300 import _build, _lib
    _build.build()
    L = _lib.load()
    P = ctypes.c_void_p
    fake = P(1 << 20)
    d = _lib.DiffuseParams(n_particles=100, n_sub=4, ndim=3, boundary=0, n_class=1, layout=7,
                           scale=1.0)
    d.unit_x[0] = d.unit_y[1] = d.unit_z[2] = 1.0
    assert L.sc_diffuse_steps(ctypes.byref(d), fake, None, fake, None, fake, None) == _lib.SC_ERR_ARG
    assert b"layout=7" in L.sc_last_error()
    # FP32 rows need native draws: with the caller's normals they are refused
    d.layout = 1
    assert L.sc_diffuse_steps(ctypes.byref(d), fake, None, fake, fake, fake, None) == _lib.SC_ERR_ARG
    assert b"layout 1" in L.sc_last_error()
    # ... and the identity transform
    d.scale = 2.0
    assert L.sc_diffuse_steps(ctypes.byref(d), fake, None, fake, None, fake, None) == _lib.SC_ERR_ARG
    s = _lib.StepParams(px=1.6e-7, res=1e-9, depth_cutoff=1e-6, nw=64, nh=64, n_signal=1999,
                        n_sub=4, n_particles=100, max_key=1000, row_layout=3)
    assert L.sc_emitter_steps(ctypes.byref(s), fake, fake, None, fake, None, None, fake, None,
                              None, None) == _lib.SC_ERR_ARG
    assert b"row_layout=3" in L.sc_last_error()
    p = _lib.SplatParams(nw=64, nh=64, tile=8, halo=14, warps=4, tiles_x=8, tiles_y=8, n_r=1000,
                         sat_pitch=1004, n_images=1, rec_per_image=0, box_kernel=2, px=1.6e-7,
                         res=1e-9)
    assert L.sc_splat(fake, fake, fake, fake, None, ctypes.byref(p), fake,
                      L.sc_splat_workspace_bytes(ctypes.byref(p)), fake, None,
                      None) == _lib.SC_ERR_ARG
    assert b"box_kernel=2" in L.sc_last_error()
    assert L.sc_set_l2_fetch_granularity(17) == _lib.SC_ERR_ARG
    assert b"17 bytes" in L.sc_last_error()
    assert L.sc_box_block_floats(14) == 196 and L.sc_box_block_floats(13) == 172


def test_merge_camera_checks_on_the_host():
    """sc_merge_camera refuses, before any CUDA call, the cases it does not
    take: injected draws, several images per call, a camera of another size,
    no Poisson tables, an undersized workspace."""
    from scopyon_gb300 import _build, _lib
    _build.build()
    L = _lib.load()
    P = ctypes.c_void_p
    fake = P(1 << 20)
    sp = _lib.SplatParams(nw=64, nh=64, tile=8, halo=14, warps=4, tiles_x=8, tiles_y=8, n_r=1000,
                          sat_pitch=1004, n_images=1, rec_per_image=0, px=1.6e-7, res=1e-9)
    ws = L.sc_splat_workspace_bytes(ctypes.byref(sp))
    cp = _lib.CameraParams(nw=64, nh=64, camera=_lib.CAM_SCMOS, exact=1, bit=12, qe=0.7,
                           fullwell=30000.0, offset0=100.0, gain0=7.5)
    cp.d_poisson_table = 1 << 20

    def call(cp_, sp_, ws_bytes):
        return L.sc_merge_camera(ctypes.byref(sp_), fake, ctypes.c_size_t(ws_bytes),
                                 ctypes.byref(cp_), None, None, None, None, None, None, fake,
                                 None, None)

    assert call(cp, sp, ws) == _lib.SC_ERR_ARG and b"native" in L.sc_last_error()
    cp.exact = 0
    cp.nh = 32
    assert call(cp, sp, ws) == _lib.SC_ERR_ARG and b"camera 64x32" in L.sc_last_error()
    cp.nh = 64
    cp.d_poisson_table = None
    assert call(cp, sp, ws) == _lib.SC_ERR_ARG and b"Poisson" in L.sc_last_error()
    cp.d_poisson_table = 1 << 20
    assert call(cp, sp, ws - 4) == _lib.SC_ERR_CAPACITY
    sp.n_images = 2
    assert call(cp, sp, 2 * ws) == _lib.SC_ERR_ARG and b"one image" in L.sc_last_error()
