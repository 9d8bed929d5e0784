"""ctypes binding of ``libscopyon_gb300.so`` (declarations in include/scopyon_gb300.h).

The library is the only compute path: if it is missing this module raises on
first use; there is no CPU fallback.
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SCOPYON_GB300_LIB") or os.path.join(HERE, "libscopyon_gb300.so")

SC_OK, SC_ERR_ARG, SC_ERR_CUDA, SC_ERR_TIMEOUT, SC_ERR_NAN, SC_ERR_CAPACITY = 0, -1, -2, -3, -4, -5
PSF_BORN_WOLF, PSF_GAUSSIAN = 0, 1
CAM_EMCCD, CAM_CCD, CAM_CMOS_TABLE, CAM_SCMOS = 0, 1, 2, 3
STEP_REC_BYTES = 64
STATUS_WORDS = 4

c_double_p = ctypes.c_void_p  # device pointers travel as integers


class StepParams(ctypes.Structure):
    _fields_ = [("px", ctypes.c_double), ("res", ctypes.c_double),
                ("depth_cutoff", ctypes.c_double), ("focal", ctypes.c_double * 3),
                ("nw", ctypes.c_int32), ("nh", ctypes.c_int32), ("n_signal", ctypes.c_int32),
                ("n_sub", ctypes.c_int32), ("n_particles", ctypes.c_int32),
                ("max_key", ctypes.c_int32),
                ("amplitude0", ctypes.c_double), ("penetration", ctypes.c_double),
                ("x_sec", ctypes.c_double), ("qy", ctypes.c_double), ("beer", ctypes.c_double),
                ("norm_coeff", ctypes.c_double),
                ("bleaching", ctypes.c_int32), ("with_optinfo", ctypes.c_int32),
                ("box_p", ctypes.c_int32), ("box_nq", ctypes.c_int32),
                ("row_layout", ctypes.c_int32), ("pad", ctypes.c_int32)]


class SplatParams(ctypes.Structure):
    _fields_ = [("nw", ctypes.c_int32), ("nh", ctypes.c_int32), ("tile", ctypes.c_int32),
                ("halo", ctypes.c_int32), ("warps", ctypes.c_int32),
                ("tiles_x", ctypes.c_int32), ("tiles_y", ctypes.c_int32),
                ("n_r", ctypes.c_int32), ("sat_pitch", ctypes.c_int32),
                ("n_images", ctypes.c_int32), ("rec_per_image", ctypes.c_int32),
                ("box_p", ctypes.c_int32), ("box_nq", ctypes.c_int32),
                ("n_slots", ctypes.c_int32), ("box_stages", ctypes.c_int32),
                ("first_wait_polls", ctypes.c_int32), ("box_kernel", ctypes.c_int32),
                ("pad", ctypes.c_int32),
                ("px", ctypes.c_double), ("res", ctypes.c_double)]


class CameraParams(ctypes.Structure):
    _fields_ = [("nw", ctypes.c_int32), ("nh", ctypes.c_int32), ("camera", ctypes.c_int32),
                ("exact", ctypes.c_int32), ("rounding", ctypes.c_int32), ("bit", ctypes.c_int32),
                ("qe", ctypes.c_double), ("background", ctypes.c_double),
                ("readout_noise", ctypes.c_double), ("emgain", ctypes.c_double),
                ("fullwell", ctypes.c_double), ("offset0", ctypes.c_double),
                ("gain0", ctypes.c_double), ("table_n", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("counter", ctypes.c_uint64),
                ("d_frame", ctypes.c_void_p), ("d_photons64", ctypes.c_void_p),
                ("d_expect64", ctypes.c_void_p), ("d_poisson_table", ctypes.c_void_p)]


class BatchPlan(ctypes.Structure):
    _fields_ = [("d_work", ctypes.c_void_p), ("d_tile_field_off", ctypes.c_void_p),
                ("d_tile_field", ctypes.c_void_p), ("d_field", ctypes.c_void_p),
                ("d_chunk", ctypes.c_void_p), ("d_counters", ctypes.c_void_p),
                ("n_work", ctypes.c_int32), ("n_fields", ctypes.c_int32),
                ("n_chunks", ctypes.c_int32), ("chunk_pixels", ctypes.c_int32),
                ("spin_limit", ctypes.c_int32), ("target_extra", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("pad", ctypes.c_int32)]


class BWParams(ctypes.Structure):
    _fields_ = [("nw", ctypes.c_int32), ("nh", ctypes.c_int32), ("n_frames", ctypes.c_int32),
                ("n_emit", ctypes.c_int32), ("n_r", ctypes.c_int32), ("sat_pitch", ctypes.c_int32),
                ("key_hi", ctypes.c_int32), ("pad", ctypes.c_int32), ("px", ctypes.c_double),
                ("res", ctypes.c_double), ("inv_pen", ctypes.c_double),
                ("z_focal", ctypes.c_double), ("cnorm", ctypes.c_double),
                ("d_key_slot", ctypes.c_void_p)]


class DiffuseParams(ctypes.Structure):
    _fields_ = [("n_particles", ctypes.c_int32), ("n_sub", ctypes.c_int32),
                ("ndim", ctypes.c_int32), ("boundary", ctypes.c_int32),
                ("n_class", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("step0", ctypes.c_int64), ("seed", ctypes.c_uint64), ("d_frame", ctypes.c_void_p),
                ("lower", ctypes.c_double * 3), ("upper", ctypes.c_double * 3),
                ("scale", ctypes.c_double), ("origin", ctypes.c_double * 3),
                ("unit_x", ctypes.c_double * 3), ("unit_y", ctypes.c_double * 3),
                ("unit_z", ctypes.c_double * 3), ("d_class_box", ctypes.c_void_p),
                ("d_trans", ctypes.c_void_p), ("d_uniforms", ctypes.c_void_p)]


class GaussParams(ctypes.Structure):
    _fields_ = [("nw", ctypes.c_int32), ("nh", ctypes.c_int32), ("n_frames", ctypes.c_int32),
                ("n_emit", ctypes.c_int32), ("half_win", ctypes.c_int32), ("tile", ctypes.c_int32),
                ("px", ctypes.c_double), ("inv_pen", ctypes.c_double), ("z_focal", ctypes.c_double)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_SIG = {
    "sc_get_version": (_I, []),
    "sc_box_block_floats": (_I, [_I]),
    "sc_set_l2_fetch_granularity": (_I, [_I]),
    "sc_copy_async": (_I, [_P, _P, ctypes.c_size_t, _P]),
    "sc_struct_sizes": (_I, [_P, _I]),
    "sc_counter_add": (_I, [_P, ctypes.c_int64, _P]),
    "sc_stage_rows": (_I, [_P, ctypes.c_int64, _P, _P, _P]),
    "sc_last_error": (ctypes.c_char_p, []),
    "sc_psf_radial": (_I, [_I, _D, _D, _D, _P, _I, _I, _D, _P, _P]),
    "sc_diffuse_steps": (_I, [ctypes.POINTER(DiffuseParams), _P, _P, _P, _P, _P, _P]),
    "sc_native_records": (_I, [ctypes.POINTER(DiffuseParams), ctypes.POINTER(StepParams), _P, _P,
                               _P, _P, _P, _P, _P, _P, ctypes.POINTER(SplatParams), _P,
                               ctypes.c_size_t, _P, _P]),
    "sc_psf_quadrant_sat": (_I, [_P, _I, _I, _D, _P, _I, _P]),
    "sc_psf_box_table": (_I, [_P, _I, _I, _I, _I, _P, _P]),
    "sc_emitter_steps": (_I, [ctypes.POINTER(StepParams), _P, _P, _P, _P, _P, _P, _P, _P, _P,
                              _P]),
    "sc_bin_workspace_bytes": (ctypes.c_size_t, [_I, _I]),
    "sc_bin_reset": (_I, [ctypes.POINTER(SplatParams), _P, ctypes.c_size_t, _P]),
    "sc_bin_finish": (_I, [_I, ctypes.POINTER(SplatParams), _P, ctypes.c_size_t, _P, _P, _P]),
    "sc_bin_steps": (_I, [_P, _I, ctypes.POINTER(SplatParams), _P, ctypes.c_size_t, _P, _P, _P,
                          _P]),
    "sc_bin_steps_static": (_I, [_P, _I, ctypes.POINTER(SplatParams), _P, _P, _P, _P]),
    "sc_splat_fp64": (_I, [_P, _P, _I, _P, ctypes.POINTER(SplatParams), _P, _P, _P]),
    "sc_splat_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(SplatParams)]),
    "sc_batch_frame": (_I, [_P, _P, _P, _P, _P, ctypes.POINTER(SplatParams),
                            ctypes.POINTER(BatchPlan), ctypes.POINTER(CameraParams), _P, _P, _P,
                            _P, _P, _P, ctypes.c_size_t, _P, _P, _P, _P]),
    "sc_splat": (_I, [_P, _P, _P, _P, _P, ctypes.POINTER(SplatParams), _P, ctypes.c_size_t, _P,
                      _P, _P]),
    "sc_camera": (_I, [ctypes.POINTER(CameraParams), _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                       _P, _P, _P, _P, _P]),
    "sc_merge_camera": (_I, [ctypes.POINTER(SplatParams), _P, ctypes.c_size_t,
                             ctypes.POINTER(CameraParams), _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sc_emccd_exact": (_I, [_P, _D, _D, _P, _I, _D, _P, _P, _P]),
    "sc_bw_work_bytes": (ctypes.c_size_t, [ctypes.POINTER(BWParams)]),
    "sc_bw_forward": (_I, [ctypes.POINTER(BWParams), _P, _P, _P, _P, ctypes.c_size_t, _P, _P,
                           _P]),
    "sc_bw_backward": (_I, [ctypes.POINTER(BWParams), _P, _P, _P, _P, _P, _P]),
    "sc_log_cube": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _I, _P, ctypes.c_size_t, _P, _P]),
    "sc_log_peaks": (_I, [_P, _I, _I, _I, _D, _P, _P, _I, _P]),
    "sc_poisson_table_bytes": (ctypes.c_size_t, []),
    "sc_poisson_table": (_I, [_P, ctypes.c_size_t, _P]),
    "sc_gauss_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(GaussParams)]),
    "sc_gauss_forward": (_I, [ctypes.POINTER(GaussParams), _P, _P, _P, _P, ctypes.c_size_t, _P,
                              _P, _P]),
    "sc_gauss_backward": (_I, [ctypes.POINTER(GaussParams), _P, _P, _P, ctypes.c_size_t, _P, _P,
                                 _P, _P]),
    "sc_reduce_scratch_bytes": (ctypes.c_size_t, [ctypes.c_int64, _I]),
    "sc_dgrad_scratch_bytes": (ctypes.c_size_t, [ctypes.c_int64]),
    "sc_diffusion_positions": (_I, [_P, _I, _I, _P, _D, ctypes.c_uint64, _P, _P, _P]),
    "sc_gauss_nll": (_I, [_P, _P, ctypes.c_int64, _P, _D, _P, ctypes.c_size_t, _P, _P, _P]),
    "sc_diffusion_dD": (_I, [_P, _P, _I, _I, _P, _P, _P, ctypes.c_size_t, _P, _P]),
    "sc_segment_sum": (_I, [_P, ctypes.c_int64, _I, _P, ctypes.c_size_t, _P, _P]),
    "sc_spot_fit": (_I, [_P, _I, _I, _P, _I, _D, _P, _P]),
    "sc_poisson_nll": (_I, [_P, _P, ctypes.c_int64, _I, _P, ctypes.c_size_t, _P, _P, _P]),
}


class ScopyonGPUError(RuntimeError):
    """A library call failed; ``code`` is the SC_ERR_* value."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


class ScopyonInputError(ScopyonGPUError, ValueError):
    """Invalid input found on the device (a non-finite position, a malformed
    record): a ValueError, as the reference raises for the same inputs."""


_lock = threading.Lock()
_lib = None


def declared_symbols():
    return sorted(_SIG)


def load():
    """Load the library (once) and attach prototypes; raise if it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libscopyon_gb300.so is not built (%s); run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first" % LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIG.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc, what=""):
    """Map a library return code to an exception."""
    if rc == SC_OK:
        return
    msg = load().sc_last_error().decode(errors="replace")
    text = "%s failed (%d): %s" % (what or "scopyon_gb300", rc, msg)
    if rc == SC_ERR_ARG:
        raise ValueError(text)
    if rc == SC_ERR_TIMEOUT:
        raise TimeoutError(text)
    if rc == SC_ERR_NAN:
        raise ValueError(text)
    raise ScopyonGPUError(rc, text)


def call(name, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc


_POISSON = {}


def poisson_table(device):
    """The camera's Poisson tables on ``device`` (built once per device)."""
    import torch
    dev = torch.device(device)
    key = (dev.type, dev.index if dev.index is not None else torch.cuda.current_device())
    t = _POISSON.get(key)
    if t is None:
        nbytes = load().sc_poisson_table_bytes()
        t = torch.empty((nbytes + 15) // 16 * 4, dtype=torch.int32, device=dev)
        with torch.cuda.device(dev):
            call("sc_poisson_table", ptr(t), t.numel() * 4, stream_ptr())
            torch.cuda.current_stream().synchronize()  # ready for every stream
        _POISSON[key] = t
    return t


def ptr(t):
    """Device address of a torch tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    """The CUDA stream handle of ``stream`` (a torch stream), by default of
    the current stream of the current device (read without building a
    stream object where torch offers that)."""
    import torch
    if stream is not None:
        return ctypes.c_void_p(stream.cuda_stream)
    raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if raw is not None:
        return ctypes.c_void_p(raw(torch.cuda.current_device()))
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
