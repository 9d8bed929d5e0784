"""Brownian input trajectories generated on the GPU.

``sample_inputs`` has the signature and semantics of ``scopyon.sample_inputs``
(reference src/scopyon/sampling.py:121-162): uniform initial points drawn from
``rng`` column by column (``sample_points``, :14-86), then a Gaussian step
N(0, sqrt(2 D dt)) per particle and axis at every later time point
(``move_points``, :88-119).  Instead of a host list of copies (16 GB for
20,000 particles over 20,000 time points) it returns a ``DeviceTrajectories``
whose positions live on the GPU and advance frame by frame inside
``generate_images``.

Normals: from Philox4x32-10 keyed by a seed drawn from ``rng`` (default), or,
with ``exact=True``, drawn from ``rng`` itself in the reference's order so that
the trajectories are bit-identical to the reference's.
"""

import collections.abc
import numbers
import warnings

import numpy
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr

__all__ = ["sample_inputs", "sample_points", "DeviceTrajectories"]

_BOUNDARY = {"none": 0, "periodic": 1, "reflecting": 2}


def sample_points(rng, N=None, conc=None, lower=None, upper=None, start=0, ndim=3):
    """Uniform initial points and the next free id (reference sampling.py:14-86)."""
    if N is None and conc is None:
        raise ValueError("Either one of N or conc must be given.")
    lower = (numpy.ones(ndim) * lower if isinstance(lower, numbers.Number)
             else numpy.array(lower, dtype=float) if lower is not None else numpy.zeros(ndim))
    upper = (numpy.ones(ndim) * upper if isinstance(upper, numbers.Number)
             else numpy.array(upper, dtype=float) if upper is not None else numpy.ones(ndim))
    if len(lower) < ndim or len(upper) < ndim:
        raise ValueError("The wrong size of limits was given [(lower={}, upper={}) != {}]."
                         .format(len(lower), len(upper), ndim))
    for d in range(ndim):
        if lower[d] > upper[d]:
            lower[d], upper[d] = upper[d], lower[d]
    if N is None:
        lengths = upper - lower
        size = numpy.prod(lengths[lengths != 0])
        if isinstance(conc, collections.abc.Iterable):
            n_list = [rng.poisson(size * c) for c in conc]
        else:
            n_list = [rng.poisson(size * conc)]
    elif not isinstance(N, collections.abc.Iterable):
        n_list = [N]
    else:
        n_list = list(N)
    n = int(sum(n_list))
    if n <= 0:
        return numpy.zeros((0, len(lower) + 2)), start
    maxdim = len(lower)
    out = numpy.zeros((n, maxdim + 2))
    for d in range(maxdim):
        out[:, d] = rng.uniform(lower[d], upper[d], n) if lower[d] < upper[d] else lower[d]
    out[:, maxdim] = numpy.arange(start, start + n)
    out[:, maxdim + 1] = 1.0
    return out, start + n


class DeviceTrajectories:
    """Particle positions on the GPU at a sorted list of time points.

    Built by ``sample_inputs`` (one diffusion class) or ``concatenate``
    (several classes, e.g. two populations with different D).  Positions
    advance only forwards: frame f of ``generate_images`` moves them through
    the frame's time points.  Iterating yields ``(t, points)`` host copies
    like the reference's list, by replaying the trajectory on the device.
    """

    def __init__(self, times, points, D, ndim, seed, normals=None, boundary="none",
                 lower=None, upper=None, klass=None, device=None, class_box=None,
                 transmat=None, uniforms=None):
        self.times = numpy.asarray(times, dtype=float)
        self.points0 = numpy.asarray(points, dtype=float)   # (N, ndim + 2) host
        self.ndim = int(ndim)
        self.D = numpy.atleast_2d(numpy.asarray(D, dtype=float))  # (n_class, ndim)
        self.seed = int(seed) & (2 ** 64 - 1)
        self.normals = normals  # host (T-1, N, ndim) or None
        self.boundary = boundary
        self.lower = numpy.zeros(3) if lower is None else numpy.resize(numpy.asarray(lower, float), 3)
        self.upper = numpy.ones(3) if upper is None else numpy.resize(numpy.asarray(upper, float), 3)
        self.klass = (numpy.zeros(len(self.points0), dtype=numpy.int32) if klass is None
                      else numpy.asarray(klass, dtype=numpy.int32))
        self.device = torch.device(device or "cuda")
        # optional walls per class: (n_class, 6) lower xyz, upper xyz
        self.class_box = None if class_box is None else torch.as_tensor(
            numpy.asarray(class_box, dtype=float).reshape(-1, 6), device=self.device)
        # optional class transitions (sampling2): rates (n_class, n_class) in 1/s,
        # and in exact mode the uniforms (T-1, N) drawn in the reference's order
        self.transmat = None if transmat is None else numpy.asarray(transmat, dtype=float)
        self.uniforms = uniforms
        self._pos = None
        self._cls = None  # device classes, changed in place by transitions
        self._index = 0

    # -- reference-compatible access -----------------------------------
    def __len__(self):
        return len(self.times)

    @property
    def n_particles(self):
        return len(self.points0)

    def ids(self):
        return self.points0[:, self.ndim]

    def states(self):
        return self.points0[:, self.ndim + 1]

    def __iter__(self):
        fresh = self.copy()
        for k in range(len(self.times)):
            pts = fresh.materialize(k)
            yield (float(self.times[k]), pts)

    def __getitem__(self, k):
        return float(self.times[k]), self.copy().materialize(k)

    def copy(self):
        box = None if self.class_box is None else self.class_box.cpu().numpy()
        return type(self)(self.times, self.points0, self.D, self.ndim, self.seed,
                          self.normals, self.boundary, self.lower, self.upper, self.klass,
                          self.device, class_box=box, transmat=self.transmat,
                          uniforms=self.uniforms)

    def materialize(self, k):
        """Host (N, ndim + 2) points at time index k (advances this object)."""
        self.advance_to(k)
        pos = self._pos.cpu().numpy()
        out = self.points0.copy()
        out[:, : self.ndim] = pos[:, : self.ndim]
        return out

    # -- device state ----------------------------------------------------
    def reset(self):
        pos = numpy.zeros((self.n_particles, 3))
        pos[:, : self.ndim] = self.points0[:, : self.ndim]
        if self.native:  # native moves keep FP32 positions (sc_diffuse_steps)
            pos = pos.astype(numpy.float32).astype(numpy.float64)
        if self._pos is None:
            self._pos = torch.from_numpy(pos).to(self.device)
            self._cls = torch.from_numpy(self.klass).to(self.device)
        else:  # in place: captured frame graphs keep these addresses
            self._pos.copy_(torch.from_numpy(pos))
            self._cls.copy_(torch.from_numpy(self.klass))
        self._index = 0

    def classes(self):
        """Current class of every particle (host int32)."""
        if self._cls is None:
            return self.klass.copy()
        return self._cls.cpu().numpy()

    def _transitions(self, g0, n):
        """Cumulative transition probabilities of steps g0 .. g0 + n - 1,
        [n][n_class][n_class], as sampling2.__transition_states forms them
        (src/scopyon/sampling2.py:52-68); a step of zero length keeps the class
        (its rows are -1 below the class and 1 from it on)."""
        nc = self.D.shape[0]
        out = numpy.zeros((n, nc, nc))
        for s in range(n):
            g = g0 + s
            if g + 1 < len(self.times) and self.times[g + 1] > self.times[g]:
                dt = self.times[g + 1] - self.times[g]
                P = 1 - numpy.exp(-self.transmat * dt)
                P.ravel()[:: nc + 1] = 1.0 - P.sum(axis=1)
                out[s] = P.cumsum(axis=1)
            else:
                out[s] = numpy.where(numpy.arange(nc)[None, :] >= numpy.arange(nc)[:, None],
                                     1.0, -1.0)
        return out

    def _sigma(self, g0, n):
        """sqrt(2 D dt) per step (of n from time index g0), class and axis, as the reference."""
        sig = numpy.zeros((n, self.D.shape[0], 3))
        for s in range(n):
            g = g0 + s
            if g + 1 < len(self.times) and self.times[g + 1] > self.times[g]:
                dt = self.times[g + 1] - self.times[g]
                sig[s, :, : self.ndim] = numpy.sqrt(2 * self.D * dt)
        return sig

    def params(self, g0, n, scale=1.0, origin=(0.0, 0.0, 0.0), unit_x=(1.0, 0.0, 0.0),
               unit_y=(0.0, 1.0, 0.0)):
        p = _lib.DiffuseParams()
        p.n_particles, p.n_sub, p.ndim = self.n_particles, n, self.ndim
        p.boundary = _BOUNDARY[self.boundary]
        p.n_class = self.D.shape[0]
        p.step0, p.seed = g0, self.seed
        unit_z = numpy.cross(unit_x, unit_y)
        for d in range(3):
            p.lower[d], p.upper[d] = float(self.lower[d]), float(self.upper[d])
            p.origin[d] = float(origin[d])
            p.unit_x[d], p.unit_y[d], p.unit_z[d] = float(unit_x[d]), float(unit_y[d]), float(unit_z[d])
        p.scale = float(scale)
        p.d_class_box = None if self.class_box is None else self.class_box.data_ptr()
        return p

    @property
    def native(self):
        """Philox normals: positions are FP32 values, moved in FP32 on the device."""
        return self.normals is None

    def compact_rows(self, transform=None):
        """Whether frames can use the 16-byte FP32 rows of sc_diffuse_steps
        (layout 1): native draws and the identity preprocessing transform."""
        t = transform or {}
        if not self.native or float(t.get("scale", 1.0)) != 1.0:
            return False
        if self.ndim == 2:
            return True
        return (numpy.array_equal(numpy.asarray(t.get("origin", (0.0, 0.0, 0.0)), float), numpy.zeros(3))
                and numpy.array_equal(numpy.asarray(t.get("unit_x", (1.0, 0.0, 0.0)), float), [1.0, 0.0, 0.0])
                and numpy.array_equal(numpy.asarray(t.get("unit_y", (0.0, 1.0, 0.0)), float), [0.0, 1.0, 0.0]))

    def run(self, g0, n, out, transform=None, stream=None, layout=0):
        """Write the formatted positions of time indices g0 .. g0+n-1 to ``out``
        ([n][N][5] float64 on the device; with layout 1, [n][N][4] float32
        rows [depth, x, y, 0]; None: no rows) and move the particles past them."""
        if self._pos is None or self._index > g0:
            self.reset()
        if self._index < g0:
            self.advance_to(g0, transform, stream)
        p = self.params(g0, n, **(transform or {}))
        p.layout = layout
        sig = torch.from_numpy(self._sigma(g0, n)).to(self.device)
        normals = None
        if self.normals is not None:
            nrm = numpy.zeros((n, self.n_particles, self.ndim))
            for s in range(n):
                g = g0 + s
                if g < len(self.normals):
                    nrm[s] = self.normals[g]
            normals = torch.from_numpy(nrm).to(self.device)
        trans = unif = None
        if self.transmat is not None:
            trans = torch.from_numpy(self._transitions(g0, n)).to(self.device)
            p.d_trans = trans.data_ptr()
            if self.uniforms is not None:
                u = numpy.zeros((n, self.n_particles))
                for s in range(n):
                    if g0 + s < len(self.uniforms):
                        u[s] = self.uniforms[g0 + s]
                unif = torch.from_numpy(u).to(self.device)
                p.d_uniforms = unif.data_ptr()
        call("sc_diffuse_steps", p, ptr(self._pos), ptr(self._cls), ptr(sig), ptr(normals),
             ptr(out), stream_ptr(stream))
        self._index = g0 + n

    def prepare_uniform(self, n_sub):
        """Device sigma / class tensors for frames of n_sub steps on a uniform time grid."""
        dt = numpy.diff(self.times)
        # spacing equal to 1e-9 relative: long time axes carry rounding of t itself
        if len(dt) == 0 or not numpy.allclose(dt, dt[0], rtol=0, atol=1e-9 * abs(dt[0])):
            raise ValueError("graph replay needs uniformly spaced time points")
        if self.normals is not None:
            raise ValueError("graph replay draws Philox normals; exact trajectories replay eagerly")
        sig = numpy.zeros((n_sub, self.D.shape[0], 3))
        sig[:, :, : self.ndim] = numpy.sqrt(2 * self.D * dt[0])
        self._g_sigma = torch.from_numpy(sig).to(self.device)
        self._g_trans = None
        if self.transmat is not None:
            nc = self.D.shape[0]
            P = 1 - numpy.exp(-self.transmat * dt[0])
            P.ravel()[:: nc + 1] = 1.0 - P.sum(axis=1)
            self._g_trans = torch.from_numpy(
                numpy.repeat(P.cumsum(axis=1)[None], n_sub, axis=0)).to(self.device)
        if self._pos is None:
            self.reset()

    def graph_params(self, g0, n_sub, transform=None):
        """Launch parameters of a captured frame: the uniform sigma and, with
        transitions, their table for n_sub steps from step g0 of the frame."""
        p = self.params(g0, n_sub, **(transform or {}))
        if self._g_trans is not None:
            p.d_trans = self._g_trans.data_ptr()
        return p

    def launch_frame(self, n_sub, out, d_frame, transform=None, stream=None, layout=0):
        """Enqueue one frame's sub-steps, step index taken from the device counter
        ``d_frame`` (frame f covers steps f * n_sub ... f * n_sub + n_sub - 1),
        rows in ``out`` as ``run`` writes them for ``layout``.
        Fixed arguments only, so it can be captured in a CUDA graph."""
        p = self.graph_params(0, n_sub, transform)
        p.layout = layout
        p.d_frame = d_frame.data_ptr()
        call("sc_diffuse_steps", p, ptr(self._pos), ptr(self._cls), ptr(self._g_sigma), None,
             ptr(out), stream_ptr(stream))

    def state_dict(self):
        """The trajectory's state as host arrays: the time index reached, the
        positions and the classes there.  With the construction arguments
        (and the seed) it is all that later positions depend on, since the
        Philox normals and transition uniforms are keyed by (seed, particle,
        step)."""
        if self._pos is None:
            self.reset()
        return {"index": int(self._index), "pos": self._pos.cpu().numpy().copy(),
                "cls": self._cls.cpu().numpy().copy(), "seed": self.seed}

    def load_state_dict(self, state):
        """Resume from ``state_dict()``: the positions and classes are copied
        into the existing device buffers (a captured frame graph keeps
        them)."""
        if int(state["seed"]) != self.seed:
            raise ValueError("the state is of trajectories with another seed")
        pos = numpy.asarray(state["pos"], dtype=numpy.float64)
        cls = numpy.asarray(state["cls"], dtype=numpy.int32)
        if pos.shape != (self.n_particles, 3) or cls.shape != (self.n_particles,):
            raise ValueError("the state holds %s positions for %d particles"
                             % (pos.shape, self.n_particles))
        if self._pos is None:
            self.reset()
        self._pos.copy_(torch.from_numpy(pos))
        self._cls.copy_(torch.from_numpy(cls))
        self._index = int(state["index"])

    def advance_to(self, k, transform=None, stream=None):
        if self._pos is None or self._index > k:
            self.reset()
        while self._index < k:
            n = min(k - self._index, 64)
            self.run(self._index, n, None, transform, stream)  # positions only, no rows


def concatenate(*trajs):
    """One DeviceTrajectories from several with the same time points (populations)."""
    first = trajs[0]
    for t in trajs[1:]:
        if not numpy.array_equal(t.times, first.times) or t.ndim != first.ndim:
            raise ValueError("trajectories to concatenate need the same times and ndim")
        if t.normals is not None or first.normals is not None:
            raise ValueError("exact (injected-normal) trajectories cannot be concatenated")
    points = numpy.vstack([t.points0 for t in trajs])
    D = numpy.vstack([t.D for t in trajs])
    klass, off = [], 0
    for t in trajs:
        klass.append(t.klass + off)
        off += t.D.shape[0]
    return DeviceTrajectories(first.times, points, D, first.ndim, first.seed, None, first.boundary,
                              first.lower, first.upper, numpy.concatenate(klass), first.device)


def sample_inputs(t, *, N=None, conc=None, lower=None, upper=None, D=None, start=0, ndim=3,
                  rng=None, exact=False, boundary="none", device=None):
    """Device trajectories with the reference's model (sampling.py:121-162).

    ``boundary`` ('none', 'periodic', 'reflecting') confines the particles to
    [lower, upper]; the reference has no boundary.  ``exact=True`` draws every
    normal from ``rng`` up front (host memory: T x N x ndim doubles) so that
    the trajectories equal the reference's bit for bit.
    """
    if rng is None:
        warnings.warn("A random number generator [rng] is not given.")
        rng = numpy.random.RandomState()
    if boundary not in _BOUNDARY:
        raise ValueError("boundary must be one of %s" % sorted(_BOUNDARY))
    times = numpy.array(sorted(t), dtype=float)
    points, _ = sample_points(rng, N=N, conc=conc, lower=lower, upper=upper, start=start, ndim=ndim)
    if D is None:
        Dv = numpy.zeros(ndim)
    elif not isinstance(D, collections.abc.Iterable):
        Dv = numpy.ones(ndim) * D
    else:
        Dv = numpy.asarray(D, dtype=float)
        if len(Dv) != ndim:
            raise ValueError("D must be a scalar or one value per axis")
    normals = None
    if exact:
        normals = numpy.zeros((max(len(times) - 1, 0), len(points), ndim))
        for g in range(len(times) - 1):
            if times[g + 1] > times[g]:
                normals[g] = rng.standard_normal((len(points), ndim))
        seed = 0
    else:
        seed = (int(rng.randint(0, 2 ** 31 - 1)) << 31) | int(rng.randint(0, 2 ** 31 - 1))
    lo = numpy.ones(ndim) * lower if isinstance(lower, numbers.Number) else (
        numpy.array(lower, float) if lower is not None else numpy.zeros(ndim))
    hi = numpy.ones(ndim) * upper if isinstance(upper, numbers.Number) else (
        numpy.array(upper, float) if upper is not None else numpy.ones(ndim))
    return DeviceTrajectories(times, points, Dv, ndim, seed, normals, boundary,
                              numpy.minimum(lo, hi), numpy.maximum(lo, hi), device=device)
