"""Multi-state Brownian points on the GPU: ``scopyon.sampling2.sample``.

The reference (src/scopyon/sampling2.py:70-148) places ``N[i]`` points of
each state i uniformly in [lower, upper] (state block by state block, axis by
axis, :15-31), then at every later time point moves each point by
N(0, sqrt(2 D[state] dt)) per axis (:33-50), wraps it into the box when
``periodic`` (a flat axis stays on its wall), and, with a rate matrix
``transmat``, lets it change state with probability 1 - exp(-rate dt)
(:52-68).  It returns one (n, ndim + 2) array [coords, state, id] per time
point.

``sample`` here returns a ``StateTrajectories``: the points live on the GPU
and move frame by frame (``sc_diffuse_steps`` with a transition table, or
inside the frame graph's records kernel).  Indexing and iteration give the
reference's arrays; passed to ``generate_images`` it is a device trajectory
whose diffusion class is the state.  Draws come from Philox keyed by a seed
drawn from ``rng`` or, with ``exact=True``, from ``rng`` itself in the
reference's order (normals, then one uniform per point per time step), so
that positions and states equal the reference's bit for bit.

The reference calls ``numpy.searchsorted(..., side='leff')``, which numpy 2
rejects and older numpy read as 'left'; the transition here is 'left'.
"""

import collections.abc
import numbers
import warnings

import numpy

from .sampling import DeviceTrajectories

__all__ = ["sample", "StateTrajectories"]


class StateTrajectories(DeviceTrajectories):
    """Device trajectories whose class is a Markov state; indexing and
    iteration give the reference's (n, ndim + 2) arrays [coords, state, id]."""

    def points(self, k):
        """Host (n, ndim + 2) [coords, state, id] at time index k."""
        walk = self.copy()
        walk.advance_to(k)
        pos = walk._pos.cpu().numpy()
        out = numpy.zeros((self.n_particles, self.ndim + 2))
        out[:, : self.ndim] = pos[:, : self.ndim]
        out[:, self.ndim] = walk.classes()
        out[:, self.ndim + 1] = self.points0[:, self.ndim]
        return out

    def __getitem__(self, k):
        if k < 0:
            k += len(self.times)
        if not 0 <= k < len(self.times):
            raise IndexError("time index out of range")
        return self.points(k)

    def __iter__(self):
        walk = self.copy()
        for k in range(len(self.times)):
            walk.advance_to(k)
            pos = walk._pos.cpu().numpy()
            out = numpy.zeros((self.n_particles, self.ndim + 2))
            out[:, : self.ndim] = pos[:, : self.ndim]
            out[:, self.ndim] = walk.classes()
            out[:, self.ndim + 1] = self.points0[:, self.ndim]
            yield out


def _box(value, ndim, default):
    if value is None:
        return numpy.ones(ndim) * default
    if isinstance(value, numbers.Number):
        return numpy.ones(ndim) * value
    return numpy.array(value, dtype=float)


def sample(t, N, *, lower=None, upper=None, D=None, transmat=None, ndim=3, periodic=False,
           rng=None, exact=False, device=None):
    """Points of several states at the time points ``t`` (reference
    sampling2.sample's arguments and defaults: lower 0, upper 1, D 0).

    Returns a ``StateTrajectories`` (list-like: one (n, ndim + 2) array per
    time point).  ``exact=True`` draws every normal and uniform from ``rng``
    up front, in the reference's order (host memory: T x n x (ndim + 1)
    doubles)."""
    N = list(N) if isinstance(N, collections.abc.Iterable) else [N]
    lower = _box(lower, ndim, 0.0)
    upper = _box(upper, ndim, 1.0)
    if len(lower) < ndim or len(upper) < ndim:
        raise ValueError("The wrong size of limits was given [(lower={}, upper={}) != {}]."
                         .format(len(lower), len(upper), ndim))
    for d in range(ndim):
        if lower[d] > upper[d]:
            lower[d], upper[d] = upper[d], lower[d]
    if D is None:
        D = numpy.zeros(len(N))
    elif not isinstance(D, collections.abc.Iterable):
        D = numpy.ones(len(N)) * D
    else:
        D = numpy.asarray(D, dtype=float)
        if len(D) != len(N):
            raise ValueError("D must have one value per state")
    if transmat is not None:
        transmat = numpy.asarray(transmat, dtype=float)
        if transmat.ndim != 2 or transmat.shape[0] != transmat.shape[1]:
            raise ValueError("transmat must be a square matrix")
        if not (transmat.diagonal() == 0).all():
            raise ValueError("transmat must have a zero diagonal")
        if transmat.shape[0] != len(N):
            raise ValueError("transmat needs one row per state")
    if rng is None:
        warnings.warn("A random number generator [rng] is not given.")
        rng = numpy.random.RandomState()
    times = numpy.asarray(t, dtype=float)
    if (numpy.diff(times) < 0).any():
        raise ValueError("time points must not decrease")
    # initial points, state block by state block and axis by axis (:15-31)
    n = int(sum(N))
    points = numpy.zeros((n, ndim + 2))
    klass = numpy.zeros(n, dtype=numpy.int32)
    tot = 0
    for i, cnt in enumerate(N):
        for d in range(ndim):
            points[tot:tot + cnt, d] = (rng.uniform(lower[d], upper[d], cnt)
                                        if lower[d] < upper[d] else lower[d])
        klass[tot:tot + cnt] = i
        tot += cnt
    points[:, ndim] = numpy.arange(n)  # id
    points[:, ndim + 1] = 1.0
    normals = uniforms = None
    if exact:
        steps = max(len(times) - 1, 0)
        normals = numpy.zeros((steps, n, ndim))
        uniforms = numpy.zeros((steps, n)) if transmat is not None else None
        for g in range(steps):
            if times[g + 1] > times[g]:
                normals[g] = rng.standard_normal((n, ndim))
                if transmat is not None:
                    uniforms[g] = rng.uniform(0, 1, n)
        seed = 0
    else:
        seed = (int(rng.randint(0, 2 ** 31 - 1)) << 31) | int(rng.randint(0, 2 ** 31 - 1))
    Dk = numpy.repeat(D[:, None], ndim, axis=1)
    return StateTrajectories(times, points, Dk, ndim, seed, normals,
                             "periodic" if periodic else "none", lower, upper, klass=klass,
                             device=device, transmat=transmat, uniforms=uniforms)
