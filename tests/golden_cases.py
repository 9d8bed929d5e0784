"""Helpers that turn the reference golden fixture into oracle / engine inputs."""

import json

import numpy

import oracle as O

FRAME_CASES = (("fa", 1, "egfp"), ("fb", 3, "tritc"), ("fc", 2, "tritc"), ("fd", 2, "egfp"))


class FixedNormals:
    """Stands in for an rng whose one ``normal`` call returned ``values``."""

    def __init__(self, values):
        self.values = values

    def normal(self, *args, **kwargs):
        return self.values


def case_tree(g, name):
    return json.loads(str(g["%s_config" % name]))


def case_inputs(g, name):
    """Formatted ``[(t, (N,5))]`` inputs of a frame case, as the reference builds them."""
    tree = case_tree(g, name)
    pre = tree["preprocessing"]

    def fmt(a):
        return O.format_data(a, pre["scale"], pre["origin"], pre["unit_x"], pre["unit_y"])

    if "%s_inputs" % name in g:
        return [(0.0, fmt(g["%s_inputs" % name]))]
    return [(float(t), fmt(p)) for t, p in zip(g["%s_input_t" % name], g["%s_input_pts" % name])]


def case_raw_inputs(g, name):
    """Unformatted inputs, as a user passes them to ``form_image`` / ``generate_images``."""
    if "%s_inputs" % name in g:
        return g["%s_inputs" % name]
    return [(float(t), p) for t, p in zip(g["%s_input_t" % name], g["%s_input_pts" % name])]


def case_frames_draws(g, name, nframes):
    frames = []
    for f in range(nframes):
        prefix = "%s_f%d_" % (name, f)
        frames.append({k[len(prefix):]: g[k] for k in g.files if k.startswith(prefix)})
    return frames


def case_bleach(g, name):
    ids = [int(i) for i in g["%s_true_ids" % name]]
    times = g["%s_bleach_times" % name]
    return dict(zip(ids, times)) if len(times) else {}


def case_params(g, name, tag):
    tree = case_tree(g, name)
    fpn = "%s_fpn_normals" % name
    rng = FixedNormals(g[fpn]) if fpn in g else None
    return O.Params(tree["default"], float(g["cat_%s_psf_wavelength" % tag]),
                    float(g["cat_%s_fluoem_norm_sum" % tag]), rng=rng,
                    cmos_table=g["cmos_table"])
