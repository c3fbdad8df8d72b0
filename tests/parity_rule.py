"""The per-sample radiance rule of the GPU parity tests against the oracle.

The CUDA path shades with fast maths, as the reference's GPU build does (its
megakernel is the code it replaces), and the oracle in IEEE single
precision, so a sample's radiance may differ in its last bits -- and by more
where the path is ill-conditioned: a near-specular GGX lobe (roughness 0.05,
alpha 0.0025) turns a direction error of 1e-6 into a relative change of its
value of ~1e-3, and a ray grazing an edge, an occluder, a hemisphere or
total-internal-reflection test, or a roulette draw at its threshold flips a
decision.  The fast sine and cosine of the direction samplers are accurate
to ~1e-6 absolute, but near a GGX lobe's axis the sampler takes the inverse
cosine of a value within ulps of 1, where fast division's few ulps move the
sampled direction by up to ~1e-4 (measured: with a probe of 1e-5 on
directions, deviations reach 109x the response; with 1e-4, 6x).

A sample is within tolerance when its relative error -- the largest channel
difference over the largest channel of the oracle's value, floored at 1e-3
-- is at most TOL.  A sample outside it must be explained: the oracle's
rounding-sensitivity probe (orc_render_sensitivity: the same sample
re-rendered PROBE_COPIES times with its scattered directions, normals and
throughput moved by PROBE_EPS relative and its surface and light points,
texture coordinates and direction-sampling numbers by PROBE_EPS_POS, the
size of those fast-maths errors, in pseudo-random directions) must move the oracle's own value of that sample by at least
1/RATIO of the GPU's deviation from it: the deviation is then of the size
that rounding of that magnitude produces there.  The excuse is proportional:
a sample 50% off needs a probe response of 6%, which only a decision that
such perturbations flip gives (measured: the deviations outside TOL are at
most 5x the probe's response).  And at least MIN_WITHIN of all samples must
be within TOL, so that the rule cannot hide a systematic error.
"""

import numpy as np

TOL = 1e-4
PROBE_EPS = 1e-4
PROBE_EPS_POS = 1e-5
PROBE_COPIES = 16
RATIO = 8.0
MIN_WITHIN = 0.99


def rel_err(gpu, ref):
    return np.abs(gpu - ref).max(-1) / np.maximum(np.abs(ref).max(-1), 1e-3)


def check_samples(gpu, ref, response, label=""):
    """gpu, ref: [..., 3] radiance; response: the probe's [...] response.
    Asserts the rule and returns a one-line summary."""
    err = rel_err(gpu, ref)
    outside = err > TOL
    unexplained = outside & (response * RATIO < err)
    worst = float((err[outside] / np.maximum(response[outside], 1e-30)).max()) if outside.any() else 0.0
    summary = (f"{label}: {outside.sum()} of {err.size} samples outside {TOL:g} "
               f"(max error {err.max():.2e}); largest deviation / probe response among them {worst:.2f}; "
               f"unexplained {unexplained.sum()}")
    print(summary)
    assert not unexplained.any(), summary + f"; first unexplained at {np.argwhere(unexplained)[:5].tolist()}"
    assert 1.0 - outside.mean() >= MIN_WITHIN, summary
    return summary
