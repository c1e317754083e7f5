"""Generate the golden fixtures in this folder from the FP64 oracle.

    python -m tests.golden.make_golden

The reference has no golden FP/BP vectors of its own (its operator tests are
relational), so these fixtures pin the oracle's outputs on small seeded cases:
tests check the oracle against them (regression) and the GPU kernels against
them (parity without rerunning the oracle). ``reference_pins.json`` (not
written by this script) holds outputs the reference's notebooks print: the one
numeric projection output it publishes for this path, and the reprs of its
unit cone geometry.
"""
import json
import os

import numpy as np

import tomosipo_gb300 as ts

HERE = os.path.dirname(os.path.abspath(__file__))


def _helical(n):
    t = np.linspace(0, 3 * np.pi, n, endpoint=False)
    rng = np.random.default_rng(5)
    c, s = np.cos(t), np.sin(t)
    rise = 0.3 * (t / (2 * np.pi) - 0.75)
    src = np.stack([rise, -2.5 * c, 2.5 * s], 1) + rng.normal(0, 0.5 / 24, (n, 3))
    det = np.stack([rise, 1.0 * c, -1.0 * s], 1) + rng.normal(0, 0.5 / 24, (n, 3))
    sv, su = 1.2 / 20, 1.8 / 30
    dv = np.stack([np.full(n, sv), 0 * t, 0 * t], 1)
    du = np.stack([0 * t, s * su, c * su], 1)
    return ts.cone_vec(shape=(20, 30), src_pos=src, det_pos=det, det_v=dv, det_u=du)


def build_case(name):
    """(vg, pg, x, y): geometry plus seeded volume and sinogram inputs."""
    vg = ts.volume(shape=(20, 22, 24), size=(0.9, 1.0, 1.1), pos=(0.02, -0.03, 0.01))
    R = ts.rotate(pos=0, axis=(0.3, 1.0, -0.5), angles=0.6)
    if name == "parallel":
        pg = ts.parallel(angles=12, shape=(20, 30), size=(1.2, 1.8))
    elif name == "cone":
        pg = ts.cone(angles=12, shape=(20, 30), size=(1.2, 1.8), src_orig_dist=2.5, src_det_dist=3.5)
    elif name == "parallel_vec_rotated":
        pg = R * ts.parallel(angles=12, shape=(20, 30), size=(1.2, 1.8)).to_vec()
    elif name == "cone_vec_helical":
        pg = _helical(12)
    else:
        raise KeyError(name)
    rng = np.random.default_rng(sum(map(ord, name)))
    x = rng.random(vg.shape)
    y = rng.random((pg.det_shape[0], pg.num_angles, pg.det_shape[1]))
    return vg, pg, x, y


CASES = ["parallel", "cone", "parallel_vec_rotated", "cone_vec_helical"]


def main():
    from oracle import oracle as orc

    meta = {}
    for name in CASES:
        vg, pg, x, y = build_case(name)
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            fp=orc.fp(vg, pg, x),
            bp_matched=orc.bp_matched(vg, pg, y),
            bp_bilinear=orc.bp_bilinear(vg, pg, y),
        )
        meta[name] = {"volume": list(vg.shape), "sinogram": [pg.det_shape[0], pg.num_angles, pg.det_shape[1]]}
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main()
