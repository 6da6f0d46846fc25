"""mamo text dumps (rta's -m output): the formatting of the plugin mirror
equals, byte for byte, what the reference's own dump code wrote for the same
arrays (binary_bvh::dump_acceleration_structure and ::dump_primitives,
bbvh/bbvh.h:36-65; cam_ray_generator_shirley::dump_rays,
librta/raytrav.h:353-366), special values included: -0, +-inf, NaN with and
without the sign bit, subnormal, integral and large values."""
import os

import numpy as np

from rta_gb300 import plugin as P


def golden(golden_dir):
    return np.load(os.path.join(golden_dir, "mamo_dumps.npz"))


def text(z, key):
    return z[key].tobytes().decode()


def test_bvh_dump_matches_reference_code(golden_dir):
    z = golden(golden_dir)
    assert P.format_bvh_dump(z["nodes"]) == text(z, "bvh_text")


def test_triangle_dump_matches_reference_code(golden_dir):
    z = golden(golden_dir)
    assert P.format_tri_dump(z["tris"]) == text(z, "tri_text")


def test_ray_dump_matches_reference_code(golden_dir):
    z = golden(golden_dir)
    r = z["rays"]
    assert P.format_ray_dump(r[:, 0:3], r[:, 3:6], r[:, 6], int(z["w"]), int(z["h"])) == text(z, "ray_text")
