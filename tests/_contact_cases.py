"""Builds the reference's known-answer contact cases as ShapeSets + pair lists (shared by the
oracle tests and the GPU parity tests)."""
import json
from pathlib import Path

import numpy as np

from parry_gb300.shapes import ShapeSet, pose7

KA = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def cuboid_epa():
    c = KA["cuboid_cuboid_epa"]
    s = ShapeSet()
    pairs = []
    for case in c["cases"]:
        a = s.add_cuboid(c["half_extents"], pose7(case["pos1"]))
        b = s.add_cuboid(c["half_extents"], pose7(case["pos2"]))
        pairs.append((a, b))
    return s, np.array(pairs, np.uint32), c


def triangle_touch():
    c = KA["triangle_vertex_touches_triangle_edge_epa"]
    s = ShapeSet()
    a = s.add_triangle(*c["tri1"])
    b = s.add_triangle(*c["tri2"])
    return s, np.array([(a, b)], np.uint32), c


def ball_ball():
    c = KA["ball_ball_prediction"]
    s = ShapeSet()
    a = s.add_ball(c["radius"], pose7(c["pos1"]))
    b = s.add_ball(c["radius"], pose7(c["pos2"]))
    return s, np.array([(a, b)], np.uint32), c


def ball_cuboid():
    c = KA["ball_cuboid_contact_query"]
    s = ShapeSet()
    cub = s.add_cuboid(c["cuboid_half_extents"])
    pairs = []
    for case in c["cases"]:
        b = s.add_ball(c["ball_radius"], pose7(case["ball_pos"]))
        pairs.append((b, cub))
    return s, np.array(pairs, np.uint32), c
