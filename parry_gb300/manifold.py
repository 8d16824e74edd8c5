"""Host-side view of persistent contact manifolds in the C-ABI layout (parrygpu_manifold).

Mirrors parry3d's ContactManifold / TrackedContact (src/query/contact_manifolds/contact_manifold.rs:
TrackedContact at 108-226, ContactManifold at 662-800) as one fixed-size record per pair:

    n_points  u32         number of valid entries of `points`
    status    u32         0 = updated, 2 = Unsupported (shape pair without a manifold generator;
                          the record is otherwise left untouched, as the reference leaves its manifold)
    local_n1  f32[3]      contact normal in shape 1's local frame (also the GJK warm-start cache)
    local_n2  f32[3]      contact normal in shape 2's local frame
    points    24 x TrackedContact:
        local_p1 f32[3], local_p2 f32[3], dist f32, fid1 u32, fid2 u32, data f32

`data` is the per-contact user payload (ContactData in the reference, e.g. an accumulated impulse):
new contacts start at 0 and match_contacts carries it over from the previous frame's contact with
the same (fid1, fid2). 24 points bound every supported pair: a face-face cuboid pair yields at most
4 + 4 vertex contacts and 16 edge-edge crossings.

fid1 / fid2 are PackedFeatureId words (src/shape/packed_feature_id.rs): the top two bits give the
feature kind (1 vertex, 2 edge, 3 face; 0 = unknown) and the low 30 bits its index.
"""
from __future__ import annotations

import numpy as np

MAX_POINTS = 24
RECORD_WORDS = 8 + 10 * MAX_POINTS
PAIR_NONE = 0xFFFFFFFF  # a pair row (PAIR_NONE, PAIR_NONE) is an empty slot: skipped, record untouched

STATUS_OK = 0
STATUS_UNSUPPORTED = 2

TRACKED_CONTACT_DTYPE = np.dtype([("local_p1", "<f4", 3), ("local_p2", "<f4", 3), ("dist", "<f4"), ("fid1", "<u4"),
                                  ("fid2", "<u4"), ("data", "<f4")])
MANIFOLD_DTYPE = np.dtype([("n_points", "<u4"), ("status", "<u4"), ("local_n1", "<f4", 3), ("local_n2", "<f4", 3),
                           ("points", TRACKED_CONTACT_DTYPE, MAX_POINTS)])
assert TRACKED_CONTACT_DTYPE.itemsize == 40 and MANIFOLD_DTYPE.itemsize == 4 * RECORD_WORDS

FEATURE_UNKNOWN = 0


def feature_vertex(i: int) -> int:
    return (1 << 30) | int(i)


def feature_edge(i: int) -> int:
    return (2 << 30) | int(i)


def feature_face(i: int) -> int:
    return (3 << 30) | int(i)


def new_manifolds(k: int) -> np.ndarray:
    """k empty manifolds (ContactManifold::new())."""
    return np.zeros(k, MANIFOLD_DTYPE)


def as_words(m: np.ndarray) -> np.ndarray:
    """The (k, RECORD_WORDS) uint32 view of a MANIFOLD_DTYPE array (no copy)."""
    assert m.dtype == MANIFOLD_DTYPE and m.flags.c_contiguous
    return m.view(np.uint32).reshape(len(m), RECORD_WORDS)


def as_records(words: np.ndarray) -> np.ndarray:
    """The MANIFOLD_DTYPE view of (k, RECORD_WORDS) uint32 words (no copy)."""
    assert words.dtype == np.uint32 and words.flags.c_contiguous
    return words.reshape(-1).view(MANIFOLD_DTYPE)


def find_deepest_contact(m) -> int | None:
    """Index of the point with the smallest dist (ContactManifold::find_deepest_contact), or None."""
    n = int(m["n_points"])
    if n == 0:
        return None
    d = m["points"]["dist"][:n]
    best = 0
    for i in range(1, n):
        if d[i] < d[best]:
            best = i
    return best
