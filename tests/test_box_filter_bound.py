"""The centre-per-lane scans drop a candidate when its float distance to the
bounding box of a batch's centres, squared, exceeds R^2 (1 + 2^-12).  That is
exact only if no (centre, candidate) pair whose float d^2 is <= R^2 -- the
reference's in-ball test -- has a box distance above the bound.  This checks
the argument on the CPU with numpy float32 arithmetic (IEEE round to nearest,
the same operations in the same order as the device): candidates placed on and
just around the sphere of radius R about a box corner centre, far from the
origin and near it, with R from 1e-3 to 8 nm.
"""
import numpy as np

F = np.float32


def ref_d2(c, q):
    """The reference's squared distance: ((dx^2 + dy^2) + dz^2) in float."""
    d = (c - q).astype(F)
    s = d * d
    return ((s[..., 0] + s[..., 1]).astype(F) + s[..., 2]).astype(F)


def box_d2(lo, hi, q):
    """The scans' squared distance of q to the box [lo, hi], in float."""
    g = np.maximum(np.maximum((lo - q).astype(F), (q - hi).astype(F)), F(0))
    s = g * g
    return ((s[..., 0] + s[..., 1]).astype(F) + s[..., 2]).astype(F)


def test_box_filter_never_drops_an_in_ball_pair():
    rng = np.random.default_rng(7)
    worst = 0.0
    for offset in (0.0, 3.0, 250.0, 4096.0):
        for R in (1e-3, 0.37, 1.0, 2.0, 2.5, 8.0):
            R2 = F(F(R) * F(R))
            bound = F(R2 * F(1.0 + 2.0 ** -12))
            for _ in range(20):
                # 32 centres in a box a cell block wide, away from the origin
                base = (rng.uniform(-1, 1, 3) * offset).astype(F)
                cen = (base + rng.uniform(0, R, (32, 3))).astype(F)
                lo, hi = cen.min(axis=0), cen.max(axis=0)
                # candidates on the sphere of radius R about each centre, nudged
                # by a few ulps either way
                u = rng.normal(size=(32, 64, 3))
                u /= np.linalg.norm(u, axis=2, keepdims=True)
                scale = R * (1 + rng.uniform(-4e-7, 4e-7, (32, 64, 1)))
                q = (cen[:, None, :].astype(np.float64) + u * scale).astype(F)
                d2 = ref_d2(cen[:, None, :], q)
                bd = box_d2(lo, hi, q)
                inball = d2 <= R2
                assert not np.any(inball & (bd > bound))
                if inball.any():
                    worst = max(worst, float(np.max(bd[inball] / R2)))
    # the margin is far from being used up
    assert worst < 1 + 2.0 ** -18
