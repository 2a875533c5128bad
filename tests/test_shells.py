"""Shell lookup of the intensity-map cells (get_r_index_imap, imap.c:196-208)
on the CPU: the walk from shell 0 and its bisection form agree on every
radius, for contiguous, gapped, overlapping and unsorted-end shell sets."""
import numpy as np
import pytest


def _shells(kind, rng):
    if kind == "contiguous":
        e = np.sort(rng.uniform(100, 3000, 65))
        return e[:-1], e[1:]
    if kind == "gaps":
        e = np.sort(rng.uniform(100, 3000, 128))
        return e[0::2], e[1::2]
    if kind == "overlap":
        r0 = np.sort(rng.uniform(100, 3000, 40))
        return r0, r0 + rng.uniform(10, 400, 40)
    if kind == "one":
        return np.array([500.0]), np.array([900.0])
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["contiguous", "gaps", "overlap", "one"])
def test_bisection_matches_walk(built, kind):
    import oracle as orc
    rng = np.random.default_rng(21)
    r0, rf = _shells(kind, rng)
    r = rng.uniform(0, 3500, 200000).astype(np.float32)
    # every edge and its float neighbours
    e = np.concatenate([r0, rf]).astype(np.float32)
    r = np.concatenate([r, e, np.nextafter(e, np.float32(0)), np.nextafter(e, np.float32(1e9))])
    walk, bis = orc.shell_index(r0, rf, r)
    assert np.array_equal(walk, bis)
    assert set(np.unique(walk)) <= set(range(-1, len(r0) + 1))
