"""Shared test set-up.  GPU tests carry @pytest.mark.gpu and run only on a
machine with a GB300; everything else runs on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle32():
    from oracle import build
    build.build_oracle()
    from oracle.pyoracle import Oracle
    return Oracle("f32")


@pytest.fixture(scope="session")
def oracle64():
    from oracle import build
    build.build_oracle()
    from oracle.pyoracle import Oracle
    return Oracle("f64")


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))


def per_body_rel(a, ref):
    """Per-particle relative L2 error |a_i - ref_i| / |ref_i| of (n, 3)
    vectors (or n scalars), the norm the parity bounds are stated in."""
    import numpy as np
    a = np.asarray(a, np.float64)
    r = np.asarray(ref, np.float64)
    if a.ndim == 1:
        a, r = a[:, None], r[:, None]
    num = np.linalg.norm(a - r, axis=1)
    den = np.linalg.norm(r, axis=1)
    return num / np.where(den > 0, den, 1.0)


def err_summary(e):
    import numpy as np
    e = np.asarray(e, np.float64)
    return {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)), "max": float(e.max())}


def mix64(idx):
    import numpy as np
    with np.errstate(over="ignore"):
        x = np.asarray(idx, np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def neighbour_sets_fp32(pos, ii, rule, rad=None, chunk=32):
    """Brute-force FP32 enumeration of the neighbour sets of bodies ii over
    all bodies, with the reference's expression r2 = (dx*dx + dy*dy) + dz*dz,
    dx = x_i - x_j (numpy float32 rounds each operation, no contraction).
    rule "ref": fl(r2) <= 1 (sph.c:231); "cubic": fl(r2) < fl((2 max(h_i,
    h_j))^2).  Returns (counts, order-independent hashes: sum of mix64(j)
    mod 2^64)."""
    import numpy as np
    pos = np.asarray(pos, np.float32)
    ii = np.asarray(ii)
    counts = np.zeros(len(ii), np.uint32)
    hashes = np.zeros(len(ii), np.uint64)
    mj = mix64(np.arange(len(pos)))
    for a in range(0, len(ii), chunk):
        sel = ii[a:a + chunk]
        d = pos[sel][:, None, :] - pos[None, :, :]
        r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
        if rule == "ref":
            m = r2 <= np.float32(1.0)
        else:
            h = np.asarray(rad, np.float32)
            s = np.float32(2.0) * np.maximum(h[sel][:, None], h[None, :])
            m = r2 < s * s
        counts[a:a + chunk] = m.sum(1)
        with np.errstate(over="ignore"):
            hashes[a:a + chunk] = np.where(m, mj[None, :], np.uint64(0)).sum(1, dtype=np.uint64)
    return counts, hashes
