"""The Newton kernel's table of rotation terms (FRAME_TERMS in ndt_align.cu) against the
rotation R = Rx(roll) Ry(pitch) Rz(yaw) and its first and second derivatives, evaluated
independently here (closed form for R, central differences for the derivatives)."""
import os
import re

import numpy as np

SRC = os.path.join(os.path.dirname(__file__), "..", "cuda_ndt_matcher_gb300", "csrc",
                   "ndt_align.cu")


def table():
    text = open(SRC).read()
    body = re.search(r"FRAME_TERMS\[90\]\s*=\s*\{([^}]*)\}", text).group(1)
    words = [int(w, 16) for w in re.findall(r"0x([0-9a-fA-F]+)u", body)]
    assert len(words) == 90
    return words


def evaluate(words, ang):
    sr, cr = np.sin(ang[0]), np.cos(ang[0])
    sp, cp = np.sin(ang[1]), np.cos(ang[1])
    sy, cy = np.sin(ang[2]), np.cos(ang[2])
    f = [sr, cr, sp, cp, sy, cy, 1.0, np.nan]
    coef = {0: 0.0, 1: 1.0, 2: -1.0}
    out = []
    for w in words:
        t0 = f[w & 7] * f[(w >> 3) & 7] * f[(w >> 6) & 7]
        t1 = f[(w >> 9) & 7] * f[(w >> 12) & 7] * f[(w >> 15) & 7]
        c0, c1 = coef[(w >> 18) & 3], coef[(w >> 20) & 3]
        out.append((c0 * t0 if c0 else 0.0) + (c1 * t1 if c1 else 0.0))
    return np.array(out).reshape(10, 3, 3)


def rot(a):
    r, p, y = a
    Rx = np.array([[1, 0, 0], [0, np.cos(r), -np.sin(r)], [0, np.sin(r), np.cos(r)]])
    Ry = np.array([[np.cos(p), 0, np.sin(p)], [0, 1, 0], [-np.sin(p), 0, np.cos(p)]])
    Rz = np.array([[np.cos(y), -np.sin(y), 0], [np.sin(y), np.cos(y), 0], [0, 0, 1]])
    return Rx @ Ry @ Rz


def test_frame_terms_match_rotation_derivatives():
    words = table()
    rng = np.random.default_rng(7)
    h = 1e-4
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for _ in range(20):
        a = rng.uniform(-np.pi, np.pi, 3)
        m = evaluate(words, a)
        np.testing.assert_allclose(m[0], rot(a), atol=1e-15)
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            d = (rot(a + e) - rot(a - e)) / (2 * h)
            np.testing.assert_allclose(m[1 + k], d, atol=1e-7)
        for n, (k, l) in enumerate(pairs):
            ek, el = np.zeros(3), np.zeros(3)
            ek[k] = h
            el[l] = h
            d2 = (rot(a + ek + el) - rot(a + ek - el) - rot(a - ek + el) + rot(a - ek - el)) \
                / (4 * h * h)
            if (k, l) == (1, 1):
                # the reference's point-Hessian table has +sin(pitch) in this entry
                # (src/ndt_cuda/src/derivatives/angular.rs:136-139) where d2R/dpitch2 has
                # -sin(pitch); the kernel keeps the reference's value
                np.testing.assert_allclose(d2[0, 2], -np.sin(a[1]), atol=1e-6)
                d2[0, 2] = np.sin(a[1])
            np.testing.assert_allclose(m[4 + n], d2, atol=1e-6)
