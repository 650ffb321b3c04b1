"""Unit checks of the oracle's building blocks against independent restatements (numpy / Python)."""
import math

import numpy as np
import pytest


def test_half_rounding_matches_numpy(oracle_mod):
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.standard_normal(20000).astype(np.float32) * 10,
                           rng.standard_normal(5000).astype(np.float32) * 1e-5,      # subnormal halves
                           np.array([65504, 65519, 65520, 1e6, -0.0, 5.96e-8, 2.98e-8, 2.99e-8], np.float32)])
    L = oracle_mod.lib()
    got = np.array([L.orc_f16_to_f32(L.orc_f32_to_f16(float(v))) for v in vals], np.float32)
    want = vals.astype(np.float16).astype(np.float32)
    np.testing.assert_array_equal(got, want)


def _pcg3d(x, y, z):
    M = 0xFFFFFFFF
    v = [(x * 1664525 + 1013904223) & M, (y * 1664525 + 1013904223) & M, (z * 1664525 + 1013904223) & M]
    v[0] = (v[0] + v[1] * v[2]) & M; v[1] = (v[1] + v[2] * v[0]) & M; v[2] = (v[2] + v[0] * v[1]) & M
    v = [a ^ (a >> 16) for a in v]
    v[0] = (v[0] + v[1] * v[2]) & M; v[1] = (v[1] + v[2] * v[0]) & M; v[2] = (v[2] + v[0] * v[1]) & M
    return v


def test_pcg3d_hash(oracle_mod):
    """src/shaders/lib.js:4-10, 16 restated in Python integers."""
    L = oracle_mod.lib()
    out = np.zeros(3, np.float32)
    for (x, y, z) in [(0, 0, 0), (1, 2, 3), (-5, 7, 1013), (127, 127, 127), (2 ** 31 - 1, -2 ** 31, 12345)]:
        L.orc_hash3f(x, y, z, oracle_mod._ptr(out))
        want = [np.float32(np.float32(v) * np.float32(2.0 ** -32)) for v in _pcg3d(x & 0xFFFFFFFF, y & 0xFFFFFFFF, z & 0xFFFFFFFF)]
        assert list(out) == want


def _build_campfire_py(seed=7):
    """src/scene.js:13-42, 92-98 restated in Python doubles (JS Number semantics)."""
    s = [seed & 0xFFFFFFFF]

    def R():
        s[0] = (s[0] * 1664525 + 1013904223) & 0xFFFFFFFF
        return s[0] / 4294967296
    logs = [[-0.40, 0.055, -0.17, 0.062, 0.38, 0.065, -0.13, 0.8], [-0.36, 0.060, 0.15, 0.058, 0.41, 0.050, 0.19, 0.8]]
    for i in range(5):
        ang = (i / 5) * math.pi * 2 + 0.35 + (R() - 0.5) * 0.4
        rb = 0.30 + R() * 0.06
        base = [math.cos(ang) * rb, 0.03, math.sin(ang) * rb]
        topR = 0.035 + R() * 0.03
        ta = ang + math.pi + (R() - 0.5) * 0.8
        top = [math.cos(ta) * topR, 0.36 + R() * 0.1, math.sin(ta) * topR]
        logs.append(base + [0.032 + R() * 0.012] + top + [1.0])
    logs.append([-0.12, 0.035, 0.02, 0.035, 0.10, 0.03, -0.05, 1.0])
    out = np.zeros(128, np.float32)
    for i, l in enumerate(logs):
        out[i * 8:(i + 1) * 8] = l
    return out


@pytest.mark.parametrize("seed", [7, 1, 12345])
def test_build_campfire(oracle_mod, seed):
    np.testing.assert_array_equal(oracle_mod.build_campfire(seed), _build_campfire_py(seed))


def test_noise_table_properties(tables):
    noise, curl = tables
    assert noise.shape == (128, 128, 128, 4) and curl.shape == noise.shape
    # fBm channels are centred near 0.5, Worley in [0, 1]
    for c in range(3):
        assert 0.40 < noise[..., c].mean() < 0.60
        assert noise[..., c].min() >= 0.0 - 1e-3 and noise[..., c].max() <= 1.0 + 1e-3
    assert noise[..., 3].min() >= 0.0 and noise[..., 3].max() <= 1.0
    # values are exactly representable halves
    np.testing.assert_array_equal(noise, noise.astype(np.float16).astype(np.float32))
    np.testing.assert_array_equal(curl, curl.astype(np.float16).astype(np.float32))


def test_curl_table_matches_numpy(tables):
    """src/noise.js:69-80: periodic central-difference curl of the noise xyz times N/2."""
    noise, curl = tables
    L = noise[..., :3].astype(np.float32) * np.float32(2) - np.float32(1)   # [z, y, x, c]
    d = lambda ax: np.roll(L, -1, axis=ax) - np.roll(L, 1, axis=ax)
    dx, dy, dz = d(2), d(1), d(0)
    c = np.stack([dy[..., 2] - dz[..., 1], dz[..., 0] - dx[..., 2], dx[..., 1] - dy[..., 0]], -1) * np.float32(64)
    np.testing.assert_array_equal(curl[..., :3], c.astype(np.float16).astype(np.float32))
    w = np.sqrt((c[..., 0] * c[..., 0] + c[..., 1] * c[..., 1]) + c[..., 2] * c[..., 2])
    np.testing.assert_array_equal(curl[..., 3], w.astype(np.float16).astype(np.float32))


def test_level_hierarchy(oracle_mod):
    """src/sim.js:79-92: level dims, spacing and coarse sweep counts of the configured grids."""
    O = oracle_mod.OracleSim((48, 96, 48), 0.0125)
    assert [l[0] for l in O.levels] == [(48, 96, 48), (24, 48, 24), (12, 24, 12), (6, 12, 6)]
    mu = (math.cos(math.pi / 6) + math.cos(math.pi / 24) + math.cos(math.pi / 6)) / 3
    assert O.coarse_iters == max(8, min(64, math.ceil(math.log(0.05) / math.log(mu * mu))))
    O2 = oracle_mod.OracleSim((128, 256, 128), 0.005)
    assert [l[0] for l in O2.levels][-1] == (4, 8, 4) and len(O2.levels) == 6
    assert O2.levels[2][1] == pytest.approx(0.02, rel=1e-6)
