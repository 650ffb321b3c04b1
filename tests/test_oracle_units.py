"""Unit checks of the oracle's building blocks against independent restatements (numpy / Python)."""
import math

import numpy as np
import pytest

import numpy_fire as NF


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


def _block(res, dx=0.0125, dt=1.0 / 120.0, **extra):
    import fire_sim as F
    nx, ny, nz = res
    P = F.param_defaults().copy()
    for k, v in dict(nx=nx, ny=ny, nz=nz, dx=dx, dt=dt, **extra).items():
        P[NF.IDX[k]] = v
    return P


def test_adv1_matches_numpy_restatement(oracle_mod):
    """The oracle's first MacCormack pass (src/sim.js:123-157: RK2 midpoint back-trace, trilinear samples,
    outside fade, wind carried in from the open sides) against the numpy restatement, both in FP64."""
    res = (10, 14, 8)
    nx, ny, nz = res
    rng = np.random.default_rng(11)
    vel = np.zeros((nz, ny, nx, 4))
    vel[..., :3] = rng.uniform(-2.5, 2.5, (nz, ny, nx, 3))   # back-traces of up to ~2 cells, some leave the box
    S = rng.uniform(0.0, 1.0, (nz, ny, nx, 4))
    S2 = rng.uniform(0.0, 1.0, (nz, ny, nx, 4))
    P = _block(res, windX=0.7, windZ=-0.4)
    orc = oracle_mod.OracleSim(res, float(np.float32(0.0125)), dbl=True)
    orc.set_params(P)
    for k, a in (("vel", vel), ("S", S), ("S2", S2)):
        orc.put(k, a)
    orc.stage("adv1")
    velX, SX, S2X = NF.adv1(P, vel, S, S2)
    b = NF.backtrace(vel, NF.centres(S.shape), NF.par(P, "dt"), NF.par(P, "dx"))
    fade = NF.outside_fade(b, res)
    assert (fade < 1.0).any() and (fade > 0.0).any()   # the case reaches the open sides
    np.testing.assert_allclose(orc.get("velX", np.float64)[..., :3], velX[..., :3], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(orc.get("SX", np.float64), SX, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(orc.get("S2X", np.float64), S2X, rtol=1e-9, atol=1e-12)


def test_adv2_matches_numpy_restatement(oracle_mod):
    """The oracle's MacCormack correction and limiter (src/sim.js:159-197: reverse sample of the hats at the
    forward-traced point, min/max of the 8 clamped texels around the back-traced point, revert where that
    point's stencil leaves the domain, non-negative scalars) against the numpy restatement, both in FP64."""
    res = (9, 12, 7)
    nx, ny, nz = res
    rng = np.random.default_rng(12)
    sh = (nz, ny, nx, 4)
    vel = np.zeros(sh)
    vel[..., :3] = rng.uniform(-2.5, 2.5, sh[:3] + (3,))
    S, S2 = rng.uniform(0, 1, sh), rng.uniform(0, 1, sh)
    velX, SX, S2X = vel + rng.normal(0, 0.3, sh), S + rng.normal(0, 0.2, sh), S2 + rng.normal(0, 0.2, sh)
    velX[..., 3] = 0.0
    P = _block(res)
    orc = oracle_mod.OracleSim(res, float(np.float32(0.0125)), dbl=True)
    orc.set_params(P)
    for k, a in (("vel", vel), ("S", S), ("S2", S2), ("velX", velX), ("SX", SX), ("S2X", S2X)):
        orc.put(k, a)
    orc.stage("adv2")
    b = NF.backtrace(vel, NF.centres(S.shape), NF.par(P, "dt"), NF.par(P, "dx"))
    revert = NF.outside_fade(b, res) < 1.0
    assert revert.any() and (~revert).any()
    for name, want, ch in zip(("velY", "SY", "S2Y"), NF.adv2(P, vel, S, S2, velX, SX, S2X), (3, 4, 4)):
        np.testing.assert_allclose(orc.get(name, np.float64)[..., :ch], want[..., :ch], rtol=1e-9, atol=1e-12, err_msg=name)


def test_div_matches_numpy_restatement(oracle_mod):
    """Divergence minus the expansion target (src/sim.js:399-413): clamped central differences of velX,
    the floor's mirrored normal velocity, minus phi (velX.w)."""
    res = (9, 11, 8)
    nx, ny, nz = res
    rng = np.random.default_rng(13)
    vx = rng.uniform(-2, 2, (nz, ny, nx, 4))
    P = _block(res)
    orc = oracle_mod.OracleSim(res, float(np.float32(0.0125)), dbl=True)
    orc.set_params(P)
    orc.put("velX", vx)
    orc.stage("div")
    np.testing.assert_allclose(orc.get_level(0, "b", np.float64), NF.div(P, vx), rtol=1e-12, atol=1e-12)


def test_project_matches_numpy_restatement(oracle_mod):
    """Projection (src/sim.js:526-550): minus the central pressure gradient with the open-side (-p) and floor
    (+p) ghosts, zero in solids, no flow into the floor, speed capped at 20."""
    res = (9, 11, 8)
    nx, ny, nz = res
    rng = np.random.default_rng(14)
    vx = np.zeros((nz, ny, nx, 4))
    vx[..., :3] = rng.uniform(-3, 3, (nz, ny, nx, 3))
    p = rng.uniform(-0.02, 0.02, (nz, ny, nx))
    p[2, 5, 4] = 3.0                                    # a gradient that pushes the speed past the cap
    geo = np.zeros((nz, ny, nx, 4))
    geo[3:5, 2:4, 3:6, 2] = 1.0                         # a solid block (geo.b > 0.5)
    P = _block(res)
    orc = oracle_mod.OracleSim(res, float(np.float32(0.0125)), dbl=True)
    orc.set_params(P)
    orc.put("velX", vx)
    orc.put("geo", geo)
    orc.put_level(0, "p", p)
    orc.stage("project")
    want = NF.project(P, vx, p, geo)
    assert (np.linalg.norm(vx[..., :3] - 0, axis=-1) < 20).all() and np.isclose(np.linalg.norm(want[..., :3], axis=-1).max(), 20.0)
    np.testing.assert_allclose(orc.get("vel", np.float64)[..., :3], want[..., :3], rtol=1e-12, atol=1e-12)


def test_multigrid_operators_match_numpy_restatement(oracle_mod):
    """One red-black colour sweep, the fused residual + restriction and the mirror-ghost prolongation
    (src/sim.js:417-495) of the oracle's FP64 mode against the numpy restatements."""
    res = (12, 16, 10)
    orc = oracle_mod.OracleSim(res, 0.0125, dbl=True)
    (nx, ny, nz), h = orc.levels[0]
    (cx, cy, cz), _ = orc.levels[1]
    rng = np.random.default_rng(31)
    p = rng.normal(0, 1, (nz, ny, nx))
    b = rng.normal(0, 50, (nz, ny, nx))
    orc.put_level(0, "p", p)
    orc.put_level(0, "b", b)
    orc.mg_smooth(0, 1)
    want = NF.smooth_colour(p, b, h, 1)
    assert not np.array_equal(want, p)
    np.testing.assert_allclose(orc.get_level(0, "p", np.float64), want, rtol=1e-12, atol=1e-12)
    orc.mg_restrict(0)
    np.testing.assert_allclose(orc.get_level(1, "b", np.float64), NF.restrict(want, b, h, (cx, cy, cz)), rtol=1e-11, atol=1e-9)
    assert not orc.get_level(1, "p", np.float64).any()
    pc = rng.normal(0, 1, (cz, cy, cx))
    orc.put_level(1, "p", pc)
    orc.mg_prolong(0)
    np.testing.assert_allclose(orc.get_level(0, "p", np.float64), NF.prolong_add(want, pc), rtol=1e-12, atol=1e-12)


def test_vcycle_matches_numpy_restatement(oracle_mod):
    """The step's V(2,2) cycle (src/sim.js:576-599): pre-sweeps and residual restriction down the hierarchy,
    coarseIters sweeps on the coarsest level (src/sim.js:88-92), prolongation and post-sweeps back up."""
    res = (16, 24, 16)
    orc = oracle_mod.OracleSim(res, 0.0125, dbl=True)
    assert len(orc.levels) >= 3
    rng = np.random.default_rng(41)
    (nx, ny, nz), _ = orc.levels[0]
    p0 = rng.normal(0, 1, (nz, ny, nx))
    b0 = rng.normal(0, 30, (nz, ny, nx))
    orc.put_level(0, "p", p0)
    orc.put_level(0, "b", b0)
    orc.vcycle(2, 2)
    want = NF.vcycle(orc.levels, orc.coarse_iters, p0, b0)
    np.testing.assert_allclose(orc.get_level(0, "p", np.float64), want, rtol=1e-9, atol=1e-9 * np.abs(want).max())
