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


def _trilinear(f, c):
    """textureSampleLevel with a linear, clamp-to-edge sampler at positions c (..., 3) in cell units (texel i's
    centre at i + 0.5), as a weighted sum of the 8 texels."""
    nz, ny, nx = f.shape[:3]
    u = c - 0.5
    i0 = np.floor(u).astype(np.int64)
    fr = u - i0
    out = np.zeros(c.shape[:-1] + (f.shape[-1],))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = ((fr[..., 0] if dx else 1 - fr[..., 0]) * (fr[..., 1] if dy else 1 - fr[..., 1]) *
                     (fr[..., 2] if dz else 1 - fr[..., 2]))
                ix = np.clip(i0[..., 0] + dx, 0, nx - 1)
                iy = np.clip(i0[..., 1] + dy, 0, ny - 1)
                iz = np.clip(i0[..., 2] + dz, 0, nz - 1)
                out += w[..., None] * f[iz, iy, ix]
    return out


def test_adv1_matches_numpy_restatement(oracle_mod):
    """The oracle's first MacCormack pass (src/sim.js:123-157: RK2 midpoint back-trace, trilinear samples,
    outside fade, wind carried in from the open sides) against a numpy restatement, both in FP64."""
    import fire_sim as F
    res, dx, dt = (10, 14, 8), 0.0125, 1.0 / 120.0
    nx, ny, nz = res
    rng = np.random.default_rng(11)
    vel = np.zeros((nz, ny, nx, 4))
    vel[..., :3] = rng.uniform(-2.5, 2.5, (nz, ny, nx, 3))   # back-traces of up to ~2 cells, some leave the box
    S = rng.uniform(0.0, 1.0, (nz, ny, nx, 4))
    S2 = rng.uniform(0.0, 1.0, (nz, ny, nx, 4))
    p = F.param_defaults().copy()
    idx = {n: i for i, n in enumerate(F.SIM_FIELDS)}
    for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("dx", dx), ("dt", dt), ("windX", 0.7), ("windZ", -0.4)):
        p[idx[k]] = v
    orc = oracle_mod.OracleSim(res, float(np.float32(dx)), dbl=True)
    orc.set_params(p)
    for k, a in (("vel", vel), ("S", S), ("S2", S2)):
        orc.put(k, a)
    orc.stage("adv1")
    dt64, dx64 = float(p[idx["dt"]]), float(p[idx["dx"]])
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    c = np.stack([i, j, k], -1) + 0.5
    v0 = _trilinear(vel, c)[..., :3]
    mid = c - 0.5 * dt64 * v0 / dx64
    b = c - dt64 * _trilinear(vel, mid)[..., :3] / dx64
    lo = np.minimum(b[..., 0], b[..., 2])
    hi = np.maximum(b[..., 0] - nx, np.maximum(b[..., 1] - ny, b[..., 2] - nz))
    fade = np.clip(1.0 - np.maximum(-lo, hi), 0.0, 1.0)
    t = np.clip((b[..., 1] * dx64 - 0.03) / (0.4 - 0.03), 0.0, 1.0)
    ws = t * t * (3.0 - 2.0 * t)
    wind = np.stack([float(p[idx["windX"]]) * ws, 0.0 * ws, float(p[idx["windZ"]]) * ws], -1)
    sv = _trilinear(vel, b)[..., :3]
    want_v = wind * (1.0 - fade[..., None]) + sv * fade[..., None]
    assert (fade < 1.0).any() and (fade > 0.0).any()   # the case reaches the open sides
    np.testing.assert_allclose(orc.get("velX", np.float64)[..., :3], want_v, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(orc.get("SX", np.float64), _trilinear(S, b) * fade[..., None], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(orc.get("S2X", np.float64), _trilinear(S2, b) * fade[..., None], rtol=1e-9, atol=1e-12)


def test_adv2_matches_numpy_restatement(oracle_mod):
    """The oracle's MacCormack correction and limiter (src/sim.js:159-197: reverse sample of the hats at the
    forward-traced point, min/max of the 8 clamped texels around the back-traced point, revert where that
    point's stencil leaves the domain, non-negative scalars) against a numpy restatement, both in FP64."""
    import fire_sim as F
    res, dx, dt = (9, 12, 7), 0.0125, 1.0 / 120.0
    nx, ny, nz = res
    rng = np.random.default_rng(12)
    sh = (nz, ny, nx, 4)
    vel = np.zeros(sh)
    vel[..., :3] = rng.uniform(-2.5, 2.5, sh[:3] + (3,))
    fields = {"vel": vel, "S": rng.uniform(0, 1, sh), "S2": rng.uniform(0, 1, sh)}
    hats = {"velX": vel + rng.normal(0, 0.3, sh), "SX": fields["S"] + rng.normal(0, 0.2, sh),
            "S2X": fields["S2"] + rng.normal(0, 0.2, sh)}
    hats["velX"][..., 3] = 0.0
    p = F.param_defaults().copy()
    idx = {n: i for i, n in enumerate(F.SIM_FIELDS)}
    for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("dx", dx), ("dt", dt)):
        p[idx[k]] = v
    orc = oracle_mod.OracleSim(res, float(np.float32(dx)), dbl=True)
    orc.set_params(p)
    for k, a in list(fields.items()) + list(hats.items()):
        orc.put(k, a)
    orc.stage("adv2")
    dt64, dx64 = float(p[idx["dt"]]), float(p[idx["dx"]])
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    c = np.stack([i, j, k], -1) + 0.5
    v = vel[..., :3]
    fw = c + dt64 * v / dx64
    mid = c - 0.5 * dt64 * _trilinear(vel, c)[..., :3] / dx64
    b = c - dt64 * _trilinear(vel, mid)[..., :3] / dx64 - 0.5
    b0 = np.floor(b).astype(np.int64)
    lo_b = np.minimum(b[..., 0] + 0.5, b[..., 2] + 0.5)
    hi_b = np.maximum(b[..., 0] + 0.5 - nx, np.maximum(b[..., 1] + 0.5 - ny, b[..., 2] + 0.5 - nz))
    revert = np.clip(1.0 - np.maximum(-lo_b, hi_b), 0.0, 1.0) < 1.0
    assert revert.any() and (~revert).any()
    for name, hat, out, ch in (("vel", "velX", "velY", 3), ("S", "SX", "SY", 4), ("S2", "S2X", "S2Y", 4)):
        f, h = fields[name], hats[hat]
        N = h + 0.5 * (f - _trilinear(h, fw))
        N[revert] = h[revert]
        mn = np.full(f.shape, 1e9)
        mx = np.full(f.shape, -1e9)
        for q in range(8):
            qx = np.clip(b0[..., 0] + (q & 1), 0, nx - 1)
            qy = np.clip(b0[..., 1] + ((q >> 1) & 1), 0, ny - 1)
            qz = np.clip(b0[..., 2] + ((q >> 2) & 1), 0, nz - 1)
            t = f[qz, qy, qx]
            mn, mx = np.minimum(mn, t), np.maximum(mx, t)
        want = np.minimum(np.maximum(N, np.minimum(mn, h)), np.maximum(mx, h))
        if name != "vel":
            want = np.maximum(want, 0.0)
        got = orc.get(out, np.float64)
        np.testing.assert_allclose(got[..., :ch], want[..., :ch], rtol=1e-9, atol=1e-12, err_msg=out)


def _setup_small(oracle_mod, res, seed):
    import fire_sim as F
    nx, ny, nz = res
    p = F.param_defaults().copy()
    idx = {n: i for i, n in enumerate(F.SIM_FIELDS)}
    for k, v in (("nx", nx), ("ny", ny), ("nz", nz), ("dx", 0.0125), ("dt", 1.0 / 120.0)):
        p[idx[k]] = v
    orc = oracle_mod.OracleSim(res, float(np.float32(0.0125)), dbl=True)
    orc.set_params(p)
    return orc, float(p[idx["dx"]]), np.random.default_rng(seed)


def test_div_matches_numpy_restatement(oracle_mod):
    """Divergence minus the expansion target (src/sim.js:399-413): clamped central differences of velX,
    the floor's mirrored normal velocity, minus phi (velX.w)."""
    res = (9, 11, 8)
    nx, ny, nz = res
    orc, dx, rng = _setup_small(oracle_mod, res, 13)
    vx = rng.uniform(-2, 2, (nz, ny, nx, 4))
    orc.put("velX", vx)
    orc.stage("div")
    pad = lambda a: np.pad(a, 1, mode="edge")
    u, v, w = (pad(vx[..., c]) for c in range(3))
    R, L = u[1:-1, 1:-1, 2:], u[1:-1, 1:-1, :-2]
    T, B = v[1:-1, 2:, 1:-1], v[1:-1, :-2, 1:-1].copy()
    F_, K = w[2:, 1:-1, 1:-1], w[:-2, 1:-1, 1:-1]
    B[:, 0, :] = -vx[:, 0, :, 1]
    want = ((R - L) + (T - B) + (F_ - K)) / (2.0 * dx) - vx[..., 3]
    np.testing.assert_allclose(orc.get_level(0, "b", np.float64), want, rtol=1e-12, atol=1e-12)


def test_project_matches_numpy_restatement(oracle_mod):
    """Projection (src/sim.js:526-550): minus the central pressure gradient with the open-side (-p) and floor
    (+p) ghosts, zero in solids, no flow into the floor, speed capped at 20."""
    res = (9, 11, 8)
    nx, ny, nz = res
    orc, dx, rng = _setup_small(oracle_mod, res, 14)
    vx = np.zeros((nz, ny, nx, 4))
    vx[..., :3] = rng.uniform(-3, 3, (nz, ny, nx, 3))
    p = rng.uniform(-0.02, 0.02, (nz, ny, nx))
    p[2, 5, 4] = 3.0                                    # a gradient that pushes the speed past the cap
    geo = np.zeros((nz, ny, nx, 4))
    geo[3:5, 2:4, 3:6, 2] = 1.0                         # a solid block (geo.b > 0.5)
    orc.put("velX", vx)
    orc.put("geo", geo)
    orc.put_level(0, "p", p)
    orc.stage("project")
    pp = np.pad(p, 1)
    # ghosts: -me beyond the open sides and the top, +me below the floor (y < 0)
    me = p
    xm = np.where(np.arange(nx)[None, None, :] > 0, pp[1:-1, 1:-1, :-2], -me)
    xp = np.where(np.arange(nx)[None, None, :] < nx - 1, pp[1:-1, 1:-1, 2:], -me)
    ym = np.where(np.arange(ny)[None, :, None] > 0, pp[1:-1, :-2, 1:-1], me)
    yp = np.where(np.arange(ny)[None, :, None] < ny - 1, pp[1:-1, 2:, 1:-1], -me)
    zm = np.where(np.arange(nz)[:, None, None] > 0, pp[:-2, 1:-1, 1:-1], -me)
    zp = np.where(np.arange(nz)[:, None, None] < nz - 1, pp[2:, 1:-1, 1:-1], -me)
    g = np.stack([xp - xm, yp - ym, zp - zm], -1) / (2.0 * dx)
    v = vx[..., :3] - g
    v[geo[..., 2] > 0.5] = 0.0
    v[:, 0, :, 1] = np.maximum(v[:, 0, :, 1], 0.0)
    vl = np.linalg.norm(v, axis=-1)
    cap = vl > 20.0
    assert cap.any()
    v[cap] *= (20.0 / vl[cap])[:, None]
    np.testing.assert_allclose(orc.get("vel", np.float64)[..., :3], v, rtol=1e-12, atol=1e-12)


def _neighbours(p):
    """The six neighbour values of every cell with the ghost rules applied (ghosts use the cell's own value)."""
    nz, ny, nx = p.shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    get = lambda a, b, c: p[np.clip(a, 0, nz - 1), np.clip(b, 0, ny - 1), np.clip(c, 0, nx - 1)]
    xm = np.where(i > 0, get(k, j, i - 1), -p)
    xp = np.where(i < nx - 1, get(k, j, i + 1), -p)
    zm = np.where(k > 0, get(k - 1, j, i), -p)
    zp = np.where(k < nz - 1, get(k + 1, j, i), -p)
    ym = np.where(j > 0, get(k, j - 1, i), p)
    yp = np.where(j < ny - 1, get(k, j + 1, i), -p)
    return xm, xp, ym, yp, zm, zp


def test_multigrid_operators_match_numpy_restatement(oracle_mod):
    """One red-black colour sweep, the fused residual + restriction and the mirror-ghost prolongation
    (src/sim.js:417-495) of the oracle's FP64 mode against numpy restatements (the helpers below)."""
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
    want = _smooth_colour(p, b, h, 1)
    assert not np.array_equal(want, p)
    np.testing.assert_allclose(orc.get_level(0, "p", np.float64), want, rtol=1e-12, atol=1e-12)
    orc.mg_restrict(0)
    np.testing.assert_allclose(orc.get_level(1, "b", np.float64), _restrict(want, b, h, (cx, cy, cz)), rtol=1e-11, atol=1e-9)
    assert not orc.get_level(1, "p", np.float64).any()
    pc = rng.normal(0, 1, (cz, cy, cx))
    orc.put_level(1, "p", pc)
    orc.mg_prolong(0)
    np.testing.assert_allclose(orc.get_level(0, "p", np.float64), _prolong_add(want, pc), rtol=1e-12, atol=1e-12)


def _smooth_colour(p, b, h, colour):
    """One red-black colour sweep (src/sim.js:417-437): the cells with (x + y + z + colour) even."""
    nz, ny, nx = p.shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    nb = _neighbours(p)
    inside = [i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1]
    ssum = sum(np.where(m, v, 0.0) for m, v in zip(inside, nb))
    diag = 6.0 + (i == 0) + (i == nx - 1) + (k == 0) + (k == nz - 1) + (j == ny - 1) - (j == 0)
    return np.where((i + j + k + colour) % 2 == 0, (ssum - h * h * b) / diag, p)


def _restrict(p, b, h, cdims):
    cx, cy, cz = cdims
    xm, xp, ym, yp, zm, zp = _neighbours(p)
    r = b - (xm + xp + ym + yp + zm + zp - 6.0 * p) / (h * h)
    return r[:2 * cz, :2 * cy, :2 * cx].reshape(cz, 2, cy, 2, cx, 2).mean(axis=(1, 3, 5))


def _prolong_add(p, pc):
    nz, ny, nx = p.shape
    cz, cy, cx = pc.shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    g = (np.stack([i, j, k], -1) + 0.5) * 0.5 - 0.5
    g0 = np.floor(g).astype(np.int64)
    f = g - g0
    nc = np.array([cx, cy, cz])
    acc = np.zeros(p.shape)
    for q8 in range(8):
        o = np.array([q8 & 1, (q8 >> 1) & 1, (q8 >> 2) & 1])
        q = g0 + o
        qc = np.clip(q, 0, nc - 1)
        val = pc[qc[..., 2], qc[..., 1], qc[..., 0]]
        val = np.where((q[..., 0] < 0) | (q[..., 0] >= cx), -val, val)
        val = np.where((q[..., 2] < 0) | (q[..., 2] >= cz), -val, val)
        val = np.where(q[..., 1] >= cy, -val, val)
        w = np.where(o == 1, f, 1.0 - f)
        acc += val * w[..., 0] * w[..., 1] * w[..., 2]
    return p + acc


def test_vcycle_matches_numpy_restatement(oracle_mod):
    """The step's V(2,2) cycle (src/sim.js:576-599): pre-sweeps and residual restriction down the hierarchy,
    coarseIters sweeps on the coarsest level (src/sim.js:88-92), prolongation and post-sweeps back up — the
    oracle's FP64 cycle against one composed from the numpy operators."""
    res = (16, 24, 16)
    orc = oracle_mod.OracleSim(res, 0.0125, dbl=True)
    levels = orc.levels
    assert len(levels) >= 3
    rng = np.random.default_rng(41)
    (nx, ny, nz), _ = levels[0]
    p0 = rng.normal(0, 1, (nz, ny, nx))
    b0 = rng.normal(0, 30, (nz, ny, nx))
    orc.put_level(0, "p", p0)
    orc.put_level(0, "b", b0)
    orc.vcycle(2, 2)
    P, B = [p0], [b0]
    n = len(levels)
    for l in range(n - 1):
        h = levels[l][1]
        for _ in range(2):
            P[l] = _smooth_colour(_smooth_colour(P[l], B[l], h, 0), B[l], h, 1)
        B.append(_restrict(P[l], B[l], h, levels[l + 1][0]))
        cx, cy, cz = levels[l + 1][0]
        P.append(np.zeros((cz, cy, cx)))
    for _ in range(orc.coarse_iters):
        P[n - 1] = _smooth_colour(_smooth_colour(P[n - 1], B[n - 1], levels[n - 1][1], 0), B[n - 1], levels[n - 1][1], 1)
    for l in range(n - 2, -1, -1):
        P[l] = _prolong_add(P[l], P[l + 1])
        for _ in range(2):
            P[l] = _smooth_colour(_smooth_colour(P[l], B[l], levels[l][1], 0), B[l], levels[l][1], 1)
    np.testing.assert_allclose(orc.get_level(0, "p", np.float64), P[0], rtol=1e-9, atol=1e-9 * np.abs(P[0]).max())
